"""CPU-only checks of the C-ABI library: it builds, loads without a GPU and
exports every entry point that include/lss.h and include/lss_phantom.h
declare; the Python binding covers the same set; without a device the
engine refuses cleanly."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import aworkefficientgpualgorithmforlevelsetsegmentation_gb300 as lss
from aworkefficientgpualgorithmforlevelsetsegmentation_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return set(re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\b(lss_\w+)\s*\(", text, flags=re.M))


def test_headers_declare_entry_points():
    names = declared("lss.h") | declared("lss_phantom.h")
    assert "lss_create" in names and "lss_step" in names and "lss_batch_run" in names
    assert len(names) >= 40


def test_library_exports_every_declared_symbol():
    L = lss.load()
    for name in sorted(declared("lss.h") | declared("lss_phantom.h")):
        assert hasattr(L, name), name


def test_binding_matches_headers():
    assert set(_lib.SIGNATURES) == declared("lss.h") | declared("lss_phantom.h")


def test_defaults_and_errors_without_device():
    L = lss.load()
    c = _lib.lss_config()
    assert L.lss_config_default(C.byref(c)) == 0 and c.mode == 1 and c.ref_quirk_i3 == 1
    p = _lib.lss_params()
    assert L.lss_params_default(0, C.byref(p)) == 0
    assert abs(p.temporal_threshold - 0.008) < 1e-9 and p.neighbourhood == 6
    assert L.lss_params_default(1, C.byref(p)) == 0 and p.phi_max == 4 and p.neighbourhood == 26
    assert L.lss_params_default(7, C.byref(p)) == 1
    assert L.lss_create(None, None) == 1
    assert L.lss_step(None, 1, None) == 1
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    # Kernel-level compaction: argument and size checks come before any
    # device call (the pointers below are never dereferenced).
    p = C.c_void_p(256)
    assert L.lss_compact_u32(None, p, p, 5, p, None) == 1           # LSS_ERR_INVALID_ARGUMENT
    assert L.lss_compact_u32(p, p, p, 1 << 40, p, None) == 9        # LSS_ERR_CAPACITY
    assert L.lss_compact_u32_noalloc(p, p, None, 5, p, None) == 1
    assert L.lss_compact_u32_noalloc(p, p, p, (1 << 26) + 1, p, None) == 9
    if not has_gpu:
        h = C.c_void_p()
        assert L.lss_create(C.byref(h), None) == 7  # LSS_ERR_NO_DEVICE
        assert L.lss_compact_u32(p, p, p, 5, p, None) == 7
        assert L.lss_compact_u32_noalloc(p, p, p, 5, p, None) == 7


def test_phantoms_are_deterministic():
    from aworkefficientgpualgorithmforlevelsetsegmentation_gb300 import phantoms as P
    a = P.config2(0.25)["image"]
    b = P.config2(0.25)["image"]
    assert np.array_equal(a, b)
    assert a.dtype == np.float32 and a.shape == (64, 64, 64)
    # intensities of the inner shell around 0.8, background 0
    assert 0.7 < float(a[32, 32, 32]) < 0.9
    e = P.ellipsoid((8, 8, 8), (3.5, 3.5, 3.5), (2, 2, 2), 1.0, 0.0, 0.0, 0)
    assert e[4, 4, 4] == 1.0 and e[0, 0, 0] == 0.0


STRUCTS = ["lss_config", "lss_params", "lss_conv", "lss_stats", "lss_grads"]


def test_struct_layouts_match_header(tmp_path):
    """Every struct the binding mirrors has the header's size and field
    offsets, as a C compiler lays them out on this machine."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "lss.h"', "int main(void) {"]
    for sname in STRUCTS:
        st = getattr(_lib, sname)
        lines.append(f'printf("{sname} %zu\\n", sizeof({sname}));')
        for f, _ in st._fields_:
            lines.append(f'printf("{sname}.{f} %zu\\n", offsetof({sname}, {f}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = dict(l.split() for l in subprocess.run([str(exe)], check=True, capture_output=True,
                                                text=True).stdout.splitlines())
    for sname in STRUCTS:
        st = getattr(_lib, sname)
        assert int(got[sname]) == C.sizeof(st), sname
        for f, _ in st._fields_:
            assert int(got[f"{sname}.{f}"]) == getattr(st, f).offset, (sname, f)


def test_readback_out_arrays_are_checked():
    """Read-backs accept a caller-owned output array only with the volume's
    shape and dtype, C-contiguous and writeable."""
    from aworkefficientgpualgorithmforlevelsetsegmentation_gb300.segmenter import _out
    a = np.empty((3, 4, 5), np.uint8)
    assert _out(a, (3, 4, 5), np.uint8) is a
    fresh = _out(None, (3, 4, 5), np.float32)
    assert fresh.shape == (3, 4, 5) and fresh.dtype == np.float32 and not fresh.any()
    ro = np.empty((3, 4, 5), np.uint8)
    ro.flags.writeable = False
    for bad in (np.empty((3, 4, 6), np.uint8), np.empty((3, 4, 5), np.int8),
                np.empty((5, 4, 3), np.uint8).transpose(2, 1, 0), ro):
        with pytest.raises(ValueError):
            _out(bad, (3, 4, 5), np.uint8)


def test_phantom_library_matches_solver_library_and_defaults():
    """libphantom.so (host-only generators) gives the same bits as the
    generators inside liblss.so, and the workloads' parameter defaults equal
    lss_params_default(LSS_MODE_NS)."""
    from aworkefficientgpualgorithmforlevelsetsegmentation_gb300 import phantoms as P
    L, G = lss.load(), _lib.load_phantom()
    shape = (21, 18, 27)
    outs = []
    for lib in (L, G):
        a = np.zeros(shape, np.float32)
        ax = np.array([9, 8, 7, 5, 4, 3], np.float32)
        vals = np.array([0.3, 0.7], np.float32)
        assert lib.lss_phantom_shells(27, 18, 21, 2, C.c_void_p(ax.ctypes.data), C.c_void_p(vals.ctypes.data),
                                      0.1, 2.0, 8, 5, 1.0, 0.04, 6, C.c_void_p(a.ctypes.data)) == 0
        s = np.zeros(shape, np.float32)
        sp = np.array([13.2, 8.5, 10.1, 3.0], np.float32)
        assert lib.lss_phantom_sdf_spheres(27, 18, 21, C.c_void_p(sp.ctypes.data), 1, -4.0, 4.0,
                                           C.c_void_p(s.ctypes.data)) == 0
        outs.append((a, s, lib.lss_phantom_uniform(4, 17)))
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])
    assert outs[0][2] == outs[1][2]
    p = _lib.lss_params()
    assert L.lss_params_default(1, C.byref(p)) == 0
    q = _lib.lss_params(**P.NS_DEFAULTS)  # the same float32 / int32 fields
    for k, _ in _lib.lss_params._fields_:
        assert getattr(p, k) == getattr(q, k), k
