"""ORACLE — test infrastructure only.

ctypes wrapper of the CPU oracle (oracle/_build/liboracle.so).  Imported only
by tests/, __graft_entry__.smoke() and bench.py's CPU legs, always as the
parity reference or the timed CPU baseline, never as the thing measured or
shipped.

  RefOracle — the reference-faithful solver (ref_model.hpp), either with the
              restated kernels or, where oracle/_ref was built, with the
              reference's own kernel sources compiled for the CPU.
  NsOracle  — the FP64 LSS_MODE_NS solver (ns_model.hpp).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build  # type: ignore[attr-defined]

_HERE = os.path.dirname(os.path.abspath(__file__))
_libs: dict[str, C.CDLL] = {}

_DTYPES = {0: np.uint8, 1: np.int8, 2: np.uint16, 3: np.int16, 4: np.uint32, 5: np.int32,
           6: np.float32}
_P = C.c_void_p


def _ptr(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


def _declare(lib: C.CDLL, prefix: str) -> None:
    f = lambda n: getattr(lib, prefix + n)  # noqa: E731
    f("create").restype = _P
    f("create").argtypes = [_P, C.c_uint32, C.c_uint32, C.c_uint32, C.c_int, C.c_float, C.c_int]
    f("destroy").argtypes = [_P]
    f("last_error").restype = C.c_char_p
    f("set_params").argtypes = [_P] + [C.c_float] * 5
    f("initialize_seed").argtypes = [_P] + [C.c_float] * 4
    f("set_phi").argtypes = [_P, _P]
    f("step").argtypes = [_P, C.c_int]
    f("active_count").restype = C.c_uint64
    f("active_count").argtypes = [_P]
    f("iterations").argtypes = [_P]
    f("finished").argtypes = [_P]
    f("padded_dims").argtypes = [_P, _P]
    f("get_buffer").argtypes = [_P, C.c_int, _P]
    for n in ("read_mask", "read_phi", "read_export", "read_active_volume"):
        f(n).argtypes = [_P, _P]
    for n in ("freeze", "clear_current", "clear_all"):
        f(n).argtypes = [_P]
    f("estimate_params").argtypes = [_P, _P, _P]


def lib() -> C.CDLL:
    if "oracle" not in _libs:
        path = _build.build()
        L = C.CDLL(path)
        _declare(L, "oref_")
        L.ons_create.restype = _P
        L.ons_create.argtypes = [C.c_int, C.c_int, C.c_int, _P, C.c_int, C.c_int, C.c_int]
        L.ons_destroy.argtypes = [_P]
        L.ons_set_params.argtypes = [_P] + [C.c_double] * 8 + [C.c_int]
        L.ons_set_threads.argtypes = [_P, C.c_int]
        L.ons_set_alpha_role.argtypes = [_P, C.c_int]
        L.ons_set_data_term.argtypes = [_P, C.c_int]
        L.ons_set_bias.argtypes = [_P, _P]
        L.ons_set_phi.argtypes = [_P, _P]
        L.ons_set_state.argtypes = [_P, _P, _P, C.c_uint64]
        L.ons_step.restype = C.c_uint64
        L.ons_step.argtypes = [_P, C.c_int]
        L.ons_run.argtypes = [_P, C.c_double, C.c_int, C.c_int, C.c_uint64]
        for n in ("ons_active_count", "ons_initial_count", "ons_updates"):
            getattr(L, n).restype = C.c_uint64
            getattr(L, n).argtypes = [_P]
        L.ons_read_active.argtypes = [_P, _P]
        L.ons_read_phi.argtypes = [_P, _P]
        L.ons_read_phi64.argtypes = [_P, _P]
        L.ons_expand_given.restype = C.c_uint64
        L.ons_expand_given.argtypes = [_P, _P, C.c_uint64, _P, _P, _P]
        L.ons_adj_run.argtypes = [_P, C.c_int, _P, C.c_double, _P, _P]
        L.ons_adj_loss.restype = C.c_double
        L.ons_adj_loss.argtypes = [_P, C.c_int, _P, C.c_double]
        L.ons_adj_dice.restype = C.c_double
        L.ons_adj_dice.argtypes = [_P, C.c_int, _P, C.c_double]
        L.ons_set_param.argtypes = [_P, C.c_int, C.c_double]
        L.ons_set_bias64.argtypes = [_P, _P]
        _libs["oracle"] = L
    return _libs["oracle"]


def reference_lib() -> C.CDLL | None:
    """The reference's own kernels compiled for the CPU, if oracle/_ref was
    built here (it exists only where the reference sources are mounted)."""
    if "ref" not in _libs:
        path = os.path.join(_HERE, "_ref", "libref_oracle.so")
        if not os.path.exists(path):
            return None
        L = C.CDLL(path)
        _declare(L, "oref_refk_")
        _libs["ref"] = L
    return _libs["ref"]


class RefOracle:
    """Reference-faithful solver on the CPU (Segmenter's solver path)."""

    BUFFERS = {"phi_read": 0, "phi_write": 1, "export": 2, "tag": 3, "coord": 4, "valid": 5,
               "active": 6, "frozen": 7}

    def __init__(self, volume: np.ndarray, dtype_code: int, z_anisotropy: float = 1.0,
                 quirk_i3: bool = True, use_reference_kernels: bool = False):
        if use_reference_kernels:
            L = reference_lib()
            if L is None:
                raise RuntimeError("oracle/_ref was not built")
            self._pre = "oref_refk_"
        else:
            L = lib()
            self._pre = "oref_"
        self._L = L
        v = np.ascontiguousarray(volume, dtype=_DTYPES[dtype_code])
        nz, ny, nx = v.shape
        self.shape = (nz, ny, nx)
        h = self._f("create")(_ptr(v), nx, ny, nz, dtype_code, z_anisotropy, int(quirk_i3))
        if not h:
            raise ValueError(self._f("last_error")().decode())
        self._h = C.c_void_p(h)
        d = np.zeros(3, np.uint32)
        self._f("padded_dims")(self._h, _ptr(d))
        self.padded = (int(d[2]), int(d[1]), int(d[0]))  # z, y, x

    def _f(self, name):
        return getattr(self._L, self._pre + name)

    def _chk(self, rc):
        if rc != 0:
            raise RuntimeError(self._f("last_error")().decode())

    def close(self):
        if getattr(self, "_h", None):
            self._f("destroy")(self._h)
            self._h = None

    __del__ = close

    def set_params(self, target, window, curvature, time_step, convergence=0.0):
        self._chk(self._f("set_params")(self._h, target, window, curvature, time_step, convergence))

    def initialize_seed(self, cx, cy, cz, r):
        self._chk(self._f("initialize_seed")(self._h, cx, cy, cz, r))

    def set_phi(self, phi: np.ndarray):
        p = np.ascontiguousarray(phi, np.float32)
        self._chk(self._f("set_phi")(self._h, _ptr(p)))

    def step(self, k: int = 1) -> int:
        r = self._f("step")(self._h, k)
        if r < 0:
            raise RuntimeError(self._f("last_error")().decode())
        return r

    @property
    def n(self) -> int:
        return int(self._f("active_count")(self._h))

    @property
    def iterations(self) -> int:
        return int(self._f("iterations")(self._h))

    def finished(self) -> bool:
        return bool(self._f("finished")(self._h))

    def buffer(self, name: str) -> np.ndarray:
        N = self.padded[0] * self.padded[1] * self.padded[2]
        which = self.BUFFERS[name]
        if which in (4, 5):
            out = np.zeros(N, np.uint32)
        elif which == 6:
            out = np.zeros(max(self.n, 1), np.uint32)
        else:
            out = np.zeros(N, np.uint8)
        self._chk(self._f("get_buffer")(self._h, which, _ptr(out)))
        return out[: self.n] if which == 6 else out

    def active(self) -> np.ndarray:
        return self.buffer("active")

    def read_mask(self) -> np.ndarray:
        out = np.zeros(self.shape, np.uint8)
        self._chk(self._f("read_mask")(self._h, _ptr(out)))
        return out

    def read_phi(self) -> np.ndarray:
        out = np.zeros(self.shape, np.float32)
        self._chk(self._f("read_phi")(self._h, _ptr(out)))
        return out

    def read_export(self) -> np.ndarray:
        out = np.zeros(self.shape, np.int8)
        self._chk(self._f("read_export")(self._h, _ptr(out)))
        return out

    def read_active_volume(self) -> np.ndarray:
        out = np.zeros(self.shape, np.uint8)
        self._chk(self._f("read_active_volume")(self._h, _ptr(out)))
        return out

    def freeze(self):
        self._chk(self._f("freeze")(self._h))

    def clear_current(self):
        self._chk(self._f("clear_current")(self._h))

    def clear_all(self):
        self._chk(self._f("clear_all")(self._h))

    def estimate_params(self):
        t = C.c_float()
        w = C.c_float()
        self._chk(self._f("estimate_params")(self._h, C.byref(t), C.byref(w)))
        return t.value, w.value


class NsOracle:
    """FP64 LSS_MODE_NS solver on the CPU (multi-threaded)."""

    def __init__(self, image: np.ndarray, brick=(8, 8, 8), threads: int = 1):
        self._L = lib()
        img = np.ascontiguousarray(image, np.float32)
        self.shape = img.shape
        nz, ny, nx = img.shape
        self._img = img
        self._h = C.c_void_p(self._L.ons_create(nx, ny, nz, _ptr(img), *brick))
        self._L.ons_set_threads(self._h, threads)

    def close(self):
        if getattr(self, "_h", None):
            self._L.ons_destroy(self._h)
            self._h = None

    __del__ = close

    def set_params(self, T, eps, alpha, dt, lo=-4.0, hi=4.0, thr_t=0.01, thr_s=0.0, nbh=26,
                   alpha_data=1, data_literal=0):
        self._L.ons_set_params(self._h, T, eps, alpha, dt, lo, hi, thr_t, thr_s, nbh)
        self._L.ons_set_alpha_role(self._h, int(alpha_data))
        self._L.ons_set_data_term(self._h, int(data_literal))

    def set_threads(self, t: int):
        self._L.ons_set_threads(self._h, t)

    def set_bias(self, bias: np.ndarray | None):
        if bias is None:
            self._L.ons_set_bias(self._h, None)
        else:
            self._bias = np.ascontiguousarray(bias, np.float32)
            self._L.ons_set_bias(self._h, _ptr(self._bias))

    def set_phi(self, phi: np.ndarray):
        p = np.ascontiguousarray(phi, np.float32)
        self._L.ons_set_phi(self._h, _ptr(p))

    def set_state(self, phi: np.ndarray, active_linear: np.ndarray):
        p = np.ascontiguousarray(phi, np.float32)
        a = np.ascontiguousarray(active_linear, np.uint64)
        self._L.ons_set_state(self._h, _ptr(p), _ptr(a), a.size)

    def step(self, k: int = 1) -> int:
        return int(self._L.ons_step(self._h, k))

    def run(self, rel=1e-3, patience=5, max_it=2000, abs_thr=0) -> int:
        return int(self._L.ons_run(self._h, rel, patience, max_it, abs_thr))

    @property
    def n(self) -> int:
        return int(self._L.ons_active_count(self._h))

    @property
    def n0(self) -> int:
        return int(self._L.ons_initial_count(self._h))

    @property
    def updates(self) -> int:
        return int(self._L.ons_updates(self._h))

    def active(self) -> np.ndarray:
        out = np.zeros(max(self.n, 1), np.uint64)
        self._L.ons_read_active(self._h, _ptr(out))
        return out[: self.n]

    def read_phi(self) -> np.ndarray:
        out = np.zeros(self.shape, np.float32)
        self._L.ons_read_phi(self._h, _ptr(out))
        return out

    def read_phi64(self) -> np.ndarray:
        out = np.zeros(self.shape, np.float64)
        self._L.ons_read_phi64(self._h, _ptr(out))
        return out

    def expand_given(self, active_linear, before, after) -> np.ndarray:
        a = np.ascontiguousarray(active_linear, np.uint64)
        b = np.ascontiguousarray(before, np.float32)
        c = np.ascontiguousarray(after, np.float32)
        out = np.zeros(a.size * 27 + 1, np.uint64)
        m = self._L.ons_expand_given(self._h, _ptr(a), a.size, _ptr(b), _ptr(c), _ptr(out))
        return out[:m]

    # ---- FP64 adjoint (ns_adjoint.hpp) ----
    def adjoint(self, K: int, target: np.ndarray, tau: float = 0.5) -> dict:
        """K iterations from the current state with the active sets recorded
        (and kept for adjoint_loss), the soft-Dice loss and its gradients."""
        t = np.ascontiguousarray(target, np.uint8)
        out = np.zeros(4, np.float64)
        db = np.zeros(self.shape, np.float64)
        self._L.ons_adj_run(self._h, K, _ptr(t), tau, _ptr(out), _ptr(db))
        return {"loss": out[0], "d_target": out[1], "d_window": out[2], "d_curvature": out[3],
                "d_bias": db}

    def adjoint_loss(self, K: int, target: np.ndarray, tau: float = 0.5) -> float:
        """The loss of K iterations replaying the active sets of adjoint()."""
        t = np.ascontiguousarray(target, np.uint8)
        return float(self._L.ons_adj_loss(self._h, K, _ptr(t), tau))

    def adjoint_dice(self, K: int, target: np.ndarray, tau: float = 0.5) -> float:
        """The soft-Dice coefficient (1 - loss) of the same replay, computed
        without the subtraction from 1: finite differences of the loss are
        minus those of this value, at ~1000x finer resolution near loss 1."""
        t = np.ascontiguousarray(target, np.uint8)
        return float(self._L.ons_adj_dice(self._h, K, _ptr(t), tau))

    def set_param(self, which: str, value: float):
        self._L.ons_set_param(self._h, {"T": 0, "eps": 1, "alpha": 2}[which], value)

    def set_bias64(self, bias: np.ndarray | None):
        if bias is None:
            self._L.ons_set_bias64(self._h, None)
        else:
            self._bias64 = np.ascontiguousarray(bias, np.float64)
            self._L.ons_set_bias64(self._h, _ptr(self._bias64))
