"""Generates tests/golden/ref_cases.npz: the LSS_MODE_REF cases of
tests/ref_cases.py run through the reference's own kernel sources compiled
for the CPU (oracle/_ref; needs the reference sources mounted).  The GPU
parity tests compare the CUDA engine with these fixtures on machines where the
reference is absent.  It first copies the reference's test volumes
(code/gpuseg/bin/data/test/Bucky.raw, 32^3 u8; Hydrogen.raw, 128^3 u8) into
tests/golden/reference_volumes.npz, which the cases read.
Run: python tests/golden/make_golden.py
"""
import hashlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import build as OB  # noqa: E402
from oracle import oracle as O  # noqa: E402
from tests.ref_cases import CASES, LARGE, run_case  # noqa: E402


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()[:32]


def copy_reference_volumes():
    sys.path.insert(0, os.path.join(ROOT, "oracle", "ref_shim"))
    import build_ref  # noqa: E402
    root = build_ref.reference_root()
    data = os.path.join(root, "code", "gpuseg", "bin", "data", "test")
    vols = {"bucky": np.fromfile(os.path.join(data, "Bucky.raw"), np.uint8).reshape(32, 32, 32),
            "hydrogen": np.fromfile(os.path.join(data, "Hydrogen.raw"), np.uint8).reshape(128, 128, 128)}
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_volumes.npz")
    np.savez_compressed(path, **vols)
    print(path, os.path.getsize(path), "bytes")


def main():
    if OB.build_reference() is None:
        raise SystemExit("reference sources not mounted")
    copy_reference_volumes()
    out = {}
    for name in sorted(CASES):
        snaps = run_case(name, lambda v, d: O.RefOracle(v, d, use_reference_kernels=True))
        kinds, ns, hashes = [], [], []
        for s in snaps:
            kinds.append(s[0])
            if s[0] in ("init", "step", "seed"):
                ns.append(s[1])
                hashes.append(digest(s[2]))
            else:
                ns.append(-1)
                hashes.append(digest(s[1]))
        out[name + "/kinds"] = np.array(kinds)
        out[name + "/n"] = np.array(ns, np.int64)
        out[name + "/sha"] = np.array(hashes)
        if name in LARGE:  # the digests above cover them; keep the file small
            continue
        last_list = [s for s in snaps if s[0] in ("init", "step", "seed")][-1][2]
        out[name + "/final_active"] = last_list.astype(np.uint32)
        out[name + "/final_mask"] = np.packbits(snaps[-3][1].ravel())
        out[name + "/final_export"] = snaps[-1][1]
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ref_cases.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
