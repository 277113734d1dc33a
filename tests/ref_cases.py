"""Deterministic LSS_MODE_REF cases shared by the oracle pin, the golden
fixtures and the GPU parity tests.

Each case is an integer volume, the reference's parameters, seeds and a step
schedule.  Volumes are either small blobs drawn from numpy's PCG64 (identical
on every platform) or one of the reference's own test volumes
(code/gpuseg/bin/data/test/Bucky.raw, 32^3 u8, and Hydrogen.raw, 128^3 u8),
copied into tests/golden/reference_volumes.npz by tests/golden/make_golden.py.
A schedule entry is an int (substeps of one RequestUpdateSegmentation call)
or an action tuple: ("params", T, eps, alpha, dt), ("seed", x, y, z, r),
("mask",) (a readback, which clears the tag volume as the reference does),
("freeze",), ("clear",).
"""
from __future__ import annotations

import os

import numpy as np

VOLUMES = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_volumes.npz")

DT = {"u8": (0, np.uint8), "s8": (1, np.int8), "u16": (2, np.uint16), "s16": (3, np.int16),
      "u32": (4, np.uint32), "s32": (5, np.int32)}


def blob_volume(shape, dtype, lo, hi, centre_val, radius, seed):
    """A bright ball of value ~centre_val on a noisy background."""
    rng = np.random.default_rng(seed)
    nz, ny, nx = shape
    z, y, x = np.mgrid[0:nz, 0:ny, 0:nx]
    c = np.array(shape) / 2.0
    r = np.sqrt((z - c[0]) ** 2 + (y - c[1]) ** 2 + ((x - c[2]) * 0.8) ** 2)
    v = rng.integers(lo, hi, size=shape)
    inside = r < radius
    v[inside] = centre_val + rng.integers(-8, 9, size=int(inside.sum()))
    return v.astype(DT[dtype][1])


CASES = {
    # name: (shape zyx, dtype, volume args, params (T, eps, alpha, dt), seeds, schedule)
    "ball_u8": ((32, 32, 32), "u8", (10, 60, 140, 9, 1), (140, 40, 0.16, 0.25),
                [(16, 16, 16, 3)], [1] * 12 + [5] * 6),
    "ragged_s16": ((20, 27, 33), "s16", (-400, -200, 300, 7, 2), (300, 60, 0.2, 0.3),
                   [(16, 13, 10, 3)], [1] * 8 + [6] * 4),
    "two_seeds_u16": ((32, 48, 40), "u16", (100, 900, 2000, 10, 3), (2000, 150, 0.1, 0.27),
                      [(12, 20, 16, 2), (26, 28, 16, 3)], [2] * 10),
    "many_active_s8": ((16, 16, 32), "s8", (-100, -20, 80, 12, 4), (80, 50, 0.3, 0.25),
                       [(16, 8, 8, 9)], [1] * 10 + [4] * 3),
    "param_change_u8": ((32, 32, 32), "u8", (0, 80, 150, 10, 5), (150, 40, 0.2, 0.25),
                        [(16, 16, 16, 4)], [3, 3, ("params", 150, 60, 0.25, 0.25), 1, 3, 3,
                                           ("mask",), 4, 4]),
    "negative_dt_s32": ((16, 32, 16), "s32", (0, 500, 1000, 6, 6), (1000, 300, 0.1, -0.2),
                        [(8, 16, 8, 4)], [2] * 6),
    "freeze_u32": ((16, 16, 16), "u32", (0, 50, 120, 5, 7), (120, 30, 0.15, 0.25),
                   [(8, 8, 8, 3)], [4, 4, ("freeze",), ("clear",), ("seed", 5, 5, 5, 2), 3, 3]),
    "no_curvature_u8": ((24, 24, 24), "u8", (0, 40, 100, 8, 8), (100, 50, 0.0, 0.5),
                        [(12, 12, 12, 3)], [1] * 10),
    # The reference's test volumes.  Bucky.raw with the parameters of
    # code/gpuseg/bin/parameters/Bucky.par (growLevel 140, growWindow 80,
    # curvatureInfluence 0.16, timeStep 0.253333, numSubSteps 15), seeded in a
    # bright lobe of the shell.
    "bucky_par": ((32, 32, 32), "u8", "bucky", (140, 80, 0.16, 0.253333),
                  [(16, 4, 16, 3)], [15] * 20 + [("mask",)] + [15] * 4),
    # Hydrogen.raw seeded with the REPRODUCIBLE_SEED constants of
    # Segmenter.cpp:507-513 (64, 88, 98, radius 15), growing through the dim
    # region around the orbital (T 0, window 12): large active sets, the
    # many-active path.
    "hydrogen_seed_u8": ((128, 128, 128), "u8", "hydrogen", (0, 12, 0.16, 0.25),
                         [(64, 88, 98, 15)], [15] * 10),
    # Hydrogen.raw seeded in the orbital's bright core, growing outwards.
    "hydrogen_core_u8": ((128, 128, 128), "u8", "hydrogen", (40, 40, 0.16, 0.25),
                         [(64, 64, 62, 4)], [15] * 8),
}

# Cases on the reference's 128^3 test volume: the slowest for the reference
# kernels compiled for the CPU.
LARGE = ("hydrogen_seed_u8", "hydrogen_core_u8")


def reference_volume(which: str) -> np.ndarray:
    with np.load(VOLUMES) as z:
        return np.ascontiguousarray(z[which])


def make_volume(name):
    shape, dt, va, *_ = CASES[name]
    if isinstance(va, str):
        v = reference_volume(va)
        assert v.shape == shape and v.dtype == DT[dt][1]
        return v
    return blob_volume(shape, dt, *va)


def run_case(name, make, ops_log=None):
    """Runs a case on any object with the RefOracle-like interface returned by
    make(volume, dtype_code); returns the snapshot list."""
    shape, dt, va, params, seeds, schedule = CASES[name]
    vol = make_volume(name)
    o = make(vol, DT[dt][0])
    o.set_params(*params)
    for s in seeds:
        o.initialize_seed(*s)
    snaps = [("init", o.n, o.active().copy())]
    for item in schedule:
        if isinstance(item, int):
            o.step(item)
            snaps.append(("step", o.n, o.active().copy()))
        elif item[0] == "params":
            o.set_params(*item[1:])
        elif item[0] == "seed":
            o.initialize_seed(*item[1:])
            snaps.append(("seed", o.n, o.active().copy()))
        elif item[0] == "mask":
            snaps.append(("mask", o.read_mask().copy()))
        elif item[0] == "freeze":
            o.freeze()
        elif item[0] == "clear":
            o.clear_current()
    snaps.append(("final_mask", o.read_mask().copy()))
    snaps.append(("final_phi", o.read_phi().copy()))
    snaps.append(("final_export", o.read_export().copy()))
    return snaps
