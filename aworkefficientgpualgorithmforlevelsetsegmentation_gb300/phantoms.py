"""Seeded synthetic workloads standing in for the reference's BrainWeb
volumes (absent from the reference; never reproduced here).  Each function
returns numpy arrays generated by the deterministic C generators of
include/lss_phantom.h (identical bits on x86-64 and aarch64).

  config1  128^3 ellipsoid (semi-axes 40/30/25, 0.7 on 0.2, noise 0.05, seed 1),
           phi0 = signed distance to a radius-5 sphere at the centre;
           T=0.7 eps=0.12 alpha=0.9 dt=0.5, 300 iterations.
  config2  256^3 three nested ellipsoid shells 0.25/0.55/0.8 (semi-axes
           100/110/90, 78/86/70, 52/58/46), boundaries displaced by value noise
           of amplitude 4 voxels (lattice 32, seed 2), Gaussian blur sigma 1,
           noise 0.04 (seed 3); four radius-3 seeds at the centre +-16 voxels
           along x and y; T=0.8 eps=0.1 alpha=0.85 dt=0.5; run until the active
           count stays under 0.1% of the initial count for 5 iterations
           (at most 2000).
  config3  48 single-ellipsoid volumes, each axis drawn from
           {64, 96, 128, 192, 256} (seed 4), semi-axes 20-45% of the axis,
           foreground U(0.6, 0.9), background U(0.1, 0.3), noise 0.05;
           T = foreground, eps=0.1, alpha=0.9; a radius-3 seed at the centre.
  config4  192^3 two shells 0.45/0.75 (noise 0.05), target = the inner
           ellipsoid; T=0.6 eps=0.1 alpha=0.9, K=64, checkpoints every 8.
  config5  512x512x768 three-shell phantom scaled to the box with 16 random
           radius-4 seeds in the inner shell; batch of 8 x 384^3 + 64 x 64^3.
The scale argument shrinks a workload uniformly for tests.

The generators run from _build/libphantom.so (host code only), so making a
workload does not load the solver library.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L

# The defaults lss_params_default(LSS_MODE_NS) fills (tests/test_abi.py checks
# that the two agree); kept here so that making a workload needs no solver
# library.
NS_DEFAULTS = {"target": 0.5, "window": 0.1, "curvature": 0.5, "time_step": 0.5, "phi_min": -4.0,
               "phi_max": 4.0, "temporal_threshold": 0.01, "spatial_threshold": 0.0,
               "convergence_threshold": 0.0, "neighbourhood": 26, "alpha_role": 1, "data_term": 0}


def _p(a):
    return C.c_void_p(a.ctypes.data)


def ellipsoid(shape_zyx, centre_xyz, axes_xyz, fg, bg, noise, seed) -> np.ndarray:
    nz, ny, nx = shape_zyx
    out = np.zeros(shape_zyx, np.float32)
    c = np.asarray(centre_xyz, np.float32)
    a = np.asarray(axes_xyz, np.float32)
    rc = L.load_phantom().lss_phantom_ellipsoid(nx, ny, nz, _p(c), _p(a), fg, bg, noise, seed, _p(out))
    if rc:
        raise L.LssError(rc, "lss_phantom_ellipsoid")
    return out


def shells(shape_zyx, axes_xyz_list, values, bg, disp_amp, lattice, disp_seed, blur, noise,
           noise_seed) -> np.ndarray:
    nz, ny, nx = shape_zyx
    out = np.zeros(shape_zyx, np.float32)
    ax = np.ascontiguousarray(np.asarray(axes_xyz_list, np.float32).ravel())
    vals = np.asarray(values, np.float32)
    rc = L.load_phantom().lss_phantom_shells(nx, ny, nz, len(values), _p(ax), _p(vals), bg, disp_amp,
                                     max(1, int(lattice)), disp_seed, blur, noise, noise_seed, _p(out))
    if rc:
        raise L.LssError(rc, "lss_phantom_shells")
    return out


def sdf_spheres(shape_zyx, spheres_xyzr, lo=-4.0, hi=4.0) -> np.ndarray:
    nz, ny, nx = shape_zyx
    out = np.zeros(shape_zyx, np.float32)
    s = np.ascontiguousarray(np.asarray(spheres_xyzr, np.float32).ravel())
    rc = L.load_phantom().lss_phantom_sdf_spheres(nx, ny, nz, _p(s), len(s) // 4, lo, hi, _p(out))
    if rc:
        raise L.LssError(rc, "lss_phantom_sdf_spheres")
    return out


def uniform(seed: int, index: int) -> float:
    return float(L.load_phantom().lss_phantom_uniform(seed, index))


def ns_params(T, eps, alpha, dt=0.5, **kw):
    """LSS_MODE_NS parameters with alpha weighting the data term."""
    p = L.lss_params(**NS_DEFAULTS)
    p.target, p.window, p.curvature, p.time_step = T, eps, alpha, dt
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def config1(scale: float = 1.0):
    n = max(16, int(round(128 * scale)))
    s = n / 128
    c = (n - 1) / 2
    img = ellipsoid((n, n, n), (c, c, c), (40 * s, 30 * s, 25 * s), 0.7, 0.2, 0.05, 1)
    spheres = [(c, c, c, 5.0)]
    return {"name": f"config1_{n}", "image": img, "spheres": spheres,
            "phi0": sdf_spheres(img.shape, spheres), "params": ns_params(0.7, 0.12, 0.9),
            "iterations": 300}


SHELL_AXES = [(100, 110, 90), (78, 86, 70), (52, 58, 46)]
SHELL_VALUES = [0.25, 0.55, 0.8]


def config2(scale: float = 1.0):
    n = max(32, int(round(256 * scale)))
    s = n / 256
    img = shells((n, n, n), [[a * s for a in ax] for ax in SHELL_AXES], SHELL_VALUES, 0.0, 4 * s,
                 32 * s, 2, 1.0, 0.04, 3)
    c = (n - 1) / 2
    o = 16 * s
    spheres = [(c + o, c, c, 3.0), (c - o, c, c, 3.0), (c, c + o, c, 3.0), (c, c - o, c, 3.0)]
    return {"name": f"config2_{n}", "image": img, "spheres": spheres,
            "phi0": sdf_spheres(img.shape, spheres), "params": ns_params(0.8, 0.1, 0.85),
            "conv": {"rel": 1e-3, "patience": 5, "max_iterations": 2000}}


def config3(count: int = 48, seed: int = 4, scale: float = 1.0):
    sides = [64, 96, 128, 192, 256]
    vols = []
    k = 0
    for i in range(count):
        dims = []
        for _ in range(3):
            dims.append(sides[min(4, int(uniform(seed, k) * 5))])
            k += 1
        nx, ny, nz = [max(16, int(round(d * scale))) for d in dims]
        frac = [0.20 + 0.25 * uniform(seed, k + j) for j in range(3)]
        k += 3
        cen = [(0.4 + 0.2 * uniform(seed, k + j)) * (d - 1) for j, d in enumerate((nx, ny, nz))]
        k += 3
        fg = 0.6 + 0.3 * uniform(seed, k)
        bg = 0.1 + 0.2 * uniform(seed, k + 1)
        k += 2
        axes = [f * d for f, d in zip(frac, (nx, ny, nz))]
        img = ellipsoid((nz, ny, nx), cen, axes, fg, bg, 0.05, 1000 + i)
        vols.append({"image": img, "spheres": [(cen[0], cen[1], cen[2], 3.0)],
                     "params": ns_params(fg, 0.1, 0.9), "axes": axes, "centre": cen})
    return {"name": f"config3_{count}", "volumes": vols,
            "conv": {"rel": 1e-3, "patience": 5, "max_iterations": 2000}}


def config4(scale: float = 1.0):
    n = max(32, int(round(192 * scale)))
    s = n / 192
    outer, inner = (80 * s, 86 * s, 70 * s), (50 * s, 56 * s, 44 * s)
    img = shells((n, n, n), [outer, inner], [0.45, 0.75], 0.0, 0.0, 32, 0, 0.0, 0.05, 5)
    c = (n - 1) / 2
    target = ellipsoid((n, n, n), (c, c, c), inner, 1.0, 0.0, 0.0, 0) > 0.5
    spheres = [(c, c, c, 8.0 * s)]
    return {"name": f"config4_{n}", "image": img, "target": target.astype(np.uint8),
            "spheres": spheres, "phi0": sdf_spheres(img.shape, spheres),
            "params": ns_params(0.6, 0.1, 0.9), "K": 64, "checkpoint_every": 8}


def config5(scale: float = 1.0, seed: int = 6):
    nx, ny, nz = [max(32, int(round(d * scale))) for d in (512, 512, 768)]
    sx, sy, sz = nx / 256, ny / 256, nz / 256
    axes = [(a * sx, b * sy, c * sz) for a, b, c in SHELL_AXES]
    img = shells((nz, ny, nx), axes, SHELL_VALUES, 0.0, 4 * sx, 32 * sx, 2, 1.0, 0.04, 3)
    cx, cy, cz = (nx - 1) / 2, (ny - 1) / 2, (nz - 1) / 2
    spheres = []
    k = 0
    ia = axes[2]
    while len(spheres) < 16:
        u = [2 * uniform(seed, k + j) - 1 for j in range(3)]
        k += 3
        if u[0] ** 2 + u[1] ** 2 + u[2] ** 2 > 0.36:
            continue
        spheres.append((cx + u[0] * ia[0], cy + u[1] * ia[1], cz + u[2] * ia[2], 4.0))
    return {"name": f"config5_{nx}x{ny}x{nz}", "image": img, "spheres": spheres,
            "params": ns_params(0.8, 0.1, 0.85),
            "conv": {"rel": 1e-3, "patience": 5, "max_iterations": 2000}}
