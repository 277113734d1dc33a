"""Python mirror of the reference's solver object over the C ABI.

`Segmenter` keeps the member names and argument meaning of the reference's
`Segmenter` (code/gpuseg/code/Segmenter.hpp:37-73) in snake case:

    reference                              here
    LoadVolume(volumeDesc)                 load_volume(volume, dtype, z_anisotropy)
    InitializeSeed(seed, sphereSize)       initialize_seed(seed_xyz, sphere_size)
    RequestUpdateSegmentation(dt)          request_update_segmentation(num_sub_steps)
    GetSaveableSegmentation()              get_saveable_segmentation()
    GetActiveElementCount()                get_active_element_count()
    IsSegmentationFinished()               is_segmentation_finished()
    ClearCurrentSegmentation()             clear_current_segmentation()
    ClearAllSegmentations()                clear_all_segmentations()
    FreezeCurrentSegmentation()            freeze_current_segmentation()
    CalculateSegmentationParameters()      calculate_segmentation_parameters()
    growLevel/growWindow/curvatureInfluence/timeStep parameters
                                           set_parameters(...)

Errors raise LssError carrying the lss_status; the reference asserted instead.
Volumes are numpy arrays indexed [z, y, x].
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L

MODE_REF, MODE_NS = 0, 1
ALPHA_CURVATURE, ALPHA_DATA = 0, 1
DATA_NORMALISED, DATA_LITERAL = 0, 1
DTYPES = {np.dtype(np.uint8): 0, np.dtype(np.int8): 1, np.dtype(np.uint16): 2,
          np.dtype(np.int16): 3, np.dtype(np.uint32): 4, np.dtype(np.int32): 5,
          np.dtype(np.float32): 6}


def _ptr(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


def _cuda_ptr(x, shape, dtype, writeable=False):
    """Device address of a CUDA array (any object with __cuda_array_interface__,
    e.g. a torch CUDA tensor) after checking its shape, dtype and C layout, or
    None for anything else (host arrays)."""
    ai = getattr(x, "__cuda_array_interface__", None)
    if ai is None:
        return None
    shape = tuple(shape)
    dt = np.dtype(dtype)
    if tuple(ai["shape"]) != shape or np.dtype(ai["typestr"]) != dt:
        raise ValueError(f"device array must be {dt} of shape {shape}")
    strides = ai.get("strides")
    if strides is not None:
        want = tuple(int(np.prod(shape[i + 1:])) * dt.itemsize for i in range(len(shape)))
        if tuple(strides) != want:
            raise ValueError("device array must be C-contiguous")
    if writeable and ai["data"][1]:
        raise ValueError("device array is read-only")
    return C.c_void_p(ai["data"][0])


def _out(out, shape, dtype) -> np.ndarray:
    """A new zeroed array, or the caller's `out` (e.g. a view of pinned host
    memory reused across calls) after checking its shape, dtype and layout."""
    if out is None:
        return np.zeros(shape, dtype)
    if out.shape != tuple(shape) or out.dtype != np.dtype(dtype) or not out.flags.c_contiguous \
            or not out.flags.writeable:
        raise ValueError(f"out must be a writeable C-contiguous {np.dtype(dtype)} array of shape {tuple(shape)}")
    return out


def config(mode: int = MODE_NS, device: int = 0, brick=(0, 0, 0), threads_per_brick: int = 0,
           quirk_i3: bool = True, use_graph: bool = True, hbm_budget_bytes: int = 0,
           brick_workers: int = 0) -> L.lss_config:
    c = L.lss_config()
    lib = L.load()
    lib.lss_config_default(C.byref(c))
    c.mode, c.device = mode, device
    c.brick_x, c.brick_y, c.brick_z = brick
    c.threads_per_brick = threads_per_brick
    c.ref_quirk_i3 = int(quirk_i3)
    c.use_graph = int(use_graph)
    c.hbm_budget_bytes = hbm_budget_bytes
    c.brick_workers = brick_workers
    return c


def default_params(mode: int) -> L.lss_params:
    p = L.lss_params()
    L.load().lss_params_default(mode, C.byref(p))
    return p


class Segmenter:
    """One volume, one engine (LSS_MODE_REF or LSS_MODE_NS)."""

    def __init__(self, mode: int = MODE_NS, **cfg):
        self._lib = L.load()
        self.mode = mode
        self._cfg = config(mode, **cfg)
        h = C.c_void_p()
        rc = self._lib.lss_create(C.byref(h), C.byref(self._cfg))
        if rc != 0:
            raise L.LssError(rc, "lss_create failed")
        self._h = h
        self.shape: tuple[int, int, int] | None = None
        self.params = default_params(mode)

    # -- plumbing ---------------------------------------------------------
    def _chk(self, rc: int):
        if rc != 0:
            raise L.LssError(rc, self._lib.lss_last_error_string(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            self._lib.lss_destroy(self._h)
            self._h = None

    __del__ = close

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- the solver path (reference members) --------------------------------
    def load_volume(self, volume: np.ndarray, dtype=None, z_anisotropy: float = 1.0):
        v = np.ascontiguousarray(volume if dtype is None else volume.astype(dtype))
        code = DTYPES[v.dtype]
        nz, ny, nx = v.shape
        self._vol = v
        self._chk(self._lib.lss_load_volume(self._h, _ptr(v), nx, ny, nz, code, z_anisotropy))
        self.shape = (nz, ny, nx)

    def load_volume_raw(self, path: str, shape_zyx, dtype, z_anisotropy: float = 1.0):
        nz, ny, nx = shape_zyx
        self._chk(self._lib.lss_load_volume_raw(self._h, path.encode(), nx, ny, nz,
                                                DTYPES[np.dtype(dtype)], z_anisotropy))
        self.shape = (nz, ny, nx)

    def unload_volume(self):
        self._chk(self._lib.lss_unload_volume(self._h))

    def set_parameters(self, target=None, window=None, curvature=None, time_step=None, **extra):
        p = self.params
        if target is not None: p.target = target
        if window is not None: p.window = window
        if curvature is not None: p.curvature = curvature
        if time_step is not None: p.time_step = time_step
        for k, v in extra.items():
            setattr(p, k, v)
        self._chk(self._lib.lss_set_params(self._h, C.byref(p)))

    def initialize_seed(self, seed_xyz, sphere_size: float):
        x, y, z = seed_xyz
        self._chk(self._lib.lss_initialize_seed(self._h, float(x), float(y), float(z),
                                                float(sphere_size)))

    def set_seed_spheres(self, spheres):
        s = np.ascontiguousarray(np.asarray(spheres, np.float32).reshape(-1, 4))
        self._chk(self._lib.lss_set_seed_spheres(self._h, _ptr(s), s.shape[0]))

    def set_phi(self, phi: np.ndarray):
        p = np.ascontiguousarray(phi, np.float32)
        self._chk(self._lib.lss_set_phi(self._h, _ptr(p)))

    def request_update_segmentation(self, num_sub_steps: int = 1) -> int:
        done = C.c_int32()
        self._chk(self._lib.lss_step(self._h, num_sub_steps, C.byref(done)))
        return done.value

    step = request_update_segmentation

    def step_dense(self, n: int) -> float:
        """n dense all-voxel iterations (same arithmetic); returns device ms."""
        ms = C.c_double()
        self._chk(self._lib.lss_step_dense(self._h, n, C.byref(ms)))
        return ms.value

    def step_until_converged(self, rel: float = 1e-3, patience: int = 5, max_iterations: int = 2000,
                             abs_threshold: int = 0) -> int:
        c = L.lss_conv(rel, patience, max_iterations, abs_threshold)
        done = C.c_int32()
        self._chk(self._lib.lss_step_until_converged(self._h, C.byref(c), C.byref(done)))
        return done.value

    def is_segmentation_finished(self) -> bool:
        f = C.c_int32()
        self._chk(self._lib.lss_is_finished(self._h, C.byref(f)))
        return bool(f.value)

    def get_active_element_count(self) -> int:
        n = C.c_uint64()
        self._chk(self._lib.lss_active_count(self._h, C.byref(n)))
        return n.value

    @property
    def n(self) -> int:
        return self.get_active_element_count()

    def active(self) -> np.ndarray:
        """The active list as packed coordinates x | y<<10 | z<<20 (list order)."""
        n = self.get_active_element_count()
        out = np.zeros(max(n, 1), np.uint32)
        m = C.c_uint64()
        self._chk(self._lib.lss_read_active_packed(self._h, _ptr(out), n, C.byref(m)))
        return out[:n]

    def active_xyz(self) -> np.ndarray:
        n = self.get_active_element_count()
        out = np.zeros((max(n, 1), 3), np.uint32)
        m = C.c_uint64()
        self._chk(self._lib.lss_read_active(self._h, _ptr(out), n, C.byref(m)))
        return out[:n]

    def active_linear(self) -> np.ndarray:
        xyz = self.active_xyz().astype(np.uint64)
        nz, ny, nx = self.shape
        return xyz[:, 0] + nx * (xyz[:, 1] + ny * xyz[:, 2])

    def read_phi(self, out=None) -> np.ndarray:
        out = _out(out, self.shape, np.float32)
        self._chk(self._lib.lss_read_phi(self._h, _ptr(out)))
        return out

    def get_saveable_segmentation(self, out=None) -> np.ndarray:
        out = _out(out, self.shape, np.uint8)
        self._chk(self._lib.lss_read_mask(self._h, _ptr(out)))
        return out

    read_mask = get_saveable_segmentation

    def save_segmentation_raw(self, path: str):
        self._chk(self._lib.lss_save_mask_raw(self._h, path.encode()))

    def read_export(self) -> np.ndarray:
        out = np.zeros(self.shape, np.int8)
        self._chk(self._lib.lss_read_export(self._h, _ptr(out)))
        return out

    def read_active_volume(self) -> np.ndarray:
        out = np.zeros(self.shape, np.uint8)
        self._chk(self._lib.lss_read_active_volume(self._h, _ptr(out)))
        return out

    def freeze_current_segmentation(self):
        self._chk(self._lib.lss_freeze_current(self._h))

    def clear_current_segmentation(self):
        self._chk(self._lib.lss_clear_current(self._h))

    def clear_all_segmentations(self):
        self._chk(self._lib.lss_clear_all(self._h))

    def calculate_segmentation_parameters(self):
        t, w = C.c_float(), C.c_float()
        self._chk(self._lib.lss_estimate_params(self._h, C.byref(t), C.byref(w)))
        self.params.target, self.params.window = t.value, w.value
        return t.value, w.value

    def stats(self) -> dict:
        s = L.lss_stats()
        self._chk(self._lib.lss_get_stats(self._h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in L.lss_stats._fields_}

    def adjoint(self, K: int, checkpoint_every: int, target_mask, sigmoid_scale: float = 0.5,
                bias=None, want_dbias: bool = True, d_bias_out=None):
        """lss_adjoint_run.  target_mask, bias and d_bias_out are host arrays or
        CUDA arrays (device memory is used in place); d_bias_out, when given,
        receives the bias gradient and is returned as "d_bias"."""
        keep = []

        def arg(x, dtype, writeable=False):
            p = _cuda_ptr(x, self.shape, dtype, writeable)
            if p is not None:
                return p
            a = np.ascontiguousarray(x, dtype) if not writeable else _out(x, self.shape, dtype)
            keep.append(a)
            return _ptr(a)

        t = arg(target_mask, np.uint8)
        b = None if bias is None else arg(bias, np.float32)
        db, dbp = None, None
        if want_dbias:
            if d_bias_out is not None and _cuda_ptr(d_bias_out, self.shape, np.float32, True) is not None:
                db, dbp = d_bias_out, _cuda_ptr(d_bias_out, self.shape, np.float32, True)
            else:
                db = _out(d_bias_out, self.shape, np.float32)
                dbp = _ptr(db)
        g = L.lss_grads()
        self._chk(self._lib.lss_adjoint_run(self._h, K, checkpoint_every, t, sigmoid_scale, b, dbp, C.byref(g)))
        return {"loss": g.loss, "d_target": g.d_target, "d_window": g.d_window,
                "d_curvature": g.d_curvature, "d_bias": db,
                "active_voxel_iterations": g.active_voxel_iterations}


class Batch:
    """The batched form: many f32 volumes, one persistent launch."""

    def __init__(self, **cfg):
        self._lib = L.load()
        c = config(MODE_NS, **cfg)
        h = C.c_void_p()
        rc = self._lib.lss_batch_create(C.byref(h), C.byref(c))
        if rc != 0:
            raise L.LssError(rc, "lss_batch_create failed")
        self._h = h
        self.shapes: list[tuple[int, int, int]] = []

    def _chk(self, rc):
        if rc != 0:
            raise L.LssError(rc, self._lib.lss_batch_last_error_string(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            self._lib.lss_batch_destroy(self._h)
            self._h = None

    __del__ = close

    def add_volume(self, image: np.ndarray, params: L.lss_params, spheres) -> int:
        v = np.ascontiguousarray(image, np.float32)
        s = np.ascontiguousarray(np.asarray(spheres, np.float32).reshape(-1, 4))
        nz, ny, nx = v.shape
        idx = C.c_int32()
        self._chk(self._lib.lss_batch_add_volume(self._h, _ptr(v), nx, ny, nz, C.byref(params),
                                                 _ptr(s), s.shape[0], C.byref(idx)))
        self.shapes.append((nz, ny, nx))
        return idx.value

    def run(self, rel=1e-3, patience=5, max_iterations=2000, abs_threshold=0) -> int:
        c = L.lss_conv(rel, patience, max_iterations, abs_threshold)
        it = C.c_int32()
        self._chk(self._lib.lss_batch_run(self._h, C.byref(c), C.byref(it)))
        return it.value

    def read_phi(self, i: int, out=None) -> np.ndarray:
        out = _out(out, self.shapes[i], np.float32)
        self._chk(self._lib.lss_batch_read_phi(self._h, i, _ptr(out)))
        return out

    def read_mask(self, i: int, out=None) -> np.ndarray:
        out = _out(out, self.shapes[i], np.uint8)
        self._chk(self._lib.lss_batch_read_mask(self._h, i, _ptr(out)))
        return out

    def stats(self, i: int) -> dict:
        s = L.lss_stats()
        self._chk(self._lib.lss_batch_get_stats(self._h, i, C.byref(s)))
        return {k: getattr(s, k) for k, _ in L.lss_stats._fields_}
