"""LSS_MODE_NS on the GPU against the FP64 oracle (oracle/ns_model.hpp).

Tolerances (the NS parity criteria):
  * one iteration from an identical state: max |phi_gpu - phi_fp64| <= 1e-4;
  * active lists: bit-exact (order included) given identical phi, i.e. the
    oracle's expansion rule applied to the GPU's own before/after values;
  * after running to the stopping rule: mask disagreement <= 0.01% of voxels
    and Dice >= 0.999 against the FP64 run.
"""
import numpy as np
import pytest

import aworkefficientgpualgorithmforlevelsetsegmentation_gb300 as lss
from aworkefficientgpualgorithmforlevelsetsegmentation_gb300 import phantoms as P
from oracle.oracle import NsOracle
from tests.gpu_util import dice

pytestmark = pytest.mark.gpu

PHI_TOL = 1e-4


# Every instantiated (brick shape, threads per brick); 32 = one warp per brick.
ALL_CONFIGS = [(8, 8, 8, 256), (8, 8, 8, 128), (8, 8, 8, 512), (8, 8, 4, 128), (8, 8, 4, 256),
               (4, 4, 4, 64), (8, 8, 4, 32), (8, 8, 8, 32), (4, 4, 4, 32)]


def make_gpu(cfg, brick=(8, 8, 8), threads=256, **pk):
    s = lss.Segmenter(lss.MODE_NS, brick=brick, threads_per_brick=threads)
    s.load_volume(cfg["image"])
    p = cfg["params"]
    s.set_parameters(p.target, p.window, p.curvature, p.time_step, alpha_role=p.alpha_role, **pk)
    s.set_phi(cfg["phi0"])
    return s


def make_oracle(cfg, brick=(8, 8, 8), nbh=26):
    p = cfg["params"]
    o = NsOracle(cfg["image"], brick=brick, threads=8)
    o.set_params(p.target, p.window, p.curvature, p.time_step, p.phi_min, p.phi_max,
                 p.temporal_threshold, p.spatial_threshold, nbh, p.alpha_role)
    return o


@pytest.mark.parametrize("which,scale,brick,threads", [("config1", 0.5, (8, 8, 8), 256),
                                                      ("config2", 0.25, (8, 8, 8), 256),
                                                      ("config2", 0.25, (8, 8, 4), 128),
                                                      ("config1", 0.5, (4, 4, 4), 64),
                                                      ("config2", 0.25, (8, 8, 4), 32),
                                                      ("config1", 0.5, (4, 4, 4), 32)])
def test_ns_each_iteration_vs_fp64(which, scale, brick, threads):
    cfg = getattr(P, which)(scale)
    s = make_gpu(cfg, brick=brick, threads=threads)
    o = make_oracle(cfg, brick=brick)
    o.set_phi(cfg["phi0"])
    assert np.array_equal(s.active_linear(), o.active()), "initial active set"
    worst = 0.0
    for it in range(40):
        before = s.read_phi()
        act = s.active_linear()
        o.set_state(before, act)
        assert np.array_equal(o.active(), act)
        o.step(1)
        s.step(1)
        after = s.read_phi()
        err = float(np.max(np.abs(after.astype(np.float64) - o.read_phi64())))
        worst = max(worst, err)
        assert err <= PHI_TOL, (it, err)
        flat_b, flat_a = before.ravel(), after.ravel()
        idx = act.astype(np.int64)
        expect = o.expand_given(act, flat_b[idx], flat_a[idx])
        assert np.array_equal(s.active_linear(), expect), it
        if s.n == 0:
            break
    assert worst < PHI_TOL


@pytest.mark.parametrize("which,scale", [("config1", 0.5), ("config2", 0.25)])
def test_ns_converged_mask_vs_fp64(which, scale):
    cfg = getattr(P, which)(scale)
    s = make_gpu(cfg)
    it_g = s.step_until_converged(1e-3, 5, 2000)
    o = make_oracle(cfg)
    o.set_phi(cfg["phi0"])
    it_o = o.run(1e-3, 5, 2000)
    mg = s.get_saveable_segmentation().astype(bool)
    mo = o.read_phi() <= 0
    disagree = float(np.mean(mg != mo))
    assert disagree <= 1e-4, disagree
    assert dice(mg, mo) >= 0.999
    # The stopping rule counts voxels whose |dphi| crosses the temporal
    # threshold; in the tail of the run fp32 and fp64 round a few of them
    # differently, so the iteration of the stop may move by a few percent.
    assert abs(it_g - it_o) <= max(10, 0.05 * it_o), (it_g, it_o)
    st = s.stats()
    assert st["voxel_updates"] > 0 and st["iterations"] == it_g


def test_ns_brick_workers_are_voxel_exact():
    """One block per SM with four brick workers of 256 threads (named
    barriers) gives the same field and list as a block per brick, bit for
    bit, in the one-volume and the batched form."""
    cfg = P.config2(0.25)
    a = make_gpu(cfg, brick=(8, 8, 8), threads=256)
    s = lss.Segmenter(lss.MODE_NS, brick=(8, 8, 8), threads_per_brick=256, brick_workers=4)
    s.load_volume(cfg["image"])
    p = cfg["params"]
    s.set_parameters(p.target, p.window, p.curvature, p.time_step, alpha_role=p.alpha_role)
    s.set_phi(cfg["phi0"])
    assert s.stats()["block_threads"] == 1024
    for k in (1, 7, 30):
        a.step(k)
        s.step(k)
        assert np.array_equal(a.read_phi(), s.read_phi()), k
        assert np.array_equal(a.active_linear(), s.active_linear()), k
    assert a.step_until_converged(1e-3, 5, 2000) == s.step_until_converged(1e-3, 5, 2000)
    assert np.array_equal(a.get_saveable_segmentation(), s.get_saveable_segmentation())
    vols = P.config3(6, scale=0.25)["volumes"]
    out = []
    for workers in (1, 4):
        b = lss.Batch(brick=(8, 8, 8), threads_per_brick=256, brick_workers=workers)
        for v in vols:
            b.add_volume(v["image"], v["params"], v["spheres"])
        it = b.run(1e-3, 5, 2000)
        out.append((it, [b.read_phi(i) for i in range(len(vols))]))
    assert out[0][0] == out[1][0]
    assert all(np.array_equal(x, y) for x, y in zip(out[0][1], out[1][1]))


def test_ns_brick_configs_are_voxel_exact():
    cfg = P.config2(0.25)
    ref_phi = ref_act = None
    for (bx, by, bz, t) in ALL_CONFIGS:
        s = make_gpu(cfg, brick=(bx, by, bz), threads=t)
        s.step(30)
        phi = s.read_phi()
        act = np.sort(s.active_linear())
        if ref_phi is None:
            ref_phi, ref_act = phi, act
        else:
            assert np.array_equal(phi, ref_phi), (bx, by, bz, t)
            assert np.array_equal(act, ref_act), (bx, by, bz, t)
        st = s.stats()
        assert (st["brick_x"], st["brick_y"], st["brick_z"], st["threads_per_brick"]) == (bx, by, bz, t)


def test_ns_six_neighbourhood_vs_fp64():
    cfg = P.config1(0.25)
    s = make_gpu(cfg, neighbourhood=6)
    o = make_oracle(cfg, nbh=6)
    o.set_phi(cfg["phi0"])
    for _ in range(20):
        o.step(1)
        s.step(1)
        assert np.array_equal(s.active_linear(), o.active())
    assert float(np.max(np.abs(s.read_phi() - o.read_phi()))) < 1e-3


def test_ns_ragged_dims_and_alpha_role():
    img = P.ellipsoid((21, 30, 37), (18, 15, 10), (12, 9, 6), 0.7, 0.2, 0.05, 9)
    phi0 = P.sdf_spheres(img.shape, [(18, 15, 10, 3)])
    for role in (lss.ALPHA_DATA, lss.ALPHA_CURVATURE):
        p = P.ns_params(0.7, 0.12, 0.3 if role == lss.ALPHA_CURVATURE else 0.7)
        p.alpha_role = role
        cfg = {"image": img, "phi0": phi0, "params": p}
        s = make_gpu(cfg)
        o = make_oracle(cfg)
        o.set_phi(phi0)
        for _ in range(25):
            before = s.read_phi()
            o.set_state(before, s.active_linear())
            o.step(1)
            s.step(1)
            assert float(np.max(np.abs(s.read_phi() - o.read_phi64()))) <= PHI_TOL


def test_ns_param_change_reinitialises_active_set():
    cfg = P.config1(0.25)
    s = make_gpu(cfg)
    s.step(10)
    phi = s.read_phi()
    s.set_parameters(target=0.65)
    s.step(1)
    o = make_oracle(cfg)
    o._L.ons_set_params(o._h, 0.65, 0.12, 0.9, 0.5, -4.0, 4.0, 0.01, 0.0, 26)
    o.set_phi(phi)  # re-init from the current phi, as the engine does
    o.step(1)
    assert np.array_equal(s.active_linear(), o.active())
    # The step ran with the new target (the precomputed speed follows it).
    assert float(np.max(np.abs(s.read_phi().astype(np.float64) - o.read_phi64()))) <= 1e-4


def test_ns_seeds_and_readbacks():
    cfg = P.config1(0.25)
    s = lss.Segmenter(lss.MODE_NS, brick=(8, 8, 8), threads_per_brick=256)
    s.load_volume(cfg["image"])
    p = cfg["params"]
    s.set_parameters(p.target, p.window, p.curvature, p.time_step)
    s.set_seed_spheres(cfg["spheres"])
    assert np.allclose(s.read_phi(), cfg["phi0"], atol=1e-6)
    n0 = s.get_active_element_count()
    assert n0 == len(s.active_xyz()) > 0
    av = s.read_active_volume()
    assert int((av == 127).sum()) == n0
    s.step(20)
    m = s.get_saveable_segmentation()
    assert np.array_equal(m.astype(bool), s.read_phi() <= 0)
    # Read-backs into caller-owned arrays (reused across calls).
    mb, pb = np.full(m.shape, 7, np.uint8), np.full(m.shape, 9.0, np.float32)
    assert s.get_saveable_segmentation(out=mb) is mb and np.array_equal(mb, m)
    assert s.read_phi(out=pb) is pb and np.array_equal(pb, s.read_phi())
    s.freeze_current_segmentation()
    s.clear_current_segmentation()
    assert s.get_active_element_count() == 0
    assert np.array_equal(s.get_saveable_segmentation(), m)  # the frozen part stays
    s.clear_all_segmentations()
    assert s.get_saveable_segmentation().sum() == 0


def test_ns_estimate_params():
    cfg = P.config1(0.25)
    s = make_gpu(cfg)
    s.step(60)
    t, w = s.calculate_segmentation_parameters()
    img, m = cfg["image"], s.read_phi() <= 0
    assert abs(t - img[m].mean()) < 1e-4
    assert abs(w - img[m].std(ddof=1)) < 1e-4


def test_ns_host_fault_injection(monkeypatch):
    cfg = P.config1(0.25)
    s = make_gpu(cfg)
    monkeypatch.setenv("LSS_FAULT", "timeout")
    with pytest.raises(lss.LssError) as e:
        s.step(2)
    assert e.value.status == 5
    monkeypatch.setenv("LSS_FAULT", "alloc")
    t = lss.Segmenter(lss.MODE_NS)
    with pytest.raises(lss.LssError) as e:
        t.load_volume(cfg["image"])
    assert e.value.status == 8
    monkeypatch.delenv("LSS_FAULT")
    s.step(2)  # the engine stays usable after a reported failure
    t.load_volume(cfg["image"])


def test_ns_hbm_budget_refuses():
    cfg = P.config1(0.25)
    s = lss.Segmenter(lss.MODE_NS, hbm_budget_bytes=64 << 10)  # 32^3 needs > 384 KiB
    with pytest.raises(lss.LssError) as e:
        s.load_volume(cfg["image"])
    assert e.value.status == 9


def test_batch_matches_plain_runs():
    c3 = P.config3(count=5, scale=0.25)
    b = lss.Batch(brick=(8, 8, 8), threads_per_brick=256)
    for v in c3["volumes"]:
        b.add_volume(v["image"], v["params"], v["spheres"])
    b.run(1e-3, 5, 300)
    for i, v in enumerate(c3["volumes"]):
        s = lss.Segmenter(lss.MODE_NS, brick=(8, 8, 8), threads_per_brick=256)
        s.load_volume(v["image"])
        p = v["params"]
        s.set_parameters(p.target, p.window, p.curvature, p.time_step)
        s.set_seed_spheres(v["spheres"])
        it = s.step_until_converged(1e-3, 5, 300)
        st = b.stats(i)
        assert st["iterations"] == it, i
        assert np.array_equal(b.read_phi(i), s.read_phi()), i
        assert np.array_equal(b.read_mask(i), s.get_saveable_segmentation()), i


def test_ns_every_config_uses_both_tma_buffers():
    """Dense mode (negative thresholds: every voxel active) on a volume with
    more bricks than blocks, so every block processes several bricks and both
    TMA buffers are used; all configurations agree bit for bit, and with the
    FP64 oracle within tolerance."""
    img = P.ellipsoid((72, 96, 136), (60, 45, 30), (40, 30, 20), 0.7, 0.2, 0.05, 12)
    phi0 = P.sdf_spheres(img.shape, [(60, 45, 30, 6)])
    p = P.ns_params(0.7, 0.12, 0.9, temporal_threshold=-1.0, spatial_threshold=-1.0)
    cfg = {"image": img, "phi0": phi0, "params": p}
    ref = None
    for (bx, by, bz, t) in ALL_CONFIGS:
        s = make_gpu(cfg, brick=(bx, by, bz), threads=t, temporal_threshold=-1.0,
                     spatial_threshold=-1.0)
        assert s.get_active_element_count() == img.size
        s.step(4)
        phi = s.read_phi()
        if ref is None:
            ref = phi
            o = make_oracle(cfg)
            o._L.ons_set_params(o._h, 0.7, 0.12, 0.9, 0.5, -4.0, 4.0, -1.0, -1.0, 26)
            o.set_phi(phi0)
            o.step(4)
            assert float(np.max(np.abs(phi.astype(np.float64) - o.read_phi64()))) <= 4 * PHI_TOL
        else:
            assert np.array_equal(phi, ref), (bx, by, bz, t)


@pytest.mark.parametrize("shape", [(64, 64, 64), (29, 50, 37)])
def test_dense_pass_equals_all_active_sparse(shape):
    """The dense all-voxel kernel (the baseline of the sparse-vs-dense
    comparison) and the sparse engine with every voxel active compute the same
    field bit for bit, borders (clamp-to-edge) included."""
    cfg = P.config2(0.25)
    img = np.ascontiguousarray(cfg["image"][:shape[0], :shape[1], :shape[2]])
    phi0 = np.ascontiguousarray(cfg["phi0"][:shape[0], :shape[1], :shape[2]])
    sub = dict(cfg, image=img, phi0=phi0)
    a = make_gpu(sub, temporal_threshold=-1.0, spatial_threshold=-1.0)
    b = make_gpu(sub, temporal_threshold=-1.0, spatial_threshold=-1.0)
    a.step(7)
    b.step_dense(7)
    assert np.array_equal(a.read_phi(), b.read_phi())


def test_ns_reload_same_shape_equals_fresh_engine():
    """Loading a new volume of the same shape reuses the engine's buffers;
    the state afterwards is that of a fresh engine: same field, list, mask and
    statistics after seeding and running."""
    a_cfg, b_cfg = P.config1(0.25), P.config2(0.125)
    assert a_cfg["image"].shape == b_cfg["image"].shape
    p = b_cfg["params"]
    s = make_gpu(a_cfg)
    s.step(7)
    s.freeze_current_segmentation()
    s.load_volume(b_cfg["image"])  # same shape: the reload path
    s.set_parameters(p.target, p.window, p.curvature, p.time_step, alpha_role=p.alpha_role)
    fresh = lss.Segmenter(lss.MODE_NS, brick=(8, 8, 8), threads_per_brick=256)
    fresh.load_volume(b_cfg["image"])
    fresh.set_parameters(p.target, p.window, p.curvature, p.time_step, alpha_role=p.alpha_role)
    for e in (s, fresh):
        assert e.get_active_element_count() == 0
        assert np.all(e.get_saveable_segmentation() == 0)
        e.set_seed_spheres(b_cfg["spheres"])
        e.step_until_converged(1e-3, 5, 500)
    assert np.array_equal(s.read_phi(), fresh.read_phi())
    assert np.array_equal(s.active_linear(), fresh.active_linear())
    assert np.array_equal(s.get_saveable_segmentation(), fresh.get_saveable_segmentation())
    assert s.stats()["iterations"] == fresh.stats()["iterations"]
    assert s.stats()["voxel_updates"] == fresh.stats()["voxel_updates"]


def test_ns_freeze_and_clear_on_device():
    """Frozen segmentations stay in the mask after the current one is cleared
    and reseeded elsewhere; clearing all removes them."""
    cfg = P.config1(0.25)
    s = make_gpu(cfg)
    s.step(20)
    m1 = s.get_saveable_segmentation().astype(bool)
    assert m1.any()
    assert np.array_equal(m1, s.read_phi() <= 0)
    s.freeze_current_segmentation()
    s.clear_current_segmentation()
    assert np.array_equal(s.get_saveable_segmentation().astype(bool), m1)
    nz, ny, nx = cfg["image"].shape
    s.set_seed_spheres([(2, 2, 2, 1.5)])
    s.step(3)
    m2 = s.get_saveable_segmentation().astype(bool)
    assert np.array_equal(m2, m1 | (s.read_phi() <= 0))
    s.freeze_current_segmentation()
    s.clear_all_segmentations()
    assert not s.get_saveable_segmentation().any()


def test_ns_pinned_host_buffers_match_pageable():
    """Pinned host buffers are read and written in place by the kernels
    (volume, phi and reload uploads; phi and mask read-backs, with and without
    a frozen segmentation); every result equals the pageable-numpy path, for
    rows of a multiple of four voxels and for odd rows."""
    torch = pytest.importorskip("torch")

    def pinned(a):
        t = torch.empty(a.shape, dtype={np.float32: torch.float32, np.uint8: torch.uint8}[a.dtype.type],
                        pin_memory=True).numpy()
        t[...] = a
        return t

    p = P.ns_params(0.6, 0.2, 0.7)
    for shape in [(40, 48, 64), (29, 50, 37)]:
        rng = np.random.default_rng(shape[2])
        nz, ny, nx = shape
        imgs = [(0.5 + 0.2 * rng.standard_normal(shape)).astype(np.float32) for _ in range(2)]
        phi0 = P.sdf_spheres(shape, [((nx - 1) / 2, (ny - 1) / 2, (nz - 1) / 2, 6.0)])
        a = lss.Segmenter(lss.MODE_NS, brick=(8, 8, 8), threads_per_brick=256)
        b = lss.Segmenter(lss.MODE_NS, brick=(8, 8, 8), threads_per_brick=256)
        for img in imgs:  # the second load is a same-shape reload
            a.load_volume(img)
            b.load_volume(pinned(img))
            for s in (a, b):
                s.set_parameters(p.target, p.window, p.curvature, p.time_step, alpha_role=p.alpha_role)
            a.set_phi(phi0)
            b.set_phi(pinned(phi0))
            a.step(12)
            b.step(12)
            phi_b = b.read_phi(out=pinned(np.zeros(shape, np.float32)))
            assert np.array_equal(a.read_phi(), phi_b)
            mask_b = b.get_saveable_segmentation(out=pinned(np.full(shape, 9, np.uint8)))
            assert np.array_equal(a.get_saveable_segmentation(), mask_b)
            assert np.array_equal(b.get_saveable_segmentation(), mask_b)
        a.freeze_current_segmentation()
        b.freeze_current_segmentation()
        for s in (a, b):
            s.set_phi(np.full(shape, 1.0, np.float32))
        frozen_b = b.get_saveable_segmentation(out=pinned(np.zeros(shape, np.uint8)))
        assert np.array_equal(a.get_saveable_segmentation(), frozen_b) and frozen_b.any()
