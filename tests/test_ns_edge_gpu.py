"""LSS_MODE_NS edge cases and full-size properties on the GPU.

Edge cases: degenerate and flat volumes, an empty active set, zero
iterations, runs split over several calls, status codes of misuse.  Full size
(the 256^3 three-shell workload): properties that need no CPU run of the same
size — every brick configuration gives the same field bit for bit, a run
split over calls equals one call, phi stays in its clamp range, the active
list is sorted brick-major without duplicates, and the converged mask is the
mask of phi <= 0.  One full-size case does run the FP64 oracle to convergence
(about 30 s on 8 host threads): the converged mask against the GPU's.
"""
import os

import numpy as np
import pytest

import aworkefficientgpualgorithmforlevelsetsegmentation_gb300 as lss
from aworkefficientgpualgorithmforlevelsetsegmentation_gb300 import phantoms as P
from oracle.oracle import NsOracle

pytestmark = pytest.mark.gpu

PHI_TOL = 1e-4


def seg(img, p, brick=(8, 8, 8), threads=256):
    s = lss.Segmenter(lss.MODE_NS, brick=brick, threads_per_brick=threads)
    s.load_volume(img)
    s.set_parameters(p.target, p.window, p.curvature, p.time_step, alpha_role=p.alpha_role)
    return s


def oracle(img, p, brick=(8, 8, 8)):
    # Active lists are in brick-major order: the oracle uses the same bricks.
    o = NsOracle(img, brick=brick, threads=8)
    o.set_params(p.target, p.window, p.curvature, p.time_step, alpha_data=p.alpha_role)
    return o


@pytest.mark.parametrize("shape", [(1, 1, 1), (2, 3, 5), (1, 40, 33), (9, 1, 17), (13, 11, 1)])
def test_degenerate_and_flat_volumes_match_fp64(shape):
    rng = np.random.default_rng(sum(shape))
    img = (0.5 + 0.3 * rng.standard_normal(shape)).astype(np.float32)
    nz, ny, nx = shape
    phi0 = P.sdf_spheres(shape, [((nx - 1) / 2, (ny - 1) / 2, (nz - 1) / 2, 1.5)])
    p = P.ns_params(0.6, 0.3, 0.7)
    for brick, threads in [((8, 8, 8), 256), ((4, 4, 4), 32)]:
        s = seg(img, p, brick, threads)
        s.set_phi(phi0)
        o = oracle(img, p, brick)
        o.set_phi(phi0)
        assert np.array_equal(s.active_linear(), o.active())
        for _ in range(6):
            before = s.read_phi()
            o.set_state(before, s.active_linear())
            o.step(1)
            s.step(1)
            assert float(np.max(np.abs(s.read_phi() - o.read_phi64()))) <= PHI_TOL


def test_empty_active_set_and_zero_iterations():
    img = np.full((24, 24, 24), 0.5, np.float32)
    p = P.ns_params(0.5, 0.1, 0.5)
    s = seg(img, p)
    s.set_phi(np.full(img.shape, 4.0, np.float32))  # uniform: nothing active
    assert s.get_active_element_count() == 0
    s.step(0)
    s.step(5)
    assert np.all(s.read_phi() == 4.0) and s.get_active_element_count() == 0
    s.step_until_converged(1e-3, 5, 100)
    assert s.stats()["voxel_updates"] == 0


def test_split_run_equals_one_run():
    cfg = P.config2(0.25)
    p = cfg["params"]
    a, b = seg(cfg["image"], p), seg(cfg["image"], p)
    a.set_seed_spheres(cfg["spheres"])
    b.set_seed_spheres(cfg["spheres"])
    a.step(37)
    for k in (1, 5, 2, 13, 16):
        b.step(k)
    assert np.array_equal(a.read_phi(), b.read_phi())
    assert np.array_equal(a.active_linear(), b.active_linear())


def test_misuse_returns_status_codes():
    s = lss.Segmenter(lss.MODE_NS)
    with pytest.raises(lss.LssError) as e:
        s.step(1)  # no volume
    assert e.value.status == 2  # LSS_ERR_STATE
    s.load_volume(np.zeros((8, 8, 8), np.float32))
    with pytest.raises(lss.LssError) as e:
        s.step(1)  # no seed / phi
    assert e.value.status == 2
    with pytest.raises(lss.LssError) as e:
        s.set_parameters(window=0.0)
    assert e.value.status == 1  # LSS_ERR_INVALID_ARGUMENT
    with pytest.raises(lss.LssError):
        s.load_volume(np.zeros((0, 8, 8), np.float32))


@pytest.fixture(scope="module")
def full():
    return P.config2(1.0)


def test_full_size_configs_agree_and_split_runs_agree(full):
    p = full["params"]
    ref_phi = ref_act = None
    # (4, 4, 4) x 32: one 1024-thread block per SM whose block prefix sum
    # spans 32 warps, over more than 32 x 1024 membership words' worth of bricks.
    for brick, threads in [((8, 8, 8), 256), ((8, 8, 4), 32), ((4, 4, 4), 64), ((8, 8, 8), 512),
                           ((4, 4, 4), 32)]:
        s = seg(full["image"], p, brick, threads)
        s.set_seed_spheres(full["spheres"])
        s.step(60)
        s.step(60)
        phi, act = s.read_phi(), np.sort(s.active_linear())
        if ref_phi is None:
            ref_phi, ref_act = phi, act
            one = seg(full["image"], p, brick, threads)
            one.set_seed_spheres(full["spheres"])
            one.step(120)
            assert np.array_equal(one.read_phi(), phi)
        else:
            assert np.array_equal(phi, ref_phi), (brick, threads)
            assert np.array_equal(act, ref_act), (brick, threads)


def test_full_size_six_neighbourhood_configs_agree(full):
    """The 6-neighbour rule at full size, where blocks take several bricks an
    iteration: the deferred plane dilation (8^3 and 8x8x4 bricks) and the
    direct per-word dilation of 4^3 bricks give the same field and list."""
    p = full["params"]
    ref_phi = ref_act = None
    for brick, threads in [((4, 4, 4), 64), ((8, 8, 8), 256), ((8, 8, 4), 128), ((8, 8, 8), 32)]:
        s = lss.Segmenter(lss.MODE_NS, brick=brick, threads_per_brick=threads)
        s.load_volume(full["image"])
        s.set_parameters(p.target, p.window, p.curvature, p.time_step, alpha_role=p.alpha_role, neighbourhood=6)
        s.set_seed_spheres(full["spheres"])
        s.step(150)
        phi, act = s.read_phi(), np.sort(s.active_linear())
        if ref_phi is None:
            ref_phi, ref_act = phi, act
        else:
            assert np.array_equal(phi, ref_phi), (brick, threads)
            assert np.array_equal(act, ref_act), (brick, threads)


def test_full_size_run_invariants(full):
    p = full["params"]
    s = seg(full["image"], p)
    s.set_seed_spheres(full["spheres"])
    it = s.step_until_converged(1e-3, 5, 2000)
    assert 100 < it < 2000
    phi = s.read_phi()
    assert float(phi.min()) >= p.phi_min and float(phi.max()) <= p.phi_max
    assert np.array_equal(s.get_saveable_segmentation().astype(bool), phi <= 0)
    act = s.active_linear()
    assert np.unique(act).size == act.size
    # Brick-major order: brick index non-decreasing along the list.
    nz, ny, nx = phi.shape
    x, y, z = act % nx, (act // nx) % ny, act // (nx * ny)
    brick = ((z // 8) * (ny // 8) + (y // 8)) * (nx // 8) + (x // 8)
    assert np.all(np.diff(brick) >= 0)
    st = s.stats()
    assert st["iterations"] == it and st["voxel_updates"] > 0
    # The segmentation fills the inner shell region: the seeds are inside it.
    inner = P.shells(phi.shape, [[a for a in ax] for ax in P.SHELL_AXES], P.SHELL_VALUES, 0.0, 4, 32, 2,
                     1.0, 0.0, 3) >= 0.7
    m = phi <= 0
    assert (m & inner).sum() / max(1, inner.sum()) > 0.9


def test_full_size_converged_mask_vs_fp64(full):
    """The 256^3 three-shell workload run to the stopping rule on the GPU (seeded
    through the sphere-union kernel, as the benchmark does) and by the FP64
    oracle (from the same spheres' signed distances): masks disagree on at most
    0.01 % of voxels and Dice >= 0.999."""
    p = full["params"]
    s = seg(full["image"], p)
    s.set_seed_spheres(full["spheres"])
    it_g = s.step_until_converged(1e-3, 5, 2000)
    mg = s.get_saveable_segmentation().astype(bool)
    o = NsOracle(full["image"], brick=(8, 8, 8), threads=os.cpu_count() or 1)
    o.set_params(p.target, p.window, p.curvature, p.time_step, p.phi_min, p.phi_max,
                 p.temporal_threshold, p.spatial_threshold, 26, p.alpha_role)
    o.set_phi(full["phi0"])
    it_o = o.run(1e-3, 5, 2000)
    mo = o.read_phi() <= 0
    assert float(np.mean(mg != mo)) <= 1e-4
    inter = float(np.logical_and(mg, mo).sum())
    assert 2.0 * inter / (mg.sum() + mo.sum()) >= 0.999
    assert abs(it_g - it_o) <= max(10, 0.05 * it_o), (it_g, it_o)
