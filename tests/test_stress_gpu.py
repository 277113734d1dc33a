"""The large workloads at their stated sizes.

  * Config 5, the 512x512x768 three-shell phantom with 16 radius-4 seeds
    (the `bench.py --workload stress` plain run), to the stopping rule on
    the GPU and by the FP64 oracle: masks disagree on at most 0.01 % of
    voxels, Dice >= 0.999, iteration counts within 5 %.
  * A field past 2^31 bytes: a 1024x1024x656 f32 volume (2.75 GB a field)
    holding one textured ellipsoid in a 128^3 box that lies wholly at byte
    offsets above 2^31, run 48 iterations; the same box as a 128^3 volume
    gives the same phi and mask bit for bit (the update, the active set and
    the seeding are local, so only the index arithmetic differs).
  * The mixed stress batch (8 volumes of 384^3 and 64 of 64^3 in one
    persistent launch under a 150 GB HBM budget): every volume's phi and
    mask equal its own plain run (the 8 copies of the 384^3 volume through
    one plain run)."""
import os

import numpy as np
import pytest

import aworkefficientgpualgorithmforlevelsetsegmentation_gb300 as lss
from aworkefficientgpualgorithmforlevelsetsegmentation_gb300 import phantoms as P
from oracle.oracle import NsOracle

pytestmark = pytest.mark.gpu


def seg(img, p, brick=(8, 8, 8), threads=256):
    s = lss.Segmenter(lss.MODE_NS, brick=brick, threads_per_brick=threads)
    s.load_volume(img)
    s.set_parameters(p.target, p.window, p.curvature, p.time_step, alpha_role=p.alpha_role)
    return s


def test_config5_full_size_mask_vs_fp64():
    cfg = P.config5(1.0)
    img, p, conv = cfg["image"], cfg["params"], cfg["conv"]
    assert img.shape == (768, 512, 512)
    s = seg(img, p)
    s.set_seed_spheres(cfg["spheres"])
    it_g = s.step_until_converged(conv["rel"], conv["patience"], conv["max_iterations"])
    mg = s.get_saveable_segmentation().astype(bool)
    del s
    o = NsOracle(img, brick=(8, 8, 8), threads=os.cpu_count() or 1)
    o.set_params(p.target, p.window, p.curvature, p.time_step, p.phi_min, p.phi_max,
                 p.temporal_threshold, p.spatial_threshold, 26, p.alpha_role)
    o.set_phi(P.sdf_spheres(img.shape, cfg["spheres"]))
    it_o = o.run(conv["rel"], conv["patience"], conv["max_iterations"])
    mo = o.read_phi() <= 0
    assert mo.sum() > 10**6
    assert float(np.mean(mg != mo)) <= 1e-4
    inter = float(np.logical_and(mg, mo).sum())
    assert 2.0 * inter / (mg.sum() + mo.sum()) >= 0.999
    assert abs(it_g - it_o) <= max(10, 0.05 * it_o), (it_g, it_o)


def test_field_past_2_31_bytes_matches_small_volume():
    nx, ny, nz, m = 1024, 1024, 656, 128
    x0, y0, z0 = 836, 836, 520  # the box; its first voxel lies at byte 2.18e9
    assert 4 * ((z0 * ny + y0) * nx + x0) > 2**31
    block = P.ellipsoid((m, m, m), (64.0, 64.0, 64.0), (22.0, 17.0, 13.0), 0.8, 0.2, 0.05, 77)
    big = np.full((nz, ny, nx), 0.2, np.float32)
    big[z0:z0 + m, y0:y0 + m, x0:x0 + m] = block
    p = P.ns_params(0.8, 0.1, 0.85)
    steps = 48
    sb = seg(big, p)
    sb.set_seed_spheres([(x0 + 64.0, y0 + 64.0, z0 + 64.0, 5.0)])
    sb.step(steps)
    crop = (slice(z0, z0 + m), slice(y0, y0 + m), slice(x0, x0 + m))
    phi_b = sb.read_phi()[crop].copy()
    mask_b = sb.get_saveable_segmentation()[crop].copy()
    nb_updates = sb.stats()["voxel_updates"]
    del sb, big
    ss = seg(block, p)
    ss.set_seed_spheres([(64.0, 64.0, 64.0, 5.0)])
    ss.step(steps)
    assert ss.stats()["voxel_updates"] == nb_updates > 0
    assert np.array_equal(ss.read_phi(), phi_b)
    mask_s = ss.get_saveable_segmentation()
    assert np.array_equal(mask_s, mask_b)
    assert 1000 < int(mask_s.sum()) < m**3 // 4


def test_stress_batch_matches_plain_runs():
    big = P.config2(1.5)
    vols = [(big["image"], big["params"], big["spheres"]) for _ in range(8)]
    rng = np.random.default_rng(9)
    m = 64
    for i in range(64):
        c = (m - 1) / 2 + rng.uniform(-0.1, 0.1, 3) * m
        axes = rng.uniform(0.2, 0.4, 3) * m
        fg, bg = rng.uniform(0.6, 0.9), rng.uniform(0.1, 0.3)
        img = P.ellipsoid((m, m, m), tuple(c), tuple(axes), fg, bg, 0.05, 2000 + i)
        vols.append((img, P.ns_params(fg, 0.1, 0.9), [(c[0], c[1], c[2], 3.0)]))
    rel, patience, cap = 1e-3, 5, 2000
    b = lss.Batch(brick=(8, 8, 8), threads_per_brick=256, hbm_budget_bytes=150 << 30)
    for img, prm, sp in vols:
        b.add_volume(img, prm, sp)
    b.run(rel, patience, cap)
    assert b.stats(0)["device_bytes"] < 150 << 30

    def plain(img, prm, sp):
        s = lss.Segmenter(lss.MODE_NS, brick=(8, 8, 8), threads_per_brick=256)
        s.load_volume(img)
        s.set_parameters(prm.target, prm.window, prm.curvature, prm.time_step, alpha_role=prm.alpha_role)
        s.set_seed_spheres(sp)
        it = s.step_until_converged(rel, patience, cap)
        return it, s.read_phi(), s.get_saveable_segmentation()

    it, phi, mask = plain(*vols[0])
    for i in range(8):
        assert b.stats(i)["iterations"] == it, i
        assert np.array_equal(b.read_phi(i), phi), i
        assert np.array_equal(b.read_mask(i), mask), i
    for i in range(8, len(vols)):
        it, phi, mask = plain(*vols[i])
        assert b.stats(i)["iterations"] == it, i
        assert np.array_equal(b.read_phi(i), phi), i
        assert np.array_equal(b.read_mask(i), mask), i
