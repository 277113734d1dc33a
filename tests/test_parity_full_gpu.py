"""Parity at the workloads' full stated sizes.

  * LSS_MODE_REF at 256^3 (the `bench.py --workload ref` case): every
    iteration's active count and the active-list, mask, phi and export
    digests against fixtures made on the CPU by the reference's own kernel
    sources (tests/golden/make_golden_ref256.py), for a fresh run and for a
    rerun after ClearCurrentSegmentation; and lss_step_until_converged stops
    at the same iteration with the same state.  Bit for bit.
  * LSS_MODE_NS at 256^3 (the headline workload): per-iteration phi within
    1e-4 max-abs of the FP64 oracle started from the GPU's own state, and the
    active list bit-exact given identical phi, over windows of iterations
    spread across the whole run to convergence.
  * The batched form on the 48 mixed-size volumes: every volume's final mask
    against the FP64 oracle run to the same stopping rule (at most 0.01 % of
    voxels disagree, Dice >= 0.999).
"""
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

import aworkefficientgpualgorithmforlevelsetsegmentation_gb300 as lss
from aworkefficientgpualgorithmforlevelsetsegmentation_gb300 import phantoms as P
from oracle.oracle import NsOracle
from tests.golden import make_golden_ref256 as R256
from tests.gpu_util import RefGpu, dice

pytestmark = pytest.mark.gpu

PHI_TOL = 1e-4
GOLD256 = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_config2_256.npz")


class _RefGpu256(RefGpu):
    def clear_current(self):
        self.s.clear_current_segmentation()


def test_ref_256_matches_reference_kernels_every_iteration():
    gold = np.load(GOLD256)
    u8, spheres = R256.workload()
    g = _RefGpu256(u8, 0)
    runs = R256.run(g, spheres)
    for tag, (counts, snaps, final) in zip(("fresh", "rerun"), runs):
        want = gold[tag + "/counts"]
        assert counts.size == want.size, (tag, counts.size, want.size)
        bad = np.flatnonzero(counts != want)
        assert bad.size == 0, (tag, "first differing iteration", int(bad[0]) if bad.size else None)
        its = gold[tag + "/snap_iterations"]
        assert sorted(snaps) == list(its), tag
        for i, h in zip(its, gold[tag + "/snap_sha"]):
            assert snaps[int(i)] == h, (tag, int(i))
        assert [final["mask"], final["phi"], final["export"]] == list(gold[tag + "/final_sha"]), tag
        assert final["mask_voxels"] == int(gold[tag + "/mask_voxels"])
    # The stopping rule on the device: the same iteration, the same state.
    c = _RefGpu256(u8, 0)
    c.set_params(*R256.PARAMS)
    for (x, y, z, r) in spheres:
        c.initialize_seed(x, y, z, r)
    it = c.s.step_until_converged(R256.REL, R256.PATIENCE, R256.MAX_IT)
    assert it == gold["fresh/counts"].size - 1
    assert R256.digest(c.active()) == gold["fresh/snap_sha"][-1]
    assert R256.digest(c.read_mask()) == gold["fresh/final_sha"][0]


@pytest.fixture(scope="module")
def full():
    return P.config2(1.0)


def test_ns_256_per_iteration_vs_fp64(full):
    """Windows of three iterations at the start, the widening front, the peak
    and the tail of the 256^3 run (seeded by the sphere-union kernel, as the
    benchmark does): each iteration from the GPU's state, the oracle's FP64
    update within 1e-4 and its expansion rule on the GPU's own values equal
    to the GPU's next list (order included)."""
    p = full["params"]
    s = lss.Segmenter(lss.MODE_NS, brick=(8, 8, 8), threads_per_brick=256)
    s.load_volume(full["image"])
    s.set_parameters(p.target, p.window, p.curvature, p.time_step, alpha_role=p.alpha_role)
    s.set_seed_spheres(full["spheres"])
    o = NsOracle(full["image"], brick=(8, 8, 8), threads=os.cpu_count() or 1)
    o.set_params(p.target, p.window, p.curvature, p.time_step, p.phi_min, p.phi_max,
                 p.temporal_threshold, p.spatial_threshold, 26, p.alpha_role)
    done, worst, checked = 0, 0.0, 0
    for start in (0, 40, 150, 260, 380, 425):
        s.step(start - done)
        done = start
        for _ in range(3):
            before = s.read_phi()
            act = s.active_linear()
            if act.size == 0:
                break
            o.set_state(before, act)
            assert np.array_equal(o.active(), act), done
            o.step(1)
            s.step(1)
            done += 1
            after = s.read_phi()
            err = float(np.max(np.abs(after.astype(np.float64) - o.read_phi64())))
            worst = max(worst, err)
            assert err <= PHI_TOL, (done, err)
            idx = act.astype(np.int64)
            expect = o.expand_given(act, before.ravel()[idx], after.ravel()[idx])
            assert np.array_equal(s.active_linear(), expect), done
            checked += 1
    assert checked >= 15 and worst <= PHI_TOL


def _oracle_run(v, conv):
    p = v["params"]
    o = NsOracle(v["image"], brick=(8, 8, 8), threads=4)
    o.set_params(p.target, p.window, p.curvature, p.time_step, p.phi_min, p.phi_max,
                 p.temporal_threshold, p.spatial_threshold, 26, p.alpha_role)
    o.set_phi(P.sdf_spheres(v["image"].shape, v["spheres"]))
    it = o.run(conv["rel"], conv["patience"], conv["max_iterations"])
    mask = o.read_phi() <= 0
    o.close()
    return it, mask


def test_batch_48_volumes_masks_vs_fp64():
    """The 48-volume batch (158 M voxels) in one persistent launch with the
    autotuned brick configuration, as the benchmark runs it; the FP64 oracle
    runs each volume on the host (several volumes at a time)."""
    cfg = P.config3(48)
    vols, conv = cfg["volumes"], cfg["conv"]
    b = lss.Batch(brick=(0, 0, 0), threads_per_brick=0)
    for v in vols:
        b.add_volume(v["image"], v["params"], v["spheres"])
    b.run(conv["rel"], conv["patience"], conv["max_iterations"])
    gpu = [(b.stats(i)["iterations"], b.read_mask(i).astype(bool)) for i in range(len(vols))]
    workers = max(1, (os.cpu_count() or 4) // 4)
    order = sorted(range(len(vols)), key=lambda i: -vols[i]["image"].size)  # longest first
    with ThreadPoolExecutor(workers) as ex:
        res = dict(zip(order, ex.map(lambda i: _oracle_run(vols[i], conv), order)))
    rows, total_dis, total_vox = [], 0, 0
    for i, (it_g, mg) in enumerate(gpu):
        it_o, mo = res[i]
        dis = int(np.count_nonzero(mg != mo))
        total_dis += dis
        total_vox += mg.size
        rows.append((i, mg.shape, it_g, it_o, dis / mg.size, dice(mg, mo)))
    table = "\n".join(f"{r[0]:2d} {r[1]} it {r[2]}/{r[3]} disagree {r[4]:.2e} dice {r[5]:.6f}" for r in rows)
    assert total_dis / total_vox <= 1e-4, table
    assert all(r[4] <= 1e-4 for r in rows), table
    assert all(r[5] >= 0.999 for r in rows), table
    # The stopping rule counts voxels whose |dphi| crosses the temporal
    # threshold; in the tail of a run fp32 and fp64 round a few of them
    # differently, so the stop may move by some iterations while the mask
    # no longer changes (measured: at most 32 of 521 iterations).
    assert all(abs(r[2] - r[3]) <= max(10, 0.1 * r[3]) for r in rows), table
