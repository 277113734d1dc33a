"""LSS_MODE_REF on the GPU against the reference: bit for bit.

Each case of tests/ref_cases.py runs through the C ABI and is compared with
(1) the committed golden fixtures generated from the reference's own kernel
sources and (2) the restated CPU oracle, on every snapshot: active list
(order included), count, masks, phi and export volume."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_util import RefGpu
from tests.ref_cases import CASES, DT, make_volume, run_case
from tests.test_oracle_golden import check_against_golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("graph", [True, False])
@pytest.mark.parametrize("name", sorted(CASES))
def test_ref_case_matches_golden_and_oracle(name, graph):
    gpu = run_case(name, lambda v, d: RefGpu(v, d, use_graph=graph))
    check_against_golden(name, gpu)
    cpu = run_case(name, lambda v, d: O.RefOracle(v, d))
    assert len(gpu) == len(cpu)
    for g, c in zip(gpu, cpu):
        assert g[0] == c[0]
        for u, v in zip(g[1:], c[1:]):
            assert np.array_equal(np.asarray(u), np.asarray(v)), g[0]


def test_ref_without_quirk_matches_oracle():
    vol = make_volume("ball_u8")
    g = RefGpu(vol, 0, quirk_i3=False)
    c = O.RefOracle(vol, 0, quirk_i3=False)
    for o in (g, c):
        o.set_params(140, 40, 0.16, 0.25)
        o.initialize_seed(16, 16, 16, 3)
    for _ in range(15):
        g.step(1)
        c.step(1)
        assert np.array_equal(g.active(), c.active())
    assert np.array_equal(g.read_phi(), c.read_phi())


def test_ref_long_run_and_active_volume():
    vol = make_volume("two_seeds_u16")
    g = RefGpu(vol, 2)
    c = O.RefOracle(vol, 2)
    for o in (g, c):
        o.set_params(2000, 150, 0.1, 0.27)
        o.initialize_seed(12, 20, 16, 2)
    for k in (1, 7, 30, 60):
        g.step(k)
        c.step(k)
        assert g.n == c.n
        assert np.array_equal(g.active(), c.active())
        assert np.array_equal(g.read_active_volume(), c.read_active_volume())
    assert np.array_equal(g.read_mask(), c.read_mask())


def test_ref_estimate_params_close_to_reference():
    vol = make_volume("ball_u8")
    g = RefGpu(vol, 0)
    c = O.RefOracle(vol, 0)
    for o in (g, c):
        o.set_params(140, 40, 0.16, 0.25)
        o.initialize_seed(16, 16, 16, 3)
        o.step(10)
    tg, wg = g.estimate_params()
    tc, wc = c.estimate_params()
    # the reference sums in float, sequentially; the device reduction in double
    assert abs(tg - tc) <= 1e-4 * max(1.0, abs(tc))
    assert abs(wg - wc) <= 1e-3 * max(1.0, abs(wc))


def test_ref_finished_rule_and_errors():
    import aworkefficientgpualgorithmforlevelsetsegmentation_gb300 as lss
    s = lss.Segmenter(lss.MODE_REF)
    with pytest.raises(lss.LssError):
        s.request_update_segmentation(1)  # no volume
    with pytest.raises(lss.LssError):
        s.load_volume(np.zeros((8, 8, 8), np.float32))  # REF takes integer voxels
    with pytest.raises(lss.LssError):
        s.load_volume(np.zeros((8, 8, 1100), np.uint8))  # > 1024 after padding
    s.load_volume(make_volume("ball_u8"))
    s.set_parameters(140, 40, 0.16, 0.25, convergence_threshold=1e9)
    s.initialize_seed((16, 16, 16), 3)
    assert not s.is_segmentation_finished()
    assert s.request_update_segmentation(510) == 510
    assert s.is_segmentation_finished()
    assert s.request_update_segmentation(5) == 0  # finished: RequestUpdateSegmentation does nothing


@pytest.mark.parametrize("use_graph", [True, False])
def test_ref_run_to_convergence_stops_where_the_rule_says(use_graph):
    """The stopping rule of a run to convergence is evaluated on the device
    after every iteration and read back once per chunk of launched
    iterations; iterations launched after it stopped must change nothing.
    The run stops at the iteration the rule, applied to the oracle's count
    after every single iteration, names, with the oracle's state; a cap below
    that runs exactly the cap."""
    import aworkefficientgpualgorithmforlevelsetsegmentation_gb300 as lss
    from aworkefficientgpualgorithmforlevelsetsegmentation_gb300 import phantoms as P

    cfg = P.config2(0.25)
    vol = np.clip(np.rint(cfg["image"] * 255.0), 0, 255).astype(np.uint8)
    rel, patience = 1e-3, 5

    def gpu():
        s = lss.Segmenter(lss.MODE_REF, use_graph=use_graph)
        s.load_volume(vol)
        s.set_parameters(204, 26, 0.1, 0.25)
        for (x, y, z, r) in cfg["spheres"]:
            s.initialize_seed((x, y, z), r)
        return s

    c = O.RefOracle(vol, 0)
    c.set_params(204, 26, 0.1, 0.25)
    for (x, y, z, r) in cfg["spheres"]:
        c.initialize_seed(x, y, z, r)
    n0, ns = c.n, []

    def stop_at(rel_, patience_, abs_):
        streak = 0
        for i, n in enumerate(ns):
            if n <= abs_:
                return i + 1
            streak = streak + 1 if n < rel_ * n0 else 0
            if streak >= patience_:
                return i + 1
        return None

    it = None
    while it is None and len(ns) < 2000:
        c.step(1)
        ns.append(c.n)
        it = stop_at(rel, patience, 0)
    assert it is not None and 40 < it < 2000
    s = gpu()
    assert s.step_until_converged(rel, patience, 2000) == it
    assert s.stats()["iterations"] == it
    assert s.get_active_element_count() == c.n
    assert np.array_equal(s.active(), c.active())
    assert np.array_equal(s.read_phi(), c.read_phi())
    assert np.array_equal(s.get_saveable_segmentation(), c.read_mask())
    # A cap that falls inside a chunk of launched iterations.
    cap = it - 3
    s2 = gpu()
    assert s2.step_until_converged(rel, patience, cap) == cap
    c2 = O.RefOracle(vol, 0)
    c2.set_params(204, 26, 0.1, 0.25)
    for (x, y, z, r) in cfg["spheres"]:
        c2.initialize_seed(x, y, z, r)
    c2.step(cap)
    assert np.array_equal(s2.active(), c2.active())
    assert np.array_equal(s2.read_phi(), c2.read_phi())
    # The absolute threshold: the run stops at the first count at or below
    # it (a count the run passes through about half way).
    abs_thr = ns[it // 2]
    s4 = gpu()
    assert s4.step_until_converged(rel, patience, 2000, abs_threshold=abs_thr) == stop_at(rel, patience, abs_thr)
    # The engine keeps working after a run that stopped early (its rebuilds
    # and further steps are not halted).
    s.clear_current_segmentation()
    for (x, y, z, r) in cfg["spheres"]:
        s.initialize_seed((x, y, z), r)
    s.request_update_segmentation(7)
    c3 = O.RefOracle(vol, 0)
    c3.set_params(204, 26, 0.1, 0.25)
    for (x, y, z, r) in cfg["spheres"]:
        c3.initialize_seed(x, y, z, r)
    c3.step(7)
    assert np.array_equal(s.active(), c3.active())
    assert np.array_equal(s.read_phi(), c3.read_phi())
