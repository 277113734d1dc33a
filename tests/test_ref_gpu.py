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
