"""The restated REF oracle against the reference's own kernel sources
compiled for the CPU (oracle/_ref, built only where the reference sources
are mounted; skipped elsewhere).  Every buffer of the solver is compared
bit for bit after every step."""
import numpy as np
import pytest

from oracle import oracle as O
from oracle import build as OB
from tests.ref_cases import CASES, DT, make_volume, run_case

ref_lib = None
try:
    OB.build_reference()
    ref_lib = O.reference_lib()
except Exception:  # reference sources absent
    ref_lib = None

needs_ref = pytest.mark.skipif(ref_lib is None, reason="reference sources not mounted")


def _mk(refk):
    return lambda vol, dt: O.RefOracle(vol, dt, use_reference_kernels=refk)


def _same(a, b):
    assert len(a) == len(b)
    for x, y in zip(a, b):
        assert x[0] == y[0]
        for u, v in zip(x[1:], y[1:]):
            assert np.array_equal(np.asarray(u), np.asarray(v)), x[0]


@needs_ref
@pytest.mark.parametrize("name", sorted(CASES))
def test_restated_matches_reference_kernels(name):
    _same(run_case(name, _mk(False)), run_case(name, _mk(True)))


@needs_ref
@pytest.mark.parametrize("name", ["ball_u8", "many_active_s8", "param_change_u8"])
def test_all_buffers_match_each_step(name):
    shape, dt, va, params, seeds, schedule = CASES[name]
    vol = make_volume(name)
    a = O.RefOracle(vol, DT[dt][0])
    b = O.RefOracle(vol, DT[dt][0], use_reference_kernels=True)
    for o in (a, b):
        o.set_params(*params)
        for s in seeds:
            o.initialize_seed(*s)
    for k in range(12):
        if k == 5:
            for o in (a, b):
                o.set_params(params[0], params[1] + 7, params[2], params[3])
        a.step(1)
        b.step(1)
        for buf in O.RefOracle.BUFFERS:
            assert np.array_equal(a.buffer(buf), b.buffer(buf)), (k, buf)


@needs_ref
def test_quirk_is_what_reference_does():
    """The restated oracle without the three-of-four quirk diverges from the
    reference kernels (the quirk is real), with it they agree."""
    vol = make_volume("ball_u8")
    a = O.RefOracle(vol, 0, quirk_i3=False)
    b = O.RefOracle(vol, 0, use_reference_kernels=True)
    for o in (a, b):
        o.set_params(140, 40, 0.16, 0.25)
        o.initialize_seed(16, 16, 16, 3)
        o.step(6)
    assert not np.array_equal(a.active(), b.active())


@needs_ref
def test_estimate_params_matches():
    vol = make_volume("ball_u8")
    a = O.RefOracle(vol, 0)
    b = O.RefOracle(vol, 0, use_reference_kernels=True)
    for o in (a, b):
        o.set_params(140, 40, 0.16, 0.25)
        o.initialize_seed(16, 16, 16, 3)
        o.step(10)
    assert a.estimate_params() == b.estimate_params()
