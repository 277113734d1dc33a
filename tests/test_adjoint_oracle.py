"""The FP64 adjoint oracle (oracle/ns_adjoint.hpp) against central finite
differences of its own FP64 forward, under the fixed-active-set convention
(the sets recorded by the adjoint's forward pass are replayed)."""
import numpy as np
import pytest

from aworkefficientgpualgorithmforlevelsetsegmentation_gb300 import phantoms as P
from oracle.oracle import NsOracle


@pytest.fixture(scope="module")
def case():
    cfg = P.config4(0.25)  # 48^3 two-shell phantom
    p = cfg["params"]
    o = NsOracle(cfg["image"], threads=8)
    o.set_params(p.target, p.window, p.curvature, p.time_step, alpha_data=p.alpha_role)
    o.set_phi(cfg["phi0"])
    K = 16
    r = o.adjoint(K, cfg["target"], 0.5)
    return cfg, o, K, r


def test_scalar_gradients_match_central_differences(case):
    cfg, o, K, r = case
    p = cfg["params"]
    base = {"T": p.target, "eps": p.window, "alpha": p.curvature}
    # h = 1e-5: the loss is piecewise smooth (the clamp of D, |I - T| and the
    # upwind selection have kinks); a step this small stays on one piece.
    h = 1e-5
    for name, key in (("T", "d_target"), ("eps", "d_window"), ("alpha", "d_curvature")):
        o.set_param(name, base[name] + h)
        lp = o.adjoint_loss(K, cfg["target"])
        o.set_param(name, base[name] - h)
        lm = o.adjoint_loss(K, cfg["target"])
        o.set_param(name, base[name])
        fd = (lp - lm) / (2 * h)
        assert abs(fd - r[key]) <= 1e-4 * abs(fd), (name, fd, r[key])


def test_bias_gradients_match_central_differences(case):
    cfg, o, K, r = case
    db = r["d_bias"].ravel()
    support = np.flatnonzero(db)
    assert support.size > 100
    rng = np.random.default_rng(7)
    idx = rng.choice(support, 32, replace=False)
    h = 1e-3
    b = np.zeros(cfg["image"].size, np.float64)
    for i in idx:
        b[i] = h
        o.set_bias64(b.reshape(cfg["image"].shape))
        lp = o.adjoint_loss(K, cfg["target"])
        b[i] = -h
        o.set_bias64(b.reshape(cfg["image"].shape))
        lm = o.adjoint_loss(K, cfg["target"])
        b[i] = 0.0
        fd = (lp - lm) / (2 * h)
        assert abs(fd - db[i]) <= 1e-3 * abs(fd) + 1e-12, (i, fd, db[i])
    o.set_bias64(None)


def test_state_is_unchanged(case):
    cfg, o, K, r = case
    phi = o.read_phi64().copy()
    act = o.active().copy()
    o.adjoint(K, cfg["target"])
    assert np.array_equal(o.read_phi64(), phi) and np.array_equal(o.active(), act)
