"""The differentiation form at its stated size: the 192^3 two-shell phantom,
K = 64 unrolled iterations from the radius-8 seed, phi checkpointed every 8,
soft-Dice of sigmoid(-phi/0.5) against the inner ellipsoid, T = 0.6,
eps = 0.1, alpha = 0.9, bias 0 (the `bench.py --workload adjoint` call).

  * GPU adjoint against the FP64 adjoint oracle: loss within 1e-6, dT, deps,
    dalpha within 1e-3 relative, the bias gradient within 1e-3 relative L2.
  * GPU gradients against central finite differences of the FP64 forward
    (the oracle's recorded active sets replayed) on the three scalars and 32
    random bias voxels.  The loss has kinks (the clamp of D, |I - T|, the
    upwind selection, the phi clamp): at h = 1e-3 the difference quotient of
    T and eps straddles some of them and is itself off by a few 1e-3, so the
    test runs an h-study (1e-3, 1e-4, 1e-5): the quotient converges to the
    adjoint as h shrinks, and the GPU gradient is within 1e-3 of it at
    h = 1e-4 and 1e-5; at h = 1e-3 within 1e-2.  The bias voxels are drawn
    from those whose gradient is at least 1e-4 of the largest (smaller ones
    change the loss by less than the resolution of an FP64 sum of 7 M terms);
    all quotients are taken on the Dice coefficient itself (1 - loss), which
    keeps the digits that subtracting from 1 rounds away.
  * 200 Adam steps (lr 1e-2) of T, eps and alpha through a torch.autograd
    wrapper of lss_adjoint_run (test harness only).
"""
import numpy as np
import pytest

import aworkefficientgpualgorithmforlevelsetsegmentation_gb300 as lss
from aworkefficientgpualgorithmforlevelsetsegmentation_gb300 import phantoms as P
from oracle.oracle import NsOracle

pytestmark = pytest.mark.gpu


def rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


@pytest.fixture(scope="module")
def case():
    cfg = P.config4(1.0)
    p = cfg["params"]
    K, every = cfg["K"], cfg["checkpoint_every"]
    s = lss.Segmenter(lss.MODE_NS, brick=(8, 8, 8), threads_per_brick=256)
    s.load_volume(cfg["image"])
    s.set_parameters(p.target, p.window, p.curvature, p.time_step, alpha_role=p.alpha_role)
    s.set_phi(cfg["phi0"])
    g = s.adjoint(K, every, cfg["target"], 0.5, bias=np.zeros(cfg["image"].shape, np.float32))
    o = NsOracle(cfg["image"], threads=8)
    o.set_params(p.target, p.window, p.curvature, p.time_step, alpha_data=p.alpha_role)
    o.set_phi(cfg["phi0"])
    r = o.adjoint(K, cfg["target"], 0.5)
    return cfg, s, g, o, r


def test_gpu_adjoint_192_matches_fp64_adjoint(case):
    cfg, s, g, o, r = case
    assert abs(g["loss"] - r["loss"]) <= 1e-6, (g["loss"], r["loss"])
    for key in ("d_target", "d_window", "d_curvature"):
        assert rel(g[key], r[key]) <= 1e-3, (key, g[key], r[key])
    db, ob = g["d_bias"].astype(np.float64), r["d_bias"]
    assert np.linalg.norm(db - ob) <= 1e-3 * np.linalg.norm(ob)
    # The same forward as the sparse engine: 64 iterations of active voxels.
    assert g["active_voxel_iterations"] > 64 * 1000


def test_gpu_adjoint_192_matches_central_differences(case):
    cfg, s, g, o, r = case
    p = cfg["params"]
    K, tgt = cfg["K"], cfg["target"]
    base = {"T": p.target, "eps": p.window, "alpha": p.curvature}
    study = {}
    for name, key in (("T", "d_target"), ("eps", "d_window"), ("alpha", "d_curvature")):
        for h in (1e-3, 1e-4, 1e-5):
            o.set_param(name, base[name] + h)
            cp = o.adjoint_dice(K, tgt)
            o.set_param(name, base[name] - h)
            cm = o.adjoint_dice(K, tgt)
            o.set_param(name, base[name])
            fd = -(cp - cm) / (2 * h)  # loss = 1 - coefficient
            study[(name, h)] = (fd, rel(g[key], fd), rel(r[key], fd))
    msg = "\n".join(f"{k}: fd {v[0]:.6e} gpu-rel {v[1]:.2e} fp64-adjoint-rel {v[2]:.2e}" for k, v in study.items())
    for name in ("T", "eps", "alpha"):
        assert study[(name, 1e-3)][1] <= 1e-2, msg
        assert study[(name, 1e-4)][1] <= 1e-3, msg
        assert study[(name, 1e-5)][1] <= 1e-3, msg
        # the FP64 adjoint converges on the quotient as h shrinks
        assert study[(name, 1e-5)][2] <= study[(name, 1e-3)][2] + 1e-6, msg

    db = g["d_bias"].ravel().astype(np.float64)
    support = np.flatnonzero(np.abs(db) >= 1e-4 * np.abs(db).max())
    assert support.size >= 1000
    rng = np.random.default_rng(7)
    idx = rng.choice(support, 32, replace=False)
    b = np.zeros(db.size, np.float64)
    errs = {1e-3: [], 1e-4: []}
    for i in idx:
        for h in errs:
            b[i] = h
            o.set_bias64(b.reshape(cfg["image"].shape))
            cp = o.adjoint_dice(K, tgt)
            b[i] = -h
            o.set_bias64(b.reshape(cfg["image"].shape))
            cm = o.adjoint_dice(K, tgt)
            b[i] = 0.0
            fd = -(cp - cm) / (2 * h)  # loss = 1 - coefficient
            errs[h].append(rel(db[i], fd))
    o.set_bias64(None)
    e3, e4 = np.array(errs[1e-3]), np.array(errs[1e-4])
    assert np.median(e3) <= 1e-3 and e3.max() <= 1e-2, (e3, e4)
    assert e4.max() <= 1e-3, (e3, e4)


def test_autograd_adam_fit_192(case):
    """200 Adam steps (lr 1e-2) on T, eps, alpha at 192^3, K = 64, every 8."""
    torch = pytest.importorskip("torch")
    cfg, s, _, _, _ = case
    p = cfg["params"]
    K, every = cfg["K"], cfg["checkpoint_every"]
    shape = cfg["image"].shape
    tgt = torch.empty(shape, dtype=torch.uint8, pin_memory=True).numpy()
    tgt[...] = cfg["target"]
    bias_h = torch.zeros(shape, dtype=torch.float32, pin_memory=True).numpy()
    dbias_h = torch.empty(shape, dtype=torch.float32, pin_memory=True).numpy()

    class LevelSetLoss(torch.autograd.Function):
        """loss(T, eps, alpha) through lss_adjoint_run (harness only)."""

        @staticmethod
        def forward(ctx, T, eps, alpha):
            s.set_parameters(float(T), float(eps), float(alpha), p.time_step, alpha_role=p.alpha_role)
            s.set_phi(cfg["phi0"])
            g = s.adjoint(K, every, tgt, 0.5, bias=bias_h, d_bias_out=dbias_h)
            ctx.save_for_backward(torch.tensor([g["d_target"], g["d_window"], g["d_curvature"]],
                                               dtype=torch.float64))
            return torch.tensor(g["loss"], dtype=torch.float64)

        @staticmethod
        def backward(ctx, gl):
            (gs,) = ctx.saved_tensors
            return gl * gs[0], gl * gs[1], gl * gs[2]

    T = torch.tensor(p.target, dtype=torch.float64, requires_grad=True)
    eps = torch.tensor(p.window, dtype=torch.float64, requires_grad=True)
    alpha = torch.tensor(p.curvature, dtype=torch.float64, requires_grad=True)
    opt = torch.optim.Adam([T, eps, alpha], lr=1e-2)
    losses = []
    for _ in range(200):
        opt.zero_grad()
        loss = LevelSetLoss.apply(T, eps, alpha)
        loss.backward()
        opt.step()
        with torch.no_grad():
            eps.clamp_(0.02, 1.0)
            alpha.clamp_(0.0, 1.0)
        losses.append(float(loss.detach()))
    # From T = 0.6 the seed shrinks (the inner shell is at 0.75) and the loss
    # is ~1; the fit raises T towards the shell and the front grows into the
    # target (about 0.5 voxel an iteration at most, so 64 iterations cannot
    # fill the whole ellipsoid at this size).
    assert min(losses[-20:]) < losses[0] - 0.1, (losses[0], losses[-20:])
    T, eps, alpha = (float(t.detach()) for t in (T, eps, alpha))
    assert T > 0.65, (T, eps, alpha)
