"""The GPU adjoint (lss_adjoint_run) against the FP64 adjoint oracle, its
checkpointing, the engine state it must leave alone, and a torch.autograd
wrapper (test harness only) driving an Adam fit of T / eps / alpha."""
import numpy as np
import pytest

import aworkefficientgpualgorithmforlevelsetsegmentation_gb300 as lss
from aworkefficientgpualgorithmforlevelsetsegmentation_gb300 import phantoms as P
from oracle.oracle import NsOracle

pytestmark = pytest.mark.gpu


def make(cfg, brick=(8, 8, 8), threads=256):
    p = cfg["params"]
    s = lss.Segmenter(lss.MODE_NS, brick=brick, threads_per_brick=threads)
    s.load_volume(cfg["image"])
    s.set_parameters(p.target, p.window, p.curvature, p.time_step, alpha_role=p.alpha_role)
    s.set_phi(cfg["phi0"])
    return s


def oracle_adjoint(cfg, K, bias=None):
    p = cfg["params"]
    o = NsOracle(cfg["image"], threads=8)
    o.set_params(p.target, p.window, p.curvature, p.time_step, alpha_data=p.alpha_role)
    if bias is not None:
        o.set_bias(bias)
    o.set_phi(cfg["phi0"])
    return o.adjoint(K, cfg["target"], 0.5)


def rel(a, b):
    return abs(a - b) / max(abs(b), 1e-30)


@pytest.mark.parametrize("brick,threads,K,every", [((8, 8, 8), 256, 16, 4), ((8, 8, 4), 32, 24, 5),
                                                   ((4, 4, 4), 64, 12, 12)])
def test_gpu_adjoint_matches_fp64_adjoint(brick, threads, K, every):
    cfg = P.config4(0.25)
    rng = np.random.default_rng(3)
    bias = (0.05 * rng.standard_normal(cfg["image"].shape)).astype(np.float32)
    g = make(cfg, brick, threads).adjoint(K, every, cfg["target"], 0.5, bias=bias)
    o = oracle_adjoint(cfg, K, bias)
    # Pinned host buffers for the bias, the target and the bias gradient are
    # read and written in place: same results.
    torch = pytest.importorskip("torch")
    pb = torch.empty(bias.shape, dtype=torch.float32, pin_memory=True).numpy()
    pt = torch.empty(bias.shape, dtype=torch.uint8, pin_memory=True).numpy()
    pb[...], pt[...] = bias, cfg["target"]
    db_pinned = torch.empty(bias.shape, dtype=torch.float32, pin_memory=True).numpy()
    gp = make(cfg, brick, threads).adjoint(K, every, pt, 0.5, bias=pb, d_bias_out=db_pinned)
    # (The float atomics of the reverse pass sum in no fixed order.)
    assert gp["d_bias"] is db_pinned and np.allclose(db_pinned, g["d_bias"], rtol=1e-4, atol=1e-9)
    assert rel(gp["loss"], g["loss"]) <= 1e-9 and rel(gp["d_target"], g["d_target"]) <= 1e-5
    assert gp["active_voxel_iterations"] == g["active_voxel_iterations"] > 0
    assert abs(g["loss"] - o["loss"]) <= 1e-5
    for key in ("d_target", "d_window", "d_curvature"):
        assert rel(g[key], o[key]) <= 1e-3, (key, g[key], o[key])
    db, ob = g["d_bias"].astype(np.float64), o["d_bias"]
    assert np.linalg.norm(db - ob) <= 1e-3 * np.linalg.norm(ob)


def test_gpu_adjoint_ragged_volume_matches_fp64_adjoint():
    """A volume whose sides are not multiples of the brick: partial bricks at
    the far faces in the active lists, the dilation and the layout kernels."""
    c = P.config4(0.25)
    sl = (slice(3, 44), slice(1, 46), slice(5, 42))  # 41 x 45 x 37
    cfg = dict(c, image=np.ascontiguousarray(c["image"][sl]), target=np.ascontiguousarray(c["target"][sl]),
               phi0=np.ascontiguousarray(c["phi0"][sl]))
    rng = np.random.default_rng(5)
    bias = (0.05 * rng.standard_normal(cfg["image"].shape)).astype(np.float32)
    for brick, threads in [((8, 8, 8), 256), ((4, 4, 4), 64)]:
        g = make(cfg, brick, threads).adjoint(12, 5, cfg["target"], 0.5, bias=bias)
        o = oracle_adjoint(cfg, 12, bias)
        assert abs(g["loss"] - o["loss"]) <= 1e-5
        for key in ("d_target", "d_window", "d_curvature"):
            assert rel(g[key], o[key]) <= 1e-3, (brick, key, g[key], o[key])
        db, ob = g["d_bias"].astype(np.float64), o["d_bias"]
        assert np.linalg.norm(db - ob) <= 1e-3 * np.linalg.norm(ob)


def test_gpu_adjoint_checkpoint_spacing_is_invisible():
    cfg = P.config4(0.25)
    s = make(cfg)
    ref = s.adjoint(20, 20, cfg["target"])
    # The forward's recorded sets are the sparse engine's: the same number of
    # active-voxel updates over the same 20 iterations.
    fresh = make(cfg)
    fresh.step(20)
    assert ref["active_voxel_iterations"] == fresh.stats()["voxel_updates"] > 0
    for every in (1, 4, 7):
        g = s.adjoint(20, every, cfg["target"])
        assert g["loss"] == ref["loss"]
        for key in ("d_target", "d_window", "d_curvature"):
            assert rel(g[key], ref[key]) <= 1e-5
        assert np.allclose(g["d_bias"], ref["d_bias"], rtol=1e-4, atol=1e-9)
        assert g["active_voxel_iterations"] == ref["active_voxel_iterations"]


def test_gpu_adjoint_leaves_engine_state():
    cfg = P.config4(0.25)
    s = make(cfg)
    s.step(5)
    phi, act = s.read_phi(), s.active_linear()
    s.adjoint(16, 4, cfg["target"])
    assert np.array_equal(s.read_phi(), phi)
    assert np.array_equal(s.active_linear(), act)
    s.step(3)  # the engine keeps running from where it was


def test_autograd_wrapper_and_adam_fit():
    torch = pytest.importorskip("torch")
    cfg = P.config4(0.25)
    s = make(cfg)
    K, every = 24, 6

    class LevelSetLoss(torch.autograd.Function):
        """loss(T, eps, alpha, bias) through lss_adjoint_run (harness only)."""

        @staticmethod
        def forward(ctx, T, eps, alpha, bias):
            p = cfg["params"]
            s.set_parameters(float(T), float(eps), float(alpha), p.time_step, alpha_role=p.alpha_role)
            s.set_phi(cfg["phi0"])
            g = s.adjoint(K, every, cfg["target"], 0.5, bias=bias.detach().cpu().numpy())
            ctx.save_for_backward(torch.tensor([g["d_target"], g["d_window"], g["d_curvature"]],
                                               dtype=torch.float64),
                                  torch.from_numpy(g["d_bias"]))
            return torch.tensor(g["loss"], dtype=torch.float64)

        @staticmethod
        def backward(ctx, gl):
            gs, gb = ctx.saved_tensors
            return gl * gs[0], gl * gs[1], gl * gs[2], (gl * gb).to(torch.float32)

    T = torch.tensor(0.6, dtype=torch.float64, requires_grad=True)
    eps = torch.tensor(0.1, dtype=torch.float64, requires_grad=True)
    alpha = torch.tensor(0.9, dtype=torch.float64, requires_grad=True)
    bias = torch.zeros(cfg["image"].shape, dtype=torch.float32)
    opt = torch.optim.Adam([T, eps, alpha], lr=1e-2)
    losses = []
    for _ in range(20):
        opt.zero_grad()
        loss = LevelSetLoss.apply(T, eps, alpha, bias)
        loss.backward()
        opt.step()
        with torch.no_grad():
            eps.clamp_(0.02, 1.0)
            alpha.clamp_(0.0, 1.0)
        losses.append(float(loss.detach()))
    assert losses[-1] < losses[0] - 1e-3, losses


@pytest.mark.parametrize("shape", [(40, 48, 56), (37, 45, 43)])
def test_gpu_adjoint_device_buffers_match_host_buffers(shape):
    """Target, bias and the bias gradient as CUDA arrays (used in place when
    the rows need no padding, scattered and gathered on the device otherwise)
    give the host-buffer call's results."""
    torch = pytest.importorskip("torch")
    cfg = P.config4(0.5)  # 96^3; a centred crop keeps the seed and the shells
    crop = tuple(slice((m - c) // 2, (m - c) // 2 + c) for m, c in zip(cfg["image"].shape, shape))
    img = np.ascontiguousarray(cfg["image"][crop])
    tgt = np.ascontiguousarray(cfg["target"][crop])
    phi0 = np.ascontiguousarray(cfg["phi0"][crop])
    p = cfg["params"]
    rng = np.random.default_rng(5)
    bias = (0.02 * rng.standard_normal(shape)).astype(np.float32)

    def run(t, b, db):
        s = lss.Segmenter(lss.MODE_NS, brick=(8, 8, 8), threads_per_brick=256)
        s.load_volume(img)
        s.set_parameters(p.target, p.window, p.curvature, p.time_step, alpha_role=p.alpha_role)
        s.set_phi(phi0)
        return s.adjoint(12, 4, t, 0.5, bias=b, d_bias_out=db)

    h = run(tgt, bias, None)
    dev = torch.device("cuda:0")
    db = torch.full(shape, 7.0, dtype=torch.float32, device=dev)  # overwritten, not added to
    d = run(torch.from_numpy(tgt).to(dev), torch.from_numpy(bias).to(dev), db)
    torch.cuda.synchronize()
    assert d["d_bias"] is db
    assert d["loss"] == h["loss"]
    for key in ("d_target", "d_window", "d_curvature"):
        assert rel(d[key], h[key]) <= 1e-5, (key, d[key], h[key])
    assert np.allclose(db.cpu().numpy(), h["d_bias"], rtol=1e-4, atol=1e-9)
    assert h["active_voxel_iterations"] == d["active_voxel_iterations"] > 0


@pytest.mark.parametrize("brick,threads", [((8, 8, 8), 256), ((8, 8, 4), 32), ((4, 4, 4), 64)])
def test_gpu_adjoint_calls_on_one_engine_match_fresh_engines(brick, threads):
    """Between calls the engine keeps the forward's two copies of phi_0 and
    copies again only the bricks the previous call touched, while its phi is
    unchanged and no host staging went through them: device buffers, so the
    later calls take that path.  Each call equals the same call on a fresh
    engine: the same call again, a call whose bias reaches other bricks, the
    first bias once more, a call after new parameters (phi unchanged: still
    partial copies), and a call after further iterations of the engine (phi
    changed: full copies)."""
    torch = pytest.importorskip("torch")
    cfg = P.config4(0.25)
    shape = cfg["image"].shape
    dev = torch.device("cuda:0")
    rng = np.random.default_rng(11)
    b1 = (0.05 * rng.standard_normal(shape)).astype(np.float32)
    b2 = (0.3 * rng.standard_normal(shape) + 0.2).astype(np.float32)
    tgt = torch.from_numpy(cfg["target"]).to(dev)
    K, every = 16, 4

    def call(s, bias):
        db = torch.empty(shape, dtype=torch.float32, device=dev)
        g = s.adjoint(K, every, tgt, 0.5, bias=torch.from_numpy(bias).to(dev), d_bias_out=db)
        torch.cuda.synchronize()
        g["d_bias"] = db.cpu().numpy()
        return g

    def fresh(bias, steps=0, target=None):
        e = make(cfg, brick, threads)
        if target is not None:
            e.set_parameters(target=target)
        if steps:
            e.step(steps)
        return call(e, bias)

    def same(g, h):
        assert g["loss"] == h["loss"]
        assert g["active_voxel_iterations"] == h["active_voxel_iterations"] > 0
        for key in ("d_target", "d_window", "d_curvature"):
            assert rel(g[key], h[key]) <= 1e-5, (key, g[key], h[key])
        assert np.allclose(g["d_bias"], h["d_bias"], rtol=1e-4, atol=1e-9)

    s = make(cfg, brick, threads)
    r1 = call(s, b1)
    same(r1, fresh(b1))
    same(call(s, b1), r1)
    r2 = call(s, b2)
    assert r2["active_voxel_iterations"] != r1["active_voxel_iterations"]
    same(r2, fresh(b2))
    same(call(s, b1), r1)
    t2 = cfg["params"].target - 0.03
    s.set_parameters(target=t2)
    same(call(s, b1), fresh(b1, target=t2))
    s.set_parameters(target=cfg["params"].target)
    same(call(s, b1), r1)
    s.step(3)
    same(call(s, b1), fresh(b1, steps=3))
    same(call(s, b2), fresh(b2, steps=3))
