"""GPU adjoint of the sphere step (cdx_adj_*): against the FP64 CPU adjoint, against central finite
differences of the GPU rollout itself, across checkpoint spacings, and through torch.autograd."""
import numpy as np
import pytest

from cardillocxx_gb300 import scenes
from cardillocxx_gb300.adjoint import Rollout, rollout
from cardillocxx_gb300.scenes import make_scene

pytestmark = pytest.mark.gpu

GROUND = {"kind": "halfspace", "pos": (0, 0, 0), "dir": (0, 0, 1), "mu": 0.3}
WALL = {"kind": "halfspace", "pos": (-0.3, 0, 0), "dir": (1, 0, 0), "mu": 0.3}
MATCH_RTOL = 1e-10   # GPU vs CPU FP64 adjoint (same operations; summation order of the mu sums)
FD_RTOL = 1e-4       # the target: adjoint vs central differences (eps 1e-6)


def small_scene():
    bodies = [
        {"pos": (0.0, 0.0, 0.0499), "radius": 0.05, "vel": (1.0, 0.2, 0.0)},
        {"pos": (0.2, 0.0, 0.0499), "radius": 0.05},
        {"pos": (0.2, 0.0, 0.1498), "radius": 0.05, "vel": (0.1, 0, 0), "omega": (0, 3, 0)},
        {"pos": (-0.25, 0.1, 0.0499), "radius": 0.05, "vel": (-0.5, 0, 0)},
        {"pos": (0.5, 0.5, 0.3), "radius": 0.03, "vel": (0.0, 0.0, -0.5)},
        {"pos": (0.56, 0.53, 0.35), "radius": 0.04, "vel": (-0.2, 0.0, -0.1), "omega": (1, 2, 3)},
    ]
    return make_scene(bodies, [GROUND, WALL])


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def test_gpu_rollout_and_adjoint_match_cpu_adjoint(gpu, oracle_mod):
    s = scenes.generate("diff_256x256", scale=3 / 256)
    cfg = scenes.config_for("diff_256x256")
    mu = np.array([0.3, 0.2, 0.5])
    rng = np.random.default_rng(1)
    g = rng.normal(size=(3, s["pos"].shape[0], 3))
    R = Rollout(s, cfg, checkpoint_every=7)
    A = oracle_mod.AdjOracle(s, cfg)
    xg = R.forward(30, s["pos"], s["vel"], s["omega"], mu)
    xc = A.rollout(30, s["pos"], s["vel"], s["omega"], mu)
    for a, b in zip(xg, xc):
        assert rel(a, b) <= 1e-13
    gg = R.backward(*g)
    gc = A.gradient(30, s["pos"], s["vel"], s["omega"], mu, *g)
    for name, a, b in zip(("x", "v", "w", "mu"), gg, gc):
        assert rel(a, b) <= MATCH_RTOL, (name, rel(a, b))


def test_gpu_adjoint_matches_central_differences(gpu):
    s = small_scene()
    cfg = scenes.config_for("diff_256x256")
    R = Rollout(s, cfg, checkpoint_every=4)
    rng = np.random.default_rng(2)
    N = s["pos"].shape[0]
    a, b, c = rng.normal(size=(3, N, 3))
    mu = np.array([0.3])
    args = [s["pos"], s["vel"], s["omega"], mu]

    def loss(*p):
        xT, vT, wT = R.forward(25, *p)
        return (a * xT).sum() + (b * vT).sum() + (c * wT).sum()

    loss(*args)
    grads = R.backward(a, b, c)
    eps = 1e-6
    for k in range(4):
        d = rng.normal(size=np.shape(args[k]))
        ap, am = list(args), list(args)
        ap[k] = args[k] + eps * d
        am[k] = args[k] - eps * d
        fd = (loss(*ap) - loss(*am)) / (2 * eps)
        an = float((grads[k] * d).sum())
        assert abs(fd - an) <= FD_RTOL * abs(fd), (k, fd, an)


def test_checkpoint_spacing_does_not_change_the_gradient(gpu):
    s = small_scene()
    cfg = scenes.config_for("diff_256x256")
    rng = np.random.default_rng(3)
    g = rng.normal(size=(3, s["pos"].shape[0], 3))
    outs = []
    for every in (1, 3, 50):
        R = Rollout(s, cfg, checkpoint_every=every)
        R.forward(17, s["pos"], s["vel"], s["omega"], [0.3])
        outs.append(R.backward(*g))
        R.close()
    for o in outs[1:]:
        for a, b in zip(o, outs[0]):
            assert np.array_equal(a, b)


def test_torch_autograd_function_com_loss(gpu):
    torch = pytest.importorskip("torch")
    s = scenes.generate("diff_256x256", scale=2 / 256)
    cfg = scenes.config_for("diff_256x256")
    N = s["pos"].shape[0]
    R = Rollout(s, cfg, checkpoint_every=10)
    scene_of = torch.as_tensor(s["body_scene"], dtype=torch.long)
    m = torch.as_tensor(s["mass"])
    target = torch.tensor([[0.4, 0.5, 0.3], [0.6, 0.4, 0.2]], dtype=torch.float64)

    def loss_of(mu_t, v_t):
        x0 = torch.as_tensor(s["pos"])
        w0 = torch.as_tensor(s["omega"])
        xT, vT, wT = rollout(R, 40, x0, v_t, w0, mu_t)
        com = torch.zeros(2, 3, dtype=torch.float64).index_add(0, scene_of, xT * m[:, None])
        com = com / torch.zeros(2, dtype=torch.float64).index_add(0, scene_of, m)[:, None]
        return ((com - target) ** 2).sum()

    mu = torch.tensor([0.3, 0.3], dtype=torch.float64, requires_grad=True)
    v0 = torch.as_tensor(s["vel"]).clone().requires_grad_(True)
    L = loss_of(mu, v0)
    L.backward()
    eps = 1e-6
    with torch.no_grad():
        for k in range(2):
            e = torch.zeros(2, dtype=torch.float64)
            e[k] = eps
            fd = (loss_of(mu + e, v0) - loss_of(mu - e, v0)).item() / (2 * eps)
            assert abs(fd - mu.grad[k].item()) <= FD_RTOL * max(abs(fd), 1e-12), (k, fd, mu.grad[k].item())
        d = torch.as_tensor(np.random.default_rng(5).normal(size=(N, 3)))
        fd = (loss_of(mu, v0 + eps * d) - loss_of(mu, v0 - eps * d)).item() / (2 * eps)
        an = (v0.grad * d).sum().item()
        assert abs(fd - an) <= FD_RTOL * abs(fd), (fd, an)


def subscene(s, keep):
    """The scenes `keep` of a batched scene dict, renumbered 0..len(keep)-1."""
    keep = list(keep)
    bs, ss = s["body_scene"], s["static_scene"]
    bsel = np.isin(bs, keep)
    ssel = np.isin(ss, keep)
    remap = {k: i for i, k in enumerate(keep)}
    out = {}
    for k, v in s.items():
        if isinstance(v, np.ndarray) and k.startswith("static_"):
            out[k] = v[ssel].copy()
        elif isinstance(v, np.ndarray) and v.shape[:1] == bs.shape:
            out[k] = v[bsel].copy()
        else:
            out[k] = v
    out["body_scene"] = np.array([remap[k] for k in bs[bsel]], np.int32)
    out["static_scene"] = np.array([remap[k] for k in ss[ssel]], np.int32)
    out["num_scenes"] = len(keep)
    return out, bsel


def test_differentiation_workload_mu_gradient(gpu, oracle_mod):
    # the full 256 scenes x 256 spheres, 200 steps, 50 sweeps, checkpoints every 20 steps.
    # (1) Every scene's friction gradient of its COM loss against central differences (eps 1e-6):
    # scenes are independent, so one +eps and one -eps rollout give all 256 differences. The loss
    # is piecewise smooth: a contact found one step earlier or later is a jump, and a cone
    # projection switching between sticking and sliding inside some sweep is a kink; scenes whose
    # two rollouts saw different contact events are left out and counted, kinks stay in.
    # (2) Six of the scenes through the FP64 CPU adjoint: the same function, so the same gradient.
    s = scenes.generate("diff_256x256")
    cfg = scenes.config_for("diff_256x256")
    nsc = int(s["num_scenes"])
    R = Rollout(s, cfg, checkpoint_every=20)
    sc = s["body_scene"]
    m = s["mass"]
    M = np.bincount(sc, weights=m, minlength=nsc)
    target = np.random.default_rng(6).uniform((0.2, 0.2, 0.1), (0.8, 0.8, 0.5), size=(nsc, 3))
    mu = np.full(nsc, 0.3)

    def per_scene(mu_v):
        xT, vT, wT = R.forward(200, s["pos"], s["vel"], s["omega"], mu_v)
        com = np.stack([np.bincount(sc, weights=m * xT[:, k], minlength=nsc) for k in range(3)], 1) / M[:, None]
        gx = 2 * (com - target)[sc] * (m / M[sc])[:, None]
        return ((com - target) ** 2).sum(1), gx, R.contact_counts()

    _, gx, _ = per_scene(mu)
    zero = np.zeros_like(gx)
    gx0, gv0, gw0, gmu = R.backward(gx, zero, zero)
    eps = 1e-6
    Lp, _, cp = per_scene(mu + eps)
    Lm, _, cm = per_scene(mu - eps)
    fd = (Lp - Lm) / (2 * eps)
    smooth = (cp == cm) & (np.abs(fd) > 1e-6)
    err = np.abs(fd - gmu)[smooth] / np.abs(fd)[smooth]
    assert smooth.sum() >= 0.8 * nsc, f"only {smooth.sum()} of {nsc} scenes comparable"
    assert np.median(err) <= 1e-5, np.median(err)
    assert np.mean(err <= 1e-4) >= 0.9, (np.mean(err <= 1e-4), np.sort(err)[-8:])

    keep = [0, 31, 77, 128, 182, 255]
    sub, sel = subscene(s, keep)
    A = oracle_mod.AdjOracle(sub, cfg)
    c = A.gradient(200, sub["pos"], sub["vel"], sub["omega"], mu[keep], gx[sel], zero[sel], zero[sel])
    assert rel(gmu[keep], c[3]) <= 1e-9, (gmu[keep], c[3])
    assert rel(gv0[sel], c[1]) <= 1e-9
    assert rel(gx0[sel], c[0]) <= 1e-9
