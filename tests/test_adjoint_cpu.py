"""The FP64 CPU adjoint (the checker of the GPU adjoint) against central finite differences and its
forward model against the oracle's restatement of the reference step (CPU only)."""
import numpy as np
import pytest

from cardillocxx_gb300 import scenes
from cardillocxx_gb300.scenes import make_scene

GROUND = {"kind": "halfspace", "pos": (0, 0, 0), "dir": (0, 0, 1), "mu": 0.3}
WALL = {"kind": "halfspace", "pos": (-0.3, 0, 0), "dir": (1, 0, 0), "mu": 0.3}
FD_RTOL = 1e-6  # central differences, eps 1e-6, smooth branch: truncation and rounding ~1e-9


def small_scene():
    bodies = [
        {"pos": (0.0, 0.0, 0.0499), "radius": 0.05, "vel": (1.0, 0.2, 0.0)},         # sliding on the ground
        {"pos": (0.2, 0.0, 0.0499), "radius": 0.05},                                 # resting, loaded
        {"pos": (0.2, 0.0, 0.1498), "radius": 0.05, "vel": (0.1, 0, 0), "omega": (0, 3, 0)},
        {"pos": (-0.25, 0.1, 0.0499), "radius": 0.05, "vel": (-0.5, 0, 0)},           # into the wall
        {"pos": (0.5, 0.5, 0.3), "radius": 0.03, "vel": (0.0, 0.0, -0.5)},
        {"pos": (0.56, 0.53, 0.35), "radius": 0.04, "vel": (-0.2, 0.0, -0.1), "omega": (1, 2, 3)},
    ]
    return make_scene(bodies, [GROUND, WALL])


def fd_check(A, nsteps, x0, v0, w0, mu, seed, eps=1e-6, which="xvwm"):
    rng = np.random.default_rng(seed)
    N = x0.shape[0]
    a, b, c = rng.normal(size=(3, N, 3))

    def loss(*args):
        xT, vT, wT = A.rollout(nsteps, *args)
        return (a * xT).sum() + (b * vT).sum() + (c * wT).sum()

    grads = A.gradient(nsteps, x0, v0, w0, mu, a, b, c)
    out = {}
    for k, name in enumerate("xvwm"):
        if name not in which:
            continue
        d = rng.normal(size=np.shape([x0, v0, w0, mu][k]))
        args_p = [x0, v0, w0, mu]
        args_m = [x0, v0, w0, mu]
        args_p[k] = args_p[k] + eps * d
        args_m[k] = args_m[k] - eps * d
        fd = (loss(*args_p) - loss(*args_m)) / (2 * eps)
        an = float((grads[k] * d).sum())
        out[name] = (fd, an)
    return out


@pytest.mark.parametrize("nsteps", [1, 5, 40])
def test_cpu_adjoint_matches_central_differences(oracle_mod, nsteps):
    s = small_scene()
    cfg = scenes.config_for("diff_256x256")
    A = oracle_mod.AdjOracle(s, cfg)
    for name, (fd, an) in fd_check(A, nsteps, s["pos"], s["vel"], s["omega"], np.array([0.3]), seed=nsteps).items():
        assert abs(fd - an) <= FD_RTOL * max(abs(fd), 1e-12), (name, fd, an)


def test_cpu_adjoint_batched_scenes_and_friction(oracle_mod):
    # two generated scenes of the differentiation workload: per-scene mu gradients and velocity /
    # angular-velocity gradients; positions perturbed with a smaller step (some spheres start exactly
    # on the floor, where a contact appears or not)
    s = scenes.generate("diff_256x256", scale=2 / 256)
    cfg = scenes.config_for("diff_256x256")
    A = oracle_mod.AdjOracle(s, cfg)
    mu = np.array([0.3, 0.45])
    res = fd_check(A, 20, s["pos"], s["vel"], s["omega"], mu, seed=3, which="vwm")
    res.update(fd_check(A, 20, s["pos"], s["vel"], s["omega"], mu, seed=4, eps=1e-8, which="x"))
    for name, (fd, an) in res.items():
        tol = 1e-5 if name == "x" else FD_RTOL
        assert abs(fd - an) <= tol * max(abs(fd), 1e-12), (name, fd, an)


def test_cpu_adjoint_model_is_the_reference_step(oracle_mod):
    # the world-frame model steps exactly like the restated reference step (no warm start, fixed
    # sweeps): positions, velocities and world-frame angular velocities over 60 steps
    s = small_scene()
    cfg = scenes.config_for("diff_256x256", **{"pj.warmstart": False})
    A = oracle_mod.AdjOracle(s, cfg)
    xT, vT, wT = A.rollout(60, s["pos"], s["vel"], s["omega"], np.array([0.3]))
    o = oracle_mod.Oracle(s, cfg)
    o.step(60)
    st = o.state()
    q = st["quat"]  # x, y, z, w
    x, y, z, w = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    R = np.stack([
        np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)], -1),
        np.stack([2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)], -1),
        np.stack([2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], -1)], 1)
    w_world = np.einsum("nij,nj->ni", R, st["omega"])
    np.testing.assert_allclose(xT, st["pos"], rtol=0, atol=1e-9)
    np.testing.assert_allclose(vT, st["vel"], rtol=0, atol=1e-9)
    np.testing.assert_allclose(wT, w_world, rtol=0, atol=1e-8)
