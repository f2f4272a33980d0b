"""Solid cylinder statics (C_RB_Cylinder, coal::Cylinder; collision_coal.cpp:307-310): spheres rain on a
horizontal and a vertical cylinder standing on the ground; the plain FP64 method against the oracle
bit for bit, the split form beside it."""
import numpy as np
import pytest

from cardillocxx_gb300 import PhysicsEngine, scenes
from cardillocxx_gb300.scenes import make_scene

pytestmark = pytest.mark.gpu


def assert_same(a, b, what):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape, (what, a.shape, b.shape)
    if not np.array_equal(a, b):
        raise AssertionError(f"{what}: not bit-identical, max |diff| {np.nanmax(np.abs(a - b)):.3e}")


def cylinder_scene(n_side=8):
    rng = np.random.default_rng(7)
    bodies = []
    for i in range(n_side):
        for j in range(n_side):
            for k in range(3):
                x = -0.35 + 0.7 * i / (n_side - 1) + rng.uniform(-0.01, 0.01)
                y = -0.35 + 0.7 * j / (n_side - 1) + rng.uniform(-0.01, 0.01)
                bodies.append({"pos": (x, y, 0.55 + 0.11 * k), "radius": 0.04 + 0.01 * rng.uniform(), "mu": 0.4})
    statics = [{"kind": "halfspace", "pos": (0, 0, 0), "dir": (0, 0, 1), "mu": 0.4},
               {"kind": "cylinder", "pos": (0.0, -0.15, 0.2), "dir": (1, 0, 0), "radius": 0.12,
                "half_length": 0.3, "mu": 0.5},
               {"kind": "cylinder", "pos": (0.1, 0.2, 0.15), "dir": (0, 0, 1), "radius": 0.1,
                "half_length": 0.15, "mu": 0.5}]
    return make_scene(bodies, statics)


def test_cylinder_statics_bit_identical(oracle_mod):
    s = cylinder_scene()
    cfg = scenes.config_for("pile_1k")
    eng = PhysicsEngine(cfg).load_scene(s)
    orc = oracle_mod.Oracle(s, cfg)
    for done in range(50, 401, 50):
        eng.step(50)
        orc.step(50)
        g, o = eng.state(), orc.state()
        for key in ("pos", "quat", "vel", "omega"):
            assert_same(g[key], o[key], f"{key} after {done} steps")
    gc, oc = eng.contacts(), orc.contacts()
    for key in ("id_a", "id_b", "point", "lambda", "normal"):
        assert_same(gc[key], oc[key], f"contact {key}")
    # spheres rest on both cylinders (static ids 1 and 2)
    assert (gc["id_a"] == 1).sum() > 0 and (gc["id_a"] == 2).sum() > 0


def test_cylinder_statics_split_form():
    s = cylinder_scene()
    cfg = scenes.config_for("pile_1k")
    e64 = PhysicsEngine(cfg).load_scene(s)
    e32 = PhysicsEngine(dict(cfg, **{"gpu.precision": "split"})).load_scene(s)
    e64.step(250)
    e32.step(250)
    c64, c32 = e64.contacts(), e32.contacts()
    assert (c32["id_a"] == 1).sum() > 0 and (c32["id_a"] == 2).sum() > 0
    # both settle on the same supports: mean heights agree to a few millimetres
    z64, z32 = e64.state()["pos"][:, 2], e32.state()["pos"][:, 2]
    assert np.isfinite(z32).all() and abs(z64.mean() - z32.mean()) < 5e-3
    # one converged step from the same state agrees with FP64
    st = e64.state()
    tight = dict(cfg, **{"pj.max_iterations": 3000, "pj.warmstart": False})
    a = PhysicsEngine(tight).load_scene(s)
    b = PhysicsEngine(dict(tight, **{"gpu.precision": "split"})).load_scene(s)
    for e in (a, b):
        e.set_state(st["pos"], st["quat"], st["vel"], st["omega"])
        e.step(1)
    vs = np.abs(st["vel"]).max() + 9.81e-3
    assert np.abs(a.state()["vel"] - b.state()["vel"]).max() <= 1e-3 * vs
