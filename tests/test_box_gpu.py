"""Solid box statics (C_RB_Cube, coal::Box; collision_coal.cpp:288-290): spheres rain into a tray walled
by boxes around a turned, tilted box; the stacked_spheres scene (a column of spheres in a tube of four
box walls on a box floor that a trajectory heaves and turns, examples/scenes/stacked_spheres). The
plain FP64 method against the oracle bit for bit, the split form beside it."""
import math

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


def quat_axis_angle(axis, deg):
    a = np.asarray(axis, float) / np.linalg.norm(axis)
    h = math.radians(deg) / 2
    return (*(math.sin(h) * a), math.cos(h))


def tray_scene(n_side=8):
    rng = np.random.default_rng(11)
    bodies = []
    for i in range(n_side):
        for j in range(n_side):
            for k in range(3):
                x = -0.33 + 0.66 * i / (n_side - 1) + rng.uniform(-0.01, 0.01)
                y = -0.33 + 0.66 * j / (n_side - 1) + rng.uniform(-0.01, 0.01)
                bodies.append({"pos": (x, y, 0.5 + 0.11 * k), "radius": 0.04 + 0.01 * rng.uniform(), "mu": 0.4})
    t = 0.05
    walls = [{"kind": "box", "pos": (sx * (0.4 + t), 0.0, 0.2), "half_extents": (t, 0.4 + 2 * t, 0.2), "mu": 0.3}
             for sx in (-1, 1)]
    walls += [{"kind": "box", "pos": (0.0, sy * (0.4 + t), 0.2), "half_extents": (0.4, t, 0.2), "mu": 0.3}
              for sy in (-1, 1)]
    # a turned and tilted block in the middle: spheres land on its faces, edges and corners
    q = quat_axis_angle((0.3, 0.2, 1.0), 35.0)
    statics = [{"kind": "halfspace", "pos": (0, 0, 0), "dir": (0, 0, 1), "mu": 0.4}] + walls + \
              [{"kind": "box", "pos": (0.05, -0.02, 0.12), "half_extents": (0.18, 0.1, 0.08), "quat": q, "mu": 0.5}]
    return make_scene(bodies, statics)


def test_box_statics_bit_identical(oracle_mod):
    s = tray_scene()
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
    # spheres touch the walls and rest on the middle block (static ids 1-4 and 5)
    assert (gc["id_a"] == 5).sum() > 0 and np.isin(gc["id_a"], [1, 2, 3, 4]).sum() > 0
    # nothing leaves the tray
    p = eng.state()["pos"]
    assert np.abs(p[:, :2]).max() < 0.4


def test_box_statics_split_form():
    s = tray_scene()
    cfg = scenes.config_for("pile_1k")
    e64 = PhysicsEngine(cfg).load_scene(s)
    e32 = PhysicsEngine(dict(cfg, **{"gpu.precision": "split"})).load_scene(s)
    e64.step(450)
    e32.step(450)
    c32 = e32.contacts()
    assert (c32["id_a"] == 5).sum() > 0 and np.isin(c32["id_a"], [1, 2, 3, 4]).sum() > 0
    z64, z32 = e64.state()["pos"][:, 2], e32.state()["pos"][:, 2]
    assert np.isfinite(z32).all() and abs(z64.mean() - z32.mean()) < 5e-3
    assert np.abs(e32.state()["pos"][:, :2]).max() < 0.4
    # one converged step from the same state agrees with FP64
    st = e64.state()
    tight = dict(cfg, **{"pj.max_iterations": 3000, "pj.warmstart": False})
    a = PhysicsEngine(tight).load_scene(s)
    b = PhysicsEngine(dict(tight, **{"gpu.precision": "split"})).load_scene(s)
    for e in (a, b):
        e.set_state(st["pos"], st["quat"], st["vel"], st["omega"])
        e.step(1)
    assert a.contacts()["id_a"].shape == b.contacts()["id_a"].shape
    vs = np.abs(st["vel"]).max() + 9.81e-3
    assert np.abs(a.state()["vel"] - b.state()["vel"]).max() <= 1e-3 * vs


# ---- the stacked_spheres scene (examples/scenes/stacked_spheres/StackedSpheresScene.hpp:10-60) ----
R_SPH, N_SPH = 0.05, 20
WALL_T, TUBE_W = R_SPH * 0.25, R_SPH * 3.0
TUBE_H = N_SPH * 2 * R_SPH + 0.5
CUBE_H = 6 * R_SPH


def stacked_spheres_scene():
    # four static box walls around a square tube, the floor box (made static by its trajectory,
    # World::setTrajectory) and a column of spheres resting on it, each touching the next
    hw, ht = WALL_T / 2, TUBE_H / 2
    statics = [{"kind": "box", "pos": (sx * (TUBE_W / 2 + hw), 0.0, ht), "half_extents": (hw, TUBE_W / 2, ht)}
               for sx in (-1, 1)]
    statics += [{"kind": "box", "pos": (0.0, sy * (TUBE_W / 2 + hw), ht), "half_extents": (TUBE_W / 2 + WALL_T, hw, ht)}
                for sy in (-1, 1)]
    statics += [{"kind": "box", "pos": (0.0, 0.0, CUBE_H / 2), "half_extents": (TUBE_W / 2, TUBE_W / 2, CUBE_H / 2)}]
    for st in statics:
        st["mu"] = 0.2
    bodies = []
    z = CUBE_H + R_SPH
    for _ in range(1, N_SPH):
        bodies.append({"pos": (0.0, 0.0, z), "radius": R_SPH, "mass": 1.0, "mu": 0.2})
        z += 2 * R_SPH
    return make_scene(bodies, statics)


def floor_twist(t):
    # the scene's velocity callback: heave A sin(2 pi f t), turn 5 rad/s about x (A = 0.01, f = 10)
    return (0.0, 0.0, 0.01 * math.sin(2 * math.pi * 10.0 * t)), (5.0, 0.0, 0.0)


def stacked_config():
    # the scene's settings (scene.config): dt 5e-3, geometric friction, margin 0, the Nesterov loop
    # with an absolute tolerance; alpha 0.2 instead of 0.01 and a cap of 3,000 sweeps keep it short
    cfg = dict(scenes.config_for("pile_1k"))
    cfg.update({"sim.dt": 5e-3, "friction.combine": "geom", "collision.security_margin": 0.0,
                "collision.match_max_dist": 0.02, "pj.nesterov": True, "pj.alpha": 0.2, "pj.tol_abs": 5e-8,
                "pj.tol_rel": 0.0, "pj.max_iterations": 3000, "pj.warmstart": True})
    return cfg


def test_stacked_spheres_scene_bit_identical(oracle_mod):
    s = stacked_spheres_scene()
    cfg = stacked_config()
    eng = PhysicsEngine(cfg).load_scene(s)
    orc = oracle_mod.Oracle(s, cfg)
    dt = cfg["sim.dt"]
    for k in range(120):
        v, w = floor_twist(k * dt)
        for e in (eng, orc):
            e.set_static_motion([4], vel=[v], omega=[w])
        eng.step(1)
        orc.step(1)
        if k % 20 == 19:
            g, o = eng.state(), orc.state()
            for key in ("pos", "quat", "vel", "omega"):
                assert_same(g[key], o[key], f"{key} after {k + 1} steps")
            gs, os_ = eng.static_state(), orc.static_state()
            for key in ("pos", "quat", "vel", "omega"):
                assert_same(gs[key], os_[key], f"static {key} after {k + 1} steps")
    gc, oc = eng.contacts(), orc.contacts()
    for key in ("id_a", "id_b", "point", "lambda", "normal"):
        assert_same(gc[key], oc[key], f"contact {key}")
    # the floor box has turned about x by 5 rad/s over 119.5 steps (its first drift ran before the
    # first twist), and the column is still in the tube
    q = eng.static_state()["quat"][4]
    assert abs(q[1]) < 1e-12 and abs(q[2]) < 1e-12
    assert abs(2 * math.atan2(q[0], q[3]) - 5.0 * 119.5 * 5e-3) < 1e-3
    p = eng.state()["pos"]
    assert np.isfinite(p).all() and np.abs(p[:, :2]).max() < TUBE_W / 2


def test_stacked_spheres_scene_split_form():
    s = stacked_spheres_scene()
    cfg = stacked_config()
    e64 = PhysicsEngine(dict(cfg, **{"pj.nesterov": False, "pj.max_iterations": 200})).load_scene(s)
    e32 = PhysicsEngine(dict(cfg, **{"pj.nesterov": False, "pj.max_iterations": 200,
                                     "gpu.precision": "split"})).load_scene(s)
    dt = cfg["sim.dt"]
    for k in range(60):
        v, w = floor_twist(k * dt)
        for e in (e64, e32):
            e.set_static_motion([4], vel=[v], omega=[w])
        e64.step(1)
        e32.step(1)
    p64, p32 = e64.state()["pos"], e32.state()["pos"]
    assert np.isfinite(p32).all() and np.abs(p32[:, :2]).max() < TUBE_W / 2
    assert abs(p64[:, 2].mean() - p32[:, 2].mean()) < 2e-2
    np.testing.assert_allclose(e32.static_state()["quat"], e64.static_state()["quat"], atol=1e-12)


def test_box_without_positive_extents_is_refused():
    from cardillocxx_gb300 import CdxError
    cfg = scenes.config_for("pile_1k")
    for ext in ((0.0, 0.2, 0.1), (0.3, -0.2, 0.1), (0.3, float("nan"), 0.1)):
        s = make_scene([{"pos": (0.0, 0.0, 0.5), "radius": 0.05}],
                       [{"kind": "box", "pos": (0, 0, 0), "half_extents": ext}])
        with pytest.raises(CdxError) as e:
            PhysicsEngine(cfg).load_scene(s)
        assert e.value.status == 1, ext
    s = make_scene([{"pos": (0.0, 0.0, 0.5), "radius": 0.05}],
                   [{"kind": "box", "pos": (0, 0, 0), "half_extents": (0.3, 0.2, 0.1)}])
    del s["static_half_extents"]
    with pytest.raises(CdxError) as e:
        PhysicsEngine(cfg).load_scene(s)
    assert e.value.status == 1
