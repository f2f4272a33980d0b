"""Prescribed static motion (the results of Trajectory::update, trajectory.cpp:69-120, evaluated on the
host and applied after the first drift, where updateStateDependentTerms runs it): the plain FP64
method against the oracle, bit for bit, over a run whose ground and drum move every step; the split
form beside it."""
import math

import numpy as np
import pytest

from cardillocxx_gb300 import PhysicsEngine, scenes

pytestmark = pytest.mark.gpu


def assert_same(a, b, what):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape, (what, a.shape, b.shape)
    if not np.array_equal(a, b):
        raise AssertionError(f"{what}: not bit-identical, max |diff| {np.nanmax(np.abs(a - b)):.3e}")


def ground_motion(t):
    # a conveyor ground that also heaves: velocity only (a halfspace's plane stays where it was built)
    return {"vel": [(0.2 * math.sin(40.0 * t), 0.0, 0.05 * math.cos(40.0 * t))]}


def drum_motion(t):
    # the drum's centre follows a prescribed path; its velocity is that path's difference quotient,
    # as Trajectory::update differentiates a position callback
    def p(tt):
        return (0.0, 0.0, 0.01 * math.sin(25.0 * tt))
    h = 1e-3
    p0, p1 = p(t), p(t + h)
    return {"pos": [p0], "quat": [(0.0, 0.0, 0.0, 1.0)], "vel": [tuple((b - a) / h for a, b in zip(p0, p1))],
            "omega": [(1.5, 0.0, 0.0)]}


def run_pair(oracle_mod, scene, cfg, steps, motion, statics):
    eng = PhysicsEngine(cfg).load_scene(scene)
    orc = oracle_mod.Oracle(scene, cfg)
    dt = cfg["sim.dt"]
    for k in range(steps):
        m = motion(k * dt)
        eng.set_static_motion(statics, **m)
        orc.set_static_motion(statics, **m)
        eng.step(1)
        orc.step(1)
        g, o = eng.state(), orc.state()
        for key in ("pos", "quat", "vel", "omega"):
            assert_same(g[key], o[key], f"{key} after {k + 1} steps")
        gs, os_ = eng.static_state(), orc.static_state()
        for key in ("pos", "quat", "vel", "omega"):
            assert_same(gs[key], os_[key], f"static {key} after {k + 1} steps")
    gc, oc = eng.contacts(), orc.contacts()
    for key in ("id_a", "id_b", "point", "lambda"):
        assert_same(gc[key], oc[key], f"contact {key}")
    return eng


def test_prescribed_ground_motion_bit_identical(oracle_mod):
    s = scenes.generate("pile_1k", scale=0.1)
    cfg = scenes.config_for("pile_1k")
    ref = PhysicsEngine(cfg).load_scene(s)
    ref.step(200)
    st = ref.state()
    for k in st:
        s[k] = st[k].copy()
    eng = run_pair(oracle_mod, s, cfg, 40, ground_motion, [0])
    assert eng.stats()["num_contacts"] > 20


def test_prescribed_drum_motion_bit_identical_and_split(oracle_mod):
    d = scenes.generate("drum_1m", num_bodies=120, r=(0.02, 0.03), drum=(0.3, 0.3, 2.0))
    cfg = scenes.config_for("drum_1m", **{"sim.dt": 1e-3})
    ref = PhysicsEngine(cfg).load_scene(d)
    ref.step(300)
    st = ref.state()
    for k in st:
        d[k] = st[k].copy()
    e64 = run_pair(oracle_mod, d, cfg, 40, drum_motion, [0])
    # the split form with the same motion: finite, and close to the FP64 run
    e32 = PhysicsEngine(dict(cfg, **{"gpu.precision": "split"})).load_scene(d)
    for k in range(40):
        e32.set_static_motion([0], **drum_motion(k * 1e-3))
        e32.step(1)
    v32, v64 = e32.state()["vel"], e64.state()["vel"]
    assert np.isfinite(v32).all()
    vs = np.abs(v64).max() + 9.81e-3
    assert np.abs(v32 - v64).max() <= 0.05 * vs
    assert_same(e32.static_state()["pos"], e64.static_state()["pos"], "split static position")


def test_prescribed_motion_rejects_bad_input():
    from cardillocxx_gb300 import CdxError
    s = scenes.generate("pile_1k", scale=0.05)
    e = PhysicsEngine(scenes.config_for("pile_1k")).load_scene(s)
    with pytest.raises(CdxError):
        e.set_static_motion([99], vel=[(0.0, 0.0, 1.0)])
    with pytest.raises(CdxError):
        e.set_static_motion([0], vel=[(float("nan"), 0.0, 0.0)])
