"""Edge cases of the scene: no bodies, no statics, a batched scene whose middle scene is empty, and
a scene whose spheres never touch. Both GPU forms step them; the plain FP64 method stays bit-identical
to the oracle."""
import numpy as np
import pytest

from cardillocxx_gb300 import PhysicsEngine, scenes
from cardillocxx_gb300.scenes import make_scene

pytestmark = pytest.mark.gpu

FORMS = ({"gpu.precision": "fp64"}, {"gpu.precision": "split"})


def assert_same(a, b, what):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape, (what, a.shape, b.shape)
    if not np.array_equal(a, b):
        raise AssertionError(f"{what}: not bit-identical, max |diff| {np.nanmax(np.abs(a - b)):.3e}")


def test_scene_without_bodies_steps():
    s = make_scene([], [{"kind": "halfspace", "pos": (0, 0, 0), "dir": (0, 0, 1)}])
    for over in FORMS:
        e = PhysicsEngine(dict(scenes.config_for("pile_1k"), **over)).load_scene(s)
        e.step(3)
        assert e.stats()["num_contacts"] == 0
        assert e.state()["pos"].shape == (0, 3)


def test_scene_without_statics_matches_the_oracle(oracle_mod):
    # two spheres meet head on in zero gravity: one pair contact, no statics at all
    bodies = [{"pos": (-0.2, 0.0, 0.0), "radius": 0.1, "vel": (1.0, 0.0, 0.0)},
              {"pos": (0.2, 0.01, 0.0), "radius": 0.1, "vel": (-1.0, 0.0, 0.0)}]
    s = make_scene(bodies, [])
    cfg = dict(scenes.config_for("pile_1k"), **{"sim.gravity": (0.0, 0.0, 0.0)})
    eng = PhysicsEngine(cfg).load_scene(s)
    orc = oracle_mod.Oracle(s, cfg)
    eng.step(300)
    orc.step(300)
    g, o = eng.state(), orc.state()
    for key in ("pos", "quat", "vel", "omega"):
        assert_same(g[key], o[key], key)
    # they met: without restitution the normal approach speed is gone, momentum stays zero
    np.testing.assert_allclose(g["vel"].sum(axis=0), 0.0, atol=1e-12)
    assert np.abs(g["vel"][:, 0]).max() < 0.05
    split = PhysicsEngine(dict(cfg, **{"gpu.precision": "split"})).load_scene(s)
    split.step(300)
    np.testing.assert_allclose(split.state()["vel"], g["vel"], atol=1e-5)


def test_batched_scene_with_an_empty_scene_in_the_middle(oracle_mod):
    # scenes 0 and 2 hold spheres resting on their ground; scene 1 holds only its ground
    bodies, ids = [], []
    for sc in (0, 2):
        for k in range(3):
            bodies.append({"pos": (0.3 * k, 0.0, 0.05 + 0.02 * k), "radius": 0.05})
            ids.append(sc)
    statics = [{"kind": "halfspace", "pos": (0, 0, 0), "dir": (0, 0, 1)} for _ in range(3)]
    s = make_scene(bodies, statics, scene_ids=ids, static_scene_ids=[0, 1, 2])
    cfg = scenes.config_for("pile_1k")
    eng = PhysicsEngine(cfg).load_scene(s)
    orc = oracle_mod.Oracle(s, cfg)
    eng.step(100)
    orc.step(100)
    for key in ("pos", "vel"):
        assert_same(eng.state()[key], orc.state()[key], key)
    split = PhysicsEngine(dict(cfg, **{"gpu.precision": "split"})).load_scene(s)
    split.step(100)
    # the spheres placed exactly on their ground (gap 0, security margin 0): the split form's FP32
    # impulses leave them a few 1e-10 m/s, which can lift one 1e-13 m clear, so it falls for a step
    # (g h^2 = 1e-5 m) before its contact returns; the FP64 method keeps them exactly in place
    np.testing.assert_allclose(split.state()["pos"], eng.state()["pos"], atol=2e-5)
    c = eng.contacts()
    assert set(c["id_a"].tolist()) == {0, 2}  # no contact with the empty scene's ground


def test_spheres_that_never_touch():
    # a 6 x 6 x 6 lattice of spacing 0.5 m, jittered by at most 0.05 m: centres at least 0.4 m apart
    rng = np.random.default_rng(3)
    bodies = [{"pos": tuple(0.5 * np.array([i, j, k]) + rng.uniform(-0.05, 0.05, 3)), "radius": 0.05,
               "vel": tuple(rng.uniform(-1, 1, 3))} for i in range(6) for j in range(6) for k in range(6)]
    s = make_scene(bodies, [])
    for over in FORMS:
        e = PhysicsEngine(dict(scenes.config_for("pile_1k"), **over, **{"sim.gravity": (0.0, 0.0, 0.0)})).load_scene(s)
        e.step(5)
        assert e.stats()["num_contacts"] == 0
        v = np.array([b["vel"] for b in bodies])
        np.testing.assert_allclose(e.state()["vel"], v, rtol=0, atol=1e-12)
