"""The condensed solver (solver.type=condensed) in the plain FP64 method, against the oracle's restatement
of CondensedSolver::solve (condensed_solver.cpp:443-760), for its three deterministic sweep modes:
colored (the GPU's Jones-Plassmann rounds give the greedy Welsh-Powell colors), gauss_seidel (the
sequential order, run through the per-body chains of blocks) and jacobi (two passes). The same
per-block updates in the same order and the same stop test: the results are compared bit for bit.
The converged solution also agrees with projected Jacobi's."""
import numpy as np
import pytest

from cardillocxx_gb300 import CdxError, PhysicsEngine, scenes
from cardillocxx_gb300.scenes import make_scene

pytestmark = pytest.mark.gpu

COND = {"solver.type": "condensed", "condensed.sweep_mode": "colored", "pj.tol_abs": 1e-6, "pj.tol_rel": 1e-6,
        "pj.max_iterations": 5000}


def assert_same(a, b, what):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape, (what, a.shape, b.shape)
    if not np.array_equal(a, b):
        raise AssertionError(f"{what}: not bit-identical, max |diff| {np.nanmax(np.abs(a - b)):.3e}")


def run_pair(oracle_mod, scene, cfg, steps, every=1):
    eng = PhysicsEngine(cfg).load_scene(scene)
    orc = oracle_mod.Oracle(scene, cfg)
    done = 0
    while done < steps:
        k = min(every, steps - done)
        eng.step(k)
        orc.step(k)
        done += k
        g, o = eng.state(), orc.state()
        for key in ("pos", "quat", "vel", "omega"):
            assert_same(g[key], o[key], f"{key} after {done} steps")
        gc, oc = eng.contacts(), orc.contacts()
        for key in ("id_a", "id_b", "point", "lambda"):
            assert_same(gc[key], oc[key], f"contact {key} after {done} steps")
        gs, os_ = eng.stats(), orc.stats()
        assert gs["iterations"] == os_["iterations"], (gs["iterations"], os_["iterations"])
        assert gs["residual_last"] == os_["residual_last"]
        assert gs["residual"] == os_["residual"]
    return eng, orc


def test_condensed_colored_pile_bit_identical(oracle_mod):
    s = scenes.generate("pile_1k", scale=0.3)
    cfg = scenes.config_for("pile_1k", **COND)
    eng, _ = run_pair(oracle_mod, s, cfg, 150, every=25)
    st = eng.stats()
    assert st["num_contacts"] > 50 and 1 < st["iterations"] < 5000


def test_condensed_colored_relaxation_alpha_and_mixtures(oracle_mod):
    # pj.relaxation multiplies pj.alpha in the condensed update; frictionless and frictional blocks
    # (a zero-friction subset), a rotating drum wall (contact velocity in rhs), implicit gyroscopy
    s = scenes.generate("pile_1k", scale=0.08)
    s["mu"][::3] = 0.0
    cfg = scenes.config_for("pile_1k", **dict(COND, **{"pj.relaxation": 0.8, "pj.alpha": 0.9,
                                                       "moreau.implicit_gyroscopy": True}))
    run_pair(oracle_mod, s, cfg, 60, every=20)
    d = scenes.generate("drum_1m", num_bodies=150, r=(0.02, 0.03), drum=(0.3, 0.3, 2.0))
    cd = scenes.config_for("drum_1m", **dict(COND, **{"sim.dt": 1e-3}))
    run_pair(oracle_mod, d, cd, 40, every=20)


def test_condensed_without_tolerance_diverges_like_the_reference(oracle_mod):
    # with pj.tol_abs = pj.tol_rel = 0 the residual is a division by zero: the reference throws
    # "Condensed solver diverged" at the first sweep; here the step reports CDX_ERR_NONFINITE
    s = scenes.generate("pile_1k", scale=0.05)
    base = scenes.config_for("pile_1k")
    ref = PhysicsEngine(base).load_scene(s)
    ref.step(300)  # resting: contacts exist
    st = ref.state()
    sc = dict(s)
    for k in st:
        sc[k] = st[k].copy()
    cfg = dict(base, **{"solver.type": "condensed", "condensed.sweep_mode": "colored"})
    e = PhysicsEngine(cfg).load_scene(sc)
    with pytest.raises(CdxError) as err:
        e.step(1)
    assert err.value.status == 4 and "diverged" in str(err.value)
    with pytest.raises(RuntimeError):
        oracle_mod.Oracle(sc, cfg).step(1)


def test_condensed_agrees_with_projected_jacobi_at_convergence():
    s = scenes.generate("pile_1k", scale=0.3)
    base = scenes.config_for("pile_1k")
    ref = PhysicsEngine(base).load_scene(s)
    ref.step(250)
    st = ref.state()
    sc = dict(s)
    for k in st:
        sc[k] = st[k].copy()
    tight = {"pj.tol_abs": 1e-9, "pj.tol_rel": 1e-9, "pj.max_iterations": 100000, "pj.warmstart": False}
    e_pj = PhysicsEngine(dict(base, **tight)).load_scene(sc)
    e_cd = PhysicsEngine(dict(base, **tight, **{"solver.type": "condensed", "condensed.sweep_mode": "colored",
                                                "pj.alpha": 1.0, "pj.relaxation": 1.0})).load_scene(sc)
    e_pj.step(1)
    e_cd.step(1)
    vs = np.abs(st["vel"]).max() + 9.81e-3
    assert np.abs(e_pj.state()["vel"] - e_cd.state()["vel"]).max() <= 1e-4 * vs
    # colored Gauss-Seidel with alpha 1 needs fewer sweeps than Jacobi with alpha 0.5
    assert e_cd.stats()["iterations"] < e_pj.stats()["iterations"]
    # the stored impulses: normal compressive (non-negative), tangential in the solver's own convention
    # (opposite to projected Jacobi's). A pile's impulses need not be unique where its velocities
    # are, so only their conventions are compared.
    cd, pj = e_cd.contacts(), e_pj.contacts()
    assert (cd["lambda"][:, 0] >= 0).all()
    t_cd, t_pj = cd["lambda"][:, 1:], pj["lambda"][:, 1:]
    if np.abs(t_pj).max() > 0:
        assert np.sum(t_cd * t_pj) < 0


@pytest.mark.parametrize("mode", ["gauss_seidel", "jacobi"])
def test_condensed_sequential_and_jacobi_modes_bit_identical(oracle_mod, mode):
    s = scenes.generate("pile_1k", scale=0.3)
    cfg = scenes.config_for("pile_1k", **dict(COND, **{"condensed.sweep_mode": mode}))
    eng, _ = run_pair(oracle_mod, s, cfg, 150, every=50)
    st = eng.stats()
    assert st["num_contacts"] > 50 and 1 < st["iterations"] < 5000
    # a frictionless subset, relaxation and alpha below 1, implicit gyroscopy
    s2 = scenes.generate("pile_1k", scale=0.08)
    s2["mu"][::3] = 0.0
    c2 = scenes.config_for("pile_1k", **dict(COND, **{"condensed.sweep_mode": mode, "pj.relaxation": 0.8,
                                                      "pj.alpha": 0.9, "moreau.implicit_gyroscopy": True}))
    run_pair(oracle_mod, s2, c2, 40, every=20)


def test_condensed_default_mode_is_sequential_gauss_seidel():
    # condensed.sweep_mode defaults to gauss_seidel (config.hpp:118), which now runs as is
    s = scenes.generate("pile_1k", scale=0.05)
    e = PhysicsEngine(scenes.config_for("pile_1k", **{"solver.type": "condensed", "pj.tol_abs": 1e-6,
                                                      "pj.tol_rel": 1e-6})).load_scene(s)
    e.step(300)
    assert np.isfinite(e.state()["vel"]).all() and e.stats()["num_contacts"] > 0 and e.stats()["levels"] >= 1
