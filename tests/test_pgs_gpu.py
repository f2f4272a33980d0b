"""Projected Gauss-Seidel (solver.type=projected_gauss_seidel) in the plain FP64 method, against the
oracle's restatement of ProjectedGaussSeidelSolver::solve (projected_gauss_seidel.cpp:56-264): the
GPU runs a sweep's blocks in parallel wherever the sequential order lets it (a block waits for the
previous block of each of its bodies), so every block sees the velocities of the sequential sweep
and the results are compared bit for bit."""
import numpy as np
import pytest

from cardillocxx_gb300 import CdxError, PhysicsEngine, scenes

pytestmark = pytest.mark.gpu

PGS = {"solver.type": "projected_gauss_seidel", "gpu.precision": "fp64", "pj.tol_abs": 1e-6, "pj.tol_rel": 1e-6,
       "pj.max_iterations": 5000}


def assert_same(a, b, what):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape, (what, a.shape, b.shape)
    if not np.array_equal(a, b):
        raise AssertionError(f"{what}: not bit-identical, max |diff| {np.nanmax(np.abs(a - b)):.3e}")


def run_pair(oracle_mod, scene, cfg, steps, every=1):
    eng = PhysicsEngine(cfg).load_scene(scene)
    orc = oracle_mod.Oracle(scene, cfg, omp_mode=1)
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


def test_pgs_pile_bit_identical(oracle_mod):
    s = scenes.generate("pile_1k", scale=0.3)
    cfg = scenes.config_for("pile_1k", **PGS)
    eng, _ = run_pair(oracle_mod, s, cfg, 150, every=25)
    st = eng.stats()
    assert st["num_contacts"] > 50 and 1 < st["iterations"] < 5000


def test_pgs_relaxation_alpha_mixtures_restitution_and_drum(oracle_mod):
    # pj.relaxation and pj.alpha both scale the update; frictionless and frictional blocks (the
    # frictionless ones first in the row order), restitution in the bias, implicit gyroscopy, a
    # rotating drum wall (contact velocity in rhs)
    s = scenes.generate("pile_1k", scale=0.08)
    s["mu"][::3] = 0.0
    s["rest_n"][::2] = 0.3
    s["rest_t"][::5] = 0.2
    cfg = scenes.config_for("pile_1k", **dict(PGS, **{"pj.relaxation": 0.8, "pj.alpha": 0.9,
                                                      "moreau.implicit_gyroscopy": True}))
    run_pair(oracle_mod, s, cfg, 60, every=20)
    d = scenes.generate("drum_1m", num_bodies=150, r=(0.02, 0.03), drum=(0.3, 0.3, 2.0))
    cd = scenes.config_for("drum_1m", **dict(PGS, **{"sim.dt": 1e-3}))
    run_pair(oracle_mod, d, cd, 40, every=20)


def test_pgs_settled_200k_pile_bit_identical(oracle_mod):
    # the committed 200k-sphere pile: bodies are numbered bottom-up, so a sweep's chains of
    # dependent blocks run through the whole height of the pile (about 1,000 blocks deep)
    import os
    path = os.path.join(os.path.dirname(__file__), "golden", "pile_200k_settled.npz")
    s = scenes.settled_pile(path)
    cfg = scenes.config_for("pile_200k", **dict(PGS, **{"pj.max_iterations": 4, "pj.tol_abs": 1e-9,
                                                        "pj.tol_rel": 1e-9}))
    eng, _ = run_pair(oracle_mod, s, cfg, 2, every=1)
    assert eng.stats()["num_contacts"] > 400000 and eng.stats()["iterations"] == 4


def test_pgs_without_tolerance_diverges_like_the_reference(oracle_mod):
    # pj.tol_abs = pj.tol_rel = 0 makes the residual a division by zero: the reference throws
    # "Projected Gauss-Seidel diverged" at the first sweep; here the step reports CDX_ERR_NONFINITE
    s = scenes.generate("pile_1k", scale=0.05)
    base = scenes.config_for("pile_1k")
    ref = PhysicsEngine(base).load_scene(s)
    ref.step(300)
    st = ref.state()
    sc = dict(s)
    for k in st:
        sc[k] = st[k].copy()
    cfg = dict(base, **{"solver.type": "pgs", "gpu.precision": "fp64"})
    e = PhysicsEngine(cfg).load_scene(sc)
    with pytest.raises(CdxError) as err:
        e.step(1)
    assert err.value.status == 4 and "Gauss-Seidel diverged" in str(err.value)
    with pytest.raises(RuntimeError):
        oracle_mod.Oracle(sc, cfg).step(1)


def test_pgs_wait_timeout_then_recovers():
    # a wait limit far below a sweep's time makes the cooperative solve give up at its first wait:
    # the step fails with CDX_ERR_TIMEOUT and the context keeps working once the limit is restored
    s = scenes.generate("pile_1k", scale=0.3)
    cfg = scenes.config_for("pile_1k", **PGS)
    e = PhysicsEngine(cfg).load_scene(s)
    e.step(100)
    st = e.state()
    e.set_config(dict(cfg, **{"gpu.coop_wait_ns": 1}))
    with pytest.raises(CdxError) as err:
        e.step(1)
    assert err.value.status == 5
    e.set_config(cfg)
    e.set_state(**st)
    e.step(5)
    assert np.isfinite(e.state()["vel"]).all() and e.stats()["iterations"] >= 1


def test_pgs_agrees_with_projected_jacobi_at_convergence():
    s = scenes.generate("pile_1k", scale=0.3)
    base = scenes.config_for("pile_1k")
    ref = PhysicsEngine(base).load_scene(s)
    ref.step(250)
    st = ref.state()
    sc = dict(s)
    for k in st:
        sc[k] = st[k].copy()
    tight = {"pj.tol_abs": 1e-9, "pj.tol_rel": 1e-9, "pj.max_iterations": 100000, "pj.warmstart": False,
             "gpu.precision": "fp64"}
    e_pj = PhysicsEngine(dict(base, **tight)).load_scene(sc)
    e_gs = PhysicsEngine(dict(base, **tight, **{"solver.type": "pgs", "pj.alpha": 1.0,
                                                "pj.relaxation": 1.0})).load_scene(sc)
    e_pj.step(1)
    e_gs.step(1)
    vs = np.abs(st["vel"]).max() + 9.81e-3
    assert np.abs(e_pj.state()["vel"] - e_gs.state()["vel"]).max() <= 1e-6 * vs
    assert e_gs.stats()["iterations"] < e_pj.stats()["iterations"]
    assert (e_gs.contacts()["lambda"][:, 0] >= 0).all()
