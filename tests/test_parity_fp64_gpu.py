"""Parity of the plain FP64 GPU method against the CPU oracle (GPU tests).

The bar set by the path's definition is impulses within 1e-10 relative per iteration and
trajectories within 1e-9 over the run; the plain method is built to be bit-identical (same
operation order, no FMA contraction, deterministic gathers), so these tests assert exact equality
and report the largest difference when it fails.
"""
import os

import numpy as np
import pytest

from cardillocxx_gb300 import PhysicsEngine, scenes
from cardillocxx_gb300.scenes import make_scene

pytestmark = pytest.mark.gpu

IT_RTOL = 1e-10   # per-iteration impulse tolerance (relative)
TRAJ_TOL = 1e-9   # trajectory tolerance over the run


def _max_rel(a, b):
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    if a.size == 0:
        return 0.0
    den = np.maximum(np.abs(b), 1e-300)
    return float(np.max(np.abs(a - b) / np.maximum(den, np.max(np.abs(b)) * 1e-300 + 1e-300)))


def assert_same(a, b, what, atol=0.0):
    a = np.asarray(a)
    b = np.asarray(b)
    assert a.shape == b.shape, (what, a.shape, b.shape)
    if atol == 0.0:
        if not np.array_equal(a, b):
            d = np.abs(a.astype(float) - b.astype(float))
            raise AssertionError(f"{what}: not bit-identical, max |diff| {np.nanmax(d):.3e}")
    else:
        np.testing.assert_allclose(a, b, rtol=0, atol=atol, err_msg=what)


def run_pair(oracle_mod, scene, cfg, nsteps, check_every=None):
    eng = PhysicsEngine(cfg).load_scene(scene)
    orc = oracle_mod.Oracle(scene, cfg)
    check_every = check_every or nsteps
    done = 0
    while done < nsteps:
        k = min(check_every, nsteps - done)
        eng.step(k)
        orc.step(k)
        done += k
        g, o = eng.state(), orc.state()
        for key in ("pos", "quat", "vel", "omega"):
            assert_same(g[key], o[key], f"{key} after {done} steps")
        gc, oc = eng.contacts(), orc.contacts()
        for key in ("id_a", "id_b", "point", "lambda", "normal"):
            assert_same(gc[key], oc[key], f"contact {key} after {done} steps")
        gs, os_ = eng.stats(), orc.stats()
        assert gs["iterations"] == os_["iterations"]
        assert gs["num_contacts"] == os_["num_contacts"]
        assert gs["num_rows"] == os_["num_rows"]
        assert gs["residual"] == os_["residual"]
    return eng, orc


def test_known_answer_scenes(gpu, oracle_mod):
    ground = {"kind": "halfspace", "pos": (0, 0, 0), "dir": (0, 0, 1), "mu": 0.3}
    drum = {"kind": "drum", "pos": (0, 0, 0), "dir": (1, 0, 0), "radius": 1.0, "omega": (2.0, 0, 0), "mu": 0.4}
    cfg = scenes.config_for("pile_1k")
    cases = [
        make_scene([{"pos": (0.0, 0.0, 0.05), "radius": 0.05, "vel": (1.0, 0, 0)}], [ground]),
        make_scene([{"pos": (0.5, 0.0, -0.9), "radius": 0.1, "mu": 0.4}], [drum]),
        make_scene([{"pos": (0.2, 0.3, 5.0), "radius": 0.05, "vel": (0.3, -0.2, 1.0)}], [ground]),
        make_scene([{"pos": (0.0, 0.0, 0.05), "radius": 0.05}, {"pos": (0.0, 0.0, 0.15), "radius": 0.05}], [ground]),
    ]
    for s in cases:
        run_pair(oracle_mod, s, cfg, 20, 5)


def test_pile_small_bit_identical(gpu, oracle_mod):
    s = scenes.generate("pile_1k", scale=0.2)
    run_pair(oracle_mod, s, scenes.config_for("pile_1k"), 240, 40)


def test_per_iteration_impulses(gpu, oracle_mod):
    s = scenes.generate("pile_1k", scale=0.3)
    cfg = scenes.config_for("pile_1k")
    eng, orc = run_pair(oracle_mod, s, cfg, 200, 200)
    eng.set_trace(True)
    orc.set_trace(True)
    eng.step(1)
    orc.step(1)
    nrows = orc.stats()["num_rows"]
    assert nrows > 0
    tg, to = eng.trace(nrows), orc.trace(nrows)
    assert tg.shape == to.shape and tg.shape[0] == 50
    scale = np.maximum(np.abs(to).max(axis=1, keepdims=True), 1e-300)
    rel = np.abs(tg - to) / scale
    assert rel.max() <= IT_RTOL, f"per-iteration impulse rel diff {rel.max():.3e}"
    assert_same(tg, to, "trace")


def test_pile_1k_full_run_trajectory(gpu, oracle_mod):
    # the 1,000-sphere pile over its full 500 steps (the plain method's CPU-runnable case)
    s = scenes.generate("pile_1k")
    cfg = scenes.config_for("pile_1k")
    eng = PhysicsEngine(cfg).load_scene(s)
    orc = oracle_mod.Oracle(s, cfg, omp_mode=1)
    eng.step(500)
    orc.step(500)
    g, o = eng.state(), orc.state()
    for key in ("pos", "quat", "vel", "omega"):
        d = np.abs(g[key] - o[key]).max()
        assert d <= TRAJ_TOL, f"{key} trajectory diff {d:.3e}"
        assert_same(g[key], o[key], key)


def test_batched_scenes_parity(gpu, oracle_mod):
    s = scenes.generate("batch_4096", scale=0.005)
    assert s["num_scenes"] > 10
    run_pair(oracle_mod, s, scenes.config_for("batch_4096"), 60, 30)


def test_drum_parity(gpu, oracle_mod):
    s = scenes.generate("drum_1m", scale=0.0004)
    run_pair(oracle_mod, s, scenes.config_for("drum_1m"), 60, 20)


def test_frictionless_mixture_and_options(gpu, oracle_mod):
    s = scenes.generate("pile_1k", scale=0.15)
    s["mu"][::3] = 0.0  # a third of the spheres frictionless: rows partitioned frictionless-first
    cfg = scenes.config_for("pile_1k", **{"pj.warmstart": True, "friction.combine": "arith"})
    run_pair(oracle_mod, s, cfg, 120, 60)
    cfg2 = scenes.config_for("pile_1k", **{"friction.enable": False, "pj.warmstart": False})
    run_pair(oracle_mod, s, cfg2, 80, 40)


def test_stop_rules_match(gpu, oracle_mod):
    s = scenes.generate("pile_1k", scale=0.15)
    # the reference's velocity-increment test (every 10th sweep) and the residual test
    cfg = scenes.config_for("pile_1k", **{"pj.tol_abs": 1e-6, "pj.tol_rel": 1e-4, "pj.max_iterations": 200})
    run_pair(oracle_mod, s, cfg, 100, 50)
    cfg2 = scenes.config_for("pile_1k", **{"gpu.residual_tol": 1e-3, "pj.max_iterations": 200})
    run_pair(oracle_mod, s, cfg2, 100, 50)


def test_csr_solver_dropin(gpu, oracle_mod):
    rng = np.random.default_rng(7)
    nb = 40
    nv = 6 * nb
    nfl = 6
    nfr = 30
    rows, cols, vals = [], [], []
    ptr = [0]
    for r in range(nfl + 3 * nfr):
        a, b = sorted(rng.choice(nb, 2, replace=False))
        for body in (a, b):
            for k in range(6):
                cols.append(6 * body + k)
                vals.append(rng.normal())
        ptr.append(len(cols))
    ptr = np.array(ptr, np.int32)
    col = np.array(cols, np.int32)
    val = np.array(vals)
    nrows = nfl + 3 * nfr
    m = rng.uniform(0.5, 2.0, nv)
    args = dict(row_ptr=ptr, col=col, val=val, contact_bias=rng.normal(size=nrows) * 0.1,
                mu=rng.uniform(0.1, 0.6, nrows), restitution=rng.uniform(0, 0.2, nrows), minv=1.0 / m,
                mdiag=1.0 / (1.0 / m), v=rng.normal(size=nv), f_ext=rng.normal(size=nv), f_gyro=rng.normal(size=nv) * 1e-3,
                dt=1e-3, alpha=0.3, max_iter=40, tol_abs=0.0, tol_rel=0.0, lam0=np.abs(rng.normal(size=nrows)) * 0.01,
                nfl=nfl)
    xo, lo, ito = oracle_mod.pj_solve_csr(**args)
    eng = PhysicsEngine(scenes.config_for("pile_1k"))
    xg, lg, itg = eng.pj_solve_csr(**args)
    assert ito == itg == 40
    assert_same(xg, xo, "csr x")
    assert_same(lg, lo, "csr lambda")
    args.update(tol_abs=1e-7, tol_rel=1e-5, max_iter=2000)
    xo, lo, ito = oracle_mod.pj_solve_csr(**args)
    xg, lg, itg = eng.pj_solve_csr(**args)
    assert ito == itg
    assert_same(xg, xo, "csr x (early exit)")


def test_csr_dropin_across_fresh_contexts(gpu, oracle_mod):
    # contexts created and destroyed in turn (a new one may reuse the old one's address) each keep
    # their own work buffers
    rng = np.random.default_rng(5)
    nb, nv = 10, 60
    cols, vals, ptr = [], [], [0]
    for _ in range(3 * 8):
        a, b = sorted(rng.choice(nb, 2, replace=False))
        for body in (a, b):
            for k in range(6):
                cols.append(6 * body + k)
                vals.append(rng.normal())
        ptr.append(len(cols))
    m = rng.uniform(0.5, 2.0, nv)
    args = dict(row_ptr=np.array(ptr, np.int32), col=np.array(cols, np.int32), val=np.array(vals),
                contact_bias=np.zeros(24), mu=np.full(24, 0.4), restitution=np.zeros(24), minv=1.0 / m,
                mdiag=1.0 / (1.0 / m), v=rng.normal(size=nv), f_ext=rng.normal(size=nv), f_gyro=np.zeros(nv), dt=1e-3,
                alpha=0.3, max_iter=30, tol_abs=0.0, tol_rel=0.0, lam0=np.zeros(24))
    xo, lo, _ = oracle_mod.pj_solve_csr(**args)
    for _ in range(4):
        eng = PhysicsEngine({})
        x, lam, _ = eng.pj_solve_csr(**args)
        eng.close()
        del eng
        assert_same(x, xo, "csr x, fresh context")
        assert_same(lam, lo, "csr lambda, fresh context")


def test_accelerated_loops_bit_identical(gpu, oracle_mod):
    # Nesterov and Chebyshev loops of the reference (projected_jacobi.cpp:379-449, 179-222): the
    # GPU runs the same sweeps, extrapolations, restarts and stop tests as the oracle, bit for bit
    s = scenes.generate("pile_1k", scale=0.2)
    for extra in ({"pj.nesterov": True}, {"pj.chebyshev": True},
                  {"pj.nesterov": True, "pj.nesterov_beta_threshold": 0.5, "pj.nesterov_restart_limit": 3},
                  {"pj.anderson": True}, {"pj.anderson": True, "pj.anderson_m": 5}):
        cfg = scenes.config_for("pile_1k", **{"pj.tol_abs": 1e-6, "pj.tol_rel": 1e-5, "pj.max_iterations": 400,
                                              **extra})
        eng, orc = run_pair(oracle_mod, s, cfg, 150, 50)
        assert orc.stats()["iterations"] < 400


def test_accelerated_loops_with_zero_tolerances_run_the_cap(gpu, oracle_mod):
    # with both tolerances 0 the reference's residual is not finite: Nesterov restarts every sweep,
    # Chebyshev and Anderson never stop early; all still match the oracle
    s = scenes.generate("pile_1k", scale=0.15)
    for extra in ({"pj.nesterov": True}, {"pj.chebyshev": True}, {"pj.anderson": True}):
        cfg = scenes.config_for("pile_1k", **extra)
        eng, orc = run_pair(oracle_mod, s, cfg, 60, 30)
        assert orc.stats()["iterations"] == cfg["pj.max_iterations"]


def test_true_delassus_block_preconditioner(gpu, oracle_mod):
    # pj.rdiag_true_delassus (projected_jacobi.cpp:81-98, 341-347): per-contact Delassus blocks,
    # the step-wide diagonal test and the per-row application, with frictionless contacts mixed in,
    # under the standard and the Chebyshev loop; bit for bit against the oracle
    s = scenes.generate("pile_1k", scale=0.15)
    s["mu"][::3] = 0.0
    for extra in ({}, {"pj.chebyshev": True}, {"friction.enable": False}):
        cfg = scenes.config_for("pile_1k", **{"pj.rdiag_true_delassus": True, "friction.combine": "min", **extra})
        run_pair(oracle_mod, s, cfg, 80, 40)


def test_csr_dropin_with_configuration(gpu, oracle_mod):
    # cdx_pj_solve_csr_cfg: the solver-level drop-in under the reference's pj.* settings, bit for bit
    # against the oracle: every loop, with and without the Delassus block preconditioner. W here is
    # general (its 3x3 blocks are not diagonal), so the blocks take the Cholesky inverse.
    from tests.csr_cases import csr_problem
    p = csr_problem()
    eng = PhysicsEngine(scenes.config_for("pile_1k"))
    base = {"pj.alpha": 0.3, "pj.max_iterations": 400, "pj.tol_abs": 1e-9, "pj.tol_rel": 1e-8}
    for block in (False, True):
        for extra in ({}, {"pj.nesterov": True}, {"pj.chebyshev": True}, {"pj.anderson": True},
                      {"pj.anderson": True, "pj.anderson_m": 4},
                      {"pj.nesterov": True, "pj.nesterov_beta_threshold": 0.5, "pj.nesterov_restart_limit": 3}):
            cfg = dict(base, **extra, **{"pj.rdiag_true_delassus": block})
            xo, lo, ito = oracle_mod.pj_solve_csr_cfg(cfg, **p)
            xg, lg, itg = eng.pj_solve_csr_cfg(cfg, **p)
            what = f"block={block} {extra}"
            assert itg == ito, what
            assert_same(xg, xo, "x " + what)
            assert_same(lg, lo, "lambda " + what)


def test_implicit_gyroscopy_parity(gpu, oracle_mod):
    # moreau.implicit_gyroscopy: spinning spheres, bit for bit against the oracle; the split form
    # follows the plain method to FP32 order
    s = scenes.generate("pile_1k", scale=0.15)
    s["omega"] = np.random.default_rng(3).normal(size=s["omega"].shape) * 20.0
    cfg = scenes.config_for("pile_1k", **{"moreau.implicit_gyroscopy": True})
    run_pair(oracle_mod, s, cfg, 60, 30)
    e32 = PhysicsEngine(dict(cfg, **{"gpu.precision": "split"})).load_scene(s)
    e32.step(60)
    e64 = PhysicsEngine(cfg).load_scene(s)
    e64.step(60)
    np.testing.assert_allclose(e32.state()["pos"], e64.state()["pos"], rtol=0, atol=1e-5)


def with_state(scene, st):
    s = dict(scene)
    for k in ("pos", "quat", "vel", "omega"):
        s[k] = st[k].copy()
    return s


def test_checkpoint_and_resume_with_the_warm_start_memory(oracle_mod):
    # state + contact memory (cdx_get_state / cdx_get_contacts) taken after 120 steps and loaded
    # into a fresh context (cdx_set_state / cdx_set_contacts) and into the oracle: the resumed runs
    # continue bit for bit as the uninterrupted one, warm start included
    s = scenes.generate("pile_1k", scale=0.3)
    cfg = scenes.config_for("pile_1k")
    run = PhysicsEngine(cfg).load_scene(s)
    run.step(120)
    st, mem = run.state(), run.contacts()
    assert mem["id_a"].shape[0] > 50
    resumed = PhysicsEngine(cfg).load_scene(with_state(s, st))
    resumed.set_contacts({k: mem[k][::-1] for k in ("id_a", "id_b", "point", "lambda")})  # any order
    back = resumed.contacts()
    for k in ("id_a", "id_b", "point", "lambda"):
        assert_same(back[k], mem[k], f"loaded memory {k}")
    orc = oracle_mod.Oracle(with_state(s, st), cfg).set_contacts(mem)
    cold = PhysicsEngine(cfg).load_scene(with_state(s, st))
    for e in (run, resumed, orc, cold):
        e.step(5)
    a, b, o = run.state(), resumed.state(), orc.state()
    for k in ("pos", "quat", "vel", "omega"):
        assert_same(b[k], a[k], f"resumed {k}")
        assert_same(o[k], a[k], f"oracle resumed {k}")
    assert_same(resumed.contacts()["lambda"], run.contacts()["lambda"], "impulses after resuming")
    # without the memory the first step starts from zero impulses and the run differs
    assert not np.array_equal(cold.state()["vel"], a["vel"])


def test_contact_memory_is_validated():
    s = scenes.generate("pile_1k", scale=0.05)
    e = PhysicsEngine(scenes.config_for("pile_1k")).load_scene(s)
    S = s["static_kind"].shape[0]
    ok = {"id_a": np.array([0]), "id_b": np.array([S]), "point": np.zeros((1, 3)), "lambda": np.ones((1, 3))}
    e.set_contacts(ok)
    from cardillocxx_gb300 import CdxError
    for bad in ({"id_b": np.array([S + 10 ** 6])}, {"id_a": np.array([S + 1]), "id_b": np.array([S])},
                {"lambda": np.full((1, 3), np.nan)}):
        with pytest.raises(CdxError):
            e.set_contacts(dict(ok, **bad))
    with pytest.raises(CdxError):
        e.set_contacts({k: np.concatenate([v, v]) for k, v in ok.items()})  # a pair twice
    e.set_contacts({k: v[:0] for k, v in ok.items()})
    e.step(1)


PILE_200K = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "pile_200k_settled.npz")


def test_settled_pile_200k_is_bit_identical_to_the_oracle(oracle_mod):
    # the benchmark's input at full size: 200,000 settled spheres, about 480,000 contacts, 100 sweeps a
    # step from zero impulses, then warm-started steps. Three steps of the plain FP64 method against the
    # oracle (OpenMP over all host threads, bit-identical to its sequential mode): states, contacts,
    # impulses and sweep counts equal bit for bit after every step
    s = scenes.settled_pile(PILE_200K)
    cfg = scenes.config_for("pile_200k")
    assert s["pos"].shape[0] == 200000
    eng = PhysicsEngine(dict(cfg, **{"gpu.precision": "fp64"})).load_scene(s)
    orc = oracle_mod.Oracle(s, cfg, omp_mode=1, num_threads=os.cpu_count() or 1)
    for k in range(3):
        eng.step(1)
        orc.step(1)
        g, o = eng.state(), orc.state()
        for key in ("pos", "quat", "vel", "omega"):
            assert_same(g[key], o[key], f"{key} after step {k + 1}")
        gc, oc = eng.contacts(), orc.contacts()
        assert gc["id_a"].shape[0] > 400000
        for key in ("id_a", "id_b", "point", "lambda", "normal"):
            assert_same(gc[key], oc[key], f"contact {key} after step {k + 1}")
        gs, os_ = eng.stats(), orc.stats()
        assert gs["iterations"] == os_["iterations"] == 100
        assert gs["num_rows"] == os_["num_rows"]
        assert gs["residual"] == os_["residual"]
