"""The reference's loop controls in the split form, and the failure paths a step reports.

pj.tol_abs / pj.tol_rel (the standard loop's velocity-increment exit, projected_jacobi.cpp:140-144,
371-377) and pj.nesterov (nesterov_loop, :379-449) run in the split form's cooperative solve; the
plain FP64 method runs them bit for bit as the oracle does, so it is the reference here. The split
form's FP32 sweeps stop at the same sweep or within one check interval, at the same solution to
FP32 accuracy. Failures: a grid barrier that waits too long ends the step with CDX_ERR_TIMEOUT
(bounded wait, no hang) and the context steps on; a state that is not finite after a step gives
CDX_ERR_NONFINITE.
"""
import numpy as np
import pytest

from cardillocxx_gb300 import CdxError, PhysicsEngine, scenes

pytestmark = pytest.mark.gpu

G, H = 9.81, 1e-3


def settled_small_pile():
    s = scenes.generate("pile_1k", scale=0.3)
    base = scenes.config_for("pile_1k")
    ref = PhysicsEngine(base).load_scene(s)
    ref.step(250)
    return s, base, ref.state()


def one_step(scene, cfg, st):
    e = PhysicsEngine(cfg).load_scene(scene)
    e.set_state(st["pos"], st["quat"], st["vel"], st["omega"])
    e.step(1)
    return e


def test_split_tolerance_exit_stops_where_fp64_stops():
    s, base, st = settled_small_pile()
    c = dict(base, **{"pj.warmstart": False, "pj.max_iterations": 5000, "pj.tol_abs": 1e-6, "pj.tol_rel": 1e-6})
    e64 = one_step(s, c, st)
    e32 = one_step(s, dict(c, **{"gpu.precision": "split"}), st)
    it64, it32 = e64.stats()["iterations"], e32.stats()["iterations"]
    assert it64 < 5000 and it32 < 5000  # the exit ended both loops
    assert it64 % 10 == 1 and it32 % 10 == 1  # tested after sweeps 1, 11, 21, ...
    assert abs(it64 - it32) <= max(20, it64 // 10)
    names = PhysicsEngine.split_variants()
    assert names[e32.stats()["contact_variant"]].startswith("coop")
    vscale = np.abs(st["vel"]).max() + G * H
    assert np.abs(e64.state()["vel"] - e32.state()["vel"]).max() <= 2e-3 * vscale
    # no tolerance: the loop runs to the cap
    e = one_step(s, dict(c, **{"gpu.precision": "split", "pj.tol_abs": 0.0, "pj.tol_rel": 0.0,
                               "pj.max_iterations": 300}), st)
    assert e.stats()["iterations"] == 300


def test_split_nesterov_tracks_fp64_nesterov():
    s, base, st = settled_small_pile()
    c = dict(base, **{"pj.warmstart": False, "pj.max_iterations": 4000, "pj.tol_abs": 1e-7, "pj.tol_rel": 1e-7})
    std64 = one_step(s, c, st)
    nes = dict(c, **{"pj.nesterov": True})
    n64 = one_step(s, nes, st)
    n32 = one_step(s, dict(nes, **{"gpu.precision": "split"}), st)
    i_std, i64, i32 = std64.stats()["iterations"], n64.stats()["iterations"], n32.stats()["iterations"]
    assert i64 < 4000 and i32 < 4000
    assert i64 < i_std  # the accelerated loop needs fewer sweeps for the same exit
    # Nesterov's restarts react to the last bits of the residual, and the split form's FP32
    # reductions run in no fixed order: its sweep count varies from run to run around the FP64 one
    assert i32 <= 1.5 * i64 + 30 and i32 < i_std, (i32, i64, i_std)
    vscale = np.abs(st["vel"]).max() + G * H
    assert np.abs(n64.state()["vel"] - n32.state()["vel"]).max() <= 2e-3 * vscale
    assert np.isfinite(n32.state()["pos"]).all()
    # Nesterov over a run with warm start: the pile falls and settles as with the FP64 method
    runs = []
    for prec in ("fp64", "split"):
        run = PhysicsEngine(dict(base, **{"pj.nesterov": True, "pj.tol_abs": 1e-6, "pj.tol_rel": 1e-6,
                                          "pj.max_iterations": 500, "gpu.precision": prec})).load_scene(s)
        run.set_state(st["pos"], st["quat"], st["vel"], st["omega"])
        run.step(60)
        runs.append(run.state())
    assert np.isfinite(runs[1]["vel"]).all()
    assert abs(runs[0]["pos"][:, 2].mean() - runs[1]["pos"][:, 2].mean()) < 2e-3
    assert abs(np.abs(runs[0]["vel"]).mean() - np.abs(runs[1]["vel"]).mean()) < 0.05 * np.abs(runs[0]["vel"]).mean()


def test_split_nesterov_residual_exit():
    s, base, st = settled_small_pile()
    c = dict(base, **{"pj.warmstart": False, "pj.max_iterations": 20000, "pj.nesterov": True,
                      "pj.tol_abs": 1e-100, "pj.tol_rel": 0.0, "gpu.residual_tol": 1e-4, "gpu.check_every": 1})
    e32 = one_step(s, dict(c, **{"gpu.precision": "split"}), st)
    e64 = one_step(s, c, st)
    for e in (e32, e64):
        assert e.stats()["iterations"] < 20000
        assert e.stats()["residual_last"] <= 1e-4
    # the FP64 complementarity residual of the split result is at the same level
    assert e32.stats()["residual"] <= 3e-4


def test_cooperative_barrier_timeout_is_reported_and_the_context_steps_on():
    # a barrier wait limit of 1 ns: the first block to arrive gives up, every block returns, and the
    # step fails with CDX_ERR_TIMEOUT instead of hanging; with the normal limit the context steps on
    s, base, st = settled_small_pile()
    names = PhysicsEngine.split_variants()
    c = dict(base, **{"gpu.precision": "split", "gpu.sweep_variant": names.index("coop-t1024-u1-g2"),
                      "gpu.coop_wait_ns": 1})
    e = PhysicsEngine(c).load_scene(s)
    e.set_state(st["pos"], st["quat"], st["vel"], st["omega"])
    with pytest.raises(CdxError) as err:
        e.step(1)
    assert err.value.status == 5
    e.set_config(dict(c, **{"gpu.coop_wait_ns": 0}))
    e.set_state(st["pos"], st["quat"], st["vel"], st["omega"])
    e.step(3)
    assert e.stats()["iterations"] == c["pj.max_iterations"]
    assert np.isfinite(e.state()["vel"]).all()
    ref = one_step(s, dict(c, **{"gpu.coop_wait_ns": 0}), st)
    assert ref.stats()["num_contacts"] > 0


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_nonfinite_state_is_reported(precision):
    s = scenes.generate("pile_1k", scale=0.05)
    c = dict(scenes.config_for("pile_1k"), **{"gpu.precision": precision})
    e = PhysicsEngine(c).load_scene(s)
    e.step(2)
    st = e.state()
    vel = st["vel"].copy()
    vel[3, 1] = np.nan
    e.set_state(st["pos"], st["quat"], vel, st["omega"])
    with pytest.raises(CdxError) as err:
        e.step(1)
    assert err.value.status == 4
    # the context stays usable: a finite state steps again
    e.set_state(st["pos"], st["quat"], st["vel"], st["omega"])
    e.step(2)
    assert np.isfinite(e.state()["pos"]).all()


def test_split_resumes_with_the_warm_start_memory():
    # the split form's contact memory taken after a run and loaded into a fresh context continues
    # the run: the same contacts, impulses and velocities to FP32 summation order
    s = scenes.generate("pile_1k", scale=0.3)
    c = dict(scenes.config_for("pile_1k"), **{"gpu.precision": "split"})
    run = PhysicsEngine(c).load_scene(s)
    run.step(150)
    st, mem = run.state(), run.contacts()
    sc = dict(s)
    for k in st:
        sc[k] = st[k].copy()
    resumed = PhysicsEngine(c).load_scene(sc).set_contacts(mem)
    back = resumed.contacts()
    assert np.array_equal(back["id_a"], mem["id_a"]) and np.array_equal(back["id_b"], mem["id_b"])
    assert np.array_equal(back["lambda"], mem["lambda"])
    cold = PhysicsEngine(c).load_scene(sc)
    for e in (run, resumed, cold):
        e.step(1)
    a, b = run.contacts(), resumed.contacts()
    assert np.array_equal(a["id_a"], b["id_a"]) and np.array_equal(a["id_b"], b["id_b"])
    lmax = np.abs(a["lambda"]).max()
    assert np.abs(a["lambda"] - b["lambda"]).max() <= 1e-5 * lmax
    assert np.abs(cold.contacts()["lambda"] - a["lambda"]).max() > 1e-3 * lmax  # the memory mattered
    vs = np.abs(st["vel"]).max() + G * H
    assert np.abs(run.state()["vel"] - resumed.state()["vel"]).max() <= 1e-5 * vs
