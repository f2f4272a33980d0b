"""Split-precision form (FP32 contacts/Delassus/projection, FP64 state and residual) -- GPU tests.

Known answers hold to FP32 accuracy; against the plain FP64 method the split form agrees to the
FP32 rounding level on one step from the same state, and statistically over a run.
"""
import numpy as np
import pytest

from cardillocxx_gb300 import PhysicsEngine, scenes
from cardillocxx_gb300.scenes import make_scene

pytestmark = pytest.mark.gpu

G = 9.81
H = 1e-3
F32_RTOL = 2e-5  # FP32 contact arithmetic: relative tolerance on impulses and velocities
# split form against the FP64 method on a converged step with the same contact set (FP32 rounding
# of the contact algebra and of the summation of W^T lambda)
SAME_CONTACTS_RTOL = 1e-5
# two split-form shapes (the same FP32 sweep, another summation order) after a few hundred sweeps
SAME_SWEEP_RTOL = 1e-4


def cfg(**kw):
    c = {"sim.dt": H, "moreau.theta": 0.5, "friction.enable": True, "friction.combine": "min",
         "pj.max_iterations": 50, "pj.alpha": 0.5, "pj.tol_abs": 0.0, "pj.tol_rel": 0.0, "pj.warmstart": True,
         "gpu.precision": "split"}
    c.update(kw)
    return c


GROUND = {"kind": "halfspace", "pos": (0, 0, 0), "dir": (0, 0, 1), "mu": 0.3}


def test_split_resting_and_sliding(gpu):
    r, mu = 0.05, 0.3
    s = make_scene([{"pos": (0.0, 0.0, r - 1e-5), "radius": r, "vel": (1.0, 0, 0), "mu": mu}], [GROUND])
    e = PhysicsEngine(cfg()).load_scene(s)
    n = 10
    e.step(n)
    st = e.state()
    m = s["mass"][0]
    np.testing.assert_allclose(st["vel"][0, 0], 1.0 - n * mu * G * H, rtol=F32_RTOL)
    lever = r - 0.5e-5  # centre to contact point (midpoint of the 10 micrometre overlap)
    np.testing.assert_allclose(st["omega"][0, 1], n * H * 5 * mu * G * lever / (2 * r * r), rtol=1e-4)
    lam = e.contacts()["lambda"][0]
    np.testing.assert_allclose(lam[0], m * G * H, rtol=F32_RTOL)
    assert e.stats()["residual"] < 1e-5


def test_split_free_fall_is_fp64_exact(gpu):
    s = make_scene([{"pos": (0.2, 0.3, 5.0), "radius": 0.05, "vel": (0.3, -0.2, 1.0)}], [GROUND])
    e = PhysicsEngine(cfg()).load_scene(s)
    e.step(200)
    t = 200 * H
    np.testing.assert_allclose(e.state()["pos"][0], [0.2 + 0.3 * t, 0.3 - 0.2 * t, 5.0 + t - 0.5 * G * t * t],
                               rtol=0, atol=1e-12)


def test_split_drum_drag(gpu):
    r, mu, w = 0.1, 0.4, 2.0
    drum = {"kind": "drum", "pos": (0, 0, 0), "dir": (1, 0, 0), "radius": 1.0, "omega": (w, 0, 0), "mu": mu}
    # 10 micrometres of overlap: an exactly touching pair can round to a positive FP32 gap
    s = make_scene([{"pos": (0.5, 0.0, -0.90001), "radius": r, "mu": mu}], [drum])
    e = PhysicsEngine(cfg()).load_scene(s)
    e.step(1)
    v = e.state()["vel"][0]
    np.testing.assert_allclose(v[1], mu * G * H, rtol=1e-4)
    assert abs(v[2]) < 1e-6


def test_split_one_step_matches_fp64(gpu):
    s = scenes.generate("pile_1k", scale=0.3)
    base = scenes.config_for("pile_1k")
    ref = PhysicsEngine(base).load_scene(s)
    ref.step(250)
    st = ref.state()
    # one step from the same state, no warm start, iterated far enough that both forms converge
    c = dict(base, **{"pj.warmstart": False, "pj.max_iterations": 3000})
    e64 = PhysicsEngine(c).load_scene(s)
    e32 = PhysicsEngine(dict(c, **{"gpu.precision": "split"})).load_scene(s)
    for e in (e64, e32):
        e.set_state(st["pos"], st["quat"], st["vel"], st["omega"])
        e.step(1)
    c64, c32 = e64.contacts(), e32.contacts()
    assert np.array_equal(c64["id_a"], c32["id_a"]) and np.array_equal(c64["id_b"], c32["id_b"])
    # the same contacts: the two forms differ by FP32 rounding only (measured 2-5e-7 relative)
    lmax = np.abs(c64["lambda"]).max()
    dl = np.abs(c64["lambda"] - c32["lambda"]).max() / lmax
    v64, v32 = e64.state()["vel"], e32.state()["vel"]
    vscale = np.abs(st["vel"]).max() + G * H
    dv = np.abs(v64 - v32).max() / vscale
    assert dl <= SAME_CONTACTS_RTOL and dv <= SAME_CONTACTS_RTOL, (dl, dv)
    np.testing.assert_allclose(e64.state()["pos"], e32.state()["pos"], rtol=0, atol=1e-7)


def test_split_every_sweep_shape_computes_the_same_sweep(gpu):
    # every launch shape and scatter mode (atomicAdd, reductions, per-warp run sums) runs the same
    # projected Jacobi sweep; only the FP32 summation order of W^T lambda differs
    s = scenes.generate("pile_1k", scale=0.3)
    base = scenes.config_for("pile_1k")
    ref = PhysicsEngine(base).load_scene(s)
    ref.step(250)
    st = ref.state()
    c = dict(base, **{"gpu.precision": "split", "pj.warmstart": False, "pj.max_iterations": 200})
    names = PhysicsEngine.split_variants()
    assert len(names) >= 2
    out = []
    runs = [(v, {"gpu.coop_smem_contacts": 1} if "hyb" in names[v] else {}) for v in range(len(names))]
    # a cooperative solve on a reduced grid: more contacts and bodies a block, the same sweep
    runs.append((names.index("coop-t1024-u1-g2"), {"gpu.coop_blocks": 3}))
    for v, extra in runs:
        # the hybrid cooperative shape runs when a block's contacts exceed its shared-memory cap
        e = PhysicsEngine(dict(c, **{"gpu.sweep_variant": v}, **extra)).load_scene(s)
        e.set_state(st["pos"], st["quat"], st["vel"], st["omega"])
        e.step(1)
        # the per-scene shapes apply to a single scene too (it fits one block)
        assert e.stats()["contact_variant"] == v, names[v]
        out.append((f"{names[v]} {extra}", e.contacts()["lambda"], e.state()["vel"]))
    _, lam0, vel0 = out[0]
    lmax = np.abs(lam0).max()
    vscale = np.abs(st["vel"]).max() + G * H
    for label, lam, vel in out:
        assert lam.shape == lam0.shape, label
        dl, dv = np.abs(lam - lam0).max() / lmax, np.abs(vel - vel0).max() / vscale
        assert dl <= SAME_SWEEP_RTOL and dv <= SAME_SWEEP_RTOL, (label, dl, dv)


def test_split_residual_is_fp64_and_decreases(gpu):
    s = scenes.generate("pile_1k", scale=0.3)
    base = scenes.config_for("pile_1k", **{"gpu.precision": "split"})
    e = PhysicsEngine(base).load_scene(s)
    e.step(250)
    res = {}
    for it in (10, 100, 1000):
        ee = PhysicsEngine(dict(base, **{"pj.max_iterations": it, "pj.warmstart": False})).load_scene(s)
        st = e.state()
        ee.set_state(st["pos"], st["quat"], st["vel"], st["omega"])
        ee.step(1)
        res[it] = ee.stats()["residual"]
    assert res[1000] < res[100] < res[10]
    assert res[1000] < 1e-4


def test_split_residual_stop_rule(gpu):
    s = scenes.generate("pile_1k", scale=0.3)
    c = scenes.config_for("pile_1k", **{"gpu.precision": "split", "pj.max_iterations": 400,
                                        "gpu.residual_tol": 1e-3})
    e = PhysicsEngine(c).load_scene(s)
    e.step(200)
    st = e.stats()
    assert st["iterations"] < 400
    assert st["residual_last"] <= 1e-3


def test_split_pile_statistics_match_fp64(gpu):
    s = scenes.generate("pile_1k", scale=0.5)
    base = scenes.config_for("pile_1k")
    e64 = PhysicsEngine(base).load_scene(s)
    e32 = PhysicsEngine(dict(base, **{"gpu.precision": "split"})).load_scene(s)
    e64.step(400)
    e32.step(400)
    z64, z32 = e64.state()["pos"][:, 2], e32.state()["pos"][:, 2]
    assert abs(z64.mean() - z32.mean()) < 2e-3
    assert abs(e64.stats()["num_contacts"] - e32.stats()["num_contacts"]) <= 0.05 * e64.stats()["num_contacts"] + 5
    assert np.isfinite(e32.state()["vel"]).all()


def test_split_batched_and_graph_off(gpu):
    s = scenes.generate("batch_4096", scale=0.01)
    c = scenes.config_for("batch_4096", **{"gpu.precision": "split"})
    a = PhysicsEngine(c).load_scene(s)
    b = PhysicsEngine(dict(c, **{"gpu.graph": False})).load_scene(s)
    a.step(150)
    b.step(150)
    za, zb = a.state()["pos"][:, 2], b.state()["pos"][:, 2]
    assert np.isfinite(za).all() and np.isfinite(zb).all()
    assert abs(za.mean() - zb.mean()) < 1e-3
    assert a.stats()["iterations"] == b.stats()["iterations"] == 50


def test_newton_raphson_fp64_matches_ieee(gpu):
    # the split form's FP64 final pass uses Newton-Raphson reciprocals / inverse square roots;
    # they must agree with correctly rounded IEEE results to a couple of ulps
    from cardillocxx_gb300 import PhysicsEngine as PE
    rng = np.random.default_rng(3)
    x = np.concatenate([10.0 ** rng.uniform(-29, 29, 200000), rng.uniform(0.5, 2.0, 100000),
                        [1.0, 2.0, 4.0, 1e-31, 1e31, 3.0]])
    r, q = PE({}).selftest_nr64(x)
    exact_r, exact_q = 1.0 / x, 1.0 / np.sqrt(x)
    eps = np.finfo(float).eps
    assert np.max(np.abs(r - exact_r) / np.abs(exact_r)) <= 2 * eps
    assert np.max(np.abs(q - exact_q) / np.abs(exact_q)) <= 2 * eps


def test_batched_scenes_solver_matches_fp64_and_streaming(gpu):
    # thousands-of-scenes workload at 40 scenes: the per-scene block solver (chosen automatically
    # for several scenes) against the plain FP64 method and the streaming sweep on one converged step
    s = scenes.generate("batch_4096", scale=40 / 4096)
    assert s["num_scenes"] >= 30
    base = scenes.config_for("batch_4096")
    ref = PhysicsEngine(base).load_scene(s)
    ref.step(150)
    st = ref.state()
    c = dict(base, **{"pj.warmstart": False, "pj.max_iterations": 2000})
    e64 = PhysicsEngine(c).load_scene(s)
    e32 = PhysicsEngine(dict(c, **{"gpu.precision": "split"})).load_scene(s)
    e32s = PhysicsEngine(dict(c, **{"gpu.precision": "split", "gpu.sweep_variant": "0"})).load_scene(s)
    for e in (e64, e32, e32s):
        e.set_state(st["pos"], st["quat"], st["vel"], st["omega"])
        e.step(1)
    names = PhysicsEngine.split_variants()
    assert names[e32.stats()["contact_variant"]].startswith("scenes"), names[e32.stats()["contact_variant"]]
    assert e32.stats()["iterations"] == 2000
    c64, c32 = e64.contacts(), e32.contacts()
    assert np.array_equal(np.sort(c64["id_a"] * 10**7 + c64["id_b"]), np.sort(c32["id_a"] * 10**7 + c32["id_b"]))
    vscale = np.abs(st["vel"]).max() + 9.81 * 1e-3
    for other in (e64, e32s):
        dv = np.abs(other.state()["vel"] - e32.state()["vel"]).max() / vscale
        assert dv <= SAME_CONTACTS_RTOL, dv
    np.testing.assert_allclose(e64.state()["pos"], e32.state()["pos"], rtol=0, atol=1e-7)
    # then a run of the batched workload with warm start: stays finite and resting
    e = PhysicsEngine(dict(base, **{"gpu.precision": "split"})).load_scene(s)
    e.set_state(st["pos"], st["quat"], st["vel"], st["omega"])
    e.step(50)
    v = e.state()["vel"]
    assert np.isfinite(v).all() and np.abs(v).max() < 5.0


def test_device_counted_steps_match_host_counted_and_redo_on_growth(gpu):
    # after the first step the split form finds its contact totals on the device; a falling pile
    # outgrows the buffers several times, so some steps are undone and redone synchronously.
    # Host-counted steps (gpu.sync_counts) run the same physics.
    s = scenes.generate("pile_1k")
    base = dict(scenes.config_for("pile_1k"), **{"gpu.precision": "split", "gpu.contact_capacity": 0.1})
    a = PhysicsEngine(base).load_scene(s)
    b = PhysicsEngine(dict(base, **{"gpu.sync_counts": True})).load_scene(s)
    a.step(1)
    b.step(1)
    za, zb = [], []
    for k in range(10):
        a.step(40)
        b.step(40)
        za.append(a.state()["pos"][:, 2].mean())
        zb.append(b.state()["pos"][:, 2].mean())
    assert a.stats()["redone_steps"] >= 1
    assert b.stats()["redone_steps"] == 0
    assert a.stats()["num_contacts"] > 1000
    np.testing.assert_allclose(za, zb, rtol=0, atol=2e-3)
    # one step from the same state without warm start (the two runs' histories differ): the same
    # contacts, velocities to FP32 summation order; the second step of a2 counts on the device
    st = a.state()
    cold = dict(base, **{"pj.warmstart": False, "gpu.contact_capacity": 8})
    a2 = PhysicsEngine(cold).load_scene(s)
    b2 = PhysicsEngine(dict(cold, **{"gpu.sync_counts": True})).load_scene(s)
    for e in (a2, b2):
        for _ in range(2):
            e.set_state(st["pos"], st["quat"], st["vel"], st["omega"])
            e.step(1)
    ca, cb = a2.contacts(), b2.contacts()
    assert np.array_equal(ca["id_a"], cb["id_a"]) and np.array_equal(ca["id_b"], cb["id_b"])
    vs = np.abs(st["vel"]).max() + 9.81e-3
    assert np.abs(a2.state()["vel"] - b2.state()["vel"]).max() <= 1e-4 * vs


def test_whole_step_graph_replays_the_same_step(gpu):
    # device-counted steps with the cooperative solver are captured whole into a CUDA graph and
    # replayed; the trajectory matches the directly launched steps (gpu.graph off) to FP32 order
    s = scenes.generate("pile_1k", scale=0.5)
    base = dict(scenes.config_for("pile_1k"), **{"gpu.precision": "split"})
    names = PhysicsEngine.split_variants()
    coop = str(names.index("coop-t1024-u1-g2"))
    a = PhysicsEngine(dict(base, **{"gpu.sweep_variant": coop})).load_scene(s)
    b = PhysicsEngine(dict(base, **{"gpu.sweep_variant": coop, "gpu.graph": False})).load_scene(s)
    for e in (a, b):
        e.step(120)
    assert a.stats()["graph_steps"] >= 100
    assert b.stats()["graph_steps"] == 0
    za, zb = a.state()["pos"][:, 2], b.state()["pos"][:, 2]
    assert abs(za.mean() - zb.mean()) < 2e-3
    assert np.isfinite(a.state()["vel"]).all()


def test_pinned_state_transfers_match_pageable(gpu):
    # pinned caller arrays are read and written by a kernel directly; pageable ones go through the
    # staging buffer: both give the same state, and a state set from pinned memory steps the same
    torch = pytest.importorskip("torch")
    s = scenes.generate("pile_1k", scale=0.2)
    cfg = scenes.config_for("pile_1k")
    eng = PhysicsEngine(cfg).load_scene(s)
    eng.step(20)
    ref = eng.state()
    pins = {k: torch.empty(v.shape, dtype=torch.float64, pin_memory=True).numpy() for k, v in ref.items()}
    eng.state_into(pins["pos"], pins["quat"], pins["vel"], pins["omega"])
    for k in ref:
        assert np.array_equal(pins[k], ref[k]), k
    # partial download: only velocities
    v = torch.empty(ref["vel"].shape, dtype=torch.float64, pin_memory=True).numpy()
    eng.state_into(None, None, v, None)
    assert np.array_equal(v, ref["vel"])
    # upload from pinned memory into a second engine, then both step identically
    eng2 = PhysicsEngine(cfg).load_scene(s)
    eng2.set_state(pins["pos"], pins["quat"], pins["vel"], pins["omega"])
    eng2.synchronize()
    st2 = eng2.state()
    for k in ref:
        assert np.array_equal(st2[k], ref[k]), k


def test_per_scene_solver_on_overflowing_device_counted_steps(gpu):
    # the per-scene kernel (pinned) on device-counted steps whose contacts outgrow the buffers (a
    # step that overflowed them solves nothing and is redone); the run matches host-counted steps
    names = PhysicsEngine.split_variants()
    v = names.index("scenes-t256-c1")
    s = scenes.generate("pile_1k")
    base = dict(scenes.config_for("pile_1k"), **{"gpu.precision": "split", "gpu.contact_capacity": 0.1,
                                                 "gpu.sweep_variant": v})
    a = PhysicsEngine(base).load_scene(s)
    b = PhysicsEngine(dict(base, **{"gpu.sync_counts": True})).load_scene(s)
    za, zb = [], []
    for _ in range(10):
        a.step(40)
        b.step(40)
        za.append(a.state()["pos"][:, 2].mean())
        zb.append(b.state()["pos"][:, 2].mean())
    assert b.stats()["redone_steps"] == 0
    assert a.stats()["num_contacts"] > 1024  # more than the 1,024 slots it started with
    assert a.stats()["contact_variant"] == v
    np.testing.assert_allclose(za, zb, rtol=0, atol=2e-3)


def test_hybrid_cooperative_solve_streams_what_shared_memory_cannot_hold(gpu):
    # a cap on the contacts a block keeps in shared memory: the plain cooperative shape no longer
    # fits and falls back to streaming; the hybrid shape keeps the first contacts of every block in
    # shared memory and reads the rest every sweep, in one launch. Same sweeps, FP32 order apart.
    s = scenes.generate("pile_1k")
    base = scenes.config_for("pile_1k")
    ref = PhysicsEngine(base).load_scene(s)
    ref.step(300)
    st = ref.state()
    names = PhysicsEngine.split_variants()
    c = dict(base, **{"gpu.precision": "split", "pj.warmstart": False, "pj.max_iterations": 100,
                      "gpu.coop_smem_contacts": 4})
    out = {}
    for name in ("coop-t1024-u1-g2", "coop-hyb-t1024-u1-g2", "sweep-u1-t256-b4-g2"):
        e = PhysicsEngine(dict(c, **{"gpu.sweep_variant": names.index(name)})).load_scene(s)
        e.set_state(st["pos"], st["quat"], st["vel"], st["omega"])
        e.step(1)
        out[name] = (e.stats(), e.contacts()["lambda"], e.state()["vel"])
    assert out["coop-t1024-u1-g2"][0]["contact_variant"] == names.index("sweep-u1-t256-b4-g2")  # did not fit
    assert out["coop-hyb-t1024-u1-g2"][0]["contact_variant"] == names.index("coop-hyb-t1024-u1-g2")
    assert out["coop-hyb-t1024-u1-g2"][0]["num_contacts"] > 4 * 152  # more than the cap holds
    lam0, vel0 = out["sweep-u1-t256-b4-g2"][1:]
    lam1, vel1 = out["coop-hyb-t1024-u1-g2"][1:]
    vscale = np.abs(st["vel"]).max() + G * H
    dl, dv = np.abs(lam1 - lam0).max() / np.abs(lam0).max(), np.abs(vel1 - vel0).max() / vscale
    assert dl <= SAME_SWEEP_RTOL and dv <= SAME_SWEEP_RTOL, (dl, dv)


def test_batched_scenes_alpha_autotuner(gpu):
    # gpu.tune_alpha: the per-scene solve's alpha picked per scene by trial solves of the same step.
    # Every alpha has the same fixed points, so both runs stop at the same residual tolerance with
    # the same physics; the tuned one needs no more sweeps in total.
    s = scenes.generate("batch_4096", scale=48 / 4096)
    base = scenes.config_for("batch_4096")
    ref = PhysicsEngine(base).load_scene(s)
    ref.step(200)
    st = ref.state()
    ns = int(s["num_scenes"])
    rule = {"gpu.precision": "split", "gpu.residual_tol": 1e-4, "pj.max_iterations": 400, "gpu.autotune": False}
    plain = PhysicsEngine(dict(base, **rule)).load_scene(s)
    tuned = PhysicsEngine(dict(base, **rule, **{"gpu.tune_alpha": True, "gpu.tune_alpha_every": 3})).load_scene(s)
    sweeps = {}
    for name, e in (("plain", plain), ("tuned", tuned)):
        e.set_state(st["pos"], st["quat"], st["vel"], st["omega"])
        tot = 0
        for _ in range(6):
            e.step(1)
            it = e.scene_solve(ns)["sweeps"]
            tot += int(it.sum())
        sweeps[name] = tot
        # every scene stopped on the tolerance, not at the cap
        assert it.max() < 400 and e.stats()["residual_last"] <= 1e-4 * 1.0001
    a = tuned.scene_solve(ns)["alpha"]
    a0 = float(base["pj.alpha"])
    # a pick above pj.alpha is kept with a 15 % margin below it
    cand = {c if c <= a0 else max(a0, 0.85 * c) for c in (0.2, 0.3, 0.4, 0.5, 0.6, 0.7, 0.85, 1.0, a0)}
    assert all(any(abs(x - c) < 1e-6 for c in cand) for x in a), a
    assert np.allclose(plain.scene_solve(ns)["alpha"], base["pj.alpha"])
    # the tuner keeps pj.alpha where no candidate beats it; the FP32 reductions' order varies, so
    # a scene's sweep count can move by one from run to run
    assert sweeps["tuned"] <= sweeps["plain"] + 6 * ns, sweeps
    vscale = np.abs(st["vel"]).max() + 9.81e-3
    assert np.isfinite(tuned.state()["vel"]).all()
    assert np.abs(tuned.state()["vel"] - plain.state()["vel"]).max() <= 1e-2 * vscale


def test_split_contact_set_equals_fp64_on_the_settled_pile(gpu):
    # the FP32 narrow phase leaves the pairs within a few 1e-7 of the threshold to the FP64
    # distance: from the settled 200k pile at rest (its resting contacts have gaps of that size)
    # the split form finds exactly the FP64 method's contacts
    import os
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "pile_200k_settled.npz")
    s = scenes.settled_pile(path)
    cfg = scenes.config_for("pile_200k")
    out = {}
    for prec in ("fp64", "split"):
        e = PhysicsEngine(dict(cfg, **{"gpu.precision": prec})).load_scene(s)
        e.step(1)
        out[prec] = e.contacts()
        e.close()
    a, b = out["fp64"], out["split"]
    ka = a["id_a"].astype(np.int64) << 32 | a["id_b"].astype(np.int64)
    kb = b["id_a"].astype(np.int64) << 32 | b["id_b"].astype(np.int64)
    assert ka.size > 400_000
    assert np.array_equal(np.sort(ka), np.sort(kb))
