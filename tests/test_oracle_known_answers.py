"""Known-answer tests that pin the CPU oracle (CPU only).

The reference ships no tests or golden vectors for this path, so the oracle is pinned by physics
with closed-form answers (Moreau midpoint free fall, resting load m*g*h, Coulomb sliding,
drum wall drag) and by the projection branches of projected_jacobi.cpp:100-119.
"""
import math

import numpy as np
import pytest

from cardillocxx_gb300.scenes import make_scene
from tests.csr_cases import csr_problem

G = 9.81
H = 1e-3


def cfg(**kw):
    c = {"sim.dt": H, "moreau.theta": 0.5, "friction.enable": True, "friction.combine": "min",
         "pj.max_iterations": 50, "pj.alpha": 0.5, "pj.tol_abs": 0.0, "pj.tol_rel": 0.0, "pj.warmstart": True,
         "collision.match_max_dist": 0.02}
    c.update(kw)
    return c


GROUND = {"kind": "halfspace", "pos": (0, 0, 0), "dir": (0, 0, 1), "mu": 0.3}


def test_free_fall_midpoint_exact(oracle_mod):
    s = make_scene([{"pos": (0.2, 0.3, 5.0), "radius": 0.05, "vel": (0.3, -0.2, 1.0)}], [GROUND])
    o = oracle_mod.Oracle(s, cfg())
    n = 200
    o.step(n)
    t = n * H
    st = o.state()
    exp = np.array([0.2 + 0.3 * t, 0.3 - 0.2 * t, 5.0 + 1.0 * t - 0.5 * G * t * t])
    np.testing.assert_allclose(st["pos"][0], exp, rtol=0, atol=1e-12)
    np.testing.assert_allclose(st["vel"][0], [0.3, -0.2, 1.0 - G * t], rtol=0, atol=1e-12)
    assert o.stats()["num_contacts"] == 0


def test_resting_contact_carries_weight(oracle_mod):
    r = 0.05
    s = make_scene([{"pos": (0.0, 0.0, r), "radius": r}], [GROUND])
    m = s["mass"][0]
    o = oracle_mod.Oracle(s, cfg())
    o.step(1)
    c = o.contacts()
    assert c["id_a"].tolist() == [0] and c["id_b"].tolist() == [1]
    np.testing.assert_allclose(c["lambda"][0, 0], m * G * H, rtol=1e-12)
    assert abs(c["lambda"][0, 1]) < 1e-15 and abs(c["lambda"][0, 2]) < 1e-15
    assert abs(o.state()["vel"][0, 2]) < 1e-13
    np.testing.assert_allclose(c["normal"][0], [0, 0, 1])


def test_sliding_friction_decelerates_mu_g(oracle_mod):
    r, mu, v0 = 0.05, 0.3, 1.0
    s = make_scene([{"pos": (0.0, 0.0, r), "radius": r, "vel": (v0, 0, 0), "mu": mu}], [dict(GROUND, mu=mu)])
    o = oracle_mod.Oracle(s, cfg())
    n = 10
    o.step(n)
    st = o.state()
    np.testing.assert_allclose(st["vel"][0, 0], v0 - n * mu * G * H, rtol=1e-10)
    # friction torque r mu m g about +y, I = 2/5 m r^2
    np.testing.assert_allclose(st["omega"][0, 1], n * H * 5 * mu * G / (2 * r), rtol=1e-9)
    lam = o.contacts()["lambda"][0]
    m = s["mass"][0]
    np.testing.assert_allclose(math.hypot(lam[1], lam[2]), mu * lam[0], rtol=1e-12)
    np.testing.assert_allclose(lam[0], m * G * H, rtol=1e-10)


def test_rotating_drum_drags_sphere(oracle_mod):
    r, mu, w = 0.1, 0.4, 2.0
    drum = {"kind": "drum", "pos": (0, 0, 0), "dir": (1, 0, 0), "radius": 1.0, "omega": (w, 0, 0), "mu": mu}
    s = make_scene([{"pos": (0.5, 0.0, -0.9), "radius": r, "mu": mu}], [drum])
    o = oracle_mod.Oracle(s, cfg())
    o.step(1)
    c = o.contacts()
    m = s["mass"][0]
    np.testing.assert_allclose(c["normal"][0], [0, 0, 1], atol=1e-15)
    np.testing.assert_allclose(c["lambda"][0, 0], m * G * H, rtol=1e-10)
    v = o.state()["vel"][0]
    # wall point at the bottom moves along +y (omega x r_wall); sliding friction mu g h
    np.testing.assert_allclose(v[1], mu * G * H, rtol=1e-9)
    assert abs(v[2]) < 1e-12


def test_static_drum_holds_sphere(oracle_mod):
    r = 0.1
    drum = {"kind": "drum", "pos": (0, 0, 0), "dir": (1, 0, 0), "radius": 1.0, "mu": 0.3}
    s = make_scene([{"pos": (0.5, 0.0, -0.9), "radius": r}], [drum])
    o = oracle_mod.Oracle(s, cfg())
    o.step(5)
    v = o.state()["vel"][0]
    assert np.abs(v).max() < 1e-12


def test_ceiling_contact_uses_south_pole_frame(oracle_mod):
    # a sphere pressed up against a ceiling: normal (0,0,-1) takes the south-pole branch of
    # tangentFrameFromNormal (tangent_frame.hpp:34-41)
    r = 0.05
    ceiling = {"kind": "halfspace", "pos": (0, 0, 1.0), "dir": (0, 0, -1), "mu": 0.3}
    s = make_scene([{"pos": (0.0, 0.0, 1.0 - r), "radius": r, "vel": (0, 0, 0.5)}], [ceiling])
    o = oracle_mod.Oracle(s, cfg(**{"sim.gravity": (0.0, 0.0, 0.0)}))
    o.step(1)
    c = o.contacts()
    np.testing.assert_allclose(c["normal"][0], [0, 0, -1])
    assert o.state()["vel"][0, 2] == pytest.approx(0.0, abs=1e-13)


def _one_contact_problem(v, mu=0.3):
    # one body with unit mass, one frictional contact with rows n = e_z, t1 = e_x, t2 = e_y
    row_ptr = np.array([0, 1, 2, 3], np.int32)
    col = np.array([2, 0, 1], np.int32)
    val = np.ones(3)
    ones6 = np.ones(6)
    return dict(row_ptr=row_ptr, col=col, val=val, contact_bias=np.zeros(3), mu=np.full(3, mu),
                restitution=np.zeros(3), minv=ones6, mdiag=ones6, v=np.asarray(v, float), f_ext=np.zeros(6),
                f_gyro=np.zeros(6), dt=H, alpha=1.0, max_iter=50, tol_abs=0.0, tol_rel=0.0, lam0=np.zeros(3))


@pytest.mark.parametrize("v,lam_exp,x_exp", [
    ((0, 0, 1, 0, 0, 0), (0, 0, 0), (0, 0, 1)),           # separating: normal clamp to 0
    ((0.1, 0, -1, 0, 0, 0), (1, -0.1, 0), (0, 0, 0)),      # sticking: inside the disk
    ((1.0, 0, -1, 0, 0, 0), (1, -0.3, 0), (0.7, 0, 0)),    # sliding: scaled onto the disk
    ((0, 0, -1, 0, 0, 0), (1, 0, 0), (0, 0, 0)),           # ||lambda_t|| = 0 branch
])
def test_projection_branches(oracle_mod, v, lam_exp, x_exp):
    x, lam, it = oracle_mod.pj_solve_csr(**_one_contact_problem(v))
    np.testing.assert_allclose(lam, lam_exp, atol=1e-14)
    np.testing.assert_allclose(x[:3], x_exp, atol=1e-14)
    assert it == 50


def test_velocity_residual_early_exit(oracle_mod):
    # the reference's own stop test (every 10th sweep, projected_jacobi.cpp:371-377)
    p = _one_contact_problem((0.1, 0, -1, 0, 0, 0))
    p.update(tol_abs=1e-6, tol_rel=1e-6, max_iter=1000)
    x, lam, it = oracle_mod.pj_solve_csr(**p)
    assert it in (1, 11, 21)
    np.testing.assert_allclose(lam, (1, -0.1, 0), atol=1e-12)


def test_warm_start_carries_impulse(oracle_mod):
    r = 0.05
    s = make_scene([{"pos": (0.0, 0.0, r), "radius": r}], [GROUND])
    o = oracle_mod.Oracle(s, cfg(**{"pj.max_iterations": 1}))
    m = s["mass"][0]
    o.step(1)
    l1 = o.contacts()["lambda"][0, 0]
    o.step(1)
    l2 = o.contacts()["lambda"][0, 0]
    # one sweep per step at alpha 0.5: the warm start lets the impulse keep converging to m g h
    assert l1 == pytest.approx(0.5 * m * G * H, rel=1e-12)
    assert l2 > l1
    o2 = oracle_mod.Oracle(s, cfg(**{"pj.max_iterations": 1, "pj.warmstart": False}))
    o2.step(2)
    assert o2.contacts()["lambda"][0, 0] < l2


def test_pile_settles_without_nan(oracle_mod):
    from cardillocxx_gb300 import scenes
    s = scenes.generate("pile_1k", scale=0.1)
    o = oracle_mod.Oracle(s, scenes.config_for("pile_1k"))
    o.step(150)
    st = o.state()
    assert np.isfinite(st["pos"]).all() and np.isfinite(st["quat"]).all()
    np.testing.assert_allclose(np.linalg.norm(st["quat"], axis=1), 1.0, atol=1e-14)
    assert o.stats()["num_contacts"] > 0


def test_omp_modes_bit_identical(oracle_mod):
    from cardillocxx_gb300 import scenes
    s = scenes.generate("pile_1k", scale=0.2)
    c = scenes.config_for("pile_1k")
    a = oracle_mod.Oracle(s, c, omp_mode=0)
    b = oracle_mod.Oracle(s, c, omp_mode=1, num_threads=4)
    a.step(120)
    b.step(120)
    for k in ("pos", "quat", "vel", "omega"):
        assert np.array_equal(a.state()[k], b.state()[k]), k


def test_accelerated_loops_precedence_and_fixed_point(oracle_mod):
    # precedence of the flags (projected_jacobi.cpp:470-489): Nesterov > Chebyshev > Anderson; and
    # every loop converges to the plain loop's fixed point (same step, tight tolerances)
    from cardillocxx_gb300 import scenes
    s = scenes.generate("pile_1k", scale=0.1)
    base = scenes.config_for("pile_1k")
    warm = oracle_mod.Oracle(s, base)
    warm.step(60)
    st = warm.state()
    s2 = dict(s, pos=st["pos"], quat=st["quat"], vel=st["vel"], omega=st["omega"])

    def one(**extra):
        c = scenes.config_for("pile_1k", **{"pj.tol_abs": 1e-10, "pj.tol_rel": 1e-9, "pj.max_iterations": 20000,
                                            "pj.warmstart": False, **extra})
        o = oracle_mod.Oracle(s2, c)
        o.step(1)
        return o.state()["vel"], o.stats()["iterations"]

    v_plain, it_plain = one()
    v_cheb, _ = one(**{"pj.chebyshev": True})
    v_and, it_and = one(**{"pj.anderson": True})
    v_and5, _ = one(**{"pj.anderson": True, "pj.anderson_m": 5})
    v_nes, _ = one(**{"pj.nesterov": True})
    assert np.array_equal(one(**{"pj.chebyshev": True, "pj.anderson": True})[0], v_cheb)
    assert np.array_equal(one(**{"pj.nesterov": True, "pj.anderson": True})[0], v_nes)
    scale = np.max(np.abs(v_plain))
    for v in (v_cheb, v_and, v_and5, v_nes):
        assert np.max(np.abs(v - v_plain)) <= 1e-5 * scale
    assert it_and < it_plain


def test_delassus_block_inverse(oracle_mod):
    # invertSmallSpd (misc/block_diagonal.hpp:15-27) restated as a Cholesky inverse; Eigen's
    # isDiagonal test (off-diagonals <= 1e-12 of the largest diagonal) picks the per-row path
    rng = np.random.default_rng(7)
    M = rng.normal(size=(3, 3))
    A = M @ M.T + 3 * np.eye(3)
    X, diag = oracle_mod.block_inverse(A)
    assert not diag
    np.testing.assert_allclose(X @ A, np.eye(3), atol=1e-13)
    X1, d1 = oracle_mod.block_inverse([[4.0]])
    assert d1 and X1[0, 0] == 0.25
    near = np.diag([2.0, 5.0, 5.0])
    near[0, 1] = near[1, 0] = 1e-13 * 5.0
    assert oracle_mod.block_inverse(near)[1]
    near[0, 1] = 1e-11 * 5.0
    assert not oracle_mod.block_inverse(near)[1]


def test_true_delassus_block_matches_row_scale_for_spheres(oracle_mod):
    # for sphere contacts with isotropic inertia a contact's 3x3 Delassus block is diagonal up to
    # rounding, so pj.rdiag_true_delassus (projected_jacobi.cpp:81-98, 341-347) takes the per-row
    # path and ends where the default row scale ends, up to rounding
    from cardillocxx_gb300 import scenes
    s = scenes.generate("pile_1k", scale=0.2)
    out = []
    for blk in (False, True):
        o = oracle_mod.Oracle(s, scenes.config_for("pile_1k", **{"pj.rdiag_true_delassus": blk}))
        o.step(120)
        out.append((o.state(), o.stats()))
    assert out[0][1]["num_contacts"] == out[1][1]["num_contacts"] > 0
    np.testing.assert_allclose(out[1][0]["vel"], out[0][0]["vel"], rtol=0, atol=1e-10)
    assert not np.array_equal(out[1][0]["vel"], out[0][0]["vel"])  # different rounding: the key is live


def test_csr_with_configuration(oracle_mod):
    # the solver-level drop-in under the configuration: the plain loop equals the explicit-argument
    # form bit for bit; every loop reaches the plain loop's fixed point. The Delassus block
    # preconditioner changes the metric of the cone projection (its blocks are not diagonal here),
    # so it has a fixed point of its own, which its accelerated loops reach too.
    p = csr_problem()
    keys = {"pj.alpha": 0.3, "pj.max_iterations": 60, "pj.tol_abs": 0.0, "pj.tol_rel": 0.0}
    x0, l0, it0 = oracle_mod.pj_solve_csr(**{k: v for k, v in p.items()}, alpha=0.3, max_iter=60, tol_abs=0.0,
                                          tol_rel=0.0)
    x1, l1, it1 = oracle_mod.pj_solve_csr_cfg(keys, **p)
    assert it0 == it1 == 60 and np.array_equal(x0, x1) and np.array_equal(l0, l1)
    tight = {"pj.alpha": 0.3, "pj.max_iterations": 50000, "pj.tol_abs": 1e-12, "pj.tol_rel": 1e-11}
    for base in ({}, {"pj.rdiag_true_delassus": True}):
        ref, _, it_ref = oracle_mod.pj_solve_csr_cfg(dict(tight, **base), **p)
        assert it_ref < 50000
        for extra in ({"pj.nesterov": True}, {"pj.chebyshev": True}, {"pj.anderson": True, "pj.anderson_m": 3}):
            x, lam, it = oracle_mod.pj_solve_csr_cfg(dict(tight, **base, **extra), **p)
            assert it < 50000, extra
            np.testing.assert_allclose(x, ref, rtol=0, atol=1e-7 * np.abs(ref).max(), err_msg=str((base, extra)))


def test_implicit_gyroscopy_drops_the_gyroscopic_force(oracle_mod):
    # moreau.implicit_gyroscopy (pj_assembler.cpp:32-61, 152-153): for isotropic spheres the
    # linearised gyroscopic block of S is exactly zero, so only dt f_gyro leaves the right-hand side.
    # A spinning sphere in free flight keeps its body-frame spin exactly; the explicit form differs
    # from that by the rounding of w x (I w) only
    s = make_scene([{"pos": (0.0, 0.0, 1.0), "radius": 0.05, "omega": (3.0, -7.0, 11.0)}], [GROUND])
    o_imp = oracle_mod.Oracle(s, cfg(**{"moreau.implicit_gyroscopy": True}))
    o_imp.step(20)
    assert np.array_equal(o_imp.state()["omega"][0], [3.0, -7.0, 11.0])
    o_exp = oracle_mod.Oracle(s, cfg())
    o_exp.step(20)
    np.testing.assert_allclose(o_exp.state()["omega"][0], [3.0, -7.0, 11.0], rtol=1e-12)


# ---- projected Gauss-Seidel (projected_gauss_seidel.cpp:56-264) ----
PGS = {"solver.type": "pgs", "pj.alpha": 1.0, "pj.relaxation": 1.0, "pj.tol_abs": 1e-12, "pj.tol_rel": 1e-12,
       "pj.max_iterations": 10000}


def test_pgs_one_sweep_is_sequential(oracle_mod):
    # two equal spheres stacked on the ground (touching within 1e-6 m), at rest, frictionless: one
    # sweep visits the ground
    # contact first (it stops the lower sphere, lambda_0 = -m g h inside the solver), then the
    # sphere-sphere contact, which sees the lower sphere's corrected velocity and shares it
    # (lambda_1 = -m g h / 2): both spheres leave the sweep at -g h / 2. A Jacobi sweep would leave
    # the upper sphere at -g h.
    r = 0.05
    s = make_scene([{"pos": (0.0, 0.0, r), "radius": r, "mu": 0.0},
                    {"pos": (0.0, 0.0, 3 * r - 1e-6), "radius": r, "mu": 0.0}], [dict(GROUND, mu=0.0)])
    m = s["mass"][0]
    o = oracle_mod.Oracle(s, cfg(**dict(PGS, **{"pj.max_iterations": 1, "pj.warmstart": False,
                                                "pj.tol_abs": 1.0, "pj.tol_rel": 1.0})))
    o.step(1)
    c = o.contacts()
    assert c["id_a"].tolist() == [0, 1] and c["id_b"].tolist() == [1, 2]
    np.testing.assert_allclose(c["lambda"][:, 0], [m * G * H, m * G * H / 2], rtol=1e-12)
    np.testing.assert_allclose(o.state()["vel"][:, 2], [-G * H / 2, -G * H / 2], rtol=1e-12)
    assert o.stats()["iterations"] == 1


def test_pgs_resting_contact_and_sliding_friction(oracle_mod):
    r, mu, v0 = 0.05, 0.3, 1.0
    s = make_scene([{"pos": (0.0, 0.0, r), "radius": r, "vel": (v0, 0, 0), "mu": mu}], [dict(GROUND, mu=mu)])
    m = s["mass"][0]
    o = oracle_mod.Oracle(s, cfg(**PGS))
    o.step(1)
    c = o.contacts()
    # stored convention: the normal impulse non-negative; it carries the weight
    np.testing.assert_allclose(c["lambda"][0, 0], m * G * H, rtol=1e-9)
    assert abs(o.state()["vel"][0, 2]) < 1e-10
    o.step(9)
    # sliding: v decreases by mu g per unit time, the spin grows by the friction torque
    np.testing.assert_allclose(o.state()["vel"][0, 0], v0 - mu * G * 10 * H, rtol=1e-8)
    np.testing.assert_allclose(o.state()["omega"][0, 1], 10 * H * 5 * mu * G / (2 * r), rtol=1e-8)
    o.step(190)
    # rolling from t = 2 v0 / (7 mu g): v = 5 v0 / 7
    np.testing.assert_allclose(o.state()["vel"][0, 0], 5 * v0 / 7, rtol=1e-8)


def test_pgs_converges_to_the_projected_jacobi_solution(oracle_mod):
    from cardillocxx_gb300 import scenes
    s = scenes.generate("pile_1k", scale=0.1)
    base = scenes.config_for("pile_1k")
    o = oracle_mod.Oracle(s, base)
    o.step(200)
    st = o.state()
    sc = dict(s)
    for k in st:
        sc[k] = st[k].copy()
    tight = {"pj.tol_abs": 1e-10, "pj.tol_rel": 1e-10, "pj.max_iterations": 100000, "pj.warmstart": False}
    pj = oracle_mod.Oracle(sc, dict(base, **tight))
    pj.step(1)
    gs = oracle_mod.Oracle(sc, dict(base, **tight, **{"solver.type": "pgs", "pj.alpha": 1.0, "pj.relaxation": 1.0}))
    gs.step(1)
    assert gs.stats()["num_contacts"] > 20
    vs = np.abs(st["vel"]).max() + G * 1e-3
    assert np.abs(pj.state()["vel"] - gs.state()["vel"]).max() <= 1e-6 * vs
    # Gauss-Seidel with alpha 1 takes fewer sweeps than Jacobi with alpha 0.5
    assert gs.stats()["iterations"] < pj.stats()["iterations"]
    # without a tolerance the velocity-increment residual divides by zero: the reference throws
    # "Projected Gauss-Seidel diverged" (projected_gauss_seidel.cpp:144-147)
    with pytest.raises(RuntimeError):
        oracle_mod.Oracle(sc, dict(base, **{"solver.type": "pgs"})).step(1)


# ---- prescribed static motion (Trajectory::update, trajectory.cpp:69-120) ----
def test_prescribed_wall_velocity_moves_resting_sphere(oracle_mod):
    # the ground's twist set for one step: its velocity enters the contact (its plane stays where it
    # was built, collision_coal.cpp:386-391); a resting sphere leaves the step at the wall's normal
    # velocity, and a tangential wall velocity drags it by kinetic friction, mu g h a step
    r, mu = 0.05, 0.3
    s = make_scene([{"pos": (0.0, 0.0, r), "radius": r, "mu": mu}], [dict(GROUND, mu=mu)])
    o = oracle_mod.Oracle(s, cfg())
    o.set_static_motion([0], vel=[(0.0, 0.0, 0.1)])
    o.step(1)
    np.testing.assert_allclose(o.state()["vel"][0, 2], 0.1, rtol=1e-9)
    st = o.static_state()
    np.testing.assert_allclose(st["vel"][0], [0.0, 0.0, 0.1])
    np.testing.assert_allclose(st["pos"][0], [0.0, 0.0, 0.5 * H * 0.1], rtol=1e-12)
    c = oracle_mod.Oracle(s, cfg())
    c.set_static_motion([0], vel=[(1.0, 0.0, 0.0)])
    c.step(1)
    np.testing.assert_allclose(c.state()["vel"][0, 0], mu * G * H, rtol=1e-9)
    # a prescribed pose: the drum moved down by 1 mm leaves a sphere that rested on its wall free
    R = 0.3
    d = make_scene([{"pos": (0.0, 0.0, -R + r), "radius": r}],
                   [{"kind": "drum", "pos": (0, 0, 0), "dir": (0, 1, 0), "radius": R, "mu": 0.3}])
    od = oracle_mod.Oracle(d, cfg())
    od.step(1)
    assert od.stats()["num_contacts"] == 1
    od.set_static_motion([0], pos=[(0.0, 0.0, -1e-3)], quat=[(0.0, 0.0, 0.0, 1.0)])
    od.step(1)
    assert od.stats()["num_contacts"] == 0
    np.testing.assert_allclose(od.static_state()["pos"][0], [0.0, 0.0, -1e-3])


# ---- solid cylinder (C_RB_Cylinder, coal::Cylinder; collision_coal.cpp:307-310) ----
def cyl(**kw):
    c = {"kind": "cylinder", "pos": (0.0, 0.0, 0.0), "dir": (0.0, 0.0, 1.0), "radius": 0.2, "half_length": 0.1,
         "mu": 0.3}
    c.update(kw)
    return c


@pytest.mark.parametrize("centre, normal", [
    ((0.05, -0.03, 0.15), (0.0, 0.0, 1.0)),                                 # on the top cap
    ((0.25, 0.0, 0.02), (1.0, 0.0, 0.0)),                                   # against the side
    ((0.2 + 0.03, 0.0, 0.1 + 0.04), (0.6, 0.0, 0.8)),                       # on the rim: centre 0.05 from it
    ((0.17, 0.0, 0.0), (1.0, 0.0, 0.0)),                                    # centre inside, nearer the side
    ((0.0, 0.0, -0.09), (0.0, 0.0, -1.0)),                                  # centre inside, nearer the bottom cap
])
def test_cylinder_contact_geometry(oracle_mod, centre, normal):
    # zero gravity, at rest: one contact whose normal points from the cylinder to the sphere and
    # whose point is the midpoint of the two surfaces' nearest points
    r = 0.05
    s = make_scene([{"pos": centre, "radius": r}], [cyl()])
    o = oracle_mod.Oracle(s, cfg(**{"sim.gravity": (0.0, 0.0, 0.0)}))
    o.step(1)
    c = o.contacts()
    assert c["id_a"].tolist() == [0] and c["id_b"].tolist() == [1]
    np.testing.assert_allclose(c["normal"][0], normal, atol=1e-12)


def test_sphere_rests_on_cylinder_cap_and_side(oracle_mod):
    r = 0.05
    # touching within 1e-9 m (0.1 + 0.05 rounds above 0.15)
    for body, c in (({"pos": (0.02, 0.0, 0.1 + r - 1e-9)}, cyl()),
                    ({"pos": (0.0, 0.0, 0.2 + r - 1e-9)}, cyl(dir=(1.0, 0.0, 0.0)))):
        s = make_scene([dict(body, radius=r)], [c])
        m = s["mass"][0]
        o = oracle_mod.Oracle(s, cfg())
        o.step(1)
        lam = o.contacts()["lambda"][0]
        np.testing.assert_allclose(lam[0], m * G * H, rtol=1e-10)
        assert abs(o.state()["vel"][0, 2]) < 1e-12


# ---- solid box (C_RB_Cube, coal::Box; collision_coal.cpp:288-290) ----
def box(**kw):
    b = {"kind": "box", "pos": (0.0, 0.0, 0.0), "half_extents": (0.3, 0.2, 0.1), "mu": 0.3}
    b.update(kw)
    return b


def _rotz(deg):
    a = math.radians(deg) / 2
    return (0.0, 0.0, math.sin(a), math.cos(a))


@pytest.mark.parametrize("centre, normal", [
    ((0.1, -0.05, 0.14), (0.0, 0.0, 1.0)),                                  # on the top face
    ((0.33, 0.05, 0.0), (1.0, 0.0, 0.0)),                                   # against the +x face
    ((-0.1, -0.24, 0.02), (0.0, -1.0, 0.0)),                                # against the -y face
    ((0.3 + 0.03, 0.0, 0.1 + 0.04), (0.6, 0.0, 0.8)),                       # on an edge: centre 0.05 from it
    ((0.3 + 0.02, 0.2 + 0.02, 0.1 + 0.01), (2 / 3, 2 / 3, 1 / 3)),          # on a corner: centre 0.03 from it
    ((0.28, 0.0, 0.0), (1.0, 0.0, 0.0)),                                    # centre inside, nearest +x
    ((0.0, 0.0, -0.09), (0.0, 0.0, -1.0)),                                  # centre inside, nearest -z
])
@pytest.mark.parametrize("turn", [0.0, 30.0])
def test_box_contact_geometry(oracle_mod, centre, normal, turn):
    # zero gravity, at rest: one contact whose normal points from the box to the sphere, in the box's
    # own axes (the box turned about z by `turn` degrees, the sphere with it)
    r = 0.05
    q = _rotz(turn)
    c, s_ = math.cos(math.radians(turn)), math.sin(math.radians(turn))
    rot = np.array([[c, -s_, 0.0], [s_, c, 0.0], [0.0, 0.0, 1.0]])
    x = rot @ np.array(centre)
    sc = make_scene([{"pos": tuple(x), "radius": r}], [box(quat=q)])
    o = oracle_mod.Oracle(sc, cfg(**{"sim.gravity": (0.0, 0.0, 0.0)}))
    o.step(1)
    k = o.contacts()
    assert k["id_a"].tolist() == [0] and k["id_b"].tolist() == [1]
    np.testing.assert_allclose(k["normal"][0], rot @ np.array(normal), atol=1e-12)
    # the point is the midpoint of the box's nearest point and the sphere's deepest point
    n = rot @ np.array(normal)
    loc = np.array(centre)
    e = np.array([0.3, 0.2, 0.1])
    if np.all(np.abs(loc) <= e):
        f = int(np.argmin(e - np.abs(loc)))
        qb = loc.copy()
        qb[f] = math.copysign(e[f], loc[f])
    else:
        qb = np.clip(loc, -e, e)
    np.testing.assert_allclose(k["point"][0], 0.5 * ((rot @ qb) + (x - r * n)), atol=1e-12)


def test_box_far_sphere_has_no_contact(oracle_mod):
    sc = make_scene([{"pos": (0.3 + 0.04, 0.2 + 0.04, 0.0), "radius": 0.05}], [box()])
    o = oracle_mod.Oracle(sc, cfg(**{"sim.gravity": (0.0, 0.0, 0.0)}))
    o.step(1)
    # 0.04 * sqrt(2) = 0.0566 > 0.05 from the edge: apart
    assert o.stats()["num_contacts"] == 0


def test_sphere_rests_on_box_and_slides_on_it(oracle_mod):
    r = 0.05
    # resting on the top face of a box turned about z: the impulse carries the weight
    s = make_scene([{"pos": (0.05, 0.02, 0.1 + r - 1e-9), "radius": r}], [box(quat=_rotz(40.0))])
    m = s["mass"][0]
    o = oracle_mod.Oracle(s, cfg())
    o.step(1)
    np.testing.assert_allclose(o.contacts()["lambda"][0][0], m * G * H, rtol=1e-10)
    assert abs(o.state()["vel"][0, 2]) < 1e-12
    # sliding along the top face: Coulomb friction takes mu g h a step off the speed
    mu = 0.3
    s = make_scene([{"pos": (0.0, 0.0, 0.1 + r - 1e-9), "radius": r, "vel": (1.0, 0.0, 0.0), "mu": mu}],
                   [box(mu=mu, half_extents=(3.0, 3.0, 0.1))])
    o = oracle_mod.Oracle(s, cfg())
    o.step(1)
    v = o.state()["vel"][0, 0]
    assert 1.0 - mu * G * H - 1e-9 < v < 1.0


def test_box_moves_with_its_prescribed_pose(oracle_mod):
    # a box turned by a prescribed orientation carries its faces with it: a sphere above the +x end
    # of a long thin box touches it only once the box is tilted up at that end
    r = 0.05
    sc = make_scene([{"pos": (0.9, 0.0, 0.1 + r + 0.05), "radius": r}],
                    [box(half_extents=(1.0, 0.2, 0.1))])
    o = oracle_mod.Oracle(sc, cfg(**{"sim.gravity": (0.0, 0.0, 0.0)}))
    o.step(1)
    assert o.stats()["num_contacts"] == 0
    a = math.radians(4.0) / 2  # about -y: the +x end rises by 0.9 * sin(4 deg) = 0.063
    o.set_static_motion([0], quat=[(0.0, -math.sin(a), 0.0, math.cos(a))])
    o.step(1)
    assert o.stats()["num_contacts"] == 1
    c = o.contacts()
    np.testing.assert_allclose(c["normal"][0], [-math.sin(2 * a), 0.0, math.cos(2 * a)], atol=1e-12)


def test_cylinder_axis_turns_with_the_static(oracle_mod):
    # coal poses the cylinder with the static's transform every step: a prescribed quarter turn about
    # z swings a cylinder lying along x onto y, under a sphere that it did not reach before
    r = 0.05
    sc = make_scene([{"pos": (0.0, 0.32, 0.0), "radius": r}],
                    [cyl(dir=(1.0, 0.0, 0.0), radius=0.1, half_length=0.3)])
    o = oracle_mod.Oracle(sc, cfg(**{"sim.gravity": (0.0, 0.0, 0.0)}))
    o.step(1)
    assert o.stats()["num_contacts"] == 0
    a = math.pi / 4
    o.set_static_motion([0], quat=[(0.0, 0.0, math.sin(a), math.cos(a))])
    o.step(1)
    assert o.stats()["num_contacts"] == 1
    np.testing.assert_allclose(o.contacts()["normal"][0], [0.0, 1.0, 0.0], atol=1e-12)


def test_scene_without_bodies_and_a_lone_sphere(oracle_mod):
    # nothing to collide: no contacts, no sweeps
    o = oracle_mod.Oracle(make_scene([], [{"kind": "halfspace", "pos": (0, 0, 0), "dir": (0, 0, 1)}]), cfg())
    o.step(3)
    st = o.stats()
    assert st["num_contacts"] == 0 and st["iterations"] == 0
    # a sphere with no statics falls freely: after n midpoint steps from rest x = x0 - g h^2 n^2 / 2
    o = oracle_mod.Oracle(make_scene([{"pos": (0.0, 0.0, 1.0), "radius": 0.1}], []), cfg())
    n = 7
    o.step(n)
    np.testing.assert_allclose(o.state()["pos"][0, 2], 1.0 - G * H * H * n * n / 2, rtol=0, atol=1e-14)
    np.testing.assert_allclose(o.state()["vel"][0, 2], -G * H * n, rtol=1e-12)
