"""Frozen golden fixtures (tests/golden/*.npz, made by tests/golden/make_golden.py).

CPU: the oracle reproduces every fixture bit-for-bit (it is IEEE FP64 without contraction, so
this holds across hosts). GPU: the plain FP64 method reproduces them bit-for-bit too.
"""
import numpy as np
import pytest

from tests.golden.make_golden import NAMES, load


def _check(state, contacts, d, tag):
    for k in ("pos", "quat", "vel", "omega"):
        assert np.array_equal(state[k], d[f"out_{k}"]), f"{tag}: {k}"
    for k in ("id_a", "id_b", "point", "lambda", "normal"):
        assert np.array_equal(contacts[k], d[f"contact_{k}"]), f"{tag}: contact {k}"


@pytest.mark.parametrize("name", NAMES)
def test_oracle_reproduces_fixture(oracle_mod, name):
    scene, meta, d = load(name)
    o = oracle_mod.Oracle(scene, meta["cfg"])
    o.step(meta["steps"])
    _check(o.state(), o.contacts(), d, name)
    assert o.stats() == meta["stats"]


def test_oracle_csr_fixture(oracle_mod):
    import os
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "csr.npz"))
    args = {k: d[k] for k in ("row_ptr", "col", "val", "contact_bias", "mu", "restitution", "minv", "mdiag", "v",
                              "f_ext", "f_gyro", "lam0")}
    x, lam, it = oracle_mod.pj_solve_csr(**args, dt=1e-3, alpha=0.3, max_iter=40, tol_abs=0.0, tol_rel=0.0,
                                         nfl=int(d["nfl"]))
    assert it == int(d["out_iters"])
    assert np.array_equal(x, d["out_x"]) and np.array_equal(lam, d["out_lambda"])


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_gpu_fp64_reproduces_fixture(gpu, name):
    from cardillocxx_gb300 import PhysicsEngine
    scene, meta, d = load(name)
    e = PhysicsEngine(meta["cfg"]).load_scene(scene)
    e.step(meta["steps"])
    _check(e.state(), e.contacts(), d, name)
    st = e.stats()
    assert st["iterations"] == meta["stats"]["iterations"]
    assert st["residual"] == meta["stats"]["residual"]


@pytest.mark.gpu
def test_gpu_csr_fixture(gpu):
    import os
    from cardillocxx_gb300 import PhysicsEngine
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "csr.npz"))
    args = {k: d[k] for k in ("row_ptr", "col", "val", "contact_bias", "mu", "restitution", "minv", "mdiag", "v",
                              "f_ext", "f_gyro", "lam0")}
    x, lam, it = PhysicsEngine({}).pj_solve_csr(**args, dt=1e-3, alpha=0.3, max_iter=40, tol_abs=0.0, tol_rel=0.0,
                                               nfl=int(d["nfl"]))
    assert it == int(d["out_iters"])
    assert np.array_equal(x, d["out_x"]) and np.array_equal(lam, d["out_lambda"])
