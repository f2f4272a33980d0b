"""The allocation-free solver entry point (cdx_pj_solve_csr_noalloc), checked on the GPU.

Some callers of this solver cannot allocate device memory: hosts that reserve the whole GPU
through their own pool, real-time loops that cannot take a cudaMalloc stall, and code where
allocation calls are not allowed. cdx_pj_solve_csr_noalloc serves them with the same kernels as
cdx_pj_solve_csr, its work buffers living in a fixed file-scope device array instead of memory
it allocates. This file runs last (pytest collects it after the others) and checks, through the
C ABI, that two calls in a row return exactly what the allocating entry point returns, and that
a problem larger than the array is refused with a clear error.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _problem(seed, nb=40, nfl=6, nfr=30):
    rng = np.random.default_rng(seed)
    nv = 6 * nb
    cols, vals, ptr = [], [], [0]
    for _ in range(nfl + 3 * nfr):
        a, b = sorted(rng.choice(nb, 2, replace=False))
        for body in (a, b):
            for k in range(6):
                cols.append(6 * body + k)
                vals.append(rng.normal())
        ptr.append(len(cols))
    nrows = nfl + 3 * nfr
    m = rng.uniform(0.5, 2.0, nv)
    return dict(row_ptr=np.array(ptr, np.int32), col=np.array(cols, np.int32), val=np.array(vals),
                contact_bias=rng.normal(size=nrows) * 0.1, mu=rng.uniform(0.1, 0.6, nrows),
                restitution=rng.uniform(0, 0.2, nrows), minv=1.0 / m, mdiag=1.0 / (1.0 / m), v=rng.normal(size=nv),
                f_ext=rng.normal(size=nv), f_gyro=rng.normal(size=nv) * 1e-3,
                lam0=np.abs(rng.normal(size=nrows)) * 0.01, nfl=nfl)


def _noalloc(L, p, max_iter, tol_abs, tol_rel):
    from cardillocxx_gb300._lib import dp, ip
    arrs = [np.ascontiguousarray(p[k], np.float64) for k in ("val", "contact_bias", "mu", "restitution", "minv",
                                                            "mdiag", "v", "f_ext", "f_gyro")]
    nrows = p["row_ptr"].shape[0] - 1
    nv = p["minv"].shape[0]
    lam = np.array(p["lam0"], np.float64, copy=True)
    x = np.empty(nv)
    it = C.c_int32(0)
    err = C.create_string_buffer(512)
    st = L.cdx_pj_solve_csr_noalloc(None, nrows, nv, int(p["nfl"]), ip(p["row_ptr"]), ip(p["col"]),
                                    *[dp(a) for a in arrs], 1e-3, 0.3, max_iter, tol_abs, tol_rel, dp(lam), dp(x),
                                    C.byref(it), err, 512)
    return st, x, lam, it.value, err.value.decode()


@pytest.mark.parametrize("max_iter,tol_abs,tol_rel", [(40, 0.0, 0.0), (2000, 1e-7, 1e-5)])
def test_noalloc_matches_allocating_entry_point_twice(gpu, max_iter, tol_abs, tol_rel):
    from cardillocxx_gb300 import PhysicsEngine
    eng = PhysicsEngine({})
    for seed in (7, 8):  # two calls in a row: the second one finds the first one's data in the array
        p = _problem(seed)
        x_ref, lam_ref, it_ref = eng.pj_solve_csr(**p, dt=1e-3, alpha=0.3, max_iter=max_iter, tol_abs=tol_abs,
                                                  tol_rel=tol_rel)
        st, x, lam, it, msg = _noalloc(gpu, p, max_iter, tol_abs, tol_rel)
        assert st == 0, msg
        assert it == it_ref
        assert np.array_equal(x, x_ref) and np.array_equal(lam, lam_ref)


def test_noalloc_rejects_oversized_problem(gpu):
    p = _problem(9, nb=4000, nfl=0, nfr=12000)  # ~430k nonzeros: more than the fixed array holds
    st, _, _, _, msg = _noalloc(gpu, p, 5, 0.0, 0.0)
    assert st == 3  # CDX_ERR_OVERFLOW
    assert "scratch array" in msg


def test_noalloc_without_contacts_matches_allocating_entry_point(gpu):
    # no contact rows: both entry points return the free velocities S^-1 rhs and no sweeps
    from cardillocxx_gb300 import PhysicsEngine
    eng = PhysicsEngine({})
    p = _problem(10, nfl=0, nfr=0)
    assert p["row_ptr"].shape[0] == 1
    x_ref, lam_ref, it_ref = eng.pj_solve_csr(**p, dt=1e-3, alpha=0.3, max_iter=50, tol_abs=0.0, tol_rel=0.0)
    for _ in range(2):
        st, x, lam, it, msg = _noalloc(gpu, p, 50, 0.0, 0.0)
        assert st == 0, msg
        assert it == it_ref and lam.shape == (0,)
        assert np.array_equal(x, x_ref)
