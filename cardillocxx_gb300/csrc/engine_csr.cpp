// cdx_pj_solve_csr: host side of the solver-level drop-in (ProjectedJacobiSolver::solve with
// S = diag(M), projected_jacobi.cpp:451-500). Host arrays in, host arrays out; the work buffers
// are kept by the context and only grow.
#include <algorithm>
#include <cstring>
#include <vector>

#include "engine.h"

using namespace cdx;


static int grow(Engine& E, CsrBuffers& B, int64_t nnz, int64_t nrows, int64_t nv) {
    int st;
    if (!B.ds && (st = E.dalloc((void**)&B.ds, sizeof(DevScalars), "csr"))) return st;
    if (nnz > B.nnz_cap) {
        void* old[] = {B.col, B.rowidx, B.ck_in, B.ck_out, B.nz_in, B.nz_out, B.val, B.RW};
        for (void* p : old) E.dfree(p);
        const int64_t c = std::max<int64_t>(nnz + nnz / 4, 64);
        if ((st = E.dalloc((void**)&B.col, 4 * c, "csr"))) return st;
        if ((st = E.dalloc((void**)&B.rowidx, 4 * c, "csr"))) return st;
        if ((st = E.dalloc((void**)&B.ck_in, 4 * c, "csr"))) return st;
        if ((st = E.dalloc((void**)&B.ck_out, 4 * c, "csr"))) return st;
        if ((st = E.dalloc((void**)&B.nz_in, 4 * c, "csr"))) return st;
        if ((st = E.dalloc((void**)&B.nz_out, 4 * c, "csr"))) return st;
        if ((st = E.dalloc((void**)&B.val, 8 * c, "csr"))) return st;
        if ((st = E.dalloc((void**)&B.RW, 8 * c, "csr"))) return st;
        B.nnz_cap = c;
    }
    if (nrows + 1 > B.row_cap) {
        void* old[] = {B.ptr, B.cb, B.mu, B.e, B.biasR, B.lam, B.dlam};
        for (void* p : old) E.dfree(p);
        const int64_t c = std::max<int64_t>(nrows + 1 + nrows / 4, 64);
        if ((st = E.dalloc((void**)&B.ptr, 4 * c, "csr"))) return st;
        double** d[] = {&B.cb, &B.mu, &B.e, &B.biasR, &B.lam, &B.dlam};
        for (auto p : d)
            if ((st = E.dalloc((void**)p, 8 * c, "csr"))) return st;
        B.row_cap = c;
    }
    if (nv > B.nv_cap) {
        void* old[] = {B.cstart, B.cend, B.minv, B.mdiag, B.v, B.fext, B.fgyro, B.rhs, B.x};
        for (void* p : old) E.dfree(p);
        const int64_t c = std::max<int64_t>(nv + nv / 4, 64);
        if ((st = E.dalloc((void**)&B.cstart, 4 * c, "csr"))) return st;
        if ((st = E.dalloc((void**)&B.cend, 4 * c, "csr"))) return st;
        double** d[] = {&B.minv, &B.mdiag, &B.v, &B.fext, &B.fgyro, &B.rhs, &B.x};
        for (auto p : d)
            if ((st = E.dalloc((void**)p, 8 * c, "csr"))) return st;
        B.nv_cap = c;
    }
    return E.ensure_tmp(std::max<int64_t>(nnz, nv + 1));
}

// the work buffers belong to the context: created on first use, their device memory is in the
// context's owned list and goes away with it
static CsrBuffers& buffers(Engine& E) {
    if (!E.csr) E.csr = new CsrBuffers();
    return *E.csr;
}

// the solve's options: the explicit arguments of cdx_pj_solve_csr, or a configuration
struct CsrOpts {
    double alpha = 0.0, tol_abs = 0.0, tol_rel = 0.0, residual_tol = 0.0;
    int max_iter = 1, check_every = 10;
    int nesterov = 0, chebyshev = 0, anderson = 0, anderson_m = 2, block = 0, restart_limit = 10000;
    double beta_threshold = 1.0;
};

static int grow_extra(Engine& E, CsrBuffers& B, const CsrOpts& o, int64_t nrows, int64_t nv) {
    int st;
    const int64_t nunits = nrows;  // at most one unit a row
    if (o.block && nunits > B.unit_cap) {
        if (B.Rb) E.dfree(B.Rb);
        const int64_t c = std::max<int64_t>(nunits + nunits / 4, 64);
        if ((st = E.dalloc((void**)&B.Rb, sizeof(double) * 9 * c, "csr blocks"))) return st;
        B.unit_cap = c;
    }
    if (o.block && !B.full && (st = E.dalloc((void**)&B.full, sizeof(int32_t), "csr blocks"))) return st;
    if ((o.nesterov || o.chebyshev) && (nrows > B.acc_rows || nv > B.acc_nv)) {
        double** bufs[] = {&B.xk, &B.xk1, &B.xy, &B.pk, &B.pk1, &B.py, &B.part};
        for (auto b : bufs)
            if (*b) {
                E.dfree(*b);
                *b = nullptr;
            }
        const int64_t cn = std::max<int64_t>(nv + nv / 4, 64), cr = std::max<int64_t>(nrows + nrows / 4, 64);
        for (int k = 0; k < 3; ++k)
            if ((st = E.dalloc((void**)bufs[k], sizeof(double) * cn, "csr accelerated loop"))) return st;
        for (int k = 3; k < 6; ++k)
            if ((st = E.dalloc((void**)bufs[k], sizeof(double) * cr, "csr accelerated loop"))) return st;
        if ((st = E.dalloc((void**)&B.part, sizeof(double) * (cn / 256 + 2), "csr accelerated loop"))) return st;
        B.acc_rows = cr;
        B.acc_nv = cn;
    }
    if ((o.nesterov || o.chebyshev) && !B.st && (st = E.dalloc((void**)&B.st, sizeof(AccelState), "csr loop")))
        return st;
    if (o.anderson && !o.nesterov && !o.chebyshev) {
        AndersonBufs& A = B.anderson;
        const int m = std::max(1, o.anderson_m);
        const int64_t nt = nv + nrows;
        if (!(A.st && A.m == m && nt <= A.nt_cap)) {
            double** bufs[] = {&A.z, &A.w, &A.f, &A.cand, &A.zh, &A.fh, &A.part, &A.ls};
            for (auto b : bufs)
                if (*b) {
                    E.dfree(*b);
                    *b = nullptr;
                }
            if (A.st) E.dfree(A.st);
            A.st = nullptr;
            const int64_t cap = std::max<int64_t>(nt + nt / 4, 16);
            for (int k = 0; k < 4; ++k)
                if ((st = E.dalloc((void**)bufs[k], sizeof(double) * cap, "csr Anderson loop"))) return st;
            for (int k = 4; k < 6; ++k)
                if ((st = E.dalloc((void**)bufs[k], sizeof(double) * cap * (m + 1), "csr Anderson loop"))) return st;
            if ((st = E.dalloc((void**)&A.part, sizeof(double) * anderson_chunks(cap) * anderson_sums(m),
                               "csr Anderson loop"))) return st;
            if ((st = E.dalloc((void**)&A.ls, sizeof(double) * ((int64_t)m * m + 2 * m), "csr Anderson loop"))) return st;
            if ((st = E.dalloc((void**)&A.st, sizeof(AndersonState), "csr Anderson loop"))) return st;
            A.m = m;
            A.nt_cap = cap;
        }
        A.nt = nt;
        A.plain = 1;
    }
    return CDX_OK;
}

// ProjectedJacobiSolver::solve (projected_jacobi.cpp:451-500) on the CSR problem: setup, x0, then
// the loop the options select (Nesterov > Chebyshev > Anderson > standard, :470-491)
static int csr_solve(cdx_ctx* ctx, const CsrOpts& o, int32_t nrows, int32_t nv, int32_t nfl, const int32_t* row_ptr,
                     const int32_t* col, const double* val, const double* contact_bias, const double* mu,
                     const double* restitution, const double* minv, const double* mdiag, const double* v,
                     const double* f_ext, const double* f_gyro, double dt, double* lambda_inout, double* x_out,
                     int32_t* iterations) {
    if (!ctx) return CDX_ERR_ARG;
    Engine& E = ctx->eng;
    if (nrows < 0 || nv < 0 || nfl < 0 || nfl > nrows || (nrows - nfl) % 3 != 0)
        return E.fail(CDX_ERR_ARG, "rows must be nfl frictionless rows followed by 3-row blocks");
    if (!row_ptr || (nrows > 0 && (!col || !val || !contact_bias || !mu || !restitution || !lambda_inout)) ||
        (nv > 0 && (!minv || !mdiag || !v || !f_ext || !f_gyro || !x_out)))
        return E.fail(CDX_ERR_ARG, "missing array");
    const int64_t nnz = row_ptr[nrows];
    if (nnz < 0 || row_ptr[0] != 0) return E.fail(CDX_ERR_ARG, "bad row_ptr");
    for (int r = 0; r < nrows; ++r)
        if (row_ptr[r + 1] < row_ptr[r]) return E.fail(CDX_ERR_ARG, "row_ptr must be nondecreasing");
    for (int64_t k = 0; k < nnz; ++k)
        if (col[k] < 0 || col[k] >= nv) return E.fail(CDX_ERR_ARG, "column index out of range");
    if (o.block)
        for (int r = nfl; r + 2 < nrows; r += 3)
            if (row_ptr[r + 1] - row_ptr[r] != row_ptr[r + 2] - row_ptr[r + 1] ||
                row_ptr[r + 2] - row_ptr[r + 1] != row_ptr[r + 3] - row_ptr[r + 2])
                return E.fail(CDX_ERR_ARG, "pj.rdiag_true_delassus: the rows of a contact must share their columns");
    CsrBuffers& B = buffers(E);
    int st;
    if ((st = grow(E, B, nnz, nrows, nv))) return st;
    if ((st = grow_extra(E, B, o, nrows, nv))) return st;
    cudaStream_t s = E.stream;
    auto up = [&](void* d, const void* h, size_t bytes) {
        return bytes ? cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, s) : cudaSuccess;
    };
    cudaError_t ce = cudaSuccess;
    ce = ce ? ce : up(B.ptr, row_ptr, 4 * (size_t)(nrows + 1));
    ce = ce ? ce : up(B.col, col, 4 * (size_t)nnz);
    ce = ce ? ce : up(B.val, val, 8 * (size_t)nnz);
    ce = ce ? ce : up(B.cb, contact_bias, 8 * (size_t)nrows);
    ce = ce ? ce : up(B.mu, mu, 8 * (size_t)nrows);
    ce = ce ? ce : up(B.e, restitution, 8 * (size_t)nrows);
    ce = ce ? ce : up(B.lam, lambda_inout, 8 * (size_t)nrows);
    ce = ce ? ce : up(B.minv, minv, 8 * (size_t)nv);
    ce = ce ? ce : up(B.mdiag, mdiag, 8 * (size_t)nv);
    ce = ce ? ce : up(B.v, v, 8 * (size_t)nv);
    ce = ce ? ce : up(B.fext, f_ext, 8 * (size_t)nv);
    ce = ce ? ce : up(B.fgyro, f_gyro, 8 * (size_t)nv);
    if ((st = E.cuda_check(ce, "csr upload"))) return st;
    launch_csr_rhs(nv, B.mdiag, B.v, B.fext, B.fgyro, dt, B.rhs, s);
    int32_t iters = 0;
    if (nrows == 0) {
        // no contacts: the free solution
        launch_csr_cols(nv, B.cstart, B.cstart, B.nz_out, B.rowidx, B.val, B.lam, B.rhs, B.mdiag, B.x, 0, 0, 0, 0,
                        B.ds, s);
        cudaMemsetAsync(B.cstart, 0, 4 * (size_t)nv, s);
    } else {
        launch_csr_rowidx(nrows, B.ptr, B.rowidx, B.ck_in, B.nz_in, B.col, s);
        int bits = 1;
        while (((int64_t)1 << bits) <= nv) ++bits;
        if ((st = E.cuda_check(sort_pairs(E.tmp, E.tmp_bytes, B.ck_in, B.ck_out, B.nz_in, B.nz_out, nnz, bits, s),
                               "csr sort"))) return st;
        cudaMemsetAsync(B.cstart, 0, 4 * (size_t)nv, s);
        cudaMemsetAsync(B.cend, 0, 4 * (size_t)nv, s);
        launch_ranges(B.ck_out, nnz, B.cstart, B.cend, s);
        launch_csr_setup(nrows, B.ptr, B.col, B.val, B.cb, B.e, B.minv, B.v, o.alpha, B.RW, B.biasR, s, o.block);
        const double* Rb = nullptr;
        const int32_t* full = nullptr;
        if (o.block) {
            launch_csr_blocks(nrows, nfl, B.ptr, B.col, B.val, B.minv, o.alpha, B.Rb, B.full, s);
            Rb = B.Rb;
            full = B.full;
        }
        // x0 = S^-1 (rhs + W^T lambda0)
        launch_csr_cols(nv, B.cstart, B.cend, B.nz_out, B.rowidx, B.val, B.lam, B.rhs, B.mdiag, B.x, 0, 0, 0, 0,
                        B.ds, s);
        cudaMemsetAsync(B.ds, 0, sizeof(DevScalars), s);
        const int maxit = std::max(1, o.max_iter);
        const int every = std::max(1, o.check_every);
        auto sweep = [&](int it) {
            launch_csr_rows(nrows, nfl, B.ptr, B.col, B.RW, B.biasR, B.mu, B.x, B.lam, B.dlam, B.ds, s, Rb, full);
            launch_csr_cols(nv, B.cstart, B.cend, B.nz_out, B.rowidx, B.val, B.dlam, nullptr, B.mdiag, B.x, 1, 0.0, 0.0,
                            0, B.ds, s);
            launch_check(B.ds, it, 0.0, nv, 0, s);  // res_last and the sweep count
        };
        auto poll = [&](int it, bool& stop) -> int {
            stop = false;
            if ((it + 1) % every == 0 && it + 1 < maxit) {
                cudaMemcpyAsync(&E.hs->done, &B.ds->done, 4, cudaMemcpyDeviceToHost, s);
                int r = E.cuda_check(cudaStreamSynchronize(s), "csr poll");
                if (r) return r;
                stop = E.hs->done != 0;
            }
            return CDX_OK;
        };
        if (o.nesterov || o.chebyshev) {
            // nesterov_loop / chebyshev_loop (projected_jacobi.cpp:379-449, 179-222) as in the engine
            const bool nes = o.nesterov != 0;
            launch_accel_init(B.st, s);
            if (!nes)
                launch_power_iteration(nv, 1, B.xy, B.xk, B.part, B.st, [&]() {
                    launch_csr_linear(nrows, nfl, nv, B.ptr, B.col, B.RW, Rb, full, B.cstart, B.cend, B.nz_out,
                                      B.rowidx, B.val, B.mdiag, B.xy, B.dlam, B.xk, s);
                }, s);
            launch_accel_copy(B.xk, B.x, nv, B.pk, B.lam, nrows, nullptr, s);
            launch_accel_copy(B.xk1, B.x, nv, B.pk1, B.lam, nrows, nullptr, s);
            launch_accel_copy(B.xy, B.x, nv, B.py, B.lam, nrows, nullptr, s);
            for (int it = 0; it < maxit; ++it) {
                if (nes)
                    launch_accel_copy(B.x, B.xy, nv, B.lam, B.py, nrows, B.ds, s);
                else
                    launch_accel_copy(B.x, B.xk1, nv, B.lam, B.pk1, nrows, B.ds, s);
                sweep(it);
                if (nes) {
                    launch_accel_copy(B.xk1, B.x, nv, B.pk1, B.lam, nrows, B.ds, s);
                    launch_accel_reduce(nv, ACC_VELRES, B.xk1, B.xy, nullptr, o.tol_rel, o.tol_abs, B.part, B.st,
                                        &B.st->sum_err, B.ds, s, 1);
                    launch_accel_reduce(nv, ACC_DOT, B.xy, B.xk1, B.xk, 0.0, 0.0, B.part, B.st, &B.st->sum_dot, B.ds,
                                        s, 1);
                    launch_nesterov_step(B.st, B.ds, nv, o.beta_threshold, o.restart_limit, B.xy, B.xk, B.xk1, nv,
                                         B.py, B.pk, B.pk1, nrows, o.residual_tol, s);
                } else {
                    launch_accel_reduce(nv, ACC_VELRES, B.x, B.xk1, nullptr, o.tol_rel, o.tol_abs, B.part, B.st,
                                        &B.st->sum_err, B.ds, s, 1);
                    launch_chebyshev_step(B.st, B.ds, nv, it, B.x, B.xk, B.xk1, nv, B.lam, B.pk, B.pk1, nrows,
                                          o.residual_tol, s);
                }
                bool stop;
                if ((st = poll(it, stop))) return st;
                if (stop) break;
            }
            launch_accel_copy(B.x, B.xk1, nv, B.lam, B.pk1, nrows, nullptr, s);
        } else if (o.anderson) {
            // anderson_loop (projected_jacobi.cpp:242-314) as in the engine, on the plain layout
            AndersonBufs& A = B.anderson;
            launch_anderson_begin_plain(nv, B.x, B.lam, A, s);
            for (int it = 0; it < maxit; ++it) {
                launch_anderson_scatter(nv, B.x, B.lam, A, B.ds, s);
                sweep(it);
                launch_anderson_mix(nv, B.x, B.lam, A, o.tol_rel, o.tol_abs, o.residual_tol, B.ds, s);
                bool stop;
                if ((st = poll(it, stop))) return st;
                if (stop) break;
            }
            launch_anderson_scatter(nv, B.x, B.lam, A, B.ds, s);
        } else {
            // standard_loop (projected_jacobi.cpp:371-377)
            const bool check_vel = !(o.tol_abs == 0.0 && o.tol_rel == 0.0);
            for (int it = 0; it < maxit; ++it) {
                launch_csr_rows(nrows, nfl, B.ptr, B.col, B.RW, B.biasR, B.mu, B.x, B.lam, B.dlam, B.ds, s, Rb, full);
                launch_csr_cols(nv, B.cstart, B.cend, B.nz_out, B.rowidx, B.val, B.dlam, nullptr, B.mdiag, B.x, 1,
                                o.tol_abs, o.tol_rel, check_vel && (it % 10 == 0), B.ds, s);
                launch_check(B.ds, it, o.residual_tol, nv, check_vel, s);
                bool stop;
                if ((st = poll(it, stop))) return st;
                if (stop) break;
            }
        }
        cudaMemcpyAsync(&iters, &B.ds->iters, 4, cudaMemcpyDeviceToHost, s);
    }
    if (nv) cudaMemcpyAsync(x_out, B.x, 8 * (size_t)nv, cudaMemcpyDeviceToHost, s);
    if (nrows) cudaMemcpyAsync(lambda_inout, B.lam, 8 * (size_t)nrows, cudaMemcpyDeviceToHost, s);
    if ((st = E.cuda_check(cudaStreamSynchronize(s), "csr solve"))) return st;
    if ((st = E.cuda_check(cudaGetLastError(), "csr launch"))) return st;
    if (iterations) *iterations = iters;
    return CDX_OK;
}

extern "C" int cdx_pj_solve_csr(cdx_ctx* ctx, int32_t nrows, int32_t nv, int32_t nfl, const int32_t* row_ptr,
                                const int32_t* col, const double* val, const double* contact_bias, const double* mu,
                                const double* restitution, const double* minv, const double* mdiag, const double* v,
                                const double* f_ext, const double* f_gyro, double dt, double alpha, int32_t max_iter,
                                double tol_abs, double tol_rel, double* lambda_inout, double* x_out,
                                int32_t* iterations) {
    CsrOpts o;
    o.alpha = alpha;
    o.max_iter = max_iter;
    o.tol_abs = tol_abs;
    o.tol_rel = tol_rel;
    if (ctx) o.check_every = ctx->eng.cfg.gpu_check_every;
    return csr_solve(ctx, o, nrows, nv, nfl, row_ptr, col, val, contact_bias, mu, restitution, minv, mdiag, v, f_ext,
                     f_gyro, dt, lambda_inout, x_out, iterations);
}

extern "C" int cdx_pj_solve_csr_cfg(cdx_ctx* ctx, const cdx_config* cfg, int32_t nrows, int32_t nv, int32_t nfl,
                                    const int32_t* row_ptr, const int32_t* col, const double* val,
                                    const double* contact_bias, const double* mu, const double* restitution,
                                    const double* minv, const double* mdiag, const double* v, const double* f_ext,
                                    const double* f_gyro, double dt, double* lambda_inout, double* x_out,
                                    int32_t* iterations) {
    if (!ctx || !cfg) return CDX_ERR_ARG;
    CsrOpts o;
    o.alpha = cfg->pj_alpha;
    o.max_iter = cfg->pj_max_iterations;
    o.tol_abs = cfg->pj_tol_abs;
    o.tol_rel = cfg->pj_tol_rel;
    o.residual_tol = cfg->gpu_residual_tol;
    o.check_every = cfg->gpu_check_every;
    o.nesterov = cfg->pj_nesterov;
    o.beta_threshold = cfg->pj_nesterov_beta_threshold;
    o.restart_limit = cfg->pj_nesterov_restart_limit;
    o.chebyshev = cfg->pj_chebyshev;
    o.anderson = cfg->pj_anderson;
    o.anderson_m = cfg->pj_anderson_m;
    o.block = cfg->pj_rdiag_true_delassus;
    return csr_solve(ctx, o, nrows, nv, nfl, row_ptr, col, val, contact_bias, mu, restitution, minv, mdiag, v, f_ext,
                     f_gyro, dt, lambda_inout, x_out, iterations);
}
