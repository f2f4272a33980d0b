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

extern "C" int cdx_pj_solve_csr(cdx_ctx* ctx, int32_t nrows, int32_t nv, int32_t nfl, const int32_t* row_ptr,
                                const int32_t* col, const double* val, const double* contact_bias, const double* mu,
                                const double* restitution, const double* minv, const double* mdiag, const double* v,
                                const double* f_ext, const double* f_gyro, double dt, double alpha, int32_t max_iter,
                                double tol_abs, double tol_rel, double* lambda_inout, double* x_out,
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
    CsrBuffers& B = buffers(E);
    int st;
    if ((st = grow(E, B, nnz, nrows, nv))) return st;
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
        launch_csr_setup(nrows, B.ptr, B.col, B.val, B.cb, B.e, B.minv, B.v, alpha, B.RW, B.biasR, s);
        launch_csr_cols(nv, B.cstart, B.cend, B.nz_out, B.rowidx, B.val, B.lam, B.rhs, B.mdiag, B.x, 0, 0, 0, 0,
                        B.ds, s);
        cudaMemsetAsync(B.ds, 0, sizeof(DevScalars), s);
        const bool check_vel = !(tol_abs == 0.0 && tol_rel == 0.0);
        const int maxit = std::max(1, max_iter);
        const int every = std::max(1, E.cfg.gpu_check_every);
        for (int it = 0; it < maxit; ++it) {
            launch_csr_rows(nrows, nfl, B.ptr, B.col, B.RW, B.biasR, B.mu, B.x, B.lam, B.dlam, B.ds, s);
            launch_csr_cols(nv, B.cstart, B.cend, B.nz_out, B.rowidx, B.val, B.dlam, nullptr, B.mdiag, B.x, 1,
                            tol_abs, tol_rel, check_vel && (it % 10 == 0), B.ds, s);
            launch_check(B.ds, it, 0.0, nv, check_vel, s);
            if ((it + 1) % every == 0 && it + 1 < maxit) {
                cudaMemcpyAsync(&E.hs->done, &B.ds->done, 4, cudaMemcpyDeviceToHost, s);
                if ((st = E.cuda_check(cudaStreamSynchronize(s), "csr poll"))) return st;
                if (E.hs->done) break;
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
