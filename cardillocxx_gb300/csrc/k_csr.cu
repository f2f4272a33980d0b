// Solver-level drop-in: projected Jacobi on a general sparse contact Jacobian W given as CSR,
// the exact replacement of ProjectedJacobiSolver::solve (projected_jacobi.cpp:451-500) with
// S = diag(M) (pj_assembler.cpp:127-182). FP64, compiled with --fmad=false, bit-identical to the
// CPU oracle: RW x as a row dot in CSR column order, W^T y as a per-column gather in row order
// (the order of Eigen's column-major sparse * dense kernel), no atomics.
#include "cdx_internal.h"
#include "fp64_math.cuh"

namespace cdx {
using namespace f64;

namespace {
constexpr int NT = 256;
inline int nblk(int64_t n, int nt = NT) { return (int)((n + nt - 1) / nt); }

__global__ void k_csr_rhs(int nv, const double* mdiag, const double* v, const double* fext, const double* fgyro,
                          double dt, double* rhs) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nv) return;
    rhs[j] = (mdiag[j] * v[j] + dt * fext[j]) + dt * fgyro[j];
}

__global__ void k_csr_rowidx(int nrows, const int32_t* ptr, int32_t* rowidx, uint32_t* colkey, uint32_t* nzid,
                             const int32_t* col) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrows) return;
    for (int k = ptr[r]; k < ptr[r + 1]; ++k) {
        rowidx[k] = r;
        colkey[k] = (uint32_t)col[k];
        nzid[k] = (uint32_t)k;
    }
}

// build_workspace + rdiag_sparse per row; with block, W and the bias stay unscaled
// (pj.rdiag_true_delassus, projected_jacobi.cpp:341-343)
__global__ void k_csr_setup(int nrows, const int32_t* ptr, const int32_t* col, const double* val, const double* cb,
                            const double* e, const double* minv, const double* v, double alpha, double* RW,
                            double* biasR, int block) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrows) return;
    double vp = 0.0, D = 0.0;
    for (int k = ptr[r]; k < ptr[r + 1]; ++k) vp = vp + val[k] * v[col[k]];
    vp = vp + cb[r];
    const double bias = cb[r] + e[r] * vp;
    for (int k = ptr[r]; k < ptr[r + 1]; ++k) D = D + (val[k] * val[k]) * minv[col[k]];
    if (block) {
        for (int k = ptr[r]; k < ptr[r + 1]; ++k) RW[k] = val[k];
        biasR[r] = bias;
        return;
    }
    const double R = (D > 0.0) ? (alpha / D) : 0.0;
    for (int k = ptr[r]; k < ptr[r + 1]; ++k) RW[k] = R * val[k];
    biasR[r] = R * bias;
}

// buildBlockPreconditioner (projected_jacobi.cpp:81-98): per unit (a frictionless row, or the three
// rows of a frictional contact) its block of W M^-1 W^T / alpha into Rb (9 a unit, row-major;
// a frictionless unit uses Rb[0]). The rows of one contact share their columns, so
// D_ab = sum_q (W_aq Minv_q) W_bq over them. A block that is not diagonal sets *full.
__global__ void k_csr_blocks(int nrows, int nfl, const int32_t* ptr, const int32_t* col, const double* val,
                             const double* minv, double alpha, double* Rb, int32_t* full) {
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    const int nunits = nfl + (nrows - nfl) / 3;
    if (u >= nunits) return;
    const double inv_alpha = (alpha > 0.0) ? (1.0 / alpha) : 0.0;
    double* B = Rb + 9 * (size_t)u;
    if (u < nfl) {
        double d = 0.0;
        for (int k = ptr[u]; k < ptr[u + 1]; ++k) d = d + val[k] * val[k] * minv[col[k]];
        B[0] = d * inv_alpha;
        return;
    }
    const int r0 = nfl + 3 * (u - nfl);
    const int len = ptr[r0 + 1] - ptr[r0];
    double D[9];
    for (int a = 0; a < 3; ++a)
        for (int c = 0; c < 3; ++c) {
            const int pa = ptr[r0 + a], pc = ptr[r0 + c];
            double d = 0.0;
            for (int q = 0; q < len; ++q) d = d + (val[pa + q] * minv[col[pa + q]]) * val[pc + q];
            D[3 * a + c] = d * inv_alpha;
        }
    for (int k = 0; k < 9; ++k) B[k] = D[k];
    if (!block_is_diagonal3(D)) *full = 1;
}

// BlockDiagonal::calculateInverse: per diagonal entry when every block is diagonal, else the SPD
// inverse of every block (1 x 1 blocks included)
__global__ void k_csr_block_inv(int nrows, int nfl, double* Rb, const int32_t* full) {
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    const int nunits = nfl + (nrows - nfl) / 3;
    if (u >= nunits) return;
    const bool f = *full != 0;
    double* B = Rb + 9 * (size_t)u;
    if (u < nfl) {
        const double d = B[0];
        double x;
        if (f) spd_inverse_dev(&d, 1, &x);
        else x = 1.0 / d;
        B[0] = x;
        return;
    }
    double D[9], X[9];
    for (int k = 0; k < 9; ++k) D[k] = B[k];
    if (f) {
        spd_inverse_dev(D, 3, X);
    } else {
        for (int k = 0; k < 9; ++k) X[k] = 0.0;
        for (int j = 0; j < 3; ++j) X[4 * j] = 1.0 / D[4 * j];
    }
    for (int k = 0; k < 9; ++k) B[k] = X[k];
}

// BlockDiagonal::applyTo (misc/block_diagonal.hpp:107-126) on one unit's rows g
__device__ __forceinline__ void csr_block_apply(const double* B, bool fr, bool full, double* g) {
    if (!fr) {
        g[0] = full ? B[0] * g[0] : g[0] * B[0];
        return;
    }
    if (!full) {
        for (int j = 0; j < 3; ++j) g[j] = g[j] * B[4 * j];
        return;
    }
    double s[3];
    for (int j = 0; j < 3; ++j) s[j] = B[3 * j] * g[0] + B[3 * j + 1] * g[1] + B[3 * j + 2] * g[2];
    for (int j = 0; j < 3; ++j) g[j] = s[j];
}

// linear part of the sweep map for the power iteration: delta = R_block (RW v) per unit
__global__ void k_csr_linear_rows(int nrows, int nfl, const int32_t* ptr, const int32_t* col, const double* RW,
                                  const double* Rb, const int32_t* full, const double* v, double* delta) {
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    const int nunits = nfl + (nrows - nfl) / 3;
    if (u >= nunits) return;
    const bool fr = u >= nfl;
    const int r0 = fr ? nfl + 3 * (u - nfl) : u;
    const int nr = fr ? 3 : 1;
    double g[3];
    for (int q = 0; q < nr; ++q) {
        double t = 0.0;
        for (int k = ptr[r0 + q]; k < ptr[r0 + q + 1]; ++k) t = t + RW[k] * v[col[k]];
        g[q] = t;
    }
    if (Rb) csr_block_apply(Rb + 9 * (size_t)u, fr, *full != 0, g);
    for (int q = 0; q < nr; ++q) delta[r0 + q] = g[q];
}
// Mv_j = v_j - (sum over column j's entries, row order, of W delta) / M_j
__global__ void k_csr_linear_cols(int nv, const int32_t* cstart, const int32_t* cend, const uint32_t* nz_sorted,
                                  const int32_t* rowidx, const double* val, const double* delta, const double* mdiag,
                                  const double* v, double* Mv) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nv) return;
    double acc = 0.0;
    for (int p = cstart[j]; p < cend[j]; ++p) {
        const int k = (int)nz_sorted[p];
        acc = acc + val[k] * delta[rowidx[k]];
    }
    Mv[j] = v[j] - acc / mdiag[j];
}

// dst_j (+)= sum over column j's entries (row order) of val * y[row]; then x_j = (dst or x + dst)/M
__global__ void k_csr_cols(int nv, const int32_t* cstart, const int32_t* cend, const uint32_t* nz_sorted,
                           const int32_t* rowidx, const double* val, const double* y, const double* base,
                           const double* mdiag, double* x, int mode, double tol_abs, double tol_rel, int want_velres,
                           DevScalars* ds) {
    if (mode == 1 && *(volatile int32_t*)&ds->done) return;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    double part = 0.0;
    if (j < nv) {
        double acc = mode == 0 ? base[j] : 0.0;
        for (int p = cstart[j]; p < cend[j]; ++p) {
            const int k = (int)nz_sorted[p];
            acc = acc + val[k] * y[rowidx[k]];
        }
        if (mode == 0) {
            x[j] = acc / mdiag[j];
        } else {
            const double xo = x[j];
            const double xn = xo + acc / mdiag[j];
            x[j] = xn;
            if (want_velres) {
                const double q = smax(fabs(xn), fabs(xo)) * tol_rel + tol_abs;
                const double dd = (xn - xo) / q;
                part = dd * dd;
            }
        }
    }
    if (mode == 1 && want_velres) {
        __shared__ double sh[32];
        for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
        if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = part;
        __syncthreads();
        if (threadIdx.x < 32) {
            part = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
            for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
            if (threadIdx.x == 0) atomicAdd(&ds->velres, part);
        }
    }
}

// one thread per contact unit: a frictionless row, or a 3-row frictional block
__global__ void k_csr_rows(int nrows, int nfl, const int32_t* ptr, const int32_t* col, const double* RW,
                           const double* biasR, const double* mu, const double* x, double* lam, double* dlam,
                           DevScalars* ds, const double* Rb, const int32_t* full, int dry) {
    if (!dry && *(volatile int32_t*)&ds->done) return;
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    const int nunits = nfl + (nrows - nfl) / 3;
    double maxd = 0.0, maxl = 0.0;
    if (u < nunits) {
        const bool fr = u >= nfl;
        const int r0 = fr ? nfl + 3 * (u - nfl) : u;
        const int nr = fr ? 3 : 1;
        double lo[3], ln[3], g[3];
        for (int q = 0; q < nr; ++q) {
            const int r = r0 + q;
            double t = 0.0;
            for (int k = ptr[r]; k < ptr[r + 1]; ++k) t = t + RW[k] * x[col[k]];
            g[q] = t + biasR[r];
            lo[q] = lam[r];
        }
        if (Rb) csr_block_apply(Rb + 9 * (size_t)u, fr, *full != 0, g);
        for (int q = 0; q < nr; ++q) ln[q] = lo[q] - g[q];
        ln[0] = smax(ln[0], 0.0);
        if (fr) {
            const double t1 = ln[1], t2 = ln[2];
            const double tn2 = t1 * t1 + t2 * t2;
            if (tn2 > 0) {
                const double s = smin(1.0, (mu[r0] * ln[0]) / sqrt(tn2));
                ln[1] = s * t1;
                ln[2] = s * t2;
            }
        }
        double s2 = 0.0;
        for (int q = 0; q < nr; ++q) {
            const double d = ln[q] - lo[q];
            s2 = s2 + d * d;
            maxl = smax(maxl, fabs(lo[q]));
            if (!dry) {
                lam[r0 + q] = ln[q];
                dlam[r0 + q] = d;
            }
        }
        maxd = s2;  // squared: the root of the block maximum equals the maximum of the roots
    }
    __shared__ double sh[2][32];
    for (int o = 16; o > 0; o >>= 1) {
        maxd = fmax(maxd, __shfl_xor_sync(0xffffffffu, maxd, o));
        maxl = fmax(maxl, __shfl_xor_sync(0xffffffffu, maxl, o));
    }
    if ((threadIdx.x & 31) == 0) {
        sh[0][threadIdx.x >> 5] = maxd;
        sh[1][threadIdx.x >> 5] = maxl;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        maxd = threadIdx.x < (blockDim.x >> 5) ? sh[0][threadIdx.x] : 0.0;
        maxl = threadIdx.x < (blockDim.x >> 5) ? sh[1][threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) {
            maxd = fmax(maxd, __shfl_xor_sync(0xffffffffu, maxd, o));
            maxl = fmax(maxl, __shfl_xor_sync(0xffffffffu, maxl, o));
        }
        if (threadIdx.x == 0) {
            atomicMax(&ds->maxd, (unsigned long long)__double_as_longlong(sqrt(maxd)));
            atomicMax(&ds->maxl, (unsigned long long)__double_as_longlong(maxl));
        }
    }
}
}  // namespace

void launch_csr_rhs(int nv, const double* mdiag, const double* v, const double* fext, const double* fgyro, double dt,
                    double* rhs, cudaStream_t s) {
    if (nv > 0) k_csr_rhs<<<nblk(nv), NT, 0, s>>>(nv, mdiag, v, fext, fgyro, dt, rhs);
}
void launch_csr_rowidx(int nrows, const int32_t* ptr, int32_t* rowidx, uint32_t* colkey, uint32_t* nzid,
                       const int32_t* col, cudaStream_t s) {
    if (nrows > 0) k_csr_rowidx<<<nblk(nrows), NT, 0, s>>>(nrows, ptr, rowidx, colkey, nzid, col);
}
void launch_csr_setup(int nrows, const int32_t* ptr, const int32_t* col, const double* val, const double* cb,
                      const double* e, const double* minv, const double* v, double alpha, double* RW, double* biasR,
                      cudaStream_t s, int block) {
    if (nrows > 0)
        k_csr_setup<<<nblk(nrows), NT, 0, s>>>(nrows, ptr, col, val, cb, e, minv, v, alpha, RW, biasR, block);
}
void launch_csr_blocks(int nrows, int nfl, const int32_t* ptr, const int32_t* col, const double* val,
                       const double* minv, double alpha, double* Rb, int32_t* full, cudaStream_t s) {
    const int nunits = nfl + (nrows - nfl) / 3;
    if (nunits <= 0) return;
    cudaMemsetAsync(full, 0, sizeof(int32_t), s);
    k_csr_blocks<<<nblk(nunits), NT, 0, s>>>(nrows, nfl, ptr, col, val, minv, alpha, Rb, full);
    k_csr_block_inv<<<nblk(nunits), NT, 0, s>>>(nrows, nfl, Rb, full);
}
void launch_csr_linear(int nrows, int nfl, int nv, const int32_t* ptr, const int32_t* col, const double* RW,
                       const double* Rb, const int32_t* full, const int32_t* cstart, const int32_t* cend,
                       const uint32_t* nz_sorted, const int32_t* rowidx, const double* val, const double* mdiag,
                       const double* v, double* delta, double* Mv, cudaStream_t s) {
    const int nunits = nfl + (nrows - nfl) / 3;
    if (nunits > 0) k_csr_linear_rows<<<nblk(nunits), NT, 0, s>>>(nrows, nfl, ptr, col, RW, Rb, full, v, delta);
    if (nv > 0)
        k_csr_linear_cols<<<nblk(nv), NT, 0, s>>>(nv, cstart, cend, nz_sorted, rowidx, val, delta, mdiag, v, Mv);
}
void launch_csr_cols(int nv, const int32_t* cstart, const int32_t* cend, const uint32_t* nz_sorted,
                     const int32_t* rowidx, const double* val, const double* y, const double* base,
                     const double* mdiag, double* x, int mode, double tol_abs, double tol_rel, int want_velres,
                     DevScalars* ds, cudaStream_t s) {
    if (nv > 0)
        k_csr_cols<<<nblk(nv), NT, 0, s>>>(nv, cstart, cend, nz_sorted, rowidx, val, y, base, mdiag, x, mode, tol_abs,
                                           tol_rel, want_velres, ds);
}
void launch_csr_rows(int nrows, int nfl, const int32_t* ptr, const int32_t* col, const double* RW,
                     const double* biasR, const double* mu, const double* x, double* lam, double* dlam,
                     DevScalars* ds, cudaStream_t s, const double* Rb, const int32_t* full, int dry) {
    const int nunits = nfl + (nrows - nfl) / 3;
    if (nunits > 0)
        k_csr_rows<<<nblk(nunits), NT, 0, s>>>(nrows, nfl, ptr, col, RW, biasR, mu, x, lam, dlam, ds, Rb, full, dry);
}

}  // namespace cdx
