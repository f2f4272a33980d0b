// The condensed solver's colored Gauss-Seidel sweep in FP64 (solver.type=condensed,
// condensed.sweep_mode=colored), for the plain FP64 method; compiled without FMA contraction so
// every result is rounded as written and matches the CPU oracle bit for bit.
//
// CondensedSolver::solve (src/physics/solver/condensed_solver.cpp:443-760) for sphere contacts:
// one block per contact in contact order with the contact's W rows split by side
// (Ja = -[d_r, r_A x d_r] on a dynamic body A, Jb = +[d_r, r_B x d_r] on body B;
// condensed_assembler.cpp:203-262), the diagonal inverse 1/G_ii of the block's Delassus diagonal
// (updateCompliance, :308-312), internal normal impulses <= 0 and u = u_free - u_corr. The blocks
// are colored greedily so that no two blocks of a color share a dynamic body (buildBlockAdjacency
// and colorGreedyWelshPowell, condensed_solver.cpp:175-199, misc/graph_coloring.cpp:8-40); a sweep
// runs the colors in order and each color's blocks in parallel (coloredSweep, :205-226).
//
// The coloring runs on the GPU as Jones-Plassmann rounds: a block is colored once its priority
// (degree, then lower index) exceeds that of every uncolored neighbour, with the smallest color no
// colored neighbour uses. When a block is colored, exactly its higher-priority neighbours are
// colored already, so every block gets the color the sequential greedy pass in priority order gives
// it: the same coloring as Welsh-Powell with equal degrees in block order.
#include <cstdint>

#include "cdx_internal.h"
#include "fp64_math.cuh"

namespace cdx {
namespace {

constexpr int NT = 256;
inline int nblk(int64_t n, int nt = NT) { return (int)((n + nt - 1) / nt); }
constexpr int RED_CHUNK = 256;  // chunk size of the fixed three-level reduction order (shared with the oracle)
using f64::cross3;
using f64::smin;

// one side's Jacobian row q of contact c: sign * [d_q (world), c_q (body-frame lever product)]
__device__ __forceinline__ void jac_row(const Contacts& C, int c, int q, bool sideB, double* J) {
    const int64_t cap = C.cap;
    const double* cc = sideB ? C.cB : C.cA;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const double d = C.dir[(3 * q + k) * cap + c];
        J[k] = sideB ? d : -d;
        const double l = cc[(3 * q + k) * cap + c];
        J[3 + k] = sideB ? l : -l;
    }
}

// body velocities are field-major: component k of body i at k * N + i
__device__ __forceinline__ double row_dot(const double* J, const double* u, int N, int i) {
    double t = J[0] * u[i];
    for (int k = 1; k < 6; ++k) t = t + J[k] * u[(size_t)k * N + i];
    return t;
}

__device__ __forceinline__ double minv_of(const Scene& sc, int i, int k) {
    return k < 3 ? sc.bf(BF_MINVL)[i] : sc.bf(BF_MINVA)[i];
}

}  // namespace
}  // namespace cdx
#include "cond_block.cuh"
namespace cdx {
namespace {

// u_free = v_n + M^-1 (dt f_ext) [+ M^-1 (dt f_gyro)] (CondensedAssembler::ufree, condensed_assembler.cpp:348-356;
// PgsAssembler::ufree, pgs_assembler.cpp:96-103, is the same)
__global__ void k_cond_ufree(Scene sc, double dt, double g0, double g1, double g2, int implicit_gyro, double* uf) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sc.N) return;
    const int N = sc.N;
    const double w[3] = {sc.bf(BF_WX)[i], sc.bf(BF_WY)[i], sc.bf(BF_WZ)[i]};
    const double I = sc.bf(BF_INERTIA)[i], m = sc.bf(BF_MASS)[i];
    const double Iw[3] = {I * w[0], I * w[1], I * w[2]};
    double cg[3];
    cross3(w, Iw, cg);
    const double g[3] = {g0, g1, g2};
    const double vn[6] = {sc.bf(BF_VX)[i], sc.bf(BF_VY)[i], sc.bf(BF_VZ)[i], w[0], w[1], w[2]};
    for (int k = 0; k < 6; ++k) {
        const double mi = minv_of(sc, i, k);
        const double fext = k < 3 ? m * g[k] : 0.0;
        double u = vn[k] + mi * (dt * fext);
        if (!implicit_gyro) u = u + mi * (dt * (k < 3 ? 0.0 : -cg[k - 3]));
        uf[(size_t)k * N + i] = u;
    }
}

// per contact: 1/G_ii, rhs_i = J u_free + contact velocity, the internal impulses from the warm
// start (normal sign inverted, warmstart.hpp:26-39), and the block's degree in the shared-body graph
__global__ void k_cond_setup(Scene sc, Contacts C, int gen, int nc, const double* uf, int warmstart, CondBufs B,
                             Incidence inc) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    const int64_t cap = C.cap;
    const int N = sc.N;
    const int a = C.a[c], b = C.b[c];
    const int dim = (C.flags[c] & CF_FRICTIONAL) ? 3 : 1;
    for (int q = 0; q < dim; ++q) {
        double Ja[6], Jb[6];
        jac_row(C, c, q, false, Ja);
        jac_row(C, c, q, true, Jb);
        double ga = 0.0;
        if (a >= 0) {
            ga = (Ja[0] * minv_of(sc, a, 0)) * Ja[0];
            for (int k = 1; k < 6; ++k) ga = ga + (Ja[k] * minv_of(sc, a, k)) * Ja[k];
        }
        double gb = (Jb[0] * minv_of(sc, b, 0)) * Jb[0];
        for (int k = 1; k < 6; ++k) gb = gb + (Jb[k] * minv_of(sc, b, k)) * Jb[k];
        const double G = (0.0 + ga) + gb;
        B.ginv[q * cap + c] = G > 0 ? 1.0 / G : 0.0;
        double ut = 0.0;
        if (a >= 0) ut = ut + row_dot(Ja, uf, N, a);
        ut = ut + row_dot(Jb, uf, N, b);
        B.rhs[q * cap + c] = ut + C.cb[q * cap + c];
    }
    const double* l0 = C.lam[gen];
    B.lam[c] = warmstart ? -l0[c] : 0.0;
    B.lam[cap + c] = (warmstart && dim == 3) ? l0[cap + c] : 0.0;
    B.lam[2 * cap + c] = (warmstart && dim == 3) ? l0[2 * cap + c] : 0.0;
    int deg = inc.end[b] - inc.start[b] - 1;
    if (a >= 0) deg += inc.end[a] - inc.start[a] - 1;
    B.deg[c] = deg;
    B.col[c] = -1;
}

// u_corr_i = sum over the body's blocks in block order of M^-1 J^T lambda (the initial u_corr of
// CondensedSolver::solve, condensed_solver.cpp:487-494); the incidence is in contact order
__global__ void k_cond_ucorr_init(Scene sc, Contacts C, CondBufs B, Incidence inc, double* u) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sc.N) return;
    const int N = sc.N;
    const int64_t cap = C.cap;
    double acc[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int p = inc.start[i]; p < inc.end[i]; ++p) {
        const uint32_t code = inc.val_out[p];
        const int c = (int)(code >> 1);
        const bool sideB = (code & 1u) != 0;
        const int dim = (C.flags[c] & CF_FRICTIONAL) ? 3 : 1;
        double J[3][6];
        for (int q = 0; q < dim; ++q) jac_row(C, c, q, sideB, J[q]);
        for (int k = 0; k < 6; ++k) {
            double t = J[0][k] * B.lam[c];
            for (int q = 1; q < dim; ++q) t = t + J[q][k] * B.lam[q * cap + c];
            acc[k] = acc[k] + minv_of(sc, i, k) * t;
        }
    }
    for (int k = 0; k < 6; ++k) u[(size_t)k * N + i] = acc[k];
}

// block x outranks block y: higher degree, then lower index
__device__ __forceinline__ bool outranks(int dx, int x, int dy, int y) { return dx > dy || (dx == dy && x < y); }

// One Jones-Plassmann round: an uncolored block whose priority exceeds every uncolored neighbour's
// takes the smallest color none of its (higher-priority, already colored) neighbours has. Reads
// the colors of the previous round (col_in) and writes this round's (col_out).
__global__ void k_cond_color_round(Contacts C, int nc, CondBufs B, Incidence inc, const int32_t* col_in,
                                   int32_t* col_out, int32_t* uncolored, int32_t* too_many) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    const int mine = col_in[c];
    col_out[c] = mine;
    if (mine >= 0) return;
    const int a = C.a[c], b = C.b[c];
    const int dc = B.deg[c];
    unsigned long long used[CDX_COND_MAX_COLORS / 64] = {};
    bool ready = true;
    for (int side = 0; side < 2 && ready; ++side) {
        const int body = side == 0 ? a : b;
        if (body < 0) continue;
        for (int p = inc.start[body]; p < inc.end[body]; ++p) {
            const int d = (int)(inc.val_out[p] >> 1);
            if (d == c) continue;
            const int cd = col_in[d];
            if (cd < 0) {
                if (outranks(B.deg[d], d, dc, c)) {
                    ready = false;
                    break;
                }
            } else if (cd < CDX_COND_MAX_COLORS) {
                used[cd >> 6] |= 1ull << (cd & 63);
            }
        }
    }
    if (!ready) {
        atomicAdd(uncolored, 1);
        return;
    }
    int chosen = 0;
    while (chosen < CDX_COND_MAX_COLORS && ((used[chosen >> 6] >> (chosen & 63)) & 1ull)) ++chosen;
    if (chosen >= CDX_COND_MAX_COLORS) {
        atomicExch(too_many, 1);
        chosen = CDX_COND_MAX_COLORS - 1;
    }
    col_out[c] = chosen;
}

// One block of the colored sweep (coloredSweep's body, condensed_solver.cpp:212-224, with
// blockResidual :62-69, computeBlockUpdate :139-158 and projectBlock :41-52). No two blocks of a
// color share a dynamic body, so the updates of u_corr below never overlap within a launch.
__global__ void k_cond_sweep_color(Scene sc, Contacts C, CondBufs B, const uint32_t* blocks, int n, double relax,
                                   double alpha, double* u, const DevScalars* ds) {
    if (*(volatile const int32_t*)&ds->done) return;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    double d[3];
    cond_block<false, true>(sc, C, B, (int)blocks[t], relax, alpha, u, d);
}

// Jacobi sweep, pass 1 (jacobiSweep, condensed_solver.cpp:285-296): every block against the
// previous sweep's u_corr (untouched in this pass); the increments go to dl
__global__ void k_cond_jacobi_blocks(Scene sc, Contacts C, CondBufs B, int nc, double relax, double alpha,
                                     const double* u, const DevScalars* ds) {
    if (*(volatile const int32_t*)&ds->done) return;
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    double d[3] = {0.0, 0.0, 0.0};
    cond_block<false, false>(sc, C, B, c, relax, alpha, const_cast<double*>(u), d);
    const int64_t cap = C.cap;
    for (int q = 0; q < 3; ++q) B.dl[q * cap + c] = d[q];
}

// pass 2 (:302-316): each body gathers J^T dl from its blocks in block order, u += M^-1 acc
__global__ void k_cond_jacobi_bodies(Scene sc, Contacts C, CondBufs B, Incidence inc, double* u,
                                     const DevScalars* ds) {
    if (*(volatile const int32_t*)&ds->done) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sc.N) return;
    if (inc.end[i] <= inc.start[i]) return;
    const int N = sc.N;
    const int64_t cap = C.cap;
    double acc[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int p = inc.start[i]; p < inc.end[i]; ++p) {
        const uint32_t code = inc.val_out[p];
        const int c = (int)(code >> 1);
        const bool sideB = (code & 1u) != 0;
        const int dim = (C.flags[c] & CF_FRICTIONAL) ? 3 : 1;
        double J[3][6];
        for (int q = 0; q < dim; ++q) jac_row(C, c, q, sideB, J[q]);
        for (int k = 0; k < 6; ++k) {
            double t = J[0][k] * B.dl[c];
            for (int q = 1; q < dim; ++q) t = t + J[q][k] * B.dl[q * cap + c];
            acc[k] = acc[k] + t;
        }
    }
    for (int k = 0; k < 6; ++k) {
        const size_t j = (size_t)k * N + i;
        u[j] = u[j] + minv_of(sc, i, k) * acc[k];
    }
}

// residualNorm (condensed_solver.cpp:500-506) over the stacked velocity vector (entry 6 i + k),
// in chunks of RED_CHUNK entries, each left to right, then the chunk sums left to right
__global__ void k_cond_res_partials(int N, const double* uf, const double* up, const double* uc, double tol_rel,
                                    double tol_abs, double* part, const DevScalars* ds) {
    if (*(volatile const int32_t*)&ds->done) return;
    const int nv = 6 * N;
    const int nch = (nv + RED_CHUNK - 1) / RED_CHUNK;
    const int ch = blockIdx.x * blockDim.x + threadIdx.x;
    if (ch >= nch) return;
    const int j0 = ch * RED_CHUNK, j1 = min(nv, j0 + RED_CHUNK);
    double s = 0.0;
    for (int j = j0; j < j1; ++j) {
        const size_t e = (size_t)(j % 6) * N + j / 6;
        const double diff = uc[e] - up[e];
        const double v0 = uf[e] - up[e], v1 = uf[e] - uc[e];
        const double q = f64::smax(fabs(v0), fabs(v1)) * tol_rel + tol_abs;
        const double t = diff / q;
        s = s + t * t;
    }
    part[ch] = s;
}

// the stop test after sweep `iter`: err = sqrt(1/nV) sqrt(sum); not finite: the solve diverged
// (checkResidual throws, :507-513); err < 1: converged. The chunk sums are added in groups of
// RED_GROUP (a thread a group), then the group sums in order (one block).
constexpr int RED_GROUP = 64;  // the fixed three-level order (shared with the oracle)
__global__ void k_cond_check(int N, const double* part, int nch, int iter, DevScalars* ds, int32_t* diverged,
                             double* err_out) {
    if (*(volatile const int32_t*)&ds->done) return;
    __shared__ double gs[128];
    const int ngroups = (nch + RED_GROUP - 1) / RED_GROUP;
    double tot = 0.0;
    for (int g0 = 0; g0 < ngroups; g0 += 128) {
        const int g = g0 + (int)threadIdx.x;
        if (g < ngroups) {
            double s = 0.0;
            const int c1 = min(nch, (g + 1) * RED_GROUP);
            for (int c = g * RED_GROUP; c < c1; ++c) s = s + part[c];
            gs[threadIdx.x] = s;
        }
        __syncthreads();
        if (threadIdx.x == 0)
            for (int k = 0; k < 128 && g0 + k < ngroups; ++k) tot = tot + gs[k];
        __syncthreads();
    }
    if (threadIdx.x != 0) return;
    const double err = 1.0 / sqrt((double)(6 * N)) * sqrt(tot);
    ds->iters = iter + 1;
    ds->res_last = err;
    *err_out = err;
    if (!isfinite(err)) {
        *diverged = 1;
        ds->done = 1;
    } else if (err < 1.0) {
        ds->done = 1;
    }
}

__global__ void k_cond_copy(int n, const double* src, double* dst, const DevScalars* ds) {
    if (*(volatile const int32_t*)&ds->done) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = src[i];
}

// x = u_free - u_corr; the impulses back in the stored convention (normal sign inverted,
// warmstart.hpp:41-56) and, for the complementarity residual, in the projected Jacobi convention
// (the applied impulse is minus the internal one)
__global__ void k_cond_final_body(int N, const double* uf, const double* u, double* x) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 6 * N) return;
    x[i] = uf[i] - u[i];
}
__global__ void k_cond_lambda_out(Contacts C, int gen, int nc, CondBufs B, int pj_convention) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    const int64_t cap = C.cap;
    const bool fr = (C.flags[c] & CF_FRICTIONAL) != 0;
    double* l = C.lam[gen];
    l[c] = -B.lam[c];
    l[cap + c] = fr ? (pj_convention ? -B.lam[cap + c] : B.lam[cap + c]) : 0.0;
    l[2 * cap + c] = fr ? (pj_convention ? -B.lam[2 * cap + c] : B.lam[2 * cap + c]) : 0.0;
}

__global__ void k_cond_sort_keys(int nc, const int32_t* col, uint32_t* k, uint32_t* v) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    k[c] = (uint32_t)col[c];
    v[c] = (uint32_t)c;
}

}  // namespace

void launch_cond_sort_keys(int nc, const int32_t* col, CondBufs& B, cudaStream_t s) {
    if (nc > 0) k_cond_sort_keys<<<nblk(nc), NT, 0, s>>>(nc, col, B.kin, B.vin);
}
void launch_cond_setup(const Scene& sc, Contacts& C, int gen, int nc, double dt, const double* g, int implicit_gyro,
                       int warmstart, CondBufs& B, const Incidence& inc, cudaStream_t s) {
    if (sc.N > 0) k_cond_ufree<<<nblk(sc.N), NT, 0, s>>>(sc, dt, g[0], g[1], g[2], implicit_gyro, B.uf);
    if (nc > 0) k_cond_setup<<<nblk(nc), NT, 0, s>>>(sc, C, gen, nc, B.uf, warmstart, B, inc);
    if (sc.N > 0) k_cond_ucorr_init<<<nblk(sc.N), NT, 0, s>>>(sc, C, B, inc, B.u);
}
void launch_cond_ufree(const Scene& sc, double dt, const double* g, int implicit_gyro, CondBufs& B, cudaStream_t s) {
    if (sc.N > 0) k_cond_ufree<<<nblk(sc.N), NT, 0, s>>>(sc, dt, g[0], g[1], g[2], implicit_gyro, B.uf);
}
void launch_cond_color_round(const Contacts& C, int nc, const CondBufs& B, const Incidence& inc,
                             const int32_t* col_in, int32_t* col_out, int32_t* uncolored, int32_t* too_many,
                             cudaStream_t s) {
    if (nc > 0) k_cond_color_round<<<nblk(nc), NT, 0, s>>>(C, nc, B, inc, col_in, col_out, uncolored, too_many);
}
void launch_cond_jacobi(const Scene& sc, const Contacts& C, int nc, const CondBufs& B, const Incidence& inc,
                        double relax, double alpha, double* u, const DevScalars* ds, cudaStream_t s) {
    if (nc > 0) k_cond_jacobi_blocks<<<nblk(nc, 128), 128, 0, s>>>(sc, C, B, nc, relax, alpha, u, ds);
    if (sc.N > 0) k_cond_jacobi_bodies<<<nblk(sc.N, 128), 128, 0, s>>>(sc, C, B, inc, u, ds);
}
void launch_cond_sweep_color(const Scene& sc, const Contacts& C, const CondBufs& B, const uint32_t* blocks, int n,
                             double relax, double alpha, double* u, const DevScalars* ds, cudaStream_t s) {
    if (n > 0) k_cond_sweep_color<<<nblk(n, 128), 128, 0, s>>>(sc, C, B, blocks, n, relax, alpha, u, ds);
}
int cond_chunks(int N) { return (6 * N + RED_CHUNK - 1) / RED_CHUNK; }
void launch_cond_check(int N, const CondBufs& B, double tol_rel, double tol_abs, int iter, DevScalars* ds,
                       cudaStream_t s) {
    const int nch = cond_chunks(N);
    if (nch > 0) k_cond_res_partials<<<nblk(nch, 128), 128, 0, s>>>(N, B.uf, B.up, B.u, tol_rel, tol_abs, B.part, ds);
    k_cond_check<<<1, 128, 0, s>>>(N, B.part, nch, iter, ds, B.flags, B.err);
}
void launch_cond_copy(int n, const double* src, double* dst, const DevScalars* ds, cudaStream_t s) {
    if (n > 0) k_cond_copy<<<nblk(n), NT, 0, s>>>(n, src, dst, ds);
}
void launch_cond_final(const Scene& sc, Contacts& C, int gen, int nc, const CondBufs& B, double* x, int pj_convention,
                       cudaStream_t s) {
    if (pj_convention < 0) {
        if (sc.N > 0) k_cond_final_body<<<nblk(6 * sc.N), NT, 0, s>>>(sc.N, B.uf, B.u, x);
        return;
    }
    if (nc > 0) k_cond_lambda_out<<<nblk(nc), NT, 0, s>>>(C, gen, nc, B, pj_convention);
}

}  // namespace cdx
