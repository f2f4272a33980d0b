// Projected Gauss-Seidel in FP64 (solver.type=projected_gauss_seidel), for the plain FP64 method;
// compiled without FMA contraction so every result is rounded as written and matches the CPU
// oracle bit for bit.
//
// ProjectedGaussSeidelSolver::solve (src/physics/solver/projected_gauss_seidel.cpp:56-264), plain
// loop, contact rows only. One block per contact, visited in W's row order (frictionless contacts
// first, then frictional ones; the rank of contact c is C.rank[c]); a block reads and writes the
// velocity correction u_corr of its two bodies, so a sweep is sequential along every body's list of
// blocks and free across bodies.
//  - Levels: a block's level is one more than the larger level of its predecessors (the previous
//    block of each of its bodies in sweep order); blocks of one level share no body. They are
//    computed per step by frontiers over the chains in one cooperative launch (a grid barrier a
//    level), which writes the blocks level by level.
//  - The sweeps run as one cooperative launch, one level at a time: a level's blocks are spread
//    over all threads, then a grid barrier (release/acquire, bounded wait) lets the next level
//    read what they wrote. (Per-block ready flags instead of the barrier measured slower: tens of
//    thousands of waiting threads polling L2 starve the ones that compute.)
//  - After a sweep: a grid barrier, the velocity-increment residual (the fixed three-level order
//    the oracle sums in) and the stop decision.
// Every block therefore sees exactly the u_corr of the sequential sweep, and the result is the
// sequential sweep's, bit for bit.
#include <cstdint>

#include "cdx_internal.h"
#include "fp64_math.cuh"

namespace cdx {
namespace {

constexpr int NT = 256;
inline int nblk(int64_t n, int nt = NT) { return (int)((n + nt - 1) / nt); }
constexpr int RED_CHUNK = 256;  // the fixed three-level order of the residual sum (shared with the oracle)
constexpr int RED_GROUP = 64;
constexpr unsigned long long PGS_WAIT_NS = 500000000ull;  // 0.5 s: a wait that long means a fault
using f64::smin;

__device__ __forceinline__ double minv_of(const Scene& sc, int i, int k) {
    return k < 3 ? sc.bf(BF_MINVL)[i] : sc.bf(BF_MINVA)[i];
}

// W row q of contact c on one side: sign * [d_q (world), c_q (body-frame lever product)]
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

// velocities are field-major (component k of body i at k * N + i); LD reads them through L2
// (ld.global.cg) when they change inside the launch
template <bool LD>
__device__ __forceinline__ double uget(const double* u, size_t j) {
    return LD ? __ldcg(u + j) : u[j];
}

}  // namespace
}  // namespace cdx
#include "cond_block.cuh"
namespace cdx {
namespace {

// sum over row q's nonzeros in W's column order (the lower body index first), from zero, as
// Eigen's row-major sparse product sums a row
template <bool LD>
__device__ __forceinline__ double wdot(const double (*J)[6], int a, int b, const double* u, int N) {
    double t = 0.0;
    const bool a_first = a >= 0 && a < b;
    for (int side = 0; side < 2; ++side) {
        const bool isA = (side == 0) == a_first;
        const int body = isA ? a : b;
        if (body < 0) continue;
        const double* Jr = J[isA ? 0 : 1];
        for (int k = 0; k < 6; ++k) t = t + Jr[k] * uget<LD>(u, (size_t)k * N + body);
    }
    return t;
}

// per contact: rhs_q = W_q u_free + b_q (b = contact velocity, plus e . (W v_n + b) with
// restitution; PgsAssembler::rhs, pgs_assembler.cpp:71-80), Dinv_q = 1 / sum w^2 M^-1 over the row
// (DinvDiag, :219-294; a frictionless row guards a zero sum), and the warm-started impulses with
// the normal sign inverted (projected_gauss_seidel.cpp:103-109)
__global__ void k_pgs_setup(Scene sc, Contacts C, int gen, int nc, const double* uf, int warmstart, CondBufs B) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    const int64_t cap = C.cap;
    const int N = sc.N;
    const int a = C.a[c], b = C.b[c];
    const bool fr = (C.flags[c] & CF_FRICTIONAL) != 0;
    const int dim = fr ? 3 : 1;
    for (int q = 0; q < dim; ++q) {
        double J[2][6];
        jac_row(C, c, q, false, J[0]);
        jac_row(C, c, q, true, J[1]);
        const double cb = C.cb[q * cap + c];
        const double e = q == 0 ? C.eN[c] : C.eT[c];
        // the reference adds e . v_prev to every row once some row has restitution; on a row with
        // e = 0 that adds a signed zero to cb (never -0), which leaves it as it is
        double bias = cb;
        if (e != 0.0) {
            double tv = 0.0;
            const bool a_first = a >= 0 && a < b;
            for (int side = 0; side < 2; ++side) {
                const bool isA = (side == 0) == a_first;
                const int body = isA ? a : b;
                if (body < 0) continue;
                const double* Jr = J[isA ? 0 : 1];
                const double v[6] = {sc.bf(BF_VX)[body], sc.bf(BF_VY)[body], sc.bf(BF_VZ)[body],
                                     sc.bf(BF_WX)[body], sc.bf(BF_WY)[body], sc.bf(BF_WZ)[body]};
                for (int k = 0; k < 6; ++k) tv = tv + Jr[k] * v[k];
            }
            bias = cb + e * (tv + cb);
        }
        B.rhs[q * cap + c] = wdot<false>(J, a, b, uf, N) + bias;
        double d = 0.0;
        const bool a_first = a >= 0 && a < b;
        for (int side = 0; side < 2; ++side) {
            const bool isA = (side == 0) == a_first;
            const int body = isA ? a : b;
            if (body < 0) continue;
            const double* Jr = J[isA ? 0 : 1];
            for (int k = 0; k < 6; ++k) d = d + (Jr[k] * Jr[k]) * minv_of(sc, body, k);
        }
        B.ginv[q * cap + c] = fr ? 1.0 / d : (d > 0 ? 1.0 / d : 0.0);
    }
    const double* l0 = C.lam[gen];
    B.lam[c] = warmstart ? -l0[c] : 0.0;
    B.lam[cap + c] = (warmstart && fr) ? l0[cap + c] : 0.0;
    B.lam[2 * cap + c] = (warmstart && fr) ? l0[2 * cap + c] : 0.0;
}

// u_corr = M^-1 W^T lambda (:117): per body, the rows of its blocks in row order (the incidence is
// in row order), each adding (M^-1_k w) lambda_q to component k, from zero
__global__ void k_pgs_ucorr_init(Scene sc, Contacts C, CondBufs B, Incidence inc, double* u) {
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
        for (int q = 0; q < dim; ++q) {
            double J[6];
            jac_row(C, c, q, sideB, J);
            const double l = B.lam[q * cap + c];
            for (int k = 0; k < 6; ++k) acc[k] = acc[k] + (minv_of(sc, i, k) * J[k]) * l;
        }
    }
    for (int k = 0; k < 6; ++k) u[(size_t)k * N + i] = acc[k];
}

// predecessors and successors: per contact and side, the previous and the next block of that body
// in sweep order (or -1); the incidence lists are in sweep order
__global__ void k_pgs_links(int N, Incidence inc, PgsBufs P) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N) return;
    int prev = -1;
    uint32_t prev_code = 0;
    for (int p = inc.start[t]; p < inc.end[t]; ++p) {
        const uint32_t code = inc.val_out[p];
        const int c = (int)(code >> 1);
        P.pred[(size_t)(code & 1u) * P.cap + c] = prev;
        if (prev >= 0) P.succ[(size_t)(prev_code & 1u) * P.cap + prev] = c;
        prev = c;
        prev_code = code;
    }
}

__device__ __forceinline__ int ld_acquire_s32(const int32_t* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Grid barrier of the cooperative launch (epoch-counted, release/acquire, bounded): false when the
// wait ran out or another block gave up (*err set); every thread of the block gets the same answer.
__device__ __forceinline__ bool grid_sync(unsigned* ctr, unsigned epoch, int32_t* err, unsigned long long wait_ns) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(ctr) : "memory");
        const unsigned target = epoch * gridDim.x;
        const unsigned long long t0 = global_ns();
        int ok = 1;
        while ((int)(ld_acquire_u32(ctr) - target) < 0) {
            if (ld_acquire_s32(err) != 0 || global_ns() - t0 > wait_ns) {
                atomicExch(err, 1);
                ok = 0;
                break;
            }
            __nanosleep(32);
        }
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}


// Levels by frontiers (Kahn's order over the per-body chains): a block's count of unfinished
// predecessors starts at how many it has; level 0 is the blocks with none; each level's blocks then
// count down their successors, and those reaching zero form the next level. A block joins a level
// when its last predecessor is done, so its level is one more than its predecessors' largest: the
// longest chain ending at it. The blocks are written level by level into `order` (the order
// within a level varies from run to run and does not matter: a level's blocks share no body); each
// level's range goes to P.lstart / P.lend, the number of levels to P.maxlev + 1. One grid barrier a
// level; no sort.
__global__ void __launch_bounds__(NT) k_pgs_levels(PgsBufs P, int nc, uint32_t* order, unsigned long long wait_ns) {
    const int T = gridDim.x * blockDim.x;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    int32_t* cnt = P.rflag;  // blocks placed so far
    unsigned epoch = 0;
    for (int c = t; c < nc; c += T) P.lev[c] = (P.pred[c] >= 0 ? 1 : 0) + (P.pred[P.cap + c] >= 0 ? 1 : 0);
    if (!grid_sync(P.bar, ++epoch, P.err, wait_ns)) return;
    for (int c = t; c < nc; c += T)
        if (__ldcg(P.lev + c) == 0) __stcg(order + atomicAdd(cnt, 1), (uint32_t)c);
    if (!grid_sync(P.bar, ++epoch, P.err, wait_ns)) return;
    int b0 = 0, b1 = __ldcg(cnt), L = 0;
    if (t == 0) {
        P.lstart[0] = 0;
        P.lend[0] = b1;
    }
    while (b1 < nc) {
        for (int r = b0 + t; r < b1; r += T) {
            const int c = (int)__ldcg(order + r);
            for (int side = 0; side < 2; ++side) {
                const int sc_ = P.succ[(size_t)side * P.cap + c];
                if (sc_ >= 0 && atomicSub(P.lev + sc_, 1) == 1) __stcg(order + atomicAdd(cnt, 1), (uint32_t)sc_);
            }
        }
        if (!grid_sync(P.bar, ++epoch, P.err, wait_ns)) return;
        b0 = b1;
        b1 = __ldcg(cnt);
        if (b1 == b0) {  // no progress: the chains are not in sweep order (cannot happen)
            if (t == 0) atomicExch(P.err, 3);
            return;
        }
        ++L;
        if (t == 0) {
            P.lstart[L] = b0;
            P.lend[L] = b1;
        }
    }
    if (t == 0) *P.maxlev = L;
}

// One block of pgs_sweep (:158-182): res = rhs - W_b u_corr (- C lambda, zero on contact rows),
// dlambda = (Dinv res) relax alpha, lambda += dlambda, project (:11-27, whose corrections enter
// dlambda), u_corr += M^-1 W_b^T dlambda column by column
__device__ __forceinline__ void pgs_block(const Scene& sc, const Contacts& C, const CondBufs& B, int c, double relax,
                                          double alpha, double* u) {
    const int N = sc.N;
    const int64_t cap = C.cap;
    const int a = C.a[c], b = C.b[c];
    const int dim = (C.flags[c] & CF_FRICTIONAL) ? 3 : 1;
    double J[3][2][6], rs[3], dl[3], lam[3];
    for (int q = 0; q < dim; ++q) {
        jac_row(C, c, q, false, J[q][0]);
        jac_row(C, c, q, true, J[q][1]);
        lam[q] = __ldcg(&B.lam[q * cap + c]);
        double o = B.rhs[q * cap + c];
        o = o - wdot<true>(J[q], a, b, u, N);
        o = o - 0.0 * lam[q];
        rs[q] = o;
    }
    for (int q = 0; q < dim; ++q) {
        // the block of Dinv is diagonal, stored dense: the zero entries multiply the other residuals
        double g = (q == 0 ? B.ginv[c] : 0.0) * rs[0];
        for (int j = 1; j < dim; ++j) g = g + (q == j ? B.ginv[j * cap + c] : 0.0) * rs[j];
        dl[q] = (g * relax) * alpha;
        lam[q] = lam[q] + dl[q];
    }
    const double n0 = lam[0];
    lam[0] = smin(n0, 0.0);
    dl[0] = dl[0] + (lam[0] - n0);
    if (dim == 3) {
        const double t1 = lam[1], t2 = lam[2];
        const double tn = sqrt(t1 * t1 + t2 * t2);
        if (tn > 0.0) {
            const double s = smin(1.0, -(C.mu[c] * lam[0]) / tn);
            const double p1 = s * t1, p2 = s * t2;
            dl[1] = dl[1] + (p1 - t1);
            dl[2] = dl[2] + (p2 - t2);
            lam[1] = p1;
            lam[2] = p2;
        }
    }
    for (int side = 0; side < 2; ++side) {
        const int body = side == 0 ? a : b;
        if (body < 0) continue;
        for (int k = 0; k < 6; ++k) {
            const size_t j = (size_t)k * N + body;
            const double mk = minv_of(sc, body, k);
            double v = __ldcg(u + j);
            for (int q = 0; q < dim; ++q) v = v + (mk * J[q][side][k]) * dl[q];
            __stcg(u + j, v);
        }
    }
    for (int q = 0; q < dim; ++q) __stcg(&B.lam[q * cap + c], lam[q]);
}

// The solve: sweeps until the velocity-increment residual is below 1 (or not finite: the solve
// diverged, check_residual :142-151) or max_iter sweeps.
template <int COND>
__global__ void __launch_bounds__(NT) k_pgs_solve(Scene sc, Contacts C, CondBufs B, PgsBufs P, const uint32_t* order,
                                                  int nlev, double relax, double alpha, double tol_rel,
                                                  double tol_abs, int max_iter, DevScalars* ds,
                                                  unsigned long long wait_ns) {
    const int T = gridDim.x * blockDim.x;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int N = sc.N, nv = 6 * N;
    const int nch = (nv + RED_CHUNK - 1) / RED_CHUNK;
    __shared__ int s_stop;
    unsigned epoch = 0;
    for (int it = 0; it < max_iter; ++it) {
        // one level at a time: its blocks share no body, and every earlier level is done
        for (int L = 0; L < nlev; ++L) {
            const int r1 = P.lend[L];
            for (int r = P.lstart[L] + t; r < r1; r += T) {
                const int c = (int)order[r];
                if (COND) {
                    // the condensed solver's sequential sweep (gaussSeidelSweep, condensed_solver.cpp:166-182)
                    double d[3];
                    cond_block<true, true>(sc, C, B, c, relax, alpha, B.u, d);
                } else {
                    pgs_block(sc, C, B, c, relax, alpha, B.u);
                }
            }
            if (!grid_sync(P.bar, ++epoch, P.err, wait_ns)) return;
        }
        // the residual's chunk sums; up takes u for the next sweep's test
        for (int ch = t; ch < nch; ch += T) {
            const int j0 = ch * RED_CHUNK, j1 = min(nv, j0 + RED_CHUNK);
            double s = 0.0;
            for (int j = j0; j < j1; ++j) {
                const size_t e = (size_t)(j % 6) * N + j / 6;
                const double uc = __ldcg(B.u + e), up = __ldcg(B.up + e), uf = B.uf[e];
                const double diff = uc - up;
                const double v0 = uf - up, v1 = uf - uc;
                const double q = f64::smax(fabs(v0), fabs(v1)) * tol_rel + tol_abs;
                const double tt = diff / q;
                s = s + tt * tt;
                __stcg(B.up + e, uc);
            }
            __stcg(B.part + ch, s);
        }
        if (!grid_sync(P.bar, ++epoch, P.err, wait_ns)) return;
        // the chunk sums in groups of RED_GROUP (a thread a group), then the group sums in order:
        // the fixed three-level order the oracle sums in
        const int ngroups = (nch + RED_GROUP - 1) / RED_GROUP;
        for (int g = t; g < ngroups; g += T) {
            double gsum = 0.0;
            const int c1 = min(nch, (g + 1) * RED_GROUP);
            for (int c = g * RED_GROUP; c < c1; ++c) gsum = gsum + __ldcg(B.part + c);
            __stcg(B.part + nch + g, gsum);
        }
        if (!grid_sync(P.bar, ++epoch, P.err, wait_ns)) return;
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            double tot = 0.0;
            for (int k = 0; k < ngroups; ++k) tot = tot + __ldcg(B.part + nch + k);
            const double err = 1.0 / sqrt((double)nv) * sqrt(tot);
            ds->iters = it + 1;
            ds->res_last = err;
            *B.err = err;
            int stop = 0;
            if (!isfinite(err)) {
                B.flags[0] = 1;
                stop = 1;
            } else if (err < 1.0) {
                stop = 1;
            }
            __stcg(P.stop, stop);
        }
        if (!grid_sync(P.bar, ++epoch, P.err, wait_ns)) return;
        if (threadIdx.x == 0) s_stop = __ldcg(P.stop);
        __syncthreads();
        if (s_stop) break;
    }
}

}  // namespace

void launch_pgs_setup(const Scene& sc, Contacts& C, int gen, int nc, int warmstart, CondBufs& B, const Incidence& inc,
                      PgsBufs& P, cudaStream_t s) {
    if (nc > 0) k_pgs_setup<<<nblk(nc), NT, 0, s>>>(sc, C, gen, nc, B.uf, warmstart, B);
    if (sc.N > 0) k_pgs_ucorr_init<<<nblk(sc.N), NT, 0, s>>>(sc, C, B, inc, B.u);
    launch_pgs_links(sc, nc, inc, P, s);
}
void launch_pgs_links(const Scene& sc, int nc, const Incidence& inc, PgsBufs& P, cudaStream_t s) {
    cudaMemsetAsync(P.pred, 0xff, sizeof(int32_t) * 2 * (size_t)P.cap, s);
    cudaMemsetAsync(P.succ, 0xff, sizeof(int32_t) * 2 * (size_t)P.cap, s);
    (void)nc;
    if (sc.N > 0) k_pgs_links<<<nblk(sc.N), NT, 0, s>>>(sc.N, inc, P);
}

// grid of a cooperative launch: every block resident (at most two an SM)
template <class K>
static int coop_grid(K kernel) {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, NT, 0);
    return sms * std::max(1, std::min(per, 2));
}

int launch_pgs_levels(const PgsBufs& P, int nc, uint32_t* order, unsigned long long wait_ns, cudaStream_t s) {
    cudaMemsetAsync(P.bar, 0, sizeof(unsigned), s);
    cudaMemsetAsync(P.err, 0, sizeof(int32_t), s);
    cudaMemsetAsync(P.rflag, 0, sizeof(int32_t) * 3, s);
    cudaMemsetAsync(P.maxlev, 0, sizeof(int32_t), s);
    PgsBufs a0 = P;
    int n = nc;
    uint32_t* o = order;
    unsigned long long wn = wait_ns > 0 ? wait_ns : PGS_WAIT_NS;
    void* args[] = {&a0, &n, &o, &wn};
    static int grid = 0;
    if (grid == 0) grid = coop_grid(k_pgs_levels);
    return (int)cudaLaunchCooperativeKernel((const void*)k_pgs_levels, dim3(grid), dim3(NT), args, 0, s);
}

int launch_pgs_solve(const Scene& sc, const Contacts& C, int nlev, const CondBufs& B, const PgsBufs& P,
                     const uint32_t* order, double relax, double alpha, double tol_rel, double tol_abs, int max_iter,
                     DevScalars* ds, unsigned long long wait_ns, cudaStream_t s, int condensed) {
    cudaMemsetAsync(P.bar, 0, sizeof(unsigned), s);
    cudaMemsetAsync(P.err, 0, sizeof(int32_t), s);
    cudaMemsetAsync(P.stop, 0, sizeof(int32_t), s);
    Scene a0 = sc;
    Contacts a1 = C;
    CondBufs a2 = B;
    PgsBufs a3 = P;
    const uint32_t* o = order;
    int nl = nlev, mi = max_iter;
    double rl = relax, al = alpha, tr = tol_rel, ta = tol_abs;
    unsigned long long wn = wait_ns > 0 ? wait_ns : PGS_WAIT_NS;
    void* args[] = {&a0, &a1, &a2, &a3, &o, &nl, &rl, &al, &tr, &ta, &mi, &ds, &wn};
    static int grid[2] = {0, 0};
    const void* k = condensed ? (const void*)k_pgs_solve<1> : (const void*)k_pgs_solve<0>;
    if (grid[condensed ? 1 : 0] == 0) grid[condensed ? 1 : 0] = condensed ? coop_grid(k_pgs_solve<1>) : coop_grid(k_pgs_solve<0>);
    return (int)cudaLaunchCooperativeKernel(k, dim3(grid[condensed ? 1 : 0]), dim3(NT), args, 0, s);
}

}  // namespace cdx
