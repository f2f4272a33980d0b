// Host side of the condensed solver's colored sweeps in the plain FP64 method
// (solver.type=condensed, condensed.sweep_mode=colored): CondensedSolver::solve
// (src/physics/solver/condensed_solver.cpp:443-760) with the projection local solve and the
// standard loop, for sphere contacts. Per step: the free velocities, each block's 1/G_ii and rhs,
// the warm-started impulses and u_corr; the coloring (Jones-Plassmann rounds on the GPU, equal to
// the greedy Welsh-Powell pass); the blocks sorted by color; then sweeps of one launch per color
// with the velocity-increment stop test after every sweep, evaluated on the device (the host polls
// every gpu.check_every sweeps). The result is u = u_free - u_corr; the impulses are stored with
// the normal sign inverted back (warmstart.hpp:41-56), and the step's complementarity residual is
// evaluated as for projected Jacobi on the applied impulses.
#include <algorithm>
#include <cstring>
#include <vector>

#include "engine.h"

using namespace cdx;

int Engine::ensure_cond() {
    CondBufs& B = cond;
    const int64_t cap = std::max<int64_t>(C.cap, 1);
    const int N = std::max(sc.N, 1);
    if (B.cap == cap && B.N == N) return CDX_OK;
    void* old[] = {B.ginv, B.rhs, B.lam, B.deg, B.col, B.col2, B.uf, B.u, B.up, B.part, B.flags, B.err,
                   B.kin, B.vin, B.kout, B.vout, B.cstart, B.cend, B.dl};
    for (void* p : old)
        if (p) dfree(p);
    B = CondBufs{};
    int st;
    if ((st = dalloc((void**)&B.ginv, sizeof(double) * 3 * cap, "condensed"))) return st;
    if ((st = dalloc((void**)&B.rhs, sizeof(double) * 3 * cap, "condensed"))) return st;
    if ((st = dalloc((void**)&B.lam, sizeof(double) * 3 * cap, "condensed"))) return st;
    if ((st = dalloc((void**)&B.dl, sizeof(double) * 3 * cap, "condensed"))) return st;
    if ((st = dalloc((void**)&B.deg, sizeof(int32_t) * cap, "condensed"))) return st;
    if ((st = dalloc((void**)&B.col, sizeof(int32_t) * cap, "condensed"))) return st;
    if ((st = dalloc((void**)&B.col2, sizeof(int32_t) * cap, "condensed"))) return st;
    if ((st = dalloc((void**)&B.uf, sizeof(double) * 6 * N, "condensed"))) return st;
    if ((st = dalloc((void**)&B.u, sizeof(double) * 6 * N, "condensed"))) return st;
    if ((st = dalloc((void**)&B.up, sizeof(double) * 6 * N, "condensed"))) return st;
    // the chunk sums, then the group sums of the fixed three-level order
    if ((st = dalloc((void**)&B.part, sizeof(double) * (cond_chunks(N) + cond_chunks(N) / 64 + 2), "condensed")))
        return st;
    if ((st = dalloc((void**)&B.flags, sizeof(int32_t) * 4, "condensed"))) return st;
    if ((st = dalloc((void**)&B.err, sizeof(double), "condensed"))) return st;
    uint32_t** u32[] = {&B.kin, &B.vin, &B.kout, &B.vout};
    for (auto p : u32)
        if ((st = dalloc((void**)p, sizeof(uint32_t) * cap, "condensed"))) return st;
    if ((st = dalloc((void**)&B.cstart, sizeof(int32_t) * CDX_COND_MAX_COLORS, "condensed"))) return st;
    if ((st = dalloc((void**)&B.cend, sizeof(int32_t) * CDX_COND_MAX_COLORS, "condensed"))) return st;
    B.cap = cap;
    B.N = N;
    // the color sort reuses the engine's radix-sort scratch, sized for twice the capacity
    return ensure_tmp(cap);
}

int Engine::solve_condensed() {
    const int N = sc.N;
    int st;
    cond_diverged = 0;
    last_iters = 0;
    last_res = 0;
    last_res_final = 0;
    if ((st = ensure_cond())) return st;
    CondBufs& B = cond;
    cudaMemsetAsync(ds, 0, sizeof(DevScalars), stream);
    cudaMemsetAsync(B.flags, 0, sizeof(int32_t) * 4, stream);
    launch_cond_setup(sc, C, gen, nc, cfg.sim_dt, cfg.sim_gravity, cfg.moreau_implicit_gyroscopy, cfg.pj_warmstart, B,
                      inc, stream);
    launches += 3;
    if (nc == 0) {
        // no constraint rows: the free velocity (condensed_solver.cpp:453)
        launch_cond_final(sc, C, gen, nc, B, x, -1, stream);
        ++launches;
        return CDX_OK;
    }
    if (cfg.condensed_sweep_mode == 0) return solve_condensed_gs();
    if (cfg.condensed_sweep_mode == 1) {
        // Jacobi sweeps (jacobiSweep, condensed_solver.cpp:268-317): both passes, then the stop test
        const int nv6 = 6 * N;
        launch_cond_copy(nv6, B.u, B.up, ds, stream);
        const int maxit = std::max(1, cfg.pj_max_iterations);
        const int every = std::max(1, cfg.gpu_check_every);
        for (int it = 0; it < maxit; ++it) {
            launch_cond_jacobi(sc, C, nc, B, inc, cfg.pj_relaxation, cfg.pj_alpha, B.u, ds, stream);
            launch_cond_check(N, B, cfg.pj_tol_rel, cfg.pj_tol_abs, it, ds, stream);
            launch_cond_copy(nv6, B.u, B.up, ds, stream);
            launches += 5;
            if ((it + 1) % every == 0 && it + 1 < maxit) {
                cudaMemcpyAsync(&hs->done, &ds->done, sizeof(int32_t), cudaMemcpyDeviceToHost, stream);
                if ((st = cuda_check(cudaStreamSynchronize(stream), "condensed poll"))) return st;
                if (hs->done) break;
            }
        }
        return finish_condensed();
    }
    // coloring: rounds until every block is colored
    int32_t* col_in = B.col;
    int32_t* col_out = B.col2;
    int32_t hflags[4] = {0, 0, 0, 0};
    const int max_rounds = 1 << 14;
    int rounds = 0;
    for (;;) {
        for (int r = 0; r < 8; ++r) {
            cudaMemsetAsync(B.flags + 1, 0, sizeof(int32_t), stream);
            launch_cond_color_round(C, nc, B, inc, col_in, col_out, B.flags + 1, B.flags + 2, stream);
            std::swap(col_in, col_out);
            ++launches;
            ++rounds;
        }
        cudaMemcpyAsync(hflags, B.flags, sizeof(hflags), cudaMemcpyDeviceToHost, stream);
        if ((st = cuda_check(cudaStreamSynchronize(stream), "condensed coloring"))) return st;
        if (hflags[2]) return fail(CDX_ERR_OVERFLOW, "condensed coloring needs more than 128 colors");
        if (hflags[1] == 0) break;
        if (rounds >= max_rounds) return fail(CDX_ERR_STATE, "condensed coloring did not finish");
    }
    // the blocks sorted by color (stable: contact order within a color), and each color's range
    {
        launch_cond_sort_keys(nc, col_in, B, stream);
        if ((st = cuda_check(sort_pairs(tmp, tmp_bytes, B.kin, B.kout, B.vin, B.vout, nc, 8, stream), "sort colors")))
            return st;
        cudaMemsetAsync(B.cstart, 0, sizeof(int32_t) * CDX_COND_MAX_COLORS, stream);
        cudaMemsetAsync(B.cend, 0, sizeof(int32_t) * CDX_COND_MAX_COLORS, stream);
        launch_ranges(B.kout, nc, B.cstart, B.cend, stream);
        launches += 6;
    }
    std::vector<int32_t> cs(CDX_COND_MAX_COLORS), ce(CDX_COND_MAX_COLORS);
    cudaMemcpyAsync(cs.data(), B.cstart, sizeof(int32_t) * CDX_COND_MAX_COLORS, cudaMemcpyDeviceToHost, stream);
    cudaMemcpyAsync(ce.data(), B.cend, sizeof(int32_t) * CDX_COND_MAX_COLORS, cudaMemcpyDeviceToHost, stream);
    if ((st = cuda_check(cudaStreamSynchronize(stream), "condensed colors"))) return st;
    int ncolors = 0;
    for (int k = 0; k < CDX_COND_MAX_COLORS; ++k)
        if (ce[k] > cs[k]) ncolors = k + 1;
    // sweeps with the stop test after each, evaluated on the device
    const int nv6 = 6 * N;
    launch_cond_copy(nv6, B.u, B.up, ds, stream);
    const int maxit = std::max(1, cfg.pj_max_iterations);
    const int every = std::max(1, cfg.gpu_check_every);
    for (int it = 0; it < maxit; ++it) {
        for (int k = 0; k < ncolors; ++k)
            launch_cond_sweep_color(sc, C, B, B.vout + cs[k], ce[k] - cs[k], cfg.pj_relaxation, cfg.pj_alpha, B.u, ds,
                                    stream);
        launch_cond_check(N, B, cfg.pj_tol_rel, cfg.pj_tol_abs, it, ds, stream);
        launch_cond_copy(nv6, B.u, B.up, ds, stream);
        launches += ncolors + 3;
        if ((it + 1) % every == 0 && it + 1 < maxit) {
            cudaMemcpyAsync(&hs->done, &ds->done, sizeof(int32_t), cudaMemcpyDeviceToHost, stream);
            if ((st = cuda_check(cudaStreamSynchronize(stream), "condensed poll"))) return st;
            if (hs->done) break;
        }
    }
    return finish_condensed();
}

// the result, the complementarity residual on the applied impulses, the stored impulses
int Engine::finish_condensed() {
    CondBufs& B = cond;
    launch_cond_final(sc, C, gen, nc, B, x, -1, stream);
    launch_cond_final(sc, C, gen, nc, B, x, 1, stream);
    launch_sweep_contact64(sc, C, gen, nc, x, ds, 1, stream);
    launch_final_residual(ds, stream);
    launch_cond_final(sc, C, gen, nc, B, x, 0, stream);
    launches += 5;
    int32_t hflags[4] = {0, 0, 0, 0};
    cudaMemcpyAsync(hflags, B.flags, sizeof(hflags), cudaMemcpyDeviceToHost, stream);
    int st;
    if ((st = cuda_check(cudaStreamSynchronize(stream), "condensed solve"))) return st;
    cond_diverged = hflags[0];
    return CDX_OK;
}

// condensed.sweep_mode=gauss_seidel (gaussSeidelSweep, condensed_solver.cpp:166-182): blocks in
// contact order, each seeing the u_corr of every earlier block; run by the projected Gauss-Seidel
// machinery (levels of the per-body chains, then the ordered sweep in one cooperative launch)
int Engine::solve_condensed_gs() {
    CondBufs& B = cond;
    int st;
    if ((st = ensure_pgs())) return st;
    launch_pgs_links(sc, nc, inc, pgs, stream);
    launch_cond_copy(6 * sc.N, B.u, B.up, ds, stream);
    launches += 2;
    const unsigned long long wait_ns = cfg.gpu_coop_wait_ns > 0 ? (unsigned long long)cfg.gpu_coop_wait_ns : 0ull;
    if ((st = cuda_check((cudaError_t)launch_pgs_levels(pgs, nc, B.vout, wait_ns, stream), "levels launch")))
        return st;
    ++launches;
    int32_t hl[2] = {0, 0};
    cudaMemcpyAsync(&hl[0], pgs.maxlev, sizeof(int32_t), cudaMemcpyDeviceToHost, stream);
    cudaMemcpyAsync(&hl[1], pgs.err, sizeof(int32_t), cudaMemcpyDeviceToHost, stream);
    if ((st = cuda_check(cudaStreamSynchronize(stream), "condensed levels"))) return st;
    if (hl[1] == 3) return fail(CDX_ERR_STATE, "condensed levels: the block chains made no progress");
    if (hl[1]) return fail(CDX_ERR_TIMEOUT, "condensed levels: a grid barrier wait ran out (gpu.coop_wait_ns)");
    last_levels = hl[0] + 1;
    if ((st = cuda_check((cudaError_t)launch_pgs_solve(sc, C, last_levels, B, pgs, B.vout, cfg.pj_relaxation, cfg.pj_alpha,
                                                       cfg.pj_tol_rel, cfg.pj_tol_abs, cfg.pj_max_iterations, ds,
                                                       wait_ns, stream, 1),
                         "condensed sweep launch")))
        return st;
    ++launches;
    int32_t herr = 0;
    cudaMemcpyAsync(&herr, pgs.err, sizeof(int32_t), cudaMemcpyDeviceToHost, stream);
    if ((st = cuda_check(cudaStreamSynchronize(stream), "condensed sweeps"))) return st;
    if (herr) return fail(CDX_ERR_TIMEOUT, "condensed sweeps: a wait ran out (gpu.coop_wait_ns)");
    return finish_condensed();
}
