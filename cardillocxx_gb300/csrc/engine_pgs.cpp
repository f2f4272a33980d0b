// Host side of projected Gauss-Seidel in the plain FP64 method (solver.type=projected_gauss_seidel):
// ProjectedGaussSeidelSolver::solve (src/physics/solver/projected_gauss_seidel.cpp:56-264) with its
// plain loop. Per step: the free velocities, each row's rhs and Dinv, the warm-started impulses and
// u_corr, the per-body chains of blocks in row order; then one cooperative launch runs the sweeps
// (sequential along every body's chain) with the stop test after each. The result is
// u = u_free - u_corr; the impulses are stored with the normal sign inverted back
// (projected_gauss_seidel.cpp:257-259), and the step's complementarity residual is evaluated as for
// projected Jacobi on the applied impulses.
#include <algorithm>

#include "engine.h"

using namespace cdx;

int Engine::ensure_pgs() {
    PgsBufs& P = pgs;
    const int64_t cap = std::max<int64_t>(C.cap, 1);
    if (P.cap == cap) return CDX_OK;
    void* old[] = {P.pred, P.succ, P.lstart, P.lend, P.bar, P.err, P.stop, P.lev, P.rflag, P.maxlev};
    for (void* p : old)
        if (p) dfree(p);
    P = PgsBufs{};
    int st;
    if ((st = dalloc((void**)&P.pred, sizeof(int32_t) * 2 * cap, "pgs"))) return st;
    if ((st = dalloc((void**)&P.succ, sizeof(int32_t) * 2 * cap, "pgs"))) return st;
    if ((st = dalloc((void**)&P.lstart, sizeof(int32_t) * cap, "pgs"))) return st;
    if ((st = dalloc((void**)&P.lend, sizeof(int32_t) * cap, "pgs"))) return st;
    if ((st = dalloc((void**)&P.bar, sizeof(unsigned), "pgs"))) return st;
    if ((st = dalloc((void**)&P.err, sizeof(int32_t), "pgs"))) return st;
    if ((st = dalloc((void**)&P.stop, sizeof(int32_t), "pgs"))) return st;
    if ((st = dalloc((void**)&P.lev, sizeof(int32_t) * cap, "pgs"))) return st;
    if ((st = dalloc((void**)&P.rflag, sizeof(int32_t) * 3, "pgs"))) return st;
    if ((st = dalloc((void**)&P.maxlev, sizeof(int32_t), "pgs"))) return st;
    P.cap = cap;
    return CDX_OK;
}

int Engine::solve_pgs() {
    int st;
    cond_diverged = 0;
    last_iters = 0;
    last_res = 0;
    last_res_final = 0;
    if ((st = ensure_cond())) return st;
    if ((st = ensure_pgs())) return st;
    CondBufs& B = cond;
    cudaMemsetAsync(ds, 0, sizeof(DevScalars), stream);
    cudaMemsetAsync(B.flags, 0, sizeof(int32_t) * 4, stream);
    launch_cond_ufree(sc, cfg.sim_dt, cfg.sim_gravity, cfg.moreau_implicit_gyroscopy, B, stream);
    ++launches;
    if (nc == 0) {
        // no constraint rows: the free velocity (projected_gauss_seidel.cpp:79)
        launch_cond_final(sc, C, gen, nc, B, x, -1, stream);
        ++launches;
        return CDX_OK;
    }
    launch_pgs_setup(sc, C, gen, nc, cfg.pj_warmstart, B, inc, pgs, stream);
    launch_cond_copy(6 * sc.N, B.u, B.up, ds, stream);
    launches += 4;
    const unsigned long long wait_ns = cfg.gpu_coop_wait_ns > 0 ? (unsigned long long)cfg.gpu_coop_wait_ns : 0ull;
    // the blocks' levels: the blocks level by level, each level's range
    if ((st = cuda_check((cudaError_t)launch_pgs_levels(pgs, nc, B.vout, wait_ns, stream), "pgs levels launch")))
        return st;
    ++launches;
    int32_t hl[2] = {0, 0};
    cudaMemcpyAsync(&hl[0], pgs.maxlev, sizeof(int32_t), cudaMemcpyDeviceToHost, stream);
    cudaMemcpyAsync(&hl[1], pgs.err, sizeof(int32_t), cudaMemcpyDeviceToHost, stream);
    if ((st = cuda_check(cudaStreamSynchronize(stream), "pgs levels"))) return st;
    if (hl[1] == 3) return fail(CDX_ERR_STATE, "pgs levels: the block chains made no progress");
    if (hl[1]) return fail(CDX_ERR_TIMEOUT, "pgs levels: a grid barrier wait ran out (gpu.coop_wait_ns)");
    last_levels = hl[0] + 1;
    if ((st = cuda_check((cudaError_t)launch_pgs_solve(sc, C, last_levels, B, pgs, B.vout, cfg.pj_relaxation, cfg.pj_alpha,
                                                       cfg.pj_tol_rel, cfg.pj_tol_abs, cfg.pj_max_iterations, ds,
                                                       wait_ns, stream),
                         "pgs solve launch")))
        return st;
    ++launches;
    // the result, the complementarity residual on the applied impulses, the stored impulses
    launch_cond_final(sc, C, gen, nc, B, x, -1, stream);
    launch_cond_final(sc, C, gen, nc, B, x, 1, stream);
    launch_sweep_contact64(sc, C, gen, nc, x, ds, 1, stream);
    launch_final_residual(ds, stream);
    launch_cond_final(sc, C, gen, nc, B, x, 0, stream);
    launches += 5;
    int32_t hflags[4] = {0, 0, 0, 0};
    int32_t herr = 0;
    cudaMemcpyAsync(hflags, B.flags, sizeof(hflags), cudaMemcpyDeviceToHost, stream);
    cudaMemcpyAsync(&herr, pgs.err, sizeof(int32_t), cudaMemcpyDeviceToHost, stream);
    if ((st = cuda_check(cudaStreamSynchronize(stream), "pgs solve"))) return st;
    if (herr)
        return fail(CDX_ERR_TIMEOUT, herr == 1 ? "pgs solve: a grid barrier wait ran out (gpu.coop_wait_ns)"
                                               : "pgs solve: a wait for a preceding block ran out (gpu.coop_wait_ns)");
    cond_diverged = hflags[0];
    return CDX_OK;
}
