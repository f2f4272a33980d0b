// Host side of the split-precision form: FP32 collision and projected Jacobi, FP64 state, final
// velocities and residual. The sweep loop runs as a CUDA graph with a device-side while node:
// the check kernel ends the loop at the iteration cap or when the complementarity residual
// reaches gpu.residual_tol, so a step needs no host round trip per sweep.
#include <algorithm>
#include <cstddef>
#include <cmath>
#include <cstring>
#include <vector>

#include "engine.h"
#include "split.h"

using namespace cdx;

namespace cdx {
struct SplitState {
    SplitBuf sb;
    int gen = 0;
    int prev_count = 0;
    int prev_n_static = 0;
    int nc = 0;
    int sms = 148;
    int32_t* h_nc = nullptr;  // pinned
    SplitScalars* h_ss = nullptr;
    cudaGraphExec_t exec[2] = {nullptr, nullptr};
    cudaGraph_t graph[2] = {nullptr, nullptr};
    int graph_blocks = 0;
    int graph_maxit = -1;
    float graph_tol = -1.f;
    int64_t graph_cap = -1;
    std::vector<void*> bufs;
    int last_iters = 0;
    double res_last = 0, res_final = 0;
    int variant = 0;         // contact-sweep launch shape (autotuned)
    int last_variant = 0;    // the shape that ran the last step
    int graph_variant = -1;
    int64_t tuned_at = 0;    // contact count at the last tuning
    int tune_runs = 0;
    int tune_cut = 0;        // tunings in a row that the solve's convergence cut short
    cudaEvent_t tev[2] = {nullptr, nullptr};
    // batched scenes: one block per scene
    int32_t* scene_order = nullptr;  // scene ids by decreasing body count (device)
    int scene_nbmax = 0;             // bodies of the largest scene
    int scene_best = -1;             // the fastest scenes shape once tuned (-2: the regular solver)
    int scene_tried = 0;
    int64_t scene_tuned_at = 0;      // contact count when the scenes shapes were last timed
    double scene_ms[16] = {0};
    int scene_timing = -1;           // shape timed in the current step
    // the scenes' alpha autotuner (gpu.tune_alpha): each scene's alpha, the best trial per scene,
    // each scene's sweeps and residual in the last solve, and the warm start kept for the trials
    float* scene_alpha = nullptr;
    float4* tune_best = nullptr;
    int4* scene_out = nullptr;
    int scene_bufs_n = 0;
    float4* lam_save = nullptr;
    int64_t lam_save_cap = 0;
    int64_t alpha_tuned_step = -1;
    int alpha_tunings = 0;
    // steps that find their contact totals on the device: a snapshot of the state they change, so
    // a step whose contacts outgrow the buffers or the plan can be undone and redone
    double* snap = nullptr;   // 13 N: position, quaternion, velocity, omega (body field order)
    double* ssnap = nullptr;  // 13 S: the same for the statics
    bool force_sync = false;
    int syncs = 0, redos = 0;
    // device-counted steps captured whole into a CUDA graph (one per generation), replayed while
    // the buffers, the solver shape and the cooperative plan stay the same
    cudaGraphExec_t sg_exec[2] = {nullptr, nullptr};
    long long sg_key[2][8] = {{0}};
    int64_t sg_launches[2] = {0, 0};  // kernels in each captured step
    bool sg_failed = false;
    CoopPlan gplan;
    bool gplan_ok = false;
    int64_t graph_steps = 0;
};
}  // namespace cdx

static int salloc(Engine& E, void** p, size_t bytes, const char* what) {
    int st = E.dalloc(p, bytes, what);
    if (!st) E.split->bufs.push_back(*p);
    return st;
}

static void destroy_step_graphs(SplitState* S) {
    for (int g = 0; g < 2; ++g) {
        if (S->sg_exec[g]) cudaGraphExecDestroy(S->sg_exec[g]);
        S->sg_exec[g] = nullptr;
    }
}

static void destroy_graphs(SplitState* S) {
    destroy_step_graphs(S);
    for (int g = 0; g < 2; ++g) {
        if (S->exec[g]) cudaGraphExecDestroy(S->exec[g]);
        if (S->graph[g]) cudaGraphDestroy(S->graph[g]);
        S->exec[g] = nullptr;
        S->graph[g] = nullptr;
    }
    S->graph_cap = -1;
}

// captured graphs hold the solver settings as kernel arguments, and the shapes were chosen for the
// old loop: after a configuration change they are rebuilt and the shapes chosen again
void Engine::split_config_changed() {
    if (!split) return;
    SplitState* S = split;
    destroy_graphs(S);
    S->gplan_ok = false;
    S->graph_variant = -1;
    S->variant = cfg.gpu_sweep_variant >= 0 ? std::min(cfg.gpu_sweep_variant, split_num_variants() - 1)
                                            : split_first_coop_variant();
    S->tuned_at = 0;
    S->scene_best = -1;
    S->scene_tried = 0;
    S->scene_tuned_at = 0;
    S->force_sync = true;
}

void Engine::destroy_split() {
    if (!split) return;
    destroy_graphs(split);
    for (auto& e : split->tev)
        if (e) cudaEventDestroy(e);
    for (void* p : split->bufs) dfree(p);
    if (split->h_nc) cudaFreeHost(split->h_nc);
    if (split->h_ss) cudaFreeHost(split->h_ss);
    delete split;
    split = nullptr;
}

// per-scene buffers of the alpha autotuner; a new scene count starts from the configured alpha
static int split_alpha_bufs(Engine& E) {
    SplitState* S = E.split;
    const int ns = std::max(E.sc.nscenes, 1);
    if (S->scene_bufs_n != ns) {
        int st;
        if ((st = salloc(E, (void**)&S->scene_alpha, sizeof(float) * ns, "scene alpha"))) return st;
        if ((st = salloc(E, (void**)&S->tune_best, sizeof(float4) * ns, "scene alpha"))) return st;
        if ((st = salloc(E, (void**)&S->scene_out, sizeof(int4) * ns, "scene alpha"))) return st;
        S->scene_bufs_n = ns;
        launch_s_tune_alpha(0, ns, (float)E.cfg.pj_alpha, nullptr, S->tune_best, nullptr, E.stream);
        launch_s_tune_alpha(2, ns, (float)E.cfg.pj_alpha, nullptr, S->tune_best, S->scene_alpha, E.stream);
        S->alpha_tuned_step = -1;
    }
    if (S->lam_save_cap < S->sb.cap) {
        int st;
        if ((st = salloc(E, (void**)&S->lam_save, sizeof(float4) * std::max<int64_t>(S->sb.cap, 1), "scene alpha")))
            return st;
        S->lam_save_cap = S->sb.cap;
        S->sb.lam_warm = S->lam_save;
        destroy_graphs(S);  // a captured step holds the old address
    }
    return CDX_OK;
}

// The scenes' alpha autotuner: trial solves of this step, from its warm start, with each candidate
// alpha; per scene the candidate that reaches gpu.residual_tol in the fewest sweeps (or, without a
// tolerance or when none reaches it, the lowest residual at the cap) is kept. Every alpha > 0 has
// the same fixed points (lambda = Pi(lambda - alpha D^-1 gamma) holds for all of them at a
// complementarity solution), so alpha changes how fast a scene converges, not what it converges to.
// The trial residuals are rescaled to the configured alpha, which the stop rule and the FP64
// residual keep using.
static int split_tune_alpha(Engine& E, int gen, int scene_v, int maxit, const int32_t* spos, const int32_t* sflags,
                            const int32_t* poff, int cblocks) {
    SplitState* S = E.split;
    SplitBuf& sb = S->sb;
    const int ns = std::max(E.sc.nscenes, 1);
    const int nc = S->nc;
    const float a0 = (float)E.cfg.pj_alpha;
    static const float cand[] = {0.2f, 0.3f, 0.4f, 0.5f, 0.6f, 0.7f, 0.85f, 1.0f};
    cudaMemcpyAsync(S->lam_save, sb.lam[gen], sizeof(float4) * (size_t)nc, cudaMemcpyDeviceToDevice, E.stream);
    launch_s_tune_alpha(0, ns, a0, nullptr, S->tune_best, nullptr, E.stream);
    auto trial = [&](float a, int ref) -> int {
        cudaMemcpyAsync(sb.lam[gen], S->lam_save, sizeof(float4) * (size_t)nc, cudaMemcpyDeviceToDevice, E.stream);
        launch_s_reset(sb, E.stream);
        launch_s_acc_init(sb, E.stream);
        launch_s_apply_warm(sb, gen, cblocks, E.stream);
        int st = launch_s_solve_scenes(E.sc, sb, gen, a, scene_v, maxit, (float)E.cfg.gpu_residual_tol, spos, sflags,
                                       poff, S->scene_order, S->scene_nbmax, E.stream, nullptr, a0, S->scene_out);
        if (st) return E.cuda_check((cudaError_t)st, "alpha trial solve");
        launch_s_tune_alpha(ref ? 3 : 1, ns, a, S->scene_out, S->tune_best, nullptr, E.stream);
        E.launches += 5;
        return CDX_OK;
    };
    int st;
    if ((st = trial(a0, 1))) return st;
    for (float a : cand)
        if (a != a0 && (st = trial(a, 0))) return st;
    // back to the step's own start
    cudaMemcpyAsync(sb.lam[gen], S->lam_save, sizeof(float4) * (size_t)nc, cudaMemcpyDeviceToDevice, E.stream);
    launch_s_reset(sb, E.stream);
    launch_s_acc_init(sb, E.stream);
    launch_s_apply_warm(sb, gen, cblocks, E.stream);
    launch_s_tune_alpha(2, ns, a0, nullptr, S->tune_best, S->scene_alpha, E.stream);
    E.launches += 4;
    S->alpha_tuned_step = E.steps;
    ++S->alpha_tunings;
    return E.cuda_check(cudaGetLastError(), "alpha tuning");
}

// the scenes' alpha and last sweeps (gpu.tune_alpha), for inspection
int Engine::scene_solve_info(float* alpha, int32_t* sweeps, int32_t n) {
    if (!split || !split->scene_alpha) return fail(CDX_ERR_STATE, "no per-scene solve has run");
    const int ns = std::min(n, split->scene_bufs_n);
    std::vector<int4> out(ns);
    if (alpha) cudaMemcpyAsync(alpha, split->scene_alpha, sizeof(float) * ns, cudaMemcpyDeviceToHost, stream);
    cudaMemcpyAsync(out.data(), split->scene_out, sizeof(int4) * ns, cudaMemcpyDeviceToHost, stream);
    int st = cuda_check(cudaStreamSynchronize(stream), "scene solve info");
    if (st) return st;
    if (sweeps)
        for (int i = 0; i < ns; ++i) sweeps[i] = out[i].x;
    return CDX_OK;
}

static int split_contacts(Engine& E, int64_t need) {
    SplitState* S = E.split;
    SplitBuf& b = S->sb;
    if (need <= b.cap) return CDX_OK;
    const int64_t cap = std::max<int64_t>(need + need / 4, 1024);
    SplitBuf n = b;
    n.cap = cap;
    int st;
    float4** f4[] = {&n.rec0, &n.rec1, &n.bias, &n.lam[0], &n.lam[1], &n.pt[0], &n.pt[1]};
    for (auto p : f4)
        if ((st = salloc(E, (void**)p, sizeof(float4) * cap, "split contacts"))) return st;
    if ((st = salloc(E, (void**)&n.key[0], sizeof(unsigned long long) * cap, "split contacts"))) return st;
    if ((st = salloc(E, (void**)&n.key[1], sizeof(unsigned long long) * cap, "split contacts"))) return st;
    if (E.cfg.pj_nesterov && (st = salloc(E, (void**)&n.lamk, sizeof(float4) * cap, "split contacts"))) return st;
    if (b.cap > 0 && S->prev_count > 0) {
        const int pg = S->gen ^ 1;
        cudaMemcpyAsync(n.key[pg], b.key[pg], sizeof(unsigned long long) * S->prev_count, cudaMemcpyDeviceToDevice, E.stream);
        cudaMemcpyAsync(n.lam[pg], b.lam[pg], sizeof(float4) * S->prev_count, cudaMemcpyDeviceToDevice, E.stream);
        cudaMemcpyAsync(n.pt[pg], b.pt[pg], sizeof(float4) * S->prev_count, cudaMemcpyDeviceToDevice, E.stream);
        if ((st = E.cuda_check(cudaStreamSynchronize(E.stream), "split grow"))) return st;
    }
    if (b.cap > 0) {
        void* old[] = {b.rec0, b.rec1, b.bias, b.lam[0], b.lam[1], b.pt[0], b.pt[1], b.key[0], b.key[1], b.lamk};
        for (void* p : old) {
            if (!p) continue;
            auto& v = S->bufs;
            v.erase(std::remove(v.begin(), v.end(), p), v.end());
            E.dfree(p);
        }
        ++E.reallocations;
    }
    b = n;
    destroy_graphs(S);
    return E.ensure_tmp(cap);
}

// The reference's loop controls that the split form honours, in its cooperative solve: 2 = Nesterov's
// loop (pj.nesterov), 1 = the standard loop with the velocity-increment exit (pj.tol_abs and
// pj.tol_rel not both 0), 0 = neither (every solver shape applies). pj.chebyshev and pj.anderson are
// refused when the engine is created; pj.rdiag_true_delassus needs nothing: for sphere contacts the
// Delassus blocks are diagonal, so the block preconditioner is the row scale R = alpha / D the sweep
// already uses.
static int split_loop(const cdx_config& c) {
    if (c.pj_nesterov) return 2;
    return (c.pj_tol_abs == 0.0 && c.pj_tol_rel == 0.0) ? 0 : 1;
}

// cooperative plan for n contacts under the context's gpu.coop_* keys
static bool coop_plan(const Engine& E, int v, int64_t n, CoopPlan* p) {
    return split_coop_plan(v, n, E.sc.N, E.split->sms, p, E.cfg.gpu_coop_smem_contacts, E.cfg.gpu_coop_blocks,
                           split_loop(E.cfg));
}

// Under the loop controls only the 1024-thread cooperative shapes run: the plain one while a block's
// contacts fit in shared memory, else the hybrid one. Returns the shape for n contacts, or -1.
static int loop_coop_variant(const Engine& E, int64_t n) {
    const int v0 = split_first_coop_variant();
    for (int v = v0; v < split_num_variants() && split_variant_is_coop(v); ++v) {
        CoopPlan p;
        if (coop_plan(E, v, std::max<int64_t>(n, 1), &p)) return v;
    }
    return -1;
}

// launches the cooperative solve of the configured loop
static int launch_coop(const Engine& E, const SplitBuf& sb, int gen, int v, const CoopPlan& plan, int max_iter,
                       float tol, int max_sweeps, cudaStream_t s) {
    const cdx_config& c = E.cfg;
    const int loop = split_loop(c);
    const unsigned long long wait_ns = c.gpu_coop_wait_ns > 0 ? (unsigned long long)c.gpu_coop_wait_ns : 0ull;
    if (!loop)
        return launch_s_solve_coop(sb, gen, (float)c.pj_alpha, v, plan, max_iter, tol, max_sweeps, c.gpu_check_every, s,
                                   wait_ns);
    CoopLoopArgs la = {};
    la.tol_abs = c.pj_tol_abs;
    la.tol_rel = c.pj_tol_rel;
    la.beta_threshold = c.pj_nesterov_beta_threshold;
    la.check_vel = (c.pj_tol_abs == 0.0 && c.pj_tol_rel == 0.0) ? 0 : 1;
    la.restart_limit = c.pj_nesterov_restart_limit;
    la.nv = 6 * E.sc.N;
    auto fits32 = [](double t) { return t >= 1e-12 && t <= 1e12; };
    if (c.pj_tol_rel == 0.0 && c.pj_tol_abs > 0.0)
        la.res_mode = 1;
    else if (c.pj_tol_abs == 0.0 && c.pj_tol_rel > 0.0)
        la.res_mode = 2;
    else if (fits32(c.pj_tol_abs) && fits32(c.pj_tol_rel))
        la.res_mode = 3;
    else
        la.res_mode = 0;
    return launch_s_solve_coop_loop(sb, gen, (float)c.pj_alpha, v, plan, max_iter, tol, max_sweeps, c.gpu_check_every,
                                    loop, la, wait_ns, s);
}

static int init_split(Engine& E) {
    E.split = new SplitState();
    SplitState* S = E.split;
    S->variant = E.cfg.gpu_sweep_variant >= 0 ? std::min(E.cfg.gpu_sweep_variant, split_num_variants() - 1)
                                              : split_first_coop_variant();
    SplitBuf& b = S->sb;
    const int N = E.sc.N, Ss = E.sc.S, nsc = E.sc.nscenes;
    b.N = N;
    int st;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&S->sms, cudaDevAttrMultiProcessorCount, dev);
    const size_t n1 = std::max(1, N);
    if ((st = salloc(E, (void**)&b.pos4, sizeof(float4) * n1, "split bodies"))) return st;
    if ((st = salloc(E, (void**)&b.pos64, sizeof(double4) * n1, "split bodies"))) return st;
    if ((st = salloc(E, (void**)&b.pos4lo, sizeof(float4) * n1, "split bodies"))) return st;
    if ((st = salloc(E, (void**)&b.plist, sizeof(int32_t) * SPLIT_PLIST * n1, "split bodies"))) return st;
    if ((st = salloc(E, (void**)&b.vel4, sizeof(float4) * 2 * n1, "split bodies"))) return st;
    for (int k = 0; k < SPLIT_NACC; ++k)
        if ((st = salloc(E, (void**)&b.acc[k], sizeof(float4) * 2 * n1, "split bodies"))) return st;
    if ((st = salloc(E, (void**)&b.vn4, sizeof(float4) * 2 * n1, "split bodies"))) return st;
    if ((st = salloc(E, (void**)&b.mat4, sizeof(float4) * n1, "split bodies"))) return st;
    if ((st = salloc(E, (void**)&b.vfree, sizeof(double) * 6 * n1, "split bodies"))) return st;
    if ((st = salloc(E, (void**)&b.acc64, sizeof(double) * 6 * n1, "split bodies"))) return st;
    if ((st = salloc(E, (void**)&b.origin, sizeof(double) * 3 * nsc, "split scenes"))) return st;
    const size_t s1 = std::max(1, Ss);
    float4** f4[] = {&b.st_dir, &b.st_pt, &b.st_v, &b.st_w};
    for (auto p : f4)
        if ((st = salloc(E, (void**)p, sizeof(float4) * s1, "split statics"))) return st;
    if ((st = salloc(E, (void**)&b.st_box, sizeof(float4) * 3 * s1, "split statics"))) return st;
    if ((st = salloc(E, (void**)&b.nc_dev, sizeof(int32_t), "split"))) return st;
    if ((st = salloc(E, (void**)&b.ss, sizeof(SplitScalars), "split"))) return st;
    if ((st = salloc(E, (void**)&b.part, sizeof(float2) * SPLIT_MAX_PARTS, "split"))) return st;
    if ((st = salloc(E, (void**)&b.recs, sizeof(float2) * 2 * SPLIT_MAX_PARTS, "split"))) return st;
    if ((st = salloc(E, (void**)&b.sums, sizeof(double2) * 2 * SPLIT_MAX_PARTS, "split"))) return st;
    if ((st = salloc(E, (void**)&S->snap, sizeof(double) * 13 * n1, "split snapshot"))) return st;
    if ((st = salloc(E, (void**)&S->ssnap, sizeof(double) * 13 * s1, "split snapshot"))) return st;
    {
        // batched scenes: largest first, so the longest solves start first
        std::vector<int32_t> order(nsc);
        for (int q = 0; q < nsc; ++q) order[q] = q;
        const std::vector<int32_t>& bs = E.h_scene_body_start;
        auto size = [&](int q) { return bs.size() > (size_t)q + 1 ? bs[q + 1] - bs[q] : 0; };
        std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return size(x) > size(y); });
        S->scene_nbmax = nsc > 0 ? size(order[0]) : 0;
        if ((st = salloc(E, (void**)&S->scene_order, sizeof(int32_t) * std::max(nsc, 1), "split scenes"))) return st;
        if ((st = E.cuda_check(cudaMemcpy(S->scene_order, order.data(), sizeof(int32_t) * nsc, cudaMemcpyHostToDevice),
                               "scene order")))
            return st;
    }
    if ((st = E.cuda_check(cudaMallocHost((void**)&S->h_nc, sizeof(int32_t)), "pinned"))) return st;
    if ((st = E.cuda_check(cudaMallocHost((void**)&S->h_ss, sizeof(SplitScalars)), "pinned"))) return st;
    cudaMemsetAsync(b.ss, 0, sizeof(SplitScalars), E.stream);
    cudaMemsetAsync(b.nc_dev, 0, sizeof(int32_t), E.stream);
    // scene origins: centroid of each scene's bodies (FP32 coordinates stay small)
    std::vector<double> B((size_t)BF_COUNT * N), org(3 * (size_t)nsc, 0.0);
    if (N) {
        if ((st = E.cuda_check(cudaMemcpy(B.data(), E.sc.B, sizeof(double) * B.size(), cudaMemcpyDeviceToHost), "origins"))) return st;
    }
    for (int i = 0; i < N && !b.has_restitution; ++i)
        if (B[(size_t)BF_RN * N + i] > 0 || B[(size_t)BF_RT * N + i] > 0) b.has_restitution = 1;
    if (N) {
        std::vector<float4> mat(N);
        for (int i = 0; i < N; ++i)
            mat[i] = make_float4((float)B[(size_t)BF_MU * N + i], (float)B[(size_t)BF_RN * N + i],
                                 (float)B[(size_t)BF_RT * N + i], 0.f);
        if ((st = E.cuda_check(cudaMemcpy(b.mat4, mat.data(), sizeof(float4) * N, cudaMemcpyHostToDevice), "materials")))
            return st;
    }
    if (Ss > 0) {
        std::vector<double> St((size_t)SF_COUNT * Ss);
        if ((st = E.cuda_check(cudaMemcpy(St.data(), E.sc.St, sizeof(double) * St.size(), cudaMemcpyDeviceToHost), "statics"))) return st;
        for (int i = 0; i < Ss && !b.has_restitution; ++i)
            if (St[(size_t)SF_RN * Ss + i] > 0 || St[(size_t)SF_RT * Ss + i] > 0) b.has_restitution = 1;
    }
    for (int s = 0; s < nsc; ++s) {
        const int b0 = E.h_scene_body_start[s], b1 = E.h_scene_body_start[s + 1];
        for (int k = 0; k < 3; ++k) {
            double acc = 0;
            for (int i = b0; i < b1; ++i) acc += B[(size_t)(BF_PX + k) * N + i];
            org[3 * s + k] = b1 > b0 ? std::round(acc / (b1 - b0) * 64.0) / 64.0 : 0.0;
        }
    }
    if ((st = E.cuda_check(cudaMemcpy(b.origin, org.data(), sizeof(double) * org.size(), cudaMemcpyHostToDevice), "origins"))) return st;
    const int64_t cap0 = std::max<int64_t>(1024, (int64_t)(E.cfg.gpu_contact_capacity_factor * std::max(1, N)));
    return split_contacts(E, cap0);
}

static int build_graph(Engine& E, int g) {
    SplitState* S = E.split;
    const int maxit = std::max(1, E.cfg.pj_max_iterations);
    const float tol = (float)E.cfg.gpu_residual_tol;
    cudaGraph_t graph;
    int st;
    if ((st = E.cuda_check(cudaGraphCreate(&graph, 0), "graph create"))) return st;
    cudaGraphConditionalHandle h;
    if ((st = E.cuda_check(cudaGraphConditionalHandleCreate(&h, graph, 1, cudaGraphCondAssignDefault), "cond handle"))) return st;
    alignas(cudaGraphNodeParams) unsigned char pbuf[sizeof(cudaGraphNodeParams)];
    std::memset(pbuf, 0, sizeof(pbuf));
    cudaGraphNodeParams& p = *reinterpret_cast<cudaGraphNodeParams*>(pbuf);
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = h;
    p.conditional.type = cudaGraphCondTypeWhile;
    p.conditional.size = 1;
    cudaGraphNode_t node;
    if ((st = E.cuda_check(cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &p), "cond node"))) return st;
    cudaGraph_t body = p.conditional.phGraph_out[0];
    if ((st = E.cuda_check(cudaStreamBeginCaptureToGraph(E.stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed),
                           "capture"))) return st;
    launch_s_sweep(S->sb, g, (float)E.cfg.pj_alpha, S->graph_variant, S->graph_blocks, maxit, tol, h, 1, E.stream);
    cudaGraph_t captured = nullptr;
    if ((st = E.cuda_check(cudaStreamEndCapture(E.stream, &captured), "end capture"))) return st;
    if ((st = E.cuda_check(cudaGraphInstantiate(&S->exec[g], graph, 0), "graph instantiate"))) return st;
    S->graph[g] = graph;
    return CDX_OK;
}

int Engine::step_split() {
    int st;
    if (!split && (st = init_split(*this))) return st;
    SplitState* S = split;
    SplitBuf& sb = S->sb;
    const int N = sc.N;
    const double dt = cfg.sim_dt, th = cfg.moreau_theta;
    SplitParams P;
    P.alpha = (float)cfg.pj_alpha;
    P.margin = (float)cfg.collision_security_margin;
    P.margin64 = cfg.collision_security_margin;
    P.match2 = (float)(cfg.collision_match_max_dist * cfg.collision_match_max_dist);
    P.combine = cfg.friction_combine;
    P.friction_enable = cfg.friction_enable;
    P.prev_count = cfg.pj_warmstart ? S->prev_count : 0;
    P.prev_sflags = sflags_prev;
    P.prev_spos = spos_prev;
    P.prev_poff = poff_prev;
    P.prev_n_static = S->prev_n_static;
    const int gen = S->gen;
    const int maxit = std::max(1, cfg.pj_max_iterations);
    const int pinned = cfg.gpu_sweep_variant;

    // Once a step has sized the buffers, the next steps find their contact totals on the device and
    // run to the end without stopping for the host: buffers and the cooperative plan come from the
    // previous count with a margin. Steps that tune (timing needs the host) stay synchronous, and a
    // step whose contacts outgrow the buffers or the plan is undone from a snapshot and redone
    // synchronously.
    // under the reference's loop controls only the cooperative solve runs (nothing to tune)
    const int loopk = split_loop(cfg);
    if (loopk && pinned < 0) {
        const int v = loop_coop_variant(*this, (int64_t)S->prev_count + S->prev_count / 16 + 64);
        S->variant = v >= 0 ? v : split_first_coop_variant();
    }
    auto tune_due = [&](int64_t n) {
        if (!(n > 0 && !loopk && cfg.gpu_autotune && pinned < 0 && n >= 4096 &&
              (double)n >= 1.5 * (double)S->tuned_at))
            return false;
        // the same count as the tuner's below
        const int k = maxit >= 1000 ? 40 : 12;
        int sweeps = 0;
        for (int v = 0; v < split_num_variants(); ++v) {
            CoopPlan probe;
            if (split_variant_is_coop(v))
                sweeps += coop_plan(*this, v, n, &probe) ? k : 0;
            else if (!split_variant_is_scenes(v))
                sweeps += 2;
        }
        const int expect = S->last_iters > 0 ? S->last_iters : maxit;
        return maxit > 2 * sweeps && expect > 2 * sweeps;
    };
    // the per-scene kernel (one block a scene) is a candidate for batches and for a single scene
    // small enough that one block can carry it
    const bool scene_fit = !loopk && S->scene_nbmax > 0 && S->scene_nbmax <= 3584;
    // shapes timed while the scenes had few contacts (a pile that is still falling) say little about
    // the settled problem: time them again once the count has grown by half
    if (scene_fit && pinned < 0 && cfg.gpu_autotune && S->scene_best != -1 && S->prev_count >= 64 &&
        (double)S->prev_count >= 1.5 * (double)S->scene_tuned_at) {
        S->scene_best = -1;
        S->scene_tried = 0;
    }
    const bool scene_tuning = scene_fit && pinned < 0 && S->scene_best == -1 && cfg.gpu_autotune;
    // the scenes' alpha is tuned on the first step of the scenes kernel and then every
    // gpu.tune_alpha_every steps (trial solves need the true contact count: a synchronous step)
    const bool scenes_chosen = pinned >= 0 ? split_variant_is_scenes(pinned) : (cfg.gpu_autotune ? S->scene_best >= 0 : true);
    const bool alpha_due = scene_fit && scenes_chosen && cfg.gpu_tune_alpha &&
                           (S->alpha_tuned_step < 0 || steps - S->alpha_tuned_step >= cfg.gpu_tune_alpha_every);
    const bool async = !cfg.gpu_sync_counts && S->prev_count > 0 && sb.cap > 0 && !S->force_sync && !scene_tuning &&
                       !tune_due(S->prev_count) && !alpha_due;
    S->force_sync = false;
    if (async) {
        // the warm-start layout of the last step is read on the device
        if (cfg.pj_warmstart) P.prev_count = -1;
        P.prev_n_static = -1;
    }
    // A device-counted step whose solver is the cooperative or the batched-scenes kernel is
    // captured whole (snapshot to the final scalars) into a CUDA graph and replayed.
    const bool multi0 = scene_fit;
    const bool scenes0 = async && multi0 && (pinned >= 0 ? split_variant_is_scenes(pinned) : S->scene_best >= 0);
    bool use_graph = async && cfg.gpu_use_graph && !timing && !S->sg_failed;
    if (use_graph && !scenes0) {
        // the cooperative plan is kept while it holds the estimate (the kernel balances its blocks
        // by the true count), so the graph stays valid across steps
        const int64_t est = (int64_t)S->prev_count + S->prev_count / 16 + 64;
        if (!split_variant_is_coop(S->variant)) {
            use_graph = false;
        } else if (!(S->gplan_ok && (int64_t)S->gplan.cpb * S->gplan.grid >= est)) {
            S->gplan_ok = coop_plan(*this, S->variant, est + est / 4, &S->gplan) ||
                          coop_plan(*this, S->variant, est, &S->gplan);
            if (!S->gplan_ok) use_graph = false;
        }
    }
    const long long gkey[8] = {(long long)sb.cap, (long long)S->variant, scenes0 ? 1 : 0, S->gplan.cpb, S->gplan.bpb,
                               S->gplan.vf, S->gplan.smem,
                               (long long)cfg.pj_warmstart | ((long long)(cfg.gpu_tune_alpha != 0) << 1)};
    bool capturing = false;
    int64_t launches0 = launches;
    int64_t n_static = 0;
    bool coop = false, scenes = false, multi = false;
    const int nsv = split_num_scenes_variants();
    if (use_graph && S->sg_exec[gen] && std::memcmp(gkey, S->sg_key[gen], sizeof(gkey)) == 0) {
        // replay the captured step
        if ((st = cuda_check(cudaGraphLaunch(S->sg_exec[gen], stream), "step graph launch"))) return st;
        ++S->graph_steps;
        ++S->syncs;
        S->nc = S->prev_count;
        scenes = scenes0;
        coop = !scenes0;
        launches += S->sg_launches[gen];
        goto step_issued;
    }
    if (use_graph) {
        if (S->sg_exec[gen]) {
            cudaGraphExecDestroy(S->sg_exec[gen]);
            S->sg_exec[gen] = nullptr;
        }
        if (cudaStreamBeginCapture(stream, cudaStreamCaptureModeRelaxed) == cudaSuccess)
            capturing = true;
        else {
            cudaGetLastError();
            S->sg_failed = true;
        }
    }
  {
    // ends a capture left open by an early error return
    struct CaptureGuard {
        cudaStream_t s;
        bool* on;
        ~CaptureGuard() {
            if (*on) {
                cudaGraph_t g = nullptr;
                cudaStreamEndCapture(s, &g);
                if (g) cudaGraphDestroy(g);
                cudaGetLastError();
            }
        }
    } guard{stream, &capturing};
    if (async) {
        cudaMemcpyAsync(S->snap, sc.B, sizeof(double) * 13 * (size_t)N, cudaMemcpyDeviceToDevice, stream);
        if (sc.S > 0)
            cudaMemcpyAsync(S->ssnap, sc.St, sizeof(double) * 13 * (size_t)sc.S, cudaMemcpyDeviceToDevice, stream);
        ++S->syncs;
    }

    if (timing) cudaEventRecord(ev[0], stream);
    launch_s_prep(sc, sb, dt, cfg.sim_gravity, (1.0 - th) * dt, stream, cfg.moreau_implicit_gyroscopy,
                  sc.S > 0 ? smot : nullptr, sc.S > 0 ? smflag : nullptr);
    launch_cell_keys(sc, grid, cell_key_in, cell_val_in, stream, 1);
    if ((st = cuda_check(sort_pairs(tmp, tmp_bytes, cell_key_in, cell_key_out, cell_val_in, cell_val_out, N,
                                    grid.key_bits, stream), "sort cells"))) return st;
    cudaMemsetAsync(cell_start, 0, sizeof(int32_t) * grid.ncells, stream);
    cudaMemsetAsync(cell_end, 0, sizeof(int32_t) * grid.ncells, stream);
    launch_ranges(cell_key_out, N, cell_start, cell_end, stream);
    launches += 8;
    const int64_t nflag = (int64_t)N * sc.max_statics;
    if (nflag > 0) {
        launch_s_static_flags(sc, sb, P.margin, P.margin64, sflags, stream);
        if ((st = cuda_check(exclusive_scan(tmp, tmp_bytes, sflags, spos, nflag, stream), "scan"))) return st;
        launches += 3;
    }
    launch_s_pair_count(sc, grid, sb, cell_val_out, cell_key_out, cell_start, cell_end, pcount, P, ds, stream);
    if ((st = cuda_check(exclusive_scan(tmp, tmp_bytes, pcount, poff, N + 1, stream), "scan"))) return st;
    launches += 3;
    int64_t n_pair = 0;
    if (async) {
        launch_s_totals(sb, spos, sflags, nflag, poff, N, stream);
        S->nc = S->prev_count;  // an estimate for the launch shapes; the device holds the count
        if (nflag > 0) launch_s_static_write(sc, sb, sflags, spos, gen, P, stream);
        launch_s_pair_write(sc, grid, sb, cell_val_out, cell_key_out, cell_start, cell_end, poff, -1, gen, P, ds, stream);
        launches += 3;
    } else {
        int32_t tot[4] = {0, 0, 0, 0};
        if (nflag > 0) {
            cudaMemcpyAsync(&tot[0], spos + nflag - 1, sizeof(int32_t), cudaMemcpyDeviceToHost, stream);
            cudaMemcpyAsync(&tot[1], sflags + nflag - 1, sizeof(int32_t), cudaMemcpyDeviceToHost, stream);
        }
        cudaMemcpyAsync(&tot[2], poff + N, sizeof(int32_t), cudaMemcpyDeviceToHost, stream);
        cudaMemcpyAsync(&tot[3], &ds->overflow, sizeof(int32_t), cudaMemcpyDeviceToHost, stream);
        if ((st = cuda_check(cudaStreamSynchronize(stream), "collision counts"))) return st;
        if (tot[3]) return fail(CDX_ERR_OVERFLOW, "a sphere touches more than 64 higher-index spheres");
        n_static = (int64_t)tot[0] + tot[1];
        n_pair = tot[2];
        if ((st = split_contacts(*this, n_static + n_pair))) return st;
        S->nc = (int)(n_static + n_pair);
        launch_s_totals(sb, spos, sflags, nflag, poff, N, stream);
        ++launches;
        if (nflag > 0 && n_static > 0) {
            launch_s_static_write(sc, sb, sflags, spos, gen, P, stream);
            ++launches;
        }
        if (n_pair > 0) {
            launch_s_pair_write(sc, grid, sb, cell_val_out, cell_key_out, cell_start, cell_end, poff, (int32_t)n_static, gen, P, ds,
                                stream);
            ++launches;
        }
    }
    if (timing) cudaEventRecord(ev[1], stream);
    // x0 = v_free + M^-1 W^T lambda_warm (a captured step sizes its grids by the capacity)
    const int cblocks = split_grid_blocks(capturing ? std::max<int64_t>(sb.cap, 1) : std::max(S->nc, 1), S->sms);
    launch_s_reset(sb, stream);
    launch_s_apply_warm(sb, gen, cblocks, stream);
    launches += 2;
    if (timing) cudaEventRecord(ev[2], stream);
    bool solved = false;
    // batched scenes: every scene solved by its own block. Untuned, successive steps try every
    // scenes shape and then the regular solver (one step for its own tuning, one timed), one full
    // solve each, and the fastest is kept.
    multi = S->nc > 0 && multi0;
    scenes = false;
    int scene_v = -1;
    S->scene_timing = -1;
    if (multi) {
        if (pinned >= 0) {
            scenes = split_variant_is_scenes(pinned);
            scene_v = pinned;
        } else if (S->scene_best != -1) {
            scenes = S->scene_best >= 0;
            scene_v = S->scene_best;
        } else if (cfg.gpu_autotune) {
            const int trial = S->scene_tried;  // 0..nsv-1 scenes shapes, nsv and nsv+1 the regular solver
            scenes = trial < nsv;
            scene_v = scenes ? split_first_scenes_variant() + trial : -2;
            if (trial != nsv) S->scene_timing = trial;
        } else {
            scenes = true;
            scene_v = split_first_scenes_variant();
        }
    }
    if (S->scene_timing >= 0) {
        if (!S->tev[0]) {
            cudaEventCreate(&S->tev[0]);
            cudaEventCreate(&S->tev[1]);
        }
        cudaEventRecord(S->tev[0], stream);
    }
    if (scenes) {
        float* salpha = nullptr;
        if ((st = split_alpha_bufs(*this))) return st;
        if (cfg.gpu_tune_alpha) {
            if (alpha_due && !capturing && !async) {
                if ((st = split_tune_alpha(*this, gen, scene_v, maxit, nflag > 0 ? spos : nullptr,
                                           nflag > 0 ? sflags : nullptr, poff, cblocks)))
                    return st;
            }
            salpha = S->scene_alpha;
        }
        st = launch_s_solve_scenes(sc, sb, gen, (float)cfg.pj_alpha, scene_v, maxit, (float)cfg.gpu_residual_tol,
                                   nflag > 0 ? spos : nullptr, nflag > 0 ? sflags : nullptr, poff, S->scene_order,
                                   S->scene_nbmax, stream, salpha, (float)cfg.pj_alpha, S->scene_out);
        if ((st = cuda_check((cudaError_t)st, "scenes solve"))) return st;
        S->last_variant = scene_v;
        ++launches;
        solved = true;
    }
    const int nv = split_num_variants();
    // sweeps the autotuner spends: two per streaming shape, and per feasible cooperative one a
    // launch of k0 and one of k1 sweeps (their difference times a sweep); a solve of a thousand
    // sweeps or more times 32 sweeps of difference instead of 8, where the shapes' per-sweep costs
    // (a few percent apart) decide its time and 8 sweeps measured them within the noise
    const int coop_k0 = maxit >= 1000 ? 4 : 2, coop_k1 = maxit >= 1000 ? 36 : 10;
    int tune_sweeps = 0;
    for (int v = 0; v < nv; ++v) {
        CoopPlan probe;
        if (split_variant_is_coop(v))
            tune_sweeps += (S->nc > 0 && coop_plan(*this, v, S->nc, &probe)) ? coop_k0 + coop_k1 : 0;
        else if (!split_variant_is_scenes(v))
            tune_sweeps += 2;
    }
    // the trials are the step's first sweeps: a solve expected to end sooner (the previous step's
    // sweeps, or the cap on a first step) waits for a step that needs enough of them
    const int expect = S->last_iters > 0 ? S->last_iters : maxit;
    if (!async && !scenes && !loopk && S->nc > 0 && cfg.gpu_autotune && cfg.gpu_sweep_variant < 0 && S->nc >= 4096 &&
        (double)S->nc >= 1.5 * (double)S->tuned_at && maxit > 2 * tune_sweeps && expect > 2 * tune_sweeps) {
        // autotune: the first sweeps of this step run with every shape; each is a full sweep of
        // the same math, so the step's result does not depend on which shape ran them
        if (!S->tev[0]) {
            cudaEventCreate(&S->tev[0]);
            cudaEventCreate(&S->tev[1]);
        }
        double best_t = 1e300;
        int best = S->variant;
        cudaGraphConditionalHandle none = 0;
        for (int v = 0; v < nv && !solved; ++v) {
            double t = 0;
            if (split_variant_is_scenes(v)) continue;
            if (split_variant_is_coop(v)) {
                // two launches of 2 and 10 sweeps: their difference is the cost of a sweep, the rest
                // (loading and storing the contacts) is paid once per solve of maxit sweeps (the
                // shapes differ by a few percent a sweep: 8 sweeps of difference keep that above
                // the noise of one measurement)
                CoopPlan plan;
                if (!coop_plan(*this, v, S->nc, &plan)) continue;
                float ms[2] = {0.f, 0.f};
                const int ks[2] = {coop_k0, coop_k1};
                for (int r = 0; r < 2; ++r) {
                    cudaEventRecord(S->tev[0], stream);
                    st = launch_coop(*this, sb, gen, v, plan, maxit, (float)cfg.gpu_residual_tol, ks[r], stream);
                    if ((st = cuda_check((cudaError_t)st, "cooperative launch"))) return st;
                    cudaEventRecord(S->tev[1], stream);
                    if ((st = cuda_check(cudaEventSynchronize(S->tev[1]), "autotune"))) return st;
                    cudaEventElapsedTime(&ms[r], S->tev[0], S->tev[1]);
                    ++launches;
                }
                const double per = std::max(0.0, (double)(ms[1] - ms[0]) / (ks[1] - ks[0]));
                const double fixed = std::max(0.0, (double)ms[0] - ks[0] * per);
                t = 2.0 * (per + fixed / maxit);
            } else {
                for (int r = 0; r < 2; ++r) {
                    const int vb = split_contact_blocks(v, S->nc, S->sms);
                    cudaEventRecord(S->tev[0], stream);
                    launch_s_sweep(sb, gen, (float)cfg.pj_alpha, v, vb, maxit, (float)cfg.gpu_residual_tol, none, 0,
                                   stream);
                    cudaEventRecord(S->tev[1], stream);
                    if ((st = cuda_check(cudaEventSynchronize(S->tev[1]), "autotune"))) return st;
                    float ms1 = 0;
                    cudaEventElapsedTime(&ms1, S->tev[0], S->tev[1]);
                    t += ms1;
                }
                launches += 2;
            }
            cudaMemcpyAsync(&S->h_ss->done, &sb.ss->done, sizeof(int32_t), cudaMemcpyDeviceToHost, stream);
            if ((st = cuda_check(cudaStreamSynchronize(stream), "autotune"))) return st;
            solved = S->h_ss->done != 0;
            // a trial during which the solve met its stop rule ran fewer sweeps than it timed: it
            // does not count, and the shapes after it were not timed
            if (solved) break;
            if (t < best_t) {
                best_t = t;
                best = v;
            }
        }
        // the solve ended inside the trials (a warm-started step needing few sweeps): keep the
        // current shape, time them all again on a later step that needs enough sweeps, and after
        // four such cuts stop trying at this contact count
        bool all = true;
        if (solved) {
            all = ++S->tune_cut >= 4;
        } else {
            S->variant = best;
            S->last_variant = best;
        }
        if (all) {
            S->tuned_at = S->nc;
            S->tune_cut = 0;
            ++S->tune_runs;
        }
    }
    CoopPlan plan;
    const int64_t plan_nc = async ? (int64_t)S->nc + S->nc / 16 + 64 : (int64_t)S->nc;
    if (loopk && !capturing && pinned < 0 && S->nc > 0) {
        // the loop controls run in the cooperative solve only: the plain shape, or the hybrid one
        // once a block's contacts outgrow its shared memory
        const int v = loop_coop_variant(*this, plan_nc);
        if (v >= 0) S->variant = v;
    }
    if (capturing && !scenes && split_variant_is_coop(S->variant)) plan = S->gplan;
    coop = !scenes && S->nc > 0 && split_variant_is_coop(S->variant) &&
           (capturing ? S->gplan_ok : coop_plan(*this, S->variant, plan_nc, &plan));
    if (loopk && S->nc > 0 && !coop)
        return fail(CDX_ERR_UNSUPPORTED, "pj.nesterov and pj.tol_abs/pj.tol_rel run in the cooperative solve of the "
                                         "split form, which cannot be launched here (gpu.sweep_variant must name a "
                                         "1024-thread cooperative shape)");
    if (S->nc > 0 && !solved && coop) {
        st = launch_coop(*this, sb, gen, S->variant, plan, maxit, (float)cfg.gpu_residual_tol, maxit, stream);
        if (st != 0 && capturing) {
            // a cooperative launch that cannot be captured: nothing of the step ran; end the capture
            // and issue steps directly from now on
            cudaGraph_t g = nullptr;
            cudaStreamEndCapture(stream, &g);
            if (g) cudaGraphDestroy(g);
            cudaGetLastError();
            capturing = false;
            S->sg_failed = true;
            return step_split();
        }
        S->last_variant = S->variant;
        if ((st = cuda_check((cudaError_t)st, "cooperative launch"))) return st;
        ++launches;
    } else if (S->nc > 0 && !solved) {
        // streaming sweeps (a cooperative or batched shape that does not apply runs as streaming shape 0)
        const int sv = (split_variant_is_coop(S->variant) || split_variant_is_scenes(S->variant)) ? 0 : S->variant;
        S->last_variant = sv;
        const int sblocks = split_contact_blocks(sv, std::max(S->nc, 1), S->sms);
        if (cfg.gpu_use_graph) {
            // grid sized for the capacity so a graph serves every step until the buffers grow
            const int gblocks = split_contact_blocks(sv, sb.cap, S->sms);
            const float tol = (float)cfg.gpu_residual_tol;
            if (S->graph_cap != sb.cap || S->graph_maxit != maxit || S->graph_tol != tol || S->graph_variant != sv) {
                destroy_graphs(S);
                S->graph_variant = sv;
                S->graph_blocks = gblocks;
                if ((st = build_graph(*this, 0)) || (st = build_graph(*this, 1))) return st;
                S->graph_cap = sb.cap;
                S->graph_maxit = maxit;
                S->graph_tol = tol;
            }
            if ((st = cuda_check(cudaGraphLaunch(S->exec[gen], stream), "graph launch"))) return st;
        } else {
            const int every = std::max(1, cfg.gpu_check_every);
            cudaGraphConditionalHandle none = 0;
            for (int it = 0; it < maxit; ++it) {
                if (it > 0 && it % every == 0) {
                    cudaMemcpyAsync(&S->h_ss->done, &sb.ss->done, sizeof(int32_t), cudaMemcpyDeviceToHost, stream);
                    if ((st = cuda_check(cudaStreamSynchronize(stream), "poll"))) return st;
                    if (S->h_ss->done) break;
                }
                launch_s_sweep(sb, gen, (float)cfg.pj_alpha, sv, sblocks, maxit, (float)cfg.gpu_residual_tol, none, 0,
                               stream);
            }
        }
    }
    if (S->scene_timing >= 0) cudaEventRecord(S->tev[1], stream);
    if (timing) cudaEventRecord(ev[3], stream);
    // FP64: final velocities, residual, write back, drift theta h
    launch_s_final(sc, sb, gen, cfg.pj_alpha, cfg.friction_enable, cfg.friction_combine, cblocks, th * dt, stream);
    launches += 4;
    if (timing) cudaEventRecord(ev[4], stream);
    launch_s_end_step(sb, ds, stream);
    ++launches;
    cudaMemcpyAsync(S->h_ss, sb.ss, sizeof(SplitScalars), cudaMemcpyDeviceToHost, stream);
    if (capturing) {
        cudaGraph_t g = nullptr;
        capturing = false;
        cudaError_t e = cudaStreamEndCapture(stream, &g);
        cudaGraphExec_t x = nullptr;
        if (e == cudaSuccess) e = cudaGraphInstantiate(&x, g, 0);
        if (g) cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            // the step could not be captured (nothing of it ran): issue it directly from now on
            cudaGetLastError();
            S->sg_failed = true;
            return step_split();
        }
        S->sg_exec[gen] = x;
        std::memcpy(S->sg_key[gen], gkey, sizeof(gkey));
        S->sg_launches[gen] = launches - launches0;
        if ((st = cuda_check(cudaGraphLaunch(x, stream), "step graph launch"))) return st;
        ++S->graph_steps;
    }
  }
step_issued:
    if ((st = cuda_check(cudaStreamSynchronize(stream), "split step"))) return st;
    if ((st = cuda_check(cudaGetLastError(), "split launch"))) return st;
    if (S->h_ss->pair_overflow) return fail(CDX_ERR_OVERFLOW, "a sphere touches more than 64 higher-index spheres");
    if (async && (S->h_ss->cap_err || S->h_ss->err == 4)) {
        // undo the step (state from the snapshot; everything else is rebuilt) and redo it synchronously
        cudaMemcpyAsync(sc.B, S->snap, sizeof(double) * 13 * (size_t)N, cudaMemcpyDeviceToDevice, stream);
        if (sc.S > 0)
            cudaMemcpyAsync(sc.St, S->ssnap, sizeof(double) * 13 * (size_t)sc.S, cudaMemcpyDeviceToDevice, stream);
        if ((st = cuda_check(cudaStreamSynchronize(stream), "undo step"))) return st;
        ++S->redos;
        S->force_sync = true;
        if (S->h_ss->err == 4) S->gplan_ok = false;
        return step_split();
    }
    if (S->h_ss->err) return fail(CDX_ERR_TIMEOUT, "cooperative solve: a grid barrier timed out");
    if (async) {
        S->nc = S->h_ss->n_total;
        n_static = S->h_ss->n_static;
    }
    S->last_iters = S->nc > 0 ? S->h_ss->iters : 0;
    if (!coop && !scenes) launches += (int64_t)S->last_iters;
    if (multi && pinned < 0 && S->scene_best == -1 && cfg.gpu_autotune) {
        const int trial = S->scene_tried++;
        if (S->scene_timing >= 0) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, S->tev[0], S->tev[1]);
            S->scene_ms[trial] = ms;
        }
        if (S->scene_tried > nsv + 1) {
            int best = 0;
            for (int q = 1; q <= nsv + 1; ++q)
                if (q != nsv && S->scene_ms[q] < S->scene_ms[best]) best = q;
            S->scene_best = best < nsv ? split_first_scenes_variant() + best : -2;
            S->scene_tuned_at = std::max<int64_t>(S->nc, 1);
            ++S->tune_runs;
        }
    }
    S->res_last = S->h_ss->res_last;
    S->res_final = S->nc > 0 ? S->h_ss->res_final : 0.0;
    S->prev_count = S->nc;
    S->prev_n_static = (int)n_static;
    S->gen ^= 1;
    std::swap(sflags, sflags_prev);
    std::swap(spos, spos_prev);
    std::swap(poff, poff_prev);
    // mirror into the common stats fields
    prev_count = S->nc;
    contacts_loaded = false;
    last_iters = S->last_iters;
    last_rows = 3 * S->nc;
    last_res = S->res_last;
    last_res_final = S->res_final;
    ++steps;
    if (timing) {
        float a = 0, b = 0, c2 = 0, d = 0;
        cudaEventElapsedTime(&a, ev[0], ev[1]);
        cudaEventElapsedTime(&b, ev[1], ev[2]);
        cudaEventElapsedTime(&c2, ev[2], ev[3]);
        cudaEventElapsedTime(&d, ev[3], ev[4]);
        ms[0] = a; ms[1] = b; ms[2] = c2; ms[3] = d;
    }
    // a state that is no longer finite ends the step with an error (the step completed; the context
    // stays usable and cdx_set_state can repair the state)
    if (S->h_ss->nonfinite) return fail(CDX_ERR_NONFINITE, "the state after the step is not finite (NaN or infinity)");
    return CDX_OK;
}

// The warm-start memory of the split form: the previous step's contacts in its own layout (static
// contacts by scene, static slot and sphere; pair contacts grouped by their lower sphere, ascending)
// with the slot tables its narrow phase reads for the O(1) lookup. `order` sorts the input by pair.
int Engine::set_contacts_split(const std::vector<int64_t>& order, const int32_t* ia, const int32_t* ib,
                               const double* point, const double* lambda) {
    int st;
    if (!split && (st = init_split(*this))) return st;
    SplitState* S = split;
    const int n = (int)order.size(), N = sc.N, Sn = sc.S, L = sc.max_statics;
    if ((st = split_contacts(*this, std::max(n, 1)))) return st;
    SplitBuf& sb = S->sb;
    const size_t nflag = (size_t)N * L;
    std::vector<int32_t> flags(std::max<size_t>(nflag, 1), 0), spos(std::max<size_t>(nflag, 1), 0), cnt(N + 1, 0);
    std::vector<size_t> slot_of(n, 0);
    int nstat = 0;
    for (int c = 0; c < n; ++c) {
        const int64_t o = order[c];
        const int a = ia[o], bi = ib[o] - Sn;
        const int scn = h_body_scene_of(bi);
        if (a < Sn) {
            const int b0 = h_scene_body_start[scn], nsb = h_scene_body_start[scn + 1] - b0;
            const int l = a - h_scene_static_start[scn];
            slot_of[c] = (size_t)b0 * L + (size_t)l * nsb + (size_t)(bi - b0);
            flags[slot_of[c]] = 1;
            ++nstat;
        } else {
            ++cnt[a - Sn];
        }
    }
    int acc = 0;
    for (size_t k = 0; k < nflag; ++k) {
        spos[k] = acc;
        acc += flags[k];
    }
    std::vector<int32_t> poff(N + 1, 0);
    for (int i = 0; i < N; ++i) poff[i + 1] = poff[i] + cnt[i];
    std::vector<double> org(3 * (size_t)std::max(sc.nscenes, 1));
    if ((st = cuda_check(cudaMemcpy(org.data(), sb.origin, 8 * 3 * (size_t)sc.nscenes, cudaMemcpyDeviceToHost), "origins")))
        return st;
    std::vector<unsigned long long> keys(std::max(n, 1));
    std::vector<float4> pt(std::max(n, 1)), lam(std::max(n, 1));
    std::vector<int32_t> fill(N, 0);
    for (int c = 0; c < n; ++c) {
        const int64_t o = order[c];
        const int a = ia[o], bi = ib[o] - Sn;
        const int scn = h_body_scene_of(bi);
        const int slot = a < Sn ? spos[slot_of[c]] : nstat + poff[a - Sn] + fill[a - Sn]++;
        keys[slot] = ((unsigned long long)a << 32) | (unsigned long long)ib[o];
        const double* q = point + 3 * o;
        const double* l = lambda + 3 * o;
        pt[slot] = make_float4((float)(q[0] - org[3 * scn]), (float)(q[1] - org[3 * scn + 1]),
                               (float)(q[2] - org[3 * scn + 2]), 0.f);
        lam[slot] = make_float4((float)l[0], (float)l[1], (float)l[2], 0.f);
    }
    const int pg = S->gen ^ 1;
    if (n > 0) {
        if ((st = cuda_check(cudaMemcpy(sb.key[pg], keys.data(), 8 * (size_t)n, cudaMemcpyHostToDevice), "upload"))) return st;
        if ((st = cuda_check(cudaMemcpy(sb.pt[pg], pt.data(), 16 * (size_t)n, cudaMemcpyHostToDevice), "upload"))) return st;
        if ((st = cuda_check(cudaMemcpy(sb.lam[pg], lam.data(), 16 * (size_t)n, cudaMemcpyHostToDevice), "upload"))) return st;
    }
    if (nflag > 0) {
        if ((st = cuda_check(cudaMemcpy(sflags_prev, flags.data(), 4 * nflag, cudaMemcpyHostToDevice), "upload"))) return st;
        if ((st = cuda_check(cudaMemcpy(spos_prev, spos.data(), 4 * nflag, cudaMemcpyHostToDevice), "upload"))) return st;
    }
    if ((st = cuda_check(cudaMemcpy(poff_prev, poff.data(), 4 * (size_t)(N + 1), cudaMemcpyHostToDevice), "upload")))
        return st;
    const int32_t dev2[2] = {n, nstat};
    static_assert(offsetof(SplitScalars, prev_n_static_dev) == offsetof(SplitScalars, prev_count_dev) + 4,
                  "the warm-start layout scalars are adjacent");
    if ((st = cuda_check(cudaMemcpy(&sb.ss->prev_count_dev, dev2, sizeof(dev2), cudaMemcpyHostToDevice), "upload")))
        return st;
    S->prev_count = n;
    S->prev_n_static = nstat;
    S->nc = n;
    S->force_sync = true;
    prev_count = n;
    contacts_loaded = true;
    return CDX_OK;
}

int Engine::get_contacts_split(int32_t* ia, int32_t* ib, double* point, double* lambda, double* normal,
                               int32_t* count) {
    const int n = split ? split->prev_count : 0;
    if (count) *count = n;
    if (n == 0 || (!ia && !ib && !point && !lambda && !normal)) return CDX_OK;
    SplitBuf& sb = split->sb;
    const int g = split->gen ^ 1;
    std::vector<unsigned long long> keys(n);
    std::vector<float4> pt(n), lam(n), nm(n);
    int st;
    if ((st = cuda_check(cudaMemcpy(keys.data(), sb.key[g], 8 * (size_t)n, cudaMemcpyDeviceToHost), "download"))) return st;
    if ((st = cuda_check(cudaMemcpy(pt.data(), sb.pt[g], 16 * (size_t)n, cudaMemcpyDeviceToHost), "download"))) return st;
    if ((st = cuda_check(cudaMemcpy(lam.data(), sb.lam[g], 16 * (size_t)n, cudaMemcpyDeviceToHost), "download"))) return st;
    if (!contacts_loaded &&
        (st = cuda_check(cudaMemcpy(nm.data(), sb.rec0, 16 * (size_t)n, cudaMemcpyDeviceToHost), "download"))) return st;
    std::vector<double> org(3 * (size_t)sc.nscenes);
    if ((st = cuda_check(cudaMemcpy(org.data(), sb.origin, 8 * org.size(), cudaMemcpyDeviceToHost), "download"))) return st;
    std::vector<int32_t> bscene(sc.N);
    if (sc.N && (st = cuda_check(cudaMemcpy(bscene.data(), sc.body_scene, 4 * (size_t)sc.N, cudaMemcpyDeviceToHost), "download"))) return st;
    for (int c = 0; c < n; ++c) {
        const int32_t a = (int32_t)(keys[c] >> 32), b = (int32_t)(keys[c] & 0xffffffffu);
        if (ia) ia[c] = a;
        if (ib) ib[c] = b;
        const int scn = bscene[b - sc.S];
        const float p[3] = {pt[c].x, pt[c].y, pt[c].z}, l[3] = {lam[c].x, lam[c].y, lam[c].z},
                    nn[3] = {nm[c].x, nm[c].y, nm[c].z};
        for (int k = 0; k < 3; ++k) {
            if (point) point[3 * (size_t)c + k] = (double)p[k] + org[3 * scn + k];
            if (lambda) lambda[3 * (size_t)c + k] = l[k];
            if (normal) normal[3 * (size_t)c + k] = nn[k];
        }
    }
    return CDX_OK;
}

double Engine::split_bytes_per_iter() const {
    // per contact: n and mu (16), lever lengths and body indices (16), lambda read + write (24, its
    // three words); per body: the accumulator cleared for the sweep after next (24)
    const int n = split ? split->prev_count : 0;
    return (double)n * (16 + 16 + 24) + (double)sc.N * 24.0;
}

// Kernel-level timing of the sweep (CUDA events around each launch, engine stream).
int Engine::time_sweeps(int n, double* msc, double* msb, double* bc, double* bb) {
    if (!loaded) return fail(CDX_ERR_STATE, "no scene loaded");
    if (n <= 0) return fail(CDX_ERR_ARG, "n must be positive");
    cudaEvent_t e[4];
    for (auto& x : e) cudaEventCreate(&x);
    double tc = 0, tb = 0;
    int st = CDX_OK;
    const bool sp = cfg.gpu_precision == CDX_PRECISION_SPLIT;
    if (sp && split && split->prev_count > 0) {
        SplitState* S = split;
        const int g = S->gen ^ 1;
        const int tv = split_sweep_variant();
        const int cblocks = split_contact_blocks(tv, S->prev_count, S->sms);
        *S->h_nc = S->prev_count;
        cudaMemcpyAsync(S->sb.nc_dev, S->h_nc, sizeof(int32_t), cudaMemcpyHostToDevice, stream);
        launch_s_reset(S->sb, stream);
        CoopPlan plan;
        if (split_variant_is_coop(tv) && coop_plan(*this, tv, S->prev_count, &plan)) {
            // one cooperative launch of n sweeps; reported per sweep
            cudaEventRecord(e[0], stream);
            st = launch_coop(*this, S->sb, g, tv, plan, 1 << 30, 0.f, n, stream);
            cudaEventRecord(e[1], stream);
            if (!(st = cuda_check((cudaError_t)st, "cooperative launch")) &&
                !(st = cuda_check(cudaEventSynchronize(e[1]), "time sweeps"))) {
                float a = 0;
                cudaEventElapsedTime(&a, e[0], e[1]);
                tc = a;
            }
            ++launches;
            // one sweep, with the contact records and impulses on chip: per body the velocities read
            // (24 B), the impulse sums added (24 B) and the accumulator reset (24 B)
            if (bc) *bc = (double)sc.N * 72.0;
            if (bb) *bb = 0.0;
        } else {
          for (int k = 0; k < n; ++k) {
            cudaEventRecord(e[0], stream);
            launch_s_sweep(S->sb, g, (float)cfg.pj_alpha, tv, cblocks, 1 << 30, 0.f, 0, 0, stream);
            cudaEventRecord(e[1], stream);
            cudaEventRecord(e[2], stream);
            if ((st = cuda_check(cudaEventSynchronize(e[2]), "time sweeps"))) break;
            float a = 0, b = 0;
            cudaEventElapsedTime(&a, e[0], e[1]);
            cudaEventElapsedTime(&b, e[1], e[2]);
            tc += a;
            tb += b;
        }
          launches += (int64_t)n;
          // one sweep: per contact the two records (32) and lambda read + write (24); per body the
          // accumulator cleared for the sweep after next (24)
          if (bc) *bc = (double)S->prev_count * (16 + 16 + 24) + (double)sc.N * 24.0;
          if (bb) *bb = 0.0;
        }
    } else if (!sp && prev_count > 0) {
        const int g = gen ^ 1;
        cudaMemsetAsync(ds, 0, sizeof(DevScalars), stream);
        for (int k = 0; k < n; ++k) {
            cudaEventRecord(e[0], stream);
            launch_sweep_contact64(sc, C, g, prev_count, x, ds, 0, stream);
            cudaEventRecord(e[1], stream);
            launch_sweep_body64(sc, C, inc, x, 0.0, 0.0, 0, ds, stream);
            cudaEventRecord(e[2], stream);
            if ((st = cuda_check(cudaEventSynchronize(e[2]), "time sweeps"))) break;
            float a = 0, b = 0;
            cudaEventElapsedTime(&a, e[0], e[1]);
            cudaEventElapsedTime(&b, e[1], e[2]);
            tc += a;
            tb += b;
        }
        launches += 2 * (int64_t)n;
        // contact kernel: ids, flags, RW (27 words), bias (3), mu, lambda read+write, dlambda write,
        // and the W^T products for the body sweep (directions and lever parts read, 36 words written)
        if (bc) *bc = (double)prev_count * (8 + 4 + 27 * 8 + 3 * 8 + 8 + 6 * 8 + 3 * 8 + 27 * 8 + 36 * 8);
        // body kernel: incidence ranges, x read+write, M; per contact side its incidence code,
        // the contact's flags and the 18 stored products
        if (bb) *bb = (double)sc.N * (8 + 12 * 8 + 2 * 8) + (double)prev_count * 2 * (4 + 4 + 18 * 8);
    } else {
        st = fail(CDX_ERR_STATE, "no contacts from a previous step");
    }
    for (auto& x : e) cudaEventDestroy(x);
    if (st) return st;
    if (msc) *msc = tc / n;
    if (msb) *msb = tb / n;
    return CDX_OK;
}

int Engine::split_variant() const { return split ? split->last_variant : -1; }
// the whole-problem shape for the last step's contacts: the cooperative solve where its plan fits,
// else a streaming shape (the first one when a cooperative or batched shape is selected)
int Engine::split_sweep_variant() const {
    if (!split) return -1;
    const SplitState* S = split;
    CoopPlan plan;
    if (split_variant_is_coop(S->variant) && S->prev_count > 0 &&
        coop_plan(*this, S->variant, S->prev_count, &plan))
        return S->variant;
    return (split_variant_is_coop(S->variant) || split_variant_is_scenes(S->variant)) ? 0 : S->variant;
}
int Engine::split_tune_runs() const { return split ? split->tune_runs : 0; }
int Engine::split_redos() const { return split ? split->redos : 0; }
int64_t Engine::split_graph_steps() const { return split ? split->graph_steps : 0; }

extern "C" int cdx_selftest_nr64(cdx_ctx* ctx, int32_t n, const double* x, double* rcp, double* rsq) {
    if (!ctx || n < 0 || (n > 0 && (!x || !rcp || !rsq))) return CDX_ERR_ARG;
    Engine& E = ctx->eng;
    if (n == 0) return CDX_OK;
    double* d = nullptr;
    int st = E.dalloc((void**)&d, sizeof(double) * 3 * (size_t)n, "selftest");
    if (st) return st;
    cudaMemcpyAsync(d, x, sizeof(double) * n, cudaMemcpyHostToDevice, E.stream);
    launch_nr64_selftest(n, d, d + n, d + 2 * (size_t)n, E.stream);
    cudaMemcpyAsync(rcp, d + n, sizeof(double) * n, cudaMemcpyDeviceToHost, E.stream);
    cudaMemcpyAsync(rsq, d + 2 * (size_t)n, sizeof(double) * n, cudaMemcpyDeviceToHost, E.stream);
    st = E.cuda_check(cudaStreamSynchronize(E.stream), "selftest");
    E.dfree(d);
    return st;
}
