// Device buffers and launchers of the split-precision form (k_split.cu).
#pragma once
#include <cstdint>

#include <cuda_runtime.h>

#include "cdx_internal.h"

namespace cdx {

struct SplitScalars {
    int32_t done;
    int32_t iters;
    unsigned int blocks_done;  // completion counter of the body pass (last block runs the check)
    unsigned int bar_arr;      // cooperative solve: arrivals at the grid barrier counter so far this step
    unsigned int maxd;  // bits of max ||dlambda_c|| (FP32, non-negative)
    unsigned int maxl;  // bits of max |lambda|
    float res_last;
    int32_t pad0;
    unsigned long long maxd64;  // FP64 residual pass
    unsigned long long maxl64;
    double res_final;
    // cooperative solve: grid-barrier arrival counter, the barrier epoch at the start of the next
    // launch (the counter's target is epoch x blocks), and the barrier timeout flag
    unsigned int bar;
    unsigned int bar_base;
    int32_t err;
    int32_t final_acc;                // accumulator holding the final velocities (-1: iters % 3)
    unsigned long long iters_sum;     // batched scenes: sweeps summed over scenes
    // contact totals found on the device (steps that do not stop for the host to size buffers)
    int32_t n_static;                 // static contacts (the pair contacts start here)
    int32_t n_total;                  // all contacts found (may exceed the capacity)
    int32_t cap_err;                  // the contacts did not fit the buffers: the step is redone
    // the last completed step's contact layout for the warm start, kept on the device for steps
    // launched from a CUDA graph (their parameters are fixed at capture)
    int32_t prev_count_dev;
    int32_t prev_n_static_dev;
    int32_t pair_overflow;            // copy of the narrow phase's neighbour-overflow flag
    int32_t nonfinite;                // the step's final state holds a value that is not finite
    // the cooperative solve under the reference's loop controls (pj.nesterov, pj.tol_abs/tol_rel),
    // carried across launches: Nesterov's theta, last err and restart count, and which accumulators
    // hold y (the extrapolated iterate), x_{k+1} (being formed) and x_k
    double nes_thk;
    double vel_err;                   // the last velocity-increment residual evaluated (err)
    double nes_err_prev;
    int32_t nes_restarts;
    int32_t nes_disabled;
    int32_t nes_iy, nes_ix1, nes_ixk;
    int32_t pad2;
};

// Loop controls of ProjectedJacobiSolver that the cooperative solve honours (projected_jacobi.cpp:
// 140-144, 371-377, 379-449): the velocity-increment exit every 10 sweeps of the standard loop, or
// Nesterov's loop with its restart tests and exit.
struct CoopLoopArgs {
    double tol_abs, tol_rel;   // pj.tol_abs, pj.tol_rel
    double beta_threshold;     // pj.nesterov_beta_threshold
    int check_vel;             // standard loop: the exit is on (the tolerances are not both 0)
    int restart_limit;         // pj.nesterov_restart_limit
    int nv;                    // velocities (6 per body)
    // how the velocity-increment residual is summed: 0 in FP64 term by term; 1 (pj.tol_rel = 0) the
    // squared increments in FP32, divided by tol_abs once; 2 (pj.tol_abs = 0) the squared relative
    // increments in FP32, divided by tol_rel once; 3 (both in [1e-12, 1e12]) term by term in FP32
    int res_mode;
};

struct SplitParams {
    float alpha;
    float margin;
    double margin64;  // collision.security_margin in FP64: membership decided near the threshold
    float match2;
    int combine;
    int friction_enable;
    int prev_count;  // < 0: read SplitScalars::prev_count_dev / prev_n_static_dev on the device
    // previous step's contact layout, for an O(1) warm-start lookup: static contact of slot k was
    // contact prev_spos[k] when prev_sflags[k]; pair contacts of owner i were
    // [prev_n_static + prev_poff[i], prev_n_static + prev_poff[i+1])
    const int32_t* prev_sflags;
    const int32_t* prev_spos;
    const int32_t* prev_poff;
    int prev_n_static;
};

// Contact records are two float4s so a warp reads them with 16-byte vector loads:
//   rec0 (n.x, n.y, n.z, mu)        the sign bit of mu flags a contact with a velocity bias
//   rec1 (rhoA, rhoB, A, B)          signed lever lengths along n; A = body index or -(static)-1
//                                    and B stored as int bits
//   bias (b_n, b_t1, b_t2)           static wall velocity and restitution terms (flagged contacts)
//   lam  (lambda_n, lambda_t1, lambda_t2) per generation (warm start)
// R = alpha / diag(W M^-1 W^T) is recomputed in the sweep from the inverse masses that come with
// the velocity gathers: R_n = alpha / (1/mA + 1/mB), R_t = alpha / (1/mA + 1/mB + rhoA^2/IA + rhoB^2/IB).
constexpr int SPLIT_NACC = 4;  // rotating velocity accumulators of the sweeps
constexpr int SPLIT_PLIST = 8;  // partners a body keeps from the count pass
struct SplitBuf {
    int N = 0;
    int64_t cap = 0;
    float4* pos4 = nullptr;   // N: position relative to the scene origin, radius
    double4* pos64 = nullptr; // N: FP64 position and radius in one 32-byte record (the narrow phase's FP64 test)
    float4* pos4lo = nullptr; // N: what pos4 rounded off (position relative to the scene origin, radius)
    // SPLIT_PLIST per body: the partners the narrow phase's count pass found (when they fit), so
    // the write pass does not walk the neighbour cells again
    int32_t* plist = nullptr;
    float4* vel4 = nullptr;   // 2N: free velocities (v_free, 1/m), (omega_free world, 1/I)
    // 2N each, rotating by sweep k: gather A[k % 4], add into A[(k + 1) % 4], reset A[(k + 3) % 4]
    // (read in sweep k - 1, next added into in sweep k + 2) to the free velocities
    float4* acc[SPLIT_NACC] = {nullptr, nullptr, nullptr, nullptr};
    float4* vn4 = nullptr;    // 2N: pre-solve velocities (v, omega_world)
    float4* mat4 = nullptr;   // N: (mu, normal restitution, tangential restitution, 0) in FP32, constant per
                              // body (the narrow phase reads them without FP64 conversions)
    double* vfree = nullptr;  // 6N FP64 free velocities (world frame)
    double* acc64 = nullptr;  // 6N FP64 W^T lambda, then final velocities
    double* origin = nullptr; // 3 per scene
    float4* st_dir = nullptr; // S: (normal/axis, plane offset in scene coordinates)
    float4* st_pt = nullptr;  // S: (anchor in scene coordinates, drum radius)
    float4* st_box = nullptr; // 3S: a box's axes in world (columns of its rotation), .w its half extents
    float4* st_v = nullptr;   // S: (wall velocity, kind)
    float4* st_w = nullptr;   // S: (wall angular velocity world, mu)
    float4* rec0 = nullptr;
    float4* rec1 = nullptr;
    float4* bias = nullptr;
    float4* lam[2] = {nullptr, nullptr};
    unsigned long long* key[2] = {nullptr, nullptr};
    float4* pt[2] = {nullptr, nullptr};
    int32_t* nc_dev = nullptr;
    SplitScalars* ss = nullptr;
    float2* part = nullptr;   // per-block (max ||dlambda||, max |lambda|) of the contact sweep
    float2* recs = nullptr;   // cooperative solve: 2 banks x per-block (max ||dlambda||, max |lambda|)
    double2* sums = nullptr;  // cooperative solve: 2 banks x per-block sums (velocity-increment residual, dot)
    float4* lamk = nullptr;   // Nesterov: the previous iterate's impulses (contacts outside shared memory)
    float4* lam_warm = nullptr;  // per-scene solve with tuned alpha: each guarded scene's starting impulses
    int has_restitution = 0;  // pre-solve velocities are only needed for restitution terms
};

int split_grid_blocks(int64_t n, int sms);
int launch_nr64_selftest(int n, const double* x, double* rcp, double* rsq, cudaStream_t s);
int split_contact_blocks(int variant, int64_t n, int sms);
constexpr int SPLIT_MAX_PARTS = 4096;  // capacity of the per-block partial maxima
int split_num_variants();
const char* split_variant_name(int v);
bool split_variant_is_coop(int v);
bool split_variant_is_scenes(int v);
int split_first_scenes_variant();
// the shape used until the autotuner has timed the others: the cooperative solve (where its plan
// fits; otherwise the first streaming shape runs)
int split_first_coop_variant();
int split_num_scenes_variants();
// batched scenes: the whole solve of every scene, one block per scene (order = scene ids by
// decreasing size; nbmax = bodies of the largest scene). Returns a cudaError_t.
// scene_alpha (optional): per-scene alpha, with the residual rescaled to alpha_ref; scene_out
// (optional): per-scene sweeps and residual
int launch_s_solve_scenes(const Scene& sc, const SplitBuf& sb, int gen, float alpha, int v, int max_iter, float tol,
                          const int32_t* spos, const int32_t* sflags, const int32_t* poff, const int32_t* order,
                          int nbmax, cudaStream_t s, float* scene_alpha = nullptr, float alpha_ref = 0.f,
                          int4* scene_out = nullptr);
// the scenes' alpha autotuner: op 0 resets the best (alpha = the configured one), 3 records the
// reference trial (the configured alpha), 1 keeps trial `alpha` where it beats the best, 2 writes
// the best alphas
void launch_s_tune_alpha(int op, int ns, float alpha, const int4* out, float4* best, float* scene_alpha,
                         cudaStream_t s);
// the accumulators back to the free velocities (before a warm start is applied again)
void launch_s_acc_init(const SplitBuf& sb, cudaStream_t s);
// cooperative whole-solve partition (grid = one block per SM, contact and body ranges per block)
struct CoopPlan {
    int grid = 0, nth = 0, cpb = 0, bpb = 0, vf = 0, smem = 0;
};
// smem_contacts > 0 caps the contacts a block keeps in shared memory (gpu.coop_smem_contacts);
// blocks > 0 sets the grid (gpu.coop_blocks, capped at one block per SM), 0 = one per SM
// loop = 0: the plain cooperative kernel; 1: the standard loop with the velocity-increment exit;
// 2: Nesterov's loop (64 B of shared memory a contact instead of 48). Loop kernels exist for the
// 1024-thread shapes only.
bool split_coop_plan(int v, int64_t nc, int64_t nbodies, int sms, CoopPlan* p, int smem_contacts = 0,
                     int blocks = 0, int loop = 0);
// the projected Jacobi solve, up to max_sweeps sweeps, in one cooperative launch, evaluating the
// stop rule every check_every sweeps; a block waits at most wait_ns at a grid barrier (0 = 0.2 s);
// returns the cudaError_t of the launch
int launch_s_solve_coop(const SplitBuf& sb, int gen, float alpha, int v, const CoopPlan& p, int max_iter, float tol,
                        int max_sweeps, int check_every, cudaStream_t s, unsigned long long wait_ns = 0);
// the same under the reference's loop controls (loop = 1 standard loop with the velocity-increment
// exit, 2 Nesterov); the plan must come from split_coop_plan with the same loop
int launch_s_solve_coop_loop(const SplitBuf& sb, int gen, float alpha, int v, const CoopPlan& p, int max_iter,
                             float tol, int max_sweeps, int check_every, int loop, const CoopLoopArgs& la,
                             unsigned long long wait_ns, cudaStream_t s);
// smot/smflag (optional): prescribed static motion applied after the statics' first drift
void launch_s_prep(const Scene& sc, const SplitBuf& sb, double dt, const double* g, double h1, cudaStream_t s,
                   int implicit_gyro = 0, const double* smot = nullptr, const int32_t* smflag = nullptr);
void launch_s_static_flags(const Scene& sc, const SplitBuf& sb, float margin, double margin64, int32_t* flags,
                           cudaStream_t s);
// cell_body / cell_key: the bodies and their cell keys sorted by cell
void launch_s_pair_count(const Scene& sc, const Grid& g, const SplitBuf& sb, const uint32_t* cell_body,
                         const uint32_t* cell_key, const int32_t* cell_start, const int32_t* cell_end, int32_t* counts,
                         const SplitParams& P, DevScalars* ds, cudaStream_t s);
void launch_s_static_write(const Scene& sc, const SplitBuf& sb, const int32_t* flags, const int32_t* pos, int gen,
                           const SplitParams& P, cudaStream_t s);
// base = first pair slot, or taken from the device (SplitScalars::n_static) when base < 0
void launch_s_pair_write(const Scene& sc, const Grid& g, const SplitBuf& sb, const uint32_t* cell_body,
                         const uint32_t* cell_key, const int32_t* cell_start, const int32_t* cell_end,
                         const int32_t* offsets, int32_t base, int gen, const SplitParams& P, DevScalars* ds,
                         cudaStream_t s);
// contact totals on the device: n_static, n_total, cap_err and nc_dev = min(total, capacity)
void launch_s_totals(const SplitBuf& sb, const int32_t* spos, const int32_t* sflags, int64_t nflag, const int32_t* poff,
                     int N, cudaStream_t s);
void launch_s_reset(const SplitBuf& sb, cudaStream_t s);
// end of a step: the warm-start layout for the next step and the neighbour-overflow flag, on the device
void launch_s_end_step(const SplitBuf& sb, const DevScalars* ds, cudaStream_t s);
void launch_s_apply_warm(const SplitBuf& sb, int gen, int blocks, cudaStream_t s);
// one projected Jacobi sweep (one kernel): reads A_k, scatters M^-1 W^T lambda_{k+1} into A_{k+1},
// clears A_{k+2}; its last block runs the stop rule
void launch_s_sweep(const SplitBuf& sb, int gen, float alpha, int variant, int blocks, int max_iter, float tol,
                    cudaGraphConditionalHandle h, int use_handle, cudaStream_t s);
// final FP64 velocities, residual, write-back and the closing drift by drift_h
void launch_s_final(const Scene& sc, const SplitBuf& sb, int gen, double alpha, int friction_enable, int combine,
                    int blocks, double drift_h, cudaStream_t s);

}  // namespace cdx
