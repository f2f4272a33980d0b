// Internal definitions shared by the host engine and the kernels (not part of the C ABI).
//
// Device layout (HBM, structure of arrays):
//   bodies   field-major FP64 arrays of length N (positions, quaternions, velocities, rotation
//            matrix R[9], radius, mass, inertia, friction, restitution, 1/m, 1/I, M_ii),
//   statics  field-major arrays of length S (halfspaces and drums),
//   contacts field-major arrays of length `cap` in canonical order (entity id A, entity id B):
//            direction rows n,t1,t2 (9), body-frame lever products r x d for side A and B (9+9),
//            RW coefficients R_r * w (9+9+9), contact velocity bias (3), R-scaled bias (3),
//            impulses (3), impulse increments (3), friction, restitution, flags,
//   incidence body -> (contact, side) lists in solver row order (a sorted CSR of W^T), which turns
//            the W^T scatter into a deterministic per-body gather.
#pragma once
#include <cstddef>
#include <cstdint>
#include <functional>

#include <cuda_runtime.h>

namespace cdx {

enum BodyField {
    BF_PX, BF_PY, BF_PZ,
    BF_QX, BF_QY, BF_QZ, BF_QW,
    BF_VX, BF_VY, BF_VZ,
    BF_WX, BF_WY, BF_WZ,
    BF_R0, BF_R1, BF_R2, BF_R3, BF_R4, BF_R5, BF_R6, BF_R7, BF_R8,
    BF_RAD, BF_MASS, BF_INERTIA, BF_MU, BF_RN, BF_RT,
    BF_MINVL, BF_MINVA, BF_ML, BF_MA,
    BF_COUNT
};

enum StaticField {
    SF_PX, SF_PY, SF_PZ,
    SF_QX, SF_QY, SF_QZ, SF_QW,
    SF_VX, SF_VY, SF_VZ,
    SF_WX, SF_WY, SF_WZ,
    SF_DX, SF_DY, SF_DZ,
    SF_D, SF_RAD, SF_MU, SF_RN, SF_RT,
    SF_R0, SF_R1, SF_R2, SF_R3, SF_R4, SF_R5, SF_R6, SF_R7, SF_R8,
    SF_HL,                  // cylinder half length
    SF_AX, SF_AY, SF_AZ,    // cylinder axis in the static's own frame (world axis = R a)
    SF_EX, SF_EY, SF_EZ,    // box half extents along the static's own axes
    SF_COUNT
};

// contact flags
enum : int32_t { CF_FRICTIONAL = 1 };

struct Scene {
    int N = 0;          // dynamic spheres
    int S = 0;          // static shapes
    int nscenes = 1;
    int max_statics = 0;  // max statics of any scene
    double* B = nullptr;  // BF_COUNT * N
    int32_t* body_scene = nullptr;
    double* St = nullptr;  // SF_COUNT * S
    int32_t* static_kind = nullptr;
    int32_t* static_scene = nullptr;
    int32_t* scene_body_start = nullptr;    // nscenes + 1
    int32_t* scene_static_start = nullptr;  // nscenes + 1
    __host__ __device__ double* bf(int f) const { return B + (size_t)f * N; }
    __host__ __device__ double* sf(int f) const { return St + (size_t)f * S; }
};

struct Grid {
    double lo[3];
    double cell;
    int dim[3];
    int64_t ncells;
    int key_bits;
};

// Per-step contact storage (one generation). Keys, points and impulses are double-buffered
// across steps for the warm start; everything else is rebuilt every step.
struct Contacts {
    int64_t cap = 0;
    int32_t* a = nullptr;  // body index of side A (>= 0) or -(static index) - 1
    int32_t* b = nullptr;  // body index of side B
    int32_t* flags = nullptr;
    int32_t* rank = nullptr;  // position in solver row order (frictionless first)
    double* dir = nullptr;    // 9*cap: n, t1, t2 (world)
    double* cA = nullptr;     // 9*cap
    double* cB = nullptr;     // 9*cap
    double* rd = nullptr;     // 9*cap: R_r * d_r
    double* rcA = nullptr;    // 9*cap
    double* rcB = nullptr;    // 9*cap
    double* cb = nullptr;     // 3*cap
    double* biasR = nullptr;  // 3*cap
    double* dlam = nullptr;   // 3*cap
    // 36*cap (plain FP64 method): per contact side (index 2c + side) and row r, the products
    // (s d_r) dlam_r of the W^T gather, 6 a row (direction, then lever part), written by the contact
    // sweep so the body sweep reads 144 contiguous bytes a contact side
    double* term = nullptr;
    double* rb = nullptr;     // 9*cap: inverse Delassus block / alpha (pj.rdiag_true_delassus only)
    int32_t* rb_full = nullptr;  // device flag: some block is not diagonal (full 3x3 products)
    double* mu = nullptr;
    double* eN = nullptr;
    double* eT = nullptr;
    // double-buffered generation data
    unsigned long long* key[2] = {nullptr, nullptr};
    double* point[2] = {nullptr, nullptr};  // 3*cap
    double* lam[2] = {nullptr, nullptr};    // 3*cap
};

// FP32 contact record of the split form (matrix-free rows rebuilt from the normal and lever lengths)
struct ContactsF {
    int64_t cap = 0;
    float* n = nullptr;      // 3*cap normal (A -> B)
    float* lev = nullptr;    // 2*cap signed lever lengths along n (side A, side B)
    float* R = nullptr;      // 2*cap: R_n, R_t
    float* bias = nullptr;   // 3*cap R-scaled bias
    float* lam = nullptr;    // 3*cap
    float* mu = nullptr;
    int32_t* a = nullptr;
    int32_t* b = nullptr;
};

struct DevScalars {
    int32_t n_static;        // static contacts this step
    int32_t n_pair;          // pair contacts this step
    int32_t overflow;        // per-sphere candidate buffer overflow
    int32_t nonfinite;
    unsigned long long maxd;  // bits of max ||dlambda_c|| (non-negative doubles order as integers)
    unsigned long long maxl;  // bits of max |lambda_old|
    double velres;            // sum of squared scaled velocity increments
    int32_t done;
    int32_t iters;
    double res_last;
    double res_final;
    int32_t pad[4];
};

// state of the accelerated projected Jacobi loops (device)
struct AccelState {
    double thk, err_prev, coef, omega, rho, rho2, lambda;
    double sum_err, sum_dot;  // outputs of the fixed-order reductions
    int32_t restarts, disabled, mode, nonfinite, power_stop;
};
enum AccelReduce : int { ACC_VELRES = 0, ACC_NORM2 = 1, ACC_DOT = 2, ACC_ONES = 3 };

// Anderson loop (device): the dense iterate z = [velocities in stacked order 6 i + k; impulse rows
// in the reference's row order], a ring of the last m + 1 iterates and residuals (oldest at head),
// and the mode of the current step (0 plain step, 1 mixed candidate, 2 failed least squares)
struct AndersonState {
    int32_t head, count, mode, nonfinite;
};
struct AndersonBufs {
    int m = 0;             // history window
    int64_t nt = 0;        // 6 N + rows of this solve
    int64_t nt_cap = 0;    // allocated length of each dense vector
    double *z = nullptr, *w = nullptr, *f = nullptr, *cand = nullptr;
    double *zh = nullptr, *fh = nullptr;  // (m + 1) x nt_cap each
    double *part = nullptr;               // sums x chunks
    double *ls = nullptr;                 // normal equations (m x m), right side (m), gamma (m)
    int32_t* rowmap = nullptr;            // impulse row -> index into the 3 x cap impulse array
    int64_t rowmap_cap = 0;
    int plain = 0;                        // 1: x in stacked order and lam in row order (CSR drop-in)
    AndersonState* st = nullptr;
};

// condensed solver, colored sweeps (plain FP64 method): per contact 1/G_ii, rhs and the internal
// impulses (3 rows, field-major by cap), the block's degree and color; per body the free
// velocities, u_corr and its previous sweep (6 x N, field-major); the blocks sorted by color
#define CDX_COND_MAX_COLORS 128
struct CondBufs {
    int64_t cap = 0;
    int N = 0;
    double* ginv = nullptr;
    double* rhs = nullptr;
    double* lam = nullptr;
    int32_t* deg = nullptr;
    int32_t* col = nullptr;
    int32_t* col2 = nullptr;
    double* uf = nullptr;
    double* u = nullptr;
    double* up = nullptr;
    double* part = nullptr;
    double* dl = nullptr;      // 3 x cap: the Jacobi sweep's impulse increments
    int32_t* flags = nullptr;  // [0] diverged, [1] uncolored after a round, [2] more colors than the limit
    double* err = nullptr;     // the last residual (err) evaluated
    uint32_t* kin = nullptr;   // sort by color: keys (colors) and values (contacts), in and out
    uint32_t* vin = nullptr;
    uint32_t* kout = nullptr;
    uint32_t* vout = nullptr;
    int32_t* cstart = nullptr;  // CDX_COND_MAX_COLORS per-color ranges of vout
    int32_t* cend = nullptr;
};

// projected Gauss-Seidel (k_fp64_pgs.cu): the order of the blocks and the per-body chains that
// make a sweep sequential
struct PgsBufs {
    int64_t cap = 0;
    int32_t* pred = nullptr;      // 2*cap: previous block of body A / body B in sweep order (-1: none)
    int32_t* succ = nullptr;      // 2*cap: next block of body A / body B in sweep order (-1: none)
    int32_t* lstart = nullptr;    // cap: first position of each level in the level order
    int32_t* lend = nullptr;      // cap: one past its last
    unsigned* bar = nullptr;      // grid barrier counter
    int32_t* err = nullptr;       // a wait ran out (1 barrier, 2 predecessor)
    int32_t* stop = nullptr;      // the stop decision of the last sweep
    int32_t* lev = nullptr;       // cap: the level pass's count of unfinished predecessors a block
    int32_t* rflag = nullptr;     // 3: [0] blocks placed by the level pass
    int32_t* maxlev = nullptr;    // the largest level
};

struct Incidence {
    int64_t cap = 0;
    uint32_t* key_in = nullptr;
    uint32_t* val_in = nullptr;
    uint32_t* key_out = nullptr;
    uint32_t* val_out = nullptr;
    int32_t* start = nullptr;  // N
    int32_t* end = nullptr;    // N
};

// ---- launchers (k_common.cu) ----
size_t scan_temp_bytes(int64_t n);
size_t sort_temp_bytes(int64_t n);
cudaError_t exclusive_scan(void* tmp, size_t tmp_bytes, const int32_t* in, int32_t* out, int64_t n, cudaStream_t s);
cudaError_t sort_pairs(void* tmp, size_t tmp_bytes, const uint32_t* kin, uint32_t* kout, const uint32_t* vin,
                       uint32_t* vout, int64_t n, int end_bit, cudaStream_t s);
void launch_cell_keys(const Scene& sc, const Grid& g, uint32_t* keys, uint32_t* vals, cudaStream_t s,
                      int by_inverse = 0);
void launch_ranges(const uint32_t* sorted_keys, int64_t n, int32_t* start, int32_t* end, cudaStream_t s);
// state staging: 13 doubles per body, interleaved as the C ABI's host arrays
void launch_pack_state(const Scene& sc, double* out, cudaStream_t s);
void launch_pack_state4(const Scene& sc, double* pos, double* quat, double* vel, double* omega, cudaStream_t s);
void launch_unpack_state4(const Scene& sc, const double* pos, const double* quat, const double* vel,
                          const double* omega, cudaStream_t s);
void launch_unpack_state(const Scene& sc, const double* in, int mask, cudaStream_t s);

// ---- FP64 plain method (k_fp64.cu) ----
void launch_rhs64(const Scene& sc, double dt, const double* g, double* rhs, cudaStream_t s, int implicit_gyro = 0);
// condensed solver, colored sweeps (k_fp64_condensed.cu)
void launch_cond_setup(const Scene& sc, Contacts& C, int gen, int nc, double dt, const double* g, int implicit_gyro,
                       int warmstart, CondBufs& B, const Incidence& inc, cudaStream_t s);
void launch_cond_color_round(const Contacts& C, int nc, const CondBufs& B, const Incidence& inc,
                             const int32_t* col_in, int32_t* col_out, int32_t* uncolored, int32_t* too_many,
                             cudaStream_t s);
void launch_cond_sweep_color(const Scene& sc, const Contacts& C, const CondBufs& B, const uint32_t* blocks, int n,
                             double relax, double alpha, double* u, const DevScalars* ds, cudaStream_t s);
int cond_chunks(int N);
void launch_cond_sort_keys(int nc, const int32_t* col, CondBufs& B, cudaStream_t s);
void launch_cond_check(int N, const CondBufs& B, double tol_rel, double tol_abs, int iter, DevScalars* ds,
                       cudaStream_t s);
void launch_cond_copy(int n, const double* src, double* dst, const DevScalars* ds, cudaStream_t s);
// pj_convention < 0: x = u_free - u_corr; 0: impulses as stored for the warm start; 1: impulses in
// the projected Jacobi convention (for the complementarity residual)
void launch_cond_final(const Scene& sc, Contacts& C, int gen, int nc, const CondBufs& B, double* x, int pj_convention,
                       cudaStream_t s);
// projected Gauss-Seidel (k_fp64_pgs.cu): rhs, Dinv, the warm start and u_corr (B.uf from
// launch_cond_setup's free velocity), the per-body chains; then the whole solve in one cooperative
// launch (returns the launch's cudaError_t)
void launch_pgs_setup(const Scene& sc, Contacts& C, int gen, int nc, int warmstart, CondBufs& B, const Incidence& inc,
                      PgsBufs& P, cudaStream_t s);
// levels of the blocks: the blocks level by level into `order`, each level's range in P.lstart /
// P.lend, the largest level in P.maxlev
int launch_pgs_levels(const PgsBufs& P, int nc, uint32_t* order, unsigned long long wait_ns, cudaStream_t s);
// order: the contacts sorted by level; nlev levels, their ranges in P.lstart / P.lend
// condensed: run the condensed solver's block update (its sequential gauss_seidel sweep mode)
int launch_pgs_solve(const Scene& sc, const Contacts& C, int nlev, const CondBufs& B, const PgsBufs& P,
                     const uint32_t* order, double relax, double alpha, double tol_rel, double tol_abs, int max_iter,
                     DevScalars* ds, unsigned long long wait_ns, cudaStream_t s, int condensed = 0);
// the per-body chains of blocks (predecessors and successors) from incidence lists in sweep order
// (W's row order for projected Gauss-Seidel, contact order for the condensed solver)
void launch_pgs_links(const Scene& sc, int nc, const Incidence& inc, PgsBufs& P, cudaStream_t s);
// condensed solver, Jacobi sweep (both passes)
void launch_cond_jacobi(const Scene& sc, const Contacts& C, int nc, const CondBufs& B, const Incidence& inc,
                        double relax, double alpha, double* u, const DevScalars* ds, cudaStream_t s);
void launch_cond_ufree(const Scene& sc, double dt, const double* g, int implicit_gyro, CondBufs& B, cudaStream_t s);
// nonfinite (optional): set to 1 when a body's state after the drift is not finite
void launch_drift64(const Scene& sc, double h, int compute_R, cudaStream_t s, int32_t* nonfinite = nullptr);
// prescribed static motion for the coming step (13 doubles a static: position, quaternion,
// velocity, angular velocity; flags 1/2/4/8 say which apply), after the first drift
void launch_static_motion64(const Scene& sc, const double* mot, const int32_t* flag, cudaStream_t s);
void launch_static_flags64(const Scene& sc, double margin, int32_t* flags, cudaStream_t s);
// FP32 copy of the positions (relative to the grid origin) and radii: the pair kernels' conservative
// pre-test, so that only pairs near contact reach the FP64 test
void launch_pos32(const Scene& sc, const Grid& g, float4* p32, cudaStream_t s);
// plist: PLIST64 partners per sphere, filled by the count pass and read by the write pass
constexpr int PLIST64 = 8;
void launch_pair_count64(const Scene& sc, const Grid& g, const uint32_t* cell_body, const int32_t* cell_start,
                         const int32_t* cell_end, const float4* p32, int32_t* plist, double margin, int32_t* counts,
                         DevScalars* ds, cudaStream_t s);
void launch_static_write64(const Scene& sc, double margin, const int32_t* flags, const int32_t* pos,
                           Contacts& C, int gen, int combine, int friction_enable, cudaStream_t s);
void launch_pair_write64(const Scene& sc, const Grid& g, const uint32_t* cell_body, const int32_t* cell_start,
                         const int32_t* cell_end, const float4* p32, int32_t* plist, double margin,
                         const int32_t* offsets, int32_t base, Contacts& C, int gen, int combine, int friction_enable,
                         DevScalars* ds, cudaStream_t s);
void launch_contact_setup64(const Scene& sc, Contacts& C, int gen, int nc, int prev_count, double alpha,
                            double match2, int warmstart, cudaStream_t s);
void launch_frictionless_flags(const Contacts& C, int nc, int32_t* isfl, cudaStream_t s);
void launch_rank_and_incidence(const Scene& sc, Contacts& C, int nc, const int32_t* fl_scan, const int32_t* isfl,
                               Incidence& inc, cudaStream_t s,
                               int by_contact = 0);
void launch_xinit64(const Scene& sc, const Contacts& C, int gen, const Incidence& inc, const double* rhs, double* x,
                    cudaStream_t s);
void launch_sweep_contact64(const Scene& sc, Contacts& C, int gen, int nc, const double* x, DevScalars* ds, int dry,
                            cudaStream_t s);
void launch_block_invert64(const Contacts& C, int nc, cudaStream_t s);
void launch_sweep_body64(const Scene& sc, const Contacts& C, const Incidence& inc, double* x, double tol_abs,
                         double tol_rel, int want_velres, DevScalars* ds, cudaStream_t s);
void launch_check(DevScalars* ds, int iter, double residual_tol, int nv, int check_vel, cudaStream_t s);
void launch_final_residual(DevScalars* ds, cudaStream_t s);
// accelerated loops (Nesterov, Chebyshev) of the plain FP64 method
int accel_chunks(int N);
void launch_accel_init(AccelState* st, cudaStream_t s);
// plain = 1: vectors of length N in stacked order (the solver-level drop-in), else 6 x N field-major
void launch_accel_reduce(int N, int op, const double* a, const double* b, const double* c, double tol_rel,
                         double tol_abs, double* part, AccelState* st, double* out, const DevScalars* ds,
                         cudaStream_t s, int plain = 0);
void launch_accel_copy(double* xd, const double* xs, int64_t nx, double* ld, const double* ls, int64_t nl,
                       const DevScalars* ds, cudaStream_t s);
void launch_nesterov_step(AccelState* st, DevScalars* ds, int nv, double beta_threshold, int restart_limit, double* xy,
                          double* xk, const double* xk1, int64_t nx, double* py, double* pk, const double* pk1,
                          int64_t nl, double residual_tol, cudaStream_t s);
void launch_chebyshev_step(AccelState* st, DevScalars* ds, int nv, int iter, const double* x, double* xk, double* xk1,
                           int64_t nx, const double* lam, double* pk, double* pk1, int64_t nl, double residual_tol,
                           cudaStream_t s);
int anderson_sums(int m);
int anderson_chunks(int64_t n);
void launch_anderson_begin(const Contacts& C, int gen, int nc, const int32_t* fl_scan, const int32_t* isfl, int N,
                           const double* x, AndersonBufs& A, cudaStream_t s);
void launch_anderson_begin_plain(int nv, const double* x, const double* lam, AndersonBufs& A, cudaStream_t s);
// N: bodies (6 x N field-major velocities), or the velocity count when A.plain
void launch_anderson_scatter(int N, double* x, double* lam, const AndersonBufs& A, const DevScalars* ds, cudaStream_t s);
// residual_tol (gpu.residual_tol, 0 = off): the accelerated loops also end once the sweep's
// complementarity residual is at most tol, tested right after the reference's own exit
void launch_anderson_mix(int N, const double* x, const double* lam, const AndersonBufs& A, double tol_rel,
                         double tol_abs, double residual_tol, DevScalars* ds, cudaStream_t s);
// estimateSpectralRadius's eight power steps; apply() launches Mv = M v (N bodies, or N velocities
// when plain)
void launch_power_iteration(int N, int plain, double* v, double* Mv, double* part, AccelState* st,
                            const std::function<void()>& apply, cudaStream_t s);
void launch_spectral_radius(const Scene& sc, Contacts& C, const Incidence& inc, int nc, double* v, double* Mv,
                            double* part, AccelState* st, cudaStream_t s);
void launch_writeback64(const Scene& sc, const double* x, cudaStream_t s);
void launch_trace64(const Contacts& C, int gen, int nc, const int32_t* fl_scan, const int32_t* isfl, double* out,
                    cudaStream_t s);

}  // namespace cdx

namespace cdx {
// ---- solver-level drop-in on a general CSR Jacobian (k_csr.cu) ----
void launch_csr_rhs(int nv, const double* mdiag, const double* v, const double* fext, const double* fgyro, double dt,
                    double* rhs, cudaStream_t s);
void launch_csr_rowidx(int nrows, const int32_t* ptr, int32_t* rowidx, uint32_t* colkey, uint32_t* nzid,
                       const int32_t* col, cudaStream_t s);
// block = 1: pj.rdiag_true_delassus (W and the bias unscaled; the blocks come from launch_csr_blocks)
void launch_csr_setup(int nrows, const int32_t* ptr, const int32_t* col, const double* val, const double* cb,
                      const double* e, const double* minv, const double* v, double alpha, double* RW, double* biasR,
                      cudaStream_t s, int block = 0);
// per-unit inverse Delassus blocks / alpha (9 doubles a unit) and the flag of a non-diagonal block
void launch_csr_blocks(int nrows, int nfl, const int32_t* ptr, const int32_t* col, const double* val,
                       const double* minv, double alpha, double* Rb, int32_t* full, cudaStream_t s);
// Mv = v - S^-1 W^T R_block (RW v): the linear part of the sweep map (power iteration)
void launch_csr_linear(int nrows, int nfl, int nv, const int32_t* ptr, const int32_t* col, const double* RW,
                       const double* Rb, const int32_t* full, const int32_t* cstart, const int32_t* cend,
                       const uint32_t* nz_sorted, const int32_t* rowidx, const double* val, const double* mdiag,
                       const double* v, double* delta, double* Mv, cudaStream_t s);
void launch_csr_cols(int nv, const int32_t* cstart, const int32_t* cend, const uint32_t* nz_sorted,
                     const int32_t* rowidx, const double* val, const double* y, const double* base,
                     const double* mdiag, double* x, int mode, double tol_abs, double tol_rel, int want_velres,
                     DevScalars* ds, cudaStream_t s);
// Rb/full: the block preconditioner (nullptr: the row scale folded into RW); dry: residual only
void launch_csr_rows(int nrows, int nfl, const int32_t* ptr, const int32_t* col, const double* RW,
                     const double* biasR, const double* mu, const double* x, double* lam, double* dlam,
                     DevScalars* ds, cudaStream_t s, const double* Rb = nullptr, const int32_t* full = nullptr,
                     int dry = 0);
}  // namespace cdx
