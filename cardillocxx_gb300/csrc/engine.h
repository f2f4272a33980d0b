// Host engine state (one per cdx_ctx).
#pragma once
#include <algorithm>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/cdx.h"
#include "cdx_internal.h"
#include "output.h"

namespace cdx {
const char* status_name(int st);
struct SplitState;
// work buffers of the solver-level CSR solve (engine_csr.cpp); device memory in Engine::owned
struct CsrBuffers {
    int64_t nnz_cap = 0, row_cap = 0, nv_cap = 0;
    int32_t *ptr = nullptr, *col = nullptr, *rowidx = nullptr, *cstart = nullptr, *cend = nullptr;
    uint32_t *ck_in = nullptr, *ck_out = nullptr, *nz_in = nullptr, *nz_out = nullptr;
    double *val = nullptr, *RW = nullptr, *cb = nullptr, *mu = nullptr, *e = nullptr, *biasR = nullptr,
           *lam = nullptr, *dlam = nullptr;
    double *minv = nullptr, *mdiag = nullptr, *v = nullptr, *fext = nullptr, *fgyro = nullptr, *rhs = nullptr,
           *x = nullptr;
    DevScalars* ds = nullptr;
    // block preconditioner (9 doubles a unit) and the accelerated loops' copies, grown on demand
    int64_t unit_cap = 0, acc_rows = 0, acc_nv = 0;
    double* Rb = nullptr;
    int32_t* full = nullptr;
    double *xk = nullptr, *xk1 = nullptr, *xy = nullptr, *pk = nullptr, *pk1 = nullptr, *py = nullptr,
           *part = nullptr;
    AccelState* st = nullptr;
    AndersonBufs anderson;
};
}  // namespace cdx

struct Engine {
    cdx_config cfg{};
    std::string err;
    cudaStream_t stream = nullptr;
    bool loaded = false;
    bool timing = false;
    cdx::Scene sc;
    cdx::Grid grid{};
    double rmax = 0;
    std::vector<int32_t> h_scene_body_start, h_scene_static_start;
    // scene of sphere i / of static s (host copies of the scene ranges)
    int h_body_scene_of(int64_t i) const {
        return (int)(std::upper_bound(h_scene_body_start.begin(), h_scene_body_start.end(), (int32_t)i) -
                     h_scene_body_start.begin()) - 1;
    }
    int h_static_scene_of(int64_t s) const {
        return (int)(std::upper_bound(h_scene_static_start.begin(), h_scene_static_start.end(), (int32_t)s) -
                     h_scene_static_start.begin()) - 1;
    }
    std::vector<void*> owned;

    double* rhs = nullptr;
    double* x = nullptr;
    double* stage = nullptr;  // 13 N doubles: state staging for get/set_state
    uint32_t *cell_key_in = nullptr, *cell_val_in = nullptr, *cell_key_out = nullptr, *cell_val_out = nullptr;
    float4* pos32 = nullptr;  // plain FP64 method: FP32 positions and radii for the pair pre-test
    int32_t* plist64 = nullptr;  // plain FP64 method: partners kept by the narrow phase's count pass
    int32_t *cell_start = nullptr, *cell_end = nullptr;
    int32_t *sflags = nullptr, *spos = nullptr, *pcount = nullptr, *poff = nullptr;
    int32_t *sflags_prev = nullptr, *spos_prev = nullptr, *poff_prev = nullptr;  // split form warm start
    int32_t *isfl = nullptr, *flscan = nullptr;
    cdx::Contacts C;
    cdx::Incidence inc;
    cdx::DevScalars* ds = nullptr;
    // accelerated loops: iterate copies (6N velocities, 3 cap impulses), reduction partials, state
    double *acc_xk = nullptr, *acc_xk1 = nullptr, *acc_xy = nullptr;
    double *acc_pk = nullptr, *acc_pk1 = nullptr, *acc_py = nullptr, *acc_part = nullptr;
    cdx::AccelState* acc_st = nullptr;
    int64_t acc_nx = 0, acc_nl = 0;
    int ensure_accel();
    int solve64_accel();
    cdx::AndersonBufs anderson;
    int ensure_anderson(int64_t nt);
    int solve64_anderson();
    cdx::DevScalars* hs = nullptr;  // pinned mirror
    void* tmp = nullptr;
    size_t tmp_bytes = 0;
    int nc = 0, prev_count = 0, gen = 0;
    int last_iters = 0, last_rows = 0;
    double last_res = 0, last_res_final = 0;
    int64_t steps = 0;
    int64_t launches = 0;
    int reallocations = 0;
    cudaEvent_t ev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    double ms[4] = {0, 0, 0, 0};

    bool trace_next = false, trace_done_seen = false;
    int trace_rows = 0;
    double* trace_dev = nullptr;
    std::vector<double> trace_buf;

    // frame output (output.cpp): writer, scene copies, tracked spheres, simulated time
    cdx::Output* out = nullptr;
    cdx::OutputScene oscene;
    std::vector<std::pair<int32_t, std::string>> tracked;
    double out_time = 0.0;
    bool out_started = false;
    int output_frame();
    int output_tracked();
    int track(int32_t body, const char* name);
    int output_flush();

    cdx::SplitState* split = nullptr;
    cdx::CsrBuffers* csr = nullptr;

    ~Engine();
    int fail(int st, const std::string& msg);
    int cuda_check(cudaError_t e, const char* where);
    int dalloc(void** p, size_t bytes, const char* what);
    void dfree(void* p);
    int init(const cdx_config& c);
    // replace the configuration between steps (the solver reads its settings every solve)
    int set_config(const cdx_config& c);
    int check_solver_config(const cdx_config& c);
    // condensed solver, colored sweeps (plain FP64 method; engine_condensed.cpp)
    cdx::CondBufs cond;
    int cond_diverged = 0;
    int ensure_cond();
    int solve_condensed();
    int solve_condensed_gs();
    int finish_condensed();
    // projected Gauss-Seidel (plain FP64 method; engine_pgs.cpp)
    cdx::PgsBufs pgs;
    int last_levels = 0;  // levels of the last projected Gauss-Seidel step (its longest chain of blocks)
    int ensure_pgs();
    int solve_pgs();
    void split_config_changed();
    int scene_solve_info(float* alpha, int32_t* sweeps, int32_t n);
    // prescribed static motion for the coming step (Trajectory::update); device record and flags,
    // and their host copy until a step consumes them
    double* smot = nullptr;
    int32_t* smflag = nullptr;
    std::vector<double> h_smot;
    std::vector<int32_t> h_smflag;
    bool smotion_pending = false;
    int set_static_motion(int32_t count, const int32_t* idx, const double* pos, const double* quat,
                          const double* vel, const double* omega);
    int get_static_state(double* pos, double* quat, double* vel, double* omega);
    int load_scene(const cdx_scene& s);
    int ensure_tmp(int64_t n);
    int ensure_contacts(int64_t need);
    int collide64();
    int setup64();
    int solve64();
    int step64();
    int nfl_rows();
    int step(int nsteps);
    int get_state(double* pos, double* quat, double* vel, double* omega);
    int set_state(const double* pos, const double* quat, const double* vel, const double* omega);
    int get_contacts(int32_t* ia, int32_t* ib, double* point, double* lambda, double* normal, int32_t* count);
    void fill_stats(cdx_stats* s);
    double solve_bytes_per_iter() const;

    // split-precision form (engine_split.cpp)
    int step_split();
    void destroy_split();
    int get_contacts_split(int32_t* ia, int32_t* ib, double* point, double* lambda, double* normal, int32_t* count);
    // the warm-start memory of the next step (the contacts of a last step: pair ids, points, impulses)
    int set_contacts(int32_t n, const int32_t* ia, const int32_t* ib, const double* point, const double* lambda);
    int set_contacts_split(const std::vector<int64_t>& order, const int32_t* ia, const int32_t* ib,
                           const double* point, const double* lambda);
    bool contacts_loaded = false;  // the memory came from set_contacts (no normals until the next step)
    double split_bytes_per_iter() const;
    int split_variant() const;
    int split_sweep_variant() const;
    int split_tune_runs() const;
    int split_redos() const;
    int64_t split_graph_steps() const;
    int time_sweeps(int n, double* msc, double* msb, double* bc, double* bb);
};

struct cdx_ctx {
    Engine eng;
};
