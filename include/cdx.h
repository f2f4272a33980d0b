/*
 * cdx -- GB300-native contact hot path of CardilloCxx behind a thin C ABI.
 *
 * The path is the Moreau midpoint step for sphere scenes: uniform-grid broad phase,
 * sphere-sphere / sphere-halfspace / sphere-drum narrow phase, projected Jacobi over disk-shaped
 * Coulomb cones applied matrix-free as G M^-1 G^T, then the velocity and quaternion update.
 * Kernels are hand-written CUDA for sm_103a; the host side is C++.
 *
 * Conventions
 *   - All functions return an int status (CDX_OK = 0). cdx_last_error(ctx) holds the message.
 *   - Plain pointers and sizes only. Host arrays passed in are borrowed for the call.
 *   - Interleaved host layouts: positions/velocities [3*N] (x,y,z per body), quaternions [4*N]
 *     (x,y,z,w), angular velocities in the body frame (as the reference's C_AngularVelocity3).
 *   - Entity ids (contacts, warm start): static shapes 0..S-1, then sphere i has id S+i.
 *   - One context per host thread; each context owns its device memory and one CUDA stream.
 *   - No call allocates device memory on the per-step path except when the contact buffers
 *     must grow (reported in cdx_stats.reallocations).
 */
#ifndef CDX_H
#define CDX_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CDX_OK 0
#define CDX_ERR_ARG 1
#define CDX_ERR_CUDA 2
#define CDX_ERR_OVERFLOW 3
#define CDX_ERR_NONFINITE 4
#define CDX_ERR_TIMEOUT 5
#define CDX_ERR_UNSUPPORTED 6
#define CDX_ERR_STATE 7

#define CDX_PRECISION_FP64 0  /* plain method: FP64 everywhere, bit-reproducible vs the oracle */
#define CDX_PRECISION_SPLIT 1 /* FP32 contact/Delassus/projection, FP64 state and residual check */

#define CDX_STATIC_HALFSPACE 0
#define CDX_STATIC_DRUM 1 /* hollow cylinder: spheres touch its inner wall */
#define CDX_STATIC_CYLINDER 2 /* solid finite cylinder (the reference's C_RB_Cylinder, coal::Cylinder):
                                 spheres touch its side, its caps or their rims */
#define CDX_STATIC_BOX 3      /* solid box (the reference's static C_RB_Cube, coal::Box): spheres touch its
                                 faces, edges or corners */

/* Engine configuration. Field names follow the reference's config keys
 * (src/config/config.hpp:12-237, parsed by ConfigReader::fromFile, src/config/config.cpp:22-420).
 * Keys after the gpu_ prefix are new. */
typedef struct cdx_config {
    double sim_dt;                    /* sim.dt */
    double sim_T;                     /* sim.T */
    double sim_gravity[3];            /* sim.gravity */
    double moreau_theta;              /* moreau.theta (0.5 = midpoint) */
    int32_t moreau_implicit_gyroscopy;/* moreau.implicit_gyroscopy: for isotropic spheres the linearised
                                         gyroscopic block is exactly zero, so this only drops dt f_gyro */
    int32_t friction_enable;          /* friction.enable */
    int32_t friction_combine;         /* friction.combine: 0 min, 1 arith, 2 geom */
    double friction_default_mu;       /* friction.default_mu (scene generators) */
    double restitution_default_normal;     /* restitution.default_normal */
    double restitution_default_tangential; /* restitution.default_tangential */
    int32_t pj_max_iterations;        /* pj.max_iterations */
    int32_t pj_warmstart;             /* pj.warmstart */
    double pj_tol_abs;                /* pj.tol_abs */
    double pj_tol_rel;                /* pj.tol_rel */
    double pj_alpha;                  /* pj.alpha */
    double pj_relaxation;             /* pj.relaxation (accepted, unused by PJ as in the reference) */
    int32_t solver_type;              /* solver.type: 0 projected_jacobi, 1 condensed (plain FP64 method;
                                         sweep modes gauss_seidel, jacobi, colored), 2 projected_gauss_seidel
                                         (plain FP64 method, plain loop) */
    double collision_security_margin; /* collision.security_margin */
    double collision_match_max_dist;  /* collision.match_max_dist */
    int32_t collision_broadphase;     /* collision.broadphase: 0 uniform_grid (any reference value maps here) */
    int32_t gpu_precision;            /* gpu.precision: CDX_PRECISION_FP64 | CDX_PRECISION_SPLIT */
    double gpu_residual_tol;          /* gpu.residual_tol: stop when the complementarity residual <= tol (0 off) */
    int32_t gpu_check_every;          /* gpu.check_every: the split-form stop rule runs every k sweeps */
    int32_t gpu_block;                /* gpu.block: reserved, ignored (each kernel has its own launch shape) */
    double gpu_contact_capacity_factor; /* gpu.contact_capacity: initial contact slots per body */
    int32_t gpu_use_graph;            /* gpu.graph: capture the solver loop in a CUDA graph (split form) */
    int32_t gpu_autotune;             /* gpu.autotune: pick the contact-sweep launch shape by timing (split form) */
    int32_t gpu_sweep_variant;        /* gpu.sweep_variant: pin launch shape k (split form; -1 = default/autotuned) */
    int32_t gpu_sync_counts;          /* gpu.sync_counts: every split step stops for the host to size its contact buffers */
    /* accelerated loops of ProjectedJacobiSolver (config.hpp:85-110; projected_jacobi.cpp:179-222,
     * 242-314, 379-449): Nesterov > Chebyshev > Anderson in the plain FP64 method; the split form runs
     * Nesterov and the standard loop's pj.tol_abs/pj.tol_rel exit in its cooperative solve and refuses
     * Chebyshev and Anderson with CDX_ERR_UNSUPPORTED */
    int32_t pj_nesterov;              /* pj.nesterov */
    double pj_nesterov_beta_threshold; /* pj.nesterov_beta_threshold */
    int32_t pj_nesterov_restart_limit; /* pj.nesterov_restart_limit */
    int32_t pj_chebyshev;             /* pj.chebyshev */
    int32_t pj_anderson;              /* pj.anderson */
    int32_t pj_anderson_m;            /* pj.anderson_m: history window (>= 1) */
    int32_t pj_rdiag_true_delassus;   /* pj.rdiag_true_delassus: per-contact Delassus block preconditioner (plain FP64;
                                         the split form's row scale is that block for sphere contacts) */
    /* frame output (PhysicsPipeline, physics_pipeline.cpp:62-113; config.hpp:20-23) */
    int32_t output_interval_steps;          /* output.interval_steps: VTK frames every k steps (0 = off) */
    int32_t output_write_contact_manifolds; /* output.write_contact_manifolds */
    char output_folder[256];                /* output.folder */
    char output_filename_prefix[128];       /* output.filename_prefix */
    int32_t gpu_coop_smem_contacts;         /* gpu.coop_smem_contacts: cap on the contacts a block of the
                                               cooperative solve keeps in shared memory (0 = all that fit) */
    int32_t gpu_coop_blocks;                /* gpu.coop_blocks: blocks of the cooperative solve (0 = one per SM;
                                               more than that is capped) */
    int32_t gpu_tune_alpha;                 /* gpu.tune_alpha: batched scenes (split form): the autotuner also picks
                                               each scene's pj.alpha from a candidate set by trial solves of the
                                               same step (fewest sweeps to gpu.residual_tol, else the lowest
                                               residual at the sweep cap); off keeps pj.alpha everywhere */
    int64_t gpu_coop_wait_ns;               /* gpu.coop_wait_ns: longest wait of a block of the cooperative solve
                                               at a grid barrier before the step fails with CDX_ERR_TIMEOUT
                                               (0 = 0.2 s) */
    int32_t condensed_sweep_mode;           /* condensed.sweep_mode: 0 gauss_seidel (default), 1 jacobi,
                                               2 colored (these three run on the GPU), 3 chaotic */
    int32_t gpu_tune_alpha_every;           /* gpu.tune_alpha_every: steps between two tunings of the scenes' alpha */
} cdx_config;

/* Scene: dynamic spheres plus static shapes (halfspaces, drums, cylinders, boxes). Bodies of one scene are
 * contiguous; body_scene/static_scene may be NULL for a single scene. */
typedef struct cdx_scene {
    int32_t num_bodies;
    const double* pos;     /* [3N] */
    const double* quat;    /* [4N] x,y,z,w */
    const double* vel;     /* [3N] world frame */
    const double* omega;   /* [3N] body frame */
    const double* radius;  /* [N] */
    const double* mass;    /* [N] */
    const double* inertia; /* [N] isotropic inertia diagonal */
    const double* mu;      /* [N] friction coefficient (C_Friction) */
    const double* rest_n;  /* [N] normal restitution */
    const double* rest_t;  /* [N] tangential restitution */
    const int32_t* body_scene; /* [N] nondecreasing, or NULL */
    int32_t num_statics;
    const int32_t* static_kind; /* CDX_STATIC_* */
    const double* static_pos;   /* [3S] halfspace point / drum axis point / cylinder or box centre */
    const double* static_quat;  /* [4S] */
    const double* static_vel;   /* [3S] world-frame velocity (enters the contact bias) */
    const double* static_omega; /* [3S] body-frame angular velocity (moving walls) */
    const double* static_dir;   /* [3S] halfspace normal / drum or cylinder axis, world frame at load (a
                                   cylinder's axis then turns with its orientation; ignored for boxes) */
    const double* static_radius;/* [S] drum or cylinder radius (ignored for halfspaces) */
    const double* static_mu;
    const double* static_rest_n;
    const double* static_rest_t;
    const int32_t* static_scene; /* [S] nondecreasing, or NULL */
    int32_t num_scenes;
    const double* static_half_length; /* [S] cylinder half length along its axis (C_RB_Cylinder::halfLength;
                                         ignored for other kinds; may be NULL when there is no cylinder) */
    const double* static_half_extents; /* [3S] box half extents along the box's own axes, which are the
                                          columns of static_quat's rotation (C_RB_Cube::halfExtents; ignored
                                          for other kinds; may be NULL when there is no box) */
} cdx_scene;

typedef struct cdx_stats {
    int64_t steps;
    int32_t num_contacts;      /* last step */
    int32_t num_rows;          /* contact rows (3 per frictional contact, 1 otherwise) */
    int32_t iterations;        /* PJ sweeps of the last step */
    int32_t reallocations;     /* contact-buffer growths so far */
    double residual;           /* FP64 complementarity residual of the final state, last step */
    double residual_last;      /* residual measured inside the last sweep */
    double ms_collision;       /* device time of the last step by phase (CUDA events; 0 if timing off) */
    double ms_setup;
    double ms_solve;
    double ms_integrate;
    double solve_bytes_per_iter; /* algorithmic bytes of one sweep (per-contact and per-body words) */
    int64_t kernel_launches;   /* cdx kernels launched so far */
    int32_t contact_variant;   /* split form: launch shape of the contact sweep chosen by the autotuner */
    int32_t autotune_runs;     /* split form: times the autotuner ran */
    int32_t redone_steps;      /* split form: steps undone and redone because their contacts outgrew the buffers */
    int64_t graph_steps;       /* split form: steps replayed whole from a captured CUDA graph */
    int32_t sweep_variant;     /* split form: the shape cdx_time_sweeps times (the whole-problem solver,
                                  also when a batched-scenes shape ran the step) */
    int32_t levels;            /* projected Gauss-Seidel: levels of the last step's sweep (its longest
                                  chain of dependent blocks) */
} cdx_stats;

typedef struct cdx_ctx cdx_ctx;

/* ---- configuration (ConfigReader::fromFile semantics: unknown keys ignored, bad values keep the
 * default, pj./solver. prefixes accepted) ---- */
int cdx_config_default(cdx_config* cfg);
int cdx_config_set(cdx_config* cfg, const char* key, const char* value); /* config.cpp:41-415 */
int cdx_config_from_file(const char* path, cdx_config* cfg);              /* config.cpp:22-40 */

/* ---- engine (the integrator-level drop-in: MoreauIntegrator::step, moreau.cpp:6-13, behind
 * IntegrationBase::step, integration_base.hpp:19) ---- */
int cdx_create(const cdx_config* cfg, cdx_ctx** out);
void cdx_destroy(cdx_ctx* ctx);
/* Replace the configuration between steps, from the next step on: ProjectedJacobiSolver keeps a
 * reference to the Config and reads its pj.* settings at every solve (projected_jacobi.cpp:451-500).
 * gpu.precision cannot change (CDX_ERR_STATE); output.* keep their values from cdx_create. */
int cdx_set_config(cdx_ctx* ctx, const cdx_config* cfg);
const char* cdx_last_error(const cdx_ctx* ctx);
int cdx_load_scene(cdx_ctx* ctx, const cdx_scene* scene);
int cdx_step(cdx_ctx* ctx, int32_t nsteps);
int cdx_synchronize(cdx_ctx* ctx);
int cdx_get_state(cdx_ctx* ctx, double* pos, double* quat, double* vel, double* omega);
int cdx_set_state(cdx_ctx* ctx, const double* pos, const double* quat, const double* vel, const double* omega);
int cdx_get_stats(cdx_ctx* ctx, cdx_stats* out);
/* contacts of the last step in canonical order (entity ids, points, impulses n/t1/t2, normals);
 * pass NULL arrays to query the count */
int cdx_get_contacts(cdx_ctx* ctx, int32_t* id_a, int32_t* id_b, double* point, double* lambda, double* normal,
                     int32_t* count);
/* Load the warm-start memory the next step matches against: the contacts of a last step (entity id
 * pairs, each at most once, points and impulses n/t1/t2 as cdx_get_contacts returns them). The
 * reference keeps this memory in its ContactTracker (contact_tracker.cpp:11-72) and the solver
 * copies matched impulses in (WarmstartProvider::applyWarmstart, warmstart.hpp:26-39); with the
 * state calls it checkpoints and resumes a run, warm start included. Until the next step
 * cdx_get_contacts returns this memory with zero normals. */
int cdx_set_contacts(cdx_ctx* ctx, int32_t count, const int32_t* id_a, const int32_t* id_b, const double* point,
                     const double* lambda);
/* Prescribed motion of statics for the next step: what Trajectory::update (trajectory.cpp:69-120)
 * sets from a static's position and velocity callbacks, which run on the host. For each listed
 * static the given pose (position, unit quaternion x,y,z,w) and twist (world-frame velocity,
 * body-frame angular velocity) replace its own after the first drift and before contact detection,
 * where updateStateDependentTerms runs the trajectories (dynamics_assembler.cpp:515-522); the
 * second drift then moves it by the new twist, and the twist stays until changed. Any of pos, quat,
 * vel, omega may be NULL (left as they are). As in the reference a halfspace's plane stays where
 * it was built (CollisionCoal::applyTransforms, collision_coal.cpp:386-391): its motion reaches the
 * contacts through its velocity. Calls before one step accumulate; the step consumes them. */
int cdx_set_static_motion(cdx_ctx* ctx, int32_t count, const int32_t* statics, const double* pos,
                          const double* quat, const double* vel, const double* omega);
/* the statics' current pose and twist (arrays of 3S / 4S / 3S / 3S, any may be NULL) */
int cdx_get_static_state(cdx_ctx* ctx, double* pos, double* quat, double* vel, double* omega);
/* Batched scenes (split form, per-scene solve): each scene's pj.alpha (as gpu.tune_alpha chose it;
 * pj.alpha without it) and the sweeps each scene took in its last solve (either pointer may be
 * NULL; n scenes at most). No reference counterpart: the reference runs one alpha for every
 * contact. CDX_ERR_STATE before a per-scene solve has run. */
int cdx_get_scene_solve(cdx_ctx* ctx, float* alpha, int32_t* sweeps, int32_t n);
/* track a sphere in <output.folder>/<output.filename_prefix>_tracked.csv, one row every step
 * (World::track, world.cpp:38-45; CsvWriter::writeTrackedState, csv_writer.hpp:43-52) */
int cdx_track(cdx_ctx* ctx, int32_t body, const char* name);
/* wait until the background writer has written every queued frame; CDX_ERR_STATE (with
 * cdx_last_error) when a file could not be written */
int cdx_output_flush(cdx_ctx* ctx);
/* per-sweep impulse trace of the next step (rows in solver order), for parity checks */
int cdx_set_trace(cdx_ctx* ctx, int32_t on);
int cdx_get_trace(cdx_ctx* ctx, double* out, int64_t max_values, int64_t* num_values);
int cdx_set_timing(cdx_ctx* ctx, int32_t on);
/* the stream the engine launches on (cudaStream_t as void*) */
void* cdx_stream(cdx_ctx* ctx);
/* Re-run `n` projected-Jacobi sweeps on the last step's contacts, timing every launch of the
 * contact kernel and of the body kernel with CUDA events on the engine's stream. Returns the
 * average milliseconds per launch and the algorithmic bytes one launch moves. Leaves the solver
 * temporaries (not the body state) modified: call it after the steps being measured. */
int cdx_time_sweeps(cdx_ctx* ctx, int32_t n, double* ms_contact, double* ms_body, double* bytes_contact,
                    double* bytes_body);
/* Launch shapes of the split-form sweep: how many there are, and the name of shape k
 * ("u<contacts per thread>-t<threads>-b<blocks per SM>-g<scatter mode>-w<waves>"; "?" out of range).
 * gpu.sweep_variant pins one of them. No counterpart in the reference (its solver has one loop). */
int32_t cdx_split_variant_count(void);
const char* cdx_split_variant_name(int32_t k);

/* ---- differentiable rollout (the step's adjoint)
 * The reference has no adjoint; the differentiated map is its step for sphere scenes,
 * MoreauIntegrator::step (src/physics/integration/moreau.cpp:6-13) with the contact rows of
 * dynamics_assembler.cpp:211-332 and ProjectedJacobiSolver::solve (projected_jacobi.cpp:451-500),
 * written on world-frame angular velocities (for a sphere the orientation does not enter the
 * motion). Scope: spheres and halfspaces, scenes of at most 1024 spheres, a fixed sweep count
 * (pj.max_iterations) from lambda = 0 (no warm start), one friction coefficient per scene.
 * Config keys used: sim.dt, sim.gravity, moreau.theta, pj.alpha, pj.max_iterations,
 * collision.security_margin, gpu.contact_capacity (contact slots per sphere).
 * cdx_adj_forward keeps the state every checkpoint_every steps; cdx_adj_backward recomputes each
 * segment from its checkpoint and each step's sweeps from the step's input, so memory does not grow
 * with the rollout length. States are [3N] arrays: x, v, omega (world frame); mu is [num_scenes]. */
typedef struct cdx_adj cdx_adj;
int cdx_adj_create(const cdx_config* cfg, const cdx_scene* scene, int32_t checkpoint_every, cdx_adj** out);
void cdx_adj_destroy(cdx_adj* h);
const char* cdx_adj_last_error(cdx_adj* h);
int cdx_adj_forward(cdx_adj* h, int32_t nsteps, const double* x0, const double* v0, const double* w0,
                    const double* mu_scene, double* xT, double* vT, double* wT);
/* gradient of <gxT, xT> + <gvT, vT> + <gwT, wT> (the last forward's outputs) with respect to
 * x0, v0, w0 and mu_scene */
int cdx_adj_backward(cdx_adj* h, const double* gxT, const double* gvT, const double* gwT, double* gx0, double* gv0,
                     double* gw0, double* gmu);
int cdx_adj_info(cdx_adj* h, int64_t* contact_slots, int64_t* device_bytes, int32_t* checkpoints);
/* per scene, the contacts of the last forward summed over its steps: two rollouts with equal sums
 * saw the same contact events (the loss is smooth between such events, not across them) */
int cdx_adj_contact_counts(cdx_adj* h, int64_t* per_scene);

/* ---- solver-level drop-in: ProjectedJacobiSolver::solve(dt, theta)
 * (src/physics/solver/projected_jacobi.cpp:451-500) with S = diag(M) (pj_assembler.cpp:127-182).
 * Inputs are what the solver pulls from DynamicsAssembler (dynamics_assembler.hpp:23-94):
 * W as CSR (nrows x nv; the first nfl rows are frictionless contacts, the rest 3-row frictional
 * blocks), contactVVec, muVec, restitutionVec, MinvDiag, MDiag, vVec, fVecExternal,
 * fVecGyroscopic. lambda_inout carries the warm start in and the impulses out; x_out receives
 * the stacked velocities. Host arrays; FP64; bit-reproducible vs the oracle. ---- */
int cdx_pj_solve_csr(cdx_ctx* ctx, int32_t nrows, int32_t nv, int32_t nfl, const int32_t* row_ptr,
                     const int32_t* col, const double* val, const double* contact_bias, const double* mu,
                     const double* restitution, const double* minv, const double* mdiag, const double* v,
                     const double* f_ext, const double* f_gyro, double dt, double alpha, int32_t max_iter,
                     double tol_abs, double tol_rel, double* lambda_inout, double* x_out, int32_t* iterations);
/* The same solve under a configuration, as ProjectedJacobiSolver reads it (projected_jacobi.cpp:
 * 451-500): pj.alpha, pj.max_iterations, pj.tol_abs, pj.tol_rel, the loop (pj.nesterov > pj.chebyshev >
 * pj.anderson > standard, with their parameters), pj.rdiag_true_delassus (per-contact Delassus
 * blocks; the three rows of a frictional contact must share their columns), gpu.residual_tol and
 * gpu.check_every. dt is the step of the solve (SolverBase::solve(dt, theta)). */
int cdx_pj_solve_csr_cfg(cdx_ctx* ctx, const cdx_config* cfg, int32_t nrows, int32_t nv, int32_t nfl,
                         const int32_t* row_ptr, const int32_t* col, const double* val, const double* contact_bias,
                         const double* mu, const double* restitution, const double* minv, const double* mdiag,
                         const double* v, const double* f_ext, const double* f_gyro, double dt, double* lambda_inout,
                         double* x_out, int32_t* iterations);

/* ---- solver-level solve for callers that cannot allocate device memory ----
 * No counterpart in the reference. Same inputs, outputs and results as cdx_pj_solve_csr, but no
 * context and no cudaMalloc/cudaFree or other allocating call: every device buffer (staged inputs,
 * work arrays, results) lives in one file-scope __device__ array of CDX_NOALLOC_SCRATCH_BYTES that
 * each GPU loading the library keeps until exit. For hosts that own all device memory themselves
 * (pre-reserved pools, real-time loops, code where allocation calls are not allowed).
 *   - stream: cudaStream_t as void* (NULL = the legacy default stream).
 *   - The first call on a device (with that device current) looks up the array's address with
 *     cudaGetSymbolAddress and keeps it; make it before any stream capture. cudaDeviceReset
 *     discards the array, and the kept address with it: do not reset the device between calls.
 *   - A call returns once its work on the stream has finished.
 *   - Problems that do not fit return CDX_ERR_OVERFLOW with the message in err (errlen bytes).
 *   - All calls share the array: calls that overlap on the GPU race; run them one at a time. */
#define CDX_NOALLOC_SCRATCH_BYTES (16u << 20)
int cdx_pj_solve_csr_noalloc(void* stream, int32_t nrows, int32_t nv, int32_t nfl, const int32_t* row_ptr,
                             const int32_t* col, const double* val, const double* contact_bias, const double* mu,
                             const double* restitution, const double* minv, const double* mdiag, const double* v,
                             const double* f_ext, const double* f_gyro, double dt, double alpha, int32_t max_iter,
                             double tol_abs, double tol_rel, double* lambda_inout, double* x_out, int32_t* iterations,
                             char* err, int32_t errlen);

/* ---- diagnostics: the FP64 Newton-Raphson reciprocal and reciprocal square root of the split
 * form's final pass, evaluated on the device for host-side checks against IEEE results ---- */
int cdx_selftest_nr64(cdx_ctx* ctx, int32_t n, const double* x, double* rcp, double* rsqrt);

/* ---- seeded scene generators for the benchmark scenes (host only) ---- */
typedef struct cdx_gen_params {
    int32_t kind;          /* 0 box pile(s), 1 rotating drum */
    int32_t num_scenes;    /* box piles: independent scenes laid out side by side */
    int32_t num_bodies;    /* bodies per scene (ignored when nb_lo > 0) */
    int32_t nb_lo, nb_hi;  /* per-scene body count log-uniform in [nb_lo, nb_hi] (0 = off) */
    double r_lo, r_hi;     /* radius uniform in [r_lo, r_hi] */
    double density;
    double box[3];         /* box extents (x, y, z) per scene */
    double mu, mu_lo, mu_hi; /* friction; per-scene uniform in [mu_lo, mu_hi] when mu_hi > mu_lo */
    double v_sigma;        /* initial velocity N(0, v_sigma^2) per component */
    double drum_radius, drum_length, drum_omega;
    uint64_t seed;
    int32_t max_attempts;  /* rejection-sampling attempts per body */
} cdx_gen_params;

typedef struct cdx_gen_scene cdx_gen_scene;
int cdx_gen_create(const cdx_gen_params* p, cdx_gen_scene** out);
/* fills a cdx_scene view whose arrays live in the generated object */
int cdx_gen_view(const cdx_gen_scene* g, cdx_scene* view);
void cdx_gen_destroy(cdx_gen_scene* g);

#ifdef __cplusplus
}
#endif
#endif /* CDX_H */
