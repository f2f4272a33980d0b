/*
 * Oracle for the contact hot path: a CPU, FP64 restatement of CardilloCxx's Moreau midpoint step
 * for sphere scenes (grid broad phase, sphere-sphere / -halfspace / -drum / -cylinder / -box narrow phase,
 * projected Jacobi over disk-shaped Coulomb cones, velocity and quaternion update).
 *
 * TEST INFRASTRUCTURE ONLY. Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
 * may load this library, and only as the checker or the timed CPU baseline. The product path
 * (cardillocxx_gb300) never calls it.
 *
 * Parity status: UNPINNED. The reference cannot be built here (Eigen 5.0.1, EnTT 3.13.2 and
 * coal 3.0.4 are absent and there is no network), and it ships no tests, golden vectors or
 * fixtures for this path. This file restates the reference's algorithm from its source; it is
 * pinned by analytic known-answer tests (free fall, resting load m*g, sliding deceleration mu*g,
 * projection branches) and its own frozen fixtures.
 *
 * Layouts match include/cdx.h's cdx_scene (interleaved xyz per body on the host).
 */
#ifndef CDX_ORACLE_H
#define CDX_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct or_config {
    double sim_dt;
    double sim_gravity[3];
    double moreau_theta;
    int32_t friction_enable;
    int32_t friction_combine; /* 0 min, 1 arith, 2 geom */
    int32_t pj_max_iterations;
    int32_t pj_warmstart;
    double pj_tol_abs;
    double pj_tol_rel;
    double pj_alpha;
    double collision_security_margin;
    double collision_match_max_dist;
    double residual_tol;   /* new complementarity-residual stop rule; 0 = off */
    int32_t omp_mode;      /* 0 = faithful (OpenMP on the projection only), 1 = all loops */
    int32_t num_threads;   /* 0 = OpenMP default */
    int32_t pj_nesterov;                 /* pj.nesterov */
    double pj_nesterov_beta_threshold;   /* pj.nesterov_beta_threshold */
    int32_t pj_nesterov_restart_limit;   /* pj.nesterov_restart_limit */
    int32_t pj_chebyshev;                /* pj.chebyshev */
    int32_t pj_anderson;                 /* pj.anderson */
    int32_t pj_anderson_m;               /* pj.anderson_m */
    int32_t pj_rdiag_true_delassus;      /* pj.rdiag_true_delassus */
    int32_t moreau_implicit_gyroscopy;   /* moreau.implicit_gyroscopy */
    int32_t solver_type;                 /* solver.type: 0 projected_jacobi, 1 condensed, 2 projected_gauss_seidel */
    int32_t condensed_sweep_mode;        /* condensed.sweep_mode: 0 gauss_seidel, 1 jacobi, 2 colored (3 chaotic is not restated) */
    double pj_relaxation;                /* pj.relaxation (condensed and PGS multiply it with pj.alpha) */
    int32_t pad0;
    int32_t status;                      /* out: 0, or 4 when a solve diverged (non-finite residual) */
} or_config;

typedef struct or_scene {
    int32_t num_bodies;
    const double* pos;     /* [3N] */
    const double* quat;    /* [4N] x,y,z,w */
    const double* vel;     /* [3N] world */
    const double* omega;   /* [3N] body frame */
    const double* radius;  /* [N] */
    const double* mass;    /* [N] */
    const double* inertia; /* [N] isotropic inertia diagonal */
    const double* mu;      /* [N] */
    const double* rest_n;  /* [N] */
    const double* rest_t;  /* [N] */
    const int32_t* body_scene; /* [N] or NULL */
    int32_t num_statics;
    const int32_t* static_kind; /* 0 halfspace, 1 hollow drum, 2 solid cylinder, 3 solid box */
    const double* static_pos;   /* [3S] */
    const double* static_quat;  /* [4S] */
    const double* static_vel;   /* [3S] world */
    const double* static_omega; /* [3S] body frame */
    const double* static_dir;   /* [3S] halfspace normal / drum axis (world) */
    const double* static_radius;/* [S] drum radius */
    const double* static_mu;
    const double* static_rest_n;
    const double* static_rest_t;
    const int32_t* static_scene; /* [S] or NULL */
    int32_t num_scenes;
    const double* static_half_length; /* [S] cylinder half length, or NULL */
    const double* static_half_extents; /* [3S] box half extents, or NULL */
} or_scene;

typedef struct or_stats {
    int32_t num_contacts;
    int32_t num_rows;
    int32_t iterations;
    double residual;       /* complementarity residual of the final state */
    double residual_last;  /* residual measured inside the last sweep */
} or_stats;

void* or_create(const or_config* cfg, const or_scene* scene);
void or_destroy(void* h);
/* prescribed static motion for the next step (Trajectory::update); NULL arrays leave that part */
void or_set_static_motion(void* h, int32_t count, const int32_t* statics, const double* pos, const double* quat,
                          const double* vel, const double* omega);
void or_get_static_state(void* h, double* pos, double* quat, double* vel, double* omega);
int or_step(void* h, int32_t nsteps);
void or_get_state(void* h, double* pos, double* quat, double* vel, double* omega);
void or_get_stats(void* h, or_stats* out);
/* contacts of the last step, canonical order: ids (statics first, then spheres offset by S),
 * contact points, impulses (n,t1,t2), normals */
int32_t or_get_contacts(void* h, int32_t* id_a, int32_t* id_b, double* point, double* lambda, double* normal);
/* the warm-start memory of the next step: contacts of a last step (id pairs, points, impulses) */
void or_set_contacts(void* h, int32_t n, const int32_t* id_a, const int32_t* id_b, const double* point,
                     const double* lambda);
/* per-iteration impulse trace of the next step: after or_set_trace(h,1) the next step records
 * lambda (rows in canonical contact order, 3 per contact) after every sweep */
void or_set_trace(void* h, int32_t on);
int32_t or_get_trace(void* h, double* out, int64_t max_values);

/* Solver-level drop-in (ProjectedJacobiSolver::solve with S = diag(M)):
 * W given as CSR (rows x nv), per-row contact bias, mu (at normal rows), restitution;
 * nfl = number of leading frictionless rows (1 row per contact), the rest are 3-row blocks.
 * x_out = solved velocities, lambda_inout = warm start in / impulses out. Returns iterations. */
/* the solver-level drop-in with a configuration (loop, block preconditioner, stop rules) */
int32_t or_pj_solve_csr_cfg(const or_config* cfg, int32_t nrows, int32_t nv, int32_t nfl, const int32_t* row_ptr,
                            const int32_t* col, const double* val, const double* contact_bias, const double* mu,
                            const double* restitution, const double* minv, const double* mdiag, const double* v,
                            const double* f_ext, const double* f_gyro, double dt, double* lambda_inout,
                            double* x_out);
/* the Delassus block inverse of pj.rdiag_true_delassus (n <= 3, row-major); returns 1 when the
 * block counts as diagonal, 0 otherwise, -1 for a bad size */
int32_t or_block_inverse(const double* A, int32_t n, double* X);
int32_t or_pj_solve_csr(int32_t nrows, int32_t nv, int32_t nfl, const int32_t* row_ptr, const int32_t* col,
                        const double* val, const double* contact_bias, const double* mu, const double* restitution,
                        const double* minv, const double* mdiag, const double* v, const double* f_ext,
                        const double* f_gyro, double dt, double alpha, int32_t max_iter, double tol_abs,
                        double tol_rel, double* lambda_inout, double* x_out);

/* FP64 adjoint of the world-frame sphere step (cdx_adjoint.cpp): scenes of spheres and halfspaces,
 * K fixed sweeps from lambda = 0, per-scene friction coefficient. */
typedef struct or_adj_problem {
    int32_t num_bodies;
    const double* radius;       /* [N] */
    const double* mass;         /* [N] */
    const double* inertia;      /* [N] */
    const int32_t* body_scene;  /* [N] or NULL */
    int32_t num_scenes;
    int32_t num_statics;        /* halfspaces */
    const double* static_dir;   /* [3S] outward normal */
    const double* static_pos;   /* [3S] a point on the plane */
    const int32_t* static_scene;/* [S] or NULL */
    double dt;
    double gravity[3];
    double theta;
    double alpha;
    int32_t iterations;
    double margin;
} or_adj_problem;

void* or_adj_create(const or_adj_problem* p);
void or_adj_destroy(void* h);
/* x, v, omega_world: [3N] each; mu: [num_scenes] */
int32_t or_adj_rollout(void* h, int32_t nsteps, const double* x0, const double* v0, const double* w0,
                       const double* mu_scene, double* xT, double* vT, double* wT);
/* gradient of <gxT, xT> + <gvT, vT> + <gwT, wT> with respect to x0, v0, w0 and mu */
int32_t or_adj_gradient(void* h, int32_t nsteps, const double* x0, const double* v0, const double* w0,
                        const double* mu_scene, const double* gxT, const double* gvT, const double* gwT, double* gx0,
                        double* gv0, double* gw0, double* gmu);

#ifdef __cplusplus
}
#endif
#endif
