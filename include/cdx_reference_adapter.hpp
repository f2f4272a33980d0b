// Reference-side adapters: how CardilloCxx binds the cdx C ABI at its two plugin points.
//
// This header only compiles inside the CardilloCxx source tree (it includes the reference's
// Eigen/EnTT-based headers), so it is guarded by CDX_WITH_CARDILLO. It is not part of libcdx.
//
//  * GpuProjectedJacobiSolver : cardillo::solver::SolverBase
//      replaces ProjectedJacobiSolver (src/physics/solver/projected_jacobi.hpp:22-65) and is
//      selected in PhysicsPipeline's solver factory (src/physics/pipeline/physics_pipeline.cpp:34-51).
//      It pulls the same inputs from DynamicsAssembler (dynamics_assembler.hpp:23-94), applies
//      and stores the warm start with WarmstartProvider (warmstart.hpp:26-56), and calls
//      cdx_pj_solve_csr_cfg (include/cdx.h) with the reference's pj.* settings (the loop, the
//      block preconditioner, the tolerances) for the sweeps.
//  * GpuMoreauIntegrator : cardillo::integration::IntegrationBase
//      replaces MoreauIntegrator (src/physics/integration/moreau.cpp:6-13) for sphere scenes:
//      the whole step (collision, contact rows, PJ, drift) runs in cdx_step; the ECS components
//      of the spheres are uploaded before and written back after each step.
#pragma once
#ifdef CDX_WITH_CARDILLO

#include <stdexcept>
#include <string>
#include <vector>

#include "cdx.h"
#include "physics/ecs_types.hpp"
#include "physics/integration/integration_base.hpp"
#include "physics/solver/solver_base.hpp"
#include "physics/solver/warmstart.hpp"
#include "physics/synchronization/trajectory.hpp"
#include "physics/world.hpp"

namespace cardillo::solver {

class GpuProjectedJacobiSolver : public SolverBase {
   public:
    GpuProjectedJacobiSolver(physics::DynamicsAssembler& dyn, const config::Config& cfg) : m_dyn(dyn), m_cfg(cfg) {
        cdx_config c;
        cdx_config_default(&c);
        c.gpu_check_every = 10;
        if (cdx_create(&c, &m_ctx) != CDX_OK) {
            const std::string msg = m_ctx ? cdx_last_error(m_ctx) : "cdx_create failed";
            cdx_destroy(m_ctx);
            throw std::runtime_error("GpuProjectedJacobiSolver: " + msg);
        }
    }
    ~GpuProjectedJacobiSolver() override { cdx_destroy(m_ctx); }

    VectorXr solve(real_t dt, real_t theta) override {
        (void)theta;  // S = diag(M): theta only enters through spring/damper rows
        if (m_dyn.numSprings() > 0 || m_dyn.numDampers() > 0)
            throw std::runtime_error("GpuProjectedJacobiSolver: springs and dampers are not on the GPU path");
        const int nv = (int)m_dyn.numV();
        const int nrows = m_dyn.numContactRows();
        const auto& W = m_dyn.W().asSparseRowMajor();  // compressed row-major CSR
        VectorXr p = VectorXr::Zero(nrows);
        if (m_cfg.pj_warmstart) WarmstartProvider::applyWarmstart(p, m_dyn);
        VectorXr f_gyro = m_cfg.moreau_implicit_gyroscopy ? VectorXr::Zero(nv) : m_dyn.fVecGyroscopic();
        VectorXr e = m_dyn.restitutionVec().head(nrows);
        VectorXr x(nv);
        int32_t iters = 0;
        // the reference's solver settings (config.hpp:79-112)
        cdx_config c;
        cdx_config_default(&c);
        c.pj_alpha = m_cfg.pj_alpha;
        c.pj_max_iterations = m_cfg.pj_max_iterations;
        c.pj_tol_abs = m_cfg.pj_tol_abs;
        c.pj_tol_rel = m_cfg.pj_tol_rel;
        c.pj_nesterov = m_cfg.pj_nesterov;
        c.pj_nesterov_beta_threshold = m_cfg.pj_nesterov_beta_threshold;
        c.pj_nesterov_restart_limit = m_cfg.pj_nesterov_restart_limit;
        c.pj_chebyshev = m_cfg.pj_chebyshev;
        c.pj_anderson = m_cfg.pj_anderson;
        c.pj_anderson_m = m_cfg.pj_anderson_m;
        c.pj_rdiag_true_delassus = m_cfg.pj_rdiag_true_delassus;
        c.gpu_check_every = 10;
        const int st = cdx_pj_solve_csr_cfg(m_ctx, &c, nrows, nv, m_dyn.numFrictionlessContacts(), W.outerIndexPtr(),
                                            W.innerIndexPtr(), W.valuePtr(), m_dyn.contactVVec().data(),
                                            m_dyn.muVec().data(), e.data(), m_dyn.MinvDiag().data(),
                                            m_dyn.MDiag().data(), m_dyn.vVec().data(), m_dyn.fVecExternal().data(),
                                            f_gyro.data(), dt, p.data(), x.data(), &iters);
        if (st != CDX_OK) throw std::runtime_error(std::string("GpuProjectedJacobiSolver: ") + cdx_last_error(m_ctx));
        m_last_iters = iters;
        WarmstartProvider::storeImpulse(p, m_dyn);
        return x;
    }

    const char* name() const override { return "GpuProjectedJacobi"; }

   private:
    physics::DynamicsAssembler& m_dyn;
    const config::Config& m_cfg;
    cdx_ctx* m_ctx = nullptr;
};

}  // namespace cardillo::solver

namespace cardillo::integration {

// Whole-step drop-in for sphere scenes: MoreauIntegrator::step (src/physics/integration/moreau.cpp:
// 6-13) behind IntegrationBase::step (integration_base.hpp:19). Selected where the pipeline builds
// its integrator (physics_pipeline.cpp:34-51), e.g. for integrator=gpu_moreau.
//  - Dynamic spheres are the entities with C_RB_Sphere, C_Radius and C_PhysicsObject; static
//    halfspaces the entities with C_RB_Plane and no C_PhysicsObject (the components
//    RigidBodyFactory::create gives them, rigid_body_factory.cpp:110-209). Entity ids in the
//    context: the statics first, then the spheres, each in view order.
//  - The scene is mirrored into one cdx context when the world's structure changes
//    (World::m_structure_dirty, consumed here because this step replaces the assembler's) or dt
//    changes. Each step uploads the spheres' state from the ECS (a user may have edited it),
//    runs cdx_step(1) (refreshState, the (1 - theta) h drift, collision and contact rows, the
//    projected Jacobi solve, writeVelocityToSystem and the theta h drift), and writes the new
//    state back into C_Position3, C_Orientation (setValue keeps the rotation in sync),
//    C_LinearVelocity3 and C_AngularVelocity3 (body frame). The warm-start memory stays in the
//    context across steps.
//  - Static solid cylinders are the entities with C_RB_Cylinder and no C_PhysicsObject: their axis
//    is the pose's local z (coal::Cylinder's), radius and half length from the component.
//  - Static boxes are the entities with C_RB_Cube and no C_PhysicsObject (the walls and the
//    trajectory-driven floor of the stacked_spheres scene): half extents from the component, the
//    box posed as coal poses it (makeTfFromEcs, collision_coal.cpp:43-64: orientation q * cube.q,
//    centre x + (q * cube.q) * cube.center). A box with a local offset (cube.center or cube.q not
//    the identity) that moves is not on this path (step() throws).
//  - Statics driven by a trajectory (C_StaticTrajectory): each step runs Trajectory::update
//    (trajectory.cpp:69-120; the reference runs it inside updateStateDependentTerms, after the first
//    drift, and what it computes does not depend on that drift) and hands the poses and twists it
//    set to cdx_set_static_motion, which applies them at the same point of the step; afterwards
//    their pose and twist come back from the context (cdx_get_static_state).
//  - Dynamic shapes other than spheres (boxes, meshes, capsules, cones, cylinders), dynamic planes, point
//    masses without C_RB_Sphere, constraints and soft bodies are not on this path: step() throws
//    std::runtime_error, as the reference's own components throw on what they cannot handle.
//  - precision: CDX_PRECISION_FP64 (bit-identical to the reference restatement) or
//    CDX_PRECISION_SPLIT (FP32 contacts and solve, FP64 state).
class GpuMoreauIntegrator : public IntegrationBase {
   public:
    GpuMoreauIntegrator(World& world, solver::SolverBase& solver, physics::DynamicsAssembler& dyn,
                        misc::TimingManager& timings, config::Config& config,
                        int32_t precision = CDX_PRECISION_FP64)
        : IntegrationBase(world, solver, dyn, timings, config), m_precision(precision) {}
    ~GpuMoreauIntegrator() override { cdx_destroy(m_ctx); }

    void step(real_t dt) override {
        if (!m_ctx || m_world.m_structure_dirty || dt != m_dt) rebuild(dt);
        auto& reg = m_world.ecs();
        const size_t n = m_spheres.size();
        for (size_t i = 0; i < n; ++i) {
            const entt::entity e = m_spheres[i];
            const auto& x = reg.get<C_Position3>(e).value;
            const auto& q = reg.get<C_Orientation>(e).value;
            const auto& v = reg.get<C_LinearVelocity3>(e).value;
            const auto& w = reg.get<C_AngularVelocity3>(e).value;
            for (int k = 0; k < 3; ++k) {
                m_pos[3 * i + k] = x[k];
                m_vel[3 * i + k] = v[k];
                m_omega[3 * i + k] = w[k];
            }
            m_quat[4 * i + 0] = q.x();
            m_quat[4 * i + 1] = q.y();
            m_quat[4 * i + 2] = q.z();
            m_quat[4 * i + 3] = q.w();
        }
        check(cdx_set_state(m_ctx, m_pos.data(), m_quat.data(), m_vel.data(), m_omega.data()));
        if (!m_traj.empty()) upload_trajectories(dt);
        check(cdx_step(m_ctx, 1));
        check(cdx_get_state(m_ctx, m_pos.data(), m_quat.data(), m_vel.data(), m_omega.data()));
        if (!m_traj.empty()) download_trajectories();
        for (size_t i = 0; i < n; ++i) {
            const entt::entity e = m_spheres[i];
            auto& x = reg.get<C_Position3>(e).value;
            auto& v = reg.get<C_LinearVelocity3>(e).value;
            auto& w = reg.get<C_AngularVelocity3>(e).value;
            for (int k = 0; k < 3; ++k) {
                x[k] = m_pos[3 * i + k];
                v[k] = m_vel[3 * i + k];
                w[k] = m_omega[3 * i + k];
            }
            reg.get<C_Orientation>(e).setValue(
                Quaternion4r(m_quat[4 * i + 3], m_quat[4 * i + 0], m_quat[4 * i + 1], m_quat[4 * i + 2]));
        }
    }

   private:
    // the poses (where a position callback exists) and twists Trajectory::update set, for this step
    void upload_trajectories(real_t dt) {
        physics::Trajectory::update(m_world, dt);
        auto& reg = m_world.ecs();
        std::vector<int32_t> with_pose, twist_only;
        std::vector<double> pos, quat, vel, omega, vel2, omega2;
        for (size_t t = 0; t < m_traj.size(); ++t) {
            const entt::entity e = m_traj[t];
            const auto& traj = reg.get<C_StaticTrajectory>(e);
            const auto& v = reg.get<C_LinearVelocity3>(e).value;
            const bool has_w = reg.all_of<C_AngularVelocity3>(e);
            const bool posed = traj.positionFunc.has_value();
            (posed ? with_pose : twist_only).push_back(m_traj_index[t]);
            auto& vv = posed ? vel : vel2;
            auto& ww = posed ? omega : omega2;
            for (int k = 0; k < 3; ++k) {
                vv.push_back(v[k]);
                ww.push_back(has_w ? reg.get<C_AngularVelocity3>(e).value[k] : 0.0);
            }
            if (posed) {
                const auto& x = reg.get<C_Position3>(e).value;
                const auto& q = reg.get<C_Orientation>(e).value;
                for (int k = 0; k < 3; ++k) pos.push_back(x[k]);
                quat.insert(quat.end(), {q.x(), q.y(), q.z(), q.w()});
            }
        }
        if (!with_pose.empty())
            check(cdx_set_static_motion(m_ctx, (int32_t)with_pose.size(), with_pose.data(), pos.data(), quat.data(),
                                        vel.data(), omega.data()));
        if (!twist_only.empty())
            check(cdx_set_static_motion(m_ctx, (int32_t)twist_only.size(), twist_only.data(), nullptr, nullptr,
                                        vel2.data(), omega2.data()));
    }

    // the trajectory statics' pose after the step's second drift, back into the ECS
    void download_trajectories() {
        auto& reg = m_world.ecs();
        const size_t ns = m_nstatics;
        std::vector<double> pos(3 * ns), quat(4 * ns);
        check(cdx_get_static_state(m_ctx, pos.data(), quat.data(), nullptr, nullptr));
        for (size_t t = 0; t < m_traj.size(); ++t) {
            const entt::entity e = m_traj[t];
            const size_t s = (size_t)m_traj_index[t];
            auto& x = reg.get<C_Position3>(e).value;
            for (int k = 0; k < 3; ++k) x[k] = pos[3 * s + k];
            reg.get<C_Orientation>(e).setValue(Quaternion4r(quat[4 * s + 3], quat[4 * s + 0], quat[4 * s + 1], quat[4 * s + 2]));
        }
    }

    void check(int st) const {
        if (st != CDX_OK)
            throw std::runtime_error(std::string("GpuMoreauIntegrator: ") + (m_ctx ? cdx_last_error(m_ctx) : "cdx"));
    }

    // the reference's settings for the step (config.hpp:12-237) in the context's configuration
    cdx_config make_config(real_t dt) const {
        cdx_config c;
        cdx_config_default(&c);
        const config::Config& r = m_config;
        c.sim_dt = dt;
        const auto& g = m_world.gravity();
        for (int k = 0; k < 3; ++k) c.sim_gravity[k] = g[k];
        c.moreau_theta = r.moreau_theta;
        c.moreau_implicit_gyroscopy = r.moreau_implicit_gyroscopy ? 1 : 0;
        c.friction_enable = r.friction_enable ? 1 : 0;
        c.friction_combine = r.friction_combine == "arith" ? 1 : (r.friction_combine == "geom" ? 2 : 0);
        c.restitution_default_normal = r.restitution_default_normal;
        c.restitution_default_tangential = r.restitution_default_tangential;
        c.pj_alpha = r.pj_alpha;
        c.pj_max_iterations = r.pj_max_iterations;
        c.pj_warmstart = r.pj_warmstart ? 1 : 0;
        c.pj_tol_abs = r.pj_tol_abs;
        c.pj_tol_rel = r.pj_tol_rel;
        c.pj_nesterov = r.pj_nesterov ? 1 : 0;
        c.pj_nesterov_beta_threshold = r.pj_nesterov_beta_threshold;
        c.pj_nesterov_restart_limit = r.pj_nesterov_restart_limit;
        c.pj_chebyshev = r.pj_chebyshev ? 1 : 0;
        c.pj_anderson = r.pj_anderson ? 1 : 0;
        c.pj_anderson_m = r.pj_anderson_m;
        c.pj_rdiag_true_delassus = r.pj_rdiag_true_delassus ? 1 : 0;
        c.collision_security_margin = r.collision_security_margin;
        c.collision_match_max_dist = r.collision_match_max_dist;
        c.gpu_precision = m_precision;
        return c;
    }

    void rebuild(real_t dt) {
        auto& reg = m_world.ecs();
        m_spheres.clear();
        std::vector<entt::entity> planes;
        size_t dynamic = 0;
        for (auto e : reg.view<C_PhysicsObject>()) {
            ++dynamic;
            if (!reg.all_of<C_RB_Sphere, C_Radius, C_Mass, C_InertiaDiag>(e))
                throw std::runtime_error("GpuMoreauIntegrator: only rigid spheres move on the GPU path");
            m_spheres.push_back(e);
        }
        for (auto e : reg.view<C_RB_Plane>()) {
            if (reg.all_of<C_PhysicsObject>(e))
                throw std::runtime_error("GpuMoreauIntegrator: dynamic planes are not on the GPU path");
            planes.push_back(e);
        }
        const size_t nplanes = planes.size();
        for (auto e : reg.view<C_RB_Cylinder>())
            if (!reg.all_of<C_PhysicsObject>(e)) planes.push_back(e);  // dynamic cylinders threw above
        for (auto e : reg.view<C_RB_Cube>())
            if (!reg.all_of<C_PhysicsObject>(e)) planes.push_back(e);  // dynamic boxes threw above
        const size_t n = m_spheres.size(), ns = planes.size();
        (void)dynamic;
        m_traj.clear();
        m_traj_index.clear();
        m_nstatics = ns;
        for (size_t s = 0; s < ns; ++s)
            if (reg.all_of<C_StaticTrajectory>(planes[s])) {
                m_traj.push_back(planes[s]);
                m_traj_index.push_back((int32_t)s);
            }
        std::vector<double> rad(n), mass(n), inertia(n), mu(n), rn(n), rt(n);
        m_pos.assign(3 * n, 0.0);
        m_quat.assign(4 * n, 0.0);
        m_vel.assign(3 * n, 0.0);
        m_omega.assign(3 * n, 0.0);
        const config::Config& r = m_config;
        for (size_t i = 0; i < n; ++i) {
            const entt::entity e = m_spheres[i];
            rad[i] = reg.get<C_Radius>(e).r;
            mass[i] = reg.get<C_Mass>(e).m;
            inertia[i] = reg.get<C_InertiaDiag>(e).I[0];  // isotropic for a sphere
            mu[i] = reg.all_of<C_Friction>(e) ? reg.get<C_Friction>(e).mu : r.friction_default_mu;
            rn[i] = reg.all_of<C_Restitution>(e) ? reg.get<C_Restitution>(e).normal : 0.0;
            rt[i] = reg.all_of<C_Restitution>(e) ? reg.get<C_Restitution>(e).tangential : 0.0;
        }
        std::vector<int32_t> kind(ns, CDX_STATIC_HALFSPACE);
        std::vector<double> spos(3 * ns), squat(4 * ns), svel(3 * ns, 0.0), somega(3 * ns, 0.0), sdir(3 * ns),
            srad(ns, 0.0), smu(ns), srn(ns), srt(ns), shl(ns, 0.0), she(3 * ns, 0.0);
        for (size_t s = 0; s < ns; ++s) {
            const entt::entity e = planes[s];
            Vector3r x = reg.get<C_Position3>(e).value;
            const auto& o = reg.get<C_Orientation>(e);
            Quaternion4r q = o.value;
            Vector3r nw;
            if (reg.all_of<C_RB_Cube>(e)) {
                const auto& cb = reg.get<C_RB_Cube>(e);
                const bool offset = cb.center.squaredNorm() > 0 || cb.q.vec().squaredNorm() > 0;
                if (offset) {
                    const bool moves = reg.all_of<C_StaticTrajectory>(e) ||
                                       (reg.all_of<C_LinearVelocity3>(e) && reg.get<C_LinearVelocity3>(e).value.squaredNorm() > 0) ||
                                       (reg.all_of<C_AngularVelocity3>(e) && reg.get<C_AngularVelocity3>(e).value.squaredNorm() > 0);
                    if (moves)
                        throw std::runtime_error("GpuMoreauIntegrator: a moving box with a local offset is not on the GPU path");
                    q = q * cb.q;
                    q.normalize();
                    x = x + q * cb.center;
                }
                kind[s] = CDX_STATIC_BOX;
                for (int k = 0; k < 3; ++k) she[3 * s + k] = cb.halfExtents[k];
                nw = Vector3r::Zero();
            } else if (s < nplanes) {
                // the halfspace normal in the world frame (CollisionCoal builds it from C_RB_Plane's
                // normal and the entity pose, collision_coal.cpp:290-296)
                nw = o.rotation * reg.get<C_RB_Plane>(e).normal.normalized();
            } else {
                // coal::Cylinder(radius, 2 halfLength) lies along its local z (collision_coal.cpp:307-310)
                Vector3r ez;
                ez[2] = 1.0;
                nw = o.rotation * ez;
                kind[s] = CDX_STATIC_CYLINDER;
                srad[s] = reg.get<C_RB_Cylinder>(e).radius;
                shl[s] = reg.get<C_RB_Cylinder>(e).halfLength;
            }
            for (int k = 0; k < 3; ++k) {
                spos[3 * s + k] = x[k];
                sdir[3 * s + k] = nw[k];
            }
            squat[4 * s + 0] = q.x();
            squat[4 * s + 1] = q.y();
            squat[4 * s + 2] = q.z();
            squat[4 * s + 3] = q.w();
            if (reg.all_of<C_LinearVelocity3>(e))
                for (int k = 0; k < 3; ++k) svel[3 * s + k] = reg.get<C_LinearVelocity3>(e).value[k];
            if (reg.all_of<C_AngularVelocity3>(e))
                for (int k = 0; k < 3; ++k) somega[3 * s + k] = reg.get<C_AngularVelocity3>(e).value[k];
            smu[s] = reg.all_of<C_Friction>(e) ? reg.get<C_Friction>(e).mu : r.friction_default_mu;
            srn[s] = reg.all_of<C_Restitution>(e) ? reg.get<C_Restitution>(e).normal : 0.0;
            srt[s] = reg.all_of<C_Restitution>(e) ? reg.get<C_Restitution>(e).tangential : 0.0;
        }
        cdx_destroy(m_ctx);
        m_ctx = nullptr;
        const cdx_config c = make_config(dt);
        check(cdx_create(&c, &m_ctx));
        cdx_scene sc{};
        sc.num_bodies = (int32_t)n;
        sc.pos = m_pos.data();
        sc.quat = m_quat.data();
        sc.vel = m_vel.data();
        sc.omega = m_omega.data();
        for (size_t i = 0; i < n; ++i) m_quat[4 * i + 3] = 1.0;  // overwritten by the first upload
        sc.radius = rad.data();
        sc.mass = mass.data();
        sc.inertia = inertia.data();
        sc.mu = mu.data();
        sc.rest_n = rn.data();
        sc.rest_t = rt.data();
        sc.num_statics = (int32_t)ns;
        sc.static_kind = kind.data();
        sc.static_pos = spos.data();
        sc.static_quat = squat.data();
        sc.static_vel = svel.data();
        sc.static_omega = somega.data();
        sc.static_dir = sdir.data();
        sc.static_radius = srad.data();
        sc.static_mu = smu.data();
        sc.static_rest_n = srn.data();
        sc.static_rest_t = srt.data();
        sc.num_scenes = 1;
        sc.static_half_length = shl.data();
        sc.static_half_extents = she.data();
        check(cdx_load_scene(m_ctx, &sc));
        m_dt = dt;
        m_world.m_structure_dirty = false;
    }

    int32_t m_precision;
    cdx_ctx* m_ctx = nullptr;
    real_t m_dt = 0;
    std::vector<entt::entity> m_spheres;
    std::vector<double> m_pos, m_quat, m_vel, m_omega;
    std::vector<entt::entity> m_traj;    // statics driven by a trajectory
    std::vector<int32_t> m_traj_index;   // their index among the context's statics
    size_t m_nstatics = 0;
};

}  // namespace cardillo::integration

#endif  // CDX_WITH_CARDILLO
