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
//      the whole step (collision, contact rows, PJ, drift) runs in cdx_step.
#pragma once
#ifdef CDX_WITH_CARDILLO

#include <stdexcept>
#include <string>
#include <vector>

#include "cdx.h"
#include "physics/integration/integration_base.hpp"
#include "physics/solver/solver_base.hpp"
#include "physics/solver/warmstart.hpp"

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

// Whole-step drop-in for sphere scenes. The scene is mirrored once (and again whenever the ECS
// structure changes); each step uploads the state, runs cdx_step, and writes the state back.
class GpuMoreauIntegrator : public IntegrationBase {
   public:
    using IntegrationBase::IntegrationBase;
    ~GpuMoreauIntegrator() override { cdx_destroy(m_ctx); }

    void step(real_t dt) override;  // defined in gpu_moreau.cpp next to moreau.cpp: gathers the
                                    // sphere/halfspace entities into a cdx_scene, cdx_set_state,
                                    // cdx_step(1), cdx_get_state, then writes C_Position3,
                                    // C_Orientation, C_LinearVelocity3, C_AngularVelocity3
   private:
    cdx_ctx* m_ctx = nullptr;
};

}  // namespace cardillo::integration

#endif  // CDX_WITH_CARDILLO
