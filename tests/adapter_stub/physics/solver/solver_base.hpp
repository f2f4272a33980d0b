// Minimal stand-ins for the reference interfaces the adapter header uses (names and signatures of
// SolverBase, DynamicsAssembler, Config; solver_base.hpp:14-37, dynamics_assembler.hpp:23-94,
// config.hpp:12-237), so the adapter can be compiled syntax-only without Eigen and EnTT.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace cardillo {
using real_t = double;

struct VectorXr {
    std::vector<double> v;
    VectorXr() = default;
    explicit VectorXr(long n) : v((size_t)n) {}
    static VectorXr Zero(long n) { return VectorXr(n); }
    double* data() { return v.data(); }
    const double* data() const { return v.data(); }
    VectorXr head(long n) const {
        VectorXr r(n);
        for (long i = 0; i < n; ++i) r.v[(size_t)i] = v[(size_t)i];
        return r;
    }
};

namespace config {
struct Config {
    real_t sim_dt{1e-3};
    real_t moreau_theta{1.0};
    bool friction_enable{false};
    std::string friction_combine{"min"};
    real_t friction_default_mu{0.3};
    real_t restitution_default_normal{0.0};
    real_t restitution_default_tangential{0.0};
    real_t collision_security_margin{0.0};
    real_t collision_match_max_dist{0.02};
    bool pj_warmstart{true};
    bool moreau_implicit_gyroscopy{false};
    real_t pj_alpha{1.0};
    int pj_max_iterations{100};
    real_t pj_tol_abs{1e-5}, pj_tol_rel{1e-4};
    bool pj_nesterov{false};
    real_t pj_nesterov_beta_threshold{1.0};
    int pj_nesterov_restart_limit{10000};
    bool pj_chebyshev{false};
    bool pj_anderson{false};
    int pj_anderson_m{2};
    bool pj_rdiag_true_delassus{false};
};
}  // namespace config

namespace physics {
struct SparseRowMajor {
    std::vector<int> outer, inner;
    std::vector<double> values;
    const int* outerIndexPtr() const { return outer.data(); }
    const int* innerIndexPtr() const { return inner.data(); }
    const double* valuePtr() const { return values.data(); }
};
struct TripletMatrix {
    SparseRowMajor rm;
    const SparseRowMajor& asSparseRowMajor() const { return rm; }
};
class DynamicsAssembler {
   public:
    long numV() const { return 0; }
    int numContactRows() const { return 0; }
    int numFrictionlessContacts() const { return 0; }
    long numSprings() const { return 0; }
    long numDampers() const { return 0; }
    const TripletMatrix& W() const { return w; }
    const VectorXr& contactVVec() const { return z; }
    const VectorXr& muVec() const { return z; }
    const VectorXr& restitutionVec() const { return z; }
    const VectorXr& MinvDiag() const { return z; }
    const VectorXr& MDiag() const { return z; }
    const VectorXr& vVec() const { return z; }
    const VectorXr& fVecExternal() const { return z; }
    const VectorXr& fVecGyroscopic() const { return z; }

   private:
    TripletMatrix w;
    VectorXr z;
};
}  // namespace physics

namespace solver {
class SolverBase {
   public:
    virtual ~SolverBase() = default;
    virtual VectorXr solve(real_t dt, real_t theta) = 0;
    virtual int lastIterations() const { return m_last_iters; }
    virtual real_t lastError() const { return (real_t)0; }
    virtual const char* name() const { return "SolverBase"; }

   protected:
    int m_last_iters{-1};
};
}  // namespace solver
}  // namespace cardillo
