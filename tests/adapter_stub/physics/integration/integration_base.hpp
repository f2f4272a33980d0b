// Stand-in for IntegrationBase (integration_base.hpp:19): its constructor and step(dt).
#pragma once
#include "../solver/solver_base.hpp"

namespace cardillo {
class World {};
namespace misc {
class TimingManager {};
}
namespace integration {
class IntegrationBase {
   public:
    IntegrationBase(World& w, solver::SolverBase& s, physics::DynamicsAssembler& d, misc::TimingManager& t,
                    config::Config& c)
        : m_world(w), m_solver(s), m_dyn(d), m_timings(t), m_cfg(c) {}
    virtual ~IntegrationBase() = default;
    virtual void step(real_t dt) = 0;

   protected:
    World& m_world;
    solver::SolverBase& m_solver;
    physics::DynamicsAssembler& m_dyn;
    misc::TimingManager& m_timings;
    config::Config& m_cfg;
};
}  // namespace integration
}  // namespace cardillo
