// Stand-in for IntegrationBase (integration_base.hpp:12-32): its constructor, step(dt) and the
// protected references under their reference names.
#pragma once
#include "../solver/solver_base.hpp"
#include "../world.hpp"

namespace cardillo {
namespace misc {
class TimingManager {};
}
namespace integration {
class IntegrationBase {
   public:
    explicit IntegrationBase(World& world, solver::SolverBase& solver, physics::DynamicsAssembler& dyn,
                             misc::TimingManager& timings, config::Config& config)
        : m_world(world), m_dyn(dyn), m_timings(timings), m_solver(solver), m_config(config) {}
    virtual ~IntegrationBase() = default;
    virtual void step(real_t dt) = 0;

   protected:
    World& m_world;
    physics::DynamicsAssembler& m_dyn;
    misc::TimingManager& m_timings;
    solver::SolverBase& m_solver;
    config::Config& m_config;
};
}  // namespace integration
}  // namespace cardillo
