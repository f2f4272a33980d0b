// Stand-in for WarmstartProvider (warmstart.hpp:26-56): the two calls the adapter makes.
#pragma once
#include "solver_base.hpp"

namespace cardillo::solver {
struct WarmstartProvider {
    static void applyWarmstart(VectorXr&, physics::DynamicsAssembler&) {}
    static void storeImpulse(const VectorXr&, physics::DynamicsAssembler&) {}
};
}  // namespace cardillo::solver
