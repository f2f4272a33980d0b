// Stand-in for World (world.hpp:50-102): the registry, gravity and the structure flag the adapter reads.
#pragma once
#include "ecs_types.hpp"

namespace cardillo {
class World {
   public:
    entt::registry m_reg;
    Vector3r m_gravity{{0.0, 0.0, -9.81}};
    mutable bool m_structure_dirty = true;
    entt::registry& ecs() { return m_reg; }
    const entt::registry& ecs() const { return m_reg; }
    const Vector3r& gravity() const { return m_gravity; }
};
}  // namespace cardillo
