// Stand-ins for the ECS pieces the integrator adapter uses: the component types of ecs_types.hpp
// (C_Position3 ... C_InertiaDiag, C_RB_Cylinder, C_RB_Cube and C_StaticTrajectory, lines 15-166), the Eigen types they hold (fixed-size vector,
// quaternion with x()/y()/z()/w() and the (w, x, y, z) constructor, 3x3 rotation), and the EnTT
// registry calls (view, get, all_of). Enough to compile the adapter syntax-only.
#pragma once
#include <cmath>
#include <cstdint>
#include <functional>
#include <optional>
#include <utility>
#include <vector>

#include "solver/solver_base.hpp"

namespace entt {
enum class entity : std::uint32_t {};
class registry {
   public:
    template <class... T>
    std::vector<entity> view() const { return {}; }
    template <class T>
    T& get(entity) { static T t{}; return t; }
    template <class T>
    const T& get(entity) const { static T t{}; return t; }
    template <class... T>
    bool all_of(entity) const { return true; }
};
}  // namespace entt

namespace cardillo {
struct Vector3r {
    double c[3]{0, 0, 0};
    double& operator[](int k) { return c[k]; }
    double operator[](int k) const { return c[k]; }
    Vector3r normalized() const {
        const double n = std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
        return Vector3r{{c[0] / n, c[1] / n, c[2] / n}};
    }
    double squaredNorm() const { return c[0] * c[0] + c[1] * c[1] + c[2] * c[2]; }
    static Vector3r Zero() { return Vector3r{}; }
    Vector3r operator+(const Vector3r& o) const { return Vector3r{{c[0] + o.c[0], c[1] + o.c[1], c[2] + o.c[2]}}; }
};
struct Matrix33r {
    double m[9]{1, 0, 0, 0, 1, 0, 0, 0, 1};
    Vector3r operator*(const Vector3r& v) const {
        Vector3r r;
        for (int i = 0; i < 3; ++i) r[i] = m[3 * i] * v[0] + m[3 * i + 1] * v[1] + m[3 * i + 2] * v[2];
        return r;
    }
};
struct Quaternion4r {
    double qw{1}, qx{0}, qy{0}, qz{0};
    Quaternion4r() = default;
    Quaternion4r(double w, double x, double y, double z) : qw(w), qx(x), qy(y), qz(z) {}
    double w() const { return qw; }
    double x() const { return qx; }
    double y() const { return qy; }
    double z() const { return qz; }
    static Quaternion4r Identity() { return Quaternion4r{}; }
    Vector3r vec() const { return Vector3r{{qx, qy, qz}}; }
    void normalize() {
        const double n = std::sqrt(qw * qw + qx * qx + qy * qy + qz * qz);
        qw /= n; qx /= n; qy /= n; qz /= n;
    }
    Quaternion4r operator*(const Quaternion4r& o) const {
        return Quaternion4r(qw * o.qw - qx * o.qx - qy * o.qy - qz * o.qz, qw * o.qx + qx * o.qw + qy * o.qz - qz * o.qy,
                            qw * o.qy - qx * o.qz + qy * o.qw + qz * o.qx, qw * o.qz + qx * o.qy - qy * o.qx + qz * o.qw);
    }
    Vector3r operator*(const Vector3r& v) const {  // rotation of v
        const Quaternion4r p = (*this) * Quaternion4r(0, v[0], v[1], v[2]) * Quaternion4r(qw, -qx, -qy, -qz);
        return Vector3r{{p.qx, p.qy, p.qz}};
    }
};

struct C_Mass { real_t m; };
struct C_Position3 { Vector3r value; };
struct C_LinearVelocity3 { Vector3r value; };
struct C_AngularVelocity3 { Vector3r value; };
struct C_Orientation {
    Quaternion4r value;
    Matrix33r rotation;
    void setValue(const Quaternion4r& q) { value = q; }
};
struct C_PhysicsObject {};
struct C_RB_Sphere {};
struct C_Radius { real_t r; };
struct C_RB_Plane {
    Vector3r normal;
    Vector3r up;
    real_t sizeX;
    real_t sizeY;
};
struct C_Friction { real_t mu; };
struct C_Restitution {
    real_t normal;
    real_t tangential;
};
struct C_InertiaDiag { Vector3r I; };
struct C_RB_Cylinder {
    real_t radius;
    real_t halfLength;
};
struct C_RB_Cube {
    Vector3r center{Vector3r::Zero()};
    Vector3r halfExtents;
    Quaternion4r q{Quaternion4r::Identity()};
};
using TrajectoryPose = std::pair<Vector3r, Quaternion4r>;
using TrajectoryTwist = std::pair<Vector3r, Vector3r>;
struct C_StaticTrajectory {
    std::optional<std::function<TrajectoryPose(real_t)>> positionFunc;
    std::optional<std::function<TrajectoryTwist(real_t)>> velocityFunc;
    real_t elapsed{(real_t)0};
    bool initialized{false};
    std::optional<TrajectoryPose> previousPosition;
};
}  // namespace cardillo
