// Oracle: CPU FP64 restatement of CardilloCxx's Moreau midpoint step for sphere scenes.
//
// TEST INFRASTRUCTURE ONLY (the checker and the timed CPU baseline). Nothing in the product
// package loads this file. Parity status: UNPINNED -- the reference needs Eigen 5.0.1, EnTT 3.13.2
// and coal 3.0.4, none of which exist here, and it has no tests or golden vectors for this path.
//
// Every function cites the reference lines it restates (paths relative to the reference repo).
// Floating-point rules: plain IEEE double, no FMA contraction (built with -ffp-contract=off),
// every expression evaluated left to right as written in the reference's Eigen code. Where the
// reference's result depends on Eigen's internal reduction order (vectorised dot products and
// norms), this file fixes the sequential order ((a0*b0 + a1*b1) + a2*b2); identity-matrix
// products that Eigen evaluates literally (transform::point from the inertial frame) are elided,
// which can only change the sign of an exact zero.
#include "cdx_oracle.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

inline double dot3(const double* a, const double* b) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }
inline double norm3(const double* a) { return std::sqrt(dot3(a, a)); }
inline void cross3(const double* a, const double* b, double* o) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}
inline bool finite3(const double* a) { return std::isfinite(a[0]) && std::isfinite(a[1]) && std::isfinite(a[2]); }
inline double std_min(double a, double b) { return (b < a) ? b : a; }  // std::min semantics
inline double std_max(double a, double b) { return (a < b) ? b : a; }  // std::max semantics

// Quaternion (x,y,z,w) -> row-major rotation matrix, Eigen's QuaternionBase::toRotationMatrix
// (C_Orientation::setValue, src/physics/ecs_types.hpp:37-41).
inline void rotmat(const double* q, double* R) {
    const double x = q[0], y = q[1], z = q[2], w = q[3];
    const double tx = 2.0 * x, ty = 2.0 * y, tz = 2.0 * z;
    const double twx = tx * w, twy = ty * w, twz = tz * w;
    const double txx = tx * x, txy = ty * x, txz = tz * x;
    const double tyy = ty * y, tyz = tz * y, tzz = tz * z;
    R[0] = 1.0 - (tyy + tzz); R[1] = txy - twz;         R[2] = txz + twy;
    R[3] = txy + twz;         R[4] = 1.0 - (txx + tzz); R[5] = tyz - twx;
    R[6] = txz - twy;         R[7] = tyz + twx;         R[8] = 1.0 - (txx + tyy);
}
// R^T v (transformations.hpp:34-43: inertialToBodyPoint / inertialToBodyVector)
inline void matTvec(const double* R, const double* v, double* o) {
    for (int i = 0; i < 3; ++i) o[i] = (R[0 + i] * v[0] + R[3 + i] * v[1]) + R[6 + i] * v[2];
}
// R v (bodyToInertialVector, src/rigid_body/transformations.hpp:38-40)
inline void matvec(const double* R, const double* v, double* o) {
    for (int i = 0; i < 3; ++i) o[i] = (R[3 * i] * v[0] + R[3 * i + 1] * v[1]) + R[3 * i + 2] * v[2];
}

// src/misc/math_helper.hpp:11-17 (alignQuaternionTo) with Eigen's normalize()
inline void align_quat(double* q, const double* qref) {
    if (!(std::isfinite(q[0]) && std::isfinite(q[1]) && std::isfinite(q[2]) && std::isfinite(q[3]))) {
        for (int k = 0; k < 4; ++k) q[k] = qref[k];
        return;
    }
    const double n2 = ((q[0] * q[0] + q[1] * q[1]) + q[2] * q[2]) + q[3] * q[3];
    if (n2 > 0.0) {
        const double n = std::sqrt(n2);
        for (int k = 0; k < 4; ++k) q[k] = q[k] / n;
    }
    const double d = ((qref[0] * q[0] + qref[1] * q[1]) + qref[2] * q[2]) + qref[3] * q[3];
    if (d < 0.0)
        for (int k = 0; k < 4; ++k) q[k] = -q[k];
}

// src/physics/integration/integration_base.cpp:6-30 (explicitPositionUpdate) for one entity.
inline void drift(double* x, double* q, const double* v, const double* w, double h) {
    for (int k = 0; k < 3; ++k) x[k] = x[k] + h * v[k];
    const double qprev[4] = {q[0], q[1], q[2], q[3]};
    const double hh = h * 0.5;
    const double qw = q[3];
    q[3] = q[3] - hh * dot3(q, w);
    double c[3];
    cross3(qprev, w, c);
    for (int k = 0; k < 3; ++k) q[k] = qprev[k] + hh * (qw * w[k] + c[k]);
    align_quat(q, qprev);
}

// src/collision/tangent_frame.hpp:23-50 (tangentFrameFromNormal)
inline void tangent_frame(const double* n_in, double* t1, double* t2) {
    const double len = norm3(n_in);
    if (len <= DBL_EPSILON) {
        t1[0] = 1; t1[1] = 0; t1[2] = 0;
        t2[0] = 0; t2[1] = 1; t2[2] = 0;
        return;
    }
    const double n[3] = {n_in[0] / len, n_in[1] / len, n_in[2] / len};
    if (n[2] < -0.9999999) {
        t1[0] = 0; t1[1] = -1; t1[2] = 0;
        const double d = dot3(n, t1);
        for (int k = 0; k < 3; ++k) t1[k] = t1[k] - n[k] * d;
    } else {
        const double a = 1.0 / (1.0 + n[2]);
        const double b = (-n[0] * n[1]) * a;
        t1[0] = 1.0 - (n[0] * n[0]) * a;
        t1[1] = b;
        t1[2] = -n[0];
    }
    const double t2n = dot3(t1, t1);
    if (t2n > 0.0) {
        const double s = std::sqrt(t2n);
        for (int k = 0; k < 3; ++k) t1[k] = t1[k] / s;
    }
    cross3(n, t1, t2);
}

struct Contact {
    int32_t a = -1, b = -1;    // entity ids: statics 0..S-1, spheres S..S+N-1
    int32_t sa = -1, sb = -1;  // static index of side A (or -1); body index of side A/B (or -1)
    int32_t ba = -1, bb = -1;
    double point[3], n[3], t1[3], t2[3];
    double cA[9], cB[9];  // r_X^body x d_k^body for k = n, t1, t2 (unsigned)
    double cb[3];          // static-side contact velocity per row
    double mu = 0, eN = 0, eT = 0;
    bool frictional = false;
    double lam0[3] = {0, 0, 0};
    uint64_t key() const { return ((uint64_t)(uint32_t)a << 32) | (uint32_t)b; }
};

struct Engine {
    or_config cfg{};
    int N = 0, S = 0;
    std::vector<double> pos, q, v, w, R, rad, mass, inertia, mu, rn, rt;
    std::vector<int32_t> scene;
    std::vector<double> minv, Mdiag;  // per DOF (6 per body)
    std::vector<int32_t> skind, sscene;
    std::vector<double> spos, sq, sv, sw, sdir, srad, sd, smu, srn, srt, sR, shl, sax, she;
    // warm-start memory of the previous step (canonical order, sorted by key)
    std::vector<uint64_t> prev_keys;
    std::vector<double> prev_point, prev_lambda;
    // last step's contacts for inspection
    std::vector<Contact> last;
    std::vector<double> last_lambda;
    bool trace_on = false;
    std::vector<double> trace;
    or_stats stats{};
    double rmax = 0;
    int status = 0;  // 4 once a condensed solve diverged
    // prescribed static motion of the coming step (Trajectory::update): 13 values a static and flags
    std::vector<double> smot;
    std::vector<int32_t> smflag;
};

// Sphere mass matrix, src/physics/assembly/dynamics_assembler.cpp:41-62 (rebuildMass_) with
// src/physics/world.cpp:49-72: Minv = 1/[m,m,m,I,I,I], M_ii = 1/Minv_ii.
void build_mass(Engine& E) {
    E.minv.assign(6 * (size_t)E.N, 0.0);
    E.Mdiag.assign(6 * (size_t)E.N, 0.0);
    for (int i = 0; i < E.N; ++i) {
        for (int k = 0; k < 6; ++k) {
            const double md = (k < 3) ? E.mass[i] : E.inertia[i];
            const double inv = 1.0 / md;
            E.minv[6 * i + k] = inv;
            E.Mdiag[6 * i + k] = (inv > 0.0) ? 1.0 / inv : 0.0;
        }
    }
}

// Sphere (centre xb, radius rb) against a solid cylinder (centre xa, unit axis u, radius R, half
// length h); coal answers this pair with the exact nearest points (GJK on the two convex shapes),
// restated here in closed form. In the cylinder's frame (axial coordinate ax, radial part perp of
// length rho): outside, the nearest point is on the side (|ax| <= h), a cap (rho <= R) or a rim;
// inside, on the nearer of the side and the cap (the side on a tie). The normal points from the
// cylinder to the sphere; sd is the centre's signed distance to the surface along it.
bool cylinder_geom(const double* xa, const double* u, double R, double h, const double* xb, double rb, double margin,
                   double* p1, double* p2, double* nraw) {
    double rel[3], perp[3];
    for (int k = 0; k < 3; ++k) rel[k] = xb[k] - xa[k];
    const double ax = dot3(rel, u);
    for (int k = 0; k < 3; ++k) perp[k] = rel[k] - ax * u[k];
    const double rho = norm3(perp);
    const double sg = ax < 0.0 ? -1.0 : 1.0;
    const double aax = std::fabs(ax);
    double e[3];
    if (rho > 0.0) {
        for (int k = 0; k < 3; ++k) e[k] = perp[k] / rho;
    } else {
        double t2[3];
        tangent_frame(u, e, t2);  // on the axis any radial direction is nearest
    }
    const bool out_side = rho > R, out_cap = aax > h;
    int region;  // 0 side, 1 cap, 2 rim
    double sd;
    if (!out_side && !out_cap) {
        const double dside = R - rho, dcap = h - aax;
        region = dside <= dcap ? 0 : 1;
        sd = region == 0 ? -dside : -dcap;
    } else if (!out_cap) {
        region = 0;
        sd = rho - R;
    } else if (!out_side) {
        region = 1;
        sd = aax - h;
    } else {
        region = 2;
        sd = 0.0;
    }
    double q[3], n[3];
    if (region == 0) {
        for (int k = 0; k < 3; ++k) {
            q[k] = (xa[k] + ax * u[k]) + R * e[k];
            n[k] = e[k];
        }
    } else if (region == 1) {
        for (int k = 0; k < 3; ++k) {
            q[k] = (xa[k] + (sg * h) * u[k]) + perp[k];
            n[k] = sg * u[k];
        }
    } else {
        double d[3];
        for (int k = 0; k < 3; ++k) {
            q[k] = (xa[k] + (sg * h) * u[k]) + R * e[k];
            d[k] = xb[k] - q[k];
        }
        sd = norm3(d);
        for (int k = 0; k < 3; ++k) n[k] = d[k] / sd;
    }
    if (!((sd - rb) <= margin)) return false;
    for (int k = 0; k < 3; ++k) {
        p1[k] = q[k];
        p2[k] = xb[k] - rb * n[k];
        nraw[k] = n[k];
    }
    return true;
}

// Sphere against a solid box (C_RB_Cube, coal::Box of full sides 2 halfExtents,
// collision_coal.cpp:288-290), the exact nearest points in closed form. With the box's axes the
// columns of R and c = R^T (xb - xa) the centre in its frame: outside (some |c_k| > e_k) the
// nearest point is c clamped to the box and the normal runs from it to the centre; inside, the
// nearest face (the lowest axis on a tie) gives the point and its outward normal. Normal from the
// box to the sphere; coal's GJK/EPA reports the same points up to its own tolerance.
bool box_geom(const double* xa, const double* R, const double* e, const double* xb, double rb, double margin,
              double* p1, double* p2, double* nraw) {
    double rel[3], c[3], ql[3], nl[3];
    for (int k = 0; k < 3; ++k) rel[k] = xb[k] - xa[k];
    matTvec(R, rel, c);
    const bool out = std::fabs(c[0]) > e[0] || std::fabs(c[1]) > e[1] || std::fabs(c[2]) > e[2];
    double sd;
    if (!out) {
        int f = 0;
        double best = e[0] - std::fabs(c[0]);
        for (int k = 1; k < 3; ++k) {
            const double dk = e[k] - std::fabs(c[k]);
            if (dk < best) {
                best = dk;
                f = k;
            }
        }
        const double sg = c[f] < 0.0 ? -1.0 : 1.0;
        for (int k = 0; k < 3; ++k) {
            ql[k] = c[k];
            nl[k] = 0.0;
        }
        ql[f] = sg * e[f];
        nl[f] = sg;
        sd = -best;
    } else {
        double d[3];
        for (int k = 0; k < 3; ++k) {
            ql[k] = c[k] < -e[k] ? -e[k] : (c[k] > e[k] ? e[k] : c[k]);
            d[k] = c[k] - ql[k];
        }
        sd = norm3(d);
        for (int k = 0; k < 3; ++k) nl[k] = d[k] / sd;
    }
    if (!((sd - rb) <= margin)) return false;
    double n[3], q[3];
    matvec(R, nl, n);
    matvec(R, ql, q);
    for (int k = 0; k < 3; ++k) {
        p1[k] = xa[k] + q[k];
        p2[k] = xb[k] - rb * n[k];
        nraw[k] = n[k];
    }
    return true;
}

// Narrow phase for one (static, sphere) or (sphere, sphere) pair plus makeContact
// (src/collision/collision_coal.cpp:112-163). Returns false when the shapes are apart
// (distance > collision.security_margin, coal's ShapeShapeCollider rule).
bool make_contact(const Engine& E, int a_static, int a_body, int b_body, Contact& c) {
    const double* xb = &E.pos[3 * (size_t)b_body];
    const double rb = E.rad[b_body];
    double p1[3], p2[3], nraw[3], xa[3];
    const double margin = E.cfg.collision_security_margin;
    if (a_static >= 0) {
        const int s = a_static;
        for (int k = 0; k < 3; ++k) xa[k] = E.spos[3 * s + k];
        const double* u = &E.sdir[3 * s];
        if (E.skind[s] == 0) {
            // coal::Halfspace {x : n.x <= d}; shape 1 = halfspace, shape 2 = sphere
            const double sdist = dot3(u, xb) - E.sd[s];
            const double dist = sdist - rb;
            if (!(dist <= margin)) return false;
            for (int k = 0; k < 3; ++k) {
                p1[k] = xb[k] - sdist * u[k];
                p2[k] = xb[k] - rb * u[k];
                nraw[k] = u[k];
            }
        } else if (E.skind[s] == 2) {
            // solid cylinder (C_RB_Cylinder, coal::Cylinder(radius, 2 halfLength) along the axis;
            // collision_coal.cpp:307-310): the nearest point of the side, a cap or a rim. Its axis
            // turns with the static (coal places the shape with the object's transform each step,
            // collision_coal.cpp:380-401): R times the axis in the static's frame.
            double ua[3];
            matvec(&E.sR[9 * s], &E.sax[3 * s], ua);
            if (!cylinder_geom(xa, ua, E.srad[s], E.shl[s], xb, rb, margin, p1, p2, nraw)) return false;
        } else if (E.skind[s] == 3) {
            // solid box (C_RB_Cube), posed by the static's rotation
            if (!box_geom(xa, &E.sR[9 * s], &E.she[3 * s], xb, rb, margin, p1, p2, nraw)) return false;
        } else {
            // hollow drum wall (new primitive; the reference has no counterpart)
            double rel[3];
            for (int k = 0; k < 3; ++k) rel[k] = xb[k] - xa[k];
            const double ax = dot3(rel, u);
            double perp[3];
            for (int k = 0; k < 3; ++k) perp[k] = rel[k] - ax * u[k];
            const double rho = norm3(perp);
            const double dist = (E.srad[s] - rho) - rb;
            if (!(dist <= margin)) return false;
            double e[3] = {0, 0, 0};
            if (rho > 0.0)
                for (int k = 0; k < 3; ++k) e[k] = perp[k] / rho;
            for (int k = 0; k < 3; ++k) {
                p1[k] = (xa[k] + ax * u[k]) + E.srad[s] * e[k];
                p2[k] = xb[k] + rb * e[k];
                nraw[k] = -e[k];
            }
        }
        c.a = s;
        c.sa = s;
        c.ba = -1;
    } else {
        const double* xA = &E.pos[3 * (size_t)a_body];
        const double ra = E.rad[a_body];
        double d[3];
        for (int k = 0; k < 3; ++k) d[k] = xb[k] - xA[k];
        const double dl = norm3(d);
        const double dist = (dl - ra) - rb;
        if (!(dist <= margin)) return false;
        double nn[3] = {0, 0, 0};
        if (dl > 0.0)
            for (int k = 0; k < 3; ++k) nn[k] = d[k] / dl;
        for (int k = 0; k < 3; ++k) {
            p1[k] = xA[k] + ra * nn[k];
            p2[k] = xb[k] - rb * nn[k];
            nraw[k] = nn[k];
            xa[k] = xA[k];
        }
        c.a = E.S + a_body;
        c.sa = -1;
        c.ba = a_body;
    }
    c.b = E.S + b_body;
    c.bb = b_body;

    // makeContact: sanitise points, normalise the normal with fallbacks
    if (!finite3(p1)) {
        if (finite3(p2)) { for (int k = 0; k < 3; ++k) p1[k] = p2[k]; }
        else { for (int k = 0; k < 3; ++k) p1[k] = xa[k]; }
    }
    if (!finite3(p2)) {
        if (finite3(p1)) { for (int k = 0; k < 3; ++k) p2[k] = p1[k]; }
        else { for (int k = 0; k < 3; ++k) p2[k] = xb[k]; }
    }
    double n[3];
    const double nlen = norm3(nraw);
    if (nlen > 0.0 && std::isfinite(nlen)) {
        for (int k = 0; k < 3; ++k) n[k] = nraw[k] / nlen;
    } else {
        double f[3];
        for (int k = 0; k < 3; ++k) f[k] = p2[k] - p1[k];
        double fl = norm3(f);
        if (!(fl > 0.0) || !std::isfinite(fl)) {
            for (int k = 0; k < 3; ++k) f[k] = xb[k] - xa[k];
            fl = norm3(f);
        }
        if (fl > 0.0 && std::isfinite(fl)) { for (int k = 0; k < 3; ++k) n[k] = f[k] / fl; }
        else { n[0] = 0; n[1] = 0; n[2] = 1; }
    }
    for (int k = 0; k < 3; ++k) c.n[k] = n[k];
    tangent_frame(n, c.t1, c.t2);
    for (int k = 0; k < 3; ++k) c.point[k] = (p1[k] + p2[k]) * 0.5;
    return true;
}

// Body-frame lever arms and static-side contact velocities: makeContact's transform::point /
// transform::direction (collision_coal.cpp:151-160) and rebuildW_'s accumulateDirForSide
// (dynamics_assembler.cpp:262-286) with buildContactRowByDof (contact_jacobian.hpp:17-23).
void contact_rows(const Engine& E, Contact& c) {
    const double* dirs[3] = {c.n, c.t1, c.t2};
    for (int side = 0; side < 2; ++side) {
        const double* R;
        const double* x;
        if (side == 0) {
            if (c.sa >= 0) { R = &E.sR[9 * c.sa]; x = &E.spos[3 * c.sa]; }
            else { R = &E.R[9 * (size_t)c.ba]; x = &E.pos[3 * (size_t)c.ba]; }
        } else {
            R = &E.R[9 * (size_t)c.bb];
            x = &E.pos[3 * (size_t)c.bb];
        }
        double rel[3], rbody[3];
        for (int k = 0; k < 3; ++k) rel[k] = c.point[k] - x[k];
        matTvec(R, rel, rbody);
        double* cc = side == 0 ? c.cA : c.cB;
        for (int r = 0; r < 3; ++r) {
            double db[3];
            matTvec(R, dirs[r], db);
            cross3(rbody, db, &cc[3 * r]);
        }
    }
    // static side A: contact_v_vec[row] = 0 + row . [v_world, omega_body] with sign -1
    for (int r = 0; r < 3; ++r) c.cb[r] = 0.0;
    if (c.sa >= 0) {
        const double* vs = &E.sv[3 * c.sa];
        const double* ws = &E.sw[3 * c.sa];
        for (int r = 0; r < 3; ++r) {
            const double* d = dirs[r];
            const double row[6] = {-d[0], -d[1], -d[2], -c.cA[3 * r], -c.cA[3 * r + 1], -c.cA[3 * r + 2]};
            double acc = row[0] * vs[0];
            acc = acc + row[1] * vs[1];
            acc = acc + row[2] * vs[2];
            acc = acc + row[3] * ws[0];
            acc = acc + row[4] * ws[1];
            acc = acc + row[5] * ws[2];
            c.cb[r] = 0.0 + acc;
        }
    }
}

double combine_mu(int mode, double a, double b) {  // collision_coal.cpp:94-106
    a = std_max(0.0, a);
    b = std_max(0.0, b);
    if (mode == 1) return (a + b) * 0.5;
    if (mode == 2) return std::sqrt(std_max(0.0, a * b));
    return std_min(a, b);
}

// Collision: canonical order by (entity id A, entity id B), statics first.
// Replaces collision_coal.cpp:405-548 (coal broad phase + hash-map flatten order).
void detect(Engine& E, std::vector<Contact>& out) {
    out.clear();
    const int N = E.N, S = E.S;
    // static contacts, ordered by (static, sphere)
    for (int s = 0; s < S; ++s) {
        if (E.cfg.omp_mode == 1) {
            // a static schedule hands thread t the t-th contiguous range of spheres, so appending
            // the threads' lists in thread order keeps the sphere order
            std::vector<std::vector<Contact>> part(omp_get_max_threads());
#pragma omp parallel
            {
                std::vector<Contact>& mine = part[omp_get_thread_num()];
#pragma omp for schedule(static)
                for (int i = 0; i < N; ++i) {
                    if (E.scene[i] != E.sscene[s]) continue;
                    Contact c;
                    if (make_contact(E, s, -1, i, c)) mine.push_back(c);
                }
            }
            for (auto& p : part) out.insert(out.end(), p.begin(), p.end());
            continue;
        }
        for (int i = 0; i < N; ++i) {
            if (E.scene[i] != E.sscene[s]) continue;
            Contact c;
            if (make_contact(E, s, -1, i, c)) out.push_back(c);
        }
    }
    // sphere pairs via a uniform grid (any exact candidate method yields the same set)
    if (N == 0) return;
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int i = 0; i < N; ++i)
        for (int k = 0; k < 3; ++k) {
            const double p = E.pos[3 * (size_t)i + k];
            if (std::isfinite(p)) { lo[k] = std::min(lo[k], p); hi[k] = std::max(hi[k], p); }
        }
    const double cell = 2.0 * E.rmax * 1.0001 + 1e-12;
    int64_t dim[3];
    for (int k = 0; k < 3; ++k) {
        if (!(hi[k] >= lo[k])) { lo[k] = 0; hi[k] = 0; }
        dim[k] = std::min<int64_t>((int64_t)((hi[k] - lo[k]) / cell) + 1, 1 << 20);
    }
    auto cell_of = [&](const double* p, int64_t* ci) {
        for (int k = 0; k < 3; ++k) {
            double f = std::isfinite(p[k]) ? std::floor((p[k] - lo[k]) / cell) : 0.0;
            int64_t c = (int64_t)std::max(0.0, std::min((double)(dim[k] - 1), f));
            ci[k] = c;
        }
    };
    std::vector<std::pair<uint64_t, int>> keyed(N);
    for (int i = 0; i < N; ++i) {
        int64_t ci[3];
        cell_of(&E.pos[3 * (size_t)i], ci);
        keyed[i] = {(uint64_t)((ci[2] * dim[1] + ci[1]) * dim[0] + ci[0]), i};
    }
    std::sort(keyed.begin(), keyed.end());
    std::vector<std::vector<Contact>> per(N);
#pragma omp parallel for schedule(dynamic, 256) if (E.cfg.omp_mode == 1)
    for (int i = 0; i < N; ++i) {
        int64_t ci[3];
        cell_of(&E.pos[3 * (size_t)i], ci);
        std::vector<int> cand;
        for (int dz = -1; dz <= 1; ++dz)
            for (int dy = -1; dy <= 1; ++dy)
                for (int dx = -1; dx <= 1; ++dx) {
                    const int64_t x = ci[0] + dx, y = ci[1] + dy, z = ci[2] + dz;
                    if (x < 0 || y < 0 || z < 0 || x >= dim[0] || y >= dim[1] || z >= dim[2]) continue;
                    const uint64_t key = (uint64_t)((z * dim[1] + y) * dim[0] + x);
                    auto it = std::lower_bound(keyed.begin(), keyed.end(), std::make_pair(key, -1));
                    for (; it != keyed.end() && it->first == key; ++it) {
                        const int j = it->second;
                        if (j > i && E.scene[j] == E.scene[i]) cand.push_back(j);
                    }
                }
        std::sort(cand.begin(), cand.end());
        for (int j : cand) {
            Contact c;
            if (make_contact(E, -1, i, j, c)) per[i].push_back(c);
        }
    }
    for (int i = 0; i < N; ++i)
        for (auto& c : per[i]) out.push_back(c);
}

// Contact attributes: mu, restitution (dynamics_assembler.cpp:249-258, collision_coal.cpp:188)
void contact_props(const Engine& E, Contact& c) {
    const double muA = c.sa >= 0 ? E.smu[c.sa] : E.mu[c.ba];
    const double muB = E.mu[c.bb];
    c.mu = combine_mu(E.cfg.friction_combine, muA, muB);
    const double rnA = std_max(0.0, c.sa >= 0 ? E.srn[c.sa] : E.rn[c.ba]);
    const double rtA = std_max(0.0, c.sa >= 0 ? E.srt[c.sa] : E.rt[c.ba]);
    c.eN = std_min(rnA, std_max(0.0, E.rn[c.bb]));
    c.eT = std_min(rtA, std_max(0.0, E.rt[c.bb]));
    c.frictional = E.cfg.friction_enable && c.mu > 0.0;
}

// Sparse contact Jacobian row (CSR, column order), as assembled by rebuildW_
// (dynamics_assembler.cpp:211-332) and converted by TripletMatrix::asSparseRowMajor.
struct Rows {
    int nrows = 0, nfl = 0;
    std::vector<int32_t> ptr, col;
    std::vector<double> val;
    std::vector<double> cb, mu, e;  // contact_v_vec, mu (normal row), restitution per row
    std::vector<int32_t> row_contact;  // contact index per row, row kind in contact
    std::vector<int32_t> row_base;     // per contact: first row
};

void build_rows(const Engine& E, const std::vector<Contact>& C, Rows& W) {
    W = Rows{};
    std::vector<int> order;
    for (int pass = 0; pass < 2; ++pass)
        for (int i = 0; i < (int)C.size(); ++i)
            if ((pass == 1) == C[i].frictional) order.push_back(i);
    W.row_base.assign(C.size(), -1);
    W.ptr.push_back(0);
    for (int ci : order) {
        const Contact& c = C[ci];
        const int nr = c.frictional ? 3 : 1;
        if (!c.frictional) W.nfl++;
        W.row_base[ci] = W.nrows;
        const double* dirs[3] = {c.n, c.t1, c.t2};
        for (int r = 0; r < nr; ++r) {
            // sides in column order (lower body index first)
            struct Side { int body; double s; const double* cc; };
            Side sides[2];
            int ns = 0;
            if (c.ba >= 0) sides[ns++] = {c.ba, -1.0, &c.cA[3 * r]};
            sides[ns++] = {c.bb, 1.0, &c.cB[3 * r]};
            if (ns == 2 && sides[1].body < sides[0].body) std::swap(sides[0], sides[1]);
            for (int k = 0; k < ns; ++k) {
                const Side& sd = sides[k];
                for (int j = 0; j < 3; ++j) { W.col.push_back(6 * sd.body + j); W.val.push_back(sd.s * dirs[r][j]); }
                for (int j = 0; j < 3; ++j) { W.col.push_back(6 * sd.body + 3 + j); W.val.push_back(sd.s * sd.cc[j]); }
            }
            W.ptr.push_back((int32_t)W.col.size());
            W.cb.push_back(c.cb[r]);
            W.mu.push_back(c.frictional ? c.mu : 0.0);
            W.e.push_back(r == 0 ? c.eN : c.eT);
            W.row_contact.push_back(ci);
            W.nrows++;
        }
    }
}

// ---- projected Jacobi, src/physics/solver/projected_jacobi.cpp ----
struct PJ {
    int nrows = 0, nv = 0, nfl = 0;
    const int32_t* ptr = nullptr;
    const int32_t* col = nullptr;
    const double* val = nullptr;
    std::vector<double> RW, biasR, mu;
    // pj.rdiag_true_delassus: 0 off (R folded into RW and biasR), 1 every contact block diagonal
    // (R applied per row), 2 full blocks; Rb1 per frictionless row, Rb9 per frictional contact
    int bmode = 0;
    std::vector<double> Rb1, Rb9;
    // column-major copy of W (for the all-OpenMP W^T gather; same per-column row order)
    std::vector<int32_t> cptr, crow;
    std::vector<double> cval;
};

// projected_jacobi.cpp:100-119 (project) applied to one contact's rows
inline void project_rows(double* lam, int r, bool frictional, double mu) {
    if (!frictional) { lam[r] = std_max(lam[r], 0.0); return; }
    lam[r] = std_max(lam[r], 0.0);
    const double t1 = lam[r + 1], t2 = lam[r + 2];
    const double tn2 = t1 * t1 + t2 * t2;
    if (tn2 <= 0) return;
    const double s = std_min(1.0, (mu * lam[r]) / std::sqrt(tn2));
    lam[r + 1] = s * t1;
    lam[r + 2] = s * t2;
}

// MatrixBase::isDiagonal of Eigen 3 with its default precision for double (1e-12): every
// off-diagonal entry at most 1e-12 times the largest diagonal magnitude
bool block_is_diagonal(const double* A, int n) {
    double md = -1.0;
    for (int j = 0; j < n; ++j) md = std::max(md, std::fabs(A[j * n + j]));
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < j; ++i)
            if (!(std::fabs(A[i * n + j]) <= md * 1e-12) || !(std::fabs(A[j * n + i]) <= md * 1e-12)) return false;
    return true;
}

// invertSmallSpd (misc/block_diagonal.hpp:15-27): Cholesky A = L L^T from the lower triangle,
// column by column, then the inverse column by column (forward, then back substitution of the
// identity). A block of a contact between spheres of positive mass is positive definite, so the
// reference's LDLT fallback is not reached; a failed pivot takes its last fallback, the diagonal.
void spd_inverse(const double* A, int n, double* X) {
    double L[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    bool ok = true;
    for (int j = 0; j < n && ok; ++j) {
        double s = A[j * n + j];
        for (int k = 0; k < j; ++k) s = s - L[j * 3 + k] * L[j * 3 + k];
        if (!(s > 0.0)) { ok = false; break; }
        L[j * 3 + j] = std::sqrt(s);
        for (int i = j + 1; i < n; ++i) {
            double t = A[i * n + j];
            for (int k = 0; k < j; ++k) t = t - L[i * 3 + k] * L[j * 3 + k];
            L[i * 3 + j] = t / L[j * 3 + j];
        }
    }
    if (!ok) {
        for (int i = 0; i < n * n; ++i) X[i] = 0.0;
        for (int i = 0; i < n; ++i) X[i * n + i] = 1.0 / A[i * n + i];
        return;
    }
    for (int c = 0; c < n; ++c) {
        double y[3];
        for (int i = 0; i < n; ++i) {
            double t = (i == c) ? 1.0 : 0.0;
            for (int k = 0; k < i; ++k) t = t - L[i * 3 + k] * y[k];
            y[i] = t / L[i * 3 + i];
        }
        for (int i = n - 1; i >= 0; --i) {
            double t = y[i];
            for (int k = i + 1; k < n; ++k) t = t - L[k * 3 + i] * X[k * n + c];
            X[i * n + c] = t / L[i * 3 + i];
        }
    }
}

// buildBlockPreconditioner (projected_jacobi.cpp:81-98) and BlockDiagonal::calculateInverse
// (misc/block_diagonal.hpp:86-98): per contact D / alpha, D its block of W M^-1 W^T (the rows of
// one contact share their columns; D_ab = sum over those columns of (W_ak Minv_k) W_bk, the
// order of W_sel * Minv * W_sel^T), inverted per block, or per diagonal entry when every block
// of the step is diagonal
void block_setup(PJ& P, const double* minv, double alpha) {
    const double inv_alpha = (alpha > 0.0) ? (1.0 / alpha) : 0.0;
    const int nb = (P.nrows - P.nfl) / 3;
    std::vector<double> D1(P.nfl), D9(9 * (size_t)nb);
    for (int r = 0; r < P.nfl; ++r) {
        double d = 0.0;
        for (int k = P.ptr[r]; k < P.ptr[r + 1]; ++k) d = d + P.val[k] * P.val[k] * minv[P.col[k]];
        D1[r] = d * inv_alpha;
    }
    bool diag = true;
    for (int b = 0; b < nb; ++b) {
        const int r0 = P.nfl + 3 * b;
        const int len = P.ptr[r0 + 1] - P.ptr[r0];
        for (int a = 0; a < 3; ++a)
            for (int c = 0; c < 3; ++c) {
                const int pa = P.ptr[r0 + a], pc = P.ptr[r0 + c];
                double d = 0.0;
                for (int q = 0; q < len; ++q) d = d + (P.val[pa + q] * minv[P.col[pa + q]]) * P.val[pc + q];
                D9[9 * (size_t)b + 3 * a + c] = d * inv_alpha;
            }
        diag = diag && block_is_diagonal(&D9[9 * (size_t)b], 3);
    }
    P.Rb1.assign(P.nfl, 0.0);
    P.Rb9.assign(9 * (size_t)nb, 0.0);
    P.bmode = diag ? 1 : 2;
    for (int r = 0; r < P.nfl; ++r) {
        if (diag) P.Rb1[r] = 1.0 / D1[r];
        else spd_inverse(&D1[r], 1, &P.Rb1[r]);
    }
    for (int b = 0; b < nb; ++b) {
        const double* D = &D9[9 * (size_t)b];
        double* X = &P.Rb9[9 * (size_t)b];
        if (diag) {
            for (int a = 0; a < 3; ++a) X[4 * a] = 1.0 / D[4 * a];
        } else {
            spd_inverse(D, 3, X);
        }
    }
}

// BlockDiagonal::applyTo (misc/block_diagonal.hpp:107-126): g <- R_block g, per row when every
// block is diagonal, else per contact block (rows a: (B_a0 g0 + B_a1 g1) + B_a2 g2)
void block_apply(const PJ& P, double* g) {
    const int nb = (P.nrows - P.nfl) / 3;
    if (P.bmode == 1) {
        for (int r = 0; r < P.nfl; ++r) g[r] = g[r] * P.Rb1[r];
        for (int b = 0; b < nb; ++b)
            for (int a = 0; a < 3; ++a) g[P.nfl + 3 * b + a] = g[P.nfl + 3 * b + a] * P.Rb9[9 * (size_t)b + 4 * a];
        return;
    }
    for (int r = 0; r < P.nfl; ++r) g[r] = P.Rb1[r] * g[r];
    for (int b = 0; b < nb; ++b) {
        double* v = g + P.nfl + 3 * b;
        const double* B = &P.Rb9[9 * (size_t)b];
        double s[3];
        for (int a = 0; a < 3; ++a) s[a] = B[3 * a] * v[0] + B[3 * a + 1] * v[1] + B[3 * a + 2] * v[2];
        for (int a = 0; a < 3; ++a) v[a] = s[a];
    }
}

// build_workspace (projected_jacobi.cpp:316-369) + rdiag_sparse (:57-69); with block = 1 the rows
// and the bias stay unscaled and R_block is built instead (:341-347)
void pj_setup(PJ& P, const double* cb, const double* e, const double* mu, const double* minv, const double* vn,
              double alpha, int omp_all, int block = 0) {
    P.RW.assign(P.ptr[P.nrows], 0.0);
    P.biasR.assign(P.nrows, 0.0);
    P.mu.assign(mu, mu + P.nrows);
#pragma omp parallel for schedule(static) if (omp_all)
    for (int r = 0; r < P.nrows; ++r) {
        double vp = 0.0, D = 0.0;
        for (int k = P.ptr[r]; k < P.ptr[r + 1]; ++k) vp = vp + P.val[k] * vn[P.col[k]];
        vp = vp + cb[r];
        const double bias = cb[r] + e[r] * vp;
        for (int k = P.ptr[r]; k < P.ptr[r + 1]; ++k) D = D + (P.val[k] * P.val[k]) * minv[P.col[k]];
        if (block) {
            for (int k = P.ptr[r]; k < P.ptr[r + 1]; ++k) P.RW[k] = P.val[k];
            P.biasR[r] = bias;
            continue;
        }
        const double R = (D > 0.0) ? (alpha / D) : 0.0;
        for (int k = P.ptr[r]; k < P.ptr[r + 1]; ++k) P.RW[k] = R * P.val[k];
        P.biasR[r] = R * bias;
    }
    P.bmode = 0;
    if (block) block_setup(P, minv, alpha);
    if (omp_all) {
        std::vector<int32_t> cnt(P.nv + 1, 0);
        for (int k = 0; k < P.ptr[P.nrows]; ++k) cnt[P.col[k] + 1]++;
        for (int j = 0; j < P.nv; ++j) cnt[j + 1] += cnt[j];
        P.cptr = cnt;
        P.crow.assign(P.ptr[P.nrows], 0);
        P.cval.assign(P.ptr[P.nrows], 0.0);
        std::vector<int32_t> fill(cnt.begin(), cnt.end() - 1);
        for (int r = 0; r < P.nrows; ++r)
            for (int k = P.ptr[r]; k < P.ptr[r + 1]; ++k) {
                const int j = P.col[k];
                P.crow[fill[j]] = r;
                P.cval[fill[j]] = P.val[k];
                fill[j]++;
            }
    }
}

// dst_j += sum_r W_rj * y_r in row order (Eigen's column-major sparse * dense kernel)
void wt_accumulate(const PJ& P, const double* y, double* dst, int omp_all) {
    if (omp_all) {
#pragma omp parallel for schedule(static)
        for (int j = 0; j < P.nv; ++j) {
            double a = dst[j];
            for (int k = P.cptr[j]; k < P.cptr[j + 1]; ++k) a = a + P.cval[k] * y[P.crow[k]];
            dst[j] = a;
        }
    } else {
        for (int r = 0; r < P.nrows; ++r) {
            const double yr = y[r];
            for (int k = P.ptr[r]; k < P.ptr[r + 1]; ++k) dst[P.col[k]] = dst[P.col[k]] + P.val[k] * yr;
        }
    }
}

// frictional-row mask: rows >= nfl come in 3-row blocks
struct SweepOut { double maxd = 0, maxl = 0; };

// pj_sweep (projected_jacobi.cpp:121-138). Returns the max contact update and max |lambda_old|
// (the complementarity residual of the iterate entering the sweep).
SweepOut pj_sweep(PJ& P, double* x, double* lam, double* dlam, double* acc, const double* Mdiag, int omp_all,
                  bool apply = true) {
    const int nr = P.nrows;
    std::vector<double> lnew(nr);
#pragma omp parallel for schedule(static) if (omp_all)
    for (int r = 0; r < nr; ++r) {
        double t = 0.0;
        for (int k = P.ptr[r]; k < P.ptr[r + 1]; ++k) t = t + P.RW[k] * x[P.col[k]];
        lnew[r] = t + P.biasR[r];
    }
    if (P.bmode) block_apply(P, lnew.data());
    // elementwise loops below run in OpenMP too: each entry's arithmetic is the same in any order
#pragma omp parallel for schedule(static) if (omp_all)
    for (int r = 0; r < nr; ++r) lnew[r] = lam[r] - lnew[r];
    // project(): frictionless rows, then frictional blocks (OpenMP, as the reference)
    for (int r = 0; r < P.nfl; ++r) project_rows(lnew.data(), r, false, 0.0);
    const int nb = (nr - P.nfl) / 3;
#pragma omp parallel for schedule(static)
    for (int b = 0; b < nb; ++b) {
        const int r = P.nfl + 3 * b;
        project_rows(lnew.data(), r, true, P.mu[r]);
    }
    SweepOut so;
    auto upd = [&](int r0, int n) {
        double s = 0.0, ml = 0.0;
        for (int q = 0; q < n; ++q) {
            const double d = lnew[r0 + q] - lam[r0 + q];
            dlam[r0 + q] = d;
            s = s + d * d;
            ml = std::max(ml, std::fabs(lam[r0 + q]));
        }
        so.maxd = std::max(so.maxd, std::sqrt(s));
        so.maxl = std::max(so.maxl, ml);
    };
    for (int r = 0; r < P.nfl; ++r) upd(r, 1);
    for (int b = 0; b < nb; ++b) upd(P.nfl + 3 * b, 3);
    if (!apply) return so;
    const int nv = P.nv;
#pragma omp parallel for schedule(static) if (omp_all)
    for (int r = 0; r < nr; ++r) lam[r] = lnew[r];
#pragma omp parallel for schedule(static) if (omp_all)
    for (int j = 0; j < nv; ++j) acc[j] = 0.0;
    wt_accumulate(P, dlam, acc, omp_all);
#pragma omp parallel for schedule(static) if (omp_all)
    for (int j = 0; j < nv; ++j) x[j] = x[j] + acc[j] / Mdiag[j];
    return so;
}

inline double rel_residual(const SweepOut& s) { return s.maxd / std::max(s.maxl, 1e-30); }

// projected_jacobi.cpp:140-144 (residual)
double vel_residual(const double* x, const double* xp, int nv, double tol_rel, double tol_abs) {
    double s = 0.0;
    for (int j = 0; j < nv; ++j) {
        const double q = std::max(std::fabs(x[j]), std::fabs(xp[j])) * tol_rel + tol_abs;
        const double d = (x[j] - xp[j]) / q;
        s = s + d * d;
    }
    return 1.0 / std::sqrt((double)nv) * std::sqrt(s);
}

struct SolveResult { int iters = 0; double res_last = 0, res_final = 0; };

// ProjectedJacobiSolver::solve with standard_loop (projected_jacobi.cpp:371-377, 451-500).
// rhs is consumed (becomes rhs + W^T p), x receives the velocities, lam in/out.
SolveResult pj_solve(PJ& P, double* rhs, const double* Mdiag, double* lam, double* x, int max_iter,
                     double tol_abs, double tol_rel, double residual_tol, int omp_all, std::vector<double>* trace) {
    SolveResult res;
    wt_accumulate(P, lam, rhs, omp_all);  // rhs_init += W^T p
    for (int j = 0; j < P.nv; ++j) x[j] = rhs[j] / Mdiag[j];
    if (P.nrows == 0) return res;
    std::vector<double> dlam(P.nrows), acc(P.nv), xprev(P.nv);
    const int maxit = std::max(1, max_iter);
    // with both tolerances 0 every term of residual() is a division by zero (inf or NaN), so the
    // test is never met: the copy and the test are skipped, which changes nothing
    const bool check_vel = !(tol_abs == 0.0 && tol_rel == 0.0);
    for (int it = 0; it < maxit; ++it) {
        if (check_vel) std::copy(x, x + P.nv, xprev.begin());
        SweepOut so = pj_sweep(P, x, lam, dlam.data(), acc.data(), Mdiag, omp_all);
        res.iters = it + 1;
        res.res_last = rel_residual(so);
        if (trace) trace->insert(trace->end(), lam, lam + P.nrows);
        if (check_vel && it % 10 == 0 && vel_residual(x, xprev.data(), P.nv, tol_rel, tol_abs) <= 1) break;
        if (residual_tol > 0 && res.res_last <= residual_tol) break;
    }
    SweepOut fin = pj_sweep(P, x, lam, dlam.data(), acc.data(), Mdiag, omp_all, false);
    res.res_final = rel_residual(fin);
    return res;
}

// Reductions of the accelerated loops (norms, the velocity-increment residual, dot products)
// in a fixed order: sums over consecutive chunks of RED_CHUNK entries, each left to right, then
// the chunk sums left to right. The GPU reduces in the same order, so both agree bit for bit
// (Eigen's vectorised reductions have an order of their own; any fixed order restates them).
constexpr int RED_CHUNK = 256;
template <class F>
double chunk_sum(int n, F term) {
    double tot = 0.0;
    for (int c0 = 0; c0 < n; c0 += RED_CHUNK) {
        double s = 0.0;
        const int c1 = std::min(n, c0 + RED_CHUNK);
        for (int j = c0; j < c1; ++j) s = s + term(j);
        tot = tot + s;
    }
    return tot;
}

// projected_jacobi.cpp:140-144 (residual) with the chunked sum
double vel_residual_chunked(const double* x, const double* xp, int nv, double tol_rel, double tol_abs) {
    const double s = chunk_sum(nv, [&](int j) {
        const double q = std::max(std::fabs(x[j]), std::fabs(xp[j])) * tol_rel + tol_abs;
        const double d = (x[j] - xp[j]) / q;
        return d * d;
    });
    return 1.0 / std::sqrt((double)nv) * std::sqrt(s);
}

void pj_init(PJ& P, double* rhs, const double* Mdiag, double* lam, double* x, int omp_all) {
    wt_accumulate(P, lam, rhs, omp_all);  // rhs_init += W^T p
    for (int j = 0; j < P.nv; ++j) x[j] = rhs[j] / Mdiag[j];
}

// nesterov_loop (projected_jacobi.cpp:379-449)
// residual_tol (gpu.residual_tol, 0 = off): the loop also ends once the sweep's complementarity
// residual is at most tol, tested right after the reference's own exit (in all three loops)
SolveResult pj_solve_nesterov(PJ& P, double* rhs, const double* Mdiag, double* lam, double* x, int max_iter,
                              double tol_abs, double tol_rel, double beta_threshold, int restart_limit, int omp_all,
                              std::vector<double>* trace, double residual_tol = 0.0) {
    SolveResult res;
    pj_init(P, rhs, Mdiag, lam, x, omp_all);
    if (P.nrows == 0) return res;
    const int nv = P.nv, nr = P.nrows;
    std::vector<double> dlam(nr), acc(nv);
    std::vector<double> xk(x, x + nv), pk(lam, lam + nr), xk1(xk), pk1(pk), xy(xk), py(pk);
    double thk = 1.0, err_prev = INFINITY;
    int restarts = 0;
    bool disabled = false;
    for (int it = 0; it < std::max(1, max_iter); ++it) {
        std::copy(xy.begin(), xy.end(), x);
        std::copy(py.begin(), py.end(), lam);
        SweepOut so = pj_sweep(P, x, lam, dlam.data(), acc.data(), Mdiag, omp_all);
        std::copy(x, x + nv, xk1.begin());
        std::copy(lam, lam + nr, pk1.begin());
        res.iters = it + 1;
        res.res_last = rel_residual(so);
        if (trace) trace->insert(trace->end(), lam, lam + nr);
        const double err = vel_residual_chunked(xk1.data(), xy.data(), nv, tol_rel, tol_abs);
        if (err <= 1.0 || (residual_tol > 0 && res.res_last <= residual_tol)) break;
        const double thk1 = 0.5 * (1.0 + std::sqrt(4.0 * thk * thk + 1.0));
        const double betak1 = (thk - 1.0) / thk1;
        bool restart = false;
        if (!std::isfinite(err)) {
            restart = true;
        } else if (err_prev < INFINITY && err > 1.05 * err_prev) {
            restart = true;
        } else if (betak1 > beta_threshold) {
            restart = true;
        } else if (!std::isfinite(betak1) || betak1 < 0.0 || betak1 > 1.0) {
            restart = true;
        } else {
            const double dot = chunk_sum(nv, [&](int j) { return (xy[j] - xk1[j]) * (xk1[j] - xk[j]); });
            if (dot > 0.0) restart = true;
        }
        if (restart) {
            xy = xk1;
            py = pk1;
            xk = xk1;
            pk = pk1;
            thk = 1.0;
            if (++restarts >= restart_limit) disabled = true;
        } else {
            if (disabled) {
                xy = xk1;
                py = pk1;
                thk = 1.0;
            } else {
                for (int j = 0; j < nv; ++j) xy[j] = xk1[j] + betak1 * (xk1[j] - xk[j]);
                for (int r = 0; r < nr; ++r) py[r] = pk1[r] + betak1 * (pk1[r] - pk[r]);
                thk = thk1;
            }
            xk = xk1;
            pk = pk1;
        }
        err_prev = err;
    }
    std::copy(xk1.begin(), xk1.end(), x);
    std::copy(pk1.begin(), pk1.end(), lam);
    SweepOut fin = pj_sweep(P, x, lam, dlam.data(), acc.data(), Mdiag, omp_all, false);
    res.res_final = rel_residual(fin);
    return res;
}

// estimateSpectralRadius (projected_jacobi.cpp:154-177): power iteration on the linear part of
// the sweep map, M v = v - S^-1 W^T (R W v), eight steps, clamped below 0.995
double spectral_radius(const PJ& P, const double* Mdiag, int omp_all) {
    const int nv = P.nv, nr = P.nrows;
    if (nv <= 0) return 0.0;
    const double n0 = std::sqrt(chunk_sum(nv, [](int) { return 1.0; }));
    std::vector<double> v(nv, 1.0 / n0), delta(nr), acc(nv), Mv(nv);
    double lambda = 0.0;
    for (int it = 0; it < 8; ++it) {
        for (int r = 0; r < nr; ++r) {
            double t = 0.0;
            for (int k = P.ptr[r]; k < P.ptr[r + 1]; ++k) t = t + P.RW[k] * v[P.col[k]];
            delta[r] = t;
        }
        if (P.bmode) block_apply(P, delta.data());
        std::fill(acc.begin(), acc.end(), 0.0);
        wt_accumulate(P, delta.data(), acc.data(), omp_all);
        for (int j = 0; j < nv; ++j) Mv[j] = v[j] - acc[j] / Mdiag[j];
        const double n = std::sqrt(chunk_sum(nv, [&](int j) { return Mv[j] * Mv[j]; }));
        if (!(n > 1e-300)) return 0.0;
        lambda = n;
        for (int j = 0; j < nv; ++j) v[j] = Mv[j] / n;
    }
    return std::min(lambda, 0.995);
}

// chebyshev_loop (projected_jacobi.cpp:179-222)
SolveResult pj_solve_chebyshev(PJ& P, double* rhs, const double* Mdiag, double* lam, double* x, int max_iter,
                               double tol_abs, double tol_rel, int omp_all, std::vector<double>* trace,
                               double residual_tol = 0.0) {
    SolveResult res;
    pj_init(P, rhs, Mdiag, lam, x, omp_all);
    if (P.nrows == 0) return res;
    const int nv = P.nv, nr = P.nrows;
    const double rho = spectral_radius(P, Mdiag, omp_all);
    std::vector<double> dlam(nr), acc(nv);
    std::vector<double> xk(x, x + nv), pk(lam, lam + nr), xk1(xk), pk1(pk), xk2(nv), pk2(nr);
    const double rho2 = rho * rho;
    double omega = 1.0;
    for (int it = 0; it < std::max(1, max_iter); ++it) {
        std::copy(xk1.begin(), xk1.end(), x);
        std::copy(pk1.begin(), pk1.end(), lam);
        SweepOut so = pj_sweep(P, x, lam, dlam.data(), acc.data(), Mdiag, omp_all);
        res.iters = it + 1;
        res.res_last = rel_residual(so);
        if (trace) trace->insert(trace->end(), lam, lam + nr);
        const double err = vel_residual_chunked(x, xk1.data(), nv, tol_rel, tol_abs);
        if (err <= 1.0 || (residual_tol > 0 && res.res_last <= residual_tol)) break;
        double omega_next = (it == 0) ? (1.0 / (1.0 - rho2 * 0.5)) : (1.0 / (1.0 - (rho2 * 0.25) * omega));
        bool finite = true;
        for (int j = 0; j < nv && finite; ++j) finite = std::isfinite(x[j]);
        if (!std::isfinite(omega_next) || omega_next <= 0.0 || !finite) {
            std::copy(x, x + nv, xk2.begin());
            std::copy(lam, lam + nr, pk2.begin());
            omega_next = 1.0;
        } else {
            for (int j = 0; j < nv; ++j) xk2[j] = omega_next * (x[j] - xk[j]) + xk[j];
            for (int r = 0; r < nr; ++r) pk2[r] = omega_next * (lam[r] - pk[r]) + pk[r];
        }
        xk = xk1;
        pk = pk1;
        xk1 = xk2;
        pk1 = pk2;
        omega = omega_next;
    }
    // as the reference: the loop's current extrapolated iterate is the result
    std::copy(xk1.begin(), xk1.end(), x);
    std::copy(pk1.begin(), pk1.end(), lam);
    SweepOut fin = pj_sweep(P, x, lam, dlam.data(), acc.data(), Mdiag, omp_all, false);
    res.res_final = rel_residual(fin);
    return res;
}

// Least squares min ||f - dF g|| of the Anderson step by its normal equations (dF^T dF) g = dF^T f,
// solved by Gaussian elimination with partial pivoting. The reference uses a column-pivoted QR
// (projected_jacobi.cpp:292); for a full-rank dF both give the same minimiser. The dot products
// use the chunked order. Returns false when the system is singular or not finite.
bool anderson_ls(const std::vector<std::vector<double>>& dF, const std::vector<double>& f, int n, std::vector<double>& g) {
    const int mk = (int)dF.size();
    std::vector<double> A((size_t)mk * mk), b(mk);
    for (int j = 0; j < mk; ++j) {
        for (int l = 0; l <= j; ++l) {
            const double d = chunk_sum(n, [&](int t) { return dF[j][t] * dF[l][t]; });
            A[(size_t)j * mk + l] = d;
            A[(size_t)l * mk + j] = d;
        }
        b[j] = chunk_sum(n, [&](int t) { return dF[j][t] * f[t]; });
    }
    for (int c = 0; c < mk; ++c) {
        int piv = c;
        for (int r = c + 1; r < mk; ++r)
            if (std::fabs(A[(size_t)r * mk + c]) > std::fabs(A[(size_t)piv * mk + c])) piv = r;
        if (!(std::fabs(A[(size_t)piv * mk + c]) > 0.0)) return false;
        if (piv != c) {
            for (int k = 0; k < mk; ++k) std::swap(A[(size_t)c * mk + k], A[(size_t)piv * mk + k]);
            std::swap(b[c], b[piv]);
        }
        for (int r = c + 1; r < mk; ++r) {
            const double fct = A[(size_t)r * mk + c] / A[(size_t)c * mk + c];
            for (int k = c; k < mk; ++k) A[(size_t)r * mk + k] = A[(size_t)r * mk + k] - fct * A[(size_t)c * mk + k];
            b[r] = b[r] - fct * b[c];
        }
    }
    g.assign(mk, 0.0);
    for (int r = mk - 1; r >= 0; --r) {
        double t = b[r];
        for (int k = r + 1; k < mk; ++k) t = t - A[(size_t)r * mk + k] * g[k];
        g[r] = t / A[(size_t)r * mk + r];
    }
    for (int j = 0; j < mk; ++j)
        if (!std::isfinite(g[j])) return false;
    return true;
}

// anderson_loop (projected_jacobi.cpp:242-314): z = [x; lambda], f = g(z) - z with g one sweep,
// z_{k+1} = g(z_k) - (dZ + dF) gamma over the last m residual differences
SolveResult pj_solve_anderson(PJ& P, double* rhs, const double* Mdiag, double* lam, double* x, int max_iter,
                              double tol_abs, double tol_rel, int m, int omp_all, std::vector<double>* trace,
                              double residual_tol = 0.0) {
    SolveResult res;
    pj_init(P, rhs, Mdiag, lam, x, omp_all);
    if (P.nrows == 0) return res;
    const int nv = P.nv, nr = P.nrows, nt = nv + nr;
    m = std::max(1, m);
    std::vector<double> dlam(nr), acc(nv), z(nt), w(nt), f(nt), xprev(nv), cand(nt);
    std::copy(x, x + nv, z.begin());
    std::copy(lam, lam + nr, z.begin() + nv);
    std::vector<std::vector<double>> Zh, Fh;
    for (int it = 0; it < std::max(1, max_iter); ++it) {
        std::copy(z.begin(), z.begin() + nv, x);
        std::copy(z.begin() + nv, z.end(), lam);
        std::copy(x, x + nv, xprev.begin());
        SweepOut so = pj_sweep(P, x, lam, dlam.data(), acc.data(), Mdiag, omp_all);
        std::copy(x, x + nv, w.begin());
        std::copy(lam, lam + nr, w.begin() + nv);
        for (int t = 0; t < nt; ++t) f[t] = w[t] - z[t];
        res.iters = it + 1;
        res.res_last = rel_residual(so);
        if (trace) trace->insert(trace->end(), lam, lam + nr);
        const double err = vel_residual_chunked(x, xprev.data(), nv, tol_rel, tol_abs);
        if (err <= 1.0 || (residual_tol > 0 && res.res_last <= residual_tol)) {
            z = w;
            break;
        }
        Zh.push_back(z);
        Fh.push_back(f);
        if ((int)Fh.size() > m + 1) {
            Zh.erase(Zh.begin());
            Fh.erase(Fh.begin());
        }
        const int mk = (int)Fh.size() - 1;
        if (mk < 1) {
            z = w;
            continue;
        }
        std::vector<std::vector<double>> dF(mk, std::vector<double>(nt)), dZ(mk, std::vector<double>(nt));
        for (int j = 0; j < mk; ++j)
            for (int t = 0; t < nt; ++t) {
                dF[j][t] = Fh[j + 1][t] - Fh[j][t];
                dZ[j][t] = Zh[j + 1][t] - Zh[j][t];
            }
        std::vector<double> gam;
        bool ok = anderson_ls(dF, f, nt, gam);
        if (ok) {
            for (int t = 0; t < nt && ok; ++t) {
                double s = 0.0;
                for (int j = 0; j < mk; ++j) s = s + (dZ[j][t] + dF[j][t]) * gam[j];
                cand[t] = w[t] - s;
                ok = std::isfinite(cand[t]);
            }
        }
        if (ok) {
            z = cand;
        } else {
            z = w;
            Zh.clear();
            Fh.clear();
        }
    }
    std::copy(z.begin(), z.begin() + nv, x);
    std::copy(z.begin() + nv, z.end(), lam);
    SweepOut fin = pj_sweep(P, x, lam, dlam.data(), acc.data(), Mdiag, omp_all, false);
    res.res_final = rel_residual(fin);
    return res;
}

// loop selection as ProjectedJacobiSolver::solve (projected_jacobi.cpp:470-491): Nesterov, then
// Chebyshev, then Anderson, then the standard loop
SolveResult solve_dispatch(PJ& P, const or_config& cfg, double* rhs, const double* Mdiag, double* lam, double* x,
                           double residual_tol, int omp_all, std::vector<double>* tr) {
    if (cfg.pj_nesterov)
        return pj_solve_nesterov(P, rhs, Mdiag, lam, x, cfg.pj_max_iterations, cfg.pj_tol_abs, cfg.pj_tol_rel,
                                 cfg.pj_nesterov_beta_threshold, cfg.pj_nesterov_restart_limit, omp_all, tr,
                                 residual_tol);
    if (cfg.pj_chebyshev)
        return pj_solve_chebyshev(P, rhs, Mdiag, lam, x, cfg.pj_max_iterations, cfg.pj_tol_abs, cfg.pj_tol_rel,
                                  omp_all, tr, residual_tol);
    if (cfg.pj_anderson)
        return pj_solve_anderson(P, rhs, Mdiag, lam, x, cfg.pj_max_iterations, cfg.pj_tol_abs, cfg.pj_tol_rel,
                                 cfg.pj_anderson_m, omp_all, tr, residual_tol);
    return pj_solve(P, rhs, Mdiag, lam, x, cfg.pj_max_iterations, cfg.pj_tol_abs, cfg.pj_tol_rel, residual_tol, omp_all,
                    tr);
}

// ---- the condensed solver's sweeps, src/physics/solver/condensed_solver.cpp ----
// CondensedSolver::solve (condensed_solver.cpp:443-760) with condensed.sweep_mode gauss_seidel,
// jacobi or colored, the
// projection local solve, natural ordering, no true_schur / auto_alpha, and the standard loop, for
// sphere contacts. One block per contact in contact order (condensed_assembler.cpp:203-262); its
// rows are the contact's W rows split by side: Ja = -[d_r, r_A x d_r] on body A (when dynamic),
// Jb = +[d_r, r_B x d_r] on body B. Internally the normal impulse is <= 0 (PGS's convention,
// projectBlock :41-52) and the velocity is u = u_free - u_corr.
struct CondBlock {
    int ci, dim, a, b;  // contact, rows, dynamic body of side A (-1: static) and of side B
    double Ja[18], Jb[18];  // dim x 6, row major
    double ginv[3], rhs[3], mu;
};

// Welsh-Powell greedy coloring (misc/graph_coloring.cpp:8-40) of the blocks' shared-body graph
// (buildBlockAdjacency, condensed_solver.cpp:175-199): blocks by decreasing degree, each taking the
// smallest color no already-colored neighbour uses. Equal degrees keep block order (a stable
// sort; the reference's std::sort leaves their order unspecified). Returns the color of each block.
std::vector<int> color_blocks(const std::vector<CondBlock>& B, int nbodies, int* ncolors) {
    const int n = (int)B.size();
    std::vector<std::vector<int>> inc(nbodies);
    for (int i = 0; i < n; ++i) {
        if (B[i].a >= 0) inc[B[i].a].push_back(i);
        inc[B[i].b].push_back(i);
    }
    std::vector<std::vector<int>> adj(n);
    for (const auto& list : inc)
        for (size_t x = 0; x < list.size(); ++x)
            for (size_t y = x + 1; y < list.size(); ++y) {
                adj[list[x]].push_back(list[y]);
                adj[list[y]].push_back(list[x]);
            }
    for (auto& v : adj) {
        std::sort(v.begin(), v.end());
        v.erase(std::unique(v.begin(), v.end()), v.end());
    }
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return adj[x].size() > adj[y].size(); });
    std::vector<int> color(n, -1), stamp;
    int st = 0, nc = 0;
    for (int node : order) {
        ++st;
        for (int nb : adj[node]) {
            const int c = color[nb];
            if (c < 0) continue;
            if (c >= (int)stamp.size()) stamp.resize(c + 1, -1);
            stamp[c] = st;
        }
        int chosen = 0;
        while (chosen < (int)stamp.size() && stamp[chosen] == st) ++chosen;
        color[node] = chosen;
        nc = std::max(nc, chosen + 1);
    }
    *ncolors = nc;
    return color;
}

// u_corr += M^-1 J^T delta for one side (scatterDelta, condensed_solver.cpp:78-96)
inline void cond_scatter(const double* J, int dim, const double* d, const double* minv, double* u) {
    for (int k = 0; k < 6; ++k) {
        double t = J[k] * d[0];
        for (int r = 1; r < dim; ++r) t = t + J[6 * r + k] * d[r];
        u[k] = u[k] + minv[k] * t;
    }
}
// sum_k J_rk u_k of one row against one body's six velocities
inline double cond_row(const double* Jr, const double* u) {
    double t = Jr[0] * u[0];
    for (int k = 1; k < 6; ++k) t = t + Jr[k] * u[k];
    return t;
}

// One block of the colored sweep: coloredSweep's body (condensed_solver.cpp:205-226) with
// blockResidual (:62-69), computeBlockUpdate (:139-158) and projectBlock (:41-52).
// the block's new impulses against u (lam is overwritten; d receives new - old)
void cond_block_lambda(const CondBlock& k, double relax, double alpha, const double* u, double* lam, double* d) {
    const int dim = k.dim;
    double r[3], lo[3], ln[3];
    for (int q = 0; q < dim; ++q) {
        double o = k.rhs[q];
        if (k.a >= 0) o = o - cond_row(&k.Ja[6 * q], &u[6 * (size_t)k.a]);
        o = o - cond_row(&k.Jb[6 * q], &u[6 * (size_t)k.b]);
        o = o - 0.0 * lam[q];  // contact rows carry no compliance
        r[q] = o;
        lo[q] = lam[q];
    }
    for (int q = 0; q < dim; ++q) {
        // GiiInv is the diagonal of 1/G_ii stored as a dense block (condensed_assembler.cpp:308-312)
        double g = (q == 0 ? k.ginv[0] : 0.0) * r[0];
        for (int j = 1; j < dim; ++j) g = g + (q == j ? k.ginv[j] : 0.0) * r[j];
        ln[q] = ((relax * g) * alpha) + lo[q];
    }
    ln[0] = std::min(ln[0], 0.0);
    if (dim == 3) {
        const double tn = std::sqrt(ln[1] * ln[1] + ln[2] * ln[2]);
        if (tn > 0.0) {
            const double sc = std::min(1.0, (-k.mu * ln[0]) / tn);
            ln[1] = ln[1] * sc;
            ln[2] = ln[2] * sc;
        }
    }
    for (int q = 0; q < dim; ++q) d[q] = ln[q] - lo[q];
    for (int q = 0; q < dim; ++q) lam[q] = ln[q];
}
void cond_block_update(const CondBlock& k, double relax, double alpha, const double* minv, double* lam, double* u) {
    double d[3];
    cond_block_lambda(k, relax, alpha, u, lam, d);
    if (k.a >= 0) cond_scatter(k.Ja, k.dim, d, &minv[6 * (size_t)k.a], &u[6 * (size_t)k.a]);
    cond_scatter(k.Jb, k.dim, d, &minv[6 * (size_t)k.b], &u[6 * (size_t)k.b]);
}

struct CondResult {
    int iters = 0;
    bool diverged = false;
    double err = 0;
};

// Sums in a fixed three-level order: chunks of RED_CHUNK entries left to right, then groups of
// RED_GROUP chunk sums left to right, then the group sums left to right. A GPU sums the chunks and
// the groups in parallel and only the short last level in one thread (a single FP64 chain over
// every chunk costs a GB300 ~0.15 ms: 64 cycles a dependent FP64 add).
constexpr int RED_GROUP = 64;
template <class F>
double chunk_sum3(int n, F term) {
    double tot = 0.0;
    const int per_group = RED_CHUNK * RED_GROUP;
    for (int g0 = 0; g0 < n; g0 += per_group) {
        double gs = 0.0;
        const int g1 = std::min(n, g0 + per_group);
        for (int c0 = g0; c0 < g1; c0 += RED_CHUNK) {
            double s = 0.0;
            const int c1 = std::min(g1, c0 + RED_CHUNK);
            for (int j = c0; j < c1; ++j) s = s + term(j);
            gs = gs + s;
        }
        tot = tot + gs;
    }
    return tot;
}

// residualNorm (condensed_solver.cpp:500-506): sqrt(1/nV) ||(u_cur - u_prev) / q||, q = tol_rel
// max(|u_free - u_prev|, |u_free - u_cur|) + tol_abs, the sum in the fixed three-level order
double cond_residual(const std::vector<double>& uf, const std::vector<double>& up, const std::vector<double>& uc,
                     double tol_rel, double tol_abs) {
    const int nv = (int)uf.size();
    const double s = chunk_sum3(nv, [&](int j) {
        const double diff = uc[j] - up[j];
        const double v0 = uf[j] - up[j], v1 = uf[j] - uc[j];
        const double q = std::max(std::fabs(v0), std::fabs(v1)) * tol_rel + tol_abs;
        const double t = diff / q;
        return t * t;
    });
    return 1.0 / std::sqrt((double)nv) * std::sqrt(s);
}

// The solve: u_free (CondensedAssembler::ufree, condensed_assembler.cpp:348-356), rhs (:367-462),
// the warm start with the normal sign inverted (warmstart.hpp:26-39), the initial u_corr, the
// coloring, then colored sweeps until the residual is below 1 (or diverges). x receives
// u = u_free - u_corr; lam_mem the impulses as stored for the next step (normal sign inverted back).
CondResult condensed_colored(const Engine& E, const std::vector<Contact>& C, double dt, std::vector<double>& x,
                             std::vector<double>& lam_mem) {
    const int N = E.N, nv = 6 * N;
    const bool implicit_gyro = E.cfg.moreau_implicit_gyroscopy != 0;
    std::vector<double> uf(nv);
    for (int i = 0; i < N; ++i) {
        const double* w = &E.w[3 * (size_t)i];
        const double Iw[3] = {E.inertia[i] * w[0], E.inertia[i] * w[1], E.inertia[i] * w[2]};
        double cgy[3];
        cross3(w, Iw, cgy);
        for (int k = 0; k < 6; ++k) {
            const size_t j = 6 * (size_t)i + k;
            const double vn = k < 3 ? E.v[3 * (size_t)i + k] : w[k - 3];
            const double fext = k < 3 ? E.mass[i] * E.cfg.sim_gravity[k] : 0.0;
            double u = vn + E.minv[j] * (dt * fext);
            if (!implicit_gyro) u = u + E.minv[j] * (dt * (k < 3 ? 0.0 : -cgy[k - 3]));
            uf[j] = u;
        }
    }
    CondResult res;
    if (C.empty()) {  // no constraint rows: the free velocity (condensed_solver.cpp:453)
        x = uf;
        lam_mem.clear();
        return res;
    }
    std::vector<CondBlock> B(C.size());
    for (size_t ci = 0; ci < C.size(); ++ci) {
        const Contact& c = C[ci];
        CondBlock& k = B[ci];
        k.ci = (int)ci;
        k.dim = c.frictional ? 3 : 1;
        k.a = c.ba;
        k.b = c.bb;
        k.mu = c.mu;
        const double* dirs[3] = {c.n, c.t1, c.t2};
        for (int q = 0; q < k.dim; ++q)
            for (int j = 0; j < 3; ++j) {
                k.Ja[6 * q + j] = -dirs[q][j];
                k.Ja[6 * q + 3 + j] = -c.cA[3 * q + j];
                k.Jb[6 * q + j] = dirs[q][j];
                k.Jb[6 * q + 3 + j] = c.cB[3 * q + j];
            }
        for (int q = 0; q < k.dim; ++q) {
            // G_ii = Ja diag(M^-1) Ja^T + Jb diag(M^-1) Jb^T, its diagonal (condensed_assembler.cpp:244-256)
            double ga = 0.0;
            if (k.a >= 0) {
                ga = (k.Ja[6 * q] * E.minv[6 * (size_t)k.a]) * k.Ja[6 * q];
                for (int j = 1; j < 6; ++j) ga = ga + (k.Ja[6 * q + j] * E.minv[6 * (size_t)k.a + j]) * k.Ja[6 * q + j];
            }
            double gb = (k.Jb[6 * q] * E.minv[6 * (size_t)k.b]) * k.Jb[6 * q];
            for (int j = 1; j < 6; ++j) gb = gb + (k.Jb[6 * q + j] * E.minv[6 * (size_t)k.b + j]) * k.Jb[6 * q + j];
            const double G = (0.0 + ga) + gb;
            k.ginv[q] = G > 0 ? 1.0 / G : 0.0;
            double ut = 0.0;
            if (k.a >= 0) ut = ut + cond_row(&k.Ja[6 * q], &uf[6 * (size_t)k.a]);
            ut = ut + cond_row(&k.Jb[6 * q], &uf[6 * (size_t)k.b]);
            k.rhs[q] = ut + c.cb[q];
        }
    }
    // impulses (normal <= 0 inside) and the initial u_corr = sum_blocks M^-1 J^T lambda
    std::vector<double> lam(3 * C.size(), 0.0), u(nv, 0.0);
    for (size_t ci = 0; ci < C.size(); ++ci) {
        const CondBlock& k = B[ci];
        double* l = &lam[3 * ci];
        if (E.cfg.pj_warmstart) {
            l[0] = -C[ci].lam0[0];
            if (k.dim == 3) {
                l[1] = C[ci].lam0[1];
                l[2] = C[ci].lam0[2];
            }
        }
        if (k.a >= 0) cond_scatter(k.Ja, k.dim, l, &E.minv[6 * (size_t)k.a], &u[6 * (size_t)k.a]);
        cond_scatter(k.Jb, k.dim, l, &E.minv[6 * (size_t)k.b], &u[6 * (size_t)k.b]);
    }
    // the sweep mode: 0 gauss_seidel (gaussSeidelSweep, :166-182: blocks in order, u_corr updated
    // after each), 1 jacobi (jacobiSweep, :268-317: every block against the previous sweep's
    // u_corr, then each body gathers its blocks' increments in block order), 2 colored
    const int mode = E.cfg.condensed_sweep_mode;
    std::vector<std::vector<int>> classes;
    if (mode == 2) {
        int ncol = 0;
        const std::vector<int> color = color_blocks(B, N, &ncol);
        classes.resize(ncol);
        for (size_t i = 0; i < B.size(); ++i) classes[color[i]].push_back((int)i);
    } else {
        classes.resize(1);
        for (size_t i = 0; i < B.size(); ++i) classes[0].push_back((int)i);
    }
    std::vector<std::vector<std::pair<int, int>>> blocks_of(mode == 1 ? N : 0);  // (block, side) in block order
    if (mode == 1)
        for (size_t i = 0; i < B.size(); ++i) {
            if (B[i].a >= 0) blocks_of[B[i].a].push_back({(int)i, 0});
            blocks_of[B[i].b].push_back({(int)i, 1});
        }
    std::vector<double> dl(mode == 1 ? 3 * B.size() : 0), uread;
    const double relax = E.cfg.pj_relaxation, alpha = E.cfg.pj_alpha;
    std::vector<double> uprev = u;
    for (int it = 0; it < E.cfg.pj_max_iterations; ++it) {
        if (mode == 1) {
            uread = u;
            for (size_t bi = 0; bi < B.size(); ++bi) {
                dl[3 * bi + 1] = dl[3 * bi + 2] = 0.0;
                cond_block_lambda(B[bi], relax, alpha, uread.data(), &lam[3 * bi], &dl[3 * bi]);
            }
            for (int b = 0; b < N; ++b) {
                if (blocks_of[b].empty()) continue;
                double acc[6] = {0, 0, 0, 0, 0, 0};
                for (const auto& bs : blocks_of[b]) {
                    const CondBlock& k = B[bs.first];
                    const double* J = bs.second ? k.Jb : k.Ja;
                    const double* d = &dl[3 * (size_t)bs.first];
                    for (int c = 0; c < 6; ++c) {
                        double t = J[c] * d[0];
                        for (int q = 1; q < k.dim; ++q) t = t + J[6 * q + c] * d[q];
                        acc[c] = acc[c] + t;
                    }
                }
                for (int c = 0; c < 6; ++c)
                    u[6 * (size_t)b + c] = uread[6 * (size_t)b + c] + E.minv[6 * (size_t)b + c] * acc[c];
            }
        } else {
            for (const auto& cls : classes)
                for (int bi : cls) cond_block_update(B[bi], relax, alpha, E.minv.data(), &lam[3 * (size_t)bi], u.data());
        }
        res.iters = it + 1;
        res.err = cond_residual(uf, uprev, u, E.cfg.pj_tol_rel, E.cfg.pj_tol_abs);
        if (!std::isfinite(res.err)) {
            res.diverged = true;  // checkResidual throws "Condensed solver diverged" (:507-513)
            break;
        }
        if (res.err < 1.0) break;
        uprev = u;
    }
    x.assign(nv, 0.0);
    for (int j = 0; j < nv; ++j) x[j] = uf[j] - u[j];
    lam_mem.assign(3 * C.size(), 0.0);
    for (size_t ci = 0; ci < C.size(); ++ci) {
        lam_mem[3 * ci] = -lam[3 * ci];
        if (B[ci].dim == 3) {
            lam_mem[3 * ci + 1] = lam[3 * ci + 1];
            lam_mem[3 * ci + 2] = lam[3 * ci + 2];
        }
    }
    return res;
}

// ---- projected Gauss-Seidel, src/physics/solver/projected_gauss_seidel.cpp ----
// ProjectedGaussSeidelSolver::solve (projected_gauss_seidel.cpp:56-264) with the plain loop, for
// contact rows only (no springs or dampers). The blocks are the contacts in W's row order
// (frictionless contacts first, then frictional ones, each in contact order); a sweep visits them
// in that order (pgs_sweep, :158-182). Inside, the normal impulse is <= 0 (project, :11-27) and the
// velocity is u = u_free - u_corr with u_corr = M^-1 W^T lambda.
//   u_free = v + M^-1 (h f_ext) [+ M^-1 (h f_gyro)]        PgsAssembler::ufree (pgs_assembler.cpp:96-103)
//   rhs    = W u_free + b (+ e . (W v + b) with restitution)  PgsAssembler::rhs (:71-80)
//   Dinv   = 1 / sum_nz w^2 M^-1_col per row                   PgsAssembler::DinvDiag (:219-294)
// Sums run in W's column order, from zero, as Eigen's row-major sparse kernels do; u_corr gets its
// terms column by column (W row order), as Eigen's column-major M^-1 W^T kernels do.
CondResult pgs_solve(const Engine& E, const std::vector<Contact>& C, const Rows& W, double dt, std::vector<double>& x,
                     std::vector<double>& lam_mem) {
    const int N = E.N, nv = 6 * N, nr = W.nrows;
    const bool implicit_gyro = E.cfg.moreau_implicit_gyroscopy != 0;
    std::vector<double> uf(nv), vn(nv);
    for (int i = 0; i < N; ++i) {
        const double* w = &E.w[3 * (size_t)i];
        const double Iw[3] = {E.inertia[i] * w[0], E.inertia[i] * w[1], E.inertia[i] * w[2]};
        double cgy[3];
        cross3(w, Iw, cgy);
        for (int k = 0; k < 6; ++k) {
            const size_t j = 6 * (size_t)i + k;
            const double v = k < 3 ? E.v[3 * (size_t)i + k] : w[k - 3];
            const double fext = k < 3 ? E.mass[i] * E.cfg.sim_gravity[k] : 0.0;
            double u = v + E.minv[j] * (dt * fext);
            if (!implicit_gyro) u = u + E.minv[j] * (dt * (k < 3 ? 0.0 : -cgy[k - 3]));
            uf[j] = u;
            vn[j] = v;
        }
    }
    CondResult res;
    if (nr == 0) {  // numLambda == 0: the free velocity (projected_gauss_seidel.cpp:79)
        x = uf;
        lam_mem.clear();
        return res;
    }
    auto row_dot = [&](int r, const double* u) {
        double t = 0.0;
        for (int k = W.ptr[r]; k < W.ptr[r + 1]; ++k) t = t + W.val[k] * u[W.col[k]];
        return t;
    };
    bool restitution = false;
    for (int r = 0; r < nr; ++r) restitution = restitution || W.e[r] != 0.0;
    std::vector<double> rhs(nr), dinv(nr);
    for (int r = 0; r < nr; ++r) {
        double b = W.cb[r];
        if (restitution) b = b + W.e[r] * (row_dot(r, vn.data()) + W.cb[r]);
        rhs[r] = row_dot(r, uf.data()) + b;
        double d = 0.0;
        for (int k = W.ptr[r]; k < W.ptr[r + 1]; ++k) d = d + (W.val[k] * W.val[k]) * E.minv[W.col[k]];
        // frictionless rows guard a zero diagonal (:284-287); frictional ones take cwiseInverse (:289-292)
        dinv[r] = r < W.nfl ? (d > 0 ? 1.0 / d : 0.0) : 1.0 / d;
    }
    // warm start with the normal sign inverted (:103-109), then u_corr = M^-1 W^T lambda (:117)
    std::vector<double> lam(nr, 0.0), u(nv, 0.0);
    if (E.cfg.pj_warmstart)
        for (size_t ci = 0; ci < C.size(); ++ci) {
            const int r0 = W.row_base[ci];
            lam[r0] = -C[ci].lam0[0];
            if (C[ci].frictional) {
                lam[r0 + 1] = C[ci].lam0[1];
                lam[r0 + 2] = C[ci].lam0[2];
            }
        }
    auto scatter_row = [&](int r, double d) {
        for (int k = W.ptr[r]; k < W.ptr[r + 1]; ++k) {
            const int j = W.col[k];
            u[j] = u[j] + (E.minv[j] * W.val[k]) * d;
        }
    };
    for (int r = 0; r < nr; ++r) scatter_row(r, lam[r]);
    const double relax = E.cfg.pj_relaxation, alpha = E.cfg.pj_alpha;
    // blocks: one row per frictionless contact, then three per frictional contact
    auto block_update = [&](int r0, int dim) {
        double rs[3], dl[3];
        for (int q = 0; q < dim; ++q) {
            double o = rhs[r0 + q];
            o = o - row_dot(r0 + q, u.data());
            o = o - 0.0 * lam[r0 + q];  // C is zero on contact rows
            rs[q] = o;
        }
        for (int q = 0; q < dim; ++q) {
            // the block of Dinv is diagonal, stored dense (BlockDiagonal::addBlockDiag)
            double g = (q == 0 ? dinv[r0] : 0.0) * rs[0];
            for (int j = 1; j < dim; ++j) g = g + (q == j ? dinv[r0 + j] : 0.0) * rs[j];
            dl[q] = (g * relax) * alpha;
            lam[r0 + q] = lam[r0 + q] + dl[q];
        }
        // project (:11-27): the corrections enter dlambda
        const double n0 = lam[r0];
        lam[r0] = std::min(n0, 0.0);
        dl[0] = dl[0] + (lam[r0] - n0);
        if (dim == 3) {
            const double t1 = lam[r0 + 1], t2 = lam[r0 + 2];
            const double tn = std::sqrt(t1 * t1 + t2 * t2);
            if (tn > 0.0) {
                const double s = std::min(1.0, -(W.mu[r0] * lam[r0]) / tn);
                const double p1 = s * t1, p2 = s * t2;
                dl[1] = dl[1] + (p1 - t1);
                dl[2] = dl[2] + (p2 - t2);
                lam[r0 + 1] = p1;
                lam[r0 + 2] = p2;
            }
        }
        for (int q = 0; q < dim; ++q) scatter_row(r0 + q, dl[q]);
    };
    std::vector<double> uprev = u;
    for (int it = 0; it < E.cfg.pj_max_iterations; ++it) {
        for (int r = 0; r < nr;) {
            const int dim = r < W.nfl ? 1 : 3;
            block_update(r, dim);
            r += dim;
        }
        res.iters = it + 1;
        // check_residual (:142-151): the velocity-increment residual of u_corr, summed in the
        // fixed three-level order; a non-finite value throws "Projected Gauss-Seidel diverged"
        res.err = cond_residual(uf, uprev, u, E.cfg.pj_tol_rel, E.cfg.pj_tol_abs);
        if (!std::isfinite(res.err)) {
            res.diverged = true;
            break;
        }
        if (res.err < 1.0) break;
        uprev = u;
    }
    x.assign(nv, 0.0);
    for (int j = 0; j < nv; ++j) x[j] = uf[j] - u[j];
    // storeImpulse with the normal sign inverted (:257-259)
    lam_mem.assign(3 * C.size(), 0.0);
    for (size_t ci = 0; ci < C.size(); ++ci) {
        const int r0 = W.row_base[ci];
        lam_mem[3 * ci] = -lam[r0];
        if (C[ci].frictional) {
            lam_mem[3 * ci + 1] = lam[r0 + 1];
            lam_mem[3 * ci + 2] = lam[r0 + 2];
        }
    }
    return res;
}

// MoreauIntegrator::step (src/physics/integration/moreau.cpp:6-13)
void step_once(Engine& E) {
    const int N = E.N, S = E.S, nv = 6 * N;
    const double dt = E.cfg.sim_dt, th = E.cfg.moreau_theta;
    const int omp_all = E.cfg.omp_mode == 1;
    // refreshState: f_ext = m g, f_gyro = -w x (I w)  (world.cpp:113-173); rhs (pj_assembler.cpp:152-153).
    // With moreau.implicit_gyroscopy the rhs leaves dt f_gyro out and S gains -dt G_rot with
    // G_rot = (([I w]x - [w]x I) / 2 (pj_assembler.cpp:32-61); for an isotropic I every entry of
    // G_rot is i w_k - w_k i = 0 exactly, so S stays diag(M).
    const bool implicit_gyro = E.cfg.moreau_implicit_gyroscopy != 0;
    std::vector<double> rhs(nv), vn(nv);
    // the per-body loops of the step are elementwise: OpenMP in the all-threads mode
#pragma omp parallel for schedule(static) if (omp_all)
    for (int i = 0; i < N; ++i) {
        const double* w = &E.w[3 * (size_t)i];
        const double Iw[3] = {E.inertia[i] * w[0], E.inertia[i] * w[1], E.inertia[i] * w[2]};
        double c[3];
        cross3(w, Iw, c);
        for (int k = 0; k < 3; ++k) {
            const double fext = E.mass[i] * E.cfg.sim_gravity[k];
            const double Ml = E.Mdiag[6 * i + k];
            rhs[6 * i + k] = (Ml * E.v[3 * (size_t)i + k] + dt * fext) + dt * 0.0;
            const double Ma = E.Mdiag[6 * i + 3 + k];
            rhs[6 * i + 3 + k] = implicit_gyro ? (Ma * w[k] + dt * 0.0) : (Ma * w[k] + dt * 0.0) + dt * (-c[k]);
            vn[6 * i + k] = E.v[3 * (size_t)i + k];
            vn[6 * i + 3 + k] = w[k];
        }
    }
    // drift 1: (1 - theta) h, every entity with a velocity (statics included)
    const double h1 = (1.0 - th) * dt;
#pragma omp parallel for schedule(static) if (omp_all)
    for (int i = 0; i < N; ++i) drift(&E.pos[3 * (size_t)i], &E.q[4 * (size_t)i], &E.v[3 * (size_t)i], &E.w[3 * (size_t)i], h1);
    for (int s = 0; s < S; ++s) drift(&E.spos[3 * s], &E.sq[4 * s], &E.sv[3 * s], &E.sw[3 * s], h1);
#pragma omp parallel for schedule(static) if (omp_all)
    for (int i = 0; i < N; ++i) rotmat(&E.q[4 * (size_t)i], &E.R[9 * (size_t)i]);
    for (int s = 0; s < S; ++s) rotmat(&E.sq[4 * s], &E.sR[9 * s]);
    // updateStateDependentTerms begins with DerivedEntitySync::updateEntities, which runs
    // Trajectory::update (dynamics_assembler.cpp:515-522, trajectory.cpp:69-120): the statics'
    // prescribed pose and twist, evaluated by the caller, replace their own
    for (int s = 0; s < S; ++s) {
        const int f = E.smflag.empty() ? 0 : E.smflag[s];
        if (!f) continue;
        const double* m = &E.smot[13 * (size_t)s];
        for (int k = 0; k < 3; ++k) {
            if (f & 1) E.spos[3 * s + k] = m[k];
            if (f & 4) E.sv[3 * s + k] = m[7 + k];
            if (f & 8) E.sw[3 * s + k] = m[10 + k];
        }
        if (f & 2)
            for (int k = 0; k < 4; ++k) E.sq[4 * s + k] = m[3 + k];
        rotmat(&E.sq[4 * s], &E.sR[9 * s]);
        E.smflag[s] = 0;
    }

    // updateStateDependentTerms: collision + W
    std::vector<Contact> C;
    detect(E, C);
#pragma omp parallel for schedule(static) if (omp_all)
    for (int i = 0; i < (int)C.size(); ++i) {
        contact_rows(E, C[i]);
        contact_props(E, C[i]);
    }
    // warm start: nearest previous contact of the same pair within collision.match_max_dist
    // (contact_tracker.cpp:43-72, :11-20; warmstart.hpp:26-39)
    const double max2 = E.cfg.collision_match_max_dist * E.cfg.collision_match_max_dist;
    if (E.cfg.pj_warmstart) {
        for (auto& c : C) {
            auto it = std::lower_bound(E.prev_keys.begin(), E.prev_keys.end(), c.key());
            if (it == E.prev_keys.end() || *it != c.key()) continue;
            const size_t j = (size_t)(it - E.prev_keys.begin());
            double d[3];
            for (int k = 0; k < 3; ++k) d[k] = c.point[k] - E.prev_point[3 * j + k];
            if (dot3(d, d) <= max2)
                for (int k = 0; k < 3; ++k) c.lam0[k] = E.prev_lambda[3 * j + k];
        }
    }
    Rows W;
    build_rows(E, C, W);
    PJ P;
    P.nrows = W.nrows;
    P.nv = nv;
    P.nfl = W.nfl;
    P.ptr = W.ptr.data();
    P.col = W.col.data();
    P.val = W.val.data();
    pj_setup(P, W.cb.data(), W.e.data(), W.mu.data(), E.minv.data(), vn.data(), E.cfg.pj_alpha, omp_all,
             E.cfg.pj_rdiag_true_delassus);
    std::vector<double> lam(W.nrows, 0.0), x(nv);
    for (size_t ci = 0; ci < C.size(); ++ci) {
        const int r0 = W.row_base[ci];
        const int nr = C[ci].frictional ? 3 : 1;
        for (int k = 0; k < nr; ++k) lam[r0 + k] = C[ci].lam0[k];
    }
    E.trace.clear();
    SolveResult sr;
    std::vector<double> cond_mem;
    if (E.cfg.solver_type == 1 || E.cfg.solver_type == 2) {
        // solver.type=condensed (colored sweeps) or projected_gauss_seidel; the stats residual is
        // the complementarity residual of the result with the impulses in the projected Jacobi
        // convention
        CondResult cr = E.cfg.solver_type == 1 ? condensed_colored(E, C, dt, x, cond_mem) : pgs_solve(E, C, W, dt, x, cond_mem);
        sr.iters = cr.iters;
        sr.res_last = cr.err;
        if (cr.diverged) E.status = 4;
        for (size_t ci = 0; ci < C.size(); ++ci) {
            const int r0 = W.row_base[ci];
            lam[r0] = cond_mem[3 * ci];
            if (C[ci].frictional) {
                lam[r0 + 1] = -cond_mem[3 * ci + 1];
                lam[r0 + 2] = -cond_mem[3 * ci + 2];
            }
        }
        if (!C.empty()) {
            std::vector<double> dl(W.nrows), ac(nv);
            SweepOut fin = pj_sweep(P, x.data(), lam.data(), dl.data(), ac.data(), E.Mdiag.data(), omp_all, false);
            sr.res_final = rel_residual(fin);
        }
    } else if (C.empty()) {
#pragma omp parallel for schedule(static) if (omp_all)
        for (int j = 0; j < nv; ++j) x[j] = rhs[j] / E.Mdiag[j];
    } else {
        std::vector<double>* tr = E.trace_on ? &E.trace : nullptr;
        sr = solve_dispatch(P, E.cfg, rhs.data(), E.Mdiag.data(), lam.data(), x.data(), E.cfg.residual_tol, omp_all,
                            tr);
    }
    E.trace_on = false;
    // storeImpulse (warmstart.hpp:41-56) and the tracker's memory for the next step
    E.prev_keys.resize(C.size());
    E.prev_point.resize(3 * C.size());
    E.prev_lambda.assign(3 * C.size(), 0.0);
    for (size_t ci = 0; ci < C.size(); ++ci) {
        E.prev_keys[ci] = C[ci].key();
        for (int k = 0; k < 3; ++k) E.prev_point[3 * ci + k] = C[ci].point[k];
        const int r0 = W.row_base[ci];
        const int nr = C[ci].frictional ? 3 : 1;
        for (int k = 0; k < nr; ++k) E.prev_lambda[3 * ci + k] = E.cfg.solver_type != 0 ? cond_mem[3 * ci + k] : lam[r0 + k];
    }
    E.last = C;
    E.last_lambda = E.prev_lambda;
    // writeVelocityToSystem (dynamics_assembler.cpp:145-188)
#pragma omp parallel for schedule(static) if (omp_all)
    for (int i = 0; i < N; ++i)
        for (int k = 0; k < 3; ++k) {
            E.v[3 * (size_t)i + k] = x[6 * i + k];
            E.w[3 * (size_t)i + k] = x[6 * i + 3 + k];
        }
    // drift 2: theta h
    const double h2 = th * dt;
#pragma omp parallel for schedule(static) if (omp_all)
    for (int i = 0; i < N; ++i) drift(&E.pos[3 * (size_t)i], &E.q[4 * (size_t)i], &E.v[3 * (size_t)i], &E.w[3 * (size_t)i], h2);
    for (int s = 0; s < S; ++s) drift(&E.spos[3 * s], &E.sq[4 * s], &E.sv[3 * s], &E.sw[3 * s], h2);
    E.stats.num_contacts = (int32_t)C.size();
    E.stats.num_rows = W.nrows;
    E.stats.iterations = sr.iters;
    E.stats.residual = sr.res_final;
    E.stats.residual_last = sr.res_last;
}

}  // namespace

extern "C" {

void* or_create(const or_config* cfg, const or_scene* sc) {
    Engine* E = new Engine();
    E->cfg = *cfg;
    E->N = sc->num_bodies;
    E->S = sc->num_statics;
    const size_t N = (size_t)E->N, S = (size_t)E->S;
    E->pos.assign(sc->pos, sc->pos + 3 * N);
    E->q.assign(sc->quat, sc->quat + 4 * N);
    E->v.assign(sc->vel, sc->vel + 3 * N);
    E->w.assign(sc->omega, sc->omega + 3 * N);
    E->rad.assign(sc->radius, sc->radius + N);
    E->mass.assign(sc->mass, sc->mass + N);
    E->inertia.assign(sc->inertia, sc->inertia + N);
    E->mu.assign(sc->mu, sc->mu + N);
    E->rn.assign(sc->rest_n, sc->rest_n + N);
    E->rt.assign(sc->rest_t, sc->rest_t + N);
    E->scene.assign(N, 0);
    if (sc->body_scene) E->scene.assign(sc->body_scene, sc->body_scene + N);
    E->R.assign(9 * N, 0.0);
    for (size_t i = 0; i < N; ++i) E->rmax = std::max(E->rmax, E->rad[i]);
    E->skind.assign(sc->static_kind, sc->static_kind + S);
    E->spos.assign(sc->static_pos, sc->static_pos + 3 * S);
    E->sq.assign(sc->static_quat, sc->static_quat + 4 * S);
    E->sv.assign(sc->static_vel, sc->static_vel + 3 * S);
    E->sw.assign(sc->static_omega, sc->static_omega + 3 * S);
    E->sdir.assign(3 * S, 0.0);
    E->sd.assign(S, 0.0);
    for (size_t s = 0; s < S; ++s) {
        // plane.normal.normalized() and d = n . x (collision_coal.cpp:292-297)
        const double* u = &sc->static_dir[3 * s];
        const double n2 = dot3(u, u);
        const double n = std::sqrt(n2);
        for (int k = 0; k < 3; ++k) E->sdir[3 * s + k] = n2 > 0 ? u[k] / n : u[k];
        E->sd[s] = dot3(&E->sdir[3 * s], &E->spos[3 * s]);
    }
    E->srad.assign(S, 0.0);
    if (sc->static_radius) E->srad.assign(sc->static_radius, sc->static_radius + S);
    E->shl.assign(S, 0.0);
    if (sc->static_half_length) E->shl.assign(sc->static_half_length, sc->static_half_length + S);
    E->she.assign(3 * S, 0.0);
    if (sc->static_half_extents) E->she.assign(sc->static_half_extents, sc->static_half_extents + 3 * S);
    // a cylinder's axis in the static's own frame, R(q0)^T u
    E->sax.assign(3 * S, 0.0);
    for (size_t s = 0; s < S; ++s) {
        double R0[9];
        rotmat(&E->sq[4 * s], R0);
        matTvec(R0, &E->sdir[3 * s], &E->sax[3 * s]);
    }
    E->smu.assign(sc->static_mu, sc->static_mu + S);
    E->srn.assign(sc->static_rest_n, sc->static_rest_n + S);
    E->srt.assign(sc->static_rest_t, sc->static_rest_t + S);
    E->sscene.assign(S, 0);
    if (sc->static_scene) E->sscene.assign(sc->static_scene, sc->static_scene + S);
    E->sR.assign(9 * S, 0.0);
    build_mass(*E);
#ifdef _OPENMP
    if (cfg->num_threads > 0) omp_set_num_threads(cfg->num_threads);
#endif
    return E;
}

void or_destroy(void* h) { delete (Engine*)h; }

void or_set_static_motion(void* h, int32_t count, const int32_t* statics, const double* pos, const double* quat,
                          const double* vel, const double* omega) {
    Engine& E = *(Engine*)h;
    if (E.smflag.size() != (size_t)E.S) {
        E.smflag.assign(E.S, 0);
        E.smot.assign(13 * (size_t)E.S, 0.0);
    }
    const int f = (pos ? 1 : 0) | (quat ? 2 : 0) | (vel ? 4 : 0) | (omega ? 8 : 0);
    for (int32_t c = 0; c < count; ++c) {
        const int s = statics[c];
        if (s < 0 || s >= E.S) continue;
        double* m = &E.smot[13 * (size_t)s];
        for (int k = 0; k < 3; ++k) {
            if (pos) m[k] = pos[3 * (size_t)c + k];
            if (vel) m[7 + k] = vel[3 * (size_t)c + k];
            if (omega) m[10 + k] = omega[3 * (size_t)c + k];
        }
        if (quat)
            for (int k = 0; k < 4; ++k) m[3 + k] = quat[4 * (size_t)c + k];
        E.smflag[s] |= f;
    }
}

void or_get_static_state(void* h, double* pos, double* quat, double* vel, double* omega) {
    const Engine& E = *(const Engine*)h;
    for (int s = 0; s < E.S; ++s) {
        for (int k = 0; k < 3; ++k) {
            if (pos) pos[3 * s + k] = E.spos[3 * s + k];
            if (vel) vel[3 * s + k] = E.sv[3 * s + k];
            if (omega) omega[3 * s + k] = E.sw[3 * s + k];
        }
        if (quat)
            for (int k = 0; k < 4; ++k) quat[4 * s + k] = E.sq[4 * s + k];
    }
}

int or_step(void* h, int32_t nsteps) {
    Engine* E = (Engine*)h;
    E->status = 0;
    for (int s = 0; s < nsteps && !E->status; ++s) step_once(*E);
    return E->status;
}

void or_get_state(void* h, double* pos, double* quat, double* vel, double* omega) {
    Engine* E = (Engine*)h;
    if (pos) std::copy(E->pos.begin(), E->pos.end(), pos);
    if (quat) std::copy(E->q.begin(), E->q.end(), quat);
    if (vel) std::copy(E->v.begin(), E->v.end(), vel);
    if (omega) std::copy(E->w.begin(), E->w.end(), omega);
}

void or_get_stats(void* h, or_stats* out) { *out = ((Engine*)h)->stats; }

int32_t or_get_contacts(void* h, int32_t* id_a, int32_t* id_b, double* point, double* lambda, double* normal) {
    Engine* E = (Engine*)h;
    const size_t C = E->last.size();
    for (size_t i = 0; i < C; ++i) {
        if (id_a) id_a[i] = E->last[i].a;
        if (id_b) id_b[i] = E->last[i].b;
        for (int k = 0; k < 3; ++k) {
            if (point) point[3 * i + k] = E->last[i].point[k];
            if (normal) normal[3 * i + k] = E->last[i].n[k];
            if (lambda) lambda[3 * i + k] = E->last_lambda[3 * i + k];
        }
    }
    return (int32_t)C;
}

// the tracker's memory for the next step's warm start (contact_tracker.cpp:11-72): pairs sorted by
// key, their contact points and impulses
void or_set_contacts(void* h, int32_t n, const int32_t* id_a, const int32_t* id_b, const double* point,
                     const double* lambda) {
    Engine* E = (Engine*)h;
    std::vector<size_t> order(n);
    for (int32_t i = 0; i < n; ++i) order[i] = (size_t)i;
    auto key = [&](size_t i) { return ((uint64_t)(uint32_t)id_a[i] << 32) | (uint64_t)(uint32_t)id_b[i]; };
    std::sort(order.begin(), order.end(), [&](size_t x, size_t y) { return key(x) < key(y); });
    E->prev_keys.resize(n);
    E->prev_point.resize(3 * (size_t)n);
    E->prev_lambda.resize(3 * (size_t)n);
    for (int32_t c = 0; c < n; ++c) {
        const size_t o = order[c];
        E->prev_keys[c] = key(o);
        for (int k = 0; k < 3; ++k) {
            E->prev_point[3 * (size_t)c + k] = point[3 * o + k];
            E->prev_lambda[3 * (size_t)c + k] = lambda[3 * o + k];
        }
    }
}

void or_set_trace(void* h, int32_t on) { ((Engine*)h)->trace_on = on != 0; }

int32_t or_get_trace(void* h, double* out, int64_t max_values) {
    Engine* E = (Engine*)h;
    const int64_t n = std::min<int64_t>(max_values, (int64_t)E->trace.size());
    if (out) std::copy(E->trace.begin(), E->trace.begin() + n, out);
    return (int32_t)E->trace.size();
}

int32_t or_pj_solve_csr(int32_t nrows, int32_t nv, int32_t nfl, const int32_t* row_ptr, const int32_t* col,
                        const double* val, const double* contact_bias, const double* mu, const double* restitution,
                        const double* minv, const double* mdiag, const double* v, const double* f_ext,
                        const double* f_gyro, double dt, double alpha, int32_t max_iter, double tol_abs,
                        double tol_rel, double* lambda_inout, double* x_out) {
    PJ P;
    P.nrows = nrows;
    P.nv = nv;
    P.nfl = nfl;
    P.ptr = row_ptr;
    P.col = col;
    P.val = val;
    // PjAssembler::rhs (pj_assembler.cpp:152-153): M v + dt f_ext + dt f_gyro
    std::vector<double> rhs(nv);
    for (int j = 0; j < nv; ++j) rhs[j] = (mdiag[j] * v[j] + dt * f_ext[j]) + dt * f_gyro[j];
    if (nrows == 0) {
        for (int j = 0; j < nv; ++j) x_out[j] = rhs[j] / mdiag[j];
        return 0;
    }
    pj_setup(P, contact_bias, restitution, mu, minv, v, alpha, 0);
    SolveResult r = pj_solve(P, rhs.data(), mdiag, lambda_inout, x_out, max_iter, tol_abs, tol_rel, 0.0, 0, nullptr);
    return r.iters;
}

// the solver-level drop-in with the configuration's loop, block preconditioner and stop rules
int32_t or_pj_solve_csr_cfg(const or_config* cfg, int32_t nrows, int32_t nv, int32_t nfl, const int32_t* row_ptr,
                            const int32_t* col, const double* val, const double* contact_bias, const double* mu,
                            const double* restitution, const double* minv, const double* mdiag, const double* v,
                            const double* f_ext, const double* f_gyro, double dt, double* lambda_inout,
                            double* x_out) {
    PJ P;
    P.nrows = nrows;
    P.nv = nv;
    P.nfl = nfl;
    P.ptr = row_ptr;
    P.col = col;
    P.val = val;
    std::vector<double> rhs(nv);
    for (int j = 0; j < nv; ++j) rhs[j] = (mdiag[j] * v[j] + dt * f_ext[j]) + dt * f_gyro[j];
    if (nrows == 0) {
        for (int j = 0; j < nv; ++j) x_out[j] = rhs[j] / mdiag[j];
        return 0;
    }
    pj_setup(P, contact_bias, restitution, mu, minv, v, cfg->pj_alpha, 0, cfg->pj_rdiag_true_delassus);
    SolveResult r = solve_dispatch(P, *cfg, rhs.data(), mdiag, lambda_inout, x_out, cfg->residual_tol, 0, nullptr);
    return r.iters;
}

int32_t or_block_inverse(const double* A, int32_t n, double* X) {
    if (n < 1 || n > 3) return -1;
    spd_inverse(A, n, X);
    return block_is_diagonal(A, n) ? 1 : 0;
}

}  // extern "C"
