// Plain FP64 method: collision, contact setup, projected Jacobi and Moreau drift on the GPU.
//
// Compiled with --fmad=false. Every kernel restates one stage of the reference's step with the
// same operation order as the CPU oracle, so the plain method is bit-identical to it:
//   k_rhs64           PjAssembler::rhs (pj_assembler.cpp:127-170), World forces (world.cpp:113-173)
//   k_drift64         IntegrationBase::explicitPositionUpdate (integration_base.cpp:6-30)
//   k_*_flags/count/write64  coal narrow phase + makeContact (collision_coal.cpp:112-163,405-548)
//   k_contact_setup64 rebuildW_ (dynamics_assembler.cpp:211-332), build_workspace + rdiag_sparse
//                     (projected_jacobi.cpp:316-369,57-69), warm start (contact_tracker.cpp:43-72)
//   k_xinit64         x0 = S^-1 (rhs + W^T p) (projected_jacobi.cpp:361-363)
//   k_sweep_contact64 pj_sweep's RW x + bias, project (projected_jacobi.cpp:100-131)
//   k_sweep_body64    pj_sweep's x += S^-1 W^T dlambda (projected_jacobi.cpp:134-137)
// W is never formed: each contact keeps its three directions and body-frame lever products, W^T
// is applied as a per-body gather over the body's incidence list in solver row order.
#include <algorithm>
#include <cstdio>
#include <functional>

#include "cdx_internal.h"
#include "fp64_math.cuh"

namespace cdx {
using namespace f64;

namespace {

constexpr int NT = 256;
constexpr int MAX_PAIR = 64;  // touching neighbours j > i per sphere
inline int nblk(int64_t n, int nt = NT) { return (int)((n + nt - 1) / nt); }

__device__ __forceinline__ void cell_of(const Grid& g, double x, double y, double z, int* ci) {
    const double p[3] = {x, y, z};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        double f = floor((p[k] - g.lo[k]) / g.cell);
        if (!(f >= 0.0)) f = 0.0;  // also maps NaN to 0
        if (f > (double)(g.dim[k] - 1)) f = (double)(g.dim[k] - 1);
        ci[k] = (int)f;
    }
}

struct Geom {
    double p1[3], p2[3], nraw[3], xa[3];
};

// Sphere against a solid cylinder (coal::Cylinder, collision_coal.cpp:307-310): the exact nearest
// points in closed form. In the cylinder's frame (axial coordinate ax, radial part perp of length
// rho): outside, the nearest point is on the side (|ax| <= h), a cap (rho <= R) or a rim; inside,
// on the nearer of the side and the cap (the side on a tie). The normal points from the cylinder
// to the sphere.
__device__ __forceinline__ bool cylinder_geom(const double* xa, const double* u, double R, double h,
                                              const double* xb, double rb, double margin, Geom& g) {
    double rel[3], perp[3];
    for (int k = 0; k < 3; ++k) rel[k] = xb[k] - xa[k];
    const double ax = dot3(rel, u);
    for (int k = 0; k < 3; ++k) perp[k] = rel[k] - ax * u[k];
    const double rho = norm3(perp);
    const double sg = ax < 0.0 ? -1.0 : 1.0;
    const double aax = fabs(ax);
    double e[3];
    if (rho > 0.0) {
        for (int k = 0; k < 3; ++k) e[k] = perp[k] / rho;
    } else {
        double t2[3];
        tangent_frame(u, e, t2);
    }
    const bool out_side = rho > R, out_cap = aax > h;
    int region;
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
        g.p1[k] = q[k];
        g.p2[k] = xb[k] - rb * n[k];
        g.nraw[k] = n[k];
    }
    return true;
}

// Sphere against a solid box (coal::Box, collision_coal.cpp:288-290): the exact nearest points in
// closed form. In the box's frame (R's columns are its axes, e its half extents) the centre is at
// c = R^T (xb - xa). Outside (some |c_k| > e_k) the nearest point is c clamped to the box (a face,
// edge or corner) and the normal is the direction from it to the centre; inside, it is on the face
// nearest the centre (the lowest axis on a tie), whose outward normal is the contact normal. The
// normal points from the box to the sphere.
__device__ __forceinline__ bool box_geom(const double* xa, const double* R, const double* e, const double* xb,
                                         double rb, double margin, Geom& g) {
    double rel[3], c[3], ql[3], nl[3];
    for (int k = 0; k < 3; ++k) rel[k] = xb[k] - xa[k];
    matTvec(R, rel, c);
    const bool out = fabs(c[0]) > e[0] || fabs(c[1]) > e[1] || fabs(c[2]) > e[2];
    double sd;
    if (!out) {
        int f = 0;
        double best = e[0] - fabs(c[0]);
        for (int k = 1; k < 3; ++k) {
            const double dk = e[k] - fabs(c[k]);
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
        g.p1[k] = xa[k] + q[k];
        g.p2[k] = xb[k] - rb * n[k];
        g.nraw[k] = n[k];
    }
    return true;
}

// coal::Halfspace {x : n.x <= d} (shape 1) against a sphere (shape 2), a solid cylinder, a solid
// box, or the inner wall of a drum.
__device__ __forceinline__ bool static_geom(const Scene& sc, int s, const double* xb, double rb, double margin,
                                            Geom& g) {
    const double u[3] = {sc.sf(SF_DX)[s], sc.sf(SF_DY)[s], sc.sf(SF_DZ)[s]};
    g.xa[0] = sc.sf(SF_PX)[s];
    g.xa[1] = sc.sf(SF_PY)[s];
    g.xa[2] = sc.sf(SF_PZ)[s];
    const int kind = sc.static_kind[s];
    if (kind >= 2) {
        double R[9];
        for (int k = 0; k < 9; ++k) R[k] = sc.sf(SF_R0 + k)[s];
        if (kind == 3) {
            const double e[3] = {sc.sf(SF_EX)[s], sc.sf(SF_EY)[s], sc.sf(SF_EZ)[s]};
            return box_geom(g.xa, R, e, xb, rb, margin, g);
        }
        // the cylinder's axis turns with the static: R times its axis in the static's frame
        const double a[3] = {sc.sf(SF_AX)[s], sc.sf(SF_AY)[s], sc.sf(SF_AZ)[s]};
        double ua[3];
        matvec(R, a, ua);
        return cylinder_geom(g.xa, ua, sc.sf(SF_RAD)[s], sc.sf(SF_HL)[s], xb, rb, margin, g);
    }
    if (sc.static_kind[s] == 0) {
        const double sdist = dot3(u, xb) - sc.sf(SF_D)[s];
        const double dist = sdist - rb;
        if (!(dist <= margin)) return false;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            g.p1[k] = xb[k] - sdist * u[k];
            g.p2[k] = xb[k] - rb * u[k];
            g.nraw[k] = u[k];
        }
        return true;
    }
    const double R = sc.sf(SF_RAD)[s];
    double rel[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) rel[k] = xb[k] - g.xa[k];
    const double ax = dot3(rel, u);
    double perp[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) perp[k] = rel[k] - ax * u[k];
    const double rho = norm3(perp);
    const double dist = (R - rho) - rb;
    if (!(dist <= margin)) return false;
    double e[3] = {0, 0, 0};
    if (rho > 0.0) {
#pragma unroll
        for (int k = 0; k < 3; ++k) e[k] = perp[k] / rho;
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        g.p1[k] = (g.xa[k] + ax * u[k]) + R * e[k];
        g.p2[k] = xb[k] + rb * e[k];
        g.nraw[k] = -e[k];
    }
    return true;
}

// sphere (A, lower index) against sphere (B)
__device__ __forceinline__ bool pair_geom(const double* xA, double ra, const double* xb, double rb, double margin,
                                          Geom& g) {
    double d[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) d[k] = xb[k] - xA[k];
    const double dl = norm3(d);
    const double dist = (dl - ra) - rb;
    if (!(dist <= margin)) return false;
    double nn[3] = {0, 0, 0};
    if (dl > 0.0) {
#pragma unroll
        for (int k = 0; k < 3; ++k) nn[k] = d[k] / dl;
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        g.p1[k] = xA[k] + ra * nn[k];
        g.p2[k] = xb[k] - rb * nn[k];
        g.nraw[k] = nn[k];
        g.xa[k] = xA[k];
    }
    return true;
}

__device__ __forceinline__ bool pair_touch(const double* xA, double ra, const double* xb, double rb, double margin) {
    // cheap exact-safe reject: far pairs cannot pass the exact test below
    const double dx = xb[0] - xA[0], dy = xb[1] - xA[1], dz = xb[2] - xA[2];
    const double lim = (ra + rb) * 1.000001 + fabs(margin) + 1e-300;
    if (dx * dx + dy * dy + dz * dz > lim * lim) return false;
    Geom g;
    return pair_geom(xA, ra, xb, rb, margin, g);
}

// makeContact: sanitise points, normal with fallbacks, Frisvad frame, midpoint.
__device__ __forceinline__ void finish_contact(Geom& g, const double* xb, double* n, double* t1, double* t2,
                                               double* point) {
    if (!finite3(g.p1)) {
        if (finite3(g.p2)) { for (int k = 0; k < 3; ++k) g.p1[k] = g.p2[k]; }
        else { for (int k = 0; k < 3; ++k) g.p1[k] = g.xa[k]; }
    }
    if (!finite3(g.p2)) {
        if (finite3(g.p1)) { for (int k = 0; k < 3; ++k) g.p2[k] = g.p1[k]; }
        else { for (int k = 0; k < 3; ++k) g.p2[k] = xb[k]; }
    }
    const double nlen = norm3(g.nraw);
    if (nlen > 0.0 && isfinite(nlen)) {
        for (int k = 0; k < 3; ++k) n[k] = g.nraw[k] / nlen;
    } else {
        double f[3];
        for (int k = 0; k < 3; ++k) f[k] = g.p2[k] - g.p1[k];
        double fl = norm3(f);
        if (!(fl > 0.0) || !isfinite(fl)) {
            for (int k = 0; k < 3; ++k) f[k] = xb[k] - g.xa[k];
            fl = norm3(f);
        }
        if (fl > 0.0 && isfinite(fl)) { for (int k = 0; k < 3; ++k) n[k] = f[k] / fl; }
        else { n[0] = 0; n[1] = 0; n[2] = 1; }
    }
    tangent_frame(n, t1, t2);
#pragma unroll
    for (int k = 0; k < 3; ++k) point[k] = (g.p1[k] + g.p2[k]) * 0.5;
}

__device__ __forceinline__ void write_contact(const Scene& sc, Contacts& C, int gen, int64_t c, int a_code, int b,
                                              Geom& g, const double* xb, int combine, int friction_enable) {
    double n[3], t1[3], t2[3], p[3];
    finish_contact(g, xb, n, t1, t2, p);
    const int64_t cap = C.cap;
    C.a[c] = a_code;
    C.b[c] = b;
    const uint32_t ida = a_code >= 0 ? (uint32_t)(sc.S + a_code) : (uint32_t)(-a_code - 1);
    const uint32_t idb = (uint32_t)(sc.S + b);
    C.key[gen][c] = ((unsigned long long)ida << 32) | idb;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        C.point[gen][k * cap + c] = p[k];
        C.dir[(0 + k) * cap + c] = n[k];
        C.dir[(3 + k) * cap + c] = t1[k];
        C.dir[(6 + k) * cap + c] = t2[k];
    }
    double muA, rnA, rtA;
    if (a_code >= 0) {
        muA = sc.bf(BF_MU)[a_code];
        rnA = sc.bf(BF_RN)[a_code];
        rtA = sc.bf(BF_RT)[a_code];
    } else {
        const int s = -a_code - 1;
        muA = sc.sf(SF_MU)[s];
        rnA = sc.sf(SF_RN)[s];
        rtA = sc.sf(SF_RT)[s];
    }
    const double mu = combine_mu(combine, muA, sc.bf(BF_MU)[b]);
    C.mu[c] = mu;
    C.eN[c] = smin(smax(0.0, rnA), smax(0.0, sc.bf(BF_RN)[b]));
    C.eT[c] = smin(smax(0.0, rtA), smax(0.0, sc.bf(BF_RT)[b]));
    C.flags[c] = (friction_enable && mu > 0.0) ? CF_FRICTIONAL : 0;
}

// PjAssembler::rhs (pj_assembler.cpp:127-153); implicit_gyro leaves dt f_gyro out (for isotropic
// spheres the implicit gyroscopic block of S is exactly zero)
__global__ void k_rhs64(Scene sc, double dt, double g0, double g1, double g2, double* rhs, int implicit_gyro) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sc.N) return;
    const int N = sc.N;
    const double w[3] = {sc.bf(BF_WX)[i], sc.bf(BF_WY)[i], sc.bf(BF_WZ)[i]};
    const double v[3] = {sc.bf(BF_VX)[i], sc.bf(BF_VY)[i], sc.bf(BF_VZ)[i]};
    const double I = sc.bf(BF_INERTIA)[i], m = sc.bf(BF_MASS)[i];
    const double Ml = sc.bf(BF_ML)[i], Ma = sc.bf(BF_MA)[i];
    const double g[3] = {g0, g1, g2};
    const double Iw[3] = {I * w[0], I * w[1], I * w[2]};
    double c[3];
    cross3(w, Iw, c);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const double fext = m * g[k];
        rhs[(size_t)k * N + i] = (Ml * v[k] + dt * fext) + dt * 0.0;
        rhs[(size_t)(3 + k) * N + i] = implicit_gyro ? (Ma * w[k] + dt * 0.0) : (Ma * w[k] + dt * 0.0) + dt * (-c[k]);
    }
}

// nonfinite (the closing drift of a step): set when a body's new state holds a NaN or infinity
__global__ void k_drift64(Scene sc, double h, int compute_R, int32_t* nonfinite) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < sc.N) {
        double x[3] = {sc.bf(BF_PX)[i], sc.bf(BF_PY)[i], sc.bf(BF_PZ)[i]};
        double q[4] = {sc.bf(BF_QX)[i], sc.bf(BF_QY)[i], sc.bf(BF_QZ)[i], sc.bf(BF_QW)[i]};
        const double v[3] = {sc.bf(BF_VX)[i], sc.bf(BF_VY)[i], sc.bf(BF_VZ)[i]};
        const double w[3] = {sc.bf(BF_WX)[i], sc.bf(BF_WY)[i], sc.bf(BF_WZ)[i]};
        drift(x, q, v, w, h);
        sc.bf(BF_PX)[i] = x[0]; sc.bf(BF_PY)[i] = x[1]; sc.bf(BF_PZ)[i] = x[2];
        sc.bf(BF_QX)[i] = q[0]; sc.bf(BF_QY)[i] = q[1]; sc.bf(BF_QZ)[i] = q[2]; sc.bf(BF_QW)[i] = q[3];
        if (nonfinite) {
            bool ok = true;
            for (int k = 0; k < 3; ++k) ok = ok && isfinite(x[k]) && isfinite(v[k]) && isfinite(w[k]);
            for (int k = 0; k < 4; ++k) ok = ok && isfinite(q[k]);
            if (!ok) *nonfinite = 1;
        }
        if (compute_R) {
            double R[9];
            rotmat(q, R);
#pragma unroll
            for (int k = 0; k < 9; ++k) sc.bf(BF_R0 + k)[i] = R[k];
        }
    } else if (i < sc.N + sc.S) {
        const int s = i - sc.N;
        double x[3] = {sc.sf(SF_PX)[s], sc.sf(SF_PY)[s], sc.sf(SF_PZ)[s]};
        double q[4] = {sc.sf(SF_QX)[s], sc.sf(SF_QY)[s], sc.sf(SF_QZ)[s], sc.sf(SF_QW)[s]};
        const double v[3] = {sc.sf(SF_VX)[s], sc.sf(SF_VY)[s], sc.sf(SF_VZ)[s]};
        const double w[3] = {sc.sf(SF_WX)[s], sc.sf(SF_WY)[s], sc.sf(SF_WZ)[s]};
        drift(x, q, v, w, h);
        sc.sf(SF_PX)[s] = x[0]; sc.sf(SF_PY)[s] = x[1]; sc.sf(SF_PZ)[s] = x[2];
        sc.sf(SF_QX)[s] = q[0]; sc.sf(SF_QY)[s] = q[1]; sc.sf(SF_QZ)[s] = q[2]; sc.sf(SF_QW)[s] = q[3];
        if (compute_R) {
            double R[9];
            rotmat(q, R);
#pragma unroll
            for (int k = 0; k < 9; ++k) sc.sf(SF_R0 + k)[s] = R[k];
        }
    }
}

// Prescribed static motion (Trajectory::update, trajectory.cpp:69-120, run by
// DynamicsAssembler::updateStateDependentTerms after the first drift): per static a record
// (position 3, quaternion 4, velocity 3, angular velocity 3) and flags (1 position, 2 orientation,
// 4 velocity, 8 angular velocity) set by the host for the coming step. The rotation matrix follows
// a new orientation.
__device__ __forceinline__ void apply_static_motion(const double* m, int f, double* x, double* q, double* v,
                                                    double* w) {
    if (f & 1)
        for (int k = 0; k < 3; ++k) x[k] = m[k];
    if (f & 2)
        for (int k = 0; k < 4; ++k) q[k] = m[3 + k];
    if (f & 4)
        for (int k = 0; k < 3; ++k) v[k] = m[7 + k];
    if (f & 8)
        for (int k = 0; k < 3; ++k) w[k] = m[10 + k];
}
__global__ void k_static_motion64(Scene sc, const double* mot, const int32_t* flag) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= sc.S) return;
    const int f = flag[s];
    if (!f) return;
    double x[3] = {sc.sf(SF_PX)[s], sc.sf(SF_PY)[s], sc.sf(SF_PZ)[s]};
    double q[4] = {sc.sf(SF_QX)[s], sc.sf(SF_QY)[s], sc.sf(SF_QZ)[s], sc.sf(SF_QW)[s]};
    double v[3] = {sc.sf(SF_VX)[s], sc.sf(SF_VY)[s], sc.sf(SF_VZ)[s]};
    double w[3] = {sc.sf(SF_WX)[s], sc.sf(SF_WY)[s], sc.sf(SF_WZ)[s]};
    apply_static_motion(mot + 13 * (size_t)s, f, x, q, v, w);
    for (int k = 0; k < 3; ++k) {
        sc.sf(SF_PX + k)[s] = x[k];
        sc.sf(SF_VX + k)[s] = v[k];
        sc.sf(SF_WX + k)[s] = w[k];
    }
    for (int k = 0; k < 4; ++k) sc.sf(SF_QX + k)[s] = q[k];
    double R[9];
    rotmat(q, R);
    for (int k = 0; k < 9; ++k) sc.sf(SF_R0 + k)[s] = R[k];
}

// flags laid out per scene as [static slot l][sphere within scene], so an exclusive scan yields
// positions in (static id, sphere id) order
__global__ void k_static_flags64(Scene sc, double margin, int32_t* flags) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sc.N) return;
    const int s = sc.body_scene[i];
    const int b0 = sc.scene_body_start[s], ns_b = sc.scene_body_start[s + 1] - b0;
    const int st0 = sc.scene_static_start[s], nst = sc.scene_static_start[s + 1] - st0;
    const double xb[3] = {sc.bf(BF_PX)[i], sc.bf(BF_PY)[i], sc.bf(BF_PZ)[i]};
    const double rb = sc.bf(BF_RAD)[i];
    const int L = sc.max_statics;
    for (int l = 0; l < L; ++l) {
        int f = 0;
        if (l < nst) {
            Geom g;
            f = static_geom(sc, st0 + l, xb, rb, margin, g) ? 1 : 0;
        }
        flags[(size_t)b0 * L + (size_t)l * ns_b + (i - b0)] = f;
    }
}

__global__ void k_static_write64(Scene sc, double margin, const int32_t* flags, const int32_t* pos, Contacts C,
                                 int gen, int combine, int friction_enable) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sc.N) return;
    const int s = sc.body_scene[i];
    const int b0 = sc.scene_body_start[s], ns_b = sc.scene_body_start[s + 1] - b0;
    const int st0 = sc.scene_static_start[s], nst = sc.scene_static_start[s + 1] - st0;
    const double xb[3] = {sc.bf(BF_PX)[i], sc.bf(BF_PY)[i], sc.bf(BF_PZ)[i]};
    const double rb = sc.bf(BF_RAD)[i];
    const int L = sc.max_statics;
    for (int l = 0; l < nst && l < L; ++l) {
        const size_t slot = (size_t)b0 * L + (size_t)l * ns_b + (i - b0);
        if (!flags[slot]) continue;
        Geom g;
        static_geom(sc, st0 + l, xb, rb, margin, g);
        write_contact(sc, C, gen, pos[slot], -(st0 + l) - 1, i, g, xb, combine, friction_enable);
    }
}

__global__ void k_pos32(Scene sc, Grid gr, float4* p32) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sc.N) return;
    p32[i] = make_float4((float)(sc.bf(BF_PX)[i] - gr.lo[0]), (float)(sc.bf(BF_PY)[i] - gr.lo[1]),
                         (float)(sc.bf(BF_PZ)[i] - gr.lo[2]), (float)sc.bf(BF_RAD)[i]);
}

// Conservative FP32 pre-test of a sphere pair: false only when the FP64 test (pair_touch) is
// certain to reject it too. Every FP32 quantity here is within a relative 2^-22 of its FP64 value
// (positions and radii rounded once, differences and sums a few more times), so the distance is
// within 2^-21 (|x_i| + |x_j|) + 2^-21 d of the exact one. The limit therefore widens the FP64
// limit (r_i + r_j) 1.000001 + |margin| by a relative 9e-6 and by 1e-6 (|x_i| + |x_j|) (> 2^-21 of
// it). NaN positions compare false and go on to the FP64 test.
__device__ __forceinline__ bool pair_near32(float4 pi, float ei, float4 pj, float mf) {
    const float dx = pj.x - pi.x, dy = pj.y - pi.y, dz = pj.z - pi.z;
    const float ej = fmaxf(fabsf(pj.x), fmaxf(fabsf(pj.y), fabsf(pj.z)));
    const float lim = (pi.w + pj.w) * 1.00001f + mf + 1e-6f * (ei + ej) + 1e-30f;
    return !(dx * dx + dy * dy + dz * dz > lim * lim);
}

template <bool WRITE>
__global__ void k_pairs64(Scene sc, Grid gr, const uint32_t* cell_body, const int32_t* cell_start,
                          const int32_t* cell_end, const float4* p32, int32_t* plist, double margin,
                          int32_t* counts, const int32_t* offsets, int32_t base, Contacts C, int gen, int combine,
                          int friction_enable, DevScalars* ds) {
    // threads take the spheres in cell order, so a warp walks neighbouring cells; each sphere's
    // count and contacts are its own (same values, written at its own offset)
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= sc.N) return;
    const int i = (int)cell_body[t];
    const double xi[3] = {sc.bf(BF_PX)[i], sc.bf(BF_PY)[i], sc.bf(BF_PZ)[i]};
    const float4 pi = p32[i];
    const float ei = fmaxf(fabsf(pi.x), fmaxf(fabsf(pi.y), fabsf(pi.z)));
    const float mf = (float)fabs(margin) * 1.00001f;
    const double ri = sc.bf(BF_RAD)[i];
    const int si = sc.body_scene[i];
    int ci[3];
    cell_of(gr, xi[0], xi[1], xi[2], ci);
    int list[MAX_PAIR];
    int cnt = 0;
    // the write pass takes the partners the count pass kept when they all fitted (the same walk
    // and the same tests found them); the count comes from the scanned offsets
    bool walk = true;
    if (WRITE) {
        const int kept = offsets[i + 1] - offsets[i];
        if (kept <= PLIST64) {
            for (int k = 0; k < kept; ++k) list[k] = plist[(size_t)i * PLIST64 + k];
            cnt = kept;
            walk = false;
        }
    }
    for (int dz = -1; dz <= 1 && walk; ++dz) {
        const int z = ci[2] + dz;
        if (z < 0 || z >= gr.dim[2]) continue;
        for (int dy = -1; dy <= 1; ++dy) {
            const int y = ci[1] + dy;
            if (y < 0 || y >= gr.dim[1]) continue;
            for (int dx = -1; dx <= 1; ++dx) {
                const int x = ci[0] + dx;
                if (x < 0 || x >= gr.dim[0]) continue;
                const int64_t cell = ((int64_t)z * gr.dim[1] + y) * gr.dim[0] + x;
                const int e = cell_end[cell];
                for (int p = cell_start[cell]; p < e; ++p) {
                    const int j = (int)cell_body[p];
                    if (j <= i || sc.body_scene[j] != si) continue;
                    if (!pair_near32(pi, ei, p32[j], mf)) continue;
                    const double xj[3] = {sc.bf(BF_PX)[j], sc.bf(BF_PY)[j], sc.bf(BF_PZ)[j]};
                    if (!pair_touch(xi, ri, xj, sc.bf(BF_RAD)[j], margin)) continue;
                    if (WRITE) {
                        if (cnt < MAX_PAIR) list[cnt] = j;
                    } else if (cnt < PLIST64) {
                        plist[(size_t)i * PLIST64 + cnt] = j;
                    }
                    ++cnt;
                }
            }
        }
    }
    if (!WRITE) {
        counts[i] = cnt;
        if (cnt > MAX_PAIR) atomicExch(&ds->overflow, 1);
        return;
    }
    if (cnt > MAX_PAIR) cnt = MAX_PAIR;
    // canonical order: increasing partner index
    for (int a = 1; a < cnt; ++a) {
        const int v = list[a];
        int b = a - 1;
        while (b >= 0 && list[b] > v) {
            list[b + 1] = list[b];
            --b;
        }
        list[b + 1] = v;
    }
    const int64_t o = (int64_t)base + offsets[i];
    for (int k = 0; k < cnt; ++k) {
        const int j = list[k];
        const double xj[3] = {sc.bf(BF_PX)[j], sc.bf(BF_PY)[j], sc.bf(BF_PZ)[j]};
        Geom g;
        pair_geom(xi, ri, xj, sc.bf(BF_RAD)[j], margin, g);
        write_contact(sc, C, gen, o + k, i, j, g, xj, combine, friction_enable);
    }
}

__device__ __forceinline__ void body_frame(const Scene& sc, int a_code, double* R, double* x) {
    if (a_code >= 0) {
#pragma unroll
        for (int k = 0; k < 9; ++k) R[k] = sc.bf(BF_R0 + k)[a_code];
        x[0] = sc.bf(BF_PX)[a_code]; x[1] = sc.bf(BF_PY)[a_code]; x[2] = sc.bf(BF_PZ)[a_code];
    } else {
        const int s = -a_code - 1;
#pragma unroll
        for (int k = 0; k < 9; ++k) R[k] = sc.sf(SF_R0 + k)[s];
        x[0] = sc.sf(SF_PX)[s]; x[1] = sc.sf(SF_PY)[s]; x[2] = sc.sf(SF_PZ)[s];
    }
}

__global__ void k_contact_setup64(Scene sc, Contacts C, int gen, int nc, int prev_count, double alpha,
                                  double match2, int warmstart) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    const int64_t cap = C.cap;
    const int a = C.a[c], b = C.b[c];
    const bool fr = (C.flags[c] & CF_FRICTIONAL) != 0;
    double d[9], pt[3];
#pragma unroll
    for (int k = 0; k < 9; ++k) d[k] = C.dir[k * cap + c];
#pragma unroll
    for (int k = 0; k < 3; ++k) pt[k] = C.point[gen][k * cap + c];
    // body-frame lever products (transform::point / transform::direction + buildContactRowByDof)
    double cA[9], cB[9];
    for (int side = 0; side < 2; ++side) {
        double R[9], x[3];
        body_frame(sc, side == 0 ? a : b, R, x);
        double rel[3], rb[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) rel[k] = pt[k] - x[k];
        matTvec(R, rel, rb);
        double* cc = side == 0 ? cA : cB;
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            double db[3];
            matTvec(R, &d[3 * r], db);
            cross3(rb, db, &cc[3 * r]);
        }
    }
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        C.cA[k * cap + c] = cA[k];
        C.cB[k * cap + c] = cB[k];
    }
    // static side velocity: contact_v_vec[row] += row . [v_world, omega_body]  (sign -1 on side A)
    double cbv[3] = {0.0, 0.0, 0.0};
    if (a < 0) {
        const int s = -a - 1;
        const double vs[3] = {sc.sf(SF_VX)[s], sc.sf(SF_VY)[s], sc.sf(SF_VZ)[s]};
        const double ws[3] = {sc.sf(SF_WX)[s], sc.sf(SF_WY)[s], sc.sf(SF_WZ)[s]};
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            double acc = (-d[3 * r]) * vs[0];
            acc = acc + (-d[3 * r + 1]) * vs[1];
            acc = acc + (-d[3 * r + 2]) * vs[2];
            acc = acc + (-cA[3 * r]) * ws[0];
            acc = acc + (-cA[3 * r + 1]) * ws[1];
            acc = acc + (-cA[3 * r + 2]) * ws[2];
            cbv[r] = 0.0 + acc;
        }
    }
#pragma unroll
    for (int r = 0; r < 3; ++r) C.cb[r * cap + c] = cbv[r];
    // warm start: same pair in the previous step within collision.match_max_dist
    double lam0[3] = {0.0, 0.0, 0.0};
    if (warmstart && prev_count > 0) {
        const unsigned long long key = C.key[gen][c];
        const unsigned long long* pk = C.key[gen ^ 1];
        int lo = 0, hi = prev_count;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (pk[mid] < key) lo = mid + 1;
            else hi = mid;
        }
        if (lo < prev_count && pk[lo] == key) {
            double dd[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) dd[k] = pt[k] - C.point[gen ^ 1][k * cap + lo];
            if (dot3(dd, dd) <= match2) {
#pragma unroll
                for (int k = 0; k < 3; ++k) lam0[k] = C.lam[gen ^ 1][k * cap + lo];
            }
        }
    }
    if (!fr) { lam0[1] = 0.0; lam0[2] = 0.0; }
#pragma unroll
    for (int k = 0; k < 3; ++k) C.lam[gen][k * cap + c] = lam0[k];
    // rows: contact velocity, Delassus diagonal, R = alpha / D, RW and R-scaled bias
    double vA[6] = {0, 0, 0, 0, 0, 0}, vB[6], mA[6] = {0, 0, 0, 0, 0, 0}, mB[6];
    if (a >= 0) {
        vA[0] = sc.bf(BF_VX)[a]; vA[1] = sc.bf(BF_VY)[a]; vA[2] = sc.bf(BF_VZ)[a];
        vA[3] = sc.bf(BF_WX)[a]; vA[4] = sc.bf(BF_WY)[a]; vA[5] = sc.bf(BF_WZ)[a];
        const double ml = sc.bf(BF_MINVL)[a], ma = sc.bf(BF_MINVA)[a];
        mA[0] = ml; mA[1] = ml; mA[2] = ml; mA[3] = ma; mA[4] = ma; mA[5] = ma;
    }
    vB[0] = sc.bf(BF_VX)[b]; vB[1] = sc.bf(BF_VY)[b]; vB[2] = sc.bf(BF_VZ)[b];
    vB[3] = sc.bf(BF_WX)[b]; vB[4] = sc.bf(BF_WY)[b]; vB[5] = sc.bf(BF_WZ)[b];
    {
        const double ml = sc.bf(BF_MINVL)[b], ma = sc.bf(BF_MINVA)[b];
        mB[0] = ml; mB[1] = ml; mB[2] = ml; mB[3] = ma; mB[4] = ma; mB[5] = ma;
    }
    const int nr = fr ? 3 : 1;
    const bool block = C.rb != nullptr;
    double D0 = 0.0;
    for (int r = 0; r < 3; ++r) {
        if (r >= nr) {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                C.rd[(3 * r + k) * cap + c] = 0.0;
                C.rcA[(3 * r + k) * cap + c] = 0.0;
                C.rcB[(3 * r + k) * cap + c] = 0.0;
            }
            C.biasR[r * cap + c] = 0.0;
            continue;
        }
        int ne = 0;
        double val[12], vel[12], mi[12];
        if (a >= 0) {
#pragma unroll
            for (int k = 0; k < 3; ++k) { val[ne] = -d[3 * r + k]; vel[ne] = vA[k]; mi[ne] = mA[k]; ++ne; }
#pragma unroll
            for (int k = 0; k < 3; ++k) { val[ne] = -cA[3 * r + k]; vel[ne] = vA[3 + k]; mi[ne] = mA[3 + k]; ++ne; }
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) { val[ne] = d[3 * r + k]; vel[ne] = vB[k]; mi[ne] = mB[k]; ++ne; }
#pragma unroll
        for (int k = 0; k < 3; ++k) { val[ne] = cB[3 * r + k]; vel[ne] = vB[3 + k]; mi[ne] = mB[3 + k]; ++ne; }
        double vp = 0.0, D = 0.0;
        for (int k = 0; k < ne; ++k) vp = vp + val[k] * vel[k];
        vp = vp + cbv[r];
        const double e = r == 0 ? C.eN[c] : C.eT[c];
        const double bias = cbv[r] + e * vp;
        for (int k = 0; k < ne; ++k) D = D + (val[k] * val[k]) * mi[k];
        if (r == 0) D0 = D;
        // pj.rdiag_true_delassus keeps W and the bias unscaled (projected_jacobi.cpp:341-343)
        const double Rr = block ? 1.0 : ((D > 0.0) ? (alpha / D) : 0.0);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            C.rd[(3 * r + k) * cap + c] = Rr * d[3 * r + k];
            C.rcA[(3 * r + k) * cap + c] = Rr * cA[3 * r + k];
            C.rcB[(3 * r + k) * cap + c] = Rr * cB[3 * r + k];
        }
        C.biasR[r * cap + c] = Rr * bias;
    }
    if (block) {
        // the contact's Delassus block / alpha (buildBlockPreconditioner, projected_jacobi.cpp:81-98):
        // D_rs = sum over the row entries (A linear, A angular, B linear, B angular) of
        // (W_rk Minv_k) W_sk; inverted by k_block_invert64 once every block of the step is known
        const double inv_alpha = (alpha > 0.0) ? (1.0 / alpha) : 0.0;
        if (!fr) {
            C.rb[c] = D0 * inv_alpha;
        } else {
            double w[3][12], mm[12];
            int ne = 0;
            for (int r = 0; r < 3; ++r) {
                ne = 0;
                if (a >= 0) {
                    for (int k = 0; k < 3; ++k) { w[r][ne] = -d[3 * r + k]; mm[ne] = mA[k]; ++ne; }
                    for (int k = 0; k < 3; ++k) { w[r][ne] = -cA[3 * r + k]; mm[ne] = mA[3 + k]; ++ne; }
                }
                for (int k = 0; k < 3; ++k) { w[r][ne] = d[3 * r + k]; mm[ne] = mB[k]; ++ne; }
                for (int k = 0; k < 3; ++k) { w[r][ne] = cB[3 * r + k]; mm[ne] = mB[3 + k]; ++ne; }
            }
            double Db[9];
            for (int r = 0; r < 3; ++r)
                for (int s = 0; s < 3; ++s) {
                    double acc = 0.0;
                    for (int q = 0; q < ne; ++q) acc = acc + (w[r][q] * mm[q]) * w[s][q];
                    Db[3 * r + s] = acc * inv_alpha;
                }
            for (int k = 0; k < 9; ++k) C.rb[(size_t)k * cap + c] = Db[k];
            // MatrixBase::isDiagonal (Eigen 3, precision 1e-12); one non-diagonal block switches
            // every block of the step to the full inverse (BlockDiagonal::calculateInverse)
            if (!block_is_diagonal3(Db)) *C.rb_full = 1;
        }
    }
}

// R_block = (D / alpha)^-1 per contact: per diagonal entry when every block of the step is
// diagonal, else the SPD inverse of every block (1 x 1 blocks included)
__global__ void k_block_invert64(Contacts C, int nc) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    const int64_t cap = C.cap;
    const bool full = *(const volatile int32_t*)C.rb_full != 0;
    if (!(C.flags[c] & CF_FRICTIONAL)) {
        const double d = C.rb[c];
        double x;
        if (full) spd_inverse_dev(&d, 1, &x);
        else x = 1.0 / d;
        C.rb[c] = x;
        return;
    }
    double D[9], X[9];
    for (int k = 0; k < 9; ++k) D[k] = C.rb[(size_t)k * cap + c];
    if (full) {
        spd_inverse_dev(D, 3, X);
    } else {
        for (int k = 0; k < 9; ++k) X[k] = 0.0;
        for (int j = 0; j < 3; ++j) X[4 * j] = 1.0 / D[4 * j];
    }
    for (int k = 0; k < 9; ++k) C.rb[(size_t)k * cap + c] = X[k];
}

// BlockDiagonal::applyTo (misc/block_diagonal.hpp:107-126) on one contact's rows g
__device__ __forceinline__ void block_apply64(const Contacts& C, int c, bool fr, double* g) {
    const int64_t cap = C.cap;
    const bool full = *C.rb_full != 0;
    if (!fr) {
        g[0] = full ? C.rb[c] * g[0] : g[0] * C.rb[c];
        return;
    }
    if (!full) {
        for (int j = 0; j < 3; ++j) g[j] = g[j] * C.rb[(size_t)(4 * j) * cap + c];
        return;
    }
    double B[9], s[3];
    for (int k = 0; k < 9; ++k) B[k] = C.rb[(size_t)k * cap + c];
    for (int j = 0; j < 3; ++j) s[j] = B[3 * j] * g[0] + B[3 * j + 1] * g[1] + B[3 * j + 2] * g[2];
    for (int j = 0; j < 3; ++j) g[j] = s[j];
}

__global__ void k_frictionless_flags(Contacts C, int nc, int32_t* isfl) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    isfl[c] = (C.flags[c] & CF_FRICTIONAL) ? 0 : 1;
}

// solver row order: frictionless contacts first, then frictional ones, each in canonical order
// (rebuildW_'s two passes, dynamics_assembler.cpp:236-324); incidence list input in that order
// by_contact: the incidence lists keep contact order instead of solver row order (the condensed
// solver's blocks are in contact order)
__global__ void k_rank_incidence(int N, Contacts C, int nc, const int32_t* fl_scan, const int32_t* isfl,
                                 Incidence inc, int by_contact) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    const int nfl = fl_scan[nc - 1] + isfl[nc - 1];
    const int rank = isfl[c] ? fl_scan[c] : nfl + (c - fl_scan[c]);
    C.rank[c] = rank;
    const int pos = by_contact ? c : rank;
    const int a = C.a[c];
    inc.key_in[2 * (size_t)pos] = a >= 0 ? (uint32_t)a : (uint32_t)N;
    inc.val_in[2 * (size_t)pos] = (uint32_t)(2 * c);
    inc.key_in[2 * (size_t)pos + 1] = (uint32_t)C.b[c];
    inc.val_in[2 * (size_t)pos + 1] = (uint32_t)(2 * c + 1);
}

// body gather of W^T y over the incidence list (rows in solver order); acc is accumulated in place
template <int LAMGEN>
__device__ __forceinline__ void gather_wt(const Contacts& C, const double* y, const Incidence& inc, int i,
                                          double* acc) {
    const int64_t cap = C.cap;
    const int e = inc.end[i];
    for (int p = inc.start[i]; p < e; ++p) {
        const uint32_t code = inc.val_out[p];
        const int c = (int)(code >> 1);
        const bool sideB = code & 1u;
        const double s = sideB ? 1.0 : -1.0;
        const double* cx = sideB ? C.cB : C.cA;
        const int nr = (C.flags[c] & CF_FRICTIONAL) ? 3 : 1;
        for (int r = 0; r < nr; ++r) {
            const double yr = y[r * cap + c];
#pragma unroll
            for (int k = 0; k < 3; ++k) acc[k] = acc[k] + (s * C.dir[(3 * r + k) * cap + c]) * yr;
#pragma unroll
            for (int k = 0; k < 3; ++k) acc[3 + k] = acc[3 + k] + (s * cx[(3 * r + k) * cap + c]) * yr;
        }
    }
}

__global__ void k_xinit64(Scene sc, Contacts C, int gen, Incidence inc, const double* rhs, double* x) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sc.N) return;
    const int N = sc.N;
    double acc[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) acc[k] = rhs[(size_t)k * N + i];
    gather_wt<0>(C, C.lam[gen], inc, i, acc);
    const double Ml = sc.bf(BF_ML)[i], Ma = sc.bf(BF_MA)[i];
#pragma unroll
    for (int k = 0; k < 6; ++k) x[(size_t)k * N + i] = acc[k] / (k < 3 ? Ml : Ma);
}

__device__ __forceinline__ void atomic_max_nonneg(unsigned long long* addr, double v) {
    atomicMax(addr, (unsigned long long)__double_as_longlong(v));
}

__device__ __forceinline__ double block_max(double v) {
    __shared__ double sh[32];
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    v = (threadIdx.x < (blockDim.x >> 5)) ? sh[lane] : 0.0;
    if (wid == 0)
        for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

__device__ __forceinline__ double block_sum(double v) {
    __shared__ double sh[32];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    v = (threadIdx.x < (blockDim.x >> 5)) ? sh[lane] : 0.0;
    if (wid == 0)
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__global__ void k_sweep_contact64(Scene sc, Contacts C, int gen, int nc, const double* x, DevScalars* ds,
                                  int dry) {
    if (!dry && *(volatile int32_t*)&ds->done) return;
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    double maxd = 0.0, maxl = 0.0;
    if (c < nc) {
        const int64_t cap = C.cap;
        const int N = sc.N;
        const int a = C.a[c], b = C.b[c];
        const bool fr = (C.flags[c] & CF_FRICTIONAL) != 0;
        const int nr = fr ? 3 : 1;
        double xA[6], xB[6];
        if (a >= 0) {
#pragma unroll
            for (int k = 0; k < 6; ++k) xA[k] = x[(size_t)k * N + a];
        }
#pragma unroll
        for (int k = 0; k < 6; ++k) xB[k] = x[(size_t)k * N + b];
        double* lamp = C.lam[gen];
        double lold[3], lnew[3], gr[3];
        for (int r = 0; r < nr; ++r) {
            double t = 0.0;
            if (a >= 0) {
#pragma unroll
                for (int k = 0; k < 3; ++k) t = t + (-C.rd[(3 * r + k) * cap + c]) * xA[k];
#pragma unroll
                for (int k = 0; k < 3; ++k) t = t + (-C.rcA[(3 * r + k) * cap + c]) * xA[3 + k];
            }
#pragma unroll
            for (int k = 0; k < 3; ++k) t = t + C.rd[(3 * r + k) * cap + c] * xB[k];
#pragma unroll
            for (int k = 0; k < 3; ++k) t = t + C.rcB[(3 * r + k) * cap + c] * xB[3 + k];
            gr[r] = t + C.biasR[r * cap + c];
            lold[r] = lamp[r * cap + c];
        }
        if (C.rb) block_apply64(C, c, fr, gr);
        for (int r = 0; r < nr; ++r) lnew[r] = lold[r] - gr[r];
        // project (projected_jacobi.cpp:100-119)
        lnew[0] = smax(lnew[0], 0.0);
        if (fr) {
            const double t1 = lnew[1], t2 = lnew[2];
            const double tn2 = t1 * t1 + t2 * t2;
            if (tn2 > 0) {
                const double s = smin(1.0, (C.mu[c] * lnew[0]) / sqrt(tn2));
                lnew[1] = s * t1;
                lnew[2] = s * t2;
            }
        }
        double s2 = 0.0;
        for (int r = 0; r < nr; ++r) {
            const double dl = lnew[r] - lold[r];
            s2 = s2 + dl * dl;
            maxl = smax(maxl, fabs(lold[r]));
            if (!dry) {
                lamp[r * cap + c] = lnew[r];
                C.dlam[r * cap + c] = dl;
                if (C.term) {
                    // the body sweep's products (s d) y, with s = +-1 exact: (-d) y for side A
                    double2* tb = reinterpret_cast<double2*>(C.term + (size_t)(2 * c + 1) * 18 + 6 * r);
                    tb[0] = make_double2(C.dir[(3 * r) * cap + c] * dl, C.dir[(3 * r + 1) * cap + c] * dl);
                    tb[1] = make_double2(C.dir[(3 * r + 2) * cap + c] * dl, C.cB[(3 * r) * cap + c] * dl);
                    tb[2] = make_double2(C.cB[(3 * r + 1) * cap + c] * dl, C.cB[(3 * r + 2) * cap + c] * dl);
                    if (a >= 0) {
                        double2* ta = reinterpret_cast<double2*>(C.term + (size_t)(2 * c) * 18 + 6 * r);
                        ta[0] = make_double2((-C.dir[(3 * r) * cap + c]) * dl, (-C.dir[(3 * r + 1) * cap + c]) * dl);
                        ta[1] = make_double2((-C.dir[(3 * r + 2) * cap + c]) * dl, (-C.cA[(3 * r) * cap + c]) * dl);
                        ta[2] = make_double2((-C.cA[(3 * r + 1) * cap + c]) * dl, (-C.cA[(3 * r + 2) * cap + c]) * dl);
                    }
                }
            }
        }
        maxd = s2;  // squared: the root of the block maximum equals the maximum of the roots
    }
    maxd = block_max(maxd);
    maxl = block_max(maxl);
    if (threadIdx.x == 0) {
        atomic_max_nonneg(&ds->maxd, sqrt(maxd));
        atomic_max_nonneg(&ds->maxl, maxl);
    }
}

__global__ void k_sweep_body64(Scene sc, Contacts C, Incidence inc, double* x, double tol_abs, double tol_rel,
                               int want_velres, DevScalars* ds) {
    if (*(volatile int32_t*)&ds->done) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double part = 0.0;
    if (i < sc.N) {
        const int N = sc.N;
        double acc[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        if (C.term) {
            // the same sums in the same order (incidences in row order, rows in order) from the
            // products the contact sweep stored
            const int e = inc.end[i];
            for (int p = inc.start[i]; p < e; ++p) {
                const uint32_t code = inc.val_out[p];
                const int nr = (C.flags[code >> 1] & CF_FRICTIONAL) ? 3 : 1;
                const double2* t = reinterpret_cast<const double2*>(C.term + (size_t)code * 18);
                for (int r = 0; r < nr; ++r) {
                    const double2 u0 = t[3 * r], u1 = t[3 * r + 1], u2 = t[3 * r + 2];
                    acc[0] = acc[0] + u0.x;
                    acc[1] = acc[1] + u0.y;
                    acc[2] = acc[2] + u1.x;
                    acc[3] = acc[3] + u1.y;
                    acc[4] = acc[4] + u2.x;
                    acc[5] = acc[5] + u2.y;
                }
            }
        } else {
            gather_wt<1>(C, C.dlam, inc, i, acc);
        }
        const double Ml = sc.bf(BF_ML)[i], Ma = sc.bf(BF_MA)[i];
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            const double xo = x[(size_t)k * N + i];
            const double xn = xo + acc[k] / (k < 3 ? Ml : Ma);
            x[(size_t)k * N + i] = xn;
            if (want_velres) {
                const double q = smax(fabs(xn), fabs(xo)) * tol_rel + tol_abs;
                const double dd = (xn - xo) / q;
                part = part + dd * dd;
            }
        }
    }
    if (want_velres) {
        part = block_sum(part);
        if (threadIdx.x == 0) atomicAdd(&ds->velres, part);
    }
}

__global__ void k_check(DevScalars* ds, int iter, double residual_tol, int nv, int check_vel) {
    const double maxd = __longlong_as_double((long long)ds->maxd);
    const double maxl = __longlong_as_double((long long)ds->maxl);
    const double r = maxd / smax(maxl, 1e-30);
    if (!ds->done) {
        ds->res_last = r;
        ds->iters = iter + 1;
        bool stop = false;
        if (check_vel && iter % 10 == 0) {
            const double vr = 1.0 / sqrt((double)nv) * sqrt(ds->velres);
            if (vr <= 1) stop = true;
        }
        if (residual_tol > 0 && r <= residual_tol) stop = true;
        if (stop) ds->done = 1;
    }
    ds->maxd = 0ull;
    ds->maxl = 0ull;
    ds->velres = 0.0;
}

// ---- accelerated loops (projected_jacobi.cpp:179-222 Chebyshev, :379-449 Nesterov)
// Reductions run in a fixed order that the oracle uses too: sums over chunks of RED_CHUNK
// consecutive entries of the stacked velocity vector (entry 6 i + k = component k of body i, the
// reference's layout), each chunk left to right, then the chunk sums left to right.
constexpr int RED_CHUNK = 256;
__device__ __forceinline__ double stacked(const double* v, int N, int j) { return v[(size_t)(j % 6) * N + j / 6]; }
__device__ __forceinline__ double elem(const double* v, int N, int j, int plain) {
    return plain ? v[j] : stacked(v, N, j);
}

// plain: the vectors are already in stacked order (the solver-level drop-in, N = their length)
__global__ void k_chunk_partials(int N, int op, const double* a, const double* b, const double* c, double tol_rel,
                                 double tol_abs, double* part, AccelState* st, const DevScalars* ds, int plain) {
    if (ds && *(volatile const int32_t*)&ds->done) return;
    const int nv = plain ? N : 6 * N;
    const int nch = (nv + RED_CHUNK - 1) / RED_CHUNK;
    const int ch = blockIdx.x * blockDim.x + threadIdx.x;
    if (ch >= nch) return;
    const int j0 = ch * RED_CHUNK, j1 = min(nv, j0 + RED_CHUNK);
    double s = 0.0;
    bool finite = true;
    for (int j = j0; j < j1; ++j) {
        double t;
        if (op == ACC_VELRES) {
            const double x = elem(a, N, j, plain), xp = elem(b, N, j, plain);
            const double q = smax(fabs(x), fabs(xp)) * tol_rel + tol_abs;
            const double d = (x - xp) / q;
            t = d * d;
            finite = finite && isfinite(x);
        } else if (op == ACC_NORM2) {
            const double x = elem(a, N, j, plain);
            t = x * x;
        } else if (op == ACC_DOT) {
            const double y = elem(a, N, j, plain), x1 = elem(b, N, j, plain), x0 = elem(c, N, j, plain);
            t = (y - x1) * (x1 - x0);
        } else {
            t = 1.0;
        }
        s = s + t;
    }
    part[ch] = s;
    if (!finite) st->nonfinite = 1;
}

__global__ void k_chunk_total(const double* part, int nch, double* out, const DevScalars* ds) {
    if (ds && *(volatile const int32_t*)&ds->done) return;
    double tot = 0.0;
    for (int k = 0; k < nch; ++k) tot = tot + part[k];
    *out = tot;
}

// dst = src for the velocity (6 x N, field-major) and impulse (3 x cap) vectors, unless done
__global__ void k_accel_copy(double* xd, const double* xs, int64_t nx, double* ld, const double* ls, int64_t nl,
                             const DevScalars* ds) {
    if (ds && *(volatile const int32_t*)&ds->done) return;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nx + nl; i += (int64_t)gridDim.x * blockDim.x) {
        if (i < nx)
            xd[i] = xs[i];
        else
            ld[i - nx] = ls[i - nx];
    }
}

// Nesterov: err and the restart tests (nesterov_loop), then the momentum coefficient
// (gpu.residual_tol: the loop also ends once the sweep's complementarity residual is at most tol,
// tested right after the reference's own exit)
__global__ void k_nesterov_decide(AccelState* st, DevScalars* ds, int nv, double beta_threshold, int restart_limit,
                                  double residual_tol) {
    if (ds->done) return;
    const double err = 1.0 / sqrt((double)nv) * sqrt(st->sum_err);
    if (err <= 1.0 || (residual_tol > 0 && ds->res_last <= residual_tol)) {
        ds->done = 1;
        return;
    }
    const double thk = st->thk;
    const double thk1 = 0.5 * (1.0 + sqrt(4.0 * thk * thk + 1.0));
    const double betak1 = (thk - 1.0) / thk1;
    bool restart = false;
    if (!isfinite(err)) {
        restart = true;
    } else if (st->err_prev < INFINITY && err > 1.05 * st->err_prev) {
        restart = true;
    } else if (betak1 > beta_threshold) {
        restart = true;
    } else if (!isfinite(betak1) || betak1 < 0.0 || betak1 > 1.0) {
        restart = true;
    } else if (st->sum_dot > 0.0) {
        restart = true;
    }
    if (restart) {
        st->mode = 0;
        st->thk = 1.0;
        if (++st->restarts >= restart_limit) st->disabled = 1;
    } else if (st->disabled) {
        st->mode = 0;
        st->thk = 1.0;
    } else {
        st->mode = 1;
        st->coef = betak1;
        st->thk = thk1;
    }
    st->err_prev = err;
}

// xy = mode ? xk1 + beta (xk1 - xk) : xk1;  xk = xk1   (and the same for the impulses)
__global__ void k_nesterov_update(double* xy, double* xk, const double* xk1, int64_t nx, double* py, double* pk,
                                  const double* pk1, int64_t nl, const AccelState* st, const DevScalars* ds) {
    if (*(volatile const int32_t*)&ds->done) return;
    const int mode = st->mode;
    const double b = st->coef;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nx + nl; i += (int64_t)gridDim.x * blockDim.x) {
        double *y, *k0;
        const double* k1;
        int64_t q;
        if (i < nx) {
            y = xy; k0 = xk; k1 = xk1; q = i;
        } else {
            y = py; k0 = pk; k1 = pk1; q = i - nx;
        }
        y[q] = mode ? k1[q] + b * (k1[q] - k0[q]) : k1[q];
        k0[q] = k1[q];
    }
}

// Chebyshev: err, then the next omega or the fallback to a plain step (chebyshev_loop)
__global__ void k_chebyshev_decide(AccelState* st, DevScalars* ds, int nv, int iter, double residual_tol) {
    if (ds->done) return;
    const double err = 1.0 / sqrt((double)nv) * sqrt(st->sum_err);
    if (err <= 1.0 || (residual_tol > 0 && ds->res_last <= residual_tol)) {
        ds->done = 1;
        return;
    }
    double omega_next = (iter == 0) ? (1.0 / (1.0 - st->rho2 * 0.5)) : (1.0 / (1.0 - (st->rho2 * 0.25) * st->omega));
    if (!isfinite(omega_next) || omega_next <= 0.0 || st->nonfinite) {
        st->mode = 0;
        omega_next = 1.0;
    } else {
        st->mode = 1;
    }
    st->coef = omega_next;
    st->omega = omega_next;
    st->nonfinite = 0;
}

// t = mode ? omega (x - xk) + xk : x;  xk = xk1;  xk1 = t   (and the same for the impulses)
__global__ void k_chebyshev_update(const double* x, double* xk, double* xk1, int64_t nx, const double* lam, double* pk,
                                   double* pk1, int64_t nl, const AccelState* st, const DevScalars* ds) {
    if (*(volatile const int32_t*)&ds->done) return;
    const int mode = st->mode;
    const double w = st->coef;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nx + nl; i += (int64_t)gridDim.x * blockDim.x) {
        const double* cur;
        double *k0, *k1;
        int64_t q;
        if (i < nx) {
            cur = x; k0 = xk; k1 = xk1; q = i;
        } else {
            cur = lam; k0 = pk; k1 = pk1; q = i - nx;
        }
        const double t = mode ? w * (cur[q] - k0[q]) + k0[q] : cur[q];
        k0[q] = k1[q];
        k1[q] = t;
    }
}

// Power iteration of estimateSpectralRadius (projected_jacobi.cpp:154-177): delta = R W v per
// row (the sweep's row product without bias), then M v = v - S^-1 W^T delta per body
__global__ void k_linear_contact64(Scene sc, Contacts C, int nc, const double* v) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    const int64_t cap = C.cap;
    const int N = sc.N;
    const int a = C.a[c], b = C.b[c];
    const bool fr = (C.flags[c] & CF_FRICTIONAL) != 0;
    const int nr = fr ? 3 : 1;
    double gr[3];
    double xA[6], xB[6];
    if (a >= 0)
        for (int k = 0; k < 6; ++k) xA[k] = v[(size_t)k * N + a];
    for (int k = 0; k < 6; ++k) xB[k] = v[(size_t)k * N + b];
    for (int r = 0; r < nr; ++r) {
        double t = 0.0;
        if (a >= 0) {
            for (int k = 0; k < 3; ++k) t = t + (-C.rd[(3 * r + k) * cap + c]) * xA[k];
            for (int k = 0; k < 3; ++k) t = t + (-C.rcA[(3 * r + k) * cap + c]) * xA[3 + k];
        }
        for (int k = 0; k < 3; ++k) t = t + C.rd[(3 * r + k) * cap + c] * xB[k];
        for (int k = 0; k < 3; ++k) t = t + C.rcB[(3 * r + k) * cap + c] * xB[3 + k];
        gr[r] = t;
    }
    if (C.rb) block_apply64(C, c, fr, gr);
    for (int r = 0; r < nr; ++r) C.dlam[r * cap + c] = gr[r];
}
__global__ void k_linear_body64(Scene sc, Contacts C, Incidence inc, const double* v, double* Mv) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sc.N) return;
    const int N = sc.N;
    double acc[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    gather_wt<1>(C, C.dlam, inc, i, acc);
    const double Ml = sc.bf(BF_ML)[i], Ma = sc.bf(BF_MA)[i];
    for (int k = 0; k < 6; ++k) Mv[(size_t)k * N + i] = v[(size_t)k * N + i] - acc[k] / (k < 3 ? Ml : Ma);
}
__global__ void k_power_fill(double* v, int64_t n, const AccelState* st) {
    const double f = 1.0 / sqrt(st->sum_err);  // sum_err holds the chunked count of entries here
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        v[i] = f;
}
// one power step: n = ||M v||; stop with rho = 0 when M v vanishes; else lambda = n, v = M v / n
__global__ void k_power_norm(AccelState* st) {
    if (st->power_stop) return;
    const double n = sqrt(st->sum_err);
    if (!(n > 1e-300)) {
        st->power_stop = 1;
        st->lambda = 0.0;
        return;
    }
    st->lambda = n;
}
__global__ void k_power_scale(double* v, const double* Mv, int64_t n, const AccelState* st) {
    if (st->power_stop) return;
    const double d = st->lambda;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        v[i] = Mv[i] / d;
}
__global__ void k_power_finish(AccelState* st) {
    const double rho = st->power_stop ? 0.0 : smin(st->lambda, 0.995);
    st->rho = rho;
    st->rho2 = rho * rho;
    st->omega = 1.0;
}
__global__ void k_accel_init(AccelState* st) {
    st->thk = 1.0;
    st->err_prev = INFINITY;
    st->restarts = 0;
    st->disabled = 0;
    st->mode = 0;
    st->coef = 0.0;
    st->omega = 1.0;
    st->nonfinite = 0;
    st->power_stop = 0;
    st->lambda = 0.0;
}

__global__ void k_final_residual(DevScalars* ds) {
    const double maxd = __longlong_as_double((long long)ds->maxd);
    const double maxl = __longlong_as_double((long long)ds->maxl);
    ds->res_final = maxd / smax(maxl, 1e-30);
    ds->maxd = 0ull;
    ds->maxl = 0ull;
}

__global__ void k_writeback64(Scene sc, const double* x) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sc.N) return;
    const int N = sc.N;
    sc.bf(BF_VX)[i] = x[0 * (size_t)N + i];
    sc.bf(BF_VY)[i] = x[1 * (size_t)N + i];
    sc.bf(BF_VZ)[i] = x[2 * (size_t)N + i];
    sc.bf(BF_WX)[i] = x[3 * (size_t)N + i];
    sc.bf(BF_WY)[i] = x[4 * (size_t)N + i];
    sc.bf(BF_WZ)[i] = x[5 * (size_t)N + i];
}

// ---- Anderson loop (anderson_loop, projected_jacobi.cpp:242-314) on the dense iterate
// z = [x (stacked index 6 i + k); impulse rows (frictionless contacts by rank, then three rows per
// frictional contact)]. Dot products use the chunked order of the other accelerated loops.
__device__ __forceinline__ int ring_slot(const AndersonState* as, int m, int j) { return (as->head + j) % (m + 1); }

__global__ void k_and_rowmap(Contacts C, int nc, const int32_t* fl_scan, const int32_t* isfl, int32_t* rowmap) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    const int nfl = fl_scan[nc - 1] + isfl[nc - 1];
    const int rank = C.rank[c];
    if (rank < nfl) {
        rowmap[rank] = c;
    } else {
        const int row = nfl + 3 * (rank - nfl);
        for (int r = 0; r < 3; ++r) rowmap[row + r] = (int32_t)(r * C.cap + c);
    }
}

// dense <- (x, lam); mode 0: z only (start), mode 1: w, f = w - z and the newest history slot
// plain: x of length N already in stacked order and lam in row order (no row map): the
// solver-level drop-in; else x is 6 x N field-major and lam goes through the row map
__global__ void k_and_gather(int N, const double* x, const double* lam, const int32_t* rowmap, int64_t nt, int m,
                             int64_t ld, double* z, double* w, double* f, double* zh, double* fh,
                             const AndersonState* as, const DevScalars* ds, int mode, int plain) {
    if (ds && *(volatile const int32_t*)&ds->done) return;
    const int64_t nv = plain ? (int64_t)N : 6 * (int64_t)N;
    const int slot = mode ? ring_slot(as, m, as->count - 1) : 0;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nt; t += (int64_t)gridDim.x * blockDim.x) {
        const double v = t < nv ? (plain ? x[t] : x[(size_t)(t % 6) * N + t / 6])
                                : lam[plain ? t - nv : rowmap[t - nv]];
        if (!mode) {
            z[t] = v;
        } else {
            const double zt = z[t];
            const double ft = v - zt;
            w[t] = v;
            f[t] = ft;
            zh[(size_t)slot * ld + t] = zt;
            fh[(size_t)slot * ld + t] = ft;
        }
    }
}

__global__ void k_and_scatter(int N, double* x, double* lam, const int32_t* rowmap, int64_t nt, const double* z,
                              const DevScalars* ds, int plain) {
    if (ds && *(volatile const int32_t*)&ds->done) return;
    const int64_t nv = plain ? (int64_t)N : 6 * (int64_t)N;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nt; t += (int64_t)gridDim.x * blockDim.x) {
        if (t < nv)
            x[plain ? (size_t)t : (size_t)(t % 6) * N + t / 6] = z[t];
        else
            lam[plain ? t - nv : rowmap[t - nv]] = z[t];
    }
}

// push: the newest (z, f) takes the next ring slot, the oldest leaves once m + 1 are kept
__global__ void k_and_push(AndersonState* as, int m, const DevScalars* ds) {
    if (ds->done) return;
    if (as->count < m + 1)
        ++as->count;
    else
        as->head = (as->head + 1) % (m + 1);
}

// partial sums per chunk: sum 0 = the scaled velocity increment (w vs z over the velocities),
// then (dF_j . dF_l) for l <= j < mk and (dF_j . f) for j < mk, dF_j = F_{j+1} - F_j (oldest first)
__global__ void k_and_partials(int N, int64_t nt, int m, int64_t ld, const double* z, const double* w, const double* f,
                               const double* fh, double tol_rel, double tol_abs, double* part, int nch_t,
                               const AndersonState* as, const DevScalars* ds, int plain) {
    if (ds && *(volatile const int32_t*)&ds->done) return;
    const int ch = blockIdx.x * blockDim.x + threadIdx.x;
    const int sidx = blockIdx.y;
    const int mk = as->count - 1;
    const int64_t nv = plain ? (int64_t)N : 6 * (int64_t)N;
    const int nsums = 1 + mk * (mk + 1) / 2 + (mk > 0 ? mk : 0);
    if (sidx >= nsums) return;
    const int64_t n = sidx == 0 ? nv : nt;
    const int64_t j0 = (int64_t)ch * RED_CHUNK;
    if (ch >= nch_t || j0 >= n) return;
    const int64_t j1 = j0 + RED_CHUNK < n ? j0 + RED_CHUNK : n;
    double s = 0.0;
    if (sidx == 0) {
        for (int64_t t = j0; t < j1; ++t) {
            const double a = w[t], b = z[t];
            const double q = smax(fabs(a), fabs(b)) * tol_rel + tol_abs;
            const double d = (a - b) / q;
            s = s + d * d;
        }
    } else {
        const int q = sidx - 1;
        const int na = mk * (mk + 1) / 2;
        int j, l;
        if (q < na) {
            j = 0;
            while ((j + 1) * (j + 2) / 2 <= q) ++j;
            l = q - j * (j + 1) / 2;
        } else {
            j = q - na;
            l = -1;
        }
        const double* fa0 = fh + (size_t)ring_slot(as, m, j) * ld;
        const double* fa1 = fh + (size_t)ring_slot(as, m, j + 1) * ld;
        if (l >= 0) {
            const double* fb0 = fh + (size_t)ring_slot(as, m, l) * ld;
            const double* fb1 = fh + (size_t)ring_slot(as, m, l + 1) * ld;
            for (int64_t t = j0; t < j1; ++t) s = s + (fa1[t] - fa0[t]) * (fb1[t] - fb0[t]);
        } else {
            for (int64_t t = j0; t < j1; ++t) s = s + (fa1[t] - fa0[t]) * f[t];
        }
    }
    part[(size_t)sidx * nch_t + ch] = s;
}

// one thread: the stop test, then gamma from the normal equations by Gaussian elimination with
// partial pivoting (mode 1), or a plain step (mode 0, fewer than two residuals kept), or a failed
// solve (mode 2: singular or not finite)
__global__ void k_and_solve(int nv, int nch_v, int nch_t, const double* part, double* ls, int m, AndersonState* as,
                            DevScalars* ds, double residual_tol) {
    if (ds->done) return;
    double sv = 0.0;
    for (int k = 0; k < nch_v; ++k) sv = sv + part[k];
    const double err = 1.0 / sqrt((double)nv) * sqrt(sv);
    as->nonfinite = 0;
    if (err <= 1.0 || (residual_tol > 0 && ds->res_last <= residual_tol)) {
        ds->done = 1;
        return;
    }
    const int mk = as->count - 1;
    if (mk < 1) {
        as->mode = 0;
        return;
    }
    double* A = ls;
    double* b = ls + (size_t)m * m;
    double* g = b + m;
    const int na = mk * (mk + 1) / 2;
    for (int j = 0; j < mk; ++j) {
        for (int l = 0; l <= j; ++l) {
            const double* p = part + (size_t)(1 + j * (j + 1) / 2 + l) * nch_t;
            double d = 0.0;
            for (int k = 0; k < nch_t; ++k) d = d + p[k];
            A[j * mk + l] = d;
            A[l * mk + j] = d;
        }
        const double* p = part + (size_t)(1 + na + j) * nch_t;
        double d = 0.0;
        for (int k = 0; k < nch_t; ++k) d = d + p[k];
        b[j] = d;
    }
    for (int c = 0; c < mk; ++c) {
        int piv = c;
        for (int r = c + 1; r < mk; ++r)
            if (fabs(A[r * mk + c]) > fabs(A[piv * mk + c])) piv = r;
        if (!(fabs(A[piv * mk + c]) > 0.0)) {
            as->mode = 2;
            return;
        }
        if (piv != c) {
            for (int k = 0; k < mk; ++k) {
                const double t = A[c * mk + k];
                A[c * mk + k] = A[piv * mk + k];
                A[piv * mk + k] = t;
            }
            const double t = b[c];
            b[c] = b[piv];
            b[piv] = t;
        }
        for (int r = c + 1; r < mk; ++r) {
            const double fct = A[r * mk + c] / A[c * mk + c];
            for (int k = c; k < mk; ++k) A[r * mk + k] = A[r * mk + k] - fct * A[c * mk + k];
            b[r] = b[r] - fct * b[c];
        }
    }
    for (int r = mk - 1; r >= 0; --r) {
        double t = b[r];
        for (int k = r + 1; k < mk; ++k) t = t - A[r * mk + k] * g[k];
        g[r] = t / A[r * mk + r];
    }
    for (int j = 0; j < mk; ++j)
        if (!isfinite(g[j])) {
            as->mode = 2;
            return;
        }
    as->mode = 1;
}

// candidate = w - (dZ + dF) gamma (mode 1 only); flags a non-finite entry
__global__ void k_and_candidate(int64_t nt, int m, int64_t ld, const double* w, const double* zh, const double* fh,
                                const double* gam, double* cand, AndersonState* as, const DevScalars* ds) {
    if (*(volatile const int32_t*)&ds->done || as->mode != 1) return;
    const int mk = as->count - 1;
    bool bad = false;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nt; t += (int64_t)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int j = 0; j < mk; ++j) {
            const size_t a0 = (size_t)ring_slot(as, m, j) * ld + t, a1 = (size_t)ring_slot(as, m, j + 1) * ld + t;
            s = s + ((zh[a1] - zh[a0]) + (fh[a1] - fh[a0])) * gam[j];
        }
        const double c = w[t] - s;
        cand[t] = c;
        bad = bad || !isfinite(c);
    }
    if (bad) as->nonfinite = 1;
}

// z = candidate when it exists and is finite, else w; a failed step drops the history
__global__ void k_and_select(int64_t nt, double* z, const double* w, const double* cand, AndersonState* as,
                             const DevScalars* ds) {
    if (*(volatile const int32_t*)&ds->done) return;
    const bool take = as->mode == 1 && !as->nonfinite;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nt; t += (int64_t)gridDim.x * blockDim.x)
        z[t] = take ? cand[t] : w[t];
}
__global__ void k_and_drop(AndersonState* as, const DevScalars* ds) {
    if (ds->done) return;
    if (as->mode == 2 || (as->mode == 1 && as->nonfinite)) {
        as->count = 0;
        as->head = 0;
    }
}
__global__ void k_and_init(AndersonState* as) {
    as->head = 0;
    as->count = 0;
    as->mode = 0;
    as->nonfinite = 0;
}

__global__ void k_trace64(Contacts C, int gen, int nc, const int32_t* fl_scan, const int32_t* isfl, double* out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    const int nfl = fl_scan[nc - 1] + isfl[nc - 1];
    const int rank = C.rank[c];
    const int64_t cap = C.cap;
    if (rank < nfl) {
        out[rank] = C.lam[gen][c];
    } else {
        const int row = nfl + 3 * (rank - nfl);
        for (int r = 0; r < 3; ++r) out[row + r] = C.lam[gen][r * cap + c];
    }
}

}  // namespace

void launch_rhs64(const Scene& sc, double dt, const double* g, double* rhs, cudaStream_t s, int implicit_gyro) {
    if (sc.N == 0) return;
    k_rhs64<<<nblk(sc.N), NT, 0, s>>>(sc, dt, g[0], g[1], g[2], rhs, implicit_gyro);
}
void launch_drift64(const Scene& sc, double h, int compute_R, cudaStream_t s, int32_t* nonfinite) {
    if (sc.N + sc.S == 0) return;
    k_drift64<<<nblk(sc.N + sc.S), NT, 0, s>>>(sc, h, compute_R, nonfinite);
}
void launch_static_motion64(const Scene& sc, const double* mot, const int32_t* flag, cudaStream_t s) {
    if (sc.S > 0 && mot && flag) k_static_motion64<<<nblk(sc.S), NT, 0, s>>>(sc, mot, flag);
}
void launch_static_flags64(const Scene& sc, double margin, int32_t* flags, cudaStream_t s) {
    if (sc.N == 0) return;
    k_static_flags64<<<nblk(sc.N), NT, 0, s>>>(sc, margin, flags);
}
void launch_pos32(const Scene& sc, const Grid& g, float4* p32, cudaStream_t s) {
    if (sc.N) k_pos32<<<nblk(sc.N), NT, 0, s>>>(sc, g, p32);
}
void launch_pair_count64(const Scene& sc, const Grid& g, const uint32_t* cell_body, const int32_t* cell_start,
                         const int32_t* cell_end, const float4* p32, int32_t* plist, double margin, int32_t* counts,
                         DevScalars* ds, cudaStream_t s) {
    if (sc.N == 0) return;
    Contacts dummy;
    k_pairs64<false><<<nblk(sc.N), NT, 0, s>>>(sc, g, cell_body, cell_start, cell_end, p32, plist, margin, counts,
                                                nullptr, 0, dummy, 0, 0, 0, ds);
}
void launch_static_write64(const Scene& sc, double margin, const int32_t* flags, const int32_t* pos,
                           Contacts& C, int gen, int combine, int friction_enable, cudaStream_t s) {
    if (sc.N == 0) return;
    k_static_write64<<<nblk(sc.N), NT, 0, s>>>(sc, margin, flags, pos, C, gen, combine, friction_enable);
}
void launch_pair_write64(const Scene& sc, const Grid& g, const uint32_t* cell_body, const int32_t* cell_start,
                         const int32_t* cell_end, const float4* p32, int32_t* plist, double margin,
                         const int32_t* offsets, int32_t base, Contacts& C, int gen, int combine, int friction_enable,
                         DevScalars* ds, cudaStream_t s) {
    if (sc.N == 0) return;
    k_pairs64<true><<<nblk(sc.N), NT, 0, s>>>(sc, g, cell_body, cell_start, cell_end, p32, plist, margin, nullptr,
                                               offsets, base, C, gen, combine, friction_enable, ds);
}
void launch_contact_setup64(const Scene& sc, Contacts& C, int gen, int nc, int prev_count, double alpha,
                            double match2, int warmstart, cudaStream_t s) {
    if (nc == 0) return;
    k_contact_setup64<<<nblk(nc), NT, 0, s>>>(sc, C, gen, nc, prev_count, alpha, match2, warmstart);
}
void launch_block_invert64(const Contacts& C, int nc, cudaStream_t s) {
    if (nc == 0 || !C.rb) return;
    k_block_invert64<<<nblk(nc), NT, 0, s>>>(C, nc);
}
void launch_frictionless_flags(const Contacts& C, int nc, int32_t* isfl, cudaStream_t s) {
    if (nc == 0) return;
    k_frictionless_flags<<<nblk(nc), NT, 0, s>>>(C, nc, isfl);
}
void launch_rank_and_incidence(const Scene& sc, Contacts& C, int nc, const int32_t* fl_scan, const int32_t* isfl,
                               Incidence& inc, cudaStream_t s, int by_contact) {
    if (nc == 0) return;
    k_rank_incidence<<<nblk(nc), NT, 0, s>>>(sc.N, C, nc, fl_scan, isfl, inc, by_contact);
}
void launch_xinit64(const Scene& sc, const Contacts& C, int gen, const Incidence& inc, const double* rhs, double* x,
                    cudaStream_t s) {
    if (sc.N == 0) return;
    k_xinit64<<<nblk(sc.N), NT, 0, s>>>(sc, C, gen, inc, rhs, x);
}
void launch_sweep_contact64(const Scene& sc, Contacts& C, int gen, int nc, const double* x, DevScalars* ds, int dry,
                            cudaStream_t s) {
    if (nc == 0) return;
    k_sweep_contact64<<<nblk(nc), NT, 0, s>>>(sc, C, gen, nc, x, ds, dry);
}
void launch_sweep_body64(const Scene& sc, const Contacts& C, const Incidence& inc, double* x, double tol_abs,
                         double tol_rel, int want_velres, DevScalars* ds, cudaStream_t s) {
    if (sc.N == 0) return;
    k_sweep_body64<<<nblk(sc.N), NT, 0, s>>>(sc, C, inc, x, tol_abs, tol_rel, want_velres, ds);
}
void launch_check(DevScalars* ds, int iter, double residual_tol, int nv, int check_vel, cudaStream_t s) {
    k_check<<<1, 1, 0, s>>>(ds, iter, residual_tol, nv, check_vel);
}
void launch_final_residual(DevScalars* ds, cudaStream_t s) { k_final_residual<<<1, 1, 0, s>>>(ds); }

int accel_chunks(int N) { return (6 * N + RED_CHUNK - 1) / RED_CHUNK; }
void launch_accel_reduce(int N, int op, const double* a, const double* b, const double* c, double tol_rel,
                         double tol_abs, double* part, AccelState* st, double* out, const DevScalars* ds,
                         cudaStream_t s, int plain) {
    const int nch = plain ? (N + RED_CHUNK - 1) / RED_CHUNK : accel_chunks(N);
    k_chunk_partials<<<nblk(nch, 128), 128, 0, s>>>(N, op, a, b, c, tol_rel, tol_abs, part, st, ds, plain);
    k_chunk_total<<<1, 1, 0, s>>>(part, nch, out, ds);
}
void launch_accel_copy(double* xd, const double* xs, int64_t nx, double* ld, const double* ls, int64_t nl,
                       const DevScalars* ds, cudaStream_t s) {
    k_accel_copy<<<nblk(nx + nl), NT, 0, s>>>(xd, xs, nx, ld, ls, nl, ds);
}
void launch_nesterov_step(AccelState* st, DevScalars* ds, int nv, double beta_threshold, int restart_limit, double* xy,
                          double* xk, const double* xk1, int64_t nx, double* py, double* pk, const double* pk1,
                          int64_t nl, double residual_tol, cudaStream_t s) {
    k_nesterov_decide<<<1, 1, 0, s>>>(st, ds, nv, beta_threshold, restart_limit, residual_tol);
    k_nesterov_update<<<nblk(nx + nl), NT, 0, s>>>(xy, xk, xk1, nx, py, pk, pk1, nl, st, ds);
}
void launch_chebyshev_step(AccelState* st, DevScalars* ds, int nv, int iter, const double* x, double* xk, double* xk1,
                           int64_t nx, const double* lam, double* pk, double* pk1, int64_t nl, double residual_tol,
                           cudaStream_t s) {
    k_chebyshev_decide<<<1, 1, 0, s>>>(st, ds, nv, iter, residual_tol);
    k_chebyshev_update<<<nblk(nx + nl), NT, 0, s>>>(x, xk, xk1, nx, lam, pk, pk1, nl, st, ds);
}
void launch_power_iteration(int N, int plain, double* v, double* Mv, double* part, AccelState* st,
                            const std::function<void()>& apply, cudaStream_t s) {
    const int64_t n = plain ? (int64_t)N : 6 * (int64_t)N;
    k_accel_init<<<1, 1, 0, s>>>(st);
    launch_accel_reduce(N, ACC_ONES, nullptr, nullptr, nullptr, 0.0, 0.0, part, st, &st->sum_err, nullptr, s, plain);
    k_power_fill<<<nblk(n), NT, 0, s>>>(v, n, st);
    for (int it = 0; it < 8; ++it) {
        apply();
        launch_accel_reduce(N, ACC_NORM2, Mv, nullptr, nullptr, 0.0, 0.0, part, st, &st->sum_err, nullptr, s, plain);
        k_power_norm<<<1, 1, 0, s>>>(st);
        k_power_scale<<<nblk(n), NT, 0, s>>>(v, Mv, n, st);
    }
    k_power_finish<<<1, 1, 0, s>>>(st);
}
void launch_spectral_radius(const Scene& sc, Contacts& C, const Incidence& inc, int nc, double* v, double* Mv,
                            double* part, AccelState* st, cudaStream_t s) {
    const int N = sc.N;
    launch_power_iteration(N, 0, v, Mv, part, st, [&]() {
        if (nc > 0) k_linear_contact64<<<nblk(nc), NT, 0, s>>>(sc, C, nc, v);
        k_linear_body64<<<nblk(N), NT, 0, s>>>(sc, C, inc, v, Mv);
    }, s);
}
void launch_accel_init(AccelState* st, cudaStream_t s) { k_accel_init<<<1, 1, 0, s>>>(st); }

int anderson_sums(int m) { return 1 + m * (m + 1) / 2 + m; }
int anderson_chunks(int64_t n) { return (int)((n + RED_CHUNK - 1) / RED_CHUNK); }
static int grid_of(int64_t n) { return (int)std::min<int64_t>(std::max<int64_t>(nblk(n), 1), 4096); }
void launch_anderson_begin(const Contacts& C, int gen, int nc, const int32_t* fl_scan, const int32_t* isfl, int N,
                           const double* x, AndersonBufs& A, cudaStream_t s) {
    k_and_init<<<1, 1, 0, s>>>(A.st);
    if (nc > 0) k_and_rowmap<<<nblk(nc), NT, 0, s>>>(C, nc, fl_scan, isfl, A.rowmap);
    k_and_gather<<<grid_of(A.nt), NT, 0, s>>>(N, x, C.lam[gen], A.rowmap, A.nt, A.m, A.nt_cap, A.z, A.w, A.f, A.zh,
                                              A.fh, A.st, nullptr, 0, 0);
}
void launch_anderson_begin_plain(int nv, const double* x, const double* lam, AndersonBufs& A, cudaStream_t s) {
    k_and_init<<<1, 1, 0, s>>>(A.st);
    k_and_gather<<<grid_of(A.nt), NT, 0, s>>>(nv, x, lam, nullptr, A.nt, A.m, A.nt_cap, A.z, A.w, A.f, A.zh, A.fh,
                                              A.st, nullptr, 0, 1);
}
void launch_anderson_scatter(int N, double* x, double* lam, const AndersonBufs& A, const DevScalars* ds,
                             cudaStream_t s) {
    k_and_scatter<<<grid_of(A.nt), NT, 0, s>>>(N, x, lam, A.rowmap, A.nt, A.z, ds, A.plain);
}
void launch_anderson_mix(int N, const double* x, const double* lam, const AndersonBufs& A, double tol_rel,
                         double tol_abs, double residual_tol, DevScalars* ds, cudaStream_t s) {
    const int nv = A.plain ? N : 6 * N;
    const int nch_t = anderson_chunks(A.nt), nch_v = anderson_chunks(nv);
    k_and_push<<<1, 1, 0, s>>>(A.st, A.m, ds);
    k_and_gather<<<grid_of(A.nt), NT, 0, s>>>(N, x, lam, A.rowmap, A.nt, A.m, A.nt_cap, A.z, A.w, A.f, A.zh, A.fh,
                                              A.st, ds, 1, A.plain);
    dim3 g((unsigned)nblk(nch_t, 128), (unsigned)anderson_sums(A.m));
    k_and_partials<<<g, 128, 0, s>>>(N, A.nt, A.m, A.nt_cap, A.z, A.w, A.f, A.fh, tol_rel, tol_abs, A.part, nch_t,
                                     A.st, ds, A.plain);
    k_and_solve<<<1, 1, 0, s>>>(nv, nch_v, nch_t, A.part, A.ls, A.m, A.st, ds, residual_tol);
    const double* gam = A.ls + (size_t)A.m * A.m + A.m;
    k_and_candidate<<<grid_of(A.nt), NT, 0, s>>>(A.nt, A.m, A.nt_cap, A.w, A.zh, A.fh, gam, A.cand, A.st, ds);
    k_and_select<<<grid_of(A.nt), NT, 0, s>>>(A.nt, A.z, A.w, A.cand, A.st, ds);
    k_and_drop<<<1, 1, 0, s>>>(A.st, ds);
}
void launch_writeback64(const Scene& sc, const double* x, cudaStream_t s) {
    if (sc.N == 0) return;
    k_writeback64<<<nblk(sc.N), NT, 0, s>>>(sc, x);
}
void launch_trace64(const Contacts& C, int gen, int nc, const int32_t* fl_scan, const int32_t* isfl, double* out,
                    cudaStream_t s) {
    if (nc == 0) return;
    k_trace64<<<nblk(nc), NT, 0, s>>>(C, gen, nc, fl_scan, isfl, out);
}

}  // namespace cdx
