// Split-precision form of the Moreau midpoint step.
//
// FP32: contact detection, the Delassus rows and the cone projection. For spheres the contact
// Jacobian is fully determined by the normal n and the signed lever lengths rhoA, rhoB along n
// (the contact point is the midpoint of the witness points, collision_coal.cpp:149), so a contact
// row is rebuilt on the fly from 9 floats instead of the 54 FP64 words of W and RW:
//   gamma_n  = n.dv + b_n,  gamma_t1 = t1.dv + t2.Om + b_t1,  gamma_t2 = t2.dv - t1.Om + b_t2,
//   dv = vB - vA, Om = rhoB wB - rhoA wA (world-frame angular velocities),
// and W^T dlambda is P = dl_n n + dl_t1 t1 + dl_t2 t2 on the linear DOFs and rho (dl_t1 t2 - dl_t2 t1)
// on the angular ones, scattered with float4 vector atomics pre-scaled by M^-1.
// FP64: positions, quaternions, velocities (the body state), the final velocity
// v = v_free + M^-1 W^T lambda and the complementarity residual, both on FP64 contact geometry
// recomputed from the FP64 positions.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>

#include "cdx_internal.h"
#include "fp64_math.cuh"
#include "split.h"
#include "nr64.cuh"

namespace cdx {

namespace {

constexpr int NT = 256;
constexpr int MAX_PAIR = 64;
inline int nblk(int64_t n, int nt = NT) { return (int)((n + nt - 1) / nt); }

__device__ __forceinline__ float3 f3(float4 a) { return make_float3(a.x, a.y, a.z); }
__device__ __forceinline__ float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator*(float s, float3 a) { return make_float3(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ float3 crossf(float3 a, float3 b) {
    return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

// Frisvad tangent frame (tangentFrameFromNormal) in FP32 for a unit normal
__device__ __forceinline__ void frame32(float3 n, float3& t1, float3& t2) {
    if (n.z < -0.9999999f) {
        t1 = make_float3(0.f, -1.f, 0.f);
        const float d = dot(n, t1);
        t1 = t1 - d * n;
    } else {
        const float a = __fdividef(1.f, 1.f + n.z);  // 1 + n.z >= 1e-7 on this branch
        const float b = (-n.x * n.y) * a;
        t1 = make_float3(1.f - (n.x * n.x) * a, b, -n.x);
    }
    t1 = rsqrtf(dot(t1, t1)) * t1;
    t2 = crossf(n, t1);
}

__device__ __forceinline__ float combine_mu32(int mode, float a, float b) {
    a = fmaxf(0.f, a);
    b = fmaxf(0.f, b);
    if (mode == 1) return (a + b) * 0.5f;
    if (mode == 2) return sqrtf(a * b);
    return fminf(a, b);
}

// the sign bit of the mu field flags a contact that carries a velocity bias
__device__ __forceinline__ bool split_has_bias(float mu_field) { return signbit(mu_field); }


// Max of (a, b) over the block, then one atomic per block: per-warp atomics on one address
// serialise at a single L2 slice and dominated the sweep.
template <typename T>
__device__ __forceinline__ void block_max2(T& a, T& b) {
    __shared__ T sh[2][32];
    for (int o = 16; o > 0; o >>= 1) {
        a = max(a, __shfl_xor_sync(0xffffffffu, a, o));
        b = max(b, __shfl_xor_sync(0xffffffffu, b, o));
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) {
        sh[0][wid] = a;
        sh[1][wid] = b;
    }
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
        a = lane < nw ? sh[0][lane] : T(0);
        b = lane < nw ? sh[1][lane] : T(0);
        for (int o = 16; o > 0; o >>= 1) {
            a = max(a, __shfl_xor_sync(0xffffffffu, a, o));
            b = max(b, __shfl_xor_sync(0xffffffffu, b, o));
        }
    }
}

// explicitPositionUpdate in FP64 for the split form: the same update as the plain method, with the
// quaternion normalised by one reciprocal square root instead of four divisions
__device__ __forceinline__ void drift_fast(double* x, double* q, const double* v, const double* w, double h) {
    for (int k = 0; k < 3; ++k) x[k] = x[k] + h * v[k];
    const double qp[4] = {q[0], q[1], q[2], q[3]};
    const double hh = h * 0.5;
    q[3] = qp[3] - hh * (qp[0] * w[0] + qp[1] * w[1] + qp[2] * w[2]);
    q[0] = qp[0] + hh * (qp[3] * w[0] + (qp[1] * w[2] - qp[2] * w[1]));
    q[1] = qp[1] + hh * (qp[3] * w[1] + (qp[2] * w[0] - qp[0] * w[2]));
    q[2] = qp[2] + hh * (qp[3] * w[2] + (qp[0] * w[1] - qp[1] * w[0]));
    const double n2 = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
    if (!(n2 > 0.0) || !isfinite(n2)) {
        for (int k = 0; k < 4; ++k) q[k] = qp[k];
        return;
    }
    double inv = rsqrt_nr(n2);
    if (qp[0] * q[0] + qp[1] * q[1] + qp[2] * q[2] + qp[3] * q[3] < 0.0) inv = -inv;
    for (int k = 0; k < 4; ++k) q[k] *= inv;
}

// ------------------------------------------------------------------ per-body preparation (FP64)
__global__ void k_s_prep(Scene sc, SplitBuf sb, double dt, double g0, double g1, double g2, double h1,
                         int implicit_gyro, const double* smot, const int32_t* smflag) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < sc.N) {
        const int N = sc.N;
        double x[3] = {sc.bf(BF_PX)[i], sc.bf(BF_PY)[i], sc.bf(BF_PZ)[i]};
        double q[4] = {sc.bf(BF_QX)[i], sc.bf(BF_QY)[i], sc.bf(BF_QZ)[i], sc.bf(BF_QW)[i]};
        const double v[3] = {sc.bf(BF_VX)[i], sc.bf(BF_VY)[i], sc.bf(BF_VZ)[i]};
        const double w[3] = {sc.bf(BF_WX)[i], sc.bf(BF_WY)[i], sc.bf(BF_WZ)[i]};
        const double I = sc.bf(BF_INERTIA)[i];
        const double il = sc.bf(BF_MINVL)[i], ia = sc.bf(BF_MINVA)[i];
        // free velocities S^-1 rhs = v + h M^-1 (f_ext + f_gyro)  (pj_assembler.cpp:152-153)
        const double Iw[3] = {I * w[0], I * w[1], I * w[2]};
        double c[3];
        f64::cross3(w, Iw, c);
        const double g[3] = {g0, g1, g2};
        double vf[3], wf[3];
        for (int k = 0; k < 3; ++k) {
            vf[k] = v[k] + dt * g[k];
            wf[k] = implicit_gyro ? w[k] : w[k] + dt * ia * (-c[k]);
        }
        drift_fast(x, q, v, w, h1);
        sc.bf(BF_PX)[i] = x[0]; sc.bf(BF_PY)[i] = x[1]; sc.bf(BF_PZ)[i] = x[2];
        sc.bf(BF_QX)[i] = q[0]; sc.bf(BF_QY)[i] = q[1]; sc.bf(BF_QZ)[i] = q[2]; sc.bf(BF_QW)[i] = q[3];
        double R[9];
        f64::rotmat(q, R);
        for (int k = 0; k < 9; ++k) sc.bf(BF_R0 + k)[i] = R[k];
        // world-frame angular velocities: R w
        double wfw[3];
        for (int k = 0; k < 3; ++k) wfw[k] = R[3 * k] * wf[0] + R[3 * k + 1] * wf[1] + R[3 * k + 2] * wf[2];
        for (int k = 0; k < 3; ++k) {
            sb.vfree[(size_t)k * N + i] = vf[k];
            sb.vfree[(size_t)(3 + k) * N + i] = wfw[k];
        }
        sb.vel4[2 * i] = make_float4((float)vf[0], (float)vf[1], (float)vf[2], (float)il);
        sb.vel4[2 * i + 1] = make_float4((float)wfw[0], (float)wfw[1], (float)wfw[2], (float)ia);
        if (sb.has_restitution) {
            double ww[3];
            for (int k = 0; k < 3; ++k) ww[k] = R[3 * k] * w[0] + R[3 * k + 1] * w[1] + R[3 * k + 2] * w[2];
            sb.vn4[2 * i] = make_float4((float)v[0], (float)v[1], (float)v[2], 0.f);
            sb.vn4[2 * i + 1] = make_float4((float)ww[0], (float)ww[1], (float)ww[2], 0.f);
        }
        sb.acc[0][2 * i] = sb.vel4[2 * i];
        sb.acc[0][2 * i + 1] = sb.vel4[2 * i + 1];
        sb.acc[1][2 * i] = sb.vel4[2 * i];
        sb.acc[1][2 * i + 1] = sb.vel4[2 * i + 1];
        sb.acc[2][2 * i] = sb.vel4[2 * i];
        sb.acc[2][2 * i + 1] = sb.vel4[2 * i + 1];
        const int s = sc.body_scene[i];
        const double* o = &sb.origin[3 * s];
        const double rad = sc.bf(BF_RAD)[i];
        const double xr[3] = {x[0] - o[0], x[1] - o[1], x[2] - o[2]};
        const float4 hi = make_float4((float)xr[0], (float)xr[1], (float)xr[2], (float)rad);
        sb.pos64[i] = make_double4(x[0], x[1], x[2], rad);
        sb.pos4[i] = hi;
        sb.pos4lo[i] = make_float4((float)(xr[0] - (double)hi.x), (float)(xr[1] - (double)hi.y),
                                   (float)(xr[2] - (double)hi.z), (float)(rad - (double)hi.w));
    } else if (i < sc.N + sc.S) {
        const int s = i - sc.N;
        double x[3] = {sc.sf(SF_PX)[s], sc.sf(SF_PY)[s], sc.sf(SF_PZ)[s]};
        double q[4] = {sc.sf(SF_QX)[s], sc.sf(SF_QY)[s], sc.sf(SF_QZ)[s], sc.sf(SF_QW)[s]};
        double v[3] = {sc.sf(SF_VX)[s], sc.sf(SF_VY)[s], sc.sf(SF_VZ)[s]};
        double w[3] = {sc.sf(SF_WX)[s], sc.sf(SF_WY)[s], sc.sf(SF_WZ)[s]};
        drift_fast(x, q, v, w, h1);
        // prescribed motion (Trajectory::update, after the first drift): pose and twist as given
        const int f = smflag ? smflag[s] : 0;
        if (f) {
            const double* m = smot + 13 * (size_t)s;
            if (f & 1)
                for (int k = 0; k < 3; ++k) x[k] = m[k];
            if (f & 2)
                for (int k = 0; k < 4; ++k) q[k] = m[3 + k];
            if (f & 4)
                for (int k = 0; k < 3; ++k) v[k] = m[7 + k];
            if (f & 8)
                for (int k = 0; k < 3; ++k) w[k] = m[10 + k];
            for (int k = 0; k < 3; ++k) {
                sc.sf(SF_VX + k)[s] = v[k];
                sc.sf(SF_WX + k)[s] = w[k];
            }
        }
        sc.sf(SF_PX)[s] = x[0]; sc.sf(SF_PY)[s] = x[1]; sc.sf(SF_PZ)[s] = x[2];
        sc.sf(SF_QX)[s] = q[0]; sc.sf(SF_QY)[s] = q[1]; sc.sf(SF_QZ)[s] = q[2]; sc.sf(SF_QW)[s] = q[3];
        double R[9];
        f64::rotmat(q, R);
        for (int k = 0; k < 9; ++k) sc.sf(SF_R0 + k)[s] = R[k];
        double ww[3];
        for (int k = 0; k < 3; ++k) ww[k] = R[3 * k] * w[0] + R[3 * k + 1] * w[1] + R[3 * k + 2] * w[2];
        const int scn = sc.static_scene[s];
        const double* o = &sb.origin[3 * scn];
        const int kind = sc.static_kind[s];
        double u[3] = {sc.sf(SF_DX)[s], sc.sf(SF_DY)[s], sc.sf(SF_DZ)[s]};
        if (kind == 2) {
            // a cylinder's axis turns with the static
            const double a[3] = {sc.sf(SF_AX)[s], sc.sf(SF_AY)[s], sc.sf(SF_AZ)[s]};
            for (int k = 0; k < 3; ++k) u[k] = (R[3 * k] * a[0] + R[3 * k + 1] * a[1]) + R[3 * k + 2] * a[2];
        } else if (kind == 3) {
            // a box's axes are the columns of R
            for (int k = 0; k < 3; ++k)
                sb.st_box[3 * s + k] = make_float4((float)R[k], (float)R[3 + k], (float)R[6 + k], (float)sc.sf(SF_EX + k)[s]);
        }
        const double pl[3] = {x[0] - o[0], x[1] - o[1], x[2] - o[2]};
        const double dl = u[0] * pl[0] + u[1] * pl[1] + u[2] * pl[2];
        // .w: the halfspace offset n . x, or a cylinder's half length
        sb.st_dir[s] = make_float4((float)u[0], (float)u[1], (float)u[2],
                                   kind == 2 ? (float)sc.sf(SF_HL)[s] : (float)dl);
        sb.st_pt[s] = make_float4((float)pl[0], (float)pl[1], (float)pl[2], (float)sc.sf(SF_RAD)[s]);
        sb.st_v[s] = make_float4((float)v[0], (float)v[1], (float)v[2], (float)sc.static_kind[s]);
        sb.st_w[s] = make_float4((float)ww[0], (float)ww[1], (float)ww[2], (float)sc.sf(SF_MU)[s]);
    }
}

// ------------------------------------------------------------------ narrow phase (FP32)
struct CGeom32 {
    float3 n;
    float rhoB;
    float sep;  // plane: s = n.x - d ; drum: radial distance
};

__device__ __forceinline__ bool static_test32(const SplitBuf& sb, int s, float3 x, float r, float margin,
                                              CGeom32& g) {
    const float4 dd = sb.st_dir[s];
    const float3 u = f3(dd);
    if (sb.st_v[s].w == 0.f) {
        const float sd = dot(u, x) - dd.w;
        if (!((sd - r) <= margin)) return false;
        g.n = u;
        g.rhoB = -0.5f * (sd + r);
        g.sep = sd;
        return true;
    }
    const float4 pp = sb.st_pt[s];
    const float3 rel = x - f3(pp);
    if (sb.st_v[s].w == 3.f) {
        // solid box: the FP64 method's box_geom in FP32 (centre in the box frame, clamped outside,
        // nearest face inside); n from the box to the sphere, sd the centre's signed distance
        const float4 b0 = sb.st_box[3 * s], b1 = sb.st_box[3 * s + 1], b2 = sb.st_box[3 * s + 2];
        const float c[3] = {dot(f3(b0), rel), dot(f3(b1), rel), dot(f3(b2), rel)};
        const float e[3] = {b0.w, b1.w, b2.w};
        float d[3];
        float sd;
        if (!(fabsf(c[0]) > e[0] || fabsf(c[1]) > e[1] || fabsf(c[2]) > e[2])) {
            int f = 0;
            float best = e[0] - fabsf(c[0]);
            for (int k = 1; k < 3; ++k) {
                const float dk = e[k] - fabsf(c[k]);
                if (dk < best) {
                    best = dk;
                    f = k;
                }
            }
            for (int k = 0; k < 3; ++k) d[k] = k == f ? (c[k] < 0.f ? -1.f : 1.f) : 0.f;
            sd = -best;
        } else {
            for (int k = 0; k < 3; ++k) d[k] = c[k] - fminf(fmaxf(c[k], -e[k]), e[k]);
            sd = sqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            const float inv = __frcp_rn(sd);
            for (int k = 0; k < 3; ++k) d[k] *= inv;
        }
        if (!((sd - r) <= margin)) return false;
        g.n = d[0] * f3(b0) + d[1] * f3(b1) + d[2] * f3(b2);
        g.rhoB = -0.5f * (sd + r);
        g.sep = sd;
        return true;
    }
    const float ax = dot(rel, u);
    const float3 perp = rel - ax * u;
    const float rho = sqrtf(dot(perp, perp));
    if (sb.st_v[s].w == 2.f) {
        // solid cylinder: the nearest point of the side, a cap or a rim (the FP64 method's
        // cylinder_geom in FP32); n from the cylinder to the sphere, sd the centre's signed distance
        const float R = pp.w, h = dd.w, sg = ax < 0.f ? -1.f : 1.f, aax = fabsf(ax);
        float3 e;
        if (rho > 0.f) {
            e = __frcp_rn(rho) * perp;
        } else {
            float3 t2;
            frame32(u, e, t2);
        }
        const bool out_side = rho > R, out_cap = aax > h;
        float sd;
        float3 n;
        if (!out_side && !out_cap) {
            const float dside = R - rho, dcap = h - aax;
            if (dside <= dcap) {
                n = e;
                sd = -dside;
            } else {
                n = sg * u;
                sd = -dcap;
            }
        } else if (!out_cap) {
            n = e;
            sd = rho - R;
        } else if (!out_side) {
            n = sg * u;
            sd = aax - h;
        } else {
            const float3 d = rel - ((sg * h) * u + R * e);
            sd = sqrtf(dot(d, d));
            n = __frcp_rn(sd) * d;
        }
        if (!((sd - r) <= margin)) return false;
        g.n = n;
        g.rhoB = -0.5f * (sd + r);
        g.sep = sd;
        return true;
    }
    if (!(((pp.w - rho) - r) <= margin)) return false;
    g.n = rho > 0.f ? (-__frcp_rn(rho)) * perp : make_float3(0.f, 0.f, 1.f);
    g.rhoB = -0.5f * ((pp.w - rho) + r);
    g.sep = rho;
    return true;
}

// Contact membership near the threshold. The FP32 distance of a pair or of a sphere and a static
// is off the FP64 one by the rounding of the FP32 coordinates (relative to the scene origin): at
// most a few 1e-7 of the coordinates' magnitude. A settled pile rests on contacts whose gaps are
// that small, so FP32 alone admitted and dropped hundreds of them from step to step (each new one
// starting from a zero impulse, each lost one unloading its spheres), and a warm-started step
// that the FP64 method solved in 26 sweeps took the split form about 2,000. So the FP32 test only
// settles the pairs farther than a band of 3e-7 (1 + the largest coordinate + the radii and
// extents) from the threshold (the rounding is at most 2.1e-7 of the largest coordinate, plus the
// FP32 arithmetic's few 1e-7 of the lengths compared); inside the band a pair is tested again in
// FP32 with the rounded-off low parts of its coordinates and radii added back (a band of a few
// 1e-8), and only inside that does the FP64 distance, on the FP64 positions, decide. A sphere and
// a static go from the first band straight to FP64.
__device__ __forceinline__ void geom64(const Scene& sc, int a, int b, double* n, double& rhoA, double& rhoB);
__device__ __forceinline__ float band32(float3 x, float3 y) {
    const float m = fmaxf(fmaxf(fmaxf(fabsf(x.x), fabsf(x.y)), fabsf(x.z)), fmaxf(fmaxf(fabsf(y.x), fabsf(y.y)), fabsf(y.z)));
    return 3e-7f * (1.f + m);
}
// the FP64 distance of static -a-1 and sphere b against the margin (out of line: taken by few
// spheres, it would otherwise hold its FP64 registers across the whole static loop)
__device__ __noinline__ bool member64(const Scene& sc, int a, int b, double margin) {
    double n[3], rA, rB;
    geom64(sc, a, b, n, rA, rB);
    // rhoB = -(gap + r_b) / 2 for statics: -2 rhoB - 2 r_b is the gap
    return (-2.0 * rB - 2.0 * sc.bf(BF_RAD)[b]) <= margin;
}
// a pair's FP64 test as squared lengths, |d|^2 <= (r_a + r_b + margin)^2: no square root on the
// FP64 pipe (the FP64 method's (|d| - r_a) - r_b <= margin, up to its last bit)
__device__ __forceinline__ bool pair_member64(const SplitBuf& sb, int a, int b, double margin) {
    const double4 pa = sb.pos64[a], pb = sb.pos64[b];
    const double dx = pb.x - pa.x, dy = pb.y - pa.y, dz = pb.z - pa.z;
    const double L = (pa.w + pb.w) + margin;
    return L >= 0.0 && dx * dx + dy * dy + dz * dz <= L * L;
}
__device__ __forceinline__ bool static_member(const Scene& sc, const SplitBuf& sb, int st, int i, float4 p, float margin,
                                              double margin64) {
    CGeom32 g;
    const float4 pp = sb.st_pt[st], dd = sb.st_dir[st];
    float ext = fabsf(pp.w) + fabsf(dd.w);
    if (sb.st_v[st].w == 3.f) ext += fmaxf(fmaxf(sb.st_box[3 * st].w, sb.st_box[3 * st + 1].w), sb.st_box[3 * st + 2].w);
    const float band = band32(f3(p), f3(pp)) + 3e-7f * (ext + p.w);
    if (!static_test32(sb, st, f3(p), p.w, margin + band, g)) return false;
    // the FP32 gap: sep is the signed distance of the centre (the radial one for a drum's wall)
    const float gap = sb.st_v[st].w == 1.f ? (pp.w - g.sep) - p.w : g.sep - p.w;
    if (gap <= margin - band) return true;
    return member64(sc, -st - 1, i, margin64);
}

// (at most 42 registers, as the pair kernels: one wave of 1,316 spheres an SM)
__global__ void __launch_bounds__(256, 6) k_s_static_flags(Scene sc, SplitBuf sb, float margin, double margin64,
                                                            int32_t* flags) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sc.N) return;
    const int s = sc.body_scene[i];
    const int b0 = sc.scene_body_start[s], ns_b = sc.scene_body_start[s + 1] - b0;
    const int st0 = sc.scene_static_start[s], nst = sc.scene_static_start[s + 1] - st0;
    const float4 p = sb.pos4[i];
    const int L = sc.max_statics;
    for (int l = 0; l < L; ++l) {
        int f = 0;
        if (l < nst) f = static_member(sc, sb, st0 + l, i, p, margin, margin64) ? 1 : 0;
        flags[(size_t)b0 * L + (size_t)l * ns_b + (i - b0)] = f;
    }
}

// warm start: the same pair among the previous step's contacts [lo, hi) (at most a few), within
// collision.match_max_dist of its old contact point (contact_tracker.cpp:43-72)
__device__ __forceinline__ void warm_start(const SplitBuf& sb, int gen, int lo, int hi, unsigned long long key,
                                           float3 pt, float match2, float4& lam0) {
    lam0 = make_float4(0.f, 0.f, 0.f, 0.f);
    const unsigned long long* pk = sb.key[gen ^ 1];
    for (int p = lo; p < hi; ++p) {
        const unsigned long long k = pk[p];
        if (k < key) continue;
        if (k == key) {
            const float3 d = pt - f3(sb.pt[gen ^ 1][p]);
            if (dot(d, d) <= match2) lam0 = sb.lam[gen ^ 1][p];
        }
        break;
    }
}

// rows' scaling, bias and warm start of one contact; side A body index a (< 0: static)
__device__ __forceinline__ void finish_contact32(const Scene& sc, SplitBuf& sb, int gen, int c, int a, int b,
                                                 float3 n, float rhoA, float rhoB, float3 pt, float mu_a,
                                                 float rn_a, float rt_a, const float3* wall_v, const float3* wall_w,
                                                 const float3* wall_p, const SplitParams& P, int prev_lo, int prev_hi) {
    if (c >= sb.cap) return;  // more contacts than slots: the host sees cap_err and redoes the step
    float3 vna = make_float3(0.f, 0.f, 0.f), wna = vna;
    if (a >= 0 && sb.has_restitution) {
        vna = f3(sb.vn4[2 * a]);
        wna = f3(sb.vn4[2 * a + 1]);
    }
    const float4 mb = sb.mat4[b];
    float mu = combine_mu32(P.combine, mu_a, mb.x);
    if (!P.friction_enable || !(mu > 0.f)) mu = 0.f;
    float3 t1, t2;
    frame32(n, t1, t2);
    // static-side contact velocity: row . [v_wall, w_wall] with sign -1 (dynamics_assembler.cpp:281-285)
    float cb[3] = {0.f, 0.f, 0.f};
    if (a < 0 && wall_v) {
        const float3 rA = pt - *wall_p;
        const float3 vw = *wall_v + crossf(*wall_w, rA);
        cb[0] = -dot(n, vw);
        cb[1] = -dot(t1, vw);
        cb[2] = -dot(t2, vw);
    }
    const float eN = fminf(fmaxf(0.f, rn_a), fmaxf(0.f, mb.y));
    const float eT = fminf(fmaxf(0.f, rt_a), fmaxf(0.f, mb.z));
    float4 bias = make_float4(cb[0], cb[1], cb[2], 0.f);
    if (eN > 0.f || eT > 0.f) {
        const float3 dv = f3(sb.vn4[2 * b]) - vna;
        const float3 Om = rhoB * f3(sb.vn4[2 * b + 1]) - rhoA * wna;
        const float vp0 = dot(n, dv) + cb[0];
        const float vp1 = dot(t1, dv) + dot(t2, Om) + cb[1];
        const float vp2 = dot(t2, dv) - dot(t1, Om) + cb[2];
        bias = make_float4(cb[0] + eN * vp0, cb[1] + eT * vp1, cb[2] + eT * vp2, 0.f);
    }
    const uint32_t ida = a >= 0 ? (uint32_t)(sc.S + a) : (uint32_t)(-a - 1);
    const uint32_t idb = (uint32_t)(sc.S + b);
    const unsigned long long key = ((unsigned long long)ida << 32) | idb;
    float4 lam0 = make_float4(0.f, 0.f, 0.f, 0.f);
    if ((P.prev_count >= 0 ? P.prev_count : sb.ss->prev_count_dev) > 0)
        warm_start(sb, gen, prev_lo, prev_hi, key, pt, P.match2, lam0);
    if (mu == 0.f) { lam0.y = 0.f; lam0.z = 0.f; }
    const bool has_bias = bias.x != 0.f || bias.y != 0.f || bias.z != 0.f;
    sb.rec0[c] = make_float4(n.x, n.y, n.z, has_bias ? -mu - 0.f : mu);
    sb.rec1[c] = make_float4(rhoA, rhoB, __int_as_float(a), __int_as_float(b));
    if (has_bias) sb.bias[c] = bias;
    sb.lam[gen][c] = lam0;
    sb.key[gen][c] = key;
    sb.pt[gen][c] = make_float4(pt.x, pt.y, pt.z, 0.f);
}

__global__ void k_s_static_write(Scene sc, SplitBuf sb, const int32_t* flags, const int32_t* pos, int gen,
                                 SplitParams P) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sc.N) return;
    const int s = sc.body_scene[i];
    const int b0 = sc.scene_body_start[s], ns_b = sc.scene_body_start[s + 1] - b0;
    const int st0 = sc.scene_static_start[s], nst = sc.scene_static_start[s + 1] - st0;
    const float4 p = sb.pos4[i];
    const int L = sc.max_statics;
    for (int l = 0; l < nst && l < L; ++l) {
        const size_t slot = (size_t)b0 * L + (size_t)l * ns_b + (i - b0);
        if (!flags[slot]) continue;
        const int st = st0 + l;
        CGeom32 g;
        static_test32(sb, st, f3(p), p.w, INFINITY, g);  // the flag decided membership; this fills the geometry
        const float3 pt = f3(p) + g.rhoB * g.n;
        const float3 wv = f3(sb.st_v[st]), ww = f3(sb.st_w[st]), wp = f3(sb.st_pt[st]);
        const bool moving = (wv.x != 0.f || wv.y != 0.f || wv.z != 0.f || ww.x != 0.f || ww.y != 0.f || ww.z != 0.f);
        int plo = 0, phi = 0;
        if ((P.prev_count >= 0 ? P.prev_count : sb.ss->prev_count_dev) > 0 && P.prev_sflags[slot]) {
            plo = P.prev_spos[slot];
            phi = plo + 1;
        }
        finish_contact32(sc, sb, gen, pos[slot], -st - 1, i, g.n, 0.f, g.rhoB, pt, sb.st_w[st].w,
                         (float)sc.sf(SF_RN)[st], (float)sc.sf(SF_RT)[st], moving ? &wv : nullptr, &ww, &wp, P, plo,
                         phi);
    }
}

// Six blocks of 256 an SM (at most 42 registers a thread): the 200k pile's 1,316 spheres an SM
// then run in one wave; the FP64 test near the threshold had pushed the count pass to 54
// registers and two waves (+70 us a step).
template <bool WRITE>
__global__ void __launch_bounds__(256, 6) k_s_pairs(Scene sc, Grid gr, SplitBuf sb, const uint32_t* cell_body, const uint32_t* cell_key,
                          const int32_t* cell_start, const int32_t* cell_end, int32_t* counts, const int32_t* offsets,
                          int32_t base, int gen, SplitParams P, DevScalars* ds) {
    // threads take the bodies in cell order, so a warp walks neighbouring cells (shared cache
    // lines); every body's contacts still go to its own slots (counts[i], offsets[i])
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= sc.N) return;
    const int i = (int)cell_body[t];
    const float4 pi = sb.pos4[i];
    const int si = sc.body_scene[i];
    // cell of body i: its key in the sorted key array, ((z dim_y) + y) dim_x + x
    int ci[3];
    {
        const uint32_t key = cell_key[t];
        const uint32_t dx = (uint32_t)gr.dim[0], dy = (uint32_t)gr.dim[1];
        ci[0] = (int)(key % dx);
        ci[1] = (int)((key / dx) % dy);
        ci[2] = (int)(key / (dx * dy));
    }
    int list[MAX_PAIR];
    int cnt = 0;
    // the write pass takes the partners the count pass kept when they all fitted; the count comes
    // from the offsets it was scanned into (the same walk, the same test, so the same partners)
    bool walk = true;
    if (WRITE) {
        const int kept = offsets[i + 1] - offsets[i];
        if (kept <= SPLIT_PLIST) {
            for (int k = 0; k < kept; ++k) list[k] = sb.plist[(size_t)i * SPLIT_PLIST + k];
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
            const int64_t row = ((int64_t)z * gr.dim[1] + y) * gr.dim[0];
            const int x0 = max(ci[0] - 1, 0), x1 = min(ci[0] + 1, gr.dim[0] - 1);
            // cells x0..x1 of one row are contiguous in the sorted body list
            const int pb = cell_start[row + x0];
            int pe = cell_end[row + x0];
            for (int x = x0 + 1; x <= x1; ++x) {
                const int e = cell_end[row + x];
                if (e > pe) pe = e;
            }
            int p0 = pb;
            for (int x = x0; x <= x1; ++x) {
                const int st = cell_start[row + x], e = cell_end[row + x];
                if (e > st) { p0 = st; break; }
            }
            for (int p = p0; p < pe; ++p) {
                const int j = (int)cell_body[p];
                if (j <= i) continue;
                const float4 pj = sb.pos4[j];
                const float dx = pj.x - pi.x, dy2 = pj.y - pi.y, dz2 = pj.z - pi.z;
                const float d2 = dx * dx + dy2 * dy2 + dz2 * dz2;
                const float lim = pi.w + pj.w + P.margin;
                const float band = band32(f3(pi), f3(pj)) + 3e-7f * lim;
                const float hi = lim + band;
                if (d2 > hi * hi) continue;
                if (sc.body_scene[j] != si) continue;
                const float lo = lim - band;
                if (!(lo > 0.f && d2 <= lo * lo)) {
                    // the band: coordinates and radii with what FP32 rounded off added back (the hi
                    // differences of nearby values are exact or off by half an ulp of |d|), which
                    // narrows the band to a few 1e-8 of the lengths compared; inside that, FP64
                    const float4 li = sb.pos4lo[i], lj = sb.pos4lo[j];
                    const float ex = (pj.x - pi.x) + (lj.x - li.x), ey = (pj.y - pi.y) + (lj.y - li.y);
                    const float ez = (pj.z - pi.z) + (lj.z - li.z);
                    const float e2 = ex * ex + ey * ey + ez * ez;
                    const float L = (pi.w + pj.w) + ((li.w + lj.w) + P.margin);
                    const float fb = 5e-8f + 3e-7f * L;
                    if (e2 > (L + fb) * (L + fb)) continue;
                    if (!(L - fb > 0.f && e2 <= (L - fb) * (L - fb)) && !pair_member64(sb, i, j, P.margin64)) continue;
                }
                if (WRITE) {
                    if (cnt < MAX_PAIR) list[cnt] = j;
                } else if (cnt < SPLIT_PLIST) {
                    sb.plist[(size_t)i * SPLIT_PLIST + cnt] = j;
                }
                ++cnt;
            }
        }
    }
    if (!WRITE) {
        counts[i] = cnt;
        if (cnt > MAX_PAIR) atomicExch(&ds->overflow, 1);
        return;
    }
    if (cnt > MAX_PAIR) cnt = MAX_PAIR;
    for (int a = 1; a < cnt; ++a) {
        const int v = list[a];
        int b = a - 1;
        while (b >= 0 && list[b] > v) {
            list[b + 1] = list[b];
            --b;
        }
        list[b + 1] = v;
    }
    const int c0 = (base >= 0 ? base : sb.ss->n_static) + offsets[i];
    int plo = 0, phi = 0;
    if ((P.prev_count >= 0 ? P.prev_count : sb.ss->prev_count_dev) > 0) {
        const int pns = P.prev_count >= 0 ? P.prev_n_static : sb.ss->prev_n_static_dev;
        plo = pns + P.prev_poff[i];
        phi = pns + P.prev_poff[i + 1];
    }
    const float4 ma = sb.mat4[i];
    const float mu_a = ma.x, rn_a = ma.y, rt_a = ma.z;
    for (int k = 0; k < cnt; ++k) {
        const int j = list[k];
        const float4 pj = sb.pos4[j];
        const float3 d = f3(pj) - f3(pi);
        const float dl = sqrtf(dot(d, d));
        const float3 n = dl > 0.f ? __frcp_rn(dl) * d : make_float3(0.f, 0.f, 1.f);
        const float rhoA = 0.5f * (dl + pi.w - pj.w);
        const float rhoB = 0.5f * (pi.w - pj.w - dl);
        const float3 pt = f3(pi) + rhoA * n;
        finish_contact32(sc, sb, gen, c0 + k, i, j, n, rhoA, rhoB, pt, mu_a, rn_a, rt_a, nullptr, nullptr, nullptr, P,
                         plo, phi);
    }
}

// ------------------------------------------------------------------ projected Jacobi (FP32)
// apply W^T dl (pre-scaled by M^-1) to the bodies of contact c with float4/float2 vector atomics
__device__ __forceinline__ void scatter(float4* acc, int a, int b, float3 n, float3 t1, float3 t2, float rhoA,
                                        float rhoB, float dln, float dlt1, float dlt2, float imb, float iib, float ima,
                                        float iia) {
    // accumulator layout = velocity layout: (v.xyz, 1/m), (omega.xyz, 1/I); the .w lanes get +0
    const float3 P = dln * n + dlt1 * t1 + dlt2 * t2;
    const float3 tau = dlt1 * t2 - dlt2 * t1;
    {
        const float s = rhoB * iib;
        atomicAdd(&acc[2 * b], make_float4(imb * P.x, imb * P.y, imb * P.z, 0.f));
        atomicAdd(&acc[2 * b + 1], make_float4(s * tau.x, s * tau.y, s * tau.z, 0.f));
    }
    if (a >= 0) {
        const float s = -rhoA * iia;
        atomicAdd(&acc[2 * a], make_float4(-ima * P.x, -ima * P.y, -ima * P.z, 0.f));
        atomicAdd(&acc[2 * a + 1], make_float4(s * tau.x, s * tau.y, s * tau.z, 0.f));
    }
}

__global__ void k_s_apply_warm(SplitBuf sb, int gen) {
    const int nc = *sb.nc_dev;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
        const float4 l = sb.lam[gen][c];
        if (l.x == 0.f && l.y == 0.f && l.z == 0.f) continue;
        const float4 r0 = sb.rec0[c], r1 = sb.rec1[c];
        const int a = __float_as_int(r1.z), b = __float_as_int(r1.w);
        const float3 n = f3(r0);
        float3 t1, t2;
        frame32(n, t1, t2);
        const float imb = sb.vel4[2 * b].w, iib = sb.vel4[2 * b + 1].w;
        float ima = 0.f, iia = 0.f;
        if (a >= 0) {
            ima = sb.vel4[2 * a].w;
            iia = sb.vel4[2 * a + 1].w;
        }
        scatter(sb.acc[0], a, b, n, t1, t2, r1.x, r1.y, l.x, l.y, l.z, imb, iib, ima, iia);
    }
}

// One projected Jacobi sweep, one kernel. PJ keeps x_k = x_free + M^-1 W^T lambda_k
// (projected_jacobi.cpp:361-363, 134-137), so four rotating velocity buffers replace the body
// pass: the sweep reads the body velocities x_k from A_k, computes lambda_{k+1} for every contact
// and adds the full M^-1 W^T lambda_{k+1} into A_{k+1} (float4 vector atomics), which holds x_free;
// A_{k-1}, read by the previous sweep, is reset to x_free for sweep k + 2 to add into. There is no
// separate body pass and no FP32 accumulation across sweeps. The sweep is latency-bound (contact record -> body gathers -> atomics): each thread takes
// UNROLL contacts and issues all record loads, then all gathers, before computing; read-only data
// goes through the non-coherent path; the grid is a whole number of resident waves. The last block
// to finish (completion counter, no waiting) reduces the per-block maxima and runs the stop rule.
__device__ __forceinline__ float4 ldg4(const float4* p) { return __ldg(p); }

// stop rule after a sweep: iteration cap, complementarity residual of the iterate entering the
// sweep (max_c ||dlambda_c|| / max |lambda|; the sweep reduces squared norms, sqrt is monotone),
// or a non-finite value
__device__ __forceinline__ float sweep_residual(float maxd2, float maxl) { return sqrtf(maxd2) / fmaxf(maxl, 1e-30f); }
__device__ __forceinline__ void sweep_check(SplitScalars* ss, float maxd2, float maxl, int max_iter, float tol,
                                            cudaGraphConditionalHandle handle, int use_handle) {
    if (!ss->done) {
        const float r = sweep_residual(maxd2, maxl);
        ss->res_last = r;
        ss->iters += 1;
        if (ss->iters >= max_iter || (tol > 0.f && r <= tol) || !(r == r)) ss->done = 1;
    }
    if (use_handle) cudaGraphSetConditional(handle, ss->done ? 0u : 1u);
}

// float4 reduction without a return value (the sweep never reads what it adds)
__device__ __forceinline__ void red4(float4* p, float x, float y, float z) {
    asm volatile("red.relaxed.gpu.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(p), "f"(x), "f"(y), "f"(z),
                 "f"(0.f)
                 : "memory");
}

// Sums v over each run of equal keys among the lanes of a warp; the first lane of a run gets the
// run's total. Pair contacts are stored grouped by their first body, so neighbouring lanes often
// push to the same body: one reduction per run replaces a chain of same-address atomics.
__device__ __forceinline__ bool warp_run_sum(int key, float (&v)[6]) {
    const unsigned FULL = 0xffffffffu;
    const unsigned lane = threadIdx.x & 31u;
    const int pk = __shfl_up_sync(FULL, key, 1);
    const bool head = lane == 0u || pk != key;
    const unsigned heads = __ballot_sync(FULL, head);
    if (heads != FULL) {
        const unsigned above = heads & ~((2u << lane) - 1u);
        const unsigned end = above ? (unsigned)(__ffs(above) - 1) : 32u;
        for (unsigned off = 1; off < 32u; off <<= 1) {
            const bool take = lane + off < end;
            if (!__any_sync(FULL, take)) break;
#pragma unroll
            for (int q = 0; q < 6; ++q) {
                const float t = __shfl_down_sync(FULL, v[q], off);
                if (take) v[q] += t;
            }
        }
    }
    return head;
}

// Result of the projected Jacobi update of one contact.
struct PJOut {
    float4 lam;      // new impulse (normal, t1, t2, 0)
    float3 pb, tb;   // M^-1 W^T lambda on body B: linear, angular (world frame)
    float3 pa, ta;   // the same for body A (zero for a static)
    float dn2, lm;   // ||lambda_new - lambda_old||^2, max |lambda_old|
    bool push;       // lambda_new != 0
};

// R = alpha / Delassus diagonal (projected_jacobi.cpp:57-69) from the inverse masses and the
// signed lever lengths: D_n = 1/m_A + 1/m_B, D_t = D_n + rho_A^2 / I_A + rho_B^2 / I_B
__device__ __forceinline__ void pj_rdiag(float rA, float rB, float ima, float iia, float imb, float iib, float alpha,
                                         float& Rn, float& Rt) {
    const float Dn = ima + imb;
    const float Dt = Dn + rA * rA * iia + rB * rB * iib;
    Rn = __fdividef(alpha, Dn);  // the inverse masses keep Dn, Dt far inside __fdividef's range
    Rt = __fdividef(alpha, Dt);
}

// One contact of a sweep (projected_jacobi.cpp:121-138 with project :100-119): gamma = W x + b from
// the accumulated velocities of both bodies, lambda <- Pi(lambda - R gamma), and the body shares of
// M^-1 W^T lambda (the full impulse: the accumulator being filled starts at x_free).
__device__ __forceinline__ void pj_core(float3 n, float3 t1, float3 t2, float rA, float rB, float muw, float4 l,
                                        float4 va, float4 wa, float4 vb, float4 wb, const float4* bias_c, float Rn,
                                        float Rt, PJOut& o) {
    const float3 dv = f3(vb) - f3(va);
    const float3 Om = rB * f3(wb) - rA * f3(wa);
    float gn = dot(n, dv);
    float gt1 = dot(t1, dv) + dot(t2, Om);
    float gt2 = dot(t2, dv) - dot(t1, Om);
    if (split_has_bias(muw)) {
        const float4 bs = ldg4(bias_c);
        gn += bs.x;
        gt1 += bs.y;
        gt2 += bs.z;
    }
    const float mu = fabsf(muw);
    float ln = fmaxf(l.x - Rn * gn, 0.f);
    float lt1 = l.y - Rt * gt1;
    float lt2 = l.z - Rt * gt2;
    const float tn2 = lt1 * lt1 + lt2 * lt2;
    if (tn2 > 0.f) {
        const float sc = fminf(1.f, mu * ln * rsqrtf(tn2));
        lt1 *= sc;
        lt2 *= sc;
    }
    const float dln = ln - l.x, dlt1 = lt1 - l.y, dlt2 = lt2 - l.z;
    o.lam = make_float4(ln, lt1, lt2, 0.f);
    o.dn2 = dln * dln + dlt1 * dlt1 + dlt2 * dlt2;
    o.lm = fmaxf(fabsf(l.x), fmaxf(fabsf(l.y), fabsf(l.z)));
    o.push = ln != 0.f || lt1 != 0.f || lt2 != 0.f;
    // accumulator layout = velocity layout: (v.xyz, 1/m), (omega.xyz, 1/I); the .w lanes get +0
    const float3 P = ln * n + lt1 * t1 + lt2 * t2;
    const float3 tau = lt1 * t2 - lt2 * t1;
    o.pb = vb.w * P;
    o.tb = (rB * wb.w) * tau;
    o.pa = (-va.w) * P;
    o.ta = (-rA * wa.w) * tau;
}

// The same from the packed records alone: frame and R recomputed (the inverse masses ride in the
// .w lanes of the gathered velocities)
__device__ __forceinline__ void pj_contact(float4 r0, float4 r1, float4 l, float4 va, float4 wa, float4 vb, float4 wb,
                                           const float4* bias_c, float alpha, PJOut& o) {
    const float3 n = f3(r0);
    float3 t1, t2;
    frame32(n, t1, t2);
    float Rn, Rt;
    pj_rdiag(r1.x, r1.y, va.w, wa.w, vb.w, wb.w, alpha, Rn, Rt);
    pj_core(n, t1, t2, r1.x, r1.y, r0.w, l, va, wa, vb, wb, bias_c, Rn, Rt, o);
}

// Adds a contact's shares into accumulator A. Every lane of the warp calls it (AGG 2 reduces across
// the warp). AGG: 0 float4 atomicAdd, 1 float4 reductions (no return value), 2 reductions with
// body A's share summed per run of equal body index. All three add the same terms; only the FP32
// summation order differs.
template <int AGG>
__device__ __forceinline__ void pj_push(float4* A, bool ok, int a, int b, const PJOut& o) {
    const bool go = ok && o.push;
    if (AGG == 0) {
        if (go) {
            atomicAdd(&A[2 * b], make_float4(o.pb.x, o.pb.y, o.pb.z, 0.f));
            atomicAdd(&A[2 * b + 1], make_float4(o.tb.x, o.tb.y, o.tb.z, 0.f));
            if (a >= 0) {
                atomicAdd(&A[2 * a], make_float4(o.pa.x, o.pa.y, o.pa.z, 0.f));
                atomicAdd(&A[2 * a + 1], make_float4(o.ta.x, o.ta.y, o.ta.z, 0.f));
            }
        }
    } else if (AGG == 1) {
        if (go) {
            red4(&A[2 * b], o.pb.x, o.pb.y, o.pb.z);
            red4(&A[2 * b + 1], o.tb.x, o.tb.y, o.tb.z);
            if (a >= 0) {
                red4(&A[2 * a], o.pa.x, o.pa.y, o.pa.z);
                red4(&A[2 * a + 1], o.ta.x, o.ta.y, o.ta.z);
            }
        }
    } else {
        if (go) {
            red4(&A[2 * b], o.pb.x, o.pb.y, o.pb.z);
            red4(&A[2 * b + 1], o.tb.x, o.tb.y, o.tb.z);
        }
        // lanes with nothing to add keep their key so a run stays contiguous; they add zeros
        const int key = ok ? a : -1;
        float v[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        if (go && a >= 0) {
            v[0] = o.pa.x;
            v[1] = o.pa.y;
            v[2] = o.pa.z;
            v[3] = o.ta.x;
            v[4] = o.ta.y;
            v[5] = o.ta.z;
        }
        const bool head = warp_run_sum(key, v);
        if (head && key >= 0 && (v[0] != 0.f || v[1] != 0.f || v[2] != 0.f || v[3] != 0.f || v[4] != 0.f || v[5] != 0.f)) {
            red4(&A[2 * key], v[0], v[1], v[2]);
            red4(&A[2 * key + 1], v[3], v[4], v[5]);
        }
    }
}

// One projected Jacobi sweep per launch (streaming form: contact records read from HBM/L2 every
// sweep).
template <int UNROLL, int NTH, int MINB, int AGG>
__global__ void __launch_bounds__(NTH, MINB) k_s_sweep_t(SplitBuf sb, int gen, float alpha, int max_iter, float tol,
                                                         cudaGraphConditionalHandle handle, int use_handle) {
    if (*(volatile int32_t*)&sb.ss->done) {
        // the loop is over: make sure the while node sees it even if no check runs this time
        if (use_handle && blockIdx.x == 0 && threadIdx.x == 0) cudaGraphSetConditional(handle, 0u);
        return;
    }
    const int k = sb.ss->iters;
    const float4* __restrict__ Acur = sb.acc[k % SPLIT_NACC];
    float4* Anxt = sb.acc[(k + 1) % SPLIT_NACC];
    float4* Aclr = sb.acc[(k + 3) % SPLIT_NACC];
    const int nc = *sb.nc_dev;
    float maxd = 0.f, maxl = 0.f;
    const int T = gridDim.x * blockDim.x;
    float4* __restrict__ lamp = sb.lam[gen];
    // the loop bound is the same for all lanes of a warp (the run reduction needs whole warps)
    const int lane = threadIdx.x & 31;
    for (int w0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31); w0 < nc; w0 += T * UNROLL) {
        const int c0 = w0 + lane;
        float4 r0[UNROLL], r1[UNROLL], l[UNROLL];
        bool ok[UNROLL];
#pragma unroll
        for (int u = 0; u < UNROLL; ++u) {
            const int c = c0 + u * T;
            ok[u] = c < nc;
            if (ok[u]) {
                r0[u] = ldg4(&sb.rec0[c]);
                r1[u] = ldg4(&sb.rec1[c]);
                l[u] = lamp[c];
            }
        }
        float4 vb[UNROLL], wb[UNROLL], va[UNROLL], wa[UNROLL];
#pragma unroll
        for (int u = 0; u < UNROLL; ++u) {
            if (!ok[u]) continue;
            const int a = __float_as_int(r1[u].z), b = __float_as_int(r1[u].w);
            vb[u] = ldg4(&Acur[2 * b]);
            wb[u] = ldg4(&Acur[2 * b + 1]);
            if (a >= 0) {
                va[u] = ldg4(&Acur[2 * a]);
                wa[u] = ldg4(&Acur[2 * a + 1]);
            } else {
                va[u] = make_float4(0.f, 0.f, 0.f, 0.f);
                wa[u] = va[u];
            }
        }
#pragma unroll
        for (int u = 0; u < UNROLL; ++u) {
            PJOut o = {};
            int a = -1, b = 0;
            if (ok[u]) {
                const int c = c0 + u * T;
                a = __float_as_int(r1[u].z);
                b = __float_as_int(r1[u].w);
                pj_contact(r0[u], r1[u], l[u], va[u], wa[u], vb[u], wb[u], &sb.bias[c], alpha, o);
                lamp[c] = o.lam;
                maxd = fmaxf(maxd, o.dn2);
                maxl = fmaxf(maxl, o.lm);
            }
            pj_push<AGG>(Anxt, ok[u], a, b, o);
        }
    }
    // reset the accumulator of the sweep after next to the free velocities
    const int N = sb.N;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += T) {
        const float4 v0 = ldg4(&sb.vel4[2 * i]), w0 = ldg4(&sb.vel4[2 * i + 1]);
        Aclr[2 * i] = v0;
        Aclr[2 * i + 1] = w0;
    }
    block_max2(maxd, maxl);
    __shared__ bool last;
    if (threadIdx.x == 0) {
        sb.part[blockIdx.x] = make_float2(maxd, maxl);
        __threadfence();
        last = atomicAdd(&sb.ss->blocks_done, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    float md = 0.f, ml = 0.f;
    for (int p = threadIdx.x; p < (int)gridDim.x; p += blockDim.x) {
        const volatile float* q = reinterpret_cast<volatile float*>(&sb.part[p]);
        md = fmaxf(md, q[0]);
        ml = fmaxf(ml, q[1]);
    }
    block_max2(md, ml);
    if (threadIdx.x == 0) {
        sb.ss->blocks_done = 0u;
        sweep_check(sb.ss, md, ml, max_iter, tol, handle, use_handle);
    }
}

// ---- cooperative whole solve
// one body's (v, 1/m), (omega, 1/I) pair as a single 32-byte load through L2: one sector request
// instead of two (the accumulators change inside the cooperative launch, so they bypass L1)
__device__ __forceinline__ void ldcg_body(const float4* p, float4& v, float4& w) {
    asm volatile("ld.global.cg.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w), "=f"(w.x), "=f"(w.y), "=f"(w.z), "=f"(w.w)
                 : "l"(p)
                 : "memory");
}
__device__ __forceinline__ void stcg_body(float4* p, float4 v, float4 w) {
    asm volatile("st.global.cg.v8.f32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"l"(p), "f"(v.x), "f"(v.y), "f"(v.z),
                 "f"(v.w), "f"(w.x), "f"(w.y), "f"(w.z), "f"(w.w)
                 : "memory");
}

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Grid barrier of a cooperative launch (all blocks resident) that also reduces the per-sweep maxima,
// in two halves (grid_arrive, grid_wait_max) so a block can do independent work in between.
// Block g writes (max ||dlambda||, max |lambda|) into its own record, then thread 0 adds one to the
// arrival counter and waits until it reaches the barrier's target (epoch x blocks). After the
// barrier warp 0 reads every block's record (independent loads, one round trip) and takes the
// maxima, so all blocks see the same numbers. Records alternate between two banks by epoch parity:
// a block can run one barrier ahead of a slow reader, never two. The wait is bounded: after
// COOP_WAIT_NS, or once another block has given up, the block sets *err and returns false.
constexpr unsigned long long COOP_WAIT_NS = 200000000ull;  // 0.2 s
constexpr int COOP_MAX_GRID = 320;                         // records a lane reads: COOP_MAX_GRID / 32
// Arrival half: publish the block's maxima and add one to the counter (after every thread's
// writes of the sweep, through __syncthreads and a release reduction).
__device__ __forceinline__ void grid_arrive(unsigned* ctr, float2* recs, unsigned epoch, bool reduce, float maxd,
                                            float maxl) {
    float2* bank = recs + (size_t)(epoch & 1u) * SPLIT_MAX_PARTS;
    if (reduce && threadIdx.x == 0) bank[blockIdx.x] = make_float2(maxd, maxl);
    __syncthreads();
    // a release reduction: the block's writes (ordered before it by __syncthreads) become
    // visible to any block whose acquire load sees the new count
    if (threadIdx.x == 0) asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(ctr) : "memory");
}
// Waiting half: thread 0 waits (bounded, acquire loads) for every block's arrival, then warp 0
// reduces the records.
__device__ __forceinline__ bool grid_wait_max(unsigned* ctr, float2* recs, unsigned epoch, unsigned base, int32_t* err,
                                              bool reduce, float& maxd, float& maxl, unsigned long long wait_ns) {
    __shared__ float s_md, s_ml;
    __shared__ int s_ok;
    float2* bank = recs + (size_t)(epoch & 1u) * SPLIT_MAX_PARTS;
    if (threadIdx.x < 32) {
        const unsigned FULL = 0xffffffffu;
        int ok = 1;
        if (threadIdx.x == 0) {
            const unsigned target = base + epoch * gridDim.x;
            const unsigned long long t0 = global_ns();
            while ((int)(ld_acquire(ctr) - target) < 0) {
                if (ld_acquire(reinterpret_cast<const unsigned*>(err)) != 0u || global_ns() - t0 > wait_ns) {
                    atomicExch(err, 1);
                    ok = 0;
                    break;
                }
                __nanosleep(20);
            }
        }
        ok = __shfl_sync(FULL, ok, 0);
        float md = 0.f, ml = 0.f;
        if (ok && reduce) {
            float2 v[COOP_MAX_GRID / 32];
#pragma unroll
            for (int k = 0; k < COOP_MAX_GRID / 32; ++k) {
                const int p = threadIdx.x + 32 * k;
                v[k] = p < (int)gridDim.x ? __ldcg(&bank[p]) : make_float2(0.f, 0.f);
            }
#pragma unroll
            for (int k = 0; k < COOP_MAX_GRID / 32; ++k) {
                md = fmaxf(md, v[k].x);
                ml = fmaxf(ml, v[k].y);
            }
            for (int o = 16; o > 0; o >>= 1) {
                md = fmaxf(md, __shfl_xor_sync(FULL, md, o));
                ml = fmaxf(ml, __shfl_xor_sync(FULL, ml, o));
            }
        }
        if (threadIdx.x == 0) {
            s_md = md;
            s_ml = ml;
            s_ok = ok;
        }
    }
    __syncthreads();
    maxd = s_md;
    maxl = s_ml;
    return s_ok != 0;
}

// The whole projected Jacobi solve (up to max_sweeps sweeps) in one cooperative launch. Block g
// owns contacts [g*cpb, (g+1)*cpb) and bodies [g*bpb, (g+1)*bpb). It loads its contact records and
// impulses into shared memory once (48 B a contact) and keeps them there across sweeps; the frame
// and R are recomputed each sweep (keeping t1 and R in shared memory as well measured slower: they
// crowd the free velocities out and lengthen the chain after the gathers). Each sweep then touches
// L2/HBM only for the body velocities (gathers from A_k, reductions into A_{k+1}, the reset of A_{k-1}
// from the free velocities, which also sit in shared memory when they fit). Sweeps are separated by
// a split grid barrier that also gathers the per-sweep maxima, so every block evaluates the same
// stop rule on the same numbers: a block arrives once its reductions are issued, resets A_{k-1}
// while the others arrive, then waits. A_{k-1} is safe to reset there: every block finished sweep
// k - 1 (its last reader) before this barrier's previous one let anybody through, and the first
// sweep to add into it again (k + 2) starts only after this block arrives at the next barrier.
// Block 0 records the iteration count for the host.
// HYB: a block's range may hold more contacts than its shared memory (cpb); the first cpb stay in
// shared memory and the rest are read from memory every sweep (records through the read-only
// path, impulses through L2), so problems of any size run as one launch.
// MINB > 1: that many blocks an SM (more threads an SM at fewer registers a thread, so a settled
// pile's ~3,100 contacts an SM take three passes instead of four)
template <int NTH, int UNROLL, int AGG, int HYB, int MINB = 1>
__global__ void __launch_bounds__(NTH, MINB) k_s_solve_coop(SplitBuf sb, int gen, float alpha, int max_iter, float tol,
                                                         int cpb, int bpb, int vf_smem, int max_sweeps,
                                                         int check_every, unsigned long long wait_ns) {
    extern __shared__ float4 smem[];
    SplitScalars* ss = sb.ss;
    if (*(volatile int32_t*)&ss->done) return;
    float4* s_q0 = smem;            // (n, mu with the bias flag)
    float4* s_q1 = smem + cpb;      // (rho_A, rho_B, A, B)
    float4* s_l = smem + 2 * cpb;   // lambda
    float4* s_vf = smem + 3 * cpb;  // free velocities of the block's bodies
    const int it0 = *(volatile int32_t*)&ss->iters;
    unsigned epoch = *(volatile unsigned*)&ss->bar_base;
    // arrivals so far this step: the launches before this one may have had other grid sizes (the
    // autotuner's trials), so the counter's target is counted from them (modulo 2^32)
    const unsigned bbase = *(volatile unsigned*)&ss->bar_arr - epoch * gridDim.x;
    const int nc = *sb.nc_dev, N = sb.N, tid = threadIdx.x;
    if (!HYB && (int64_t)nc > (int64_t)cpb * gridDim.x) {
        // planned from an estimate of the contact count that fell short: every block returns (no
        // barrier has been entered) and the host redoes the step with a plan from the true count
        if (blockIdx.x == 0 && tid == 0) ss->err = 4;
        return;
    }
    // contacts split evenly by the true count (cpb, planned from an estimate, sizes the arrays)
    const int cpe = (nc + (int)gridDim.x - 1) / (int)gridDim.x;
    const int cb = blockIdx.x * cpe;
    const int ncb = max(0, min(nc - cb, cpe));
    const int bb = blockIdx.x * bpb;
    const int nbb = max(0, min(N - bb, bpb));
    const int ncs = HYB ? min(ncb, cpb) : ncb;  // contacts kept in shared memory
    float4* __restrict__ lamg = sb.lam[gen];
    for (int i = tid; i < ncs; i += NTH) {
        const float4 r0 = ldg4(&sb.rec0[cb + i]), r1 = ldg4(&sb.rec1[cb + i]), l = lamg[cb + i];
        s_q0[i] = r0;
        s_q1[i] = r1;
        s_l[i] = l;
    }
    if (vf_smem)
        for (int i = tid; i < 2 * nbb; i += NTH) s_vf[i] = ldg4(&sb.vel4[2 * bb + i]);
    __syncthreads();
    int it = it0, stop = 0;
    float r = 0.f;
    for (int j = 0; j < max_sweeps; ++j) {
        // the accumulators change inside this launch: read them through L2 (ld.global.cg)
        const float4* Acur = sb.acc[it % SPLIT_NACC];
        float4* Anxt = sb.acc[(it + 1) % SPLIT_NACC];
        float4* Aclr = sb.acc[(it + 3) % SPLIT_NACC];
        float maxd2 = 0.f, maxl = 0.f;
        for (int base = 0; base < ncb; base += NTH * UNROLL) {
            float4 q0[UNROLL], q1[UNROLL], l[UNROLL];
            bool ok[UNROLL];
#pragma unroll
            for (int u = 0; u < UNROLL; ++u) {
                const int i = base + u * NTH + tid;
                ok[u] = i < ncb;
                if (ok[u]) {
                    if (!HYB || i < ncs) {
                        q0[u] = s_q0[i];
                        q1[u] = s_q1[i];
                        l[u] = s_l[i];
                    } else {
                        q0[u] = ldg4(&sb.rec0[cb + i]);
                        q1[u] = ldg4(&sb.rec1[cb + i]);
                        l[u] = __ldcg(&lamg[cb + i]);
                    }
                }
            }
            float4 vb[UNROLL], wb[UNROLL], va[UNROLL], wa[UNROLL];
#pragma unroll
            for (int u = 0; u < UNROLL; ++u) {
                if (!ok[u]) continue;
                const int a = __float_as_int(q1[u].z), b = __float_as_int(q1[u].w);
                ldcg_body(&Acur[2 * b], vb[u], wb[u]);
                if (a >= 0) {
                    ldcg_body(&Acur[2 * a], va[u], wa[u]);
                } else {
                    va[u] = make_float4(0.f, 0.f, 0.f, 0.f);
                    wa[u] = va[u];
                }
            }
#pragma unroll
            for (int u = 0; u < UNROLL; ++u) {
                PJOut o = {};
                int a = -1, b = 0;
                if (ok[u]) {
                    const int i = base + u * NTH + tid;
                    a = __float_as_int(q1[u].z);
                    b = __float_as_int(q1[u].w);
                    pj_contact(q0[u], q1[u], l[u], va[u], wa[u], vb[u], wb[u], &sb.bias[cb + i], alpha, o);
                    if (!HYB || i < ncs)
                        s_l[i] = o.lam;
                    else
                        __stcg(&lamg[cb + i], o.lam);
                    maxd2 = fmaxf(maxd2, o.dn2);
                    maxl = fmaxf(maxl, o.lm);
                }
                pj_push<AGG>(Anxt, ok[u], a, b, o);
            }
        }
        // the stop rule runs every check_every sweeps (counted across launches) and at the cap; the
        // other sweeps only synchronise
        const bool check = (it + 1) % check_every == 0 || it + 1 >= max_iter;
        if (check) block_max2(maxd2, maxl);
        grid_arrive(&ss->bar, sb.recs, ++epoch, check, maxd2, maxl);
        for (int i = tid; i < nbb; i += NTH) {
            const float4 v0 = vf_smem ? s_vf[2 * i] : ldg4(&sb.vel4[2 * (bb + i)]);
            const float4 w0 = vf_smem ? s_vf[2 * i + 1] : ldg4(&sb.vel4[2 * (bb + i) + 1]);
            stcg_body(&Aclr[2 * (bb + i)], v0, w0);
        }
        if (!grid_wait_max(&ss->bar, sb.recs, epoch, bbase, &ss->err, check, maxd2, maxl, wait_ns)) return;
        ++it;
        if (check) {
            r = sweep_residual(maxd2, maxl);
            if (it >= max_iter || (tol > 0.f && r <= tol) || !(r == r)) {
                stop = 1;
                break;
            }
        }
    }
    for (int i = tid; i < ncs; i += NTH) lamg[cb + i] = s_l[i];
    // every block has read the scalars by now (it passed a barrier with all of them)
    if (blockIdx.x == 0 && tid == 0) {
        ss->iters = it;
        ss->res_last = r;
        ss->done = stop;
        ss->bar_base = epoch;
        ss->bar_arr = bbase + epoch * gridDim.x;
    }
}

// ---- cooperative solve under the reference's loop controls
// Sum of two doubles over the block (the result is valid in warp 0).
__device__ __forceinline__ void block_sum2d(double& a, double& b) {
    __shared__ double sh[2][32];
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) {
        sh[0][wid] = a;
        sh[1][wid] = b;
    }
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
        a = lane < nw ? sh[0][lane] : 0.0;
        b = lane < nw ? sh[1][lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_xor_sync(0xffffffffu, a, o);
            b += __shfl_xor_sync(0xffffffffu, b, o);
        }
    }
}

// Grid barrier that also sums one (a, b) record per block. Every block adds the records in the
// same order (lane-wise over blocks lane, lane + 32, ..., then a butterfly over the lanes), so
// all blocks get bit-identical sums and take the same decisions from them.
__device__ __forceinline__ void grid_arrive_sum(unsigned* ctr, double2* sums, unsigned epoch, double a, double b) {
    double2* bank = sums + (size_t)(epoch & 1u) * SPLIT_MAX_PARTS;
    if (threadIdx.x == 0) bank[blockIdx.x] = make_double2(a, b);
    __syncthreads();
    if (threadIdx.x == 0) asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(ctr) : "memory");
}
__device__ __forceinline__ bool grid_wait_sum(unsigned* ctr, double2* sums, unsigned epoch, unsigned base, int32_t* err,
                                              double& a, double& b, unsigned long long wait_ns) {
    __shared__ double s_a, s_b;
    __shared__ int s_ok;
    double2* bank = sums + (size_t)(epoch & 1u) * SPLIT_MAX_PARTS;
    if (threadIdx.x < 32) {
        const unsigned FULL = 0xffffffffu;
        int ok = 1;
        if (threadIdx.x == 0) {
            const unsigned target = base + epoch * gridDim.x;
            const unsigned long long t0 = global_ns();
            while ((int)(ld_acquire(ctr) - target) < 0) {
                if (ld_acquire(reinterpret_cast<const unsigned*>(err)) != 0u || global_ns() - t0 > wait_ns) {
                    atomicExch(err, 1);
                    ok = 0;
                    break;
                }
                __nanosleep(20);
            }
        }
        ok = __shfl_sync(FULL, ok, 0);
        double sa = 0.0, sb2 = 0.0;
        if (ok) {
            for (int p = threadIdx.x; p < (int)gridDim.x; p += 32) {
                const double2 v = __ldcg(&bank[p]);
                sa += v.x;
                sb2 += v.y;
            }
            for (int o = 16; o > 0; o >>= 1) {
                sa += __shfl_xor_sync(FULL, sa, o);
                sb2 += __shfl_xor_sync(FULL, sb2, o);
            }
        }
        if (threadIdx.x == 0) {
            s_a = sa;
            s_b = sb2;
            s_ok = ok;
        }
    }
    __syncthreads();
    a = s_a;
    b = s_b;
    return s_ok != 0;
}

// The terms of residual() (projected_jacobi.cpp:140-144) for one body's six velocities:
// sum of ((x - xp) / (tol_rel max(|x|, |xp|) + tol_abs))^2, evaluated in FP64 (a tolerance far
// below FP32's range, as a caller may set to switch the exit off, stays exact).
__device__ __forceinline__ double velres_body(float4 xv, float4 xw, float4 pv, float4 pw, double tr, double ta) {
    const float x[6] = {xv.x, xv.y, xv.z, xw.x, xw.y, xw.z};
    const float p[6] = {pv.x, pv.y, pv.z, pw.x, pw.y, pw.z};
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        const double a = x[k], b = p[k];
        const double q = fmax(fabs(a), fabs(b)) * tr + ta;
        const double d = (a - b) / q;
        s += d * d;
    }
    return s;
}
// The same terms on the FP32 pipe (GB300's FP64 divisions made the residual cost more than the
// sweep): mode 1 sums (x - xp)^2, mode 2 ((x - xp) / max(|x|, |xp|))^2 (the tolerance divides the
// sum once, in FP64, so any tolerance stays exact), mode 3 the full term with both tolerances in
// FP32's comfortable range. A body's few terms are summed in FP32, the bodies in FP64.
__device__ __forceinline__ float velres_body32(float4 xv, float4 xw, float4 pv, float4 pw, int mode, float tr,
                                               float ta) {
    const float x[6] = {xv.x, xv.y, xv.z, xw.x, xw.y, xw.z};
    const float p[6] = {pv.x, pv.y, pv.z, pw.x, pw.y, pw.z};
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        const float dx = x[k] - p[k];
        float d = dx;
        if (mode == 2)
            d = dx / fmaxf(fabsf(x[k]), fabsf(p[k]));
        else if (mode == 3)
            d = dx / (fmaxf(fabsf(x[k]), fabsf(p[k])) * tr + ta);
        s += d * d;
    }
    return s;
}
__device__ __forceinline__ float nes_dot_body32(float4 yv, float4 yw, float4 v1, float4 w1, float4 v0, float4 w0) {
    return ((yv.x - v1.x) * (v1.x - v0.x) + (yv.y - v1.y) * (v1.y - v0.y) + (yv.z - v1.z) * (v1.z - v0.z)) +
           ((yw.x - w1.x) * (w1.x - w0.x) + (yw.y - w1.y) * (w1.y - w0.y) + (yw.z - w1.z) * (w1.z - w0.z));
}
// (y - x1) . (x1 - x0) over one body's six velocities (nesterov_loop's restart test), in FP64
__device__ __forceinline__ double nes_dot_body(float4 yv, float4 yw, float4 v1, float4 w1, float4 v0, float4 w0) {
    return ((double)yv.x - v1.x) * ((double)v1.x - v0.x) + ((double)yv.y - v1.y) * ((double)v1.y - v0.y) +
           ((double)yv.z - v1.z) * ((double)v1.z - v0.z) + ((double)yw.x - w1.x) * ((double)w1.x - w0.x) +
           ((double)yw.y - w1.y) * ((double)w1.y - w0.y) + ((double)yw.z - w1.z) * ((double)w1.z - w0.z);
}
__device__ __forceinline__ float4 extrap4(float4 x1, float4 x0, float c) {
    // x1 + c (x1 - x0); the .w lanes carry the inverse masses, equal in both, so they stay exact
    return make_float4(x1.x + c * (x1.x - x0.x), x1.y + c * (x1.y - x0.y), x1.z + c * (x1.z - x0.z),
                       x1.w + c * (x1.w - x0.w));
}

// The cooperative whole solve (one block per SM, contacts in shared memory, the same sweep as
// k_s_solve_coop with one contact per thread and pass) under the loop controls of
// ProjectedJacobiSolver::solve (projected_jacobi.cpp:451-500):
//   NES = 0, standard_loop (:371-377): after sweep k (counting from 0) with k % 10 == 0 the
//     velocity-increment residual err = sqrt(1/Nv) ||(x_{k+1} - x_k) / q|| (:140-144) is formed
//     over all bodies (one extra grid reduction) and the loop ends when err <= 1;
//   NES = 1, nesterov_loop (:379-449): the sweep runs from the extrapolated pair (y, p_y) and
//     gives (x_{k+1}, p_{k+1}); err = residual(x_{k+1}, y); the loop ends when err <= 1, else
//     theta and beta are updated and momentum restarts when err is not finite, err grew by more
//     than 5 %, beta exceeds pj.nesterov_beta_threshold or leaves [0, 1], or (y - x_{k+1}) .
//     (x_{k+1} - x_k) > 0; after pj.nesterov_restart_limit restarts momentum stays off. Then
//     y = x_{k+1} + beta (x_{k+1} - x_k) and p_y = p_{k+1} + beta (p_{k+1} - p_k).
// Velocities are linear in the impulses (x = x_free + M^-1 W^T lambda), so each block
// extrapolates its own bodies' velocities and its own contacts' impulses with no scatter. One
// Nesterov iteration takes three grid barriers: after the sweep (x_{k+1} complete), after the
// reductions of err and the dot product (every block then takes the same decision from the same
// sums), and after the extrapolation (y complete for the next sweep's gathers). Accumulators:
// y (read by the sweep, overwritten in place by the extrapolation once every block has passed
// the second barrier), x_{k+1} (reset to the free velocities before the sweep adds into it) and
// x_k; the last two swap roles each iteration.
// gpu.residual_tol and the iteration cap end the loop as in the plain cooperative solve (every
// check_every sweeps). The result is (x_{k+1}, p_{k+1}) of the last sweep, as in the reference.
// Shared memory a contact: records and impulses (48 B), plus p_k for Nesterov (64 B).
// The loop state lives in shared memory (thread 0 updates it; every block's thread 0 computes the
// same values from the same sums), which keeps it out of the sweep's registers.
struct CoopLoopState {
    double thk, err_prev, verr, dot;
    int restarts, disabled, iy, ix1, ixk;
    float coef;
};
template <int NTH, int HYB, int NES>
__global__ void __launch_bounds__(NTH, 1) k_s_solve_coop_loop(SplitBuf sb, int gen, float alpha, int max_iter,
                                                              float tol, int cpb, int bpb, int vf_smem, int max_sweeps,
                                                              int check_every, CoopLoopArgs la,
                                                              unsigned long long wait_ns) {
    extern __shared__ float4 smem[];
    __shared__ CoopLoopState L;
    SplitScalars* ss = sb.ss;
    if (*(volatile int32_t*)&ss->done) return;
    float4* s_q0 = smem;
    float4* s_q1 = smem + cpb;
    float4* s_l = smem + 2 * cpb;                 // lambda (Nesterov: p_y before the sweep, p_{k+1} after)
    float4* s_pk = smem + 3 * cpb;                // Nesterov: p_k
    float4* s_vf = smem + (NES ? 4 : 3) * cpb;    // free velocities of the block's bodies
    const int it0 = *(volatile int32_t*)&ss->iters;
    unsigned epoch = *(volatile unsigned*)&ss->bar_base;
    // arrivals so far this step: the launches before this one may have had other grid sizes (the
    // autotuner's trials), so the counter's target is counted from them (modulo 2^32)
    const unsigned bbase = *(volatile unsigned*)&ss->bar_arr - epoch * gridDim.x;
    const int nc = *sb.nc_dev, N = sb.N, tid = threadIdx.x;
    if (!HYB && (int64_t)nc > (int64_t)cpb * gridDim.x) {
        if (blockIdx.x == 0 && tid == 0) ss->err = 4;
        return;
    }
    const int cpe = (nc + (int)gridDim.x - 1) / (int)gridDim.x;
    const int cb = blockIdx.x * cpe;
    const int ncb = max(0, min(nc - cb, cpe));
    const int bb = blockIdx.x * bpb;
    const int nbb = max(0, min(N - bb, bpb));
    const int ncs = HYB ? min(ncb, cpb) : ncb;
    float4* __restrict__ lamg = sb.lam[gen];
    float4* __restrict__ pkg = sb.lamk;
    for (int i = tid; i < ncs; i += NTH) {
        s_q0[i] = ldg4(&sb.rec0[cb + i]);
        s_q1[i] = ldg4(&sb.rec1[cb + i]);
        s_l[i] = lamg[cb + i];
        if (NES) s_pk[i] = it0 == 0 ? s_l[i] : pkg[cb + i];
    }
    if (NES && HYB && it0 == 0)
        for (int i = ncs + tid; i < ncb; i += NTH) pkg[cb + i] = lamg[cb + i];
    if (vf_smem)
        for (int i = tid; i < 2 * nbb; i += NTH) s_vf[i] = ldg4(&sb.vel4[2 * bb + i]);
    if (tid == 0) {
        L.thk = ss->nes_thk;
        L.err_prev = ss->nes_err_prev;
        L.verr = ss->vel_err;
        L.dot = 0.0;
        L.restarts = ss->nes_restarts;
        L.disabled = ss->nes_disabled;
        L.iy = ss->nes_iy;
        L.ix1 = ss->nes_ix1;
        L.ixk = ss->nes_ixk;
        L.coef = 0.f;
    }
    __syncthreads();
    if (NES && it0 == 0) {
        // x_k = x_0 at the start: the block's own bodies, read back by this block only
        const float4* Y0 = sb.acc[L.iy];
        float4* XK0 = sb.acc[L.ixk];
        for (int i = tid; i < nbb; i += NTH) {
            float4 v0, w0;
            ldcg_body(&Y0[2 * (bb + i)], v0, w0);
            stcg_body(&XK0[2 * (bb + i)], v0, w0);
        }
        __syncthreads();
    }
    int it = it0, stop = 0;
    float r = 0.f;
    for (int j = 0; j < max_sweeps; ++j) {
        const float4* G = sb.acc[NES ? L.iy : it % SPLIT_NACC];
        float4* Add = sb.acc[NES ? L.ix1 : (it + 1) % SPLIT_NACC];
        float maxd2 = 0.f, maxl = 0.f;
        for (int base = 0; base < ncb; base += NTH) {
            const int i = base + tid;
            const bool ok = i < ncb;
            PJOut o = {};
            int a = -1, b = 0;
            if (ok) {
                float4 q0, q1, l;
                if (!HYB || i < ncs) {
                    q0 = s_q0[i];
                    q1 = s_q1[i];
                    l = s_l[i];
                } else {
                    q0 = ldg4(&sb.rec0[cb + i]);
                    q1 = ldg4(&sb.rec1[cb + i]);
                    l = __ldcg(&lamg[cb + i]);
                }
                a = __float_as_int(q1.z);
                b = __float_as_int(q1.w);
                float4 va, wa, vb, wb;
                ldcg_body(&G[2 * b], vb, wb);
                if (a >= 0) {
                    ldcg_body(&G[2 * a], va, wa);
                } else {
                    va = make_float4(0.f, 0.f, 0.f, 0.f);
                    wa = va;
                }
                pj_contact(q0, q1, l, va, wa, vb, wb, &sb.bias[cb + i], alpha, o);
                if (!HYB || i < ncs)
                    s_l[i] = o.lam;
                else
                    __stcg(&lamg[cb + i], o.lam);
                maxd2 = fmaxf(maxd2, o.dn2);
                maxl = fmaxf(maxl, o.lm);
            }
            pj_push<2>(Add, ok, a, b, o);
        }
        const bool check = (it + 1) % check_every == 0 || it + 1 >= max_iter;
        const bool velchk = NES || (la.check_vel && it % 10 == 0);
        if (check) block_max2(maxd2, maxl);
        grid_arrive(&ss->bar, sb.recs, ++epoch, check, maxd2, maxl);
        if (!NES) {
            // the standard loop's accumulator rotation: reset A_{k-1} while the others arrive
            float4* Clr = sb.acc[(it + 3) % SPLIT_NACC];
            for (int i = tid; i < nbb; i += NTH) {
                const float4 v0 = vf_smem ? s_vf[2 * i] : ldg4(&sb.vel4[2 * (bb + i)]);
                const float4 w0 = vf_smem ? s_vf[2 * i + 1] : ldg4(&sb.vel4[2 * (bb + i) + 1]);
                stcg_body(&Clr[2 * (bb + i)], v0, w0);
            }
        }
        if (!grid_wait_max(&ss->bar, sb.recs, epoch, bbase, &ss->err, check, maxd2, maxl, wait_ns)) return;
        if (velchk) {
            // the velocity-increment residual between the new velocities and those the sweep read
            // (and Nesterov's restart dot product), over the block's own bodies, then over the grid
            double e = 0.0, d = 0.0;
            const float4* XK = sb.acc[L.ixk];
            const int rm = la.res_mode;
            const float tr32 = (float)la.tol_rel, ta32 = (float)la.tol_abs;
            for (int i = tid; i < nbb; i += NTH) {
                float4 v1, w1, v0, w0;
                ldcg_body(&Add[2 * (bb + i)], v1, w1);
                ldcg_body(&G[2 * (bb + i)], v0, w0);
                if (rm)
                    e += (double)velres_body32(v1, w1, v0, w0, rm, tr32, ta32);
                else
                    e += velres_body(v1, w1, v0, w0, la.tol_rel, la.tol_abs);
                if (NES) {
                    float4 vk, wk;
                    ldcg_body(&XK[2 * (bb + i)], vk, wk);
                    d += rm ? (double)nes_dot_body32(v0, w0, v1, w1, vk, wk) : nes_dot_body(v0, w0, v1, w1, vk, wk);
                }
            }
            block_sum2d(e, d);
            grid_arrive_sum(&ss->bar, sb.sums, ++epoch, e, d);
            if (!grid_wait_sum(&ss->bar, sb.sums, epoch, bbase, &ss->err, e, d, wait_ns)) return;
            if (tid == 0) {
                double verr = (1.0 / sqrt((double)la.nv)) * sqrt(e);
                if (rm == 1) verr /= la.tol_abs;
                if (rm == 2) verr /= la.tol_rel;
                L.verr = verr;
                L.dot = d;
            }
            __syncthreads();
        }
        ++it;
        bool fin = velchk && L.verr <= 1.0;
        if (check) {
            r = sweep_residual(maxd2, maxl);
            if (it >= max_iter || (tol > 0.f && r <= tol) || !(r == r)) fin = true;
        }
        if (fin) {
            stop = 1;
            break;
        }
        if (NES) {
            if (tid == 0) {
                // nesterov_loop's momentum update (every block takes the same decision)
                const double verr = L.verr, thk = L.thk;
                const double thk1 = 0.5 * (1.0 + sqrt(4.0 * thk * thk + 1.0));
                const double betak1 = (thk - 1.0) / thk1;
                bool restart = false;
                if (!isfinite(verr)) {
                    restart = true;
                } else if (isfinite(L.err_prev) && verr > 1.05 * L.err_prev) {
                    restart = true;
                } else if (betak1 > la.beta_threshold) {
                    restart = true;
                } else if (!isfinite(betak1) || betak1 < 0.0 || betak1 > 1.0) {
                    restart = true;
                } else if (L.dot > 0.0) {
                    restart = true;
                }
                L.coef = 0.f;
                if (restart) {
                    L.thk = 1.0;
                    if (++L.restarts >= la.restart_limit) L.disabled = 1;
                } else if (L.disabled) {
                    L.thk = 1.0;
                } else {
                    L.coef = (float)betak1;
                    L.thk = thk1;
                }
                L.err_prev = verr;
            }
            __syncthreads();
            const float coef = L.coef;
            // y = x_{k+1} + beta (x_{k+1} - x_k) for the block's bodies; x_k's buffer is reset to the
            // free velocities and becomes the next x_{k+1}
            float4* Y = sb.acc[L.iy];
            const float4* X1 = sb.acc[L.ix1];
            float4* XK = sb.acc[L.ixk];
            for (int i = tid; i < nbb; i += NTH) {
                float4 v1, w1, v0, w0;
                ldcg_body(&X1[2 * (bb + i)], v1, w1);
                ldcg_body(&XK[2 * (bb + i)], v0, w0);
                stcg_body(&Y[2 * (bb + i)], extrap4(v1, v0, coef), extrap4(w1, w0, coef));
                const float4 f0 = vf_smem ? s_vf[2 * i] : ldg4(&sb.vel4[2 * (bb + i)]);
                const float4 f1 = vf_smem ? s_vf[2 * i + 1] : ldg4(&sb.vel4[2 * (bb + i) + 1]);
                stcg_body(&XK[2 * (bb + i)], f0, f1);
            }
            // p_y = p_{k+1} + beta (p_{k+1} - p_k), p_k = p_{k+1} for the block's contacts
            for (int i = tid; i < ncb; i += NTH) {
                if (!HYB || i < ncs) {
                    const float4 l1 = s_l[i], l0 = s_pk[i];
                    s_pk[i] = l1;
                    s_l[i] = extrap4(l1, l0, coef);
                } else {
                    const float4 l1 = __ldcg(&lamg[cb + i]), l0 = __ldcg(&pkg[cb + i]);
                    __stcg(&pkg[cb + i], l1);
                    __stcg(&lamg[cb + i], extrap4(l1, l0, coef));
                }
            }
            // y complete before any block gathers from it (the barrier's __syncthreads also orders
            // the swap below after every thread's use of the old indices)
            grid_arrive(&ss->bar, sb.recs, ++epoch, false, 0.f, 0.f);
            if (tid == 0) {
                const int t = L.ix1;
                L.ix1 = L.ixk;
                L.ixk = t;
            }
            float u0, u1;
            if (!grid_wait_max(&ss->bar, sb.recs, epoch, bbase, &ss->err, false, u0, u1, wait_ns)) return;
        }
    }
    for (int i = tid; i < ncs; i += NTH) {
        lamg[cb + i] = s_l[i];
        if (NES && !stop) pkg[cb + i] = s_pk[i];
    }
    if (blockIdx.x == 0 && tid == 0) {
        ss->iters = it;
        ss->res_last = r;
        ss->done = stop;
        ss->bar_base = epoch;
        ss->bar_arr = bbase + epoch * gridDim.x;
        ss->vel_err = L.verr;
        if (NES) {
            ss->final_acc = L.ix1;
            ss->nes_thk = L.thk;
            ss->nes_err_prev = L.err_prev;
            ss->nes_restarts = L.restarts;
            ss->nes_disabled = L.disabled;
            ss->nes_iy = L.iy;
            ss->nes_ix1 = L.ix1;
            ss->nes_ixk = L.ixk;
        }
    }
}

// ---- batched scenes: one block per scene
// The projected Jacobi solve of a batch of independent scenes. Block k solves scene order[k]
// (scenes ordered by decreasing size, so the long solves start first). Each scene runs its own
// stop rule (iteration cap, residual <= tol, non-finite) on its own maxima, and sweeps are
// separated by __syncthreads only, never by a grid barrier.
// The scene's velocity accumulators are the global ones, three rotating buffers: sweep k gathers
// A_k through L2 (32-byte loads), adds into A_{k+1} with L2 reductions and per-warp run sums (as
// the cooperative solve does), and resets A_{k+2} (last read in sweep k - 1) to the free
// velocities. Summing in shared memory instead (float atomics) measured three times slower on
// 4,096 scenes. With CSM the scene's contact records and impulses sit in shared memory (48 B a
// contact, up to ccap contacts; a larger scene reads them from L1/L2 every sweep).
// The final velocities go to accumulator 0; the largest per-scene sweep count and residual go to
// the step's scalars.
// 1024 / NT blocks an SM at least: 64 registers a thread, 32 warps an SM
// scene_alpha (optional): each scene's alpha; the in-sweep residual is then rescaled to alpha_ref
// (the residual's R is alpha / D, and near the fixed point it scales with alpha) for the stop rule
// and the statistics. scene_out (optional): each scene's sweeps and rescaled residual.
template <int NT, int CSM>
__global__ void __launch_bounds__(NT, 1024 / NT) k_s_solve_scenes(Scene sc, SplitBuf sb, int gen, float alpha, int max_iter,
                                                       float tol, const int32_t* spos, const int32_t* sflags,
                                                       const int32_t* poff, const int32_t* order, int L, int ccap,
                                                       float* scene_alpha, float alpha_ref, int4* scene_out) {
    extern __shared__ float4 sm4[];
    // a device-counted step whose contacts overflowed the buffers wrote only the slots below the
    // capacity, while the scene ranges below count them all: nothing runs, the host redoes the step
    if (*(volatile const int32_t*)&sb.ss->cap_err) return;
    __shared__ float s_r, s_l;
    const int s = order[blockIdx.x];
    const int b0 = sc.scene_body_start[s], nb = sc.scene_body_start[s + 1] - b0;
    const int tid = threadIdx.x;
    float a_s = scene_alpha ? scene_alpha[s] : alpha;
    float rscale = alpha_ref / a_s;
    // A tuned alpha above the configured one can lose stability when the scene's contacts change
    // after the tuning (projected Jacobi converges for alpha < 2 / the largest eigenvalue of
    // D^-1/2 W D^-1/2, and new contacts raise it). Divergence grows the impulses geometrically
    // while their relative change stays level, so the stop rule does not see it; near the bound the
    // projections can also hold the impulses in a bounded oscillation. Once the largest impulse
    // exceeds 16 times its largest over the first 8 sweeps, or the residual has not halved from
    // sweep 32 to sweep 256, the scene starts over from its warm start (kept aside at the start)
    // at the configured alpha, which it keeps from then on.
    bool guard = scene_alpha != nullptr && a_s > alpha_ref && sb.lam_warm != nullptr;  // block-uniform
    float lm_ref = 0.f, r32 = 0.f;
    const int64_t nflag = (int64_t)sc.N * L;
    int n_static = 0;
    if (nflag > 0) n_static = spos[nflag - 1] + sflags[nflag - 1];
    int cs0 = 0, cs1 = 0;
    if (L > 0) {
        cs0 = spos[(int64_t)b0 * L];
        cs1 = ((int64_t)(b0 + nb) * L < nflag) ? spos[(int64_t)(b0 + nb) * L] : n_static;
    }
    const int cp0 = n_static + poff[b0], cp1 = n_static + poff[b0 + nb];
    const int ns = cs1 - cs0, nc = ns + (cp1 - cp0);
    const bool local = CSM && nc <= ccap;  // block-uniform
    float4* q0s = sm4;
    float4* q1s = q0s + ccap;
    float4* ls = q1s + ccap;
    float4* __restrict__ lamp = sb.lam[gen];
    // A_0 holds the starting velocities; A_1 starts at the free velocities
    for (int i = tid; i < 2 * nb; i += NT) sb.acc[1][2 * b0 + i] = sb.vel4[2 * b0 + i];
    if (local)
        for (int k = tid; k < nc; k += NT) {
            const int c = k < ns ? cs0 + k : cp0 + (k - ns);
            q0s[k] = ldg4(&sb.rec0[c]);
            q1s[k] = ldg4(&sb.rec1[c]);
            ls[k] = lamp[c];
        }
    if (guard)
        for (int k = tid; k < nc; k += NT) {
            const int c = k < ns ? cs0 + k : cp0 + (k - ns);
            sb.lam_warm[c] = lamp[c];
        }
    __syncthreads();
    int it = 0;
    float r = 0.f;
    const int lane = tid & 31;
    while (true) {
        float maxd2 = 0.f, maxl = 0.f;
        const float4* Gc = sb.acc[it % 3];
        float4* Gn = sb.acc[(it + 1) % 3];
        float4* Gr = sb.acc[(it + 2) % 3];
        // the loop bound is the same for all lanes of a warp (the run sum needs whole warps)
        for (int w0 = (tid & ~31); w0 < nc; w0 += NT) {
            const int k = w0 + lane;
            const bool ok = k < nc;
            PJOut o = {};
            int a = -1, b = 0;
            if (ok) {
                const int c = k < ns ? cs0 + k : cp0 + (k - ns);
                float4 r0, r1, l;
                if (local) {
                    r0 = q0s[k];
                    r1 = q1s[k];
                    l = ls[k];
                } else {
                    r0 = ldg4(&sb.rec0[c]);
                    r1 = ldg4(&sb.rec1[c]);
                    l = lamp[c];
                }
                a = __float_as_int(r1.z);
                b = __float_as_int(r1.w);
                float4 va, wa, vb, wb;
                ldcg_body(&Gc[2 * b], vb, wb);
                if (a >= 0) {
                    ldcg_body(&Gc[2 * a], va, wa);
                } else {
                    va = make_float4(0.f, 0.f, 0.f, 0.f);
                    wa = va;
                }
                pj_contact(r0, r1, l, va, wa, vb, wb, &sb.bias[c], a_s, o);
                if (local)
                    ls[k] = o.lam;
                else
                    lamp[c] = o.lam;
                maxd2 = fmaxf(maxd2, o.dn2);
                maxl = fmaxf(maxl, o.lm);
            }
            pj_push<2>(Gn, ok, a, b, o);
        }
        for (int i = tid; i < nb; i += NT) {
            const float4 v0 = ldg4(&sb.vel4[2 * (b0 + i)]), w0 = ldg4(&sb.vel4[2 * (b0 + i) + 1]);
            stcg_body(&Gr[2 * (b0 + i)], v0, w0);
        }
        // the barriers below also order this sweep's reductions before the next sweep's gathers
        block_max2(maxd2, maxl);
        if (tid == 0) {
            s_r = sweep_residual(maxd2, maxl) * rscale;
            s_l = maxl;
        }
        __syncthreads();
        r = s_r;
        ++it;
        if (guard) {
            const float lmax = s_l;
            if (it == 32) r32 = r;
            if (it <= 8) {
                lm_ref = fmaxf(lm_ref, lmax);
            } else if (!(r == r) || !(lmax <= 16.f * lm_ref) || (it == 256 && !(r <= 0.5f * r32))) {
                guard = false;
                a_s = alpha_ref;
                rscale = 1.f;
                if (tid == 0) scene_alpha[s] = alpha_ref;
                // the next sweep gathers accumulator it % 3: the free velocities plus M^-1 W^T of
                // the warm start, as the step's warm start left them
                float4* Gx = sb.acc[it % 3];
                for (int i = tid; i < nb; i += NT) {
                    const float4 v0 = ldg4(&sb.vel4[2 * (b0 + i)]), w0 = ldg4(&sb.vel4[2 * (b0 + i) + 1]);
                    stcg_body(&Gx[2 * (b0 + i)], v0, w0);
                }
                __syncthreads();
                for (int k = tid; k < nc; k += NT) {
                    const int c = k < ns ? cs0 + k : cp0 + (k - ns);
                    const float4 l = sb.lam_warm[c];
                    if (local)
                        ls[k] = l;
                    else
                        lamp[c] = l;
                    if (l.x == 0.f && l.y == 0.f && l.z == 0.f) continue;
                    const float4 r0 = local ? q0s[k] : ldg4(&sb.rec0[c]);
                    const float4 r1 = local ? q1s[k] : ldg4(&sb.rec1[c]);
                    const int a = __float_as_int(r1.z), b = __float_as_int(r1.w);
                    const float3 n = f3(r0);
                    float3 t1, t2;
                    frame32(n, t1, t2);
                    const float imb = sb.vel4[2 * b].w, iib = sb.vel4[2 * b + 1].w;
                    const float ima = a >= 0 ? sb.vel4[2 * a].w : 0.f, iia = a >= 0 ? sb.vel4[2 * a + 1].w : 0.f;
                    scatter(Gx, a, b, n, t1, t2, r1.x, r1.y, l.x, l.y, l.z, imb, iib, ima, iia);
                }
                __syncthreads();
                if (it >= max_iter) break;
                continue;
            }
        }
        if (it >= max_iter || (tol > 0.f && r <= tol) || !(r == r)) break;
    }
    if (scene_out && tid == 0) scene_out[s] = make_int4(it, __float_as_int(r), __float_as_int(s_l), 0);
    // the final velocities to accumulator 0, where the final FP64 pass reads them
    if (it % 3 != 0) {
        const float4* Gf = sb.acc[it % 3];
        for (int i = tid; i < nb; i += NT) {
            float4 v0, w0;
            ldcg_body(&Gf[2 * (b0 + i)], v0, w0);
            stcg_body(&sb.acc[0][2 * (b0 + i)], v0, w0);
        }
    }
    if (local)
        for (int k = tid; k < nc; k += NT) lamp[k < ns ? cs0 + k : cp0 + (k - ns)] = ls[k];
    if (tid == 0) {
        if (blockIdx.x == 0) sb.ss->final_acc = 0;
        atomicMax(&sb.ss->iters, it);
        atomicMax(reinterpret_cast<unsigned*>(&sb.ss->res_last), __float_as_uint(r == r ? r : 0.f));
        atomicAdd(&sb.ss->iters_sum, (unsigned long long)it);
    }
}

// the accumulators back to the free velocities (as k_s_prep leaves them), before the warm start
__global__ void k_s_acc_init(SplitBuf sb) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sb.N) return;
    const float4 v = sb.vel4[2 * i], w = sb.vel4[2 * i + 1];
    for (int k = 0; k < 3; ++k) {
        sb.acc[k][2 * i] = v;
        sb.acc[k][2 * i + 1] = w;
    }
}

// the scenes' alpha autotuner: best (sweeps, residual, alpha) per scene over the trial solves
__global__ void k_s_tune_init(int ns, float alpha, float4* best) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < ns) best[s] = make_float4(__int_as_float(0x7fffffff), INFINITY, alpha, 0.f);
}
// The first trial (the configured alpha) is the reference. Another trial is kept when its residual
// is finite, its impulses stay at the reference's scale (the residual is relative to max |lambda|,
// so impulses that grow without bound can look converged), and it needs fewer sweeps (with a
// tolerance) or, at equal sweeps, ends lower.
__global__ void k_s_tune_pick(int ns, float cand, const int4* out, float4* best, int is_ref) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= ns) return;
    const int it = out[s].x;
    const float r = __int_as_float(out[s].y);
    const float lm = __int_as_float(out[s].z);
    if (is_ref) {
        best[s] = make_float4(__int_as_float(it), r, cand, lm);
        return;
    }
    if (!(r == r) || isinf(r) || !(lm == lm) || isinf(lm)) return;
    const float4 b = best[s];
    if (!(lm <= 1.25f * b.w && b.w <= 1.25f * lm)) return;
    const int bit = __float_as_int(b.x);
    if (it < bit || (it == bit && r < b.y)) best[s] = make_float4(__int_as_float(it), r, cand, b.w);
}
// A pick above the configured alpha is kept with a 15 % margin below it: the trial shows the pick
// stable on this step's contacts, and the next steps' contacts can lower the bound it sits under.
__global__ void k_s_tune_commit(int ns, const float4* best, float* scene_alpha, float alpha_ref) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < ns) {
        const float a = best[s].z;
        scene_alpha[s] = a > alpha_ref ? fmaxf(alpha_ref, 0.85f * a) : a;
    }
}

__global__ void k_s_totals(SplitBuf sb, const int32_t* spos, const int32_t* sflags, int64_t nflag,
                           const int32_t* poff, int N) {
    SplitScalars* ss = sb.ss;
    const int ns = nflag > 0 ? spos[nflag - 1] + sflags[nflag - 1] : 0;
    const int64_t tot = (int64_t)ns + poff[N];
    ss->n_static = ns;
    ss->n_total = (int32_t)(tot < (int64_t)INT32_MAX ? tot : INT32_MAX);
    ss->cap_err = tot > sb.cap ? 1 : 0;
    *sb.nc_dev = (int32_t)(tot < sb.cap ? tot : sb.cap);
}

__global__ void k_s_end_step(SplitBuf sb, const DevScalars* ds) {
    SplitScalars* ss = sb.ss;
    ss->prev_count_dev = *sb.nc_dev;
    ss->prev_n_static_dev = ss->n_static;
    ss->pair_overflow = ds->overflow;
}

__global__ void k_s_reset(SplitBuf sb) {
    SplitScalars* ss = sb.ss;
    ss->done = (*sb.nc_dev == 0) ? 1 : 0;
    ss->iters = 0;
    ss->blocks_done = 0u;
    ss->maxd = 0u;
    ss->maxl = 0u;
    ss->res_last = 0.f;
    ss->maxd64 = 0ull;
    ss->maxl64 = 0ull;
    ss->err = 0;
    ss->bar = 0u;
    ss->bar_base = 0u;
    ss->bar_arr = 0u;
    ss->final_acc = -1;
    ss->iters_sum = 0ull;
    ss->nonfinite = 0;
    ss->nes_thk = 1.0;
    ss->vel_err = INFINITY;
    ss->nes_err_prev = INFINITY;
    ss->nes_restarts = 0;
    ss->nes_disabled = 0;
    ss->nes_iy = 0;
    ss->nes_ix1 = 1;
    ss->nes_ixk = 2;
}

// ------------------------------------------------------------------ FP64 finalisation
// FP64 contact geometry recomputed from FP64 positions (the same formulas as the plain method)
__device__ __forceinline__ void frame64(const double* n, double* t1, double* t2);
__device__ __forceinline__ void geom64(const Scene& sc, int a, int b, double* n, double& rhoA, double& rhoB) {
    const double xb[3] = {sc.bf(BF_PX)[b], sc.bf(BF_PY)[b], sc.bf(BF_PZ)[b]};
    const double rb = sc.bf(BF_RAD)[b];
    if (a >= 0) {
        const double xa[3] = {sc.bf(BF_PX)[a], sc.bf(BF_PY)[a], sc.bf(BF_PZ)[a]};
        const double ra = sc.bf(BF_RAD)[a];
        double d[3] = {xb[0] - xa[0], xb[1] - xa[1], xb[2] - xa[2]};
        const double dl2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        double dl = 0.0;
        if (dl2 > 0.0) {
            const double inv = rsqrt_nr(dl2);
            dl = dl2 * inv;
            n[0] = d[0] * inv; n[1] = d[1] * inv; n[2] = d[2] * inv;
        } else { n[0] = 0; n[1] = 0; n[2] = 1; }
        rhoA = 0.5 * (dl + ra - rb);
        rhoB = 0.5 * (ra - rb - dl);
        return;
    }
    const int s = -a - 1;
    double u[3] = {sc.sf(SF_DX)[s], sc.sf(SF_DY)[s], sc.sf(SF_DZ)[s]};
    rhoA = 0.0;
    const int kind = sc.static_kind[s];
    if (kind >= 2) {
        double R[9];
        for (int k = 0; k < 9; ++k) R[k] = sc.sf(SF_R0 + k)[s];
        const double p[3] = {sc.sf(SF_PX)[s], sc.sf(SF_PY)[s], sc.sf(SF_PZ)[s]};
        if (kind == 3) {
            // solid box, as in the narrow phase
            const double rel[3] = {xb[0] - p[0], xb[1] - p[1], xb[2] - p[2]};
            double c[3], d[3];
            for (int k = 0; k < 3; ++k) c[k] = (R[k] * rel[0] + R[3 + k] * rel[1]) + R[6 + k] * rel[2];
            const double e[3] = {sc.sf(SF_EX)[s], sc.sf(SF_EY)[s], sc.sf(SF_EZ)[s]};
            double sd;
            if (!(fabs(c[0]) > e[0] || fabs(c[1]) > e[1] || fabs(c[2]) > e[2])) {
                int f = 0;
                double best = e[0] - fabs(c[0]);
                for (int k = 1; k < 3; ++k) {
                    const double dk = e[k] - fabs(c[k]);
                    if (dk < best) {
                        best = dk;
                        f = k;
                    }
                }
                for (int k = 0; k < 3; ++k) d[k] = k == f ? (c[k] < 0.0 ? -1.0 : 1.0) : 0.0;
                sd = -best;
            } else {
                for (int k = 0; k < 3; ++k) d[k] = c[k] - fmin(fmax(c[k], -e[k]), e[k]);
                const double dd2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
                const double inv = rsqrt_nr(dd2);
                sd = dd2 * inv;
                for (int k = 0; k < 3; ++k) d[k] *= inv;
            }
            for (int k = 0; k < 3; ++k) n[k] = (R[3 * k] * d[0] + R[3 * k + 1] * d[1]) + R[3 * k + 2] * d[2];
            rhoB = -0.5 * (sd + rb);
            return;
        }
        const double a3[3] = {sc.sf(SF_AX)[s], sc.sf(SF_AY)[s], sc.sf(SF_AZ)[s]};
        for (int k = 0; k < 3; ++k) u[k] = (R[3 * k] * a3[0] + R[3 * k + 1] * a3[1]) + R[3 * k + 2] * a3[2];
    }
    if (kind == 0) {
        const double sd = (u[0] * xb[0] + u[1] * xb[1] + u[2] * xb[2]) - sc.sf(SF_D)[s];
        n[0] = u[0]; n[1] = u[1]; n[2] = u[2];
        rhoB = -0.5 * (sd + rb);
        return;
    }
    const double p[3] = {sc.sf(SF_PX)[s], sc.sf(SF_PY)[s], sc.sf(SF_PZ)[s]};
    const double rel[3] = {xb[0] - p[0], xb[1] - p[1], xb[2] - p[2]};
    const double ax = rel[0] * u[0] + rel[1] * u[1] + rel[2] * u[2];
    const double perp[3] = {rel[0] - ax * u[0], rel[1] - ax * u[1], rel[2] - ax * u[2]};
    const double rho2 = perp[0] * perp[0] + perp[1] * perp[1] + perp[2] * perp[2];
    if (sc.static_kind[s] == 2) {
        // solid cylinder: side, cap or rim, as in the narrow phase
        const double R = sc.sf(SF_RAD)[s], h = sc.sf(SF_HL)[s];
        const double sg = ax < 0.0 ? -1.0 : 1.0, aax = fabs(ax);
        const double rho = rho2 > 0.0 ? rho2 * rsqrt_nr(rho2) : 0.0;
        double e[3] = {0.0, 0.0, 0.0};
        if (rho2 > 0.0) {
            const double inv = rsqrt_nr(rho2);
            for (int k = 0; k < 3; ++k) e[k] = perp[k] * inv;
        } else {
            double t2[3];
            frame64(u, e, t2);
        }
        const bool out_side = rho > R, out_cap = aax > h;
        double sd;
        if ((!out_side && !out_cap && (R - rho) <= (h - aax)) || (out_side && !out_cap)) {
            for (int k = 0; k < 3; ++k) n[k] = e[k];
            sd = rho - R;
        } else if (!out_side) {
            for (int k = 0; k < 3; ++k) n[k] = sg * u[k];
            sd = aax - h;
        } else {
            double d[3];
            for (int k = 0; k < 3; ++k) d[k] = rel[k] - ((sg * h) * u[k] + R * e[k]);
            const double dd2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            const double inv = rsqrt_nr(dd2);
            sd = dd2 * inv;
            for (int k = 0; k < 3; ++k) n[k] = d[k] * inv;
        }
        rhoB = -0.5 * (sd + rb);
        return;
    }
    double rho = 0.0;
    if (rho2 > 0.0) {
        const double inv = rsqrt_nr(rho2);
        rho = rho2 * inv;
        n[0] = -perp[0] * inv; n[1] = -perp[1] * inv; n[2] = -perp[2] * inv;
    } else { n[0] = 0; n[1] = 0; n[2] = 1; }
    rhoB = -0.5 * ((sc.sf(SF_RAD)[s] - rho) + rb);
}

// Frisvad frame of a unit FP64 normal. The construction is orthonormal in exact arithmetic and the
// normal is unit to ~1e-16, so the tangent is not renormalised (the residual tolerance is 1e-6).
__device__ __forceinline__ void frame64(const double* n, double* t1, double* t2) {
    if (n[2] < -0.9999999) {
        t1[0] = 0; t1[1] = -1; t1[2] = 0;
        const double d = n[0] * t1[0] + n[1] * t1[1] + n[2] * t1[2];
        for (int k = 0; k < 3; ++k) t1[k] -= n[k] * d;
    } else {
        const double a = rcp_nr(1.0 + n[2]);
        const double b = (-n[0] * n[1]) * a;
        t1[0] = 1.0 - (n[0] * n[0]) * a;
        t1[1] = b;
        t1[2] = -n[0];
    }
    if (n[2] < -0.9999999) {
        const double s = rsqrt_nr(t1[0] * t1[0] + t1[1] * t1[1] + t1[2] * t1[2]);
        for (int k = 0; k < 3; ++k) t1[k] *= s;
    }
    f64::cross3(n, t1, t2);
}

// Final FP64 velocities (world frame): v = v_free + M^-1 W^T lambda, the FP64 free velocity plus
// the impulse part of the last sweep's FP32 velocities (their difference to the FP32 free velocity,
// taken exactly in FP64).
__global__ void k_s_final_body(Scene sc, SplitBuf sb) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sc.N) return;
    const int N = sc.N;
    const int fa = sb.ss->final_acc >= 0 ? sb.ss->final_acc : sb.ss->iters % SPLIT_NACC;
    const float4* A = sb.acc[fa];
    const float4 a0 = A[2 * i], a1 = A[2 * i + 1];
    const float4 f0 = sb.vel4[2 * i], f1 = sb.vel4[2 * i + 1];
    const double d[6] = {(double)a0.x - (double)f0.x, (double)a0.y - (double)f0.y, (double)a0.z - (double)f0.z,
                         (double)a1.x - (double)f1.x, (double)a1.y - (double)f1.y, (double)a1.z - (double)f1.z};
    for (int k = 0; k < 6; ++k) {
        const size_t j = (size_t)k * N + i;
        sb.acc64[j] = sb.vfree[j] + d[k];
    }
}

// FP64 complementarity residual of (lambda, v): max_c ||lambda_c - Pi(lambda_c - R(W v + b))|| / max |lambda|
__global__ void k_s_residual(Scene sc, SplitBuf sb, int gen, double alpha, int friction_enable, int combine) {
    const int nc = *sb.nc_dev;
    const int N = sc.N;
    double maxd = 0.0, maxl = 0.0;
    float maxlf = 0.f;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
        const float4 r0 = sb.rec0[c], r1 = sb.rec1[c];
        const int2 ab = make_int2(__float_as_int(r1.z), __float_as_int(r1.w));
        double n[3], rA, rB;
        geom64(sc, ab.x, ab.y, n, rA, rB);
        double t1[3], t2[3];
        frame64(n, t1, t2);
        double dv[3], Om[3];
        for (int k = 0; k < 3; ++k) {
            dv[k] = sb.acc64[(size_t)k * N + ab.y];
            Om[k] = rB * sb.acc64[(size_t)(3 + k) * N + ab.y];
        }
        if (ab.x >= 0) {
            for (int k = 0; k < 3; ++k) {
                dv[k] -= sb.acc64[(size_t)k * N + ab.x];
                Om[k] -= rA * sb.acc64[(size_t)(3 + k) * N + ab.x];
            }
        }
        // R only scales the residual (which impulses are fixed points does not depend on it): the
        // solver's own FP32 R, from the same lever lengths and inverse masses as the sweeps
        const float imaf = ab.x >= 0 ? sb.vel4[2 * ab.x].w : 0.f, iiaf = ab.x >= 0 ? sb.vel4[2 * ab.x + 1].w : 0.f;
        float Rn32, Rt32;
        pj_rdiag(r1.x, r1.y, imaf, iiaf, sb.vel4[2 * ab.y].w, sb.vel4[2 * ab.y + 1].w, (float)alpha, Rn32, Rt32);
        const double Rn = Rn32, Rt = Rt32;
        double g[3];
        g[0] = n[0] * dv[0] + n[1] * dv[1] + n[2] * dv[2];
        g[1] = (t1[0] * dv[0] + t1[1] * dv[1] + t1[2] * dv[2]) + (t2[0] * Om[0] + t2[1] * Om[1] + t2[2] * Om[2]);
        g[2] = (t2[0] * dv[0] + t2[1] * dv[1] + t2[2] * dv[2]) - (t1[0] * Om[0] + t1[1] * Om[1] + t1[2] * Om[2]);
        // contact bias in FP64: static wall velocity (dynamics_assembler.cpp:281-285) plus
        // restitution times the pre-solve contact velocity (projected_jacobi.cpp:337-338)
        double cb[3] = {0.0, 0.0, 0.0};
        double eN = 0.0, eT = 0.0;
        if (ab.x < 0) {
            const int s = -ab.x - 1;
            const double vw0[3] = {sc.sf(SF_VX)[s], sc.sf(SF_VY)[s], sc.sf(SF_VZ)[s]};
            const double wb0[3] = {sc.sf(SF_WX)[s], sc.sf(SF_WY)[s], sc.sf(SF_WZ)[s]};
            if (vw0[0] != 0.0 || vw0[1] != 0.0 || vw0[2] != 0.0 || wb0[0] != 0.0 || wb0[1] != 0.0 || wb0[2] != 0.0) {
                double Rs[9];
                for (int k = 0; k < 9; ++k) Rs[k] = sc.sf(SF_R0 + k)[s];
                double ww[3];
                for (int k = 0; k < 3; ++k) ww[k] = Rs[3 * k] * wb0[0] + Rs[3 * k + 1] * wb0[1] + Rs[3 * k + 2] * wb0[2];
                const double xb[3] = {sc.bf(BF_PX)[ab.y], sc.bf(BF_PY)[ab.y], sc.bf(BF_PZ)[ab.y]};
                double rA[3], cr[3], vw[3];
                for (int k = 0; k < 3; ++k) rA[k] = (xb[k] + rB * n[k]) - sc.sf(SF_PX + k)[s];
                f64::cross3(ww, rA, cr);
                for (int k = 0; k < 3; ++k) vw[k] = vw0[k] + cr[k];
                cb[0] = -(n[0] * vw[0] + n[1] * vw[1] + n[2] * vw[2]);
                cb[1] = -(t1[0] * vw[0] + t1[1] * vw[1] + t1[2] * vw[2]);
                cb[2] = -(t2[0] * vw[0] + t2[1] * vw[1] + t2[2] * vw[2]);
            }
            if (sb.has_restitution) {
                eN = fmin(fmax(0.0, sc.sf(SF_RN)[s]), fmax(0.0, sc.bf(BF_RN)[ab.y]));
                eT = fmin(fmax(0.0, sc.sf(SF_RT)[s]), fmax(0.0, sc.bf(BF_RT)[ab.y]));
            }
        } else if (sb.has_restitution) {
            // (a scene without restitution skips these FP64 min/max: the FP64 pipe bounds this kernel)
            eN = fmin(fmax(0.0, sc.bf(BF_RN)[ab.x]), fmax(0.0, sc.bf(BF_RN)[ab.y]));
            eT = fmin(fmax(0.0, sc.bf(BF_RT)[ab.x]), fmax(0.0, sc.bf(BF_RT)[ab.y]));
        }
        double bias[3] = {cb[0], cb[1], cb[2]};
        if (eN > 0.0 || eT > 0.0) {
            // pre-solve velocities are still in the state arrays (written back after this pass)
            double dvn[3], Omn[3];
            auto wworld = [&](int i, double* o) {
                double R[9];
                for (int k = 0; k < 9; ++k) R[k] = sc.bf(BF_R0 + k)[i];
                const double w[3] = {sc.bf(BF_WX)[i], sc.bf(BF_WY)[i], sc.bf(BF_WZ)[i]};
                for (int k = 0; k < 3; ++k) o[k] = R[3 * k] * w[0] + R[3 * k + 1] * w[1] + R[3 * k + 2] * w[2];
            };
            double wbn[3];
            wworld(ab.y, wbn);
            for (int k = 0; k < 3; ++k) {
                dvn[k] = sc.bf(BF_VX + k)[ab.y];
                Omn[k] = rB * wbn[k];
            }
            if (ab.x >= 0) {
                double wan[3];
                wworld(ab.x, wan);
                for (int k = 0; k < 3; ++k) {
                    dvn[k] -= sc.bf(BF_VX + k)[ab.x];
                    Omn[k] -= rA * wan[k];
                }
            }
            const double vp0 = (n[0] * dvn[0] + n[1] * dvn[1] + n[2] * dvn[2]) + cb[0];
            const double vp1 = (t1[0] * dvn[0] + t1[1] * dvn[1] + t1[2] * dvn[2]) +
                               (t2[0] * Omn[0] + t2[1] * Omn[1] + t2[2] * Omn[2]) + cb[1];
            const double vp2 = (t2[0] * dvn[0] + t2[1] * dvn[1] + t2[2] * dvn[2]) -
                               (t1[0] * Omn[0] + t1[1] * Omn[1] + t1[2] * Omn[2]) + cb[2];
            bias[0] += eN * vp0;
            bias[1] += eT * vp1;
            bias[2] += eT * vp2;
        }
        const float4 l = sb.lam[gen][c];
        const double lo[3] = {l.x, l.y, l.z};
        const double mu = fabsf(r0.w);
        double ln = lo[0] - Rn * (g[0] + bias[0]);
        double lt1 = lo[1] - Rt * (g[1] + bias[1]);
        double lt2 = lo[2] - Rt * (g[2] + bias[2]);
        ln = ln < 0.0 ? 0.0 : ln;
        const double tn2 = lt1 * lt1 + lt2 * lt2;
        if (tn2 > 0.0) {
            const double s = fmin(1.0, (mu * ln) * rsqrt_nr(tn2));
            lt1 *= s;
            lt2 *= s;
        }
        const double d0 = ln - lo[0], d1 = lt1 - lo[1], d2 = lt2 - lo[2];
        maxd = fmax(maxd, d0 * d0 + d1 * d1 + d2 * d2);  // squared; the root is taken once at the end
        // max |lambda| of FP32 impulses: exact in FP32, converted once
        maxlf = fmaxf(maxlf, fmaxf(fabsf(l.x), fmaxf(fabsf(l.y), fabsf(l.z))));
    }
    maxl = (double)maxlf;
    (void)friction_enable;
    (void)combine;
    block_max2(maxd, maxl);
    if (threadIdx.x == 0) {
        atomicMax(&sb.ss->maxd64, (unsigned long long)__double_as_longlong(maxd));
        atomicMax(&sb.ss->maxl64, (unsigned long long)__double_as_longlong(maxl));
    }
}

// the write-back fused with the closing drift theta h (moreau.cpp:12): the new velocities go to the
// state and move the positions and orientations without a second pass over the bodies
__global__ void k_s_writeback_drift(Scene sc, SplitBuf sb, double h) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < sc.N) {
        const int N = sc.N;
        double R[9];
        for (int k = 0; k < 9; ++k) R[k] = sc.bf(BF_R0 + k)[i];
        const double ww[3] = {sb.acc64[3 * (size_t)N + i], sb.acc64[4 * (size_t)N + i], sb.acc64[5 * (size_t)N + i]};
        double wb[3];
        f64::matTvec(R, ww, wb);
        const double v[3] = {sb.acc64[i], sb.acc64[(size_t)N + i], sb.acc64[2 * (size_t)N + i]};
        sc.bf(BF_VX)[i] = v[0];
        sc.bf(BF_VY)[i] = v[1];
        sc.bf(BF_VZ)[i] = v[2];
        sc.bf(BF_WX)[i] = wb[0];
        sc.bf(BF_WY)[i] = wb[1];
        sc.bf(BF_WZ)[i] = wb[2];
        double x[3] = {sc.bf(BF_PX)[i], sc.bf(BF_PY)[i], sc.bf(BF_PZ)[i]};
        double q[4] = {sc.bf(BF_QX)[i], sc.bf(BF_QY)[i], sc.bf(BF_QZ)[i], sc.bf(BF_QW)[i]};
        drift_fast(x, q, v, wb, h);
        sc.bf(BF_PX)[i] = x[0]; sc.bf(BF_PY)[i] = x[1]; sc.bf(BF_PZ)[i] = x[2];
        sc.bf(BF_QX)[i] = q[0]; sc.bf(BF_QY)[i] = q[1]; sc.bf(BF_QZ)[i] = q[2]; sc.bf(BF_QW)[i] = q[3];
        // the step's state must stay finite: the host reports CDX_ERR_NONFINITE otherwise
        bool ok = true;
        for (int k = 0; k < 3; ++k) ok = ok && isfinite(x[k]) && isfinite(v[k]) && isfinite(wb[k]);
        for (int k = 0; k < 4; ++k) ok = ok && isfinite(q[k]);
        if (!ok) sb.ss->nonfinite = 1;
    } else if (i < sc.N + sc.S) {
        const int s = i - sc.N;
        double x[3] = {sc.sf(SF_PX)[s], sc.sf(SF_PY)[s], sc.sf(SF_PZ)[s]};
        double q[4] = {sc.sf(SF_QX)[s], sc.sf(SF_QY)[s], sc.sf(SF_QZ)[s], sc.sf(SF_QW)[s]};
        const double v[3] = {sc.sf(SF_VX)[s], sc.sf(SF_VY)[s], sc.sf(SF_VZ)[s]};
        const double w[3] = {sc.sf(SF_WX)[s], sc.sf(SF_WY)[s], sc.sf(SF_WZ)[s]};
        drift_fast(x, q, v, w, h);
        sc.sf(SF_PX)[s] = x[0]; sc.sf(SF_PY)[s] = x[1]; sc.sf(SF_PZ)[s] = x[2];
        sc.sf(SF_QX)[s] = q[0]; sc.sf(SF_QY)[s] = q[1]; sc.sf(SF_QZ)[s] = q[2]; sc.sf(SF_QW)[s] = q[3];
    }
}

__global__ void k_s_final_scalar(SplitBuf sb) {
    SplitScalars* ss = sb.ss;
    const double maxd = __longlong_as_double((long long)ss->maxd64);
    const double maxl = __longlong_as_double((long long)ss->maxl64);
    ss->res_final = sqrt(maxd) / fmax(maxl, 1e-30);
}

__global__ void k_nr64_selftest(int n, const double* x, double* rcp, double* rsq) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    rcp[i] = rcp_nr(x[i]);
    rsq[i] = rsqrt_nr(x[i]);
}

}  // namespace

int launch_nr64_selftest(int n, const double* x, double* rcp, double* rsq, cudaStream_t s) {
    if (n > 0) k_nr64_selftest<<<nblk(n), NT, 0, s>>>(n, x, rcp, rsq);
    return 0;
}

int split_grid_blocks(int64_t n, int sms) {
    const int64_t want = (n + NT - 1) / NT;
    const int64_t cap = (int64_t)sms * 8;
    return (int)(want < 1 ? 1 : (want < cap ? want : cap));
}

// Solver shapes the autotuner chooses between.
// Streaming sweeps (one launch per sweep): contacts per thread, threads per block, register budget
// (minimum resident blocks per SM) and scatter mode.
struct StreamVariant {
    void (*kernel)(SplitBuf, int, float, int, float, cudaGraphConditionalHandle, int);
    int unroll, nth, minb, agg;
    int per_sm;
};
static StreamVariant g_stream[] = {
    {k_s_sweep_t<1, 256, 4, 2>, 1, 256, 4, 2, 0}, {k_s_sweep_t<2, 256, 2, 2>, 2, 256, 2, 2, 0},
    {k_s_sweep_t<1, 128, 8, 2>, 1, 128, 8, 2, 0}, {k_s_sweep_t<2, 128, 4, 2>, 2, 128, 4, 2, 0},
    {k_s_sweep_t<1, 256, 4, 1>, 1, 256, 4, 1, 0}, {k_s_sweep_t<1, 256, 4, 0>, 1, 256, 4, 0, 0},
};
constexpr int N_STREAM = sizeof(g_stream) / sizeof(g_stream[0]);
// Cooperative solves (one launch for all sweeps): threads per block and contacts per thread per pass.
struct CoopVariant {
    void (*kernel)(SplitBuf, int, float, int, float, int, int, int, int, int, unsigned long long);
    int nth, unroll, agg, hyb;
    int per_sm;    // resident blocks per SM with the full shared-memory budget (0 = not queried)
    int smem_max;  // dynamic shared memory budget of one block
    int minb;      // blocks an SM the shape is built for (its shared memory is split between them)
};
static CoopVariant g_coop[] = {
    {k_s_solve_coop<1024, 1, 2, 0>, 1024, 1, 2, 0, 0, 0, 1},
    {k_s_solve_coop<512, 2, 2, 0>, 512, 2, 2, 0, 0, 0, 1},
    {k_s_solve_coop<1024, 1, 2, 1>, 1024, 1, 2, 1, 0, 0, 1},
    // two blocks an SM of 576 threads at 56 registers: 1,152 threads an SM instead of 1,024, so the
    // settled 200k pile's 3,133 contacts an SM take three passes instead of four (9.9 against 10.4 us
    // a sweep)
    {k_s_solve_coop<576, 1, 2, 0, 2>, 576, 1, 2, 0, 0, 0, 2},
    // (reductions without the warp run sums, AGG 1, measured 13.2 against 9.9 us a sweep at 1,024
    // threads: the L2 serialises reductions to one address, so the run sums pay for themselves;
    // body B's shares summed over the lanes that share B anywhere in the warp (__match_any_sync),
    // which saves about 7 of a warp's 32 reductions on the settled pile, measured 11.4 us: the
    // grouping's shuffles cost more than the reductions they save)
};
constexpr int N_COOP = sizeof(g_coop) / sizeof(g_coop[0]);
// The same shapes under the reference's loop controls (1024 threads, one contact per thread and
// pass): [hybrid][Nesterov]
struct CoopLoopVariant {
    void (*kernel)(SplitBuf, int, float, int, float, int, int, int, int, int, CoopLoopArgs, unsigned long long);
    int per_sm, smem_max;
};
static CoopLoopVariant g_coop_loop[2][2] = {
    {{k_s_solve_coop_loop<1024, 0, 0>, 0, 0}, {k_s_solve_coop_loop<1024, 0, 1>, 0, 0}},
    {{k_s_solve_coop_loop<1024, 1, 0>, 0, 0}, {k_s_solve_coop_loop<1024, 1, 1>, 0, 0}},
};

// Batched scenes (one block per scene): threads per block and contacts per thread per pass.
struct ScenesVariant {
    void (*kernel)(Scene, SplitBuf, int, float, int, float, const int32_t*, const int32_t*, const int32_t*,
                   const int32_t*, int, int, float*, float, int4*);
    int nth, csm;
    int smem_set;  // dynamic shared memory the kernel has been opted in to
};
// measured on 4,096 scenes of 16-512 spheres (1.25 M contacts, 50 sweeps), 64 registers a thread:
// records from L1/L2 with 128 threads 2.29 ms a step, with 256 threads 2.44, with 64 threads 2.72;
// records in shared memory 2.58 (fewer blocks fit)
static ScenesVariant g_scenes[] = {
    {k_s_solve_scenes<128, 0>, 128, 0, 0},
    {k_s_solve_scenes<256, 0>, 256, 0, 0},
    {k_s_solve_scenes<256, 1>, 256, 1, 0},
    // (512 threads a scene: 43.4 against 38.3 ms a step on 4,096 settled scenes at residual 1e-6,
    // where the largest scenes' sweeps set the step: fewer blocks fit an SM)
};
constexpr int N_SCENES = sizeof(g_scenes) / sizeof(g_scenes[0]);

int split_num_variants() { return N_STREAM + N_COOP + N_SCENES; }
bool split_variant_is_coop(int v) { return v >= N_STREAM && v < N_STREAM + N_COOP; }
bool split_variant_is_scenes(int v) { return v >= N_STREAM + N_COOP && v < N_STREAM + N_COOP + N_SCENES; }
int split_first_scenes_variant() { return N_STREAM + N_COOP; }
int split_first_coop_variant() { return N_STREAM; }
int split_num_scenes_variants() { return N_SCENES; }

const char* split_variant_name(int v) {
    static char names[N_STREAM + N_COOP + N_SCENES][32];
    if (v < 0 || v >= N_STREAM + N_COOP + N_SCENES) return "?";
    if (!names[v][0]) {
        if (v < N_STREAM) {
            const StreamVariant& cv = g_stream[v];
            snprintf(names[v], sizeof(names[v]), "sweep-u%d-t%d-b%d-g%d", cv.unroll, cv.nth, cv.minb, cv.agg);
        } else if (v < N_STREAM + N_COOP) {
            const CoopVariant& cv = g_coop[v - N_STREAM];
            if (cv.minb > 1)
                snprintf(names[v], sizeof(names[v]), "coop-t%d-u%d-g%d-b%d", cv.nth, cv.unroll, cv.agg, cv.minb);
            else
                snprintf(names[v], sizeof(names[v]), cv.hyb ? "coop-hyb-t%d-u%d-g%d" : "coop-t%d-u%d-g%d", cv.nth,
                         cv.unroll, cv.agg);
        } else {
            const ScenesVariant& cv = g_scenes[v - N_STREAM - N_COOP];
            snprintf(names[v], sizeof(names[v]), "scenes-t%d-c%d", cv.nth, cv.csm);
        }
    }
    return names[v];
}

void launch_s_tune_alpha(int op, int ns, float alpha, const int4* out, float4* best, float* scene_alpha,
                         cudaStream_t s) {
    if (ns <= 0) return;
    if (op == 0) k_s_tune_init<<<nblk(ns), NT, 0, s>>>(ns, alpha, best);
    if (op == 1 || op == 3) k_s_tune_pick<<<nblk(ns), NT, 0, s>>>(ns, alpha, out, best, op == 3);
    if (op == 2) k_s_tune_commit<<<nblk(ns), NT, 0, s>>>(ns, best, scene_alpha, alpha);
}
void launch_s_acc_init(const SplitBuf& sb, cudaStream_t s) {
    if (sb.N > 0) k_s_acc_init<<<nblk(sb.N), NT, 0, s>>>(sb);
}

int launch_s_solve_scenes(const Scene& sc, const SplitBuf& sb, int gen, float alpha, int v, int max_iter, float tol,
                          const int32_t* spos, const int32_t* sflags, const int32_t* poff, const int32_t* order,
                          int nbmax, cudaStream_t s, float* scene_alpha, float alpha_ref, int4* scene_out) {
    if (!split_variant_is_scenes(v) || sc.nscenes <= 0) return (int)cudaErrorInvalidValue;
    ScenesVariant& cv = g_scenes[v - N_STREAM - N_COOP];
    // shared memory (contact-resident shapes): 48 B for each of up to 3 contacts a body (a settled
    // pile has about 2.3); larger scenes read their records from L1/L2
    int ccap = cv.csm ? 3 * nbmax : 0;
    if (48 * ccap > 227 * 1024) ccap = 0;
    const int smem = 48 * ccap;
    if (smem > 227 * 1024) return (int)cudaErrorInvalidValue;
    if (smem > 48 * 1024 && smem > cv.smem_set) {
        cudaError_t e = cudaFuncSetAttribute(cv.kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return (int)e;
        cv.smem_set = smem;
    }
    cv.kernel<<<sc.nscenes, cv.nth, smem, s>>>(sc, sb, gen, alpha, max_iter, tol, spos, sflags, poff, order,
                                              sc.max_statics, ccap, scene_alpha, alpha_ref > 0.f ? alpha_ref : alpha,
                                              scene_out);
    return (int)cudaGetLastError();
}

// grid of a streaming variant: one resident wave, or fewer blocks when there is less work
int split_contact_blocks(int vi, int64_t n, int sms) {
    StreamVariant& cv = g_stream[(vi >= 0 && vi < N_STREAM) ? vi : 0];
    if (cv.per_sm == 0) {
        int b = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, cv.kernel, cv.nth, 0);
        cv.per_sm = b > 0 ? b : 1;
    }
    const int64_t per_block = (int64_t)cv.nth * cv.unroll;
    const int64_t want = (n + per_block - 1) / per_block;
    int64_t cap = (int64_t)sms * cv.per_sm;
    if (cap > SPLIT_MAX_PARTS) cap = SPLIT_MAX_PARTS;
    return (int)(want < 1 ? 1 : (want < cap ? want : cap));
}

// Partition of a cooperative solve: one block per SM (all resident), contiguous contact and body
// ranges per block. Feasible when a block's contacts (48 B each) fit in its shared memory; its free
// velocities (32 B a body) are kept there too when they also fit.
// the shared-memory budget and residency of a cooperative kernel, queried once
template <class K>
static bool coop_setup(K kernel, int nth, int* per_sm, int* smem_max, int minb = 1) {
    if (*per_sm == 0) {
        int dev = 0, optin = 0, per_sm_smem = 0, reserved = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        cudaDeviceGetAttribute(&per_sm_smem, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
        cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev);
        cudaFuncAttributes fa;
        if (cudaFuncGetAttributes(&fa, kernel) != cudaSuccess) return false;
        *smem_max = optin - (int)fa.sharedSizeBytes;
        // several blocks an SM share its shared memory
        if (minb > 1) *smem_max = std::min(*smem_max, per_sm_smem / minb - reserved - (int)fa.sharedSizeBytes);
        if (*smem_max <= 0 ||
            cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, *smem_max) != cudaSuccess)
            return false;
        int b = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kernel, nth, *smem_max);
        *per_sm = b > 0 ? b : -1;
    }
    return *per_sm >= 1;
}

bool split_coop_plan(int v, int64_t nc, int64_t nbodies, int sms, CoopPlan* p, int smem_contacts, int blocks,
                     int loop) {
    if (!split_variant_is_coop(v) || nc <= 0) return false;
    CoopVariant& cv = g_coop[v - N_STREAM];
    int per_sm = 0, smem_max = 0;
    if (loop) {
        if (cv.nth != 1024 || cv.unroll != 1) return false;
        CoopLoopVariant& lv = g_coop_loop[cv.hyb][loop == 2 ? 1 : 0];
        if (!coop_setup(lv.kernel, cv.nth, &lv.per_sm, &lv.smem_max)) return false;
        per_sm = lv.per_sm;
        smem_max = lv.smem_max;
    } else {
        if (!coop_setup(cv.kernel, cv.nth, &cv.per_sm, &cv.smem_max, cv.minb)) return false;
        per_sm = cv.per_sm;
        smem_max = cv.smem_max;
    }
    const int64_t full = (int64_t)sms * per_sm;
    if (full > COOP_MAX_GRID) return false;
    // contacts a block keeps in shared memory: all that fit, or gpu.coop_smem_contacts
    const int64_t bpc = loop == 2 ? 64 : 48;
    int64_t fit = smem_max / bpc;
    if (smem_contacts > 0) fit = std::min<int64_t>(fit, smem_contacts);
    // one block per SM: on a 2k-contact pile a grid of 16-64 blocks measured the same per sweep
    // (3.0 us; the barrier's cost barely depends on the block count) and fewer blocks were slower
    const int64_t grid = blocks > 0 ? std::min<int64_t>(blocks, full) : full;
    int64_t cpb = (nc + grid - 1) / grid;
    const int64_t bpb = (nbodies + grid - 1) / grid;
    if (cv.hyb) {
        if (cpb <= fit) return false;  // it all fits: the plain cooperative shapes cover it
        cpb = fit;
    } else if (cpb > fit) {
        return false;
    }
    const int64_t need = cpb * bpc;
    if (need > smem_max || cpb < 1) return false;
    const bool vf = need + bpb * 32 <= smem_max;
    p->grid = (int)grid;
    p->nth = cv.nth;
    p->cpb = (int)cpb;
    p->bpb = (int)bpb;
    p->vf = vf ? 1 : 0;
    p->smem = (int)(need + (vf ? bpb * 32 : 0));
    return true;
}

int launch_s_solve_coop(const SplitBuf& sb, int gen, float alpha, int v, const CoopPlan& p, int max_iter, float tol,
                        int max_sweeps, int check_every, cudaStream_t s, unsigned long long wait_ns) {
    if (!split_variant_is_coop(v)) return (int)cudaErrorInvalidValue;
    const CoopVariant& cv = g_coop[v - N_STREAM];
    SplitBuf b = sb;
    int g = gen, mi = max_iter, cpb = p.cpb, bpb = p.bpb, vf = p.vf, ms = max_sweeps, ce = check_every > 0 ? check_every : 1;
    float al = alpha, t = tol;
    unsigned long long wn = wait_ns > 0 ? wait_ns : COOP_WAIT_NS;
    void* args[] = {&b, &g, &al, &mi, &t, &cpb, &bpb, &vf, &ms, &ce, &wn};
    return (int)cudaLaunchCooperativeKernel((const void*)cv.kernel, dim3(p.grid), dim3(cv.nth), args, (size_t)p.smem, s);
}

int launch_s_solve_coop_loop(const SplitBuf& sb, int gen, float alpha, int v, const CoopPlan& p, int max_iter,
                             float tol, int max_sweeps, int check_every, int loop, const CoopLoopArgs& la,
                             unsigned long long wait_ns, cudaStream_t s) {
    if (!split_variant_is_coop(v) || loop < 1 || loop > 2) return (int)cudaErrorInvalidValue;
    const CoopVariant& cv = g_coop[v - N_STREAM];
    if (cv.nth != 1024 || cv.unroll != 1) return (int)cudaErrorInvalidValue;
    const CoopLoopVariant& lv = g_coop_loop[cv.hyb][loop == 2 ? 1 : 0];
    SplitBuf b = sb;
    int g = gen, mi = max_iter, cpb = p.cpb, bpb = p.bpb, vf = p.vf, ms = max_sweeps, ce = check_every > 0 ? check_every : 1;
    float al = alpha, t = tol;
    CoopLoopArgs a = la;
    unsigned long long wn = wait_ns > 0 ? wait_ns : COOP_WAIT_NS;
    void* args[] = {&b, &g, &al, &mi, &t, &cpb, &bpb, &vf, &ms, &ce, &a, &wn};
    return (int)cudaLaunchCooperativeKernel((const void*)lv.kernel, dim3(p.grid), dim3(cv.nth), args, (size_t)p.smem, s);
}

void launch_s_prep(const Scene& sc, const SplitBuf& sb, double dt, const double* g, double h1, cudaStream_t s,
                   int implicit_gyro, const double* smot, const int32_t* smflag) {
    if (sc.N + sc.S == 0) return;
    k_s_prep<<<nblk(sc.N + sc.S), NT, 0, s>>>(sc, sb, dt, g[0], g[1], g[2], h1, implicit_gyro, smot, smflag);
}
void launch_s_static_flags(const Scene& sc, const SplitBuf& sb, float margin, double margin64, int32_t* flags,
                           cudaStream_t s) {
    if (sc.N == 0) return;
    k_s_static_flags<<<nblk(sc.N), NT, 0, s>>>(sc, sb, margin, margin64, flags);
}
void launch_s_pair_count(const Scene& sc, const Grid& g, const SplitBuf& sb, const uint32_t* cell_body,
                         const uint32_t* cell_key, const int32_t* cell_start, const int32_t* cell_end, int32_t* counts,
                         const SplitParams& P, DevScalars* ds, cudaStream_t s) {
    if (sc.N == 0) return;
    k_s_pairs<false><<<nblk(sc.N), NT, 0, s>>>(sc, g, sb, cell_body, cell_key, cell_start, cell_end, counts, nullptr, 0,
                                               0, P, ds);
}
void launch_s_static_write(const Scene& sc, const SplitBuf& sb, const int32_t* flags, const int32_t* pos, int gen,
                           const SplitParams& P, cudaStream_t s) {
    if (sc.N == 0) return;
    k_s_static_write<<<nblk(sc.N), NT, 0, s>>>(sc, sb, flags, pos, gen, P);
}
void launch_s_pair_write(const Scene& sc, const Grid& g, const SplitBuf& sb, const uint32_t* cell_body,
                         const uint32_t* cell_key, const int32_t* cell_start, const int32_t* cell_end,
                         const int32_t* offsets, int32_t base, int gen, const SplitParams& P, DevScalars* ds,
                         cudaStream_t s) {
    if (sc.N == 0) return;
    k_s_pairs<true><<<nblk(sc.N), NT, 0, s>>>(sc, g, sb, cell_body, cell_key, cell_start, cell_end, nullptr, offsets,
                                              base, gen, P, ds);
}
void launch_s_reset(const SplitBuf& sb, cudaStream_t s) { k_s_reset<<<1, 1, 0, s>>>(sb); }
void launch_s_end_step(const SplitBuf& sb, const DevScalars* ds, cudaStream_t s) {
    k_s_end_step<<<1, 1, 0, s>>>(sb, ds);
}
void launch_s_totals(const SplitBuf& sb, const int32_t* spos, const int32_t* sflags, int64_t nflag, const int32_t* poff,
                     int N, cudaStream_t s) {
    k_s_totals<<<1, 1, 0, s>>>(sb, spos, sflags, nflag, poff, N);
}
void launch_s_apply_warm(const SplitBuf& sb, int gen, int blocks, cudaStream_t s) {
    k_s_apply_warm<<<blocks, NT, 0, s>>>(sb, gen);
}
void launch_s_sweep(const SplitBuf& sb, int gen, float alpha, int variant, int blocks, int max_iter, float tol,
                    cudaGraphConditionalHandle h, int use_handle, cudaStream_t s) {
    const StreamVariant& cv = g_stream[(variant >= 0 && variant < N_STREAM) ? variant : 0];
    cv.kernel<<<blocks, cv.nth, 0, s>>>(sb, gen, alpha, max_iter, tol, h, use_handle);
}
void launch_s_final(const Scene& sc, const SplitBuf& sb, int gen, double alpha, int friction_enable, int combine,
                    int blocks, double drift_h, cudaStream_t s) {
    if (sc.N > 0) k_s_final_body<<<nblk(sc.N), NT, 0, s>>>(sc, sb);
    k_s_residual<<<blocks, NT, 0, s>>>(sc, sb, gen, alpha, friction_enable, combine);
    if (sc.N + sc.S > 0) k_s_writeback_drift<<<nblk(sc.N + sc.S), NT, 0, s>>>(sc, sb, drift_h);
    k_s_final_scalar<<<1, 1, 0, s>>>(sb);
}

}  // namespace cdx
