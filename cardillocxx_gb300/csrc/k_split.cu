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

#include "cdx_internal.h"
#include "fp64_math.cuh"
#include "split.h"

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
        const float a = 1.f / (1.f + n.z);
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

__device__ __forceinline__ void atomic_max_f(unsigned int* addr, float v) { atomicMax(addr, __float_as_uint(v)); }

// ------------------------------------------------------------------ per-body preparation (FP64)
__global__ void k_s_prep(Scene sc, SplitBuf sb, double dt, double g0, double g1, double g2, double h1) {
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
            wf[k] = w[k] + dt * ia * (-c[k]);
        }
        f64::drift(x, q, v, w, h1);
        sc.bf(BF_PX)[i] = x[0]; sc.bf(BF_PY)[i] = x[1]; sc.bf(BF_PZ)[i] = x[2];
        sc.bf(BF_QX)[i] = q[0]; sc.bf(BF_QY)[i] = q[1]; sc.bf(BF_QZ)[i] = q[2]; sc.bf(BF_QW)[i] = q[3];
        double R[9];
        f64::rotmat(q, R);
        for (int k = 0; k < 9; ++k) sc.bf(BF_R0 + k)[i] = R[k];
        // world-frame angular velocities: R w
        double ww[3], wfw[3];
        for (int k = 0; k < 3; ++k) {
            ww[k] = R[3 * k] * w[0] + R[3 * k + 1] * w[1] + R[3 * k + 2] * w[2];
            wfw[k] = R[3 * k] * wf[0] + R[3 * k + 1] * wf[1] + R[3 * k + 2] * wf[2];
        }
        for (int k = 0; k < 3; ++k) {
            sb.vfree[(size_t)k * N + i] = vf[k];
            sb.vfree[(size_t)(3 + k) * N + i] = wfw[k];
        }
        sb.vel4[2 * i] = make_float4((float)vf[0], (float)vf[1], (float)vf[2], (float)il);
        sb.vel4[2 * i + 1] = make_float4((float)wfw[0], (float)wfw[1], (float)wfw[2], (float)ia);
        sb.vn4[2 * i] = make_float4((float)v[0], (float)v[1], (float)v[2], 0.f);
        sb.vn4[2 * i + 1] = make_float4((float)ww[0], (float)ww[1], (float)ww[2], 0.f);
        sb.acc4[2 * i] = make_float4(0.f, 0.f, 0.f, 0.f);
        sb.acc4[2 * i + 1] = make_float4(0.f, 0.f, 0.f, 0.f);
        const int s = sc.body_scene[i];
        const double* o = &sb.origin[3 * s];
        sb.pos4[i] = make_float4((float)(x[0] - o[0]), (float)(x[1] - o[1]), (float)(x[2] - o[2]),
                                 (float)sc.bf(BF_RAD)[i]);
    } else if (i < sc.N + sc.S) {
        const int s = i - sc.N;
        double x[3] = {sc.sf(SF_PX)[s], sc.sf(SF_PY)[s], sc.sf(SF_PZ)[s]};
        double q[4] = {sc.sf(SF_QX)[s], sc.sf(SF_QY)[s], sc.sf(SF_QZ)[s], sc.sf(SF_QW)[s]};
        const double v[3] = {sc.sf(SF_VX)[s], sc.sf(SF_VY)[s], sc.sf(SF_VZ)[s]};
        const double w[3] = {sc.sf(SF_WX)[s], sc.sf(SF_WY)[s], sc.sf(SF_WZ)[s]};
        f64::drift(x, q, v, w, h1);
        sc.sf(SF_PX)[s] = x[0]; sc.sf(SF_PY)[s] = x[1]; sc.sf(SF_PZ)[s] = x[2];
        sc.sf(SF_QX)[s] = q[0]; sc.sf(SF_QY)[s] = q[1]; sc.sf(SF_QZ)[s] = q[2]; sc.sf(SF_QW)[s] = q[3];
        double R[9];
        f64::rotmat(q, R);
        for (int k = 0; k < 9; ++k) sc.sf(SF_R0 + k)[s] = R[k];
        double ww[3];
        for (int k = 0; k < 3; ++k) ww[k] = R[3 * k] * w[0] + R[3 * k + 1] * w[1] + R[3 * k + 2] * w[2];
        const int scn = sc.static_scene[s];
        const double* o = &sb.origin[3 * scn];
        const double u[3] = {sc.sf(SF_DX)[s], sc.sf(SF_DY)[s], sc.sf(SF_DZ)[s]};
        const double pl[3] = {x[0] - o[0], x[1] - o[1], x[2] - o[2]};
        const double dl = u[0] * pl[0] + u[1] * pl[1] + u[2] * pl[2];
        sb.st_dir[s] = make_float4((float)u[0], (float)u[1], (float)u[2], (float)dl);
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
    const float ax = dot(rel, u);
    const float3 perp = rel - ax * u;
    const float rho = sqrtf(dot(perp, perp));
    if (!(((pp.w - rho) - r) <= margin)) return false;
    g.n = rho > 0.f ? (-1.f / rho) * perp : make_float3(0.f, 0.f, 1.f);
    g.rhoB = -0.5f * ((pp.w - rho) + r);
    g.sep = rho;
    return true;
}

__global__ void k_s_static_flags(Scene sc, SplitBuf sb, float margin, int32_t* flags) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sc.N) return;
    const int s = sc.body_scene[i];
    const int b0 = sc.scene_body_start[s], ns_b = sc.scene_body_start[s + 1] - b0;
    const int st0 = sc.scene_static_start[s], nst = sc.scene_static_start[s + 1] - st0;
    const float4 p = sb.pos4[i];
    const int L = sc.max_statics;
    for (int l = 0; l < L; ++l) {
        int f = 0;
        if (l < nst) {
            CGeom32 g;
            f = static_test32(sb, st0 + l, f3(p), p.w, margin, g) ? 1 : 0;
        }
        flags[(size_t)b0 * L + (size_t)l * ns_b + (i - b0)] = f;
    }
}

__device__ __forceinline__ void warm_start(const SplitBuf& sb, int gen, int prev_count, unsigned long long key,
                                           float3 pt, float match2, float4& lam0) {
    lam0 = make_float4(0.f, 0.f, 0.f, 0.f);
    if (prev_count <= 0) return;
    const unsigned long long* pk = sb.key[gen ^ 1];
    int lo = 0, hi = prev_count;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (pk[mid] < key) lo = mid + 1;
        else hi = mid;
    }
    if (lo < prev_count && pk[lo] == key) {
        const float3 d = pt - f3(sb.pt[gen ^ 1][lo]);
        if (dot(d, d) <= match2) lam0 = sb.lam[gen ^ 1][lo];
    }
}

// rows' scaling, bias and warm start of one contact; side A body index a (< 0: static)
__device__ __forceinline__ void finish_contact32(const Scene& sc, SplitBuf& sb, int gen, int c, int a, int b,
                                                 float3 n, float rhoA, float rhoB, float3 pt, float mu_a,
                                                 float rn_a, float rt_a, const float3* wall_v, const float3* wall_w,
                                                 const float3* wall_p, const SplitParams& P) {
    const float4 vb = sb.vel4[2 * b], wb = sb.vel4[2 * b + 1];
    float ima = 0.f, iia = 0.f;
    float3 vna = make_float3(0.f, 0.f, 0.f), wna = vna;
    if (a >= 0) {
        ima = sb.vel4[2 * a].w;
        iia = sb.vel4[2 * a + 1].w;
        vna = f3(sb.vn4[2 * a]);
        wna = f3(sb.vn4[2 * a + 1]);
    }
    const float Dn = ima + vb.w;
    const float Dt = Dn + rhoA * rhoA * iia + rhoB * rhoB * wb.w;
    const float Rn = Dn > 0.f ? P.alpha / Dn : 0.f;
    const float Rt = Dt > 0.f ? P.alpha / Dt : 0.f;
    float mu = combine_mu32(P.combine, mu_a, (float)sc.bf(BF_MU)[b]);
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
    const float eN = fminf(fmaxf(0.f, rn_a), fmaxf(0.f, (float)sc.bf(BF_RN)[b]));
    const float eT = fminf(fmaxf(0.f, rt_a), fmaxf(0.f, (float)sc.bf(BF_RT)[b]));
    float4 bias = make_float4(Rn * cb[0], Rt * cb[1], Rt * cb[2], 0.f);
    if (eN > 0.f || eT > 0.f) {
        const float3 dv = f3(sb.vn4[2 * b]) - vna;
        const float3 Om = rhoB * f3(sb.vn4[2 * b + 1]) - rhoA * wna;
        const float vp0 = dot(n, dv) + cb[0];
        const float vp1 = dot(t1, dv) + dot(t2, Om) + cb[1];
        const float vp2 = dot(t2, dv) - dot(t1, Om) + cb[2];
        bias = make_float4(Rn * (cb[0] + eN * vp0), Rt * (cb[1] + eT * vp1), Rt * (cb[2] + eT * vp2), 0.f);
    }
    const uint32_t ida = a >= 0 ? (uint32_t)(sc.S + a) : (uint32_t)(-a - 1);
    const uint32_t idb = (uint32_t)(sc.S + b);
    const unsigned long long key = ((unsigned long long)ida << 32) | idb;
    float4 lam0;
    warm_start(sb, gen, P.prev_count, key, pt, P.match2, lam0);
    if (mu == 0.f) { lam0.y = 0.f; lam0.z = 0.f; }
    sb.ab[c] = make_int2(a, b);
    sb.nmu[c] = make_float4(n.x, n.y, n.z, mu);
    sb.levR[c] = make_float4(rhoA, rhoB, Rn, Rt);
    sb.bias[c] = bias;
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
        static_test32(sb, st, f3(p), p.w, P.margin, g);
        const float3 pt = f3(p) + g.rhoB * g.n;
        const float3 wv = f3(sb.st_v[st]), ww = f3(sb.st_w[st]), wp = f3(sb.st_pt[st]);
        const bool moving = (wv.x != 0.f || wv.y != 0.f || wv.z != 0.f || ww.x != 0.f || ww.y != 0.f || ww.z != 0.f);
        finish_contact32(sc, sb, gen, pos[slot], -st - 1, i, g.n, 0.f, g.rhoB, pt, sb.st_w[st].w,
                         (float)sc.sf(SF_RN)[st], (float)sc.sf(SF_RT)[st], moving ? &wv : nullptr, &ww, &wp, P);
    }
}

template <bool WRITE>
__global__ void k_s_pairs(Scene sc, Grid gr, SplitBuf sb, const uint32_t* cell_body, const int32_t* cell_start,
                          const int32_t* cell_end, int32_t* counts, const int32_t* offsets, int32_t base, int gen,
                          SplitParams P, DevScalars* ds) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sc.N) return;
    const float4 pi = sb.pos4[i];
    const int si = sc.body_scene[i];
    // cell of body i from its FP64 position (identical to the key kernel)
    int ci[3];
    {
        const double p[3] = {sc.bf(BF_PX)[i], sc.bf(BF_PY)[i], sc.bf(BF_PZ)[i]};
        for (int k = 0; k < 3; ++k) {
            double f = floor((p[k] - gr.lo[k]) / gr.cell);
            if (!(f >= 0.0)) f = 0.0;
            if (f > (double)(gr.dim[k] - 1)) f = (double)(gr.dim[k] - 1);
            ci[k] = (int)f;
        }
    }
    int list[MAX_PAIR];
    int cnt = 0;
    for (int dz = -1; dz <= 1; ++dz) {
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
                const float lim = pi.w + pj.w + P.margin;
                if (dx * dx + dy2 * dy2 + dz2 * dz2 > lim * lim) continue;
                if (sc.body_scene[j] != si) continue;
                if (WRITE) {
                    if (cnt < MAX_PAIR) list[cnt] = j;
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
    const int c0 = base + offsets[i];
    const float mu_a = (float)sc.bf(BF_MU)[i];
    const float rn_a = (float)sc.bf(BF_RN)[i], rt_a = (float)sc.bf(BF_RT)[i];
    for (int k = 0; k < cnt; ++k) {
        const int j = list[k];
        const float4 pj = sb.pos4[j];
        const float3 d = f3(pj) - f3(pi);
        const float dl = sqrtf(dot(d, d));
        const float3 n = dl > 0.f ? (1.f / dl) * d : make_float3(0.f, 0.f, 1.f);
        const float rhoA = 0.5f * (dl + pi.w - pj.w);
        const float rhoB = 0.5f * (pi.w - pj.w - dl);
        const float3 pt = f3(pi) + rhoA * n;
        finish_contact32(sc, sb, gen, c0 + k, i, j, n, rhoA, rhoB, pt, mu_a, rn_a, rt_a, nullptr, nullptr, nullptr, P);
    }
}

// ------------------------------------------------------------------ projected Jacobi (FP32)
// apply W^T dl (pre-scaled by M^-1) to the bodies of contact c with float4/float2 vector atomics
__device__ __forceinline__ void scatter(SplitBuf& sb, int a, int b, float3 n, float3 t1, float3 t2, float rhoA,
                                        float rhoB, float dln, float dlt1, float dlt2, float imb, float iib, float ima,
                                        float iia) {
    const float3 P = dln * n + dlt1 * t1 + dlt2 * t2;
    const float3 tau = dlt1 * t2 - dlt2 * t1;
    {
        const float s = rhoB * iib;
        atomicAdd(&sb.acc4[2 * b], make_float4(imb * P.x, imb * P.y, imb * P.z, s * tau.x));
        atomicAdd(reinterpret_cast<float2*>(&sb.acc4[2 * b + 1]), make_float2(s * tau.y, s * tau.z));
    }
    if (a >= 0) {
        const float s = -rhoA * iia;
        atomicAdd(&sb.acc4[2 * a], make_float4(-ima * P.x, -ima * P.y, -ima * P.z, s * tau.x));
        atomicAdd(reinterpret_cast<float2*>(&sb.acc4[2 * a + 1]), make_float2(s * tau.y, s * tau.z));
    }
}

__global__ void k_s_apply_warm(SplitBuf sb, int gen) {
    const int nc = *sb.nc_dev;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
        const float4 l = sb.lam[gen][c];
        if (l.x == 0.f && l.y == 0.f && l.z == 0.f) continue;
        const int2 ab = sb.ab[c];
        const float4 nm = sb.nmu[c], lr = sb.levR[c];
        const float3 n = f3(nm);
        float3 t1, t2;
        frame32(n, t1, t2);
        const float imb = sb.vel4[2 * ab.y].w, iib = sb.vel4[2 * ab.y + 1].w;
        float ima = 0.f, iia = 0.f;
        if (ab.x >= 0) {
            ima = sb.vel4[2 * ab.x].w;
            iia = sb.vel4[2 * ab.x + 1].w;
        }
        scatter(sb, ab.x, ab.y, n, t1, t2, lr.x, lr.y, l.x, l.y, l.z, imb, iib, ima, iia);
    }
}

__global__ void __launch_bounds__(NT) k_s_contact(SplitBuf sb, int gen) {
    if (*(volatile int32_t*)&sb.ss->done) return;
    const int nc = *sb.nc_dev;
    float maxd = 0.f, maxl = 0.f;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
        const int2 ab = sb.ab[c];
        const float4 nm = sb.nmu[c];
        const float4 lr = sb.levR[c];
        const float4 bs = sb.bias[c];
        const float4 l = sb.lam[gen][c];
        const float3 n = f3(nm);
        float3 t1, t2;
        frame32(n, t1, t2);
        const float4 vb = sb.vel4[2 * ab.y], wb = sb.vel4[2 * ab.y + 1];
        float3 dv = f3(vb);
        float3 Om = lr.y * f3(wb);
        float ima = 0.f, iia = 0.f;
        if (ab.x >= 0) {
            const float4 va = sb.vel4[2 * ab.x], wa = sb.vel4[2 * ab.x + 1];
            dv = dv - f3(va);
            Om = Om - lr.x * f3(wa);
            ima = va.w;
            iia = wa.w;
        }
        const float gn = dot(n, dv) + bs.x;
        const float gt1 = dot(t1, dv) + dot(t2, Om) + bs.y;
        const float gt2 = dot(t2, dv) - dot(t1, Om) + bs.z;
        float ln = fmaxf(l.x - lr.z * gn, 0.f);
        float lt1 = l.y - lr.w * gt1;
        float lt2 = l.z - lr.w * gt2;
        const float tn2 = lt1 * lt1 + lt2 * lt2;
        if (tn2 > 0.f) {
            const float s = fminf(1.f, nm.w * ln * rsqrtf(tn2));
            lt1 *= s;
            lt2 *= s;
        }
        const float dln = ln - l.x, dlt1 = lt1 - l.y, dlt2 = lt2 - l.z;
        sb.lam[gen][c] = make_float4(ln, lt1, lt2, 0.f);
        maxd = fmaxf(maxd, sqrtf(dln * dln + dlt1 * dlt1 + dlt2 * dlt2));
        maxl = fmaxf(maxl, fmaxf(fabsf(l.x), fmaxf(fabsf(l.y), fabsf(l.z))));
        if (dln != 0.f || dlt1 != 0.f || dlt2 != 0.f)
            scatter(sb, ab.x, ab.y, n, t1, t2, lr.x, lr.y, dln, dlt1, dlt2, vb.w, wb.w, ima, iia);
    }
    for (int o = 16; o > 0; o >>= 1) {
        maxd = fmaxf(maxd, __shfl_xor_sync(0xffffffffu, maxd, o));
        maxl = fmaxf(maxl, __shfl_xor_sync(0xffffffffu, maxl, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomic_max_f(&sb.ss->maxd, maxd);
        atomic_max_f(&sb.ss->maxl, maxl);
    }
}

__global__ void k_s_body(SplitBuf sb, int N, int apply_only) {
    if (!apply_only && *(volatile int32_t*)&sb.ss->done) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        const float4 a0 = sb.acc4[2 * i], a1 = sb.acc4[2 * i + 1];
        float4 v = sb.vel4[2 * i], w = sb.vel4[2 * i + 1];
        v.x += a0.x; v.y += a0.y; v.z += a0.z;
        w.x += a0.w; w.y += a1.x; w.z += a1.y;
        sb.vel4[2 * i] = v;
        sb.vel4[2 * i + 1] = w;
        sb.acc4[2 * i] = make_float4(0.f, 0.f, 0.f, 0.f);
        sb.acc4[2 * i + 1] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

__global__ void k_s_check(SplitBuf sb, int max_iter, float tol, cudaGraphConditionalHandle handle, int use_handle) {
    SplitScalars* ss = sb.ss;
    if (!ss->done) {
        const float maxd = __uint_as_float(ss->maxd), maxl = __uint_as_float(ss->maxl);
        const float r = maxd / fmaxf(maxl, 1e-30f);
        ss->res_last = r;
        ss->iters += 1;
        if (ss->iters >= max_iter || (tol > 0.f && r <= tol) || !(r == r)) ss->done = 1;
    }
    ss->maxd = 0u;
    ss->maxl = 0u;
    if (use_handle) cudaGraphSetConditional(handle, ss->done ? 0u : 1u);
}

__global__ void k_s_reset(SplitBuf sb) {
    SplitScalars* ss = sb.ss;
    ss->done = (*sb.nc_dev == 0) ? 1 : 0;
    ss->iters = 0;
    ss->maxd = 0u;
    ss->maxl = 0u;
    ss->res_last = 0.f;
    ss->maxd64 = 0ull;
    ss->maxl64 = 0ull;
}

// ------------------------------------------------------------------ FP64 finalisation
// FP64 contact geometry recomputed from FP64 positions (the same formulas as the plain method)
__device__ __forceinline__ void geom64(const Scene& sc, int a, int b, double* n, double& rhoA, double& rhoB) {
    const double xb[3] = {sc.bf(BF_PX)[b], sc.bf(BF_PY)[b], sc.bf(BF_PZ)[b]};
    const double rb = sc.bf(BF_RAD)[b];
    if (a >= 0) {
        const double xa[3] = {sc.bf(BF_PX)[a], sc.bf(BF_PY)[a], sc.bf(BF_PZ)[a]};
        const double ra = sc.bf(BF_RAD)[a];
        double d[3] = {xb[0] - xa[0], xb[1] - xa[1], xb[2] - xa[2]};
        const double dl = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        if (dl > 0.0) { n[0] = d[0] / dl; n[1] = d[1] / dl; n[2] = d[2] / dl; }
        else { n[0] = 0; n[1] = 0; n[2] = 1; }
        rhoA = 0.5 * (dl + ra - rb);
        rhoB = 0.5 * (ra - rb - dl);
        return;
    }
    const int s = -a - 1;
    const double u[3] = {sc.sf(SF_DX)[s], sc.sf(SF_DY)[s], sc.sf(SF_DZ)[s]};
    rhoA = 0.0;
    if (sc.static_kind[s] == 0) {
        const double sd = (u[0] * xb[0] + u[1] * xb[1] + u[2] * xb[2]) - sc.sf(SF_D)[s];
        n[0] = u[0]; n[1] = u[1]; n[2] = u[2];
        rhoB = -0.5 * (sd + rb);
        return;
    }
    const double p[3] = {sc.sf(SF_PX)[s], sc.sf(SF_PY)[s], sc.sf(SF_PZ)[s]};
    const double rel[3] = {xb[0] - p[0], xb[1] - p[1], xb[2] - p[2]};
    const double ax = rel[0] * u[0] + rel[1] * u[1] + rel[2] * u[2];
    const double perp[3] = {rel[0] - ax * u[0], rel[1] - ax * u[1], rel[2] - ax * u[2]};
    const double rho = sqrt(perp[0] * perp[0] + perp[1] * perp[1] + perp[2] * perp[2]);
    if (rho > 0.0) { n[0] = -perp[0] / rho; n[1] = -perp[1] / rho; n[2] = -perp[2] / rho; }
    else { n[0] = 0; n[1] = 0; n[2] = 1; }
    rhoB = -0.5 * ((sc.sf(SF_RAD)[s] - rho) + rb);
}

__device__ __forceinline__ void frame64(const double* n, double* t1, double* t2) {
    if (n[2] < -0.9999999) {
        t1[0] = 0; t1[1] = -1; t1[2] = 0;
        const double d = n[0] * t1[0] + n[1] * t1[1] + n[2] * t1[2];
        for (int k = 0; k < 3; ++k) t1[k] -= n[k] * d;
    } else {
        const double a = 1.0 / (1.0 + n[2]);
        const double b = (-n[0] * n[1]) * a;
        t1[0] = 1.0 - (n[0] * n[0]) * a;
        t1[1] = b;
        t1[2] = -n[0];
    }
    const double s = 1.0 / sqrt(t1[0] * t1[0] + t1[1] * t1[1] + t1[2] * t1[2]);
    for (int k = 0; k < 3; ++k) t1[k] *= s;
    f64::cross3(n, t1, t2);
}

__global__ void k_s_final_w(Scene sc, SplitBuf sb, int gen) {
    const int nc = *sb.nc_dev;
    const int N = sc.N;
    const int64_t cap = sb.cap;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
        const int2 ab = sb.ab[c];
        double n[3], rA, rB;
        geom64(sc, ab.x, ab.y, n, rA, rB);
        for (int k = 0; k < 3; ++k) sb.g64[k * cap + c] = n[k];
        sb.g64[3 * cap + c] = rA;
        sb.g64[4 * cap + c] = rB;
        const float4 l = sb.lam[gen][c];
        if (l.x == 0.f && l.y == 0.f && l.z == 0.f) continue;
        double t1[3], t2[3];
        frame64(n, t1, t2);
        double P[3], tau[3];
        for (int k = 0; k < 3; ++k) {
            P[k] = (double)l.x * n[k] + (double)l.y * t1[k] + (double)l.z * t2[k];
            tau[k] = (double)l.y * t2[k] - (double)l.z * t1[k];
        }
        for (int k = 0; k < 3; ++k) {
            atomicAdd(&sb.acc64[(size_t)k * N + ab.y], P[k]);
            atomicAdd(&sb.acc64[(size_t)(3 + k) * N + ab.y], rB * tau[k]);
        }
        if (ab.x >= 0) {
            for (int k = 0; k < 3; ++k) {
                atomicAdd(&sb.acc64[(size_t)k * N + ab.x], -P[k]);
                atomicAdd(&sb.acc64[(size_t)(3 + k) * N + ab.x], -rA * tau[k]);
            }
        }
    }
}

// v = v_free + M^-1 W^T lambda (world frame), in place of the accumulators
__global__ void k_s_final_body(Scene sc, SplitBuf sb) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sc.N) return;
    const int N = sc.N;
    const double il = sc.bf(BF_MINVL)[i], ia = sc.bf(BF_MINVA)[i];
    for (int k = 0; k < 3; ++k) {
        const size_t jl = (size_t)k * N + i, ja = (size_t)(3 + k) * N + i;
        sb.acc64[jl] = sb.vfree[jl] + il * sb.acc64[jl];
        sb.acc64[ja] = sb.vfree[ja] + ia * sb.acc64[ja];
    }
}

// FP64 complementarity residual of (lambda, v): max_c ||lambda_c - Pi(lambda_c - R(W v + b))|| / max |lambda|
__global__ void k_s_residual(Scene sc, SplitBuf sb, int gen, double alpha, int friction_enable, int combine) {
    const int nc = *sb.nc_dev;
    const int N = sc.N;
    const int64_t cap = sb.cap;
    double maxd = 0.0, maxl = 0.0;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
        const int2 ab = sb.ab[c];
        const double n[3] = {sb.g64[c], sb.g64[cap + c], sb.g64[2 * cap + c]};
        const double rA = sb.g64[3 * cap + c], rB = sb.g64[4 * cap + c];
        double t1[3], t2[3];
        frame64(n, t1, t2);
        double dv[3], Om[3];
        for (int k = 0; k < 3; ++k) {
            dv[k] = sb.acc64[(size_t)k * N + ab.y];
            Om[k] = rB * sb.acc64[(size_t)(3 + k) * N + ab.y];
        }
        double ima = 0.0, iia = 0.0;
        if (ab.x >= 0) {
            for (int k = 0; k < 3; ++k) {
                dv[k] -= sb.acc64[(size_t)k * N + ab.x];
                Om[k] -= rA * sb.acc64[(size_t)(3 + k) * N + ab.x];
            }
            ima = sc.bf(BF_MINVL)[ab.x];
            iia = sc.bf(BF_MINVA)[ab.x];
        }
        const double imb = sc.bf(BF_MINVL)[ab.y], iib = sc.bf(BF_MINVA)[ab.y];
        const double Dn = ima + imb, Dt = Dn + rA * rA * iia + rB * rB * iib;
        const double Rn = Dn > 0 ? alpha / Dn : 0.0, Rt = Dt > 0 ? alpha / Dt : 0.0;
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
            eN = fmin(fmax(0.0, sc.sf(SF_RN)[s]), fmax(0.0, sc.bf(BF_RN)[ab.y]));
            eT = fmin(fmax(0.0, sc.sf(SF_RT)[s]), fmax(0.0, sc.bf(BF_RT)[ab.y]));
        } else {
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
        const double mu = sb.nmu[c].w;
        double ln = lo[0] - Rn * (g[0] + bias[0]);
        double lt1 = lo[1] - Rt * (g[1] + bias[1]);
        double lt2 = lo[2] - Rt * (g[2] + bias[2]);
        ln = ln < 0.0 ? 0.0 : ln;
        const double tn2 = lt1 * lt1 + lt2 * lt2;
        if (tn2 > 0.0) {
            const double s = fmin(1.0, (mu * ln) / sqrt(tn2));
            lt1 *= s;
            lt2 *= s;
        }
        const double d0 = ln - lo[0], d1 = lt1 - lo[1], d2 = lt2 - lo[2];
        maxd = fmax(maxd, sqrt(d0 * d0 + d1 * d1 + d2 * d2));
        maxl = fmax(maxl, fmax(fabs(lo[0]), fmax(fabs(lo[1]), fabs(lo[2]))));
    }
    (void)friction_enable;
    (void)combine;
    for (int o = 16; o > 0; o >>= 1) {
        maxd = fmax(maxd, __shfl_xor_sync(0xffffffffu, maxd, o));
        maxl = fmax(maxl, __shfl_xor_sync(0xffffffffu, maxl, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(&sb.ss->maxd64, (unsigned long long)__double_as_longlong(maxd));
        atomicMax(&sb.ss->maxl64, (unsigned long long)__double_as_longlong(maxl));
    }
}

// write the FP64 velocities back into the state (angular velocity to the body frame)
__global__ void k_s_writeback(Scene sc, SplitBuf sb) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sc.N) return;
    const int N = sc.N;
    double R[9];
    for (int k = 0; k < 9; ++k) R[k] = sc.bf(BF_R0 + k)[i];
    const double ww[3] = {sb.acc64[3 * (size_t)N + i], sb.acc64[4 * (size_t)N + i], sb.acc64[5 * (size_t)N + i]};
    double wb[3];
    f64::matTvec(R, ww, wb);
    sc.bf(BF_VX)[i] = sb.acc64[i];
    sc.bf(BF_VY)[i] = sb.acc64[(size_t)N + i];
    sc.bf(BF_VZ)[i] = sb.acc64[2 * (size_t)N + i];
    sc.bf(BF_WX)[i] = wb[0];
    sc.bf(BF_WY)[i] = wb[1];
    sc.bf(BF_WZ)[i] = wb[2];
}

__global__ void k_s_final_scalar(SplitBuf sb) {
    SplitScalars* ss = sb.ss;
    const double maxd = __longlong_as_double((long long)ss->maxd64);
    const double maxl = __longlong_as_double((long long)ss->maxl64);
    ss->res_final = maxd / fmax(maxl, 1e-30);
}

}  // namespace

int split_grid_blocks(int64_t n, int sms) {
    const int64_t want = (n + NT - 1) / NT;
    const int64_t cap = (int64_t)sms * 8;
    return (int)(want < 1 ? 1 : (want < cap ? want : cap));
}

void launch_s_prep(const Scene& sc, const SplitBuf& sb, double dt, const double* g, double h1, cudaStream_t s) {
    if (sc.N + sc.S == 0) return;
    k_s_prep<<<nblk(sc.N + sc.S), NT, 0, s>>>(sc, sb, dt, g[0], g[1], g[2], h1);
}
void launch_s_static_flags(const Scene& sc, const SplitBuf& sb, float margin, int32_t* flags, cudaStream_t s) {
    if (sc.N == 0) return;
    k_s_static_flags<<<nblk(sc.N), NT, 0, s>>>(sc, sb, margin, flags);
}
void launch_s_pair_count(const Scene& sc, const Grid& g, const SplitBuf& sb, const uint32_t* cell_body,
                         const int32_t* cell_start, const int32_t* cell_end, int32_t* counts, const SplitParams& P,
                         DevScalars* ds, cudaStream_t s) {
    if (sc.N == 0) return;
    k_s_pairs<false><<<nblk(sc.N), NT, 0, s>>>(sc, g, sb, cell_body, cell_start, cell_end, counts, nullptr, 0, 0, P, ds);
}
void launch_s_static_write(const Scene& sc, const SplitBuf& sb, const int32_t* flags, const int32_t* pos, int gen,
                           const SplitParams& P, cudaStream_t s) {
    if (sc.N == 0) return;
    k_s_static_write<<<nblk(sc.N), NT, 0, s>>>(sc, sb, flags, pos, gen, P);
}
void launch_s_pair_write(const Scene& sc, const Grid& g, const SplitBuf& sb, const uint32_t* cell_body,
                         const int32_t* cell_start, const int32_t* cell_end, const int32_t* offsets, int32_t base,
                         int gen, const SplitParams& P, DevScalars* ds, cudaStream_t s) {
    if (sc.N == 0) return;
    k_s_pairs<true><<<nblk(sc.N), NT, 0, s>>>(sc, g, sb, cell_body, cell_start, cell_end, nullptr, offsets, base, gen, P,
                                              ds);
}
void launch_s_reset(const SplitBuf& sb, cudaStream_t s) { k_s_reset<<<1, 1, 0, s>>>(sb); }
void launch_s_apply_warm(const SplitBuf& sb, int gen, int blocks, cudaStream_t s) {
    k_s_apply_warm<<<blocks, NT, 0, s>>>(sb, gen);
}
void launch_s_contact(const SplitBuf& sb, int gen, int blocks, cudaStream_t s) {
    k_s_contact<<<blocks, NT, 0, s>>>(sb, gen);
}
void launch_s_body(const SplitBuf& sb, int N, int blocks, int apply_only, cudaStream_t s) {
    k_s_body<<<blocks, NT, 0, s>>>(sb, N, apply_only);
}
void launch_s_check(const SplitBuf& sb, int max_iter, float tol, cudaGraphConditionalHandle h, int use_handle,
                    cudaStream_t s) {
    k_s_check<<<1, 1, 0, s>>>(sb, max_iter, tol, h, use_handle);
}
void launch_s_final(const Scene& sc, const SplitBuf& sb, int gen, double alpha, int friction_enable, int combine,
                    int blocks, cudaStream_t s) {
    if (sc.N > 0) cudaMemsetAsync(sb.acc64, 0, sizeof(double) * 6 * (size_t)sc.N, s);
    k_s_final_w<<<blocks, NT, 0, s>>>(sc, sb, gen);
    if (sc.N > 0) k_s_final_body<<<nblk(sc.N), NT, 0, s>>>(sc, sb);
    k_s_residual<<<blocks, NT, 0, s>>>(sc, sb, gen, alpha, friction_enable, combine);
    if (sc.N > 0) k_s_writeback<<<nblk(sc.N), NT, 0, s>>>(sc, sb);
    k_s_final_scalar<<<1, 1, 0, s>>>(sb);
}

}  // namespace cdx
