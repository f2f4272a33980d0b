// Differentiable rollout for sphere scenes: the forward step with iterate storage and its
// hand-written reverse. One block per scene, FP64, compiled with --fmad=false: every operation is
// rounded as written, in the order the CPU FP64 adjoint performs it.
//
// The step (world-frame angular velocities; the sphere's orientation does not enter the motion):
//   x_m = x + (1 - theta) h v                                   integration_base.cpp:6-30
//   contacts of x_m: (halfspace, sphere) then pairs (i, j), i < j  collision_coal.cpp:112-163
//   x_0 = (v + h g, omega), lambda_0 = 0                         pj_assembler.cpp:127-182
//   K sweeps (projected_jacobi.cpp:121-138, 100-119, 371-377):
//     y = W x_k, lambda' = lambda_k - R y, lambda_{k+1} = Pi(lambda'),
//     x_{k+1} = x_k + M^-1 W^T (lambda_{k+1} - lambda_k)
//   v' = x_K, omega' = x_K, x' = x_m + theta h v'                moreau.cpp:6-13
// with W x = (n.dv, t1.dv + t2.Om, t2.dv - t1.Om), dv = v_B - v_A, Om = rho_B w_B - rho_A w_A,
// rho the signed lever length along n from each centre to the contact midpoint, (t1, t2) the
// Frisvad frame of n (tangent_frame.hpp:23-50) and R = alpha / diag(W M^-1 W^T)
// (projected_jacobi.cpp:57-69).
//
// The reverse runs the sweeps backwards from the stored iterates: per sweep the adjoint of x_{k+1}
// gives w = W M^-1 xbar to the impulses, the disk projection is differentiated through its branch
// (separating: 0, sticking: identity, sliding: lambda_t = mu lambda'_n b/|b|), and
// xbar += W^T ybar with ybar = -R lambdabar'. The geometry adjoints (n, t1, t2, rho, R_t) are
// summed per contact over all sweeps, then mapped to the midpoint positions through the Frisvad
// Jacobian (forward-mode dual numbers) and d(n, rho)/d(x_A, x_B).
#include <cuda_runtime.h>

#include "adjoint.h"

namespace cdx {
namespace {

__device__ __forceinline__ double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// forward-mode dual number with three partials
struct D3 {
    double v, d[3];
};
__device__ __forceinline__ D3 dc(double v) { return {v, {0.0, 0.0, 0.0}}; }
__device__ __forceinline__ D3 operator+(D3 a, D3 b) {
    return {a.v + b.v, {a.d[0] + b.d[0], a.d[1] + b.d[1], a.d[2] + b.d[2]}};
}
__device__ __forceinline__ D3 operator-(D3 a, D3 b) {
    return {a.v - b.v, {a.d[0] - b.d[0], a.d[1] - b.d[1], a.d[2] - b.d[2]}};
}
__device__ __forceinline__ D3 operator-(D3 a) { return {-a.v, {-a.d[0], -a.d[1], -a.d[2]}}; }
__device__ __forceinline__ D3 operator*(D3 a, D3 b) {
    return {a.v * b.v, {a.d[0] * b.v + a.v * b.d[0], a.d[1] * b.v + a.v * b.d[1], a.d[2] * b.v + a.v * b.d[2]}};
}
__device__ __forceinline__ D3 operator/(D3 a, D3 b) {
    const double q = a.v / b.v;
    return {q, {(a.d[0] - q * b.d[0]) / b.v, (a.d[1] - q * b.d[1]) / b.v, (a.d[2] - q * b.d[2]) / b.v}};
}
__device__ __forceinline__ D3 dsqrt(D3 a) {
    const double s = sqrt(a.v);
    const double k = s > 0.0 ? 0.5 / s : 0.0;
    return {s, {a.d[0] * k, a.d[1] * k, a.d[2] * k}};
}
__device__ __forceinline__ double dsqrt(double a) { return sqrt(a); }
__device__ __forceinline__ double val(double a) { return a; }
__device__ __forceinline__ double val(D3 a) { return a.v; }
template <class T>
__device__ __forceinline__ T cst(double v);
template <>
__device__ __forceinline__ double cst<double>(double v) {
    return v;
}
template <>
__device__ __forceinline__ D3 cst<D3>(double v) {
    return dc(v);
}

// tangentFrameFromNormal (tangent_frame.hpp:23-50) over a generic scalar
template <class T>
__device__ void frame(const T* nin, T* t1, T* t2) {
    const T len = dsqrt(nin[0] * nin[0] + nin[1] * nin[1] + nin[2] * nin[2]);
    const T n[3] = {nin[0] / len, nin[1] / len, nin[2] / len};
    if (val(n[2]) < -0.9999999) {
        const T e[3] = {cst<T>(0.0), cst<T>(-1.0), cst<T>(0.0)};
        const T d = n[0] * e[0] + n[1] * e[1] + n[2] * e[2];
        for (int k = 0; k < 3; ++k) t1[k] = e[k] - n[k] * d;
    } else {
        const T one = cst<T>(1.0);
        const T a = one / (one + n[2]);
        const T b = (-n[0] * n[1]) * a;
        t1[0] = one - (n[0] * n[0]) * a;
        t1[1] = b;
        t1[2] = -n[0];
    }
    const T tt = t1[0] * t1[0] + t1[1] * t1[1] + t1[2] * t1[2];
    if (val(tt) > 0.0) {
        const T s = dsqrt(tt);
        for (int k = 0; k < 3; ++k) t1[k] = t1[k] / s;
    }
    t2[0] = n[1] * t1[2] - n[2] * t1[1];
    t2[1] = n[2] * t1[0] - n[0] * t1[2];
    t2[2] = n[0] * t1[1] - n[1] * t1[0];
}

// contact view: the geometry of contact c (global index)
struct CV {
    int a, b;
    double n[3], t1[3], t2[3], rA, rB;
};
__device__ __forceinline__ CV load_cv(const AdjStep& W, int c) {
    CV v;
    v.a = W.ca[c];
    v.b = W.cb[c];
    for (int k = 0; k < 3; ++k) {
        v.n[k] = W.cn[3 * c + k];
        v.t1[k] = W.ct1[3 * c + k];
        v.t2[k] = W.ct2[3 * c + k];
    }
    v.rA = W.cg[5 * c];
    v.rB = W.cg[5 * c + 1];
    return v;
}

// y = W_c x, the two bodies' 6-vectors given (A absent for a halfspace)
__device__ __forceinline__ void wx(const CV& c, const double* xa, const double* xb, double* y) {
    double dv[3], Om[3];
    for (int k = 0; k < 3; ++k) {
        const double va = c.a >= 0 ? xa[k] : 0.0, wa = c.a >= 0 ? xa[3 + k] : 0.0;
        dv[k] = xb[k] - va;
        Om[k] = c.rB * xb[3 + k] - c.rA * wa;
    }
    y[0] = dot3(c.n, dv);
    y[1] = dot3(c.t1, dv) + dot3(c.t2, Om);
    y[2] = dot3(c.t2, dv) - dot3(c.t1, Om);
}

// accumulate d(m . W z)/d(geometry): geo = gn[3], gt1[3], gt2[3], grA, grB, gRt
__device__ __forceinline__ void geo_acc(const CV& c, const double* m, const double* za, const double* zb, double* geo) {
    double dz[3], Oz[3], wa[3] = {0.0, 0.0, 0.0}, wb[3];
    for (int k = 0; k < 3; ++k) {
        const double va = c.a >= 0 ? za[k] : 0.0;
        if (c.a >= 0) wa[k] = za[3 + k];
        wb[k] = zb[3 + k];
        dz[k] = zb[k] - va;
        Oz[k] = c.rB * wb[k] - c.rA * wa[k];
    }
    double tm[3];
    for (int k = 0; k < 3; ++k) {
        geo[k] += m[0] * dz[k];
        geo[3 + k] += m[1] * dz[k] - m[2] * Oz[k];
        geo[6 + k] += m[1] * Oz[k] + m[2] * dz[k];
        tm[k] = m[1] * c.t2[k] - m[2] * c.t1[k];
    }
    geo[10] += dot3(tm, wb);
    geo[9] -= dot3(tm, wa);
}

__device__ __forceinline__ void project(const double* lp, double mu, double* out) {
    const double ln = fmax(lp[0], 0.0);
    double l1 = lp[1], l2 = lp[2];
    const double tn2 = l1 * l1 + l2 * l2;
    if (tn2 > 0.0) {
        const double sc = fmin(1.0, mu * ln / sqrt(tn2));
        l1 *= sc;
        l2 *= sc;
    }
    out[0] = ln;
    out[1] = l1;
    out[2] = l2;
}

__device__ __forceinline__ void project_adj(const double* lp, double mu, const double* lb, double* lpb, double* mub) {
    lpb[0] = lpb[1] = lpb[2] = 0.0;
    *mub = 0.0;
    const double ln = fmax(lp[0], 0.0);
    if (!(lp[0] > 0.0)) return;  // separating
    const double tn2 = lp[1] * lp[1] + lp[2] * lp[2];
    const double s = sqrt(tn2);
    if (!(tn2 > 0.0) || !(mu * ln / s < 1.0)) {  // sticking
        for (int k = 0; k < 3; ++k) lpb[k] = lb[k];
        return;
    }
    const double bh0 = lp[1] / s, bh1 = lp[2] / s;
    const double bl = bh0 * lb[1] + bh1 * lb[2];
    lpb[0] = lb[0] + mu * bl;
    const double f = mu * ln / s;
    lpb[1] = f * (lb[1] - bh0 * bl);
    lpb[2] = f * (lb[2] - bh1 * bl);
    *mub = ln * bl;
}

// W_c^T m for one side of contact c: linear and angular parts (scaled by sm, si when given)
__device__ __forceinline__ void wtm_side(const CV& c, const double* m, int side, double sm, double si, double* acc) {
    double P[3], tau[3];
    for (int k = 0; k < 3; ++k) {
        P[k] = m[0] * c.n[k] + m[1] * c.t1[k] + m[2] * c.t2[k];
        tau[k] = m[1] * c.t2[k] - m[2] * c.t1[k];
    }
    if (side) {
        for (int k = 0; k < 3; ++k) {
            acc[k] += sm * P[k];
            acc[3 + k] += si * c.rB * tau[k];
        }
    } else {
        for (int k = 0; k < 3; ++k) {
            acc[k] -= sm * P[k];
            acc[3 + k] -= si * c.rA * tau[k];
        }
    }
}

// block-wide exclusive scan of a[0..n) in shared memory; returns the total (all threads)
__device__ int block_scan(int* a, int n, int* part) {
    const int T = blockDim.x, t = threadIdx.x;
    const int per = (n + T - 1) / T;
    const int lo = min(n, t * per), hi = min(n, lo + per);
    int s = 0;
    for (int i = lo; i < hi; ++i) s += a[i];
    part[t] = s;
    __syncthreads();
    if (t == 0) {
        int run = 0;
        for (int k = 0; k < T; ++k) {
            const int v = part[k];
            part[k] = run;
            run += v;
        }
        part[T] = run;
    }
    __syncthreads();
    int run = part[t];
    for (int i = lo; i < hi; ++i) {
        const int v = a[i];
        a[i] = run;
        run += v;
    }
    const int total = part[T];
    __syncthreads();
    return total;
}

struct Smem {
    double* X;   // 6 nbmax
    double* Y;   // 3 nbmax (x_m forward, gx_m backward)
    double* U;   // 6 nbmax (backward)
    int* cnt;    // nbmax + 1
    int* cur;    // nbmax + 1
    int* part;   // ADJ_THREADS + 1
    int* misc;   // 4
};
__device__ __forceinline__ Smem carve(int nbmax) {
    extern __shared__ double smd[];
    Smem S;
    S.X = smd;
    S.Y = S.X + 6 * nbmax;
    S.U = S.Y + 3 * nbmax;
    S.cnt = reinterpret_cast<int*>(S.U + 6 * nbmax);
    S.cur = S.cnt + nbmax + 1;
    S.part = S.cur + nbmax + 1;
    S.misc = S.part + ADJ_THREADS + 1;
    return S;
}

template <int STORE>
__global__ void __launch_bounds__(ADJ_THREADS) k_adj_step(AdjProblem P, AdjStep W, const double* mu, const double* x,
                                                          const double* v, const double* w, double* xo, double* vo,
                                                          double* wo, int count, int nbmax) {
    const Smem S = carve(nbmax);
    const int sc = blockIdx.x, t = threadIdx.x, T = blockDim.x;
    const int b0 = P.body_off[sc], nb = P.body_off[sc + 1] - b0;
    const int s0 = P.static_off[sc], ns = P.static_off[sc + 1] - s0;
    const int c0 = P.contact_off[sc], cap = P.contact_off[sc + 1] - c0;
    const double hd = (1.0 - P.theta) * P.h;
    for (int i = t; i < nb; i += T) {
        const int b = b0 + i;
        for (int k = 0; k < 3; ++k) {
            S.Y[3 * i + k] = x[3 * b + k] + hd * v[3 * b + k];
            S.X[6 * i + k] = v[3 * b + k] + P.h * P.g[k];
            S.X[6 * i + 3 + k] = w[3 * b + k];
        }
    }
    __syncthreads();
    // contacts: halfspaces in (halfspace, sphere) order
    int nc = 0;
    for (int q = 0; q < ns; ++q) {
        const int si = s0 + q;
        const double* u = &P.su[3 * si];
        for (int i = t; i < nb; i += T) {
            const double sd = dot3(u, &S.Y[3 * i]) - P.soff[si];
            S.cnt[i] = (sd - P.rad[b0 + i] <= P.margin) ? 1 : 0;
        }
        __syncthreads();
        for (int i = t; i < nb; i += T) S.cur[i] = S.cnt[i];
        const int tot = block_scan(S.cnt, nb, S.part);
        for (int i = t; i < nb; i += T) {
            if (!S.cur[i]) continue;
            const int k = nc + S.cnt[i];
            if (k >= cap) continue;
            const int c = c0 + k;
            const double sd = dot3(u, &S.Y[3 * i]) - P.soff[si];
            W.ca[c] = -1;
            W.cb[c] = b0 + i;
            W.cs[c] = si;
            for (int j = 0; j < 3; ++j) W.cn[3 * c + j] = u[j];
            W.cg[5 * c] = 0.0;
            W.cg[5 * c + 1] = -0.5 * (sd + P.rad[b0 + i]);
            W.cg[5 * c + 2] = 0.0;
        }
        nc += tot;
        __syncthreads();
    }
    // sphere pairs in (i, j) order, i < j. A pair farther apart than (r_i + r_j + |margin|)
    // (1 + 1e-9) in squared distance cannot pass the exact test (its rounding errors are below
    // 1e-15 relative), so the square root is taken only for near pairs; the same d2 feeds it.
    for (int i = t; i < nb; i += T) {
        int n = 0;
        const double ri = P.rad[b0 + i];
        for (int j = i + 1; j < nb; ++j) {
            double d[3];
            for (int k = 0; k < 3; ++k) d[k] = S.Y[3 * j + k] - S.Y[3 * i + k];
            const double d2 = dot3(d, d);
            const double lim = (ri + P.rad[b0 + j] + fabs(P.margin)) * (1.0 + 1e-9);
            if (d2 > lim * lim) continue;
            const double L = sqrt(d2);
            if ((L - ri) - P.rad[b0 + j] <= P.margin && L > 0.0) ++n;
        }
        S.cnt[i] = n;
    }
    __syncthreads();
    const int ptot = block_scan(S.cnt, nb, S.part);
    for (int i = t; i < nb; i += T) {
        int k = nc + S.cnt[i];
        const double ri = P.rad[b0 + i];
        for (int j = i + 1; j < nb; ++j) {
            double d[3];
            for (int q = 0; q < 3; ++q) d[q] = S.Y[3 * j + q] - S.Y[3 * i + q];
            const double rj = P.rad[b0 + j];
            const double d2 = dot3(d, d);
            const double lim = (ri + rj + fabs(P.margin)) * (1.0 + 1e-9);
            if (d2 > lim * lim) continue;
            const double L = sqrt(d2);
            if (!((L - ri) - rj <= P.margin && L > 0.0)) continue;
            if (k < cap) {
                const int c = c0 + k;
                W.ca[c] = b0 + i;
                W.cb[c] = b0 + j;
                W.cs[c] = -1;
                for (int q = 0; q < 3; ++q) W.cn[3 * c + q] = d[q] / L;
                W.cg[5 * c] = 0.5 * (L + ri - rj);
                W.cg[5 * c + 1] = 0.5 * (ri - rj - L);
                W.cg[5 * c + 2] = L;
            }
            ++k;
        }
    }
    nc += ptot;
    if (nc > cap) {
        if (t == 0) *W.err = 1;
        nc = cap;
    }
    if (t == 0) {
        W.nc[sc] = nc;
        if (count) W.ncsum[sc] += nc;
    }
    __syncthreads();
    // frame and R per contact
    for (int k = t; k < nc; k += T) {
        const int c = c0 + k;
        double n[3], t1[3], t2[3];
        for (int q = 0; q < 3; ++q) n[q] = W.cn[3 * c + q];
        frame(n, t1, t2);
        for (int q = 0; q < 3; ++q) {
            W.ct1[3 * c + q] = t1[q];
            W.ct2[3 * c + q] = t2[q];
        }
        const int a = W.ca[c], b = W.cb[c];
        const double rA = W.cg[5 * c], rB = W.cg[5 * c + 1];
        const double ima = a >= 0 ? P.minv[a] : 0.0, iia = a >= 0 ? P.iinv[a] : 0.0;
        const double Dn = ima + P.minv[b];
        const double Dt = Dn + rA * rA * iia + rB * rB * P.iinv[b];
        W.cg[5 * c + 3] = P.alpha / Dn;
        W.cg[5 * c + 4] = P.alpha / Dt;
        for (int q = 0; q < 3; ++q) W.lam[3 * c + q] = 0.0;
    }
    // incidence lists in contact order (deterministic gathers)
    for (int i = t; i <= nb; i += T) S.cnt[i] = 0;
    __syncthreads();
    for (int k = t; k < nc; k += T) {
        const int c = c0 + k;
        atomicAdd(&S.cnt[W.cb[c] - b0], 1);
        if (W.ca[c] >= 0) atomicAdd(&S.cnt[W.ca[c] - b0], 1);
    }
    __syncthreads();
    const int itot = block_scan(S.cnt, nb, S.part);
    int* ioff = W.inc_off + b0 + sc;
    int* inc = W.inc + 2 * (int64_t)c0;
    for (int i = t; i < nb; i += T) {
        ioff[i] = S.cnt[i];
        S.cur[i] = S.cnt[i];
    }
    if (t == 0) ioff[nb] = itot;
    __syncthreads();
    for (int k = t; k < nc; k += T) {
        const int c = c0 + k;
        inc[atomicAdd(&S.cur[W.cb[c] - b0], 1)] = (k << 1) | 1;
        if (W.ca[c] >= 0) inc[atomicAdd(&S.cur[W.ca[c] - b0], 1)] = (k << 1);
    }
    __syncthreads();
    for (int i = t; i < nb; i += T) {
        const int lo = S.cnt[i], hi = (i + 1 < nb) ? S.cnt[i + 1] : itot;
        for (int p = lo + 1; p < hi; ++p) {
            const int key = inc[p];
            int q = p - 1;
            while (q >= lo && inc[q] > key) {
                inc[q + 1] = inc[q];
                --q;
            }
            inc[q + 1] = key;
        }
    }
    const int64_t N6 = 6 * (int64_t)P.N, cap3 = 3 * W.cap;
    if (STORE) {
        for (int i = t; i < 6 * nb; i += T) W.xs[6 * (int64_t)b0 + i] = S.X[i];
        for (int k = t; k < 3 * nc; k += T) W.ls[3 * (int64_t)c0 + k] = 0.0;
    }
    __syncthreads();
    const double mus = mu[sc];
    for (int it = 0; it < P.K; ++it) {
        for (int k = t; k < nc; k += T) {
            const int c = c0 + k;
            const CV cv = load_cv(W, c);
            const double Rn = W.cg[5 * c + 3], Rt = W.cg[5 * c + 4];
            double y[3], lp[3], ln[3];
            wx(cv, cv.a >= 0 ? &S.X[6 * (cv.a - b0)] : nullptr, &S.X[6 * (cv.b - b0)], y);
            lp[0] = W.lam[3 * c] - Rn * y[0];
            lp[1] = W.lam[3 * c + 1] - Rt * y[1];
            lp[2] = W.lam[3 * c + 2] - Rt * y[2];
            project(lp, mus, ln);
            for (int q = 0; q < 3; ++q) {
                W.dl[3 * c + q] = ln[q] - W.lam[3 * c + q];
                W.lam[3 * c + q] = ln[q];
            }
        }
        __syncthreads();
        for (int i = t; i < nb; i += T) {
            double acc[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
            const int b = b0 + i;
            for (int p = ioff[i]; p < ioff[i + 1]; ++p) {
                const int e = inc[p], c = c0 + (e >> 1);
                const CV cv = load_cv(W, c);
                wtm_side(cv, &W.dl[3 * c], e & 1, P.minv[b], P.iinv[b], acc);
            }
            for (int q = 0; q < 6; ++q) S.X[6 * i + q] += acc[q];
        }
        __syncthreads();
        if (STORE) {
            for (int i = t; i < 6 * nb; i += T) W.xs[(it + 1) * N6 + 6 * (int64_t)b0 + i] = S.X[i];
            for (int k = t; k < 3 * nc; k += T) W.ls[(it + 1) * cap3 + 3 * (int64_t)c0 + k] = W.lam[3 * (int64_t)c0 + k];
        }
    }
    const double hn = P.theta * P.h;
    for (int i = t; i < nb; i += T) {
        const int b = b0 + i;
        for (int k = 0; k < 3; ++k) {
            vo[3 * b + k] = S.X[6 * i + k];
            wo[3 * b + k] = S.X[6 * i + 3 + k];
            xo[3 * b + k] = S.Y[3 * i + k] + hn * S.X[6 * i + k];
        }
    }
}

__global__ void __launch_bounds__(ADJ_THREADS) k_adj_back(AdjProblem P, AdjStep W, const double* mu, double* gx,
                                                          double* gv, double* gw, double* gmu, int nbmax) {
    const Smem S = carve(nbmax);
    const int sc = blockIdx.x, t = threadIdx.x, T = blockDim.x;
    const int b0 = P.body_off[sc], nb = P.body_off[sc + 1] - b0;
    const int c0 = P.contact_off[sc];
    const int nc = W.nc[sc];
    const int* ioff = W.inc_off + b0 + sc;
    const int* inc = W.inc + 2 * (int64_t)c0;
    const int64_t N6 = 6 * (int64_t)P.N, cap3 = 3 * W.cap;
    const double hn = P.theta * P.h;
    for (int i = t; i < nb; i += T) {
        const int b = b0 + i;
        for (int k = 0; k < 3; ++k) {
            S.Y[3 * i + k] = gx[3 * b + k];
            S.X[6 * i + k] = gv[3 * b + k] + hn * gx[3 * b + k];
            S.X[6 * i + 3 + k] = gw[3 * b + k];
        }
    }
    for (int k = t; k < nc; k += T) {
        const int c = c0 + k;
        for (int q = 0; q < 12; ++q) W.geo[12 * (int64_t)c + q] = 0.0;
        for (int q = 0; q < 3; ++q) W.lbar[3 * c + q] = 0.0;
    }
    const double mus = mu[sc];
    double mub_t = 0.0;
    __syncthreads();
    for (int it = P.K - 1; it >= 0; --it) {
        const double* Xk = W.xs + it * N6;
        const double* lk = W.ls + it * cap3;
        const double* lk1 = W.ls + (it + 1) * cap3;
        for (int i = t; i < nb; i += T) {
            const int b = b0 + i;
            for (int q = 0; q < 3; ++q) {
                S.U[6 * i + q] = P.minv[b] * S.X[6 * i + q];
                S.U[6 * i + 3 + q] = P.iinv[b] * S.X[6 * i + 3 + q];
            }
        }
        __syncthreads();
        for (int k = t; k < nc; k += T) {
            const int c = c0 + k;
            const CV cv = load_cv(W, c);
            const double Rn = W.cg[5 * c + 3], Rt = W.cg[5 * c + 4];
            double* geo = &W.geo[12 * (int64_t)c];
            double* Lb = &W.lbar[3 * c];
            const double* ua = cv.a >= 0 ? &S.U[6 * (cv.a - b0)] : nullptr;
            const double* ub = &S.U[6 * (cv.b - b0)];
            const double* xa = cv.a >= 0 ? &Xk[6 * (int64_t)cv.a] : nullptr;
            const double* xb = &Xk[6 * (int64_t)cv.b];
            double wv[3], dl[3], y[3], lp[3], lpb[3], mub;
            wx(cv, ua, ub, wv);
            for (int q = 0; q < 3; ++q) dl[q] = lk1[3 * c + q] - lk[3 * c + q];
            geo_acc(cv, dl, ua, ub, geo);
            for (int q = 0; q < 3; ++q) Lb[q] += wv[q];
            wx(cv, xa, xb, y);
            lp[0] = lk[3 * c] - Rn * y[0];
            lp[1] = lk[3 * c + 1] - Rt * y[1];
            lp[2] = lk[3 * c + 2] - Rt * y[2];
            project_adj(lp, mus, Lb, lpb, &mub);
            mub_t += mub;
            const double yb[3] = {-Rn * lpb[0], -Rt * lpb[1], -Rt * lpb[2]};
            geo[11] -= lpb[1] * y[1] + lpb[2] * y[2];
            geo_acc(cv, yb, xa, xb, geo);
            for (int q = 0; q < 3; ++q) {
                Lb[q] = -wv[q] + lpb[q];
                W.dl[3 * c + q] = yb[q];
            }
        }
        __syncthreads();
        for (int i = t; i < nb; i += T) {
            double acc[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
            for (int p = ioff[i]; p < ioff[i + 1]; ++p) {
                const int e = inc[p], c = c0 + (e >> 1);
                const CV cv = load_cv(W, c);
                wtm_side(cv, &W.dl[3 * c], e & 1, 1.0, 1.0, acc);
            }
            for (int q = 0; q < 6; ++q) S.X[6 * i + q] += acc[q];
        }
        __syncthreads();
    }
    // geometry adjoints -> position adjoint per contact
    for (int k = t; k < nc; k += T) {
        const int c = c0 + k;
        const CV cv = load_cv(W, c);
        const double* g = &W.geo[12 * (int64_t)c];
        const double Rt = W.cg[5 * c + 4], L = W.cg[5 * c + 2];
        const double iia = cv.a >= 0 ? P.iinv[cv.a] : 0.0;
        const double kk = -Rt * Rt / P.alpha;
        const double rAb = g[9] + g[11] * kk * 2.0 * cv.rA * iia;
        const double rBb = g[10] + g[11] * kk * 2.0 * cv.rB * P.iinv[cv.b];
        double* db = &W.dbar[3 * c];
        if (cv.a < 0) {
            for (int q = 0; q < 3; ++q) db[q] = -0.5 * rBb * cv.n[q];
            continue;
        }
        D3 nd[3], t1d[3], t2d[3];
        for (int q = 0; q < 3; ++q) {
            nd[q] = dc(cv.n[q]);
            nd[q].d[q] = 1.0;
        }
        frame(nd, t1d, t2d);
        double nb3[3];
        for (int q = 0; q < 3; ++q) {
            nb3[q] = g[q];
            for (int r = 0; r < 3; ++r) nb3[q] += t1d[r].d[q] * g[3 + r] + t2d[r].d[q] * g[6 + r];
        }
        const double nn = dot3(cv.n, nb3);
        for (int q = 0; q < 3; ++q) db[q] = (nb3[q] - cv.n[q] * nn) / L + cv.n[q] * (0.5 * rAb - 0.5 * rBb);
    }
    __syncthreads();
    for (int i = t; i < nb; i += T) {
        for (int p = ioff[i]; p < ioff[i + 1]; ++p) {
            const int e = inc[p], c = c0 + (e >> 1);
            const double* db = &W.dbar[3 * c];
            if (e & 1) {
                for (int q = 0; q < 3; ++q) S.Y[3 * i + q] += db[q];
            } else {
                for (int q = 0; q < 3; ++q) S.Y[3 * i + q] -= db[q];
            }
        }
    }
    __syncthreads();
    const double hd = (1.0 - P.theta) * P.h;
    for (int i = t; i < nb; i += T) {
        const int b = b0 + i;
        for (int q = 0; q < 3; ++q) {
            gx[3 * b + q] = S.Y[3 * i + q];
            gv[3 * b + q] = S.X[6 * i + q] + hd * S.Y[3 * i + q];
            gw[3 * b + q] = S.X[6 * i + 3 + q];
        }
    }
    // the scene's friction adjoint: fixed-order block reduction
    double* red = S.U;
    red[t] = mub_t;
    __syncthreads();
    if (t == 0) {
        double s = 0.0;
        for (int k = 0; k < T; ++k) s += red[k];
        gmu[sc] += s;
    }
}

}  // namespace

int adj_smem_bytes(int nbmax) {
    return (int)(sizeof(double) * 15 * (size_t)nbmax + sizeof(int) * (2 * (size_t)nbmax + 2 + ADJ_THREADS + 1 + 4));
}

void launch_adj_step(const AdjProblem& P, const AdjStep& W, const double* mu, const double* x, const double* v,
                     const double* w, double* xo, double* vo, double* wo, int store, int count, int nbmax,
                     cudaStream_t s) {
    if (P.nsc == 0) return;
    const int smem = adj_smem_bytes(nbmax);
    if (store)
        k_adj_step<1><<<P.nsc, ADJ_THREADS, smem, s>>>(P, W, mu, x, v, w, xo, vo, wo, count, nbmax);
    else
        k_adj_step<0><<<P.nsc, ADJ_THREADS, smem, s>>>(P, W, mu, x, v, w, xo, vo, wo, count, nbmax);
}

void launch_adj_back(const AdjProblem& P, const AdjStep& W, const double* mu, double* gx, double* gv, double* gw,
                     double* gmu, int nbmax, cudaStream_t s) {
    if (P.nsc == 0) return;
    k_adj_back<<<P.nsc, ADJ_THREADS, adj_smem_bytes(nbmax), s>>>(P, W, mu, gx, gv, gw, gmu, nbmax);
}

int adj_set_smem_limit(int smem) {
    cudaError_t e1 = cudaFuncSetAttribute(k_adj_step<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaError_t e2 = cudaFuncSetAttribute(k_adj_step<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaError_t e3 = cudaFuncSetAttribute(k_adj_back, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    return (e1 != cudaSuccess) ? (int)e1 : (e2 != cudaSuccess) ? (int)e2 : (int)e3;
}

}  // namespace cdx
