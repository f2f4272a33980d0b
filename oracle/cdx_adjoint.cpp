// FP64 CPU adjoint of the Moreau midpoint step for sphere scenes: the checker for the GPU adjoint.
//
// TEST INFRASTRUCTURE ONLY (see cdx_oracle.h): only tests/ load it.
//
// The differentiated map is one time step of CardilloCxx's path for spheres and halfspaces
// (moreau.cpp:6-13, integration_base.cpp:6-30, collision_coal.cpp:112-163 for the contact,
// dynamics_assembler.cpp:211-332 for the rows, projected_jacobi.cpp:57-69,100-138,371-377 for the
// solver) written on world-frame angular velocities:
//   x_m  = x + (1 - theta) h v
//   contacts of x_m (fixed set, canonical order: (halfspace, sphere) then (i, j) with i < j)
//   x_0  = x_free = (v + h g, omega)            (lambda_0 = 0: no warm start)
//   K sweeps: y = W x_k; lambda' = lambda_k - R y; lambda_{k+1} = Pi(lambda'); x_{k+1} = x_k + M^-1 W^T (lambda_{k+1} - lambda_k)
//   v' = x_K (linear), omega' = x_K (angular);  x' = x_m + theta h v'
// For a sphere the rotation only maps body to world angular velocity, and the quaternion drift
// rotates about omega_body itself, so omega_world is unchanged by the drift: the world-frame state
// (x, v, omega_world) evolves on its own and the orientation does not enter the loss.
// The gyroscopic force -omega x (I omega) of an isotropic sphere is zero (and so is its
// derivative) and is left out. Restitution and moving walls are not part of this model.
//
// Contact geometry (coal's sphere rules as the oracle restates them):
//   pair:      d = x_B - x_A, L = |d|, n = d / L, rho_A = (L + r_A - r_B) / 2, rho_B = (r_A - r_B - L) / 2
//   halfspace: n = u (plane normal), s = u.x_B - off, rho_B = -(s + r_B) / 2
// (rho = signed lever length along n from the body centre to the contact midpoint), Frisvad
// frame (t1, t2) of n (tangent_frame.hpp:23-50), and
//   W x = (n.dv, t1.dv + t2.Om, t2.dv - t1.Om), dv = v_B - v_A, Om = rho_B w_B - rho_A w_A
//   R_n = alpha / (1/m_A + 1/m_B), R_t = alpha / (1/m_A + 1/m_B + rho_A^2 / I_A + rho_B^2 / I_B)
// The disk projection Pi (projected_jacobi.cpp:100-119) is differentiated branch by branch:
// separating (lambda'_n <= 0: zero Jacobian), sticking (identity), sliding
// (lambda_t = mu lambda'_n b / |b|).
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "cdx_oracle.h"

namespace {

// forward-mode dual number with three partials (Jacobian of the tangent frame)
struct D3 {
    double v, d[3];
};
inline D3 dc(double v) { return {v, {0, 0, 0}}; }
inline D3 operator+(D3 a, D3 b) { return {a.v + b.v, {a.d[0] + b.d[0], a.d[1] + b.d[1], a.d[2] + b.d[2]}}; }
inline D3 operator-(D3 a, D3 b) { return {a.v - b.v, {a.d[0] - b.d[0], a.d[1] - b.d[1], a.d[2] - b.d[2]}}; }
inline D3 operator-(D3 a) { return {-a.v, {-a.d[0], -a.d[1], -a.d[2]}}; }
inline D3 operator*(D3 a, D3 b) {
    return {a.v * b.v, {a.d[0] * b.v + a.v * b.d[0], a.d[1] * b.v + a.v * b.d[1], a.d[2] * b.v + a.v * b.d[2]}};
}
inline D3 operator/(D3 a, D3 b) {
    const double q = a.v / b.v;
    return {q, {(a.d[0] - q * b.d[0]) / b.v, (a.d[1] - q * b.d[1]) / b.v, (a.d[2] - q * b.d[2]) / b.v}};
}
inline D3 dsqrt(D3 a) {
    const double s = std::sqrt(a.v);
    const double k = s > 0 ? 0.5 / s : 0.0;
    return {s, {a.d[0] * k, a.d[1] * k, a.d[2] * k}};
}
inline double val(double x) { return x; }
inline double val(D3 x) { return x.v; }
inline double dsqrt(double x) { return std::sqrt(x); }
template <class T> T cst(double v);
template <> double cst<double>(double v) { return v; }
template <> D3 cst<D3>(double v) { return dc(v); }

// tangentFrameFromNormal (tangent_frame.hpp:23-50), generic over the scalar type
template <class T>
void frame(const T* nin, T* t1, T* t2) {
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

struct Contact {
    int a, b;  // body indices (a = -1 for a halfspace)
    int st;    // halfspace index or -1
    double n[3], t1[3], t2[3], rA, rB, L, Rn, Rt, mu;
    double Jt1[9], Jt2[9];  // d t / d n (row k = component k)
};

struct Model {
    int N = 0, S = 0, nsc = 0, K = 0;
    double h = 0, g[3] = {0, 0, 0}, theta = 0.5, alpha = 0.5, margin = 0;
    std::vector<double> rad, minv, iinv, su, soff;
    std::vector<int> scene, sscene;
};

inline double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

void detect(const Model& M, const double* xm, const double* mu_scene, std::vector<Contact>& C) {
    C.clear();
    for (int s = 0; s < M.S; ++s)
        for (int i = 0; i < M.N; ++i) {
            if (M.scene[i] != M.sscene[s]) continue;
            const double* u = &M.su[3 * s];
            const double sd = dot3(u, &xm[3 * i]) - M.soff[s];
            if (!(sd - M.rad[i] <= M.margin)) continue;
            Contact c{};
            c.a = -1;
            c.b = i;
            c.st = s;
            for (int k = 0; k < 3; ++k) c.n[k] = u[k];
            c.rA = 0.0;
            c.rB = -0.5 * (sd + M.rad[i]);
            c.L = 0.0;
            C.push_back(c);
        }
    for (int i = 0; i < M.N; ++i)
        for (int j = i + 1; j < M.N; ++j) {
            if (M.scene[i] != M.scene[j]) continue;
            double d[3];
            for (int k = 0; k < 3; ++k) d[k] = xm[3 * j + k] - xm[3 * i + k];
            const double L = std::sqrt(dot3(d, d));
            if (!((L - M.rad[i]) - M.rad[j] <= M.margin) || !(L > 0.0)) continue;
            Contact c{};
            c.a = i;
            c.b = j;
            c.st = -1;
            for (int k = 0; k < 3; ++k) c.n[k] = d[k] / L;
            c.L = L;
            c.rA = 0.5 * (L + M.rad[i] - M.rad[j]);
            c.rB = 0.5 * (M.rad[i] - M.rad[j] - L);
            C.push_back(c);
        }
    for (auto& c : C) {
        frame(c.n, c.t1, c.t2);
        D3 nd[3], t1d[3], t2d[3];
        for (int k = 0; k < 3; ++k) {
            nd[k] = dc(c.n[k]);
            nd[k].d[k] = 1.0;
        }
        frame(nd, t1d, t2d);
        for (int r = 0; r < 3; ++r)
            for (int k = 0; k < 3; ++k) {
                c.Jt1[3 * r + k] = t1d[r].d[k];
                c.Jt2[3 * r + k] = t2d[r].d[k];
            }
        const double ima = c.a >= 0 ? M.minv[c.a] : 0.0, iia = c.a >= 0 ? M.iinv[c.a] : 0.0;
        const double Dn = ima + M.minv[c.b];
        const double Dt = Dn + c.rA * c.rA * iia + c.rB * c.rB * M.iinv[c.b];
        c.Rn = M.alpha / Dn;
        c.Rt = M.alpha / Dt;
        c.mu = mu_scene[M.scene[c.b]];
    }
}

// y = W_c x (x: 6 doubles per body, v then omega)
void wx(const Contact& c, const double* X, double* y) {
    double dv[3], Om[3];
    for (int k = 0; k < 3; ++k) {
        const double va = c.a >= 0 ? X[6 * c.a + k] : 0.0, wa = c.a >= 0 ? X[6 * c.a + 3 + k] : 0.0;
        dv[k] = X[6 * c.b + k] - va;
        Om[k] = c.rB * X[6 * c.b + 3 + k] - c.rA * wa;
    }
    y[0] = dot3(c.n, dv);
    y[1] = dot3(c.t1, dv) + dot3(c.t2, Om);
    y[2] = dot3(c.t2, dv) - dot3(c.t1, Om);
}

// dst += M^-1-free W_c^T m into the 6-vectors of the two bodies, scaled per body by scl (M^-1 or 1)
void wtm(const Contact& c, const double* m, double* dst, const Model& Mo, bool scale) {
    double P[3], tau[3];
    for (int k = 0; k < 3; ++k) {
        P[k] = m[0] * c.n[k] + m[1] * c.t1[k] + m[2] * c.t2[k];
        tau[k] = m[1] * c.t2[k] - m[2] * c.t1[k];
    }
    const double smb = scale ? Mo.minv[c.b] : 1.0, sib = scale ? Mo.iinv[c.b] : 1.0;
    for (int k = 0; k < 3; ++k) {
        dst[6 * c.b + k] += smb * P[k];
        dst[6 * c.b + 3 + k] += sib * c.rB * tau[k];
    }
    if (c.a >= 0) {
        const double sma = scale ? Mo.minv[c.a] : 1.0, sia = scale ? Mo.iinv[c.a] : 1.0;
        for (int k = 0; k < 3; ++k) {
            dst[6 * c.a + k] -= sma * P[k];
            dst[6 * c.a + 3 + k] -= sia * c.rA * tau[k];
        }
    }
}

void project(const double* lp, double mu, double* out) {
    const double ln = std::fmax(lp[0], 0.0);
    double l1 = lp[1], l2 = lp[2];
    const double tn2 = l1 * l1 + l2 * l2;
    if (tn2 > 0.0) {
        const double sc = std::fmin(1.0, mu * ln / std::sqrt(tn2));
        l1 *= sc;
        l2 *= sc;
    }
    out[0] = ln;
    out[1] = l1;
    out[2] = l2;
}

// adjoint of project: lbar (adjoint of the output) -> lpbar (adjoint of the input), mubar
void project_adj(const double* lp, double mu, const double* lbar, double* lpbar, double* mubar) {
    lpbar[0] = lpbar[1] = lpbar[2] = 0.0;
    *mubar = 0.0;
    const double ln = std::fmax(lp[0], 0.0);
    if (!(lp[0] > 0.0)) return;  // separating
    const double tn2 = lp[1] * lp[1] + lp[2] * lp[2];
    const double s = std::sqrt(tn2);
    if (!(tn2 > 0.0) || !(mu * ln / s < 1.0)) {  // sticking
        for (int k = 0; k < 3; ++k) lpbar[k] = lbar[k];
        return;
    }
    const double bh[2] = {lp[1] / s, lp[2] / s};
    const double bl = bh[0] * lbar[1] + bh[1] * lbar[2];
    lpbar[0] = lbar[0] + mu * bl;
    const double f = mu * ln / s;
    lpbar[1] = f * (lbar[1] - bh[0] * bl);
    lpbar[2] = f * (lbar[2] - bh[1] * bl);
    *mubar = ln * bl;
}

struct Geo {
    double gn[3], gt1[3], gt2[3], grA, grB, gRt;
};

// accumulate d(m . W z)/d(geometry) of contact c
void geo_acc(const Contact& c, const double* m, const double* Z, Geo& G) {
    double dz[3], Oz[3], wa[3] = {0, 0, 0}, wb[3];
    for (int k = 0; k < 3; ++k) {
        const double va = c.a >= 0 ? Z[6 * c.a + k] : 0.0;
        if (c.a >= 0) wa[k] = Z[6 * c.a + 3 + k];
        wb[k] = Z[6 * c.b + 3 + k];
        dz[k] = Z[6 * c.b + k] - va;
        Oz[k] = c.rB * wb[k] - c.rA * wa[k];
    }
    double tm[3];
    for (int k = 0; k < 3; ++k) {
        G.gn[k] += m[0] * dz[k];
        G.gt1[k] += m[1] * dz[k] - m[2] * Oz[k];
        G.gt2[k] += m[1] * Oz[k] + m[2] * dz[k];
        tm[k] = m[1] * c.t2[k] - m[2] * c.t1[k];
    }
    G.grB += dot3(tm, wb);
    G.grA -= dot3(tm, wa);
}

struct StepStore {
    std::vector<Contact> C;
    std::vector<double> xm, X, lam;  // X: (K+1) x 6N, lam: (K+1) x 3nc
};

// one step; with st != nullptr every iterate is kept for the backward pass
void step(const Model& M, const double* mu, const double* x, const double* v, const double* w, double* xo,
          double* vo, double* wo, StepStore* st) {
    const int N = M.N;
    std::vector<double> xm(3 * N);
    for (int i = 0; i < 3 * N; ++i) xm[i] = x[i] + (1.0 - M.theta) * M.h * v[i];
    std::vector<Contact> C;
    detect(M, xm.data(), mu, C);
    const int nc = (int)C.size();
    std::vector<double> X(6 * N), lam(3 * nc, 0.0), dl(3 * nc), inc(6 * N);
    for (int i = 0; i < N; ++i)
        for (int k = 0; k < 3; ++k) {
            X[6 * i + k] = v[3 * i + k] + M.h * M.g[k];
            X[6 * i + 3 + k] = w[3 * i + k];
        }
    if (st) {
        st->X.assign(X.begin(), X.end());
        st->lam.assign(lam.begin(), lam.end());
    }
    for (int it = 0; it < M.K; ++it) {
        for (int c = 0; c < nc; ++c) {
            double y[3], lp[3], ln[3];
            wx(C[c], X.data(), y);
            lp[0] = lam[3 * c] - C[c].Rn * y[0];
            lp[1] = lam[3 * c + 1] - C[c].Rt * y[1];
            lp[2] = lam[3 * c + 2] - C[c].Rt * y[2];
            project(lp, C[c].mu, ln);
            for (int k = 0; k < 3; ++k) {
                dl[3 * c + k] = ln[k] - lam[3 * c + k];
                lam[3 * c + k] = ln[k];
            }
        }
        std::fill(inc.begin(), inc.end(), 0.0);
        for (int c = 0; c < nc; ++c) wtm(C[c], &dl[3 * c], inc.data(), M, true);
        for (int i = 0; i < 6 * N; ++i) X[i] += inc[i];
        if (st) {
            st->X.insert(st->X.end(), X.begin(), X.end());
            st->lam.insert(st->lam.end(), lam.begin(), lam.end());
        }
    }
    for (int i = 0; i < N; ++i)
        for (int k = 0; k < 3; ++k) {
            vo[3 * i + k] = X[6 * i + k];
            wo[3 * i + k] = X[6 * i + 3 + k];
            xo[3 * i + k] = xm[3 * i + k] + M.theta * M.h * vo[3 * i + k];
        }
    if (st) {
        st->C = C;
        st->xm = xm;
    }
}

// reverse of one step: (gx, gv, gw) hold the adjoint of the step's outputs on entry and of its
// inputs on return; gmu accumulates per scene
void step_back(const Model& M, const StepStore& st, double* gx, double* gv, double* gw, double* gmu) {
    const int N = M.N, K = M.K;
    const int nc = (int)st.C.size();
    std::vector<double> gxm(gx, gx + 3 * N), Xb(6 * N), U(6 * N), Yb(3 * nc), Lb(3 * nc, 0.0), inc(6 * N);
    for (int i = 0; i < N; ++i)
        for (int k = 0; k < 3; ++k) {
            Xb[6 * i + k] = gv[3 * i + k] + M.theta * M.h * gx[3 * i + k];
            Xb[6 * i + 3 + k] = gw[3 * i + k];
        }
    std::vector<Geo> G(nc);
    std::memset(G.data(), 0, sizeof(Geo) * nc);
    for (int k = K - 1; k >= 0; --k) {
        const double* Xk = &st.X[(size_t)k * 6 * N];
        const double* lk = &st.lam[(size_t)k * 3 * nc];
        const double* lk1 = &st.lam[(size_t)(k + 1) * 3 * nc];
        for (int i = 0; i < N; ++i)
            for (int q = 0; q < 3; ++q) {
                U[6 * i + q] = M.minv[i] * Xb[6 * i + q];
                U[6 * i + 3 + q] = M.iinv[i] * Xb[6 * i + 3 + q];
            }
        for (int c = 0; c < nc; ++c) {
            const Contact& C = st.C[c];
            double wv[3], dl[3], y[3], lp[3], lpb[3], mub;
            wx(C, U.data(), wv);
            for (int q = 0; q < 3; ++q) dl[q] = lk1[3 * c + q] - lk[3 * c + q];
            geo_acc(C, dl, U.data(), G[c]);
            for (int q = 0; q < 3; ++q) Lb[3 * c + q] += wv[q];
            wx(C, Xk, y);
            lp[0] = lk[3 * c] - C.Rn * y[0];
            lp[1] = lk[3 * c + 1] - C.Rt * y[1];
            lp[2] = lk[3 * c + 2] - C.Rt * y[2];
            project_adj(lp, C.mu, &Lb[3 * c], lpb, &mub);
            gmu[M.scene[C.b]] += mub;
            double yb[3] = {-C.Rn * lpb[0], -C.Rt * lpb[1], -C.Rt * lpb[2]};
            G[c].gRt -= lpb[1] * y[1] + lpb[2] * y[2];
            geo_acc(C, yb, Xk, G[c]);
            for (int q = 0; q < 3; ++q) {
                Lb[3 * c + q] = -wv[q] + lpb[q];
                Yb[3 * c + q] = yb[q];
            }
        }
        std::fill(inc.begin(), inc.end(), 0.0);
        for (int c = 0; c < nc; ++c) wtm(st.C[c], &Yb[3 * c], inc.data(), M, false);
        for (int i = 0; i < 6 * N; ++i) Xb[i] += inc[i];
    }
    // geometry -> midpoint positions
    for (int c = 0; c < nc; ++c) {
        const Contact& C = st.C[c];
        const Geo& g = G[c];
        const double iia = C.a >= 0 ? M.iinv[C.a] : 0.0;
        const double k = -C.Rt * C.Rt / M.alpha;
        const double rAb = g.grA + g.gRt * k * 2.0 * C.rA * iia;
        const double rBb = g.grB + g.gRt * k * 2.0 * C.rB * M.iinv[C.b];
        if (C.a < 0) {
            for (int q = 0; q < 3; ++q) gxm[3 * C.b + q] += -0.5 * rBb * C.n[q];
            continue;
        }
        double nb[3];
        for (int q = 0; q < 3; ++q) {
            nb[q] = g.gn[q];
            for (int r = 0; r < 3; ++r) nb[q] += C.Jt1[3 * r + q] * g.gt1[r] + C.Jt2[3 * r + q] * g.gt2[r];
        }
        const double nn = dot3(C.n, nb);
        double db[3];
        for (int q = 0; q < 3; ++q) db[q] = (nb[q] - C.n[q] * nn) / C.L + C.n[q] * (0.5 * rAb - 0.5 * rBb);
        for (int q = 0; q < 3; ++q) {
            gxm[3 * C.b + q] += db[q];
            gxm[3 * C.a + q] -= db[q];
        }
    }
    for (int i = 0; i < N; ++i)
        for (int q = 0; q < 3; ++q) {
            gx[3 * i + q] = gxm[3 * i + q];
            gv[3 * i + q] = Xb[6 * i + q] + (1.0 - M.theta) * M.h * gxm[3 * i + q];
            gw[3 * i + q] = Xb[6 * i + 3 + q];
        }
}

}  // namespace

extern "C" {

void* or_adj_create(const or_adj_problem* p) {
    if (!p || p->num_bodies < 0 || p->num_statics < 0) return nullptr;
    Model* M = new Model();
    M->N = p->num_bodies;
    M->S = p->num_statics;
    M->nsc = p->num_scenes > 0 ? p->num_scenes : 1;
    M->K = p->iterations;
    M->h = p->dt;
    for (int k = 0; k < 3; ++k) M->g[k] = p->gravity[k];
    M->theta = p->theta;
    M->alpha = p->alpha;
    M->margin = p->margin;
    M->rad.assign(p->radius, p->radius + M->N);
    M->minv.resize(M->N);
    M->iinv.resize(M->N);
    M->scene.resize(M->N);
    for (int i = 0; i < M->N; ++i) {
        M->minv[i] = 1.0 / p->mass[i];
        M->iinv[i] = 1.0 / p->inertia[i];
        M->scene[i] = p->body_scene ? p->body_scene[i] : 0;
    }
    M->su.resize(3 * M->S);
    M->soff.resize(M->S);
    M->sscene.resize(M->S);
    for (int s = 0; s < M->S; ++s) {
        const double* u = &p->static_dir[3 * s];
        const double n = std::sqrt(dot3(u, u));
        for (int k = 0; k < 3; ++k) M->su[3 * s + k] = u[k] / n;
        M->soff[s] = dot3(&M->su[3 * s], &p->static_pos[3 * s]);
        M->sscene[s] = p->static_scene ? p->static_scene[s] : 0;
    }
    return M;
}

void or_adj_destroy(void* h) { delete (Model*)h; }

int32_t or_adj_rollout(void* h, int32_t nsteps, const double* x0, const double* v0, const double* w0,
                       const double* mu_scene, double* xT, double* vT, double* wT) {
    const Model& M = *(Model*)h;
    std::vector<double> x(x0, x0 + 3 * M.N), v(v0, v0 + 3 * M.N), w(w0, w0 + 3 * M.N);
    std::vector<double> xn(3 * M.N), vn(3 * M.N), wn(3 * M.N);
    for (int t = 0; t < nsteps; ++t) {
        step(M, mu_scene, x.data(), v.data(), w.data(), xn.data(), vn.data(), wn.data(), nullptr);
        x.swap(xn);
        v.swap(vn);
        w.swap(wn);
    }
    std::memcpy(xT, x.data(), sizeof(double) * 3 * M.N);
    std::memcpy(vT, v.data(), sizeof(double) * 3 * M.N);
    std::memcpy(wT, w.data(), sizeof(double) * 3 * M.N);
    return 0;
}

int32_t or_adj_gradient(void* h, int32_t nsteps, const double* x0, const double* v0, const double* w0,
                        const double* mu_scene, const double* gxT, const double* gvT, const double* gwT, double* gx0,
                        double* gv0, double* gw0, double* gmu) {
    const Model& M = *(Model*)h;
    const size_t n3 = 3 * (size_t)M.N;
    // forward, keeping every step's input state
    std::vector<double> xs((nsteps + 1) * n3), vs((nsteps + 1) * n3), ws((nsteps + 1) * n3);
    std::memcpy(xs.data(), x0, sizeof(double) * n3);
    std::memcpy(vs.data(), v0, sizeof(double) * n3);
    std::memcpy(ws.data(), w0, sizeof(double) * n3);
    for (int t = 0; t < nsteps; ++t)
        step(M, mu_scene, &xs[t * n3], &vs[t * n3], &ws[t * n3], &xs[(t + 1) * n3], &vs[(t + 1) * n3],
             &ws[(t + 1) * n3], nullptr);
    std::memcpy(gx0, gxT, sizeof(double) * n3);
    std::memcpy(gv0, gvT, sizeof(double) * n3);
    std::memcpy(gw0, gwT, sizeof(double) * n3);
    for (int s = 0; s < M.nsc; ++s) gmu[s] = 0.0;
    std::vector<double> xo(n3), vo(n3), wo(n3);
    for (int t = nsteps - 1; t >= 0; --t) {
        StepStore st;
        step(M, mu_scene, &xs[t * n3], &vs[t * n3], &ws[t * n3], xo.data(), vo.data(), wo.data(), &st);
        step_back(M, st, gx0, gv0, gw0, gmu);
    }
    return 0;
}

}  // extern "C"
