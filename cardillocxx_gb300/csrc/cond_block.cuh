// One block of the condensed solver's sweeps in FP64 (CondensedSolver, condensed_solver.cpp:41-158:
// blockResidual, computeBlockUpdate with the projection, projectBlock): the shared body of the
// colored, Gauss-Seidel and Jacobi sweeps. Included by the files that run them (compiled without
// FMA contraction), after their jac_row, row_dot and minv_of.
#pragma once

namespace cdx {
namespace {

// CG: u and lambda change inside the launch (read and write them through L2). SCATTER: add
// M^-1 J^T (lambda_new - lambda_old) to u (Gauss-Seidel and colored sweeps; the Jacobi sweep
// gathers it per body afterwards). d receives lambda_new - lambda_old.
template <bool CG, bool SCATTER>
__device__ __forceinline__ void cond_block(const Scene& sc, const Contacts& C, const CondBufs& B, int c, double relax,
                                           double alpha, double* u, double* d) {
    const int N = sc.N;
    const int64_t cap = C.cap;
    const int a = C.a[c], b = C.b[c];
    const int dim = (C.flags[c] & CF_FRICTIONAL) ? 3 : 1;
    auto ld = [&](const double* p) -> double { return CG ? __ldcg(p) : *p; };
    double Ja[3][6], Jb[3][6], r[3], lo[3], ln[3];
    for (int q = 0; q < dim; ++q) {
        jac_row(C, c, q, false, Ja[q]);
        jac_row(C, c, q, true, Jb[q]);
        double o = B.rhs[q * cap + c];
        if (a >= 0) {
            double t = Ja[q][0] * ld(&u[a]);
            for (int k = 1; k < 6; ++k) t = t + Ja[q][k] * ld(&u[(size_t)k * N + a]);
            o = o - t;
        }
        {
            double t = Jb[q][0] * ld(&u[b]);
            for (int k = 1; k < 6; ++k) t = t + Jb[q][k] * ld(&u[(size_t)k * N + b]);
            o = o - t;
        }
        lo[q] = ld(&B.lam[q * cap + c]);
        o = o - 0.0 * lo[q];  // contact rows carry no compliance
        r[q] = o;
    }
    for (int q = 0; q < dim; ++q) {
        // GiiInv is diagonal but stored dense: the zero entries multiply the other residuals
        double g = (q == 0 ? B.ginv[c] : 0.0) * r[0];
        for (int j = 1; j < dim; ++j) g = g + (q == j ? B.ginv[j * cap + c] : 0.0) * r[j];
        ln[q] = ((relax * g) * alpha) + lo[q];
    }
    ln[0] = f64::smin(ln[0], 0.0);
    if (dim == 3) {
        const double tn = sqrt(ln[1] * ln[1] + ln[2] * ln[2]);
        if (tn > 0.0) {
            const double s = f64::smin(1.0, (-C.mu[c] * ln[0]) / tn);
            ln[1] = ln[1] * s;
            ln[2] = ln[2] * s;
        }
    }
    for (int q = 0; q < dim; ++q) d[q] = ln[q] - lo[q];
    if (SCATTER) {
        for (int side = 0; side < 2; ++side) {
            const int body = side == 0 ? a : b;
            if (body < 0) continue;
            double (*J)[6] = side == 0 ? Ja : Jb;
            for (int k = 0; k < 6; ++k) {
                double tk = J[0][k] * d[0];
                for (int q = 1; q < dim; ++q) tk = tk + J[q][k] * d[q];
                const size_t j = (size_t)k * N + body;
                const double v = ld(&u[j]) + minv_of(sc, body, k) * tk;
                if (CG)
                    __stcg(&u[j], v);
                else
                    u[j] = v;
            }
        }
    }
    for (int q = 0; q < dim; ++q) {
        if (CG)
            __stcg(&B.lam[q * cap + c], ln[q]);
        else
            B.lam[q * cap + c] = ln[q];
    }
}

}  // namespace
}  // namespace cdx
