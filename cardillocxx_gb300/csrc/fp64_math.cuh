// FP64 device arithmetic of the plain method. Compiled with --fmad=false: every product and sum
// is rounded on its own, in the order written, so the results are bit-identical to the CPU
// restatement of the reference (Eigen expressions evaluated left to right).
#pragma once
#include <cfloat>
#include <cuda_runtime.h>

namespace cdx {
namespace f64 {

__device__ __forceinline__ double dot3(const double* a, const double* b) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }
__device__ __forceinline__ double norm3(const double* a) { return sqrt(dot3(a, a)); }
__device__ __forceinline__ void cross3(const double* a, const double* b, double* o) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}
__device__ __forceinline__ bool finite3(const double* a) { return isfinite(a[0]) && isfinite(a[1]) && isfinite(a[2]); }
__device__ __forceinline__ double smin(double a, double b) { return (b < a) ? b : a; }  // std::min
__device__ __forceinline__ double smax(double a, double b) { return (a < b) ? b : a; }  // std::max

// quaternion (x,y,z,w) -> row-major rotation matrix (Eigen toRotationMatrix)
__device__ __forceinline__ void rotmat(const double* q, double* R) {
    const double x = q[0], y = q[1], z = q[2], w = q[3];
    const double tx = 2.0 * x, ty = 2.0 * y, tz = 2.0 * z;
    const double twx = tx * w, twy = ty * w, twz = tz * w;
    const double txx = tx * x, txy = ty * x, txz = tz * x;
    const double tyy = ty * y, tyz = tz * y, tzz = tz * z;
    R[0] = 1.0 - (tyy + tzz); R[1] = txy - twz;         R[2] = txz + twy;
    R[3] = txy + twz;         R[4] = 1.0 - (txx + tzz); R[5] = tyz - twx;
    R[6] = txz - twy;         R[7] = tyz + twx;         R[8] = 1.0 - (txx + tyy);
}
__device__ __forceinline__ void matTvec(const double* R, const double* v, double* o) {
#pragma unroll
    for (int i = 0; i < 3; ++i) o[i] = (R[0 + i] * v[0] + R[3 + i] * v[1]) + R[6 + i] * v[2];
}
// R v (a body-frame vector in world coordinates)
__device__ __forceinline__ void matvec(const double* R, const double* v, double* o) {
#pragma unroll
    for (int i = 0; i < 3; ++i) o[i] = (R[3 * i] * v[0] + R[3 * i + 1] * v[1]) + R[3 * i + 2] * v[2];
}

// alignQuaternionTo with Eigen's normalize()
__device__ __forceinline__ void align_quat(double* q, const double* qref) {
    if (!(isfinite(q[0]) && isfinite(q[1]) && isfinite(q[2]) && isfinite(q[3]))) {
#pragma unroll
        for (int k = 0; k < 4; ++k) q[k] = qref[k];
        return;
    }
    const double n2 = ((q[0] * q[0] + q[1] * q[1]) + q[2] * q[2]) + q[3] * q[3];
    if (n2 > 0.0) {
        const double n = sqrt(n2);
#pragma unroll
        for (int k = 0; k < 4; ++k) q[k] = q[k] / n;
    }
    const double d = ((qref[0] * q[0] + qref[1] * q[1]) + qref[2] * q[2]) + qref[3] * q[3];
    if (d < 0.0) {
#pragma unroll
        for (int k = 0; k < 4; ++k) q[k] = -q[k];
    }
}

// explicitPositionUpdate for one entity
__device__ __forceinline__ void drift(double* x, double* q, const double* v, const double* w, double h) {
#pragma unroll
    for (int k = 0; k < 3; ++k) x[k] = x[k] + h * v[k];
    const double qprev[4] = {q[0], q[1], q[2], q[3]};
    const double hh = h * 0.5;
    const double qw = q[3];
    q[3] = q[3] - hh * dot3(q, w);
    double c[3];
    cross3(qprev, w, c);
#pragma unroll
    for (int k = 0; k < 3; ++k) q[k] = qprev[k] + hh * (qw * w[k] + c[k]);
    align_quat(q, qprev);
}

// tangentFrameFromNormal (Frisvad with the south-pole branch)
__device__ __forceinline__ void tangent_frame(const double* n_in, double* t1, double* t2) {
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
#pragma unroll
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
        const double s = sqrt(t2n);
#pragma unroll
        for (int k = 0; k < 3; ++k) t1[k] = t1[k] / s;
    }
    cross3(n, t1, t2);
}

__device__ __forceinline__ double combine_mu(int mode, double a, double b) {
    a = smax(0.0, a);
    b = smax(0.0, b);
    if (mode == 1) return (a + b) * 0.5;
    if (mode == 2) return sqrt(smax(0.0, a * b));
    return smin(a, b);
}

// invertSmallSpd (misc/block_diagonal.hpp:15-27) for n <= 3, row-major: Cholesky from the lower
// triangle, column by column, then forward and back substitution of each identity column; a
// pivot that is not positive takes the reference's last fallback, the diagonal inverse
static __device__ __noinline__ void spd_inverse_dev(const double* A, int n, double* X) {
    double L[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    bool ok = true;
    for (int j = 0; j < n && ok; ++j) {
        double s = A[j * n + j];
        for (int k = 0; k < j; ++k) s = s - L[j * 3 + k] * L[j * 3 + k];
        if (!(s > 0.0)) {
            ok = false;
            break;
        }
        L[j * 3 + j] = sqrt(s);
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

// MatrixBase::isDiagonal (Eigen 3) with its default precision for double, 1e-12, on a 3x3 block
__device__ __forceinline__ bool block_is_diagonal3(const double* D) {
    double md = -1.0;
    for (int j = 0; j < 3; ++j) md = smax(md, fabs(D[4 * j]));
    bool diag = true;
    for (int j = 0; j < 3; ++j)
        for (int i = 0; i < j; ++i) diag = diag && (fabs(D[3 * i + j]) <= md * 1e-12) && (fabs(D[3 * j + i]) <= md * 1e-12);
    return diag;
}

}  // namespace f64
}  // namespace cdx
