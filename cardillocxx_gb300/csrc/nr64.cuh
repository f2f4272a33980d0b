// FP64 reciprocal and reciprocal square root by Newton-Raphson refinement of an FP32 seed.
//
// GB300 issues FP64 at a small fraction of its FP32 rate, and an IEEE double division or square
// root expands into a long FP64 sequence. Where a correctly rounded result is not required (the
// split form's FP64 final pass), one third-order step of the series for 1/x and 1/sqrt(x),
// started from the FP32 hardware approximation, reaches double accuracy: with e the relative
// defect of the seed (|e| <~ 2^-22), the truncation error is of order e^3 (~2^-66), below the
// rounding of the last fused multiply-add:
//   reciprocal:      e = 1 - x y,          y <- y + y (e + e^2)             (1/(1-e) = 1 + e + e^2 + ...)
//   inverse sqrt:    e = 1 - x y^2,        y <- y + y e (1/2 + 3/8 e)       ((1-e)^-1/2 = 1 + e/2 + 3e^2/8 + ...)
// Outside the FP32 exponent range the functions fall back to the IEEE operations.
#pragma once
#include <cuda_runtime.h>

namespace cdx {

__device__ __forceinline__ double rcp_nr(double x) {
    const double ax = fabs(x);
    if (!(ax > 1e-30 && ax < 1e30)) return 1.0 / x;
    const double y = (double)__frcp_rn((float)x);
    const double e = fma(-x, y, 1.0);
    return fma(y, fma(e, e, e), y);
}

__device__ __forceinline__ double rsqrt_nr(double x) {
    if (!(x > 1e-30 && x < 1e30)) return 1.0 / sqrt(x);
    const double y = (double)rsqrtf((float)x);
    const double e = fma(-x * y, y, 1.0);
    return fma(y * e, fma(0.375, e, 0.5), y);
}

}  // namespace cdx
