// FP64 reciprocal and reciprocal square root by Newton-Raphson refinement of an FP32 seed.
//
// GB300 issues FP64 at a small fraction of its FP32 rate, and an IEEE double division or square
// root expands into a long FP64 sequence. Where a correctly rounded result is not required (the
// split form's FP64 final pass), the Newton-Raphson iterations for f(y) = 1/y - x and
// f(y) = 1/y^2 - x, started from the FP32 hardware approximation, reach full double accuracy in
// two steps (the relative error squares at each step: ~2^-23 -> ~2^-46 -> below 2^-52):
//   reciprocal:      e = 1 - x y,          y <- y + y e
//   inverse sqrt:    e = 1 - x y^2,        y <- y + y e (1/2 + 3/8 e)   (second-order step)
// Outside the FP32 exponent range the functions fall back to the IEEE operations.
#pragma once
#include <cuda_runtime.h>

namespace cdx {

__device__ __forceinline__ double rcp_nr(double x) {
    const double ax = fabs(x);
    if (!(ax > 1e-30 && ax < 1e30)) return 1.0 / x;
    double y = (double)__frcp_rn((float)x);
    double e = fma(-x, y, 1.0);
    y = fma(y, e, y);
    e = fma(-x, y, 1.0);
    y = fma(y, e, y);
    return y;
}

__device__ __forceinline__ double rsqrt_nr(double x) {
    if (!(x > 1e-30 && x < 1e30)) return 1.0 / sqrt(x);
    double y = (double)rsqrtf((float)x);
    double e = fma(-x * y, y, 1.0);
    y = fma(y * e, fma(0.375, e, 0.5), y);
    e = fma(-x * y, y, 1.0);
    y = fma(y * e, fma(0.375, e, 0.5), y);
    return y;
}

}  // namespace cdx
