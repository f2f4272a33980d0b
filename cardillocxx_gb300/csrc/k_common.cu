// Shared device building blocks: uniform-grid cell keys and cell ranges (the broad phase that
// replaces coal's dynamic AABB tree, collision_coal.cpp:247-270,423-431), and the radix sort /
// exclusive scan used for the grid, the contact offsets and the W^T incidence lists.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include "cdx_internal.h"

namespace cdx {

namespace {
constexpr int NT = 256;
inline int nblk(int64_t n, int nt = NT) { return (int)((n + nt - 1) / nt); }

// by_inverse: multiply by 1 / cell instead of dividing (the split form, whose pair kernels read
// the keys back instead of recomputing cells); the plain FP64 method divides, as its pair kernels do
__global__ void k_cell_keys(Scene sc, Grid g, uint32_t* keys, uint32_t* vals, int by_inverse, double inv_cell) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sc.N) return;
    const double p[3] = {sc.bf(BF_PX)[i], sc.bf(BF_PY)[i], sc.bf(BF_PZ)[i]};
    int ci[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        double f = by_inverse ? floor((p[k] - g.lo[k]) * inv_cell) : floor((p[k] - g.lo[k]) / g.cell);
        if (!(f >= 0.0)) f = 0.0;
        if (f > (double)(g.dim[k] - 1)) f = (double)(g.dim[k] - 1);
        ci[k] = (int)f;
    }
    keys[i] = (uint32_t)(((int64_t)ci[2] * g.dim[1] + ci[1]) * g.dim[0] + ci[0]);
    vals[i] = (uint32_t)i;
}

// start[k]/end[k] of each key present in a sorted key array (absent keys keep their cleared value)
__global__ void k_ranges(const uint32_t* keys, int64_t n, int32_t* start, int32_t* end) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const uint32_t k = keys[p];
    if (p == 0 || keys[p - 1] != k) start[k] = (int32_t)p;
    if (p == n - 1 || keys[p + 1] != k) end[k] = (int32_t)(p + 1);
}
}  // namespace

size_t scan_temp_bytes(int64_t n) {
    size_t b = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, b, (const int32_t*)nullptr, (int32_t*)nullptr, (int)n);
    return b;
}

size_t sort_temp_bytes(int64_t n) {
    size_t b = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, b, (const uint32_t*)nullptr, (uint32_t*)nullptr,
                                    (const uint32_t*)nullptr, (uint32_t*)nullptr, (int)n, 0, 32);
    return b;
}

cudaError_t exclusive_scan(void* tmp, size_t tmp_bytes, const int32_t* in, int32_t* out, int64_t n, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    return cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, in, out, (int)n, s);
}

cudaError_t sort_pairs(void* tmp, size_t tmp_bytes, const uint32_t* kin, uint32_t* kout, const uint32_t* vin,
                       uint32_t* vout, int64_t n, int end_bit, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    return cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, kin, kout, vin, vout, (int)n, 0, end_bit, s);
}

void launch_cell_keys(const Scene& sc, const Grid& g, uint32_t* keys, uint32_t* vals, cudaStream_t s,
                      int by_inverse) {
    if (sc.N == 0) return;
    k_cell_keys<<<nblk(sc.N), NT, 0, s>>>(sc, g, keys, vals, by_inverse, 1.0 / g.cell);
}

void launch_ranges(const uint32_t* sorted_keys, int64_t n, int32_t* start, int32_t* end, cudaStream_t s) {
    if (n <= 0) return;
    k_ranges<<<nblk(n), NT, 0, s>>>(sorted_keys, n, start, end);
}

}  // namespace cdx

namespace cdx {
namespace {
// interleaved host layout <-> field-major device state: pos[3N], quat[4N], vel[3N], omega[3N]
__global__ void k_pack_state(Scene sc, double* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sc.N) return;
    const size_t N = sc.N;
    for (int k = 0; k < 3; ++k) {
        out[3 * (size_t)i + k] = sc.bf(BF_PX + k)[i];
        out[7 * N + 3 * (size_t)i + k] = sc.bf(BF_VX + k)[i];
        out[10 * N + 3 * (size_t)i + k] = sc.bf(BF_WX + k)[i];
    }
    for (int k = 0; k < 4; ++k) out[3 * N + 4 * (size_t)i + k] = sc.bf(BF_QX + k)[i];
}
__global__ void k_unpack_state(Scene sc, const double* in, int mask) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sc.N) return;
    const size_t N = sc.N;
    for (int k = 0; k < 3; ++k) {
        if (mask & 1) sc.bf(BF_PX + k)[i] = in[3 * (size_t)i + k];
        if (mask & 4) sc.bf(BF_VX + k)[i] = in[7 * N + 3 * (size_t)i + k];
        if (mask & 8) sc.bf(BF_WX + k)[i] = in[10 * N + 3 * (size_t)i + k];
    }
    if (mask & 2)
        for (int k = 0; k < 4; ++k) sc.bf(BF_QX + k)[i] = in[3 * N + 4 * (size_t)i + k];
}
// The state as the caller's four arrays (pos 3N, quat 4N, vel 3N, omega 3N; a NULL array is
// skipped), element by element so that consecutive threads touch consecutive doubles of the
// caller's arrays: coalesced when those live in host memory that the GPU reads or writes directly.
__global__ void k_pack_state4(Scene sc, double* pos, double* quat, double* vel, double* omega) {
    const int64_t N = sc.N, total = 13 * N;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        if (e < 3 * N) {
            if (pos) pos[e] = sc.bf(BF_PX + (int)(e % 3))[e / 3];
        } else if (e < 7 * N) {
            const int64_t j = e - 3 * N;
            if (quat) quat[j] = sc.bf(BF_QX + (int)(j % 4))[j / 4];
        } else if (e < 10 * N) {
            const int64_t j = e - 7 * N;
            if (vel) vel[j] = sc.bf(BF_VX + (int)(j % 3))[j / 3];
        } else {
            const int64_t j = e - 10 * N;
            if (omega) omega[j] = sc.bf(BF_WX + (int)(j % 3))[j / 3];
        }
    }
}
__global__ void k_unpack_state4(Scene sc, const double* pos, const double* quat, const double* vel,
                                const double* omega) {
    const int64_t N = sc.N, total = 13 * N;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        if (e < 3 * N) {
            if (pos) sc.bf(BF_PX + (int)(e % 3))[e / 3] = pos[e];
        } else if (e < 7 * N) {
            const int64_t j = e - 3 * N;
            if (quat) sc.bf(BF_QX + (int)(j % 4))[j / 4] = quat[j];
        } else if (e < 10 * N) {
            const int64_t j = e - 7 * N;
            if (vel) sc.bf(BF_VX + (int)(j % 3))[j / 3] = vel[j];
        } else {
            const int64_t j = e - 10 * N;
            if (omega) sc.bf(BF_WX + (int)(j % 3))[j / 3] = omega[j];
        }
    }
}
}  // namespace
void launch_pack_state4(const Scene& sc, double* pos, double* quat, double* vel, double* omega, cudaStream_t s) {
    if (sc.N) k_pack_state4<<<(int)std::min<int64_t>(nblk(13 * (int64_t)sc.N), 8192), NT, 0, s>>>(sc, pos, quat, vel, omega);
}
void launch_unpack_state4(const Scene& sc, const double* pos, const double* quat, const double* vel,
                          const double* omega, cudaStream_t s) {
    if (sc.N)
        k_unpack_state4<<<(int)std::min<int64_t>(nblk(13 * (int64_t)sc.N), 8192), NT, 0, s>>>(sc, pos, quat, vel, omega);
}
void launch_pack_state(const Scene& sc, double* out, cudaStream_t s) {
    if (sc.N) k_pack_state<<<nblk(sc.N), NT, 0, s>>>(sc, out);
}
void launch_unpack_state(const Scene& sc, const double* in, int mask, cudaStream_t s) {
    if (sc.N) k_unpack_state<<<nblk(sc.N), NT, 0, s>>>(sc, in, mask);
}
}  // namespace cdx
