// Device buffers and launchers of the split-precision form (k_split.cu).
#pragma once
#include <cstdint>

#include <cuda_runtime.h>

#include "cdx_internal.h"

namespace cdx {

struct SplitScalars {
    int32_t done;
    int32_t iters;
    unsigned int maxd;  // bits of max ||dlambda_c|| (FP32, non-negative)
    unsigned int maxl;  // bits of max |lambda|
    float res_last;
    int32_t pad0;
    unsigned long long maxd64;  // FP64 residual pass
    unsigned long long maxl64;
    double res_final;
};

struct SplitParams {
    float alpha;
    float margin;
    float match2;
    int combine;
    int friction_enable;
    int prev_count;
};

// Contact records are float4-aligned so a warp reads them with 16-byte vector loads:
//   ab   (body A or -(static)-1, body B)
//   nmu  (n.x, n.y, n.z, mu)
//   levR (rhoA, rhoB, R_n, R_t)        R = alpha / Delassus diagonal
//   bias (R_n b_n, R_t b_t1, R_t b_t2)  static wall velocity and restitution terms
//   lam  (lambda_n, lambda_t1, lambda_t2) per generation (warm start)
struct SplitBuf {
    int N = 0;
    int64_t cap = 0;
    float4* pos4 = nullptr;   // N: position relative to the scene origin, radius
    float4* vel4 = nullptr;   // 2N: (v, 1/m), (omega_world, 1/I)
    float4* acc4 = nullptr;   // 2N: M^-1 W^T dlambda accumulators
    float4* vn4 = nullptr;    // 2N: pre-solve velocities (v, omega_world)
    double* vfree = nullptr;  // 6N FP64 free velocities (world frame)
    double* acc64 = nullptr;  // 6N FP64 W^T lambda, then final velocities
    double* origin = nullptr; // 3 per scene
    float4* st_dir = nullptr; // S: (normal/axis, plane offset in scene coordinates)
    float4* st_pt = nullptr;  // S: (anchor in scene coordinates, drum radius)
    float4* st_v = nullptr;   // S: (wall velocity, kind)
    float4* st_w = nullptr;   // S: (wall angular velocity world, mu)
    int2* ab = nullptr;
    float4* nmu = nullptr;
    float4* levR = nullptr;
    float4* bias = nullptr;
    float4* lam[2] = {nullptr, nullptr};
    unsigned long long* key[2] = {nullptr, nullptr};
    float4* pt[2] = {nullptr, nullptr};
    double* g64 = nullptr;    // 5*cap FP64 geometry (n, rhoA, rhoB) of the final pass
    int32_t* nc_dev = nullptr;
    SplitScalars* ss = nullptr;
};

int split_grid_blocks(int64_t n, int sms);
void launch_s_prep(const Scene& sc, const SplitBuf& sb, double dt, const double* g, double h1, cudaStream_t s);
void launch_s_static_flags(const Scene& sc, const SplitBuf& sb, float margin, int32_t* flags, cudaStream_t s);
void launch_s_pair_count(const Scene& sc, const Grid& g, const SplitBuf& sb, const uint32_t* cell_body,
                         const int32_t* cell_start, const int32_t* cell_end, int32_t* counts, const SplitParams& P,
                         DevScalars* ds, cudaStream_t s);
void launch_s_static_write(const Scene& sc, const SplitBuf& sb, const int32_t* flags, const int32_t* pos, int gen,
                           const SplitParams& P, cudaStream_t s);
void launch_s_pair_write(const Scene& sc, const Grid& g, const SplitBuf& sb, const uint32_t* cell_body,
                         const int32_t* cell_start, const int32_t* cell_end, const int32_t* offsets, int32_t base,
                         int gen, const SplitParams& P, DevScalars* ds, cudaStream_t s);
void launch_s_reset(const SplitBuf& sb, cudaStream_t s);
void launch_s_apply_warm(const SplitBuf& sb, int gen, int blocks, cudaStream_t s);
void launch_s_contact(const SplitBuf& sb, int gen, int blocks, cudaStream_t s);
void launch_s_body(const SplitBuf& sb, int N, int blocks, int apply_only, cudaStream_t s);
void launch_s_check(const SplitBuf& sb, int max_iter, float tol, cudaGraphConditionalHandle h, int use_handle,
                    cudaStream_t s);
void launch_s_final(const Scene& sc, const SplitBuf& sb, int gen, double alpha, int friction_enable, int combine,
                    int blocks, cudaStream_t s);

}  // namespace cdx
