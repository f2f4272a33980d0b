// Differentiable rollout of sphere scenes on the GPU: forward steps with iterate storage and the
// hand-written reverse of each step (one block per scene, FP64). Host side in engine_adjoint.cpp.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace cdx {

constexpr int ADJ_THREADS = 256;
constexpr int ADJ_MAX_SCENE_BODIES = 1024;

// problem data (fixed for the context)
struct AdjProblem {
    int N = 0, S = 0, nsc = 0, K = 0;
    double h = 0, g[3] = {0, 0, 0}, theta = 0.5, alpha = 0.5, margin = 0;
    const double* rad = nullptr;   // [N]
    const double* minv = nullptr;  // [N] 1/m
    const double* iinv = nullptr;  // [N] 1/I
    const double* su = nullptr;    // [3S] unit halfspace normals
    const double* soff = nullptr;  // [S] plane offsets u.p
    const int32_t* body_off = nullptr;     // [nsc+1]
    const int32_t* static_off = nullptr;   // [nsc+1]
    const int32_t* contact_off = nullptr;  // [nsc+1] capacity slices
};

// per-step contact data and work buffers (contact slices per scene)
struct AdjStep {
    int32_t* nc = nullptr;  // [nsc] contacts found
    int32_t* ca = nullptr;  // [cap] body A (-1 for a halfspace)
    int32_t* cb = nullptr;  // [cap] body B
    int32_t* cs = nullptr;  // [cap] halfspace index or -1
    double* cn = nullptr;   // [3 cap]
    double* ct1 = nullptr;  // [3 cap]
    double* ct2 = nullptr;  // [3 cap]
    double* cg = nullptr;   // [5 cap]: rho_A, rho_B, L, R_n, R_t
    double* lam = nullptr;  // [3 cap] current impulses
    double* dl = nullptr;   // [3 cap] impulse increments / adjoint of y
    int32_t* inc_off = nullptr;  // [N + nsc] per-scene CSR offsets into inc (scene s: body_off[s] + s ...)
    int32_t* inc = nullptr;      // [2 cap] (contact << 1 | side)
    double* geo = nullptr;   // [12 cap] backward geometry accumulators
    double* lbar = nullptr;  // [3 cap] adjoint of the impulses
    double* dbar = nullptr;  // [3 cap] per-contact position adjoint (pair: of d = x_B - x_A; halfspace: of x_B)
    double* xs = nullptr;    // [(K+1) 6N] stored iterates x_k (STORE)
    double* ls = nullptr;    // [(K+1) 3 cap] stored impulses lambda_k (STORE)
    int32_t* err = nullptr;  // [1] contact overflow flag
    long long* ncsum = nullptr;  // [nsc] contacts summed over the steps of a forward rollout
    int64_t cap = 0;
};

// one forward step for every scene: (x, v, w) -> (xo, vo, wo); store = keep every iterate.
// nbmax = shared-memory body slots of a block (at least the largest scene, at least 64)
// count = add the step's contact count to W.ncsum
void launch_adj_step(const AdjProblem& P, const AdjStep& W, const double* mu, const double* x, const double* v,
                     const double* w, double* xo, double* vo, double* wo, int store, int count, int nbmax,
                     cudaStream_t s);
// reverse of the step stored in W: (gx, gv, gw) adjoint of the outputs in, of the inputs out (in
// place); gmu[scene] accumulates
void launch_adj_back(const AdjProblem& P, const AdjStep& W, const double* mu, double* gx, double* gv, double* gw,
                     double* gmu, int nbmax, cudaStream_t s);
int adj_smem_bytes(int nbmax);
// opt the three kernels in to smem bytes of dynamic shared memory; returns a cudaError_t
int adj_set_smem_limit(int smem);

}  // namespace cdx
