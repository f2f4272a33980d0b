// Host side of the differentiable rollout (cdx_adj_*): scene partition, device buffers,
// checkpointed forward and the reverse pass with step-level recomputation.
//
// Forward keeps the state at every checkpoint_every-th step. Backward walks the checkpoint
// segments from the last: it recomputes the segment's step inputs from its checkpoint, then for
// each step from the segment's end re-runs that step keeping every sweep's iterate and runs the
// step's reverse. Device memory is the checkpoints (9N doubles each), one segment of step inputs,
// and one step's iterates ((K+1) x (6N + 3 contact slots) doubles), so a rollout of any length fits.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <new>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/cdx.h"
#include "adjoint.h"

namespace {

using namespace cdx;

struct Adj {
    AdjProblem P;
    AdjStep W;
    int nbmax = 64;
    int ck_every = 20;
    int nsteps = 0;  // of the last forward
    cudaStream_t stream = nullptr;
    std::vector<void*> bufs;
    std::string err;
    // device state
    double* mu = nullptr;       // [nsc]
    double* gmu = nullptr;      // [nsc]
    double* cur = nullptr;      // [9N] x, v, w
    double* nxt = nullptr;      // [9N]
    double* g = nullptr;        // [9N] adjoint
    double* ck = nullptr;       // [nck 9N]
    double* seg = nullptr;      // [ck_every 9N]
    int nck = 0;
    size_t bytes = 0;

    ~Adj() {
        for (void* p : bufs) cudaFree(p);
        if (stream) cudaStreamDestroy(stream);
    }
    int fail(int code, const std::string& m) {
        err = m;
        return code;
    }
    int cuda(cudaError_t e, const char* what) {
        if (e == cudaSuccess) return CDX_OK;
        return fail(CDX_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    }
    int alloc(void** p, size_t n, const char* what) {
        if (n == 0) n = 8;
        cudaError_t e = cudaMalloc(p, n);
        if (e != cudaSuccess) return cuda(e, what);
        bufs.push_back(*p);
        bytes += n;
        return CDX_OK;
    }
    void release(void* p, size_t n) {
        if (!p) return;
        auto it = std::find(bufs.begin(), bufs.end(), p);
        if (it != bufs.end()) bufs.erase(it);
        cudaFree(p);
        bytes -= n;
    }
};

int check_last(Adj& A, const char* what) {
    int st;
    if ((st = A.cuda(cudaGetLastError(), what))) return st;
    return A.cuda(cudaStreamSynchronize(A.stream), what);
}

}  // namespace

struct cdx_adj {
    Adj a;
};

extern "C" {

int cdx_adj_create(const cdx_config* cfg, const cdx_scene* sc, int32_t checkpoint_every, cdx_adj** out) {
    if (!cfg || !sc || !out || checkpoint_every <= 0) return CDX_ERR_ARG;
    *out = nullptr;
    const int N = sc->num_bodies, S = sc->num_statics;
    if (N <= 0 || !sc->radius || !sc->mass || !sc->inertia) return CDX_ERR_ARG;
    if (cfg->pj_max_iterations <= 0) return CDX_ERR_ARG;
    const int nsc = sc->num_scenes > 0 ? sc->num_scenes : 1;
    // scenes: contiguous bodies and statics, halfspaces only, sizes within one block's reach
    std::vector<int32_t> boff(nsc + 1, 0), soff(nsc + 1, 0), coff(nsc + 1, 0);
    for (int i = 0; i < N; ++i) {
        const int s = sc->body_scene ? sc->body_scene[i] : 0;
        if (s < 0 || s >= nsc || (i > 0 && sc->body_scene && s < sc->body_scene[i - 1])) return CDX_ERR_ARG;
        ++boff[s + 1];
    }
    for (int s = 0; s < S; ++s) {
        if (sc->static_kind && sc->static_kind[s] != 0) return CDX_ERR_UNSUPPORTED;
        const int q = sc->static_scene ? sc->static_scene[s] : 0;
        if (q < 0 || q >= nsc || (s > 0 && sc->static_scene && q < sc->static_scene[s - 1])) return CDX_ERR_ARG;
        ++soff[q + 1];
    }
    int nbmax = 64;
    for (int s = 0; s < nsc; ++s) {
        nbmax = std::max(nbmax, (int)boff[s + 1]);
        const int64_t cap = (int64_t)boff[s + 1] * (int64_t)std::max(1.0, cfg->gpu_contact_capacity_factor) +
                            (int64_t)soff[s + 1] * boff[s + 1];
        boff[s + 1] += boff[s];
        soff[s + 1] += soff[s];
        if (coff[s] + cap > (int64_t)1 << 30) return CDX_ERR_OVERFLOW;
        coff[s + 1] = coff[s] + (int32_t)cap;
    }
    if (nbmax > ADJ_MAX_SCENE_BODIES) return CDX_ERR_UNSUPPORTED;
    cdx_adj* h = new (std::nothrow) cdx_adj();
    if (!h) return CDX_ERR_ARG;
    Adj& A = h->a;
    *out = h;
    int st;
    if ((st = A.cuda(cudaStreamCreateWithFlags(&A.stream, cudaStreamNonBlocking), "stream"))) return st;
    A.nbmax = nbmax;
    A.ck_every = checkpoint_every;
    AdjProblem& P = A.P;
    P.N = N;
    P.S = S;
    P.nsc = nsc;
    P.K = cfg->pj_max_iterations;
    P.h = cfg->sim_dt;
    for (int k = 0; k < 3; ++k) P.g[k] = cfg->sim_gravity[k];
    P.theta = cfg->moreau_theta;
    P.alpha = cfg->pj_alpha;
    P.margin = cfg->collision_security_margin;
    std::vector<double> minv(N), iinv(N), su(3 * (size_t)std::max(S, 1)), so(std::max(S, 1));
    for (int i = 0; i < N; ++i) {
        minv[i] = 1.0 / sc->mass[i];
        iinv[i] = 1.0 / sc->inertia[i];
    }
    for (int s = 0; s < S; ++s) {
        const double* u = &sc->static_dir[3 * s];
        const double n = std::sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
        for (int k = 0; k < 3; ++k) su[3 * s + k] = u[k] / n;
        so[s] = su[3 * s] * sc->static_pos[3 * s] + su[3 * s + 1] * sc->static_pos[3 * s + 1] +
                su[3 * s + 2] * sc->static_pos[3 * s + 2];
    }
    auto up = [&](void** d, const void* src, size_t n, const char* what) {
        int s2 = A.alloc(d, n, what);
        if (!s2 && n) s2 = A.cuda(cudaMemcpy(*d, src, n, cudaMemcpyHostToDevice), what);
        return s2;
    };
    double *rad, *dminv, *diinv, *dsu, *dso;
    int32_t *dboff, *dsoff, *dcoff;
    if ((st = up((void**)&rad, sc->radius, sizeof(double) * N, "adjoint bodies")) ||
        (st = up((void**)&dminv, minv.data(), sizeof(double) * N, "adjoint bodies")) ||
        (st = up((void**)&diinv, iinv.data(), sizeof(double) * N, "adjoint bodies")) ||
        (st = up((void**)&dsu, su.data(), sizeof(double) * su.size(), "adjoint statics")) ||
        (st = up((void**)&dso, so.data(), sizeof(double) * so.size(), "adjoint statics")) ||
        (st = up((void**)&dboff, boff.data(), sizeof(int32_t) * (nsc + 1), "adjoint scenes")) ||
        (st = up((void**)&dsoff, soff.data(), sizeof(int32_t) * (nsc + 1), "adjoint scenes")) ||
        (st = up((void**)&dcoff, coff.data(), sizeof(int32_t) * (nsc + 1), "adjoint scenes")))
        return st;
    P.rad = rad;
    P.minv = dminv;
    P.iinv = diinv;
    P.su = dsu;
    P.soff = dso;
    P.body_off = dboff;
    P.static_off = dsoff;
    P.contact_off = dcoff;
    AdjStep& W = A.W;
    const int64_t cap = coff[nsc];
    W.cap = cap;
    const size_t c8 = sizeof(double) * (size_t)cap, c4 = sizeof(int32_t) * (size_t)cap;
    if ((st = A.alloc((void**)&W.nc, sizeof(int32_t) * nsc, "adjoint contacts")) ||
        (st = A.alloc((void**)&W.ca, c4, "adjoint contacts")) || (st = A.alloc((void**)&W.cb, c4, "adjoint contacts")) ||
        (st = A.alloc((void**)&W.cs, c4, "adjoint contacts")) ||
        (st = A.alloc((void**)&W.cn, 3 * c8, "adjoint contacts")) ||
        (st = A.alloc((void**)&W.ct1, 3 * c8, "adjoint contacts")) ||
        (st = A.alloc((void**)&W.ct2, 3 * c8, "adjoint contacts")) ||
        (st = A.alloc((void**)&W.cg, 5 * c8, "adjoint contacts")) ||
        (st = A.alloc((void**)&W.lam, 3 * c8, "adjoint contacts")) ||
        (st = A.alloc((void**)&W.dl, 3 * c8, "adjoint contacts")) ||
        (st = A.alloc((void**)&W.inc_off, sizeof(int32_t) * ((size_t)N + nsc), "adjoint incidence")) ||
        (st = A.alloc((void**)&W.inc, 2 * c4, "adjoint incidence")) ||
        (st = A.alloc((void**)&W.geo, 12 * c8, "adjoint work")) ||
        (st = A.alloc((void**)&W.lbar, 3 * c8, "adjoint work")) ||
        (st = A.alloc((void**)&W.dbar, 3 * c8, "adjoint work")) ||
        (st = A.alloc((void**)&W.xs, sizeof(double) * (size_t)(P.K + 1) * 6 * N, "adjoint iterates")) ||
        (st = A.alloc((void**)&W.ls, 3 * c8 * (size_t)(P.K + 1), "adjoint iterates")) ||
        (st = A.alloc((void**)&W.err, sizeof(int32_t), "adjoint")) ||
        (st = A.alloc((void**)&W.ncsum, sizeof(long long) * nsc, "adjoint")) ||
        (st = A.alloc((void**)&A.mu, sizeof(double) * nsc, "adjoint")) ||
        (st = A.alloc((void**)&A.gmu, sizeof(double) * nsc, "adjoint")) ||
        (st = A.alloc((void**)&A.cur, sizeof(double) * 9 * N, "adjoint state")) ||
        (st = A.alloc((void**)&A.nxt, sizeof(double) * 9 * N, "adjoint state")) ||
        (st = A.alloc((void**)&A.g, sizeof(double) * 9 * N, "adjoint state")) ||
        (st = A.alloc((void**)&A.seg, sizeof(double) * 9 * (size_t)N * checkpoint_every, "adjoint segment")))
        return st;
    if ((st = A.cuda(cudaMemset(W.err, 0, sizeof(int32_t)), "adjoint"))) return st;
    if ((st = A.cuda((cudaError_t)adj_set_smem_limit(adj_smem_bytes(nbmax)), "adjoint shared memory"))) return st;
    return CDX_OK;
}

void cdx_adj_destroy(cdx_adj* h) { delete h; }

const char* cdx_adj_last_error(cdx_adj* h) { return h ? h->a.err.c_str() : "null handle"; }

int cdx_adj_forward(cdx_adj* h, int32_t nsteps, const double* x0, const double* v0, const double* w0,
                    const double* mu_scene, double* xT, double* vT, double* wT) {
    if (!h || nsteps < 0 || !x0 || !v0 || !w0 || !mu_scene) return CDX_ERR_ARG;
    Adj& A = h->a;
    const AdjProblem& P = A.P;
    const size_t n3 = 3 * (size_t)P.N;
    int st;
    const int nck = nsteps > 0 ? (nsteps + A.ck_every - 1) / A.ck_every : 0;
    if (nck > A.nck) {
        A.release(A.ck, sizeof(double) * 9 * (size_t)P.N * A.nck);
        A.ck = nullptr;
        A.nck = 0;
        if ((st = A.alloc((void**)&A.ck, sizeof(double) * 9 * (size_t)P.N * nck, "adjoint checkpoints"))) return st;
        A.nck = nck;
    }
    cudaMemcpyAsync(A.cur, x0, sizeof(double) * n3, cudaMemcpyHostToDevice, A.stream);
    cudaMemcpyAsync(A.cur + n3, v0, sizeof(double) * n3, cudaMemcpyHostToDevice, A.stream);
    cudaMemcpyAsync(A.cur + 2 * n3, w0, sizeof(double) * n3, cudaMemcpyHostToDevice, A.stream);
    cudaMemcpyAsync(A.mu, mu_scene, sizeof(double) * P.nsc, cudaMemcpyHostToDevice, A.stream);
    cudaMemsetAsync(A.W.err, 0, sizeof(int32_t), A.stream);
    cudaMemsetAsync(A.W.ncsum, 0, sizeof(long long) * P.nsc, A.stream);
    for (int t = 0; t < nsteps; ++t) {
        if (t % A.ck_every == 0)
            cudaMemcpyAsync(A.ck + (size_t)(t / A.ck_every) * 3 * n3, A.cur, sizeof(double) * 3 * n3,
                            cudaMemcpyDeviceToDevice, A.stream);
        launch_adj_step(P, A.W, A.mu, A.cur, A.cur + n3, A.cur + 2 * n3, A.nxt, A.nxt + n3, A.nxt + 2 * n3, 0, 1,
                        A.nbmax, A.stream);
        std::swap(A.cur, A.nxt);
    }
    if ((st = check_last(A, "adjoint forward"))) return st;
    int32_t e = 0;
    if ((st = A.cuda(cudaMemcpy(&e, A.W.err, sizeof(int32_t), cudaMemcpyDeviceToHost), "adjoint"))) return st;
    if (e) return A.fail(CDX_ERR_OVERFLOW, "adjoint: a scene has more contacts than its slots (raise gpu.contact_capacity)");
    A.nsteps = nsteps;
    if (xT && (st = A.cuda(cudaMemcpy(xT, A.cur, sizeof(double) * n3, cudaMemcpyDeviceToHost), "adjoint"))) return st;
    if (vT && (st = A.cuda(cudaMemcpy(vT, A.cur + n3, sizeof(double) * n3, cudaMemcpyDeviceToHost), "adjoint")))
        return st;
    if (wT && (st = A.cuda(cudaMemcpy(wT, A.cur + 2 * n3, sizeof(double) * n3, cudaMemcpyDeviceToHost), "adjoint")))
        return st;
    return CDX_OK;
}

int cdx_adj_backward(cdx_adj* h, const double* gxT, const double* gvT, const double* gwT, double* gx0, double* gv0,
                     double* gw0, double* gmu) {
    if (!h || !gxT || !gvT || !gwT) return CDX_ERR_ARG;
    Adj& A = h->a;
    const AdjProblem& P = A.P;
    const size_t n3 = 3 * (size_t)P.N;
    int st;
    cudaMemcpyAsync(A.g, gxT, sizeof(double) * n3, cudaMemcpyHostToDevice, A.stream);
    cudaMemcpyAsync(A.g + n3, gvT, sizeof(double) * n3, cudaMemcpyHostToDevice, A.stream);
    cudaMemcpyAsync(A.g + 2 * n3, gwT, sizeof(double) * n3, cudaMemcpyHostToDevice, A.stream);
    cudaMemsetAsync(A.gmu, 0, sizeof(double) * P.nsc, A.stream);
    cudaMemsetAsync(A.W.err, 0, sizeof(int32_t), A.stream);
    const int T = A.nsteps;
    for (int sg = (T + A.ck_every - 1) / A.ck_every - 1; sg >= 0; --sg) {
        const int t0 = sg * A.ck_every, t1 = std::min(T, t0 + A.ck_every);
        // the segment's step inputs, recomputed from its checkpoint
        cudaMemcpyAsync(A.seg, A.ck + (size_t)sg * 3 * n3, sizeof(double) * 3 * n3, cudaMemcpyDeviceToDevice, A.stream);
        for (int t = t0; t + 1 < t1; ++t) {
            const double* in = A.seg + (size_t)(t - t0) * 3 * n3;
            double* o = A.seg + (size_t)(t + 1 - t0) * 3 * n3;
            launch_adj_step(P, A.W, A.mu, in, in + n3, in + 2 * n3, o, o + n3, o + 2 * n3, 0, 0, A.nbmax, A.stream);
        }
        for (int t = t1 - 1; t >= t0; --t) {
            const double* in = A.seg + (size_t)(t - t0) * 3 * n3;
            launch_adj_step(P, A.W, A.mu, in, in + n3, in + 2 * n3, A.nxt, A.nxt + n3, A.nxt + 2 * n3, 1, 0, A.nbmax,
                            A.stream);
            launch_adj_back(P, A.W, A.mu, A.g, A.g + n3, A.g + 2 * n3, A.gmu, A.nbmax, A.stream);
        }
    }
    if ((st = check_last(A, "adjoint backward"))) return st;
    int32_t e = 0;
    if ((st = A.cuda(cudaMemcpy(&e, A.W.err, sizeof(int32_t), cudaMemcpyDeviceToHost), "adjoint"))) return st;
    if (e) return A.fail(CDX_ERR_OVERFLOW, "adjoint: a scene has more contacts than its slots (raise gpu.contact_capacity)");
    if (gx0 && (st = A.cuda(cudaMemcpy(gx0, A.g, sizeof(double) * n3, cudaMemcpyDeviceToHost), "adjoint"))) return st;
    if (gv0 && (st = A.cuda(cudaMemcpy(gv0, A.g + n3, sizeof(double) * n3, cudaMemcpyDeviceToHost), "adjoint")))
        return st;
    if (gw0 && (st = A.cuda(cudaMemcpy(gw0, A.g + 2 * n3, sizeof(double) * n3, cudaMemcpyDeviceToHost), "adjoint")))
        return st;
    if (gmu && (st = A.cuda(cudaMemcpy(gmu, A.gmu, sizeof(double) * P.nsc, cudaMemcpyDeviceToHost), "adjoint")))
        return st;
    return CDX_OK;
}

int cdx_adj_contact_counts(cdx_adj* h, int64_t* per_scene) {
    if (!h || !per_scene) return CDX_ERR_ARG;
    Adj& A = h->a;
    static_assert(sizeof(long long) == sizeof(int64_t), "contact sums are 64-bit");
    return A.cuda(cudaMemcpy(per_scene, A.W.ncsum, sizeof(int64_t) * A.P.nsc, cudaMemcpyDeviceToHost), "adjoint");
}

int cdx_adj_info(cdx_adj* h, int64_t* contact_slots, int64_t* device_bytes, int32_t* checkpoints) {
    if (!h) return CDX_ERR_ARG;
    if (contact_slots) *contact_slots = h->a.W.cap;
    if (device_bytes) *device_bytes = (int64_t)h->a.bytes;
    if (checkpoints) *checkpoints = h->a.nck;
    return CDX_OK;
}

}  // extern "C"
