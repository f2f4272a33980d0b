// Host side of the engine: owns the device memory and the stream, and drives one Moreau midpoint
// step as a sequence of kernel launches (MoreauIntegrator::step, src/physics/integration/moreau.cpp:6-13):
//   refreshState -> drift (1-theta)h -> collision -> contact rows -> projected Jacobi -> write
//   velocities -> drift theta h.
// The C-ABI entry points (include/cdx.h) are implemented at the end of this file.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/cdx.h"
#include "cdx_internal.h"
#include "engine.h"

using namespace cdx;

namespace cdx {

namespace {
// The rotation of a unit quaternion (x, y, z, w), row-major, in the arithmetic of the kernels'
// rotmat; the static geometry turns body-frame directions with it.
void host_rotmat(const double* q, double* R) {
    const double x = q[0], y = q[1], z = q[2], w = q[3];
    const double tx = 2.0 * x, ty = 2.0 * y, tz = 2.0 * z;
    const double twx = tx * w, twy = ty * w, twz = tz * w;
    const double txx = tx * x, txy = ty * x, txz = tz * x;
    const double tyy = ty * y, tyz = tz * y, tzz = tz * z;
    R[0] = 1.0 - (tyy + tzz); R[1] = txy - twz;         R[2] = txz + twy;
    R[3] = txy + twz;         R[4] = 1.0 - (txx + tzz); R[5] = tyz - twx;
    R[6] = txz - twy;         R[7] = tyz + twx;         R[8] = 1.0 - (txx + tyy);
}
}  // namespace

const char* status_name(int st) {
    switch (st) {
        case CDX_OK: return "ok";
        case CDX_ERR_ARG: return "invalid argument";
        case CDX_ERR_CUDA: return "CUDA error";
        case CDX_ERR_OVERFLOW: return "overflow";
        case CDX_ERR_NONFINITE: return "non-finite value";
        case CDX_ERR_TIMEOUT: return "timeout";
        case CDX_ERR_UNSUPPORTED: return "unsupported";
        case CDX_ERR_STATE: return "bad state";
    }
    return "unknown";
}

}  // namespace cdx

int Engine::fail(int st, const std::string& msg) {
    err = std::string(status_name(st)) + ": " + msg;
    return st;
}

int Engine::cuda_check(cudaError_t e, const char* where) {
    if (e == cudaSuccess) return CDX_OK;
    return fail(CDX_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

int Engine::dalloc(void** p, size_t bytes, const char* what) {
    *p = nullptr;
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) return fail(CDX_ERR_CUDA, std::string("cudaMalloc ") + what + ": " + cudaGetErrorString(e));
    owned.push_back(*p);
    return CDX_OK;
}

void Engine::dfree(void* p) {
    if (!p) return;
    auto it = std::find(owned.begin(), owned.end(), p);
    if (it != owned.end()) owned.erase(it);
    cudaFree(p);
}

Engine::~Engine() {
    delete out;  // drains the writer queue
    out = nullptr;
    if (stream) cudaStreamSynchronize(stream);
    destroy_split();
    delete csr;
    csr = nullptr;
    for (void* p : owned) cudaFree(p);
    owned.clear();
    if (hs) cudaFreeHost(hs);
    for (auto& e : ev) if (e) cudaEventDestroy(e);
    if (stream) cudaStreamDestroy(stream);
}

int Engine::init(const cdx_config& c) {
    cfg = c;
    if (cfg.output_interval_steps > 0) out = new cdx::Output(cfg);
    if (int st0 = check_solver_config(cfg)) return st0;
    int st = cuda_check(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate");
    if (st) return st;
    st = cuda_check(cudaMallocHost((void**)&hs, sizeof(DevScalars)), "cudaMallocHost");
    if (st) return st;
    std::memset(hs, 0, sizeof(DevScalars));
    for (auto& e : ev) {
        st = cuda_check(cudaEventCreate(&e), "cudaEventCreate");
        if (st) return st;
    }
    return CDX_OK;
}

// The solver settings this library runs, and a clear refusal for the others:
//  - the split form runs the reference's Nesterov loop and the standard loop's tolerance exit in
//    its cooperative solve; Chebyshev and Anderson (selected when Nesterov is off, as in
//    projected_jacobi.cpp:470-491) run in the plain FP64 method only;
//  - solver.type=condensed runs in the plain FP64 method with condensed.sweep_mode gauss_seidel,
//    jacobi or colored (chaotic, and its Nesterov and Chebyshev loops, are not built);
//  - solver.type=projected_gauss_seidel runs its plain loop in the plain FP64 method (its Nesterov
//    loop is not built).
int Engine::check_solver_config(const cdx_config& c) {
    if (c.solver_type < 0 || c.solver_type > 2)
        return fail(CDX_ERR_UNSUPPORTED,
                    "only solver.type=projected_jacobi, projected_gauss_seidel and condensed are on this path");
    if (c.gpu_precision == CDX_PRECISION_SPLIT && !c.pj_nesterov && (c.pj_chebyshev || c.pj_anderson))
        return fail(CDX_ERR_UNSUPPORTED, "pj.chebyshev and pj.anderson run in the plain FP64 method only "
                                         "(gpu.precision=fp64); the split form runs pj.nesterov and the standard loop");
    if (c.solver_type == 1) {
        if (c.gpu_precision != CDX_PRECISION_FP64)
            return fail(CDX_ERR_UNSUPPORTED, "solver.type=condensed runs in the plain FP64 method (gpu.precision=fp64)");
        if (c.condensed_sweep_mode < 0 || c.condensed_sweep_mode > 2)
            return fail(CDX_ERR_UNSUPPORTED, "condensed.sweep_mode=chaotic is not on the GPU path (its result depends "
                                             "on the order of unsynchronised updates)");
        if (c.pj_nesterov || c.pj_chebyshev)
            return fail(CDX_ERR_UNSUPPORTED, "solver.type=condensed runs its standard loop (no pj.nesterov or pj.chebyshev)");
    }
    if (c.solver_type == 2) {
        if (c.gpu_precision != CDX_PRECISION_FP64)
            return fail(CDX_ERR_UNSUPPORTED,
                        "solver.type=projected_gauss_seidel runs in the plain FP64 method (gpu.precision=fp64)");
        if (c.pj_nesterov)
            return fail(CDX_ERR_UNSUPPORTED, "solver.type=projected_gauss_seidel runs its plain loop (no pj.nesterov)");
    }
    return CDX_OK;
}

// ProjectedJacobiSolver holds a reference to the Config and reads its pj.* settings at every solve
// (projected_jacobi.cpp:451-500), so a caller may change them between steps. Here the new settings
// apply from the next step; the precision (which selects the buffers) and the frame output (whose
// writer is set up at creation) stay as created.
int Engine::set_config(const cdx_config& c) {
    if (c.gpu_precision != cfg.gpu_precision)
        return fail(CDX_ERR_STATE, "gpu.precision is fixed when the context is created");
    if (int st0 = check_solver_config(c)) return st0;
    cdx_config n = c;
    n.output_interval_steps = cfg.output_interval_steps;
    n.output_write_contact_manifolds = cfg.output_write_contact_manifolds;
    std::memcpy(n.output_folder, cfg.output_folder, sizeof(n.output_folder));
    std::memcpy(n.output_filename_prefix, cfg.output_filename_prefix, sizeof(n.output_filename_prefix));
    if (stream) cudaStreamSynchronize(stream);
    cfg = n;
    split_config_changed();
    return CDX_OK;
}

int Engine::load_scene(const cdx_scene& s) {
    if (s.num_bodies < 0 || s.num_statics < 0) return fail(CDX_ERR_ARG, "negative sizes");
    const int N = s.num_bodies, S = s.num_statics;
    if (N > 0 && (!s.pos || !s.quat || !s.vel || !s.omega || !s.radius || !s.mass || !s.inertia || !s.mu ||
                  !s.rest_n || !s.rest_t))
        return fail(CDX_ERR_ARG, "missing body arrays");
    if (S > 0 && (!s.static_kind || !s.static_pos || !s.static_quat || !s.static_vel || !s.static_omega ||
                  !s.static_dir || !s.static_mu || !s.static_rest_n || !s.static_rest_t))
        return fail(CDX_ERR_ARG, "missing static arrays");
    if ((int64_t)N * 2 + 2 >= (int64_t)INT32_MAX / 2) return fail(CDX_ERR_ARG, "too many bodies");
    const int nsc = std::max(1, s.num_scenes);
    // scene ranges (bodies and statics must be grouped by scene)
    std::vector<int32_t> bsc(N, 0), ssc(S, 0);
    if (s.body_scene) std::copy(s.body_scene, s.body_scene + N, bsc.begin());
    if (s.static_scene) std::copy(s.static_scene, s.static_scene + S, ssc.begin());
    std::vector<int32_t> bstart(nsc + 1, 0), sstart(nsc + 1, 0);
    for (int i = 0; i < N; ++i) {
        if (bsc[i] < 0 || bsc[i] >= nsc || (i > 0 && bsc[i] < bsc[i - 1])) return fail(CDX_ERR_ARG, "body_scene must be nondecreasing in [0, num_scenes)");
        bstart[bsc[i] + 1]++;
    }
    for (int i = 0; i < S; ++i) {
        if (ssc[i] < 0 || ssc[i] >= nsc || (i > 0 && ssc[i] < ssc[i - 1])) return fail(CDX_ERR_ARG, "static_scene must be nondecreasing in [0, num_scenes)");
        sstart[ssc[i] + 1]++;
    }
    int maxst = 0;
    for (int k = 0; k < nsc; ++k) {
        maxst = std::max(maxst, sstart[k + 1]);
        bstart[k + 1] += bstart[k];
        sstart[k + 1] += sstart[k];
    }
    for (int i = 0; i < N; ++i) {
        if (!(s.radius[i] > 0) || !(s.mass[i] > 0) || !(s.inertia[i] > 0))
            return fail(CDX_ERR_ARG, "bodies need positive radius, mass and inertia");
    }
    for (int i = 0; i < S; ++i) {
        const int k = s.static_kind[i];
        if (k != CDX_STATIC_HALFSPACE && k != CDX_STATIC_DRUM && k != CDX_STATIC_CYLINDER && k != CDX_STATIC_BOX)
            return fail(CDX_ERR_ARG, "unknown static kind");
        if (k == CDX_STATIC_CYLINDER &&
            (!s.static_radius || !s.static_half_length || !(s.static_radius[i] > 0) || !(s.static_half_length[i] > 0)))
            return fail(CDX_ERR_ARG, "a cylinder needs a positive radius and half length");
        if (k == CDX_STATIC_BOX) {
            if (!s.static_half_extents) return fail(CDX_ERR_ARG, "a box needs its half extents");
            for (int c = 0; c < 3; ++c)
                if (!(s.static_half_extents[3 * (size_t)i + c] > 0) || !std::isfinite(s.static_half_extents[3 * (size_t)i + c]))
                    return fail(CDX_ERR_ARG, "a box needs positive, finite half extents");
        }
    }

    // host staging: body fields (field-major)
    std::vector<double> B((size_t)BF_COUNT * N, 0.0);
    auto bf = [&](int f, int i) -> double& { return B[(size_t)f * N + i]; };
    rmax = 0;
    for (int i = 0; i < N; ++i) {
        for (int k = 0; k < 3; ++k) {
            bf(BF_PX + k, i) = s.pos[3 * (size_t)i + k];
            bf(BF_VX + k, i) = s.vel[3 * (size_t)i + k];
            bf(BF_WX + k, i) = s.omega[3 * (size_t)i + k];
        }
        for (int k = 0; k < 4; ++k) bf(BF_QX + k, i) = s.quat[4 * (size_t)i + k];
        bf(BF_RAD, i) = s.radius[i];
        bf(BF_MASS, i) = s.mass[i];
        bf(BF_INERTIA, i) = s.inertia[i];
        bf(BF_MU, i) = s.mu[i];
        bf(BF_RN, i) = s.rest_n[i];
        bf(BF_RT, i) = s.rest_t[i];
        // rebuildMass_ (dynamics_assembler.cpp:41-62): Minv = 1/m, M_ii = 1/Minv
        const double il = 1.0 / s.mass[i], ia = 1.0 / s.inertia[i];
        bf(BF_MINVL, i) = il;
        bf(BF_MINVA, i) = ia;
        bf(BF_ML, i) = il > 0.0 ? 1.0 / il : 0.0;
        bf(BF_MA, i) = ia > 0.0 ? 1.0 / ia : 0.0;
        rmax = std::max(rmax, s.radius[i]);
    }
    std::vector<double> St((size_t)SF_COUNT * S, 0.0);
    auto sf = [&](int f, int i) -> double& { return St[(size_t)f * S + i]; };
    for (int i = 0; i < S; ++i) {
        for (int k = 0; k < 3; ++k) {
            sf(SF_PX + k, i) = s.static_pos[3 * (size_t)i + k];
            sf(SF_VX + k, i) = s.static_vel[3 * (size_t)i + k];
            sf(SF_WX + k, i) = s.static_omega[3 * (size_t)i + k];
        }
        for (int k = 0; k < 4; ++k) sf(SF_QX + k, i) = s.static_quat[4 * (size_t)i + k];
        // plane.normal.normalized(), d = n . x (collision_coal.cpp:292-297)
        const double* u = &s.static_dir[3 * (size_t)i];
        const double n2 = (u[0] * u[0] + u[1] * u[1]) + u[2] * u[2];
        const double n = std::sqrt(n2);
        double un[3];
        for (int k = 0; k < 3; ++k) un[k] = n2 > 0 ? u[k] / n : u[k];
        for (int k = 0; k < 3; ++k) sf(SF_DX + k, i) = un[k];
        const double* p = &s.static_pos[3 * (size_t)i];
        sf(SF_D, i) = (un[0] * p[0] + un[1] * p[1]) + un[2] * p[2];
        sf(SF_RAD, i) = s.static_radius ? s.static_radius[i] : 0.0;
        sf(SF_HL, i) = s.static_half_length ? s.static_half_length[i] : 0.0;
        // a cylinder's axis in its own frame, R(q0)^T u, so that the axis turns with the static
        double R0[9];
        host_rotmat(&s.static_quat[4 * (size_t)i], R0);
        for (int k = 0; k < 3; ++k) sf(SF_AX + k, i) = (R0[0 + k] * un[0] + R0[3 + k] * un[1]) + R0[6 + k] * un[2];
        for (int k = 0; k < 3; ++k)
            sf(SF_EX + k, i) = (s.static_kind[i] == CDX_STATIC_BOX) ? s.static_half_extents[3 * (size_t)i + k] : 0.0;
        sf(SF_MU, i) = s.static_mu[i];
        sf(SF_RN, i) = s.static_rest_n[i];
        sf(SF_RT, i) = s.static_rest_t[i];
    }

    // grid over the initial bounding box plus statics' anchor points, padded
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int i = 0; i < N; ++i)
        for (int k = 0; k < 3; ++k) {
            lo[k] = std::min(lo[k], s.pos[3 * (size_t)i + k]);
            hi[k] = std::max(hi[k], s.pos[3 * (size_t)i + k]);
        }
    if (N == 0)
        for (int k = 0; k < 3; ++k) { lo[k] = 0; hi[k] = 1; }
    // (a scene without bodies gets a grid of a few cells: nothing is ever sorted into it)
    const double cell = N > 0 ? 2.0 * rmax * 1.0001 + 1e-9 : 1.0;
    for (int k = 0; k < 3; ++k) {
        const double pad = 0.05 * (hi[k] - lo[k]) + 2 * cell;
        lo[k] -= pad;
        hi[k] += pad;
    }
    Grid g{};
    int64_t ncells = 1;
    for (int k = 0; k < 3; ++k) {
        g.lo[k] = lo[k];
        g.dim[k] = (int)std::min<double>(std::ceil((hi[k] - lo[k]) / cell) + 1, 1 << 20);
        ncells *= g.dim[k];
    }
    // keep the dense cell table modest: coarsen cells if needed (still >= 2 rmax, so exact); the
    // count is formed in double, as a fine grid over a wide box overflows 64-bit integers
    double cs = cell;
    double nd = (double)g.dim[0] * (double)g.dim[1] * (double)g.dim[2];
    while (nd > (double)((int64_t)64 << 20)) {
        cs *= 1.25;
        nd = 1.0;
        for (int k = 0; k < 3; ++k) nd *= std::ceil((hi[k] - lo[k]) / cs) + 1.0;
    }
    if (cs != cell) {
        ncells = 1;
        for (int k = 0; k < 3; ++k) {
            g.dim[k] = (int)(std::ceil((hi[k] - lo[k]) / cs) + 1.0);
            ncells *= g.dim[k];
        }
    }
    g.cell = cs;
    g.ncells = ncells;
    g.key_bits = 1;
    while (((int64_t)1 << g.key_bits) < ncells) ++g.key_bits;
    grid = g;

    // free any previous scene
    cudaStreamSynchronize(stream);
    destroy_split();
    for (void* p : owned) cudaFree(p);
    owned.clear();
    delete csr;  // its device buffers were in the owned list
    csr = nullptr;
    sc = Scene{};
    C = Contacts{};
    inc = Incidence{};
    trace_dev = nullptr;
    tmp = nullptr;
    tmp_bytes = 0;
    nc = 0;
    prev_count = 0;
    gen = 0;

    int st;
    sc.N = N;
    sc.S = S;
    sc.nscenes = nsc;
    sc.max_statics = maxst;
    if ((st = dalloc((void**)&sc.B, sizeof(double) * B.size(), "bodies"))) return st;
    if ((st = dalloc((void**)&sc.body_scene, sizeof(int32_t) * std::max(1, N), "body_scene"))) return st;
    if ((st = dalloc((void**)&sc.St, sizeof(double) * std::max<size_t>(1, St.size()), "statics"))) return st;
    if ((st = dalloc((void**)&sc.static_kind, sizeof(int32_t) * std::max(1, S), "static_kind"))) return st;
    if ((st = dalloc((void**)&sc.static_scene, sizeof(int32_t) * std::max(1, S), "static_scene"))) return st;
    if ((st = dalloc((void**)&sc.scene_body_start, sizeof(int32_t) * (nsc + 1), "scene ranges"))) return st;
    if ((st = dalloc((void**)&sc.scene_static_start, sizeof(int32_t) * (nsc + 1), "scene ranges"))) return st;
    std::vector<int32_t> kind(s.static_kind, s.static_kind + S);
    if ((st = cuda_check(cudaMemcpy(sc.B, B.data(), sizeof(double) * B.size(), cudaMemcpyHostToDevice), "upload"))) return st;
    if (N && (st = cuda_check(cudaMemcpy(sc.body_scene, bsc.data(), sizeof(int32_t) * N, cudaMemcpyHostToDevice), "upload"))) return st;
    if (S) {
        if ((st = cuda_check(cudaMemcpy(sc.St, St.data(), sizeof(double) * St.size(), cudaMemcpyHostToDevice), "upload"))) return st;
        if ((st = cuda_check(cudaMemcpy(sc.static_kind, kind.data(), sizeof(int32_t) * S, cudaMemcpyHostToDevice), "upload"))) return st;
        if ((st = cuda_check(cudaMemcpy(sc.static_scene, ssc.data(), sizeof(int32_t) * S, cudaMemcpyHostToDevice), "upload"))) return st;
    }
    if ((st = dalloc((void**)&smot, sizeof(double) * 13 * std::max(1, S), "static motion"))) return st;
    if ((st = dalloc((void**)&smflag, sizeof(int32_t) * std::max(1, S), "static motion"))) return st;
    if ((st = cuda_check(cudaMemset(smflag, 0, sizeof(int32_t) * std::max(1, S)), "static motion"))) return st;
    h_smot.assign(13 * (size_t)S, 0.0);
    h_smflag.assign((size_t)S, 0);
    smotion_pending = false;
    if ((st = cuda_check(cudaMemcpy(sc.scene_body_start, bstart.data(), sizeof(int32_t) * (nsc + 1), cudaMemcpyHostToDevice), "upload"))) return st;
    if ((st = cuda_check(cudaMemcpy(sc.scene_static_start, sstart.data(), sizeof(int32_t) * (nsc + 1), cudaMemcpyHostToDevice), "upload"))) return st;
    h_scene_body_start = bstart;
    h_scene_static_start = sstart;

    // per-body work arrays
    if ((st = dalloc((void**)&rhs, sizeof(double) * 6 * std::max(1, N), "rhs"))) return st;
    if ((st = dalloc((void**)&x, sizeof(double) * 6 * std::max(1, N), "x"))) return st;
    if ((st = dalloc((void**)&stage, sizeof(double) * 13 * std::max(1, N), "state staging"))) return st;
    if ((st = dalloc((void**)&cell_key_in, sizeof(uint32_t) * std::max(1, N), "grid"))) return st;
    if ((st = dalloc((void**)&cell_val_in, sizeof(uint32_t) * std::max(1, N), "grid"))) return st;
    if ((st = dalloc((void**)&cell_key_out, sizeof(uint32_t) * std::max(1, N), "grid"))) return st;
    if ((st = dalloc((void**)&cell_val_out, sizeof(uint32_t) * std::max(1, N), "grid"))) return st;
    if ((st = dalloc((void**)&pos32, sizeof(float4) * std::max(1, N), "grid"))) return st;
    if ((st = dalloc((void**)&plist64, sizeof(int32_t) * PLIST64 * std::max(1, N), "grid"))) return st;
    if ((st = dalloc((void**)&cell_start, sizeof(int32_t) * ncells, "grid"))) return st;
    if ((st = dalloc((void**)&cell_end, sizeof(int32_t) * ncells, "grid"))) return st;
    const int64_t nflag = (int64_t)std::max(1, N) * std::max(1, maxst);
    if ((st = dalloc((void**)&sflags, sizeof(int32_t) * nflag, "static flags"))) return st;
    if ((st = dalloc((void**)&spos, sizeof(int32_t) * nflag, "static flags"))) return st;
    if ((st = dalloc((void**)&sflags_prev, sizeof(int32_t) * nflag, "static flags"))) return st;
    if ((st = dalloc((void**)&spos_prev, sizeof(int32_t) * nflag, "static flags"))) return st;
    if ((st = dalloc((void**)&poff_prev, sizeof(int32_t) * (N + 1), "pair offsets"))) return st;
    if ((st = dalloc((void**)&pcount, sizeof(int32_t) * (N + 1), "pair counts"))) return st;
    if ((st = dalloc((void**)&poff, sizeof(int32_t) * (N + 1), "pair offsets"))) return st;
    if ((st = dalloc((void**)&ds, sizeof(DevScalars), "scalars"))) return st;
    if ((st = dalloc((void**)&inc.start, sizeof(int32_t) * (N + 1), "incidence"))) return st;
    if ((st = dalloc((void**)&inc.end, sizeof(int32_t) * (N + 1), "incidence"))) return st;
    if ((st = cuda_check(cudaMemset(ds, 0, sizeof(DevScalars)), "memset"))) return st;
    if ((st = cuda_check(cudaMemset(pcount, 0, sizeof(int32_t) * (N + 1)), "memset"))) return st;
    const int64_t cap0 = std::max<int64_t>(1024, (int64_t)(cfg.gpu_contact_capacity_factor * std::max(1, N)));
    if ((st = ensure_contacts(cap0))) return st;
    if ((st = ensure_tmp(std::max<int64_t>(nflag, N + 1)))) return st;
    // host copies for the frame output
    oscene = cdx::OutputScene{};
    oscene.N = N;
    oscene.S = S;
    oscene.radius.assign(s.radius, s.radius + N);
    oscene.mu.assign(s.mu, s.mu + N);
    oscene.pos0.assign(s.pos, s.pos + 3 * (size_t)N);
    if (S > 0) {
        oscene.skind.assign(s.static_kind, s.static_kind + S);
        oscene.spos.assign(s.static_pos, s.static_pos + 3 * (size_t)S);
        oscene.sdir.assign(s.static_dir, s.static_dir + 3 * (size_t)S);
        oscene.smu.assign(s.static_mu, s.static_mu + S);
        oscene.srad.assign(S, 0.0);
        if (s.static_radius) oscene.srad.assign(s.static_radius, s.static_radius + S);
        oscene.shl.assign(S, 0.0);
        if (s.static_half_length) oscene.shl.assign(s.static_half_length, s.static_half_length + S);
        oscene.squat.assign(s.static_quat, s.static_quat + 4 * (size_t)S);
        oscene.she.assign(3 * (size_t)S, 0.0);
        if (s.static_half_extents) oscene.she.assign(s.static_half_extents, s.static_half_extents + 3 * (size_t)S);
    }
    if (out) {
        out->flush();
        delete out;  // a new scene starts new collections and rewrites the static geometry
        out = new cdx::Output(cfg);
        out->set_scene(oscene);
    }
    tracked.clear();
    out_time = 0.0;
    out_started = false;
    loaded = true;
    steps = 0;
    return CDX_OK;
}

int Engine::ensure_tmp(int64_t n) {
    const size_t need = std::max(scan_temp_bytes(n), sort_temp_bytes(n)) + 256;
    if (need <= tmp_bytes) return CDX_OK;
    if (tmp) dfree(tmp);
    tmp = nullptr;
    const size_t b = need + need / 4;
    int st = dalloc(&tmp, b, "scratch");
    if (st) return st;
    tmp_bytes = b;
    return CDX_OK;
}

// Contact arrays of capacity `cap`; the previous generation's keys/points/impulses survive growth.
int Engine::ensure_contacts(int64_t need) {
    if (need <= C.cap) return CDX_OK;
    const int64_t cap = std::max<int64_t>(need + need / 4, 1024);
    if (cap > (int64_t)INT32_MAX / 4) return fail(CDX_ERR_OVERFLOW, "contact count exceeds the 32-bit index range");
    Contacts n;
    n.cap = cap;
    int st;
    if ((st = dalloc((void**)&n.a, sizeof(int32_t) * cap, "contacts"))) return st;
    if ((st = dalloc((void**)&n.b, sizeof(int32_t) * cap, "contacts"))) return st;
    if ((st = dalloc((void**)&n.flags, sizeof(int32_t) * cap, "contacts"))) return st;
    if ((st = dalloc((void**)&n.rank, sizeof(int32_t) * cap, "contacts"))) return st;
    double** d9[] = {&n.dir, &n.cA, &n.cB, &n.rd, &n.rcA, &n.rcB};
    for (auto p : d9)
        if ((st = dalloc((void**)p, sizeof(double) * 9 * cap, "contacts"))) return st;
    double** d3[] = {&n.cb, &n.biasR, &n.dlam};
    for (auto p : d3)
        if ((st = dalloc((void**)p, sizeof(double) * 3 * cap, "contacts"))) return st;
    double** d1[] = {&n.mu, &n.eN, &n.eT};
    for (auto p : d1)
        if ((st = dalloc((void**)p, sizeof(double) * cap, "contacts"))) return st;
    if (cfg.gpu_precision == CDX_PRECISION_FP64)
        if ((st = dalloc((void**)&n.term, sizeof(double) * 36 * cap, "contact terms"))) return st;
    if (cfg.pj_rdiag_true_delassus && cfg.gpu_precision == CDX_PRECISION_FP64) {
        if ((st = dalloc((void**)&n.rb, sizeof(double) * 9 * cap, "contact blocks"))) return st;
        if ((st = dalloc((void**)&n.rb_full, sizeof(int32_t), "contact blocks"))) return st;
    }
    for (int gidx = 0; gidx < 2; ++gidx) {
        if ((st = dalloc((void**)&n.key[gidx], sizeof(unsigned long long) * cap, "contacts"))) return st;
        if ((st = dalloc((void**)&n.point[gidx], sizeof(double) * 3 * cap, "contacts"))) return st;
        if ((st = dalloc((void**)&n.lam[gidx], sizeof(double) * 3 * cap, "contacts"))) return st;
    }
    // carry the previous generation (field-major with the old stride)
    if (C.cap > 0 && prev_count > 0) {
        const int pg = gen ^ 1;
        st = cuda_check(cudaMemcpyAsync(n.key[pg], C.key[pg], sizeof(unsigned long long) * prev_count,
                                        cudaMemcpyDeviceToDevice, stream), "copy prev");
        if (st) return st;
        for (int k = 0; k < 3; ++k) {
            if ((st = cuda_check(cudaMemcpyAsync(n.point[pg] + k * cap, C.point[pg] + k * C.cap, sizeof(double) * prev_count,
                                                 cudaMemcpyDeviceToDevice, stream), "copy prev"))) return st;
            if ((st = cuda_check(cudaMemcpyAsync(n.lam[pg] + k * cap, C.lam[pg] + k * C.cap, sizeof(double) * prev_count,
                                                 cudaMemcpyDeviceToDevice, stream), "copy prev"))) return st;
        }
        cudaStreamSynchronize(stream);
    }
    if (C.cap > 0) {
        void* old[] = {C.a, C.b, C.flags, C.rank, C.dir, C.cA, C.cB, C.rd, C.rcA, C.rcB, C.cb, C.biasR, C.dlam,
                       C.mu, C.eN, C.eT, C.key[0], C.key[1], C.point[0], C.point[1], C.lam[0], C.lam[1],
                       C.rb, C.rb_full, C.term};
        for (void* p : old) dfree(p);
        ++reallocations;
    }
    C = n;
    // incidence (2 entries per contact) and frictionless scan
    void* oldi[] = {inc.key_in, inc.val_in, inc.key_out, inc.val_out, isfl, flscan};
    for (void* p : oldi) dfree(p);
    inc.cap = 2 * cap;
    if ((st = dalloc((void**)&inc.key_in, sizeof(uint32_t) * 2 * cap, "incidence"))) return st;
    if ((st = dalloc((void**)&inc.val_in, sizeof(uint32_t) * 2 * cap, "incidence"))) return st;
    if ((st = dalloc((void**)&inc.key_out, sizeof(uint32_t) * 2 * cap, "incidence"))) return st;
    if ((st = dalloc((void**)&inc.val_out, sizeof(uint32_t) * 2 * cap, "incidence"))) return st;
    if ((st = dalloc((void**)&isfl, sizeof(int32_t) * cap, "flags"))) return st;
    if ((st = dalloc((void**)&flscan, sizeof(int32_t) * cap, "flags"))) return st;
    return ensure_tmp(2 * cap);
}

int Engine::collide64() {
    const int N = sc.N;
    const double margin = cfg.collision_security_margin;
    launch_cell_keys(sc, grid, cell_key_in, cell_val_in, stream);
    ++launches;
    int st = cuda_check(sort_pairs(tmp, tmp_bytes, cell_key_in, cell_key_out, cell_val_in, cell_val_out, N,
                                   grid.key_bits, stream), "sort cells");
    if (st) return st;
    launches += 4;
    cudaMemsetAsync(cell_start, 0, sizeof(int32_t) * grid.ncells, stream);
    cudaMemsetAsync(cell_end, 0, sizeof(int32_t) * grid.ncells, stream);
    launch_ranges(cell_key_out, N, cell_start, cell_end, stream);
    ++launches;
    // static contacts: flags in (static, sphere) order, then positions
    const int64_t nflag = (int64_t)N * sc.max_statics;
    if (nflag > 0) {
        launch_static_flags64(sc, margin, sflags, stream);
        ++launches;
        if ((st = cuda_check(exclusive_scan(tmp, tmp_bytes, sflags, spos, nflag, stream), "scan"))) return st;
        launches += 2;
    }
    launch_pos32(sc, grid, pos32, stream);
    launch_pair_count64(sc, grid, cell_val_out, cell_start, cell_end, pos32, plist64, margin, pcount, ds, stream);
    launches += 2;
    if ((st = cuda_check(exclusive_scan(tmp, tmp_bytes, pcount, poff, N + 1, stream), "scan"))) return st;
    launches += 2;
    // totals to the host (one synchronisation per step: the contact count sizes everything after)
    int32_t tot[4] = {0, 0, 0, 0};
    if (nflag > 0) {
        cudaMemcpyAsync(&tot[0], spos + nflag - 1, sizeof(int32_t), cudaMemcpyDeviceToHost, stream);
        cudaMemcpyAsync(&tot[1], sflags + nflag - 1, sizeof(int32_t), cudaMemcpyDeviceToHost, stream);
    }
    cudaMemcpyAsync(&tot[2], poff + N, sizeof(int32_t), cudaMemcpyDeviceToHost, stream);
    cudaMemcpyAsync(&tot[3], &ds->overflow, sizeof(int32_t), cudaMemcpyDeviceToHost, stream);
    if ((st = cuda_check(cudaStreamSynchronize(stream), "collision counts"))) return st;
    if (tot[3]) return fail(CDX_ERR_OVERFLOW, "a sphere touches more than 64 higher-index spheres");
    const int64_t n_static = (int64_t)tot[0] + tot[1];
    const int64_t n_pair = tot[2];
    if ((st = ensure_contacts(n_static + n_pair))) return st;
    nc = (int)(n_static + n_pair);
    if (nflag > 0 && n_static > 0) {
        launch_static_write64(sc, margin, sflags, spos, C, gen, cfg.friction_combine, cfg.friction_enable, stream);
        ++launches;
    }
    if (n_pair > 0) {
        launch_pair_write64(sc, grid, cell_val_out, cell_start, cell_end, pos32, plist64, margin, poff,
                            (int32_t)n_static, C, gen,
                            cfg.friction_combine, cfg.friction_enable, ds, stream);
        ++launches;
    }
    return CDX_OK;
}

int Engine::setup64() {
    int st;
    const double match2 = cfg.collision_match_max_dist * cfg.collision_match_max_dist;
    if (C.rb_full) cudaMemsetAsync(C.rb_full, 0, sizeof(int32_t), stream);
    launch_contact_setup64(sc, C, gen, nc, prev_count, cfg.pj_alpha, match2, cfg.pj_warmstart, stream);
    launch_block_invert64(C, nc, stream);
    launch_frictionless_flags(C, nc, isfl, stream);
    launches += nc > 0 ? (C.rb ? 3 : 2) : 0;
    if (nc > 0) {
        if ((st = cuda_check(exclusive_scan(tmp, tmp_bytes, isfl, flscan, nc, stream), "scan"))) return st;
        launches += 2;
    }
    launch_rank_and_incidence(sc, C, nc, flscan, isfl, inc, stream, cfg.solver_type == 1 ? 1 : 0);
    int key_bits = 1;
    while (((int64_t)1 << key_bits) <= sc.N) ++key_bits;
    if (nc > 0) {
        ++launches;
        if ((st = cuda_check(sort_pairs(tmp, tmp_bytes, inc.key_in, inc.key_out, inc.val_in, inc.val_out, 2 * (int64_t)nc,
                                        key_bits, stream), "sort incidence"))) return st;
        launches += 4;
    }
    cudaMemsetAsync(inc.start, 0, sizeof(int32_t) * (sc.N + 1), stream);
    cudaMemsetAsync(inc.end, 0, sizeof(int32_t) * (sc.N + 1), stream);
    if (nc > 0) {
        launch_ranges(inc.key_out, 2 * (int64_t)nc, inc.start, inc.end, stream);
        ++launches;
    }
    return CDX_OK;
}

int Engine::ensure_accel() {
    const int64_t nx = 6 * (int64_t)sc.N, nl = 3 * C.cap;
    if (acc_st && nx == acc_nx && nl == acc_nl) return CDX_OK;
    double** bufs[] = {&acc_xk, &acc_xk1, &acc_xy, &acc_pk, &acc_pk1, &acc_py, &acc_part};
    for (auto b : bufs)
        if (*b) {
            dfree(*b);
            *b = nullptr;
        }
    if (acc_st) {
        dfree(acc_st);
        acc_st = nullptr;
    }
    int st;
    for (int k = 0; k < 3; ++k)
        if ((st = dalloc((void**)bufs[k], sizeof(double) * std::max<int64_t>(nx, 1), "accelerated loop"))) return st;
    for (int k = 3; k < 6; ++k)
        if ((st = dalloc((void**)bufs[k], sizeof(double) * std::max<int64_t>(nl, 1), "accelerated loop"))) return st;
    if ((st = dalloc((void**)&acc_part, sizeof(double) * std::max(accel_chunks(sc.N), 1), "accelerated loop"))) return st;
    if ((st = dalloc((void**)&acc_st, sizeof(AccelState), "accelerated loop"))) return st;
    acc_nx = nx;
    acc_nl = nl;
    return CDX_OK;
}

// nesterov_loop / chebyshev_loop (projected_jacobi.cpp:379-449, 179-222) of ProjectedJacobiSolver,
// plain FP64: the same sweeps as the standard loop, with the extrapolations, restarts and stop
// tests of the reference run as small device kernels so the loop needs no host decisions; the
// host polls the stop flag every gpu.check_every sweeps.
int Engine::solve64_accel() {
    const int N = sc.N, nv = 6 * N;
    int st;
    if ((st = ensure_accel())) return st;
    const int64_t nx = acc_nx, nl = acc_nl;
    double* lam = C.lam[gen];
    const bool nes = cfg.pj_nesterov != 0;
    cudaMemsetAsync(ds, 0, sizeof(DevScalars), stream);
    launch_accel_init(acc_st, stream);
    if (!nes) launch_spectral_radius(sc, C, inc, nc, acc_xy, acc_xk, acc_part, acc_st, stream);
    // xk = xk1 (= xy) = x0, pk = pk1 (= py) = lambda0
    launch_accel_copy(acc_xk, x, nx, acc_pk, lam, nl, nullptr, stream);
    launch_accel_copy(acc_xk1, x, nx, acc_pk1, lam, nl, nullptr, stream);
    launch_accel_copy(acc_xy, x, nx, acc_py, lam, nl, nullptr, stream);
    const int maxit = std::max(1, cfg.pj_max_iterations);
    const int every = std::max(1, cfg.gpu_check_every);
    int it = 0;
    for (; it < maxit; ++it) {
        // the sweep starts from y (Nesterov) or from the extrapolated iterate xk1 (Chebyshev)
        if (nes)
            launch_accel_copy(x, acc_xy, nx, lam, acc_py, nl, ds, stream);
        else
            launch_accel_copy(x, acc_xk1, nx, lam, acc_pk1, nl, ds, stream);
        launch_sweep_contact64(sc, C, gen, nc, x, ds, 0, stream);
        launch_sweep_body64(sc, C, inc, x, 0.0, 0.0, 0, ds, stream);
        launch_check(ds, it, 0.0, nv, 0, stream);  // res_last and the sweep count
        if (nes) {
            launch_accel_copy(acc_xk1, x, nx, acc_pk1, lam, nl, ds, stream);
            launch_accel_reduce(N, ACC_VELRES, acc_xk1, acc_xy, nullptr, cfg.pj_tol_rel, cfg.pj_tol_abs, acc_part,
                                acc_st, &acc_st->sum_err, ds, stream);
            launch_accel_reduce(N, ACC_DOT, acc_xy, acc_xk1, acc_xk, 0.0, 0.0, acc_part, acc_st, &acc_st->sum_dot,
                                ds, stream);
            launch_nesterov_step(acc_st, ds, nv, cfg.pj_nesterov_beta_threshold, cfg.pj_nesterov_restart_limit, acc_xy,
                                 acc_xk, acc_xk1, nx, acc_py, acc_pk, acc_pk1, nl, cfg.gpu_residual_tol, stream);
            launches += 9;
        } else {
            launch_accel_reduce(N, ACC_VELRES, x, acc_xk1, nullptr, cfg.pj_tol_rel, cfg.pj_tol_abs, acc_part, acc_st,
                                &acc_st->sum_err, ds, stream);
            launch_chebyshev_step(acc_st, ds, nv, it, x, acc_xk, acc_xk1, nx, lam, acc_pk, acc_pk1, nl,
                                  cfg.gpu_residual_tol, stream);
            launches += 7;
        }
        if ((it + 1) % every == 0 && it + 1 < maxit) {
            cudaMemcpyAsync(&hs->done, &ds->done, sizeof(int32_t), cudaMemcpyDeviceToHost, stream);
            if ((st = cuda_check(cudaStreamSynchronize(stream), "poll"))) return st;
            if (hs->done) break;
        }
    }
    // the result is the loop's current iterate (xk1, pk1), as in the reference
    launch_accel_copy(x, acc_xk1, nx, lam, acc_pk1, nl, nullptr, stream);
    launch_sweep_contact64(sc, C, gen, nc, x, ds, 1, stream);
    launch_final_residual(ds, stream);
    launches += 3;
    return CDX_OK;
}

int Engine::ensure_anderson(int64_t nt) {
    AndersonBufs& A = anderson;
    const int m = std::max(1, cfg.pj_anderson_m);
    if (A.st && A.m == m && nt <= A.nt_cap && A.rowmap_cap >= 3 * C.cap) {
        A.nt = nt;
        return CDX_OK;
    }
    double** bufs[] = {&A.z, &A.w, &A.f, &A.cand, &A.zh, &A.fh, &A.part, &A.ls};
    for (auto b : bufs)
        if (*b) {
            dfree(*b);
            *b = nullptr;
        }
    if (A.rowmap) dfree(A.rowmap);
    if (A.st) dfree(A.st);
    A.rowmap = nullptr;
    A.st = nullptr;
    const int64_t cap = std::max<int64_t>(nt + nt / 4, 16);
    int st;
    for (int k = 0; k < 4; ++k)
        if ((st = dalloc((void**)bufs[k], sizeof(double) * cap, "Anderson loop"))) return st;
    for (int k = 4; k < 6; ++k)
        if ((st = dalloc((void**)bufs[k], sizeof(double) * cap * (m + 1), "Anderson loop"))) return st;
    if ((st = dalloc((void**)&A.part, sizeof(double) * anderson_chunks(cap) * anderson_sums(m), "Anderson loop")))
        return st;
    if ((st = dalloc((void**)&A.ls, sizeof(double) * ((int64_t)m * m + 2 * m), "Anderson loop"))) return st;
    if ((st = dalloc((void**)&A.rowmap, sizeof(int32_t) * std::max<int64_t>(3 * C.cap, 1), "Anderson loop"))) return st;
    if ((st = dalloc((void**)&A.st, sizeof(AndersonState), "Anderson loop"))) return st;
    A.m = m;
    A.nt = nt;
    A.nt_cap = cap;
    A.rowmap_cap = 3 * C.cap;
    return CDX_OK;
}

// anderson_loop (projected_jacobi.cpp:242-314) of ProjectedJacobiSolver, plain FP64: z = [x; impulse
// rows], one sweep g(z), and the mixed step z = g(z) - (dZ + dF) gamma over the last m residual
// differences, with gamma from the normal equations of the least squares problem (the reference
// solves it by a column-pivoted QR; both give the minimiser for a full-rank dF, and a singular
// system falls back to a plain step and drops the history as a non-finite gamma does there).
// Every decision runs on the device; the host polls the stop flag every gpu.check_every sweeps.
int Engine::solve64_anderson() {
    const int N = sc.N, nv = 6 * N;
    int st;
    const int nrows = nfl_rows();
    if ((st = ensure_anderson((int64_t)nv + nrows))) return st;
    double* lam = C.lam[gen];
    cudaMemsetAsync(ds, 0, sizeof(DevScalars), stream);
    launch_anderson_begin(C, gen, nc, flscan, isfl, N, x, anderson, stream);
    const int maxit = std::max(1, cfg.pj_max_iterations);
    const int every = std::max(1, cfg.gpu_check_every);
    for (int it = 0; it < maxit; ++it) {
        launch_anderson_scatter(N, x, lam, anderson, ds, stream);
        launch_sweep_contact64(sc, C, gen, nc, x, ds, 0, stream);
        launch_sweep_body64(sc, C, inc, x, 0.0, 0.0, 0, ds, stream);
        launch_check(ds, it, 0.0, nv, 0, stream);  // res_last and the sweep count
        launch_anderson_mix(N, x, lam, anderson, cfg.pj_tol_rel, cfg.pj_tol_abs, cfg.gpu_residual_tol, ds, stream);
        launches += 12;
        if ((it + 1) % every == 0 && it + 1 < maxit) {
            cudaMemcpyAsync(&hs->done, &ds->done, sizeof(int32_t), cudaMemcpyDeviceToHost, stream);
            if ((st = cuda_check(cudaStreamSynchronize(stream), "poll"))) return st;
            if (hs->done) break;
        }
    }
    // stopped: (x, lambda) hold g(z); otherwise the result is the loop's z
    launch_anderson_scatter(N, x, lam, anderson, ds, stream);
    launch_sweep_contact64(sc, C, gen, nc, x, ds, 1, stream);
    launch_final_residual(ds, stream);
    launches += 3;
    return CDX_OK;
}

int Engine::solve64() {
    const int N = sc.N;
    int st;
    launch_xinit64(sc, C, gen, inc, rhs, x, stream);
    ++launches;
    hs->done = 0;
    last_iters = 0;
    last_res = 0;
    last_res_final = 0;
    if (nc == 0) return CDX_OK;
    if ((cfg.pj_nesterov || cfg.pj_chebyshev) && !trace_next) return solve64_accel();
    if (cfg.pj_anderson && !trace_next) return solve64_anderson();
    cudaMemsetAsync(ds, 0, sizeof(DevScalars), stream);
    const int maxit = std::max(1, cfg.pj_max_iterations);
    const bool check_vel = !(cfg.pj_tol_abs == 0.0 && cfg.pj_tol_rel == 0.0);
    const int every = std::max(1, cfg.gpu_check_every);
    const int nrows = nfl_rows();
    if (trace_next) {
        trace_rows = nrows;
        trace_buf.clear();
        if (trace_dev) dfree(trace_dev);
        trace_dev = nullptr;
        if ((st = dalloc((void**)&trace_dev, sizeof(double) * (size_t)std::max(1, nrows), "trace"))) return st;
    }
    int it = 0;
    for (; it < maxit; ++it) {
        launch_sweep_contact64(sc, C, gen, nc, x, ds, 0, stream);
        launch_sweep_body64(sc, C, inc, x, cfg.pj_tol_abs, cfg.pj_tol_rel, check_vel && (it % 10 == 0), ds, stream);
        launch_check(ds, it, cfg.gpu_residual_tol, 6 * N, check_vel, stream);
        launches += 3;
        if (trace_next) {
            launch_trace64(C, gen, nc, flscan, isfl, trace_dev, stream);
            std::vector<double> h(nrows);
            cudaMemcpyAsync(h.data(), trace_dev, sizeof(double) * nrows, cudaMemcpyDeviceToHost, stream);
            cudaMemcpyAsync(&hs->done, &ds->done, sizeof(int32_t), cudaMemcpyDeviceToHost, stream);
            if ((st = cuda_check(cudaStreamSynchronize(stream), "trace"))) return st;
            if (hs->done && !trace_done_seen) {
                // the sweep that set the flag is kept; later ones are no-ops
                trace_buf.insert(trace_buf.end(), h.begin(), h.end());
                trace_done_seen = true;
                break;
            }
            trace_buf.insert(trace_buf.end(), h.begin(), h.end());
            continue;
        }
        if ((it + 1) % every == 0 && it + 1 < maxit) {
            cudaMemcpyAsync(&hs->done, &ds->done, sizeof(int32_t), cudaMemcpyDeviceToHost, stream);
            if ((st = cuda_check(cudaStreamSynchronize(stream), "poll"))) return st;
            if (hs->done) break;
        }
    }
    trace_next = false;
    trace_done_seen = false;
    // final FP64 complementarity residual of the solved state
    launch_sweep_contact64(sc, C, gen, nc, x, ds, 1, stream);
    launch_final_residual(ds, stream);
    launches += 2;
    return CDX_OK;
}

int Engine::nfl_rows() {
    // rows = frictionless contacts + 3 * frictional contacts
    int32_t a = 0, b = 0;
    if (nc == 0) return 0;
    cudaMemcpyAsync(&a, flscan + nc - 1, sizeof(int32_t), cudaMemcpyDeviceToHost, stream);
    cudaMemcpyAsync(&b, isfl + nc - 1, sizeof(int32_t), cudaMemcpyDeviceToHost, stream);
    cudaStreamSynchronize(stream);
    const int nfl = a + b;
    return nfl + 3 * (nc - nfl);
}

int Engine::step64() {
    const double dt = cfg.sim_dt, th = cfg.moreau_theta;
    int st;
    if (timing) cudaEventRecord(ev[0], stream);
    cudaMemsetAsync(&ds->nonfinite, 0, sizeof(int32_t), stream);
    launch_rhs64(sc, dt, cfg.sim_gravity, rhs, stream, cfg.moreau_implicit_gyroscopy);
    launch_drift64(sc, (1.0 - th) * dt, 1, stream);
    launches += 2;
    if (smotion_pending) {
        // Trajectory::update runs here, inside updateStateDependentTerms (dynamics_assembler.cpp:515-522)
        launch_static_motion64(sc, smot, smflag, stream);
        ++launches;
    }
    if ((st = collide64())) return st;
    if (timing) cudaEventRecord(ev[1], stream);
    if ((st = setup64())) return st;
    if (timing) cudaEventRecord(ev[2], stream);
    if ((st = (cfg.solver_type == 1 ? solve_condensed() : cfg.solver_type == 2 ? solve_pgs() : solve64()))) return st;
    if (timing) cudaEventRecord(ev[3], stream);
    launch_writeback64(sc, x, stream);
    launch_drift64(sc, th * dt, 0, stream, &ds->nonfinite);
    launches += 2;
    if (timing) cudaEventRecord(ev[4], stream);
    cudaMemcpyAsync(hs, ds, sizeof(DevScalars), cudaMemcpyDeviceToHost, stream);
    if ((st = cuda_check(cudaStreamSynchronize(stream), "step"))) return st;
    if ((st = cuda_check(cudaGetLastError(), "kernel launch"))) return st;
    last_iters = nc > 0 ? hs->iters : 0;
    last_res = nc > 0 ? hs->res_last : 0.0;
    last_res_final = nc > 0 ? hs->res_final : 0.0;
    last_rows = nc > 0 ? nfl_rows() : 0;
    prev_count = nc;
    contacts_loaded = false;
    gen ^= 1;
    ++steps;
    if (timing) {
        float a = 0, b = 0, c2 = 0, d = 0;
        cudaEventElapsedTime(&a, ev[0], ev[1]);
        cudaEventElapsedTime(&b, ev[1], ev[2]);
        cudaEventElapsedTime(&c2, ev[2], ev[3]);
        cudaEventElapsedTime(&d, ev[3], ev[4]);
        ms[0] = a; ms[1] = b; ms[2] = c2; ms[3] = d;
    }
    // a state that is no longer finite (an input NaN, or a blow-up) ends the step with an error;
    // the step itself completed and the context stays usable (cdx_set_state can repair the state)
    if (hs->nonfinite) return fail(CDX_ERR_NONFINITE, "the state after the step is not finite (NaN or infinity)");
    if (cond_diverged)
        return fail(CDX_ERR_NONFINITE, std::string(cfg.solver_type == 2 ? "projected Gauss-Seidel" : "condensed solver") +
                                           " diverged: the velocity-increment residual is not finite "
                                           "(pj.tol_abs and pj.tol_rel must not both be 0)");
    return CDX_OK;
}

int Engine::step(int nsteps) {
    if (!loaded) return fail(CDX_ERR_STATE, "no scene loaded");
    int st;
    // PhysicsPipeline::step (physics_pipeline.cpp:91-113): the first frame before the first
    // step, then a frame every output.interval_steps and the tracked rows every step
    if (out && out->vtk_on() && !out_started && nsteps > 0) {
        out_started = true;
        if ((st = output_frame())) return st;
    }
    for (int k = 0; k < nsteps; ++k) {
        st = (cfg.gpu_precision == CDX_PRECISION_SPLIT) ? step_split() : step64();
        if (st) return st;
        if (smotion_pending) {
            // a prescribed motion holds for one step
            cudaMemsetAsync(smflag, 0, sizeof(int32_t) * (size_t)std::max(1, sc.S), stream);
            std::fill(h_smflag.begin(), h_smflag.end(), 0);
            smotion_pending = false;
        }
        if (out) {
            out_time += cfg.sim_dt;
            if (out->due(steps) && (st = output_frame())) return st;
            if (!tracked.empty() && (st = output_tracked())) return st;
        }
    }
    return CDX_OK;
}

int Engine::output_frame() {
    cdx::OutputFrame f;
    const size_t N = (size_t)sc.N;
    f.step = steps;
    f.time = out_time;
    f.pos.resize(3 * N);
    f.quat.resize(4 * N);
    f.vel.resize(3 * N);
    f.omega.resize(3 * N);
    int st;
    if ((st = get_state(f.pos.data(), f.quat.data(), f.vel.data(), f.omega.data()))) return st;
    int32_t nc = 0;
    if ((st = get_contacts(nullptr, nullptr, nullptr, nullptr, nullptr, &nc))) return st;
    f.nc = nc;
    f.ia.resize(nc);
    f.ib.resize(nc);
    f.point.resize(3 * (size_t)nc);
    f.lambda.resize(3 * (size_t)nc);
    f.normal.resize(3 * (size_t)nc);
    if (nc > 0 && (st = get_contacts(f.ia.data(), f.ib.data(), f.point.data(), f.lambda.data(), f.normal.data(), &nc)))
        return st;
    out->frame(std::move(f));
    return CDX_OK;
}

int Engine::output_tracked() {
    const size_t N = (size_t)sc.N;
    launch_pack_state(sc, stage, stream);
    ++launches;
    std::vector<cdx::TrackedRow> rows(tracked.size());
    int st;
    for (size_t k = 0; k < tracked.size(); ++k) {
        const size_t i = (size_t)tracked[k].first;
        cdx::TrackedRow& r = rows[k];
        r.name = tracked[k].second;
        if ((st = cuda_check(cudaMemcpyAsync(r.p, stage + 3 * i, 24, cudaMemcpyDeviceToHost, stream), "tracked")) ||
            (st = cuda_check(cudaMemcpyAsync(r.q, stage + 3 * N + 4 * i, 32, cudaMemcpyDeviceToHost, stream), "tracked")) ||
            (st = cuda_check(cudaMemcpyAsync(r.v, stage + 7 * N + 3 * i, 24, cudaMemcpyDeviceToHost, stream), "tracked")) ||
            (st = cuda_check(cudaMemcpyAsync(r.w, stage + 10 * N + 3 * i, 24, cudaMemcpyDeviceToHost, stream), "tracked")))
            return st;
    }
    if ((st = cuda_check(cudaStreamSynchronize(stream), "tracked"))) return st;
    out->tracked(out_time, std::move(rows));
    return CDX_OK;
}

int Engine::track(int32_t body, const char* name) {
    if (!loaded) return fail(CDX_ERR_STATE, "no scene loaded");
    if (body < 0 || body >= sc.N || !name) return fail(CDX_ERR_ARG, "track: body index out of range");
    if (!out) {
        out = new cdx::Output(cfg);
        out->set_scene(oscene);
        out_started = steps > 0;  // frames (when on) start at the next due step
    }
    for (auto& t : tracked)
        if (t.first == body) {
            t.second = name;
            return CDX_OK;
        }
    tracked.emplace_back(body, name);
    return CDX_OK;
}

int Engine::output_flush() {
    if (!out) return CDX_OK;
    out->flush();
    const std::string e = out->last_error();
    return e.empty() ? CDX_OK : fail(CDX_ERR_STATE, e);
}

// The device address of a host array the GPU can read and write directly (pinned or registered
// memory), else nullptr (pageable memory goes through the staging buffer and the copy engines).
static void* device_view(const void* p) {
    if (!p) return nullptr;
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return (at.type == cudaMemoryTypeHost && at.devicePointer) ? at.devicePointer : nullptr;
}

// Trajectory::update (trajectory.cpp:69-120) evaluates the statics' position and velocity callbacks
// on the host; their results enter here for the coming step and are applied where the reference
// applies them, after the first drift and before contact detection. A halfspace's plane stays as
// built (CollisionCoal::applyTransforms gives halfspaces no transform, collision_coal.cpp:386-391):
// its motion enters the contacts through its velocity.
int Engine::set_static_motion(int32_t count, const int32_t* idx, const double* pos, const double* quat,
                              const double* vel, const double* omega) {
    if (!loaded) return fail(CDX_ERR_STATE, "no scene loaded");
    if (count < 0 || (count > 0 && !idx)) return fail(CDX_ERR_ARG, "static indices missing");
    const int f = (pos ? 1 : 0) | (quat ? 2 : 0) | (vel ? 4 : 0) | (omega ? 8 : 0);
    for (int32_t c = 0; c < count; ++c) {
        const int s = idx[c];
        if (s < 0 || s >= sc.S) return fail(CDX_ERR_ARG, "static index out of range");
        double* m = &h_smot[13 * (size_t)s];
        for (int k = 0; k < 3; ++k) {
            if (pos) m[k] = pos[3 * (size_t)c + k];
            if (vel) m[7 + k] = vel[3 * (size_t)c + k];
            if (omega) m[10 + k] = omega[3 * (size_t)c + k];
        }
        if (quat)
            for (int k = 0; k < 4; ++k) m[3 + k] = quat[4 * (size_t)c + k];
        for (int k = 0; k < 13; ++k)
            if (!std::isfinite(m[k]) && (f & (k < 3 ? 1 : k < 7 ? 2 : k < 10 ? 4 : 8)))
                return fail(CDX_ERR_ARG, "static motion must be finite");
        h_smflag[s] |= f;
    }
    if (count == 0 || sc.S == 0) return CDX_OK;
    int st;
    if ((st = cuda_check(cudaMemcpyAsync(smot, h_smot.data(), sizeof(double) * h_smot.size(), cudaMemcpyHostToDevice,
                                         stream), "static motion")))
        return st;
    if ((st = cuda_check(cudaMemcpyAsync(smflag, h_smflag.data(), sizeof(int32_t) * h_smflag.size(),
                                         cudaMemcpyHostToDevice, stream), "static motion")))
        return st;
    smotion_pending = true;
    return cuda_check(cudaStreamSynchronize(stream), "static motion");
}

int Engine::get_static_state(double* pos, double* quat, double* vel, double* omega) {
    if (!loaded) return fail(CDX_ERR_STATE, "no scene loaded");
    const size_t S = (size_t)sc.S;
    if (S == 0) return CDX_OK;
    std::vector<double> St((size_t)SF_COUNT * S);
    int st;
    if ((st = cuda_check(cudaMemcpyAsync(St.data(), sc.St, sizeof(double) * St.size(), cudaMemcpyDeviceToHost, stream),
                         "download statics")))
        return st;
    if ((st = cuda_check(cudaStreamSynchronize(stream), "download statics"))) return st;
    for (size_t s = 0; s < S; ++s) {
        for (int k = 0; k < 3; ++k) {
            if (pos) pos[3 * s + k] = St[(SF_PX + k) * S + s];
            if (vel) vel[3 * s + k] = St[(SF_VX + k) * S + s];
            if (omega) omega[3 * s + k] = St[(SF_WX + k) * S + s];
        }
        if (quat)
            for (int k = 0; k < 4; ++k) quat[4 * s + k] = St[(SF_QX + k) * S + s];
    }
    return CDX_OK;
}

int Engine::get_state(double* pos, double* quat, double* vel, double* omega) {
    if (!loaded) return fail(CDX_ERR_STATE, "no scene loaded");
    const size_t N = (size_t)sc.N;
    if (N == 0) return CDX_OK;
    int st;
    {
        // pinned caller arrays: one kernel writes them directly (coalesced, over the host link)
        double* dv[4] = {pos, quat, vel, omega};
        bool direct = true;
        for (auto& p : dv)
            if (p && !(p = (double*)device_view(p))) direct = false;
        if (direct) {
            launch_pack_state4(sc, dv[0], dv[1], dv[2], dv[3], stream);
            ++launches;
            return cuda_check(cudaStreamSynchronize(stream), "download");
        }
    }
    launch_pack_state(sc, stage, stream);
    ++launches;
    // one copy per requested array straight into the caller's buffers
    if (pos && (st = cuda_check(cudaMemcpyAsync(pos, stage, 8 * 3 * N, cudaMemcpyDeviceToHost, stream), "download"))) return st;
    if (quat && (st = cuda_check(cudaMemcpyAsync(quat, stage + 3 * N, 8 * 4 * N, cudaMemcpyDeviceToHost, stream), "download"))) return st;
    if (vel && (st = cuda_check(cudaMemcpyAsync(vel, stage + 7 * N, 8 * 3 * N, cudaMemcpyDeviceToHost, stream), "download"))) return st;
    if (omega && (st = cuda_check(cudaMemcpyAsync(omega, stage + 10 * N, 8 * 3 * N, cudaMemcpyDeviceToHost, stream), "download"))) return st;
    return cuda_check(cudaStreamSynchronize(stream), "download");
}

int Engine::set_state(const double* pos, const double* quat, const double* vel, const double* omega) {
    if (!loaded) return fail(CDX_ERR_STATE, "no scene loaded");
    const size_t N = (size_t)sc.N;
    if (N == 0) return CDX_OK;
    int st;
    {
        // pinned caller arrays: one kernel reads them directly; like a copy from pinned memory this
        // runs asynchronously on the engine's stream
        const double* dv[4] = {pos, quat, vel, omega};
        bool direct = true;
        for (auto& p : dv)
            if (p && !(p = (const double*)device_view(p))) direct = false;
        if (direct) {
            launch_unpack_state4(sc, dv[0], dv[1], dv[2], dv[3], stream);
            ++launches;
            return CDX_OK;
        }
    }
    int mask = 0;
    if (pos && (st = cuda_check(cudaMemcpyAsync(stage, pos, 8 * 3 * N, cudaMemcpyHostToDevice, stream), "upload"))) return st;
    if (quat && (st = cuda_check(cudaMemcpyAsync(stage + 3 * N, quat, 8 * 4 * N, cudaMemcpyHostToDevice, stream), "upload"))) return st;
    if (vel && (st = cuda_check(cudaMemcpyAsync(stage + 7 * N, vel, 8 * 3 * N, cudaMemcpyHostToDevice, stream), "upload"))) return st;
    if (omega && (st = cuda_check(cudaMemcpyAsync(stage + 10 * N, omega, 8 * 3 * N, cudaMemcpyHostToDevice, stream), "upload"))) return st;
    mask = (pos ? 1 : 0) | (quat ? 2 : 0) | (vel ? 4 : 0) | (omega ? 8 : 0);
    launch_unpack_state(sc, stage, mask, stream);
    ++launches;
    // the warm-start memory (pair keys, points, impulses) is kept, as the reference's tracker
    // keeps it across user edits of the state; matching is by pair and contact-point distance
    return CDX_OK;
}

int Engine::get_contacts(int32_t* ia, int32_t* ib, double* point, double* lambda, double* normal, int32_t* count) {
    if (!loaded) return fail(CDX_ERR_STATE, "no scene loaded");
    if (cfg.gpu_precision == CDX_PRECISION_SPLIT) return get_contacts_split(ia, ib, point, lambda, normal, count);
    const int n = prev_count;  // contacts of the last completed step
    if (count) *count = n;
    if (n == 0 || (!ia && !ib && !point && !lambda && !normal)) return CDX_OK;
    const int g = gen ^ 1;
    std::vector<unsigned long long> keys(n);
    std::vector<double> p(3 * (size_t)n), l(3 * (size_t)n), nn(3 * (size_t)n);
    int st;
    if ((st = cuda_check(cudaMemcpy(keys.data(), C.key[g], sizeof(unsigned long long) * n, cudaMemcpyDeviceToHost), "download"))) return st;
    for (int k = 0; k < 3; ++k) {
        if ((st = cuda_check(cudaMemcpy(p.data() + (size_t)k * n, C.point[g] + k * C.cap, sizeof(double) * n, cudaMemcpyDeviceToHost), "download"))) return st;
        if ((st = cuda_check(cudaMemcpy(l.data() + (size_t)k * n, C.lam[g] + k * C.cap, sizeof(double) * n, cudaMemcpyDeviceToHost), "download"))) return st;
        // normals belong to a step's contacts: a memory loaded by set_contacts has none yet
        if (!contacts_loaded &&
            (st = cuda_check(cudaMemcpy(nn.data() + (size_t)k * n, C.dir + k * C.cap, sizeof(double) * n, cudaMemcpyDeviceToHost), "download"))) return st;
    }
    for (int c = 0; c < n; ++c) {
        if (ia) ia[c] = (int32_t)(keys[c] >> 32);
        if (ib) ib[c] = (int32_t)(keys[c] & 0xffffffffu);
        for (int k = 0; k < 3; ++k) {
            if (point) point[3 * (size_t)c + k] = p[(size_t)k * n + c];
            if (lambda) lambda[3 * (size_t)c + k] = l[(size_t)k * n + c];
            if (normal) normal[3 * (size_t)c + k] = nn[(size_t)k * n + c];
        }
    }
    return CDX_OK;
}

// Loads the warm-start memory the next step matches against (the reference's ContactTracker keeps
// the last step's contacts with their points and impulses, contact_tracker.cpp:11-72, and
// WarmstartProvider copies the matched impulses in, warmstart.hpp:26-39). Together with
// cdx_get_contacts and the state calls this checkpoints and resumes a simulation, warm start
// included. Pairs are entity ids (statics 0..S-1, sphere i = S + i), each at most once.
int Engine::set_contacts(int32_t n, const int32_t* ia, const int32_t* ib, const double* point,
                         const double* lambda) {
    if (!loaded) return fail(CDX_ERR_STATE, "no scene loaded");
    if (n < 0 || (n > 0 && (!ia || !ib || !point || !lambda))) return fail(CDX_ERR_ARG, "contact arrays missing");
    const int64_t S = sc.S, N = sc.N;
    std::vector<int64_t> order(n);
    std::vector<unsigned long long> key(n);
    for (int32_t c = 0; c < n; ++c) {
        const int64_t a = ia[c], b = ib[c];
        if (a < 0 || b < S || b >= S + N || a >= b)
            return fail(CDX_ERR_ARG, "contact pairs must be (static or sphere id, higher sphere id) in range");
        if (a >= S) {
            if (h_body_scene_of(a - S) != h_body_scene_of(b - S)) return fail(CDX_ERR_ARG, "pair across scenes");
        } else if (h_static_scene_of(a) != h_body_scene_of(b - S)) {
            return fail(CDX_ERR_ARG, "pair across scenes");
        }
        for (int k = 0; k < 3; ++k)
            if (!std::isfinite(point[3 * (size_t)c + k]) || !std::isfinite(lambda[3 * (size_t)c + k]))
                return fail(CDX_ERR_ARG, "contact points and impulses must be finite");
        key[c] = ((unsigned long long)a << 32) | (unsigned long long)b;
        order[c] = c;
    }
    std::sort(order.begin(), order.end(), [&](int64_t x, int64_t y) { return key[x] < key[y]; });
    for (int32_t c = 1; c < n; ++c)
        if (key[order[c]] == key[order[c - 1]]) return fail(CDX_ERR_ARG, "a pair appears twice");
    int st;
    if (stream && (st = cuda_check(cudaStreamSynchronize(stream), "set contacts"))) return st;
    if (cfg.gpu_precision == CDX_PRECISION_SPLIT) return set_contacts_split(order, ia, ib, point, lambda);
    if ((st = ensure_contacts(std::max<int64_t>(n, 1)))) return st;
    const int g = gen ^ 1;
    std::vector<unsigned long long> ks(n);
    std::vector<double> p(3 * (size_t)n), l(3 * (size_t)n);
    for (int32_t c = 0; c < n; ++c) {
        const int64_t o = order[c];
        ks[c] = key[o];
        for (int k = 0; k < 3; ++k) {
            p[(size_t)k * n + c] = point[3 * (size_t)o + k];
            l[(size_t)k * n + c] = lambda[3 * (size_t)o + k];
        }
    }
    if (n > 0) {
        if ((st = cuda_check(cudaMemcpy(C.key[g], ks.data(), sizeof(unsigned long long) * n, cudaMemcpyHostToDevice), "upload"))) return st;
        for (int k = 0; k < 3; ++k) {
            if ((st = cuda_check(cudaMemcpy(C.point[g] + k * C.cap, p.data() + (size_t)k * n, sizeof(double) * n, cudaMemcpyHostToDevice), "upload"))) return st;
            if ((st = cuda_check(cudaMemcpy(C.lam[g] + k * C.cap, l.data() + (size_t)k * n, sizeof(double) * n, cudaMemcpyHostToDevice), "upload"))) return st;
        }
    }
    prev_count = n;
    contacts_loaded = true;
    return CDX_OK;
}

void Engine::fill_stats(cdx_stats* s) {
    std::memset(s, 0, sizeof(*s));
    s->steps = steps;
    s->num_contacts = prev_count;
    s->num_rows = last_rows;
    s->iterations = last_iters;
    s->reallocations = reallocations;
    s->residual = last_res_final;
    s->residual_last = last_res;
    s->ms_collision = ms[0];
    s->ms_setup = ms[1];
    s->ms_solve = ms[2];
    s->ms_integrate = ms[3];
    s->solve_bytes_per_iter = solve_bytes_per_iter();
    s->kernel_launches = launches;
    s->contact_variant = split_variant();
    s->autotune_runs = split_tune_runs();
    s->redone_steps = split_redos();
    s->graph_steps = split_graph_steps();
    s->sweep_variant = split_sweep_variant();
    s->levels = last_levels;
}

double Engine::solve_bytes_per_iter() const {
    // algorithmic bytes of one sweep: per contact the rows' RW coefficients (27 words), the bias (3),
    // mu (1), lambda read+write (6), the directions and lever products read by the W^T gather
    // (9 + 9 per side counted once: 27) and the increments written and read (6), two indices;
    // per body x read+write (12) and 1/M (2)
    if (cfg.gpu_precision == CDX_PRECISION_SPLIT) return split_bytes_per_iter();
    const double w = 8.0;
    return (double)prev_count * ((27 + 3 + 1 + 6 + 27 + 6) * w + 8.0) + (double)sc.N * (14 * w);
}
