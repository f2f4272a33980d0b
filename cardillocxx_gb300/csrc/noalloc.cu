// cdx_pj_solve_csr_noalloc: the solver-level projected Jacobi solve for callers that cannot
// allocate device memory.
//
// Some hosts of this solver own every byte of GPU memory themselves: applications that reserve
// the device up front through their own pool, real-time loops where a cudaMalloc/cudaFree stall
// is not acceptable, and code running where allocation calls are not allowed at all. This entry
// point runs the same kernels as cdx_pj_solve_csr but keeps its work buffers, the staged inputs
// and the results in one file-scope device array of fixed size (CDX_NOALLOC_SCRATCH_BYTES), so
// it calls no cudaMalloc, cudaFree or allocating library routine. Every GPU that loads the
// library holds that array until the process exits.
//
// Setup: the first call on a device, with that device current, looks up the array's device
// address with cudaGetSymbolAddress (host code cannot use the symbol itself as a device pointer)
// and keeps it for that device. Make that first call before any stream capture. cudaDeviceReset
// discards the array with the context, and the kept address then no longer holds: do not reset a
// device between calls. A call returns once its work on the stream has finished (it waits on the
// stream). All calls share the one array and it keeps the last call's contents; everything that
// must start at zero is cleared by each call. Calls that overlap on the GPU (different streams
// or host threads at the same time) race on the array.
#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/cdx.h"
#include "cdx_internal.h"

namespace {

static __device__ __align__(256) unsigned char g_noalloc_scratch[CDX_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
void* g_scratch_ptr[kMaxDevices] = {nullptr};
std::mutex g_setup_mutex;

int fail(char* err, int32_t errlen, int st, const char* msg) {
    if (err && errlen > 0) {
        std::strncpy(err, msg, (size_t)errlen - 1);
        err[errlen - 1] = '\0';
    }
    return st;
}

// device address of the scratch array on the current device (looked up once per device)
int scratch_base(void** out, char* err, int32_t errlen) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return fail(err, errlen, CDX_ERR_CUDA, "cdx_pj_solve_csr_noalloc: no current CUDA device");
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            char m[256];
            std::snprintf(m, sizeof(m), "cdx_pj_solve_csr_noalloc: cudaGetSymbolAddress failed: %s",
                          cudaGetErrorString(e));
            return fail(err, errlen, CDX_ERR_CUDA, m);
        }
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return CDX_OK;
}

// bump allocator over the scratch array (256-byte aligned slices)
struct Carve {
    unsigned char* base;
    size_t used = 0;
    size_t cap;
    bool ok = true;
    template <typename T>
    T* take(size_t count) {
        const size_t bytes = ((sizeof(T) * (count ? count : 1)) + 255) & ~(size_t)255;
        if (used + bytes > cap) {
            ok = false;
            return nullptr;
        }
        T* p = reinterpret_cast<T*>(base + used);
        used += bytes;
        return p;
    }
};

}  // namespace

extern "C" int cdx_pj_solve_csr_noalloc(void* stream_ptr, int32_t nrows, int32_t nv, int32_t nfl, const int32_t* row_ptr,
                                        const int32_t* col, const double* val, const double* contact_bias,
                                        const double* mu, const double* restitution, const double* minv,
                                        const double* mdiag, const double* v, const double* f_ext,
                                        const double* f_gyro, double dt, double alpha, int32_t max_iter,
                                        double tol_abs, double tol_rel, double* lambda_inout, double* x_out,
                                        int32_t* iterations, char* err, int32_t errlen) {
    using namespace cdx;
    cudaStream_t s = (cudaStream_t)stream_ptr;
    if (nrows < 0 || nv < 0 || nfl < 0 || nfl > nrows || (nrows - nfl) % 3 != 0)
        return fail(err, errlen, CDX_ERR_ARG, "cdx_pj_solve_csr_noalloc: rows must be nfl frictionless rows then 3-row blocks");
    if (!row_ptr || (nrows > 0 && (!col || !val || !contact_bias || !mu || !restitution || !lambda_inout)) ||
        (nv > 0 && (!minv || !mdiag || !v || !f_ext || !f_gyro || !x_out)))
        return fail(err, errlen, CDX_ERR_ARG, "cdx_pj_solve_csr_noalloc: missing array");
    const int64_t nnz = row_ptr[nrows];
    if (nnz < 0 || row_ptr[0] != 0) return fail(err, errlen, CDX_ERR_ARG, "cdx_pj_solve_csr_noalloc: bad row_ptr");
    for (int r = 0; r < nrows; ++r)
        if (row_ptr[r + 1] < row_ptr[r])
            return fail(err, errlen, CDX_ERR_ARG, "cdx_pj_solve_csr_noalloc: row_ptr must be nondecreasing");
    for (int64_t k = 0; k < nnz; ++k)
        if (col[k] < 0 || col[k] >= nv)
            return fail(err, errlen, CDX_ERR_ARG, "cdx_pj_solve_csr_noalloc: column index out of range");

    void* base = nullptr;
    int st = scratch_base(&base, err, errlen);
    if (st) return st;
    // lay out every device buffer inside the scratch array; reject what does not fit
    Carve cv{(unsigned char*)base, 0, (size_t)CDX_NOALLOC_SCRATCH_BYTES};
    int32_t* d_ptr = cv.take<int32_t>(nrows + 1);
    int32_t* d_col = cv.take<int32_t>(nnz);
    int32_t* d_rowidx = cv.take<int32_t>(nnz);
    uint32_t* ck_in = cv.take<uint32_t>(nnz);
    uint32_t* ck_out = cv.take<uint32_t>(nnz);
    uint32_t* nz_in = cv.take<uint32_t>(nnz);
    uint32_t* nz_out = cv.take<uint32_t>(nnz);
    double* d_val = cv.take<double>(nnz);
    double* d_RW = cv.take<double>(nnz);
    double* d_cb = cv.take<double>(nrows);
    double* d_mu = cv.take<double>(nrows);
    double* d_e = cv.take<double>(nrows);
    double* d_biasR = cv.take<double>(nrows);
    double* d_lam = cv.take<double>(nrows);
    double* d_dlam = cv.take<double>(nrows);
    int32_t* d_cstart = cv.take<int32_t>(nv);
    int32_t* d_cend = cv.take<int32_t>(nv);
    double* d_minv = cv.take<double>(nv);
    double* d_mdiag = cv.take<double>(nv);
    double* d_v = cv.take<double>(nv);
    double* d_fext = cv.take<double>(nv);
    double* d_fgyro = cv.take<double>(nv);
    double* d_rhs = cv.take<double>(nv);
    double* d_x = cv.take<double>(nv);
    DevScalars* d_ds = cv.take<DevScalars>(1);
    const size_t sort_bytes = sort_temp_bytes(nnz > 0 ? nnz : 1) + 256;
    void* d_tmp = cv.take<unsigned char>(sort_bytes);
    if (!cv.ok) {
        char m[256];
        std::snprintf(m, sizeof(m),
                      "cdx_pj_solve_csr_noalloc: problem needs more than the %lld-byte scratch array "
                      "(nrows %d, nv %d, nnz %lld); use cdx_pj_solve_csr",
                      (long long)CDX_NOALLOC_SCRATCH_BYTES, nrows, nv, (long long)nnz);
        return fail(err, errlen, CDX_ERR_OVERFLOW, m);
    }

    auto up = [&](void* d, const void* h, size_t bytes) {
        return bytes ? cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, s) : cudaSuccess;
    };
    cudaError_t ce = cudaSuccess;
    ce = ce ? ce : up(d_ptr, row_ptr, 4 * (size_t)(nrows + 1));
    ce = ce ? ce : up(d_col, col, 4 * (size_t)nnz);
    ce = ce ? ce : up(d_val, val, 8 * (size_t)nnz);
    ce = ce ? ce : up(d_cb, contact_bias, 8 * (size_t)nrows);
    ce = ce ? ce : up(d_mu, mu, 8 * (size_t)nrows);
    ce = ce ? ce : up(d_e, restitution, 8 * (size_t)nrows);
    ce = ce ? ce : up(d_lam, lambda_inout, 8 * (size_t)nrows);
    ce = ce ? ce : up(d_minv, minv, 8 * (size_t)nv);
    ce = ce ? ce : up(d_mdiag, mdiag, 8 * (size_t)nv);
    ce = ce ? ce : up(d_v, v, 8 * (size_t)nv);
    ce = ce ? ce : up(d_fext, f_ext, 8 * (size_t)nv);
    ce = ce ? ce : up(d_fgyro, f_gyro, 8 * (size_t)nv);
    // the array keeps the previous call's contents: clear the stop flags and the column ranges
    ce = ce ? ce : cudaMemsetAsync(d_ds, 0, sizeof(DevScalars), s);
    ce = ce ? ce : (nv ? cudaMemsetAsync(d_cstart, 0, 4 * (size_t)nv, s) : cudaSuccess);
    ce = ce ? ce : (nv ? cudaMemsetAsync(d_cend, 0, 4 * (size_t)nv, s) : cudaSuccess);
    if (ce != cudaSuccess) return fail(err, errlen, CDX_ERR_CUDA, cudaGetErrorString(ce));

    launch_csr_rhs(nv, d_mdiag, d_v, d_fext, d_fgyro, dt, d_rhs, s);
    int32_t iters = 0;
    if (nrows == 0) {
        launch_csr_cols(nv, d_cstart, d_cend, nz_out, d_rowidx, d_val, d_lam, d_rhs, d_mdiag, d_x, 0, 0, 0, 0, d_ds, s);
    } else {
        launch_csr_rowidx(nrows, d_ptr, d_rowidx, ck_in, nz_in, d_col, s);
        int bits = 1;
        while (((int64_t)1 << bits) <= nv) ++bits;
        ce = sort_pairs(d_tmp, sort_bytes, ck_in, ck_out, nz_in, nz_out, nnz, bits, s);
        if (ce != cudaSuccess) return fail(err, errlen, CDX_ERR_CUDA, cudaGetErrorString(ce));
        launch_ranges(ck_out, nnz, d_cstart, d_cend, s);
        launch_csr_setup(nrows, d_ptr, d_col, d_val, d_cb, d_e, d_minv, d_v, alpha, d_RW, d_biasR, s);
        launch_csr_cols(nv, d_cstart, d_cend, nz_out, d_rowidx, d_val, d_lam, d_rhs, d_mdiag, d_x, 0, 0, 0, 0, d_ds, s);
        const bool check_vel = !(tol_abs == 0.0 && tol_rel == 0.0);
        const int maxit = max_iter > 1 ? max_iter : 1;
        int32_t done = 0;
        for (int it = 0; it < maxit; ++it) {
            launch_csr_rows(nrows, nfl, d_ptr, d_col, d_RW, d_biasR, d_mu, d_x, d_lam, d_dlam, d_ds, s);
            launch_csr_cols(nv, d_cstart, d_cend, nz_out, d_rowidx, d_val, d_dlam, nullptr, d_mdiag, d_x, 1, tol_abs,
                            tol_rel, check_vel && (it % 10 == 0), d_ds, s);
            launch_check(d_ds, it, 0.0, nv, check_vel, s);
            if ((it + 1) % 10 == 0 && it + 1 < maxit) {
                cudaMemcpyAsync(&done, &d_ds->done, 4, cudaMemcpyDeviceToHost, s);
                if ((ce = cudaStreamSynchronize(s)) != cudaSuccess)
                    return fail(err, errlen, CDX_ERR_CUDA, cudaGetErrorString(ce));
                if (done) break;
            }
        }
        cudaMemcpyAsync(&iters, &d_ds->iters, 4, cudaMemcpyDeviceToHost, s);
    }
    if (nv) cudaMemcpyAsync(x_out, d_x, 8 * (size_t)nv, cudaMemcpyDeviceToHost, s);
    if (nrows) cudaMemcpyAsync(lambda_inout, d_lam, 8 * (size_t)nrows, cudaMemcpyDeviceToHost, s);
    if ((ce = cudaStreamSynchronize(s)) != cudaSuccess) return fail(err, errlen, CDX_ERR_CUDA, cudaGetErrorString(ce));
    if ((ce = cudaGetLastError()) != cudaSuccess) return fail(err, errlen, CDX_ERR_CUDA, cudaGetErrorString(ce));
    if (iterations) *iterations = iters;
    if (err && errlen > 0) err[0] = '\0';
    return CDX_OK;
}
