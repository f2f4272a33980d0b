// C-ABI entry points (include/cdx.h). Every function validates its arguments and converts C++
// failures into status codes; no exception crosses the boundary.
#include <cstring>
#include <new>

#include "../../include/cdx.h"
#include "engine.h"
#include "split.h"

extern "C" {

int cdx_create(const cdx_config* cfg, cdx_ctx** out) {
    if (!out) return CDX_ERR_ARG;
    *out = nullptr;
    cdx_config c;
    if (cfg) c = *cfg;
    else cdx_config_default(&c);
    cdx_ctx* ctx = new (std::nothrow) cdx_ctx();
    if (!ctx) return CDX_ERR_ARG;
    const int st = ctx->eng.init(c);
    *out = ctx;  // returned even on failure so cdx_last_error can report; caller destroys
    return st;
}

void cdx_destroy(cdx_ctx* ctx) { delete ctx; }

int cdx_set_config(cdx_ctx* ctx, const cdx_config* cfg) {
    if (!ctx || !cfg) return CDX_ERR_ARG;
    return ctx->eng.set_config(*cfg);
}

const char* cdx_last_error(const cdx_ctx* ctx) { return ctx ? ctx->eng.err.c_str() : "null context"; }

int cdx_load_scene(cdx_ctx* ctx, const cdx_scene* scene) {
    if (!ctx || !scene) return CDX_ERR_ARG;
    try {
        return ctx->eng.load_scene(*scene);
    } catch (const std::exception& e) {
        return ctx->eng.fail(CDX_ERR_ARG, e.what());
    }
}

int cdx_step(cdx_ctx* ctx, int32_t nsteps) {
    if (!ctx || nsteps < 0) return CDX_ERR_ARG;
    try {
        return ctx->eng.step(nsteps);
    } catch (const std::exception& e) {
        return ctx->eng.fail(CDX_ERR_ARG, e.what());
    }
}

int cdx_synchronize(cdx_ctx* ctx) {
    if (!ctx) return CDX_ERR_ARG;
    return ctx->eng.cuda_check(cudaStreamSynchronize(ctx->eng.stream), "synchronize");
}

int cdx_get_state(cdx_ctx* ctx, double* pos, double* quat, double* vel, double* omega) {
    if (!ctx) return CDX_ERR_ARG;
    return ctx->eng.get_state(pos, quat, vel, omega);
}

int cdx_set_state(cdx_ctx* ctx, const double* pos, const double* quat, const double* vel, const double* omega) {
    if (!ctx) return CDX_ERR_ARG;
    return ctx->eng.set_state(pos, quat, vel, omega);
}

int cdx_get_stats(cdx_ctx* ctx, cdx_stats* out) {
    if (!ctx || !out) return CDX_ERR_ARG;
    ctx->eng.fill_stats(out);
    return CDX_OK;
}

int cdx_get_contacts(cdx_ctx* ctx, int32_t* id_a, int32_t* id_b, double* point, double* lambda, double* normal,
                     int32_t* count) {
    if (!ctx) return CDX_ERR_ARG;
    return ctx->eng.get_contacts(id_a, id_b, point, lambda, normal, count);
}

int cdx_set_contacts(cdx_ctx* ctx, int32_t count, const int32_t* id_a, const int32_t* id_b, const double* point,
                     const double* lambda) {
    if (!ctx) return CDX_ERR_ARG;
    try {
        return ctx->eng.set_contacts(count, id_a, id_b, point, lambda);
    } catch (const std::exception& e) {
        return ctx->eng.fail(CDX_ERR_ARG, e.what());
    }
}

int cdx_set_static_motion(cdx_ctx* ctx, int32_t count, const int32_t* statics, const double* pos,
                          const double* quat, const double* vel, const double* omega) {
    if (!ctx) return CDX_ERR_ARG;
    try {
        return ctx->eng.set_static_motion(count, statics, pos, quat, vel, omega);
    } catch (const std::exception& e) {
        return ctx->eng.fail(CDX_ERR_ARG, e.what());
    }
}

int cdx_get_static_state(cdx_ctx* ctx, double* pos, double* quat, double* vel, double* omega) {
    if (!ctx) return CDX_ERR_ARG;
    return ctx->eng.get_static_state(pos, quat, vel, omega);
}

int cdx_get_scene_solve(cdx_ctx* ctx, float* alpha, int32_t* sweeps, int32_t n) {
    if (!ctx || n < 0) return CDX_ERR_ARG;
    return ctx->eng.scene_solve_info(alpha, sweeps, n);
}

int cdx_track(cdx_ctx* ctx, int32_t body, const char* name) {
    if (!ctx) return CDX_ERR_ARG;
    try {
        return ctx->eng.track(body, name);
    } catch (const std::exception& e) {
        return ctx->eng.fail(CDX_ERR_ARG, e.what());
    }
}

int cdx_output_flush(cdx_ctx* ctx) {
    if (!ctx) return CDX_ERR_ARG;
    return ctx->eng.output_flush();
}

int cdx_set_trace(cdx_ctx* ctx, int32_t on) {
    if (!ctx) return CDX_ERR_ARG;
    ctx->eng.trace_next = on != 0;
    return CDX_OK;
}

int cdx_get_trace(cdx_ctx* ctx, double* out, int64_t max_values, int64_t* num_values) {
    if (!ctx) return CDX_ERR_ARG;
    const auto& t = ctx->eng.trace_buf;
    if (num_values) *num_values = (int64_t)t.size();
    if (out) {
        const int64_t n = max_values < (int64_t)t.size() ? max_values : (int64_t)t.size();
        std::memcpy(out, t.data(), sizeof(double) * (size_t)(n > 0 ? n : 0));
    }
    return CDX_OK;
}

int cdx_set_timing(cdx_ctx* ctx, int32_t on) {
    if (!ctx) return CDX_ERR_ARG;
    ctx->eng.timing = on != 0;
    return CDX_OK;
}

void* cdx_stream(cdx_ctx* ctx) { return ctx ? (void*)ctx->eng.stream : nullptr; }

int cdx_time_sweeps(cdx_ctx* ctx, int32_t n, double* ms_contact, double* ms_body, double* bytes_contact,
                    double* bytes_body) {
    if (!ctx) return CDX_ERR_ARG;
    return ctx->eng.time_sweeps(n, ms_contact, ms_body, bytes_contact, bytes_body);
}

int32_t cdx_split_variant_count(void) { return cdx::split_num_variants(); }
const char* cdx_split_variant_name(int32_t k) { return cdx::split_variant_name(k); }

}  // extern "C"
