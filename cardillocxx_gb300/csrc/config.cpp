// Reference-compatible configuration: the flat key=value format of ConfigReader::fromFile
// (src/config/config.cpp:22-420) for the keys on the contact path, plus gpu.* keys.
// Semantics kept from the reference: '#' starts a comment, unknown keys are ignored, a value that
// does not parse leaves the field unchanged, pj.* keys are also accepted with the solver. prefix,
// booleans are 1/true/yes/on (case-insensitive), a missing file yields the defaults.
#include <algorithm>
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>

#include "../../include/cdx.h"

namespace {

std::string trim(const std::string& s) {
    size_t b = 0, e = s.size();
    while (b < e && std::isspace((unsigned char)s[b])) ++b;
    while (e > b && std::isspace((unsigned char)s[e - 1])) --e;
    return s.substr(b, e - b);
}
std::string lower(std::string s) {
    for (auto& c : s) c = (char)std::tolower((unsigned char)c);
    return s;
}
bool as_bool(const std::string& v) {
    const std::string l = lower(v);
    return l == "1" || l == "true" || l == "yes" || l == "on";
}
// std::stod / std::stoi semantics: parse a leading number, reject when nothing parses
bool as_double(const std::string& v, double* out) {
    const char* s = v.c_str();
    char* end = nullptr;
    const double d = std::strtod(s, &end);
    if (end == s) return false;
    *out = d;
    return true;
}
bool as_int(const std::string& v, int* out) {
    const char* s = v.c_str();
    char* end = nullptr;
    const long l = std::strtol(s, &end, 10);
    if (end == s) return false;
    *out = (int)l;
    return true;
}
bool key_is(const std::string& k, const char* pj) {
    // "pj.X" also accepted as "solver.X" (config.cpp:41-110)
    if (k == pj) return true;
    if (std::strncmp(pj, "pj.", 3) == 0) return k == std::string("solver.") + (pj + 3);
    return false;
}

}  // namespace

extern "C" {

int cdx_config_default(cdx_config* c) {
    if (!c) return CDX_ERR_ARG;
    std::memset(c, 0, sizeof(*c));
    // reference defaults (src/config/config.hpp:12-237)
    c->sim_T = 5.0;
    c->sim_dt = 1e-3;
    c->sim_gravity[0] = 0.0;
    c->sim_gravity[1] = 0.0;
    c->sim_gravity[2] = -9.81;
    c->moreau_theta = 1.0;
    c->moreau_implicit_gyroscopy = 0;
    c->friction_enable = 0;
    c->friction_combine = 0;
    c->friction_default_mu = 0.3;
    c->restitution_default_normal = 0.0;
    c->restitution_default_tangential = 0.0;
    c->pj_max_iterations = 200000;
    c->pj_warmstart = 1;
    c->pj_tol_abs = 1e-5;
    c->pj_tol_rel = 1e-5;
    c->pj_alpha = 0.3;
    c->pj_relaxation = 1.0;
    c->solver_type = 0;
    c->condensed_sweep_mode = 0;  // condensed.sweep_mode = gauss_seidel (config.hpp:118)
    c->gpu_tune_alpha = 0;
    c->gpu_tune_alpha_every = 500;
    c->collision_security_margin = 0.0;
    c->collision_match_max_dist = 0.02;
    c->collision_broadphase = 0;
    // gpu.* (new)
    c->gpu_precision = CDX_PRECISION_FP64;
    c->gpu_residual_tol = 0.0;
    c->gpu_check_every = 10;
    c->gpu_block = 0;
    c->gpu_contact_capacity_factor = 8.0;
    c->gpu_use_graph = 1;
    c->gpu_autotune = 1;
    c->gpu_sweep_variant = -1;
    c->gpu_sync_counts = 0;
    c->pj_nesterov = 0;
    c->pj_nesterov_beta_threshold = 1.0;
    c->pj_nesterov_restart_limit = 10000;
    c->pj_chebyshev = 0;
    c->pj_anderson = 0;
    c->pj_anderson_m = 2;
    c->pj_rdiag_true_delassus = 0;
    // frames are off unless asked for (the reference writes every 50 steps by default)
    c->output_interval_steps = 0;
    c->output_write_contact_manifolds = 1;
    c->gpu_coop_smem_contacts = 0;
    c->gpu_coop_blocks = 0;
    std::snprintf(c->output_folder, sizeof(c->output_folder), "%s", "./vtk_out");
    std::snprintf(c->output_filename_prefix, sizeof(c->output_filename_prefix), "%s", "scene");
    return CDX_OK;
}

int cdx_config_set(cdx_config* c, const char* key_c, const char* val_c) {
    if (!c || !key_c || !val_c) return CDX_ERR_ARG;
    const std::string key = trim(key_c), val = trim(val_c);
    double d;
    int i;
    if (key_is(key, "pj.max_iterations")) {
        if (as_int(val, &i)) c->pj_max_iterations = std::max(1, i);
    } else if (key_is(key, "pj.tol_abs")) {
        if (as_double(val, &d)) c->pj_tol_abs = d;
    } else if (key_is(key, "pj.tol_rel")) {
        if (as_double(val, &d)) c->pj_tol_rel = d;
    } else if (key_is(key, "pj.relaxation")) {
        if (as_double(val, &d)) c->pj_relaxation = d;
    } else if (key_is(key, "pj.alpha")) {
        if (as_double(val, &d)) c->pj_alpha = d;
    } else if (key_is(key, "pj.warmstart")) {
        c->pj_warmstart = as_bool(val);
    } else if (key == "solver.type") {
        const std::string v = lower(val);
        if (v == "projected_jacobi" || v == "projectedjacobi" || v == "pj" || v == "gpu_pj") c->solver_type = 0;
        else if (v == "condensed" || v == "condensed_solver") c->solver_type = 1;
        else if (v == "projected_gauss_seidel" || v == "projectedgaussseidel" || v == "pgs") c->solver_type = 2;
        else return CDX_ERR_UNSUPPORTED;  // other solvers are not on this path
    } else if (key == "condensed.sweep_mode") {
        const std::string v = lower(val);
        if (v == "gauss_seidel") c->condensed_sweep_mode = 0;
        else if (v == "jacobi") c->condensed_sweep_mode = 1;
        else if (v == "colored") c->condensed_sweep_mode = 2;
        else if (v == "chaotic") c->condensed_sweep_mode = 3;
    } else if (key == "moreau.theta" || key == "solver.theta") {
        if (as_double(val, &d)) c->moreau_theta = d;
    } else if (key == "moreau.implicit_gyroscopy" || key == "solver.implicit_gyroscopy") {
        c->moreau_implicit_gyroscopy = as_bool(val);
    } else if (key == "sim.T") {
        if (as_double(val, &d) && d > 0) c->sim_T = d;
    } else if (key == "sim.dt") {
        if (as_double(val, &d) && d > 0) c->sim_dt = d;
    } else if (key == "sim.gravity") {
        std::string v = val;
        std::replace(v.begin(), v.end(), ',', ' ');
        std::istringstream ss(v);
        double gx = 0, gy = 0, gz = -9.81;
        if (ss >> gx >> gy >> gz) {
            c->sim_gravity[0] = gx;
            c->sim_gravity[1] = gy;
            c->sim_gravity[2] = gz;
        }
    } else if (key == "collision.broadphase") {
        c->collision_broadphase = 0;  // every reference broad phase maps to the uniform grid
    } else if (key == "collision.match_max_dist") {
        if (as_double(val, &d)) c->collision_match_max_dist = d < 0 ? 0 : d;
    } else if (key == "collision.security_margin") {
        if (as_double(val, &d)) c->collision_security_margin = d;
    } else if (key == "friction.enable") {
        c->friction_enable = as_bool(val);
    } else if (key == "friction.combine") {
        const std::string v = lower(val);
        if (v == "min") c->friction_combine = 0;
        else if (v == "arith") c->friction_combine = 1;
        else if (v == "geom") c->friction_combine = 2;
    } else if (key == "friction.default_mu") {
        if (as_double(val, &d)) c->friction_default_mu = d;
    } else if (key == "restitution.default_normal") {
        if (as_double(val, &d)) c->restitution_default_normal = d;
    } else if (key == "restitution.default_tangential") {
        if (as_double(val, &d)) c->restitution_default_tangential = d;
    } else if (key == "gpu.precision") {
        const std::string v = lower(val);
        if (v == "fp64" || v == "plain") c->gpu_precision = CDX_PRECISION_FP64;
        else if (v == "split" || v == "fp32") c->gpu_precision = CDX_PRECISION_SPLIT;
    } else if (key == "gpu.residual_tol") {
        if (as_double(val, &d)) c->gpu_residual_tol = d < 0 ? 0 : d;
    } else if (key == "gpu.check_every") {
        if (as_int(val, &i)) c->gpu_check_every = std::max(1, i);
    } else if (key == "gpu.block") {
        if (as_int(val, &i)) c->gpu_block = std::max(0, i);
    } else if (key == "gpu.contact_capacity") {
        if (as_double(val, &d) && d > 0) c->gpu_contact_capacity_factor = d;
    } else if (key == "gpu.graph") {
        c->gpu_use_graph = as_bool(val);
    } else if (key == "gpu.autotune") {
        c->gpu_autotune = as_bool(val);
    } else if (key == "gpu.sweep_variant") {
        if (as_int(val, &i)) c->gpu_sweep_variant = std::max(-1, i);
    } else if (key == "gpu.coop_smem_contacts") {
        if (as_int(val, &i)) c->gpu_coop_smem_contacts = std::max(0, i);
    } else if (key == "gpu.coop_blocks") {
        if (as_int(val, &i)) c->gpu_coop_blocks = std::max(0, i);
    } else if (key == "gpu.coop_wait_ns") {
        if (as_double(val, &d) && d >= 0 && d < 9e18) c->gpu_coop_wait_ns = (int64_t)d;
    } else if (key == "gpu.tune_alpha") {
        c->gpu_tune_alpha = as_bool(val);
    } else if (key == "gpu.tune_alpha_every") {
        if (as_int(val, &i) && i >= 1) c->gpu_tune_alpha_every = i;
    } else if (key == "gpu.sync_counts") {
        c->gpu_sync_counts = as_bool(val);
    } else if (key_is(key, "pj.nesterov")) {
        c->pj_nesterov = as_bool(val);
    } else if (key_is(key, "pj.nesterov_beta_threshold")) {
        if (as_double(val, &d)) c->pj_nesterov_beta_threshold = d;
    } else if (key_is(key, "pj.nesterov_restart_limit")) {
        if (as_int(val, &i)) c->pj_nesterov_restart_limit = std::max(0, i);
    } else if (key_is(key, "pj.chebyshev")) {
        c->pj_chebyshev = as_bool(val);
    } else if (key_is(key, "pj.anderson")) {
        c->pj_anderson = as_bool(val);
    } else if (key_is(key, "pj.anderson_m")) {
        if (as_int(val, &i)) c->pj_anderson_m = std::max(1, i);
    } else if (key_is(key, "pj.rdiag_true_delassus")) {
        c->pj_rdiag_true_delassus = as_bool(val);
    } else if (key == "output.interval_steps") {
        if (as_int(val, &i)) c->output_interval_steps = std::max(0, i);
    } else if (key == "output.write_contact_manifolds") {
        c->output_write_contact_manifolds = as_bool(val);
    } else if (key == "output.folder") {
        if (val.size() >= sizeof(c->output_folder)) return CDX_ERR_ARG;
        std::snprintf(c->output_folder, sizeof(c->output_folder), "%s", val.c_str());
    } else if (key == "output.filename_prefix") {
        if (val.size() >= sizeof(c->output_filename_prefix)) return CDX_ERR_ARG;
        std::snprintf(c->output_filename_prefix, sizeof(c->output_filename_prefix), "%s", val.c_str());
    }
    return CDX_OK;  // unknown keys are ignored, as in the reference
}

int cdx_config_from_file(const char* path, cdx_config* c) {
    if (!c) return CDX_ERR_ARG;
    cdx_config_default(c);
    if (!path) return CDX_OK;
    std::ifstream f(path);
    if (!f) return CDX_OK;  // defaults when the file cannot be opened
    std::string line;
    while (std::getline(f, line)) {
        std::string s = trim(line);
        if (s.empty()) continue;
        const auto hash = s.find('#');
        if (hash != std::string::npos) s = trim(s.substr(0, hash));
        if (s.empty()) continue;
        const auto eq = s.find('=');
        if (eq == std::string::npos) continue;
        const int rc = cdx_config_set(c, trim(s.substr(0, eq)).c_str(), trim(s.substr(eq + 1)).c_str());
        if (rc == CDX_ERR_UNSUPPORTED) return rc;
    }
    return CDX_OK;
}

}  // extern "C"
