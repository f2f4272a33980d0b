// Seeded scene generators for the benchmark scenes (host only).
//
// Spheres are placed by grid-accelerated random sequential addition (radii drawn first and placed
// largest first), then ordered inside each scene by the Morton code of their cell so that body
// index order is spatially coherent on the device. Mass and inertia follow the reference's sphere
// formulas: volume (4/3) pi r^3 times density, inertia (2/5) r^2 m
// (src/physics/assets/rigid_body_factory.cpp:35-108). Static walls are halfspaces, the drum is a
// hollow cylinder. The RNG is xoshiro256** seeded through SplitMix64 (Blackman and Vigna).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/cdx.h"

namespace {

struct Rng {
    uint64_t s[4];
    explicit Rng(uint64_t seed) {
        uint64_t x = seed;
        for (auto& v : s) {
            uint64_t z = (x += 0x9e3779b97f4a7c15ULL);
            z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
            z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
            v = z ^ (z >> 31);
        }
    }
    static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    uint64_t next() {
        const uint64_t r = rotl(s[1] * 5, 7) * 9;
        const uint64_t t = s[1] << 17;
        s[2] ^= s[0];
        s[3] ^= s[1];
        s[1] ^= s[2];
        s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl(s[3], 45);
        return r;
    }
    double u01() { return (double)(next() >> 11) * 0x1.0p-53; }
    double uni(double a, double b) { return a + (b - a) * u01(); }
    double normal() {  // Box-Muller, one value per call
        double u1 = u01();
        while (u1 <= 0.0) u1 = u01();
        const double u2 = u01();
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
    }
};

uint64_t spread3(uint64_t v) {
    v &= 0x1fffff;
    v = (v | v << 32) & 0x1f00000000ffffULL;
    v = (v | v << 16) & 0x1f0000ff0000ffULL;
    v = (v | v << 8) & 0x100f00f00f00f00fULL;
    v = (v | v << 4) & 0x10c30c30c30c30c3ULL;
    v = (v | v << 2) & 0x1249249249249249ULL;
    return v;
}

struct Placer {
    double lo[3], cell;
    int64_t dim[3];
    std::vector<std::vector<int>> cells;
    const std::vector<double>* pos;
    const std::vector<double>* rad;
    Placer(const double* l, const double* h, double c, const std::vector<double>* p, const std::vector<double>* r)
        : cell(c), pos(p), rad(r) {
        for (int k = 0; k < 3; ++k) {
            lo[k] = l[k];
            dim[k] = std::max<int64_t>(1, (int64_t)std::ceil((h[k] - l[k]) / c) + 1);
        }
        cells.resize((size_t)(dim[0] * dim[1] * dim[2]));
    }
    void cell_of(const double* p, int64_t* ci) const {
        for (int k = 0; k < 3; ++k) ci[k] = std::min(dim[k] - 1, std::max<int64_t>(0, (int64_t)std::floor((p[k] - lo[k]) / cell)));
    }
    bool free_at(const double* p, double r) const {
        int64_t ci[3];
        cell_of(p, ci);
        for (int64_t z = std::max<int64_t>(0, ci[2] - 1); z <= std::min(dim[2] - 1, ci[2] + 1); ++z)
            for (int64_t y = std::max<int64_t>(0, ci[1] - 1); y <= std::min(dim[1] - 1, ci[1] + 1); ++y)
                for (int64_t x = std::max<int64_t>(0, ci[0] - 1); x <= std::min(dim[0] - 1, ci[0] + 1); ++x)
                    for (int j : cells[(size_t)((z * dim[1] + y) * dim[0] + x)]) {
                        const double* q = &(*pos)[3 * (size_t)j];
                        const double dx = p[0] - q[0], dy = p[1] - q[1], dz = p[2] - q[2];
                        const double s = r + (*rad)[j] + 1e-6;
                        if (dx * dx + dy * dy + dz * dz < s * s) return false;
                    }
        return true;
    }
    void add(int j) {
        int64_t ci[3];
        cell_of(&(*pos)[3 * (size_t)j], ci);
        cells[(size_t)((ci[2] * dim[1] + ci[1]) * dim[0] + ci[0])].push_back(j);
    }
};

}  // namespace

struct cdx_gen_scene {
    std::vector<double> pos, quat, vel, omega, radius, mass, inertia, mu, rest_n, rest_t;
    std::vector<int32_t> body_scene;
    std::vector<int32_t> static_kind, static_scene;
    std::vector<double> static_pos, static_quat, static_vel, static_omega, static_dir, static_radius, static_mu,
        static_rest_n, static_rest_t;
    int32_t num_scenes = 0;
    std::string err;
};

namespace {

void add_static(cdx_gen_scene& g, int kind, const double* p, const double* dir, double radius, const double* omega,
                double mu, int scene) {
    g.static_kind.push_back(kind);
    g.static_scene.push_back(scene);
    for (int k = 0; k < 3; ++k) {
        g.static_pos.push_back(p[k]);
        g.static_dir.push_back(dir[k]);
        g.static_vel.push_back(0.0);
        g.static_omega.push_back(omega ? omega[k] : 0.0);
    }
    const double q[4] = {0, 0, 0, 1};
    for (double v : q) g.static_quat.push_back(v);
    g.static_radius.push_back(radius);
    g.static_mu.push_back(mu);
    g.static_rest_n.push_back(0.0);
    g.static_rest_t.push_back(0.0);
}

// Place n spheres with radii rr inside the region tested by `inside`, return false on failure.
template <class Inside>
bool place(Rng& rng, std::vector<double>& rr, const double* lo, const double* hi, Inside inside, int max_attempts,
           std::vector<double>& pos) {
    const int n = (int)rr.size();
    std::sort(rr.begin(), rr.end(), [](double a, double b) { return a > b; });
    pos.assign(3 * (size_t)n, 0.0);
    double rmax = 0;
    for (double r : rr) rmax = std::max(rmax, r);
    Placer P(lo, hi, 2.0 * rmax + 2e-6, &pos, &rr);
    for (int i = 0; i < n; ++i) {
        const double r = rr[i];
        bool ok = false;
        for (int a = 0; a < max_attempts && !ok; ++a) {
            double p[3];
            for (int k = 0; k < 3; ++k) p[k] = rng.uni(lo[k] + r, hi[k] - r);
            if (!inside(p, r)) continue;
            if (!P.free_at(p, r)) continue;
            for (int k = 0; k < 3; ++k) pos[3 * (size_t)i + k] = p[k];
            P.add(i);
            ok = true;
        }
        if (!ok) return false;
    }
    // spatially coherent order: Morton code of the placement cell, ties by placement index
    std::vector<std::pair<uint64_t, int>> key(n);
    for (int i = 0; i < n; ++i) {
        int64_t ci[3];
        P.cell_of(&pos[3 * (size_t)i], ci);
        key[i] = {spread3((uint64_t)ci[0]) | (spread3((uint64_t)ci[1]) << 1) | (spread3((uint64_t)ci[2]) << 2), i};
    }
    std::sort(key.begin(), key.end());
    std::vector<double> p2(pos.size()), r2(rr.size());
    for (int i = 0; i < n; ++i) {
        const int j = key[i].second;
        for (int k = 0; k < 3; ++k) p2[3 * (size_t)i + k] = pos[3 * (size_t)j + k];
        r2[i] = rr[j];
    }
    pos.swap(p2);
    rr.swap(r2);
    return true;
}

void add_bodies(cdx_gen_scene& g, Rng& rng, const std::vector<double>& pos, const std::vector<double>& rr,
                double density, double mu, double v_sigma, int scene) {
    const int n = (int)rr.size();
    for (int i = 0; i < n; ++i) {
        const double r = rr[i];
        for (int k = 0; k < 3; ++k) g.pos.push_back(pos[3 * (size_t)i + k]);
        const double q[4] = {0, 0, 0, 1};
        for (double v : q) g.quat.push_back(v);
        for (int k = 0; k < 3; ++k) g.vel.push_back(v_sigma > 0 ? v_sigma * rng.normal() : 0.0);
        for (int k = 0; k < 3; ++k) g.omega.push_back(0.0);
        g.radius.push_back(r);
        const double volume = (4.0 / 3.0) * M_PI * r * r * r;
        const double m = density * volume;
        const double c = 2.0 / 5.0 * r * r;
        g.mass.push_back(m);
        g.inertia.push_back(c * m);
        g.mu.push_back(mu);
        g.rest_n.push_back(0.0);
        g.rest_t.push_back(0.0);
        g.body_scene.push_back(scene);
    }
}

}  // namespace

extern "C" {

int cdx_gen_create(const cdx_gen_params* p, cdx_gen_scene** out) {
    if (!p || !out) return CDX_ERR_ARG;
    *out = nullptr;
    cdx_gen_scene* g = new (std::nothrow) cdx_gen_scene();
    if (!g) return CDX_ERR_ARG;
    Rng rng(p->seed);
    const int max_att = p->max_attempts > 0 ? p->max_attempts : 200000;
    auto draw_r = [&]() { return (p->r_hi > p->r_lo) ? rng.uni(p->r_lo, p->r_hi) : p->r_lo; };
    if (p->kind == 0) {
        const int S = std::max(1, p->num_scenes);
        const int cols = (int)std::ceil(std::sqrt((double)S));
        const double pitch_x = p->box[0] + 0.5, pitch_y = p->box[1] + 0.5;
        for (int s = 0; s < S; ++s) {
            int n = p->num_bodies;
            if (p->nb_lo > 0 && p->nb_hi >= p->nb_lo)
                n = (int)std::lround(std::exp(rng.uni(std::log((double)p->nb_lo), std::log((double)p->nb_hi))));
            const double mu = (p->mu_hi > p->mu_lo) ? rng.uni(p->mu_lo, p->mu_hi) : p->mu;
            std::vector<double> rr(n);
            for (auto& r : rr) r = draw_r();
            const double ox = (s % cols) * pitch_x, oy = (s / cols) * pitch_y;
            const double lo[3] = {ox, oy, 0.0}, hi[3] = {ox + p->box[0], oy + p->box[1], p->box[2]};
            std::vector<double> pos;
            if (!place(rng, rr, lo, hi, [](const double*, double) { return true; }, max_att, pos)) {
                delete g;
                return CDX_ERR_OVERFLOW;
            }
            const double up[3] = {0, 0, 1}, px[3] = {1, 0, 0}, mx[3] = {-1, 0, 0}, py[3] = {0, 1, 0},
                         my[3] = {0, -1, 0};
            const double ground[3] = {ox + 0.5 * p->box[0], oy + 0.5 * p->box[1], 0.0};
            const double w0[3] = {ox, oy + 0.5 * p->box[1], 0.5 * p->box[2]};
            const double w1[3] = {ox + p->box[0], oy + 0.5 * p->box[1], 0.5 * p->box[2]};
            const double w2[3] = {ox + 0.5 * p->box[0], oy, 0.5 * p->box[2]};
            const double w3[3] = {ox + 0.5 * p->box[0], oy + p->box[1], 0.5 * p->box[2]};
            add_static(*g, CDX_STATIC_HALFSPACE, ground, up, 0.0, nullptr, mu, s);
            add_static(*g, CDX_STATIC_HALFSPACE, w0, px, 0.0, nullptr, mu, s);
            add_static(*g, CDX_STATIC_HALFSPACE, w1, mx, 0.0, nullptr, mu, s);
            add_static(*g, CDX_STATIC_HALFSPACE, w2, py, 0.0, nullptr, mu, s);
            add_static(*g, CDX_STATIC_HALFSPACE, w3, my, 0.0, nullptr, mu, s);
            add_bodies(*g, rng, pos, rr, p->density, mu, p->v_sigma, s);
        }
        g->num_scenes = S;
    } else if (p->kind == 1) {
        const double R = p->drum_radius, L = p->drum_length;
        std::vector<double> rr(std::max(0, p->num_bodies));
        for (auto& r : rr) r = draw_r();
        const double lo[3] = {0.0, -R, -R}, hi[3] = {L, R, R};
        std::vector<double> pos;
        auto inside = [R](const double* q, double r) { return q[1] * q[1] + q[2] * q[2] <= (R - r) * (R - r); };
        if (!place(rng, rr, lo, hi, inside, max_att, pos)) {
            delete g;
            return CDX_ERR_OVERFLOW;
        }
        const double o[3] = {0, 0, 0}, ax[3] = {1, 0, 0}, w[3] = {p->drum_omega, 0, 0};
        const double e1[3] = {L, 0, 0}, mx[3] = {-1, 0, 0};
        add_static(*g, CDX_STATIC_DRUM, o, ax, R, w, p->mu, 0);
        add_static(*g, CDX_STATIC_HALFSPACE, o, ax, 0.0, nullptr, p->mu, 0);
        add_static(*g, CDX_STATIC_HALFSPACE, e1, mx, 0.0, nullptr, p->mu, 0);
        add_bodies(*g, rng, pos, rr, p->density, p->mu, p->v_sigma, 0);
        g->num_scenes = 1;
    } else {
        delete g;
        return CDX_ERR_ARG;
    }
    *out = g;
    return CDX_OK;
}

int cdx_gen_view(const cdx_gen_scene* g, cdx_scene* v) {
    if (!g || !v) return CDX_ERR_ARG;
    std::memset(v, 0, sizeof(*v));
    v->num_bodies = (int32_t)g->radius.size();
    v->pos = g->pos.data();
    v->quat = g->quat.data();
    v->vel = g->vel.data();
    v->omega = g->omega.data();
    v->radius = g->radius.data();
    v->mass = g->mass.data();
    v->inertia = g->inertia.data();
    v->mu = g->mu.data();
    v->rest_n = g->rest_n.data();
    v->rest_t = g->rest_t.data();
    v->body_scene = g->body_scene.data();
    v->num_statics = (int32_t)g->static_kind.size();
    v->static_kind = g->static_kind.data();
    v->static_pos = g->static_pos.data();
    v->static_quat = g->static_quat.data();
    v->static_vel = g->static_vel.data();
    v->static_omega = g->static_omega.data();
    v->static_dir = g->static_dir.data();
    v->static_radius = g->static_radius.data();
    v->static_mu = g->static_mu.data();
    v->static_rest_n = g->static_rest_n.data();
    v->static_rest_t = g->static_rest_t.data();
    v->static_scene = g->static_scene.data();
    v->num_scenes = g->num_scenes;
    v->static_half_length = nullptr;  // the generated scenes hold no cylinder
    return CDX_OK;
}

void cdx_gen_destroy(cdx_gen_scene* g) { delete g; }

}  // extern "C"
