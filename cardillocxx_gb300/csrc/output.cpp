// Frame output: VTK XML PolyData frames, ParaView collections and the tracked-body CSV.
//
// Files, names and arrays follow the reference's writers:
//   <prefix>_static_geo.vtp                      static shapes, once (vtk_writer.cpp:113-123)
//   <prefix>_geo_<step:04>.vtp, <prefix>_geo.pvd  dynamic bodies each output.interval_steps (:125-136)
//   <prefix>_contact_manifolds_<step:04>.vtp/.pvd contacts, when output.write_contact_manifolds (:138-143)
//   <prefix>_tracked.csv                         tracked bodies every step (csv_writer.hpp:20-95)
// The reference triangulates every body (MeshGenerator) and stores per-vertex arrays; a sphere
// frame here holds one point per sphere (its centre, with a vertex cell) and the same per-entity
// arrays plus "radius" and "quaternion", so ParaView draws the spheres with a glyph filter. A
// triangulated 200k-sphere frame would be tens of millions of vertices.
#include "output.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <sstream>

namespace fs = std::filesystem;

namespace cdx {
namespace {

// RFC 4648 base64 (the inline binary encoding of VTK XML files)
std::string base64(const unsigned char* p, size_t n) {
    static const char* tab = "ABCDEFGHIJKLMNOPQRSTUVWXYZabcdefghijklmnopqrstuvwxyz0123456789+/";
    std::string out;
    out.reserve(4 * ((n + 2) / 3));
    size_t i = 0;
    for (; i + 2 < n; i += 3) {
        const uint32_t v = (uint32_t)p[i] << 16 | (uint32_t)p[i + 1] << 8 | p[i + 2];
        out += tab[v >> 18];
        out += tab[(v >> 12) & 63];
        out += tab[(v >> 6) & 63];
        out += tab[v & 63];
    }
    if (i < n) {
        const uint32_t v = (uint32_t)p[i] << 16 | (i + 1 < n ? (uint32_t)p[i + 1] << 8 : 0u);
        out += tab[v >> 18];
        out += tab[(v >> 12) & 63];
        out += i + 1 < n ? tab[(v >> 6) & 63] : '=';
        out += '=';
    }
    return out;
}

struct VtpArray {
    const char* type;  // Float32, Int32, Int64
    std::string name;
    int ncomp;
    std::vector<unsigned char> bytes;
};

template <class T>
VtpArray make_array(const char* type, const std::string& name, int ncomp, const std::vector<T>& v) {
    VtpArray a{type, name, ncomp, {}};
    a.bytes.resize(v.size() * sizeof(T));
    if (!v.empty()) std::memcpy(a.bytes.data(), v.data(), a.bytes.size());
    return a;
}

// one DataArray: base64 of a UInt64 byte count followed by the little-endian values, uncompressed
// (vtkXMLPolyDataWriter's binary mode without a compressor, vtk_writer.cpp:507-515)
void put_array(std::ostream& o, const VtpArray& a, const char* indent) {
    std::vector<unsigned char> blob(8 + a.bytes.size());
    const uint64_t nb = a.bytes.size();
    for (int k = 0; k < 8; ++k) blob[k] = (unsigned char)(nb >> (8 * k));
    if (nb) std::memcpy(blob.data() + 8, a.bytes.data(), nb);
    o << indent << "<DataArray type=\"" << a.type << "\" Name=\"" << a.name << "\"";
    if (a.ncomp > 1) o << " NumberOfComponents=\"" << a.ncomp << "\"";
    o << " format=\"binary\">\n" << indent << "  " << base64(blob.data(), blob.size()) << "\n" << indent << "</DataArray>\n";
}

struct CellBlock {
    std::vector<int64_t> conn, off;
};

bool write_vtp(const std::string& path, const std::vector<float>& pts, const std::vector<VtpArray>& pdata,
               const CellBlock& verts, const CellBlock& polys) {
    std::ofstream o(path, std::ios::out | std::ios::trunc | std::ios::binary);
    if (!o) return false;
    const size_t np = pts.size() / 3;
    o << "<?xml version=\"1.0\"?>\n";
    o << "<VTKFile type=\"PolyData\" version=\"1.0\" byte_order=\"LittleEndian\" header_type=\"UInt64\">\n";
    o << "  <PolyData>\n";
    o << "    <Piece NumberOfPoints=\"" << np << "\" NumberOfVerts=\"" << verts.off.size()
      << "\" NumberOfLines=\"0\" NumberOfStrips=\"0\" NumberOfPolys=\"" << polys.off.size() << "\">\n";
    o << "      <PointData>\n";
    for (const auto& a : pdata) put_array(o, a, "        ");
    o << "      </PointData>\n      <CellData>\n      </CellData>\n";
    o << "      <Points>\n";
    put_array(o, make_array("Float32", "Points", 3, pts), "        ");
    o << "      </Points>\n";
    const CellBlock empty;
    const char* kinds[4] = {"Verts", "Lines", "Strips", "Polys"};
    const CellBlock* blocks[4] = {&verts, &empty, &empty, &polys};
    for (int k = 0; k < 4; ++k) {
        o << "      <" << kinds[k] << ">\n";
        put_array(o, make_array("Int64", "connectivity", 1, blocks[k]->conn), "        ");
        put_array(o, make_array("Int64", "offsets", 1, blocks[k]->off), "        ");
        o << "      </" << kinds[k] << ">\n";
    }
    o << "    </Piece>\n  </PolyData>\n</VTKFile>\n";
    return (bool)o;
}

// PvdWriter::write (io/pvd_writer.cpp:11-24)
template <class E>
bool write_pvd(const std::string& path, const std::vector<E>& entries) {
    std::ofstream out(path, std::ios::out | std::ios::trunc);
    if (!out) return false;
    out << "<?xml version=\"1.0\"?>\n";
    out << "<VTKFile type=\"Collection\" version=\"0.1\" byte_order=\"LittleEndian\">\n";
    out << "  <Collection>\n";
    for (const auto& e : entries)
        out << "    <DataSet timestep=\"" << e.time << "\" part=\"0\" file=\"" << e.file << "\"/>\n";
    out << "  </Collection>\n";
    out << "</VTKFile>\n";
    return (bool)out;
}

inline double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
inline void cross3(const double* a, const double* b, double* c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}

// tangentFrameFromNormal: Frisvad's basis with the south-pole branch (the contact frame of the solver)
void tangent_frame(const double* n_in, double* t1, double* t2) {
    const double len = std::sqrt(dot3(n_in, n_in));
    if (len <= 2.220446049250313e-16) {
        t1[0] = 1; t1[1] = 0; t1[2] = 0;
        t2[0] = 0; t2[1] = 1; t2[2] = 0;
        return;
    }
    const double n[3] = {n_in[0] / len, n_in[1] / len, n_in[2] / len};
    if (n[2] < -0.9999999) {
        t1[0] = 0; t1[1] = -1; t1[2] = 0;
        const double d = dot3(n, t1);
        for (int k = 0; k < 3; ++k) t1[k] -= n[k] * d;
    } else {
        const double a = 1.0 / (1.0 + n[2]);
        t1[0] = 1.0 - n[0] * n[0] * a;
        t1[1] = -n[0] * n[1] * a;
        t1[2] = -n[0];
    }
    const double s = std::sqrt(dot3(t1, t1));
    if (s > 0) for (int k = 0; k < 3; ++k) t1[k] /= s;
    cross3(n, t1, t2);
}

// rotation matrix (row-major) of a unit quaternion (x, y, z, w)
void quat_to_R(const double* q, double* R) {
    const double x = q[0], y = q[1], z = q[2], w = q[3];
    R[0] = 1 - 2 * (y * y + z * z); R[1] = 2 * (x * y - z * w);     R[2] = 2 * (x * z + y * w);
    R[3] = 2 * (x * y + z * w);     R[4] = 1 - 2 * (x * x + z * z); R[5] = 2 * (y * z - x * w);
    R[6] = 2 * (x * z - y * w);     R[7] = 2 * (y * z + x * w);     R[8] = 1 - 2 * (x * x + y * y);
}

// Euler angles about x, then y, then z of R = Rx(a) Ry(b) Rz(c), with a, c in [-pi, pi] and b in
// [-pi/2, pi/2] (the ranges of Eigen's canonicalEulerAngles(0, 1, 2) used by the reference's CSV,
// csv_writer.hpp:74); at b = +-pi/2 the split between a and c is a convention
void euler_xyz(const double* R, double* e) {
    e[0] = std::atan2(-R[5], R[8]);
    e[1] = std::atan2(R[2], std::hypot(R[0], R[1]));
    e[2] = std::atan2(-R[1], R[0]);
}

double combine_mu(int rule, double a, double b) {
    if (rule == 1) return 0.5 * (a + b);
    if (rule == 2) return std::sqrt(std::max(0.0, a) * std::max(0.0, b));
    return std::min(a, b);
}

}  // namespace

Output::Output(const cdx_config& cfg)
    : interval_(std::max(0, cfg.output_interval_steps)),
      manifolds_(cfg.output_write_contact_manifolds != 0),
      combine_(cfg.friction_enable ? cfg.friction_combine : -1),
      dt_(cfg.sim_dt),
      folder_(cfg.output_folder),
      prefix_(cfg.output_filename_prefix) {
    if (!folder_.empty()) {
        std::error_code ec;
        fs::create_directories(folder_, ec);
    }
    thread_ = std::thread(&Output::worker, this);
}

Output::~Output() {
    {
        std::unique_lock<std::mutex> lk(mu_);
        not_full_.wait(lk, [this] { return queue_.empty(); });  // drain what was queued
        stop_ = true;
    }
    not_empty_.notify_all();
    if (thread_.joinable()) thread_.join();
}

std::string Output::path_of(const std::string& file) const {
    return folder_.empty() ? file : (fs::path(folder_) / file).string();
}

void Output::enqueue(std::function<void()> job) {
    std::unique_lock<std::mutex> lk(mu_);
    not_full_.wait(lk, [this] { return queue_.size() < 32 || stop_; });
    if (stop_) return;
    queue_.push_back(std::move(job));
    lk.unlock();
    not_empty_.notify_one();
}

void Output::worker() {
    for (;;) {
        std::function<void()> job;
        {
            std::unique_lock<std::mutex> lk(mu_);
            not_empty_.wait(lk, [this] { return stop_ || !queue_.empty(); });
            if (queue_.empty()) return;
            job = std::move(queue_.front());
            queue_.pop_front();
            busy_ = true;
        }
        not_full_.notify_all();
        job();
        {
            std::lock_guard<std::mutex> lk(mu_);
            busy_ = false;
        }
        idle_.notify_all();
    }
}

void Output::flush() {
    std::unique_lock<std::mutex> lk(mu_);
    idle_.wait(lk, [this] { return queue_.empty() && !busy_; });
}

std::string Output::last_error() {
    std::lock_guard<std::mutex> lk(mu_);
    return err_;
}

void Output::frame(OutputFrame f) {
    const bool write_static = !static_written_;
    static_written_ = true;
    enqueue([this, f = std::move(f), write_static]() {
        const OutputScene& sc = scene_;
        const int N = sc.N, S = sc.S;
        auto fail = [this](const std::string& what) {
            std::lock_guard<std::mutex> lk(mu_);
            err_ = "cannot write " + what;
        };
        char num[32];
        std::snprintf(num, sizeof(num), "_%04lld.vtp", (long long)f.step);
        // static shapes: a square patch per halfspace sized to the initial extent of the spheres, a
        // cylinder wall per drum or cylinder, a box's faces; all at their pose at load
        if (write_static) {
            std::vector<float> pts;
            std::vector<float> vel;
            std::vector<int32_t> ids;
            CellBlock polys, verts;
            auto add_tri = [&](int64_t a, int64_t b, int64_t c) {
                polys.conn.insert(polys.conn.end(), {a, b, c});
                polys.off.push_back((int64_t)polys.conn.size());
            };
            for (int s = 0; s < S; ++s) {
                const double* p = &sc.spos[3 * s];
                double d[3] = {sc.sdir[3 * s], sc.sdir[3 * s + 1], sc.sdir[3 * s + 2]};
                const double dl = std::sqrt(dot3(d, d));
                if (dl > 0) for (int k = 0; k < 3; ++k) d[k] /= dl;
                double t1[3], t2[3];
                tangent_frame(d, t1, t2);
                double ext = 1.0, lo = -0.5, hi = 0.5;
                bool any = false;
                for (int i = 0; i < N; ++i) {
                    const double r[3] = {sc.pos0[3 * i] - p[0], sc.pos0[3 * i + 1] - p[1], sc.pos0[3 * i + 2] - p[2]};
                    const double ax = dot3(r, d), rr = sc.radius[i];
                    ext = std::max(ext, 1.25 * (std::sqrt(std::max(0.0, dot3(r, r) - ax * ax)) + rr));
                    lo = any ? std::min(lo, ax - rr) : ax - rr;
                    hi = any ? std::max(hi, ax + rr) : ax + rr;
                    any = true;
                }
                const int64_t base = (int64_t)pts.size() / 3;
                auto add_pt = [&](const double* x) {
                    for (int k = 0; k < 3; ++k) pts.push_back((float)x[k]);
                    vel.insert(vel.end(), {0.f, 0.f, 0.f});
                    ids.push_back(s);
                };
                if (sc.skind[s] == CDX_STATIC_CYLINDER) {
                    lo = -sc.shl[s];
                    hi = sc.shl[s];
                }
                if (sc.skind[s] == CDX_STATIC_BOX) {
                    // the box's eight corners and twelve triangles, in its orientation at load
                    double R[9];
                    quat_to_R(&sc.squat[4 * s], R);
                    const double* e = &sc.she[3 * s];
                    for (int j = 0; j < 8; ++j) {
                        const double l[3] = {(j & 1) ? e[0] : -e[0], (j & 2) ? e[1] : -e[1], (j & 4) ? e[2] : -e[2]};
                        double x[3];
                        for (int k = 0; k < 3; ++k) x[k] = p[k] + ((R[3 * k] * l[0] + R[3 * k + 1] * l[1]) + R[3 * k + 2] * l[2]);
                        add_pt(x);
                    }
                    static const int quads[6][4] = {{0, 2, 6, 4}, {1, 5, 7, 3}, {0, 4, 5, 1},
                                                    {2, 3, 7, 6}, {0, 1, 3, 2}, {4, 6, 7, 5}};
                    for (auto& qd : quads) {
                        add_tri(base + qd[0], base + qd[1], base + qd[2]);
                        add_tri(base + qd[0], base + qd[2], base + qd[3]);
                    }
                } else if (sc.skind[s] == CDX_STATIC_DRUM || sc.skind[s] == CDX_STATIC_CYLINDER) {
                    const int seg = 64;
                    const double R = sc.srad[s];
                    for (int j = 0; j < seg; ++j) {
                        const double ang = 2.0 * M_PI * j / seg, c = std::cos(ang), sn = std::sin(ang);
                        for (int e = 0; e < 2; ++e) {
                            const double ax = e ? hi : lo;
                            double x[3];
                            for (int k = 0; k < 3; ++k) x[k] = p[k] + ax * d[k] + R * (c * t1[k] + sn * t2[k]);
                            add_pt(x);
                        }
                    }
                    for (int j = 0; j < seg; ++j) {
                        const int64_t a0 = base + 2 * j, a1 = a0 + 1, b0 = base + 2 * ((j + 1) % seg), b1 = b0 + 1;
                        add_tri(a0, b0, b1);
                        add_tri(a0, b1, a1);
                    }
                } else {
                    const double cs[4][2] = {{-1, -1}, {1, -1}, {1, 1}, {-1, 1}};
                    for (auto& c : cs) {
                        double x[3];
                        for (int k = 0; k < 3; ++k) x[k] = p[k] + ext * (c[0] * t1[k] + c[1] * t2[k]);
                        add_pt(x);
                    }
                    add_tri(base, base + 1, base + 2);
                    add_tri(base, base + 2, base + 3);
                }
            }
            std::vector<VtpArray> arrs;
            arrs.push_back(make_array("Float32", "velocity", 3, vel));
            arrs.push_back(make_array("Int32", "entity_id", 1, ids));
            if (!write_vtp(path_of(prefix_ + "_static_geo.vtp"), pts, arrs, verts, polys)) fail("static geometry");
        }
        // per-sphere compressive force from the normal impulses (VtkWriter::enrichPressure,
        // vtk_writer.cpp:154-193); area of the sphere 4 pi r^2
        const double inv_dt = dt_ > 0 ? 1.0 / dt_ : 1.0;
        std::vector<double> force(N, 0.0);
        for (int c = 0; c < f.nc; ++c) {
            const double pn = std::max(0.0, f.lambda[3 * (size_t)c]) * inv_dt;
            if (pn <= 0) continue;
            const int ea = f.ia[c] - S, eb = f.ib[c] - S;
            if (ea >= 0 && ea < N) force[ea] += pn;
            if (eb >= 0 && eb < N) force[eb] += pn;
        }
        {
            std::vector<float> pts(3 * (size_t)N), v(3 * (size_t)N), w(3 * (size_t)N), ww(3 * (size_t)N),
                q(4 * (size_t)N), rad(N), pres(N);
            std::vector<int32_t> id(N);
            CellBlock verts, polys;
            verts.conn.resize(N);
            verts.off.resize(N);
            for (int i = 0; i < N; ++i) {
                double R[9];
                quat_to_R(&f.quat[4 * (size_t)i], R);
                const double* om = &f.omega[3 * (size_t)i];
                for (int k = 0; k < 3; ++k) {
                    pts[3 * i + k] = (float)f.pos[3 * (size_t)i + k];
                    v[3 * i + k] = (float)f.vel[3 * (size_t)i + k];
                    w[3 * i + k] = (float)om[k];
                    ww[3 * i + k] = (float)(R[3 * k] * om[0] + R[3 * k + 1] * om[1] + R[3 * k + 2] * om[2]);
                }
                for (int k = 0; k < 4; ++k) q[4 * i + k] = (float)f.quat[4 * (size_t)i + k];
                rad[i] = (float)sc.radius[i];
                const double area = 4.0 * M_PI * sc.radius[i] * sc.radius[i];
                const double p = area > 1e-12 ? force[i] / area : 0.0;
                pres[i] = std::isfinite(p) ? (float)p : 0.f;
                id[i] = S + i;
                verts.conn[i] = i;
                verts.off[i] = i + 1;
            }
            std::vector<VtpArray> arrs;
            arrs.push_back(make_array("Float32", "velocity", 3, v));
            arrs.push_back(make_array("Float32", "angular_velocity", 3, w));
            arrs.push_back(make_array("Float32", "angular_velocity_world", 3, ww));
            arrs.push_back(make_array("Float32", "entity_velocity", 3, v));
            arrs.push_back(make_array("Int32", "entity_id", 1, id));
            arrs.push_back(make_array("Float32", "entity_pressure", 1, pres));
            arrs.push_back(make_array("Float32", "radius", 1, rad));
            arrs.push_back(make_array("Float32", "quaternion", 4, q));
            const std::string file = prefix_ + "_geo" + num;
            if (!write_vtp(path_of(file), pts, arrs, verts, polys)) fail(file);
            pvd_geo_.push_back({f.step, f.time, file});
            if (!write_pvd(path_of(prefix_ + "_geo.pvd"), pvd_geo_)) fail("the geometry collection");
        }
        // contact frame: every sphere contact is a one-point manifold (contactManifoldsToPolyData,
        // vtk_writer.cpp:424-505); pressure needs three or more points, so it is 0
        if (manifolds_) {
            const int nc = f.nc;
            std::vector<float> pts(3 * (size_t)nc), nrm(3 * (size_t)nc), t1a(3 * (size_t)nc), t2a(3 * (size_t)nc),
                per(3 * (size_t)nc), pen(nc), pres(nc, 0.f), muv(nc), pn(nc), ptm(nc);
            std::vector<int32_t> ida(nc), idb(nc), patch(nc);
            CellBlock verts, polys;
            verts.conn.resize(nc);
            verts.off.resize(nc);
            for (int c = 0; c < nc; ++c) {
                const double* n = &f.normal[3 * (size_t)c];
                const double* l = &f.lambda[3 * (size_t)c];
                double t1[3], t2[3];
                tangent_frame(n, t1, t2);
                const double pnc = std::max(0.0, l[0]);
                for (int k = 0; k < 3; ++k) {
                    pts[3 * c + k] = (float)f.point[3 * (size_t)c + k];
                    nrm[3 * c + k] = (float)n[k];
                    t1a[3 * c + k] = (float)t1[k];
                    t2a[3 * c + k] = (float)t2[k];
                    per[3 * c + k] = (float)(pnc * n[k] + l[1] * t1[k] + l[2] * t2[k]);
                }
                pn[c] = (float)pnc;
                ptm[c] = (float)std::sqrt(l[1] * l[1] + l[2] * l[2]);
                // penetration and combined friction at the frame's positions
                const int a = f.ia[c], b = f.ib[c] - S;
                double depth = 0.0, mu = 0.0;
                if (b >= 0 && b < N) {
                    const double* xb = &f.pos[3 * (size_t)b];
                    const double rb = sc.radius[b];
                    if (a < S) {
                        const double* p = &sc.spos[3 * a];
                        double d[3] = {sc.sdir[3 * a], sc.sdir[3 * a + 1], sc.sdir[3 * a + 2]};
                        const double dl = std::sqrt(dot3(d, d));
                        if (dl > 0) for (int k = 0; k < 3; ++k) d[k] /= dl;
                        const double r[3] = {xb[0] - p[0], xb[1] - p[1], xb[2] - p[2]};
                        const double ax = dot3(r, d);
                        if (sc.skind[a] == CDX_STATIC_DRUM) {
                            depth = std::sqrt(std::max(0.0, dot3(r, r) - ax * ax)) + rb - sc.srad[a];
                        } else if (sc.skind[a] == CDX_STATIC_CYLINDER) {
                            // distance of the centre to the solid cylinder (outside; inside counts 0)
                            const double rho = std::sqrt(std::max(0.0, dot3(r, r) - ax * ax));
                            const double dr = std::max(0.0, rho - sc.srad[a]);
                            const double dz = std::max(0.0, std::fabs(ax) - sc.shl[a]);
                            depth = rb - std::sqrt(dr * dr + dz * dz);
                        } else if (sc.skind[a] == CDX_STATIC_BOX) {
                            // distance of the centre to the solid box (outside; inside counts 0)
                            double R[9];
                            quat_to_R(&sc.squat[4 * a], R);
                            double o2 = 0.0;
                            for (int k = 0; k < 3; ++k) {
                                const double c = (R[k] * r[0] + R[3 + k] * r[1]) + R[6 + k] * r[2];
                                const double o = std::max(0.0, std::fabs(c) - sc.she[3 * a + k]);
                                o2 += o * o;
                            }
                            depth = rb - std::sqrt(o2);
                        } else {
                            depth = rb - ax;
                        }
                        mu = combine_mu(combine_, sc.smu[a], sc.mu[b]);
                    } else {
                        const int ai = a - S;
                        const double* xa = &f.pos[3 * (size_t)ai];
                        const double r[3] = {xb[0] - xa[0], xb[1] - xa[1], xb[2] - xa[2]};
                        depth = sc.radius[ai] + rb - std::sqrt(dot3(r, r));
                        mu = combine_mu(combine_, sc.mu[ai], sc.mu[b]);
                    }
                }
                pen[c] = (float)depth;
                muv[c] = combine_ < 0 ? 0.f : (float)mu;
                ida[c] = a;
                idb[c] = f.ib[c];
                patch[c] = c;
                verts.conn[c] = c;
                verts.off[c] = c + 1;
            }
            std::vector<VtpArray> arrs;
            arrs.push_back(make_array("Float32", "normal", 3, nrm));
            arrs.push_back(make_array("Float32", "tangent1", 3, t1a));
            arrs.push_back(make_array("Float32", "tangent2", 3, t2a));
            arrs.push_back(make_array("Float32", "penetration", 1, pen));
            arrs.push_back(make_array("Float32", "pressure", 1, pres));
            arrs.push_back(make_array("Float32", "friction_mu", 1, muv));
            arrs.push_back(make_array("Int32", "id_a", 1, ida));
            arrs.push_back(make_array("Int32", "id_b", 1, idb));
            arrs.push_back(make_array("Int32", "patch_id", 1, patch));
            arrs.push_back(make_array("Float32", "pn", 1, pn));
            arrs.push_back(make_array("Float32", "pt_mag", 1, ptm));
            arrs.push_back(make_array("Float32", "percussion", 3, per));
            const std::string file = prefix_ + "_contact_manifolds" + num;
            if (!write_vtp(path_of(file), pts, arrs, verts, polys)) fail(file);
            pvd_contacts_.push_back({f.step, f.time, file});
            if (!write_pvd(path_of(prefix_ + "_contact_manifolds.pvd"), pvd_contacts_)) fail("the contact collection");
        }
    });
}

void Output::tracked(double t, std::vector<TrackedRow> rows) {
    enqueue([this, t, rows = std::move(rows)]() {
        std::ofstream& out = csv_;
        if (!out.is_open()) {
            const std::string path = path_of(prefix_ + "_tracked.csv");
            out.open(path, std::ios::out | std::ios::trunc);
            if (!out) {
                std::lock_guard<std::mutex> lk(mu_);
                err_ = "cannot write " + path;
                return;
            }
            out << "t,name,px,py,pz,vx,vy,vz,wx,wy,wz,euler_x,euler_y,euler_z\n";
        }
        // default stream formatting, as the reference's writer (csv_writer.hpp:79-90)
        for (const auto& r : rows) {
            double R[9], e[3];
            quat_to_R(r.q, R);
            euler_xyz(R, e);
            out << t << "," << r.name << "," << r.p[0] << "," << r.p[1] << "," << r.p[2] << "," << r.v[0] << ","
                << r.v[1] << "," << r.v[2] << "," << r.w[0] << "," << r.w[1] << "," << r.w[2] << "," << e[0] << ","
                << e[1] << "," << e[2] << "\n";
        }
        out.flush();
    });
}

}  // namespace cdx
