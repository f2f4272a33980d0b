// Frame output of the engine: VTK PolyData (.vtp) frames with ParaView collections (.pvd) and the
// tracked-body CSV, as the reference's PhysicsPipeline writes them (physics_pipeline.cpp:62-113).
// The host side of a frame (state and contacts copied down) is built on the calling thread; the
// formatting and the file writes run on one background writer thread behind a bounded queue
// (VtkWriter, io/vtk_writer.hpp:38-107), so the next steps run while a frame is written.
#pragma once
#include <condition_variable>
#include <cstdint>
#include <deque>
#include <fstream>
#include <functional>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/cdx.h"

namespace cdx {

// host copies of the scene that the frames need (taken when the scene is loaded)
struct OutputScene {
    int N = 0, S = 0;
    std::vector<double> radius, mu;
    std::vector<int32_t> skind;
    std::vector<double> spos, sdir, srad, smu, shl;  // shl: cylinder half lengths
    std::vector<double> squat, she;                  // orientations (x, y, z, w); box half extents
    std::vector<double> pos0;  // initial sphere centres (extent of the static meshes)
};

// one frame of host data (moved into the writer job)
struct OutputFrame {
    int64_t step = 0;
    double time = 0.0;
    std::vector<double> pos, quat, vel, omega;  // 3N, 4N (x, y, z, w), 3N, 3N (body frame)
    int32_t nc = 0;
    std::vector<int32_t> ia, ib;                // entity ids: statics first, then spheres
    std::vector<double> point, lambda, normal;  // 3 nc each
};

struct TrackedRow {
    std::string name;
    double p[3], v[3], w[3], q[4];
};

class Output {
   public:
    explicit Output(const cdx_config& cfg);
    ~Output();
    Output(const Output&) = delete;
    Output& operator=(const Output&) = delete;

    bool vtk_on() const { return interval_ > 0; }
    bool due(int64_t step) const { return interval_ > 0 && step % interval_ == 0; }
    bool contacts_on() const { return manifolds_; }
    void set_scene(OutputScene s) { scene_ = std::move(s); }
    // frames: the static geometry once, then the sphere frame and the contact frame of this step
    void frame(OutputFrame f);
    // one row per tracked body at time t (CsvWriter::writeTrackedState, io/csv_writer.hpp:43-52)
    void tracked(double t, std::vector<TrackedRow> rows);
    // waits until every queued job is written
    void flush();
    std::string last_error();

   private:
    void enqueue(std::function<void()> job);
    void worker();
    std::string path_of(const std::string& file) const;

    int interval_ = 0;
    bool manifolds_ = true;
    int combine_ = 0;
    double dt_ = 0.0;
    std::string folder_, prefix_;
    OutputScene scene_;
    bool static_written_ = false;
    // writer thread and its bounded queue (depth 32, as the reference's)
    std::thread thread_;
    std::deque<std::function<void()>> queue_;
    std::mutex mu_;
    std::condition_variable not_empty_, not_full_, idle_;
    bool stop_ = false, busy_ = false;
    std::string err_;
    // collections, touched by the writer thread only
    struct PvdEntry {
        int64_t step;
        double time;
        std::string file;
    };
    std::vector<PvdEntry> pvd_geo_, pvd_contacts_;
    std::ofstream csv_;  // opened on the first tracked row
};

}  // namespace cdx
