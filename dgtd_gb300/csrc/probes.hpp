// Point probes and running FP64 DFT accumulators (device side).
//
// Replaces the reference's point probes (PointProbe, src/components/Probes.h:132-160,
// updated by ProbesManager::updateProbe, src/solver/ProbesManager.cpp:380-405:
// GridFunction::GetValue of every field component at a located point every
// visSteps steps) and the offline DFT of exported surface snapshots the
// near-to-far post-processor runs (RCSSurfacePostProcessor.cpp:274-300:
// F(f) = (1/N) sum_n u(t_n) exp(-i 2 pi f t_n)). Here the sums are accumulated on
// the device while stepping, in FP64, so no snapshot ever leaves the GPU.
//
// An "item" is a point probe (an interpolation over the Np nodes of the element
// that contains the point) or a surface node (one face node of a face of the
// near-to-far surface). Items are stored as short weighted sums of state entries,
// so one kernel serves the FP64 reference layout and the FP32 batched layout.
#pragma once
#include <cstdint>
#include <memory>
#include <vector>

#include <cuda_runtime.h>

#include "mesh.hpp"
#include "refelem.hpp"

namespace dgtd {

struct ProbeSpec {
    std::vector<double> points;          // [n_points][3]
    std::vector<int32_t> surface_faces;  // [n_faces][3] vertex ids; winding normal points outwards
    std::vector<double> freqs;           // DFT frequencies (cycles per unit time)
    int every = 1;                       // sample after every `every`-th step
    int max_records = 0;                 // time-series capacity (samples of all points)
};

// Addressing of one field value (incidence b, component c) of a state vector:
// state[term_off + c * cstride + b * bstride].
struct ProbeStateLayout {
    bool fp32 = false;   // batched FP32 layout [e'][c][i][b]
    bool f32_ref = false;// FP32 values in the reference layout [b][c][e*Np+i]
    int Np = 0;
    int Bp = 1;          // incidence stride unit of the FP32 layout (padded batch)
    int B = 1;           // incidences
    int64_t N = 0;       // K * Np
    const int32_t* inv_perm = nullptr;   // FP32 form: internal index of each reference element (host)
};

constexpr int kMaxProbeFreqs = 64;

class ProbeSet {
public:
    static std::unique_ptr<ProbeSet> create(const RefTet& ref, const MeshTables& mesh, const ProbeSpec& spec,
                                            const ProbeStateLayout& lay);
    ~ProbeSet();

    int every() const { return every_; }
    int64_t n_points() const { return n_points_; }
    int64_t n_surface_nodes() const { return n_items_ - n_points_; }
    int n_freqs() const { return static_cast<int>(freqs_.size()); }
    int64_t n_samples() const { return n_samples_; }
    int64_t n_records() const { return n_records_; }
    int64_t kernel_launches() const { return launches_; }
    int64_t device_bytes() const { return device_bytes_; }

    void reset(cudaStream_t s);
    // Add the state at time t to the DFT sums and (while capacity lasts) to the point time series.
    void sample(const void* d_state, double t, cudaStream_t s);
    // Raw sums, [B][items][6][n_freqs][2]; time series [records][B][n_points][6] and times.
    void read(double* point_dft, double* surface_dft, double* series, double* series_t, cudaStream_t s) const;

    const std::vector<double>& surface_xyz() const { return surf_xyz_; }
    const std::vector<double>& surface_normal() const { return surf_n_; }
    const std::vector<double>& surface_weight() const { return surf_w_; }

private:
    ProbeStateLayout lay_{};
    int every_ = 1;
    int max_records_ = 0;
    int64_t n_points_ = 0, n_items_ = 0;
    std::vector<double> freqs_;
    int32_t* item_ptr_ = nullptr;     // [n_items + 1]
    int64_t* term_off_ = nullptr;     // state offset of (c = 0, b = 0)
    double* term_w_ = nullptr;
    double* acc_ = nullptr;           // [B][n_items][6][nf][2]
    double* series_ = nullptr;        // [max_records][B][n_points][6]
    std::vector<double> series_t_;
    int64_t n_samples_ = 0, n_records_ = 0, launches_ = 0, device_bytes_ = 0;
    std::vector<double> surf_xyz_, surf_n_, surf_w_;
};

}  // namespace dgtd
