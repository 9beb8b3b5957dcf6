// Point probes and running FP64 DFT accumulators (see probes.hpp).
#include "probes.hpp"

#include <algorithm>
#include <array>
#include <cmath>
#include <map>
#include <stdexcept>
#include <string>

namespace dgtd {

namespace {

void ckp(cudaError_t e, const char* what)
{
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

struct ProbeArgs {
    const int32_t* item_ptr;
    const int64_t* term_off;
    const double* term_w;
    double* acc;
    double* series;     // nullptr: no record this sample
    int64_t n_items, n_points;
    int64_t cstride, bstride;
    int64_t rec;        // record index
    int B, nf;
    double cs[kMaxProbeFreqs], sn[kMaxProbeFreqs];   // cos / sin of 2 pi f t
};

// One thread per (item, incidence): the item's six field values as a weighted sum
// of state entries (FP64 arithmetic), added to the DFT sums with exp(-i 2 pi f t).
template <typename T>
__global__ void __launch_bounds__(128) probe_sample_kernel(const T* __restrict__ st, const __grid_constant__ ProbeArgs a)
{
    const int64_t item = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const int b = blockIdx.y;
    if (item >= a.n_items) return;
    double v[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    const int q1 = a.item_ptr[item + 1];
    for (int q = a.item_ptr[item]; q < q1; ++q) {
        const double w = a.term_w[q];
        const int64_t o = a.term_off[q] + b * a.bstride;
#pragma unroll
        for (int c = 0; c < 6; ++c) v[c] += w * static_cast<double>(st[o + c * a.cstride]);
    }
    double* acc = a.acc + (static_cast<int64_t>(b) * a.n_items + item) * 6 * a.nf * 2;
    for (int c = 0; c < 6; ++c)
        for (int f = 0; f < a.nf; ++f) {
            acc[(c * a.nf + f) * 2] += v[c] * a.cs[f];
            acc[(c * a.nf + f) * 2 + 1] -= v[c] * a.sn[f];
        }
    if (a.series != nullptr && item < a.n_points) {
        double* s = a.series + ((a.rec * a.B + b) * a.n_points + item) * 6;
#pragma unroll
        for (int c = 0; c < 6; ++c) s[c] = v[c];
    }
}

template <typename T>
T* dev_copy(const std::vector<T>& v, int64_t& bytes)
{
    T* d = nullptr;
    const size_t n = std::max<size_t>(v.size(), 1);
    ckp(cudaMalloc(&d, n * sizeof(T)), "cudaMalloc probes");
    if (!v.empty()) ckp(cudaMemcpy(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice), "H2D probes");
    bytes += static_cast<int64_t>(n * sizeof(T));
    return d;
}

}  // namespace

std::unique_ptr<ProbeSet> ProbeSet::create(const RefTet& ref, const MeshTables& mesh, const ProbeSpec& spec,
                                           const ProbeStateLayout& lay)
{
    if (spec.every < 1) throw std::invalid_argument("probe sampling interval must be >= 1");
    if (spec.max_records < 0) throw std::invalid_argument("max_records must be >= 0");
    if (spec.freqs.size() > static_cast<size_t>(kMaxProbeFreqs))
        throw std::invalid_argument("at most " + std::to_string(kMaxProbeFreqs) + " DFT frequencies");
    if (spec.points.size() % 3 || spec.surface_faces.size() % 3) throw std::invalid_argument("bad probe arrays");
    const int Np = ref.Np, Nfp = ref.Nfp;
    const int64_t K = mesh.K;
    if (static_cast<int64_t>(mesh.elem_vertices.size()) != 4 * K) throw std::invalid_argument("mesh has no vertex table");
    std::unique_ptr<ProbeSet> P(new ProbeSet());
    P->lay_ = lay;
    P->every_ = spec.every;
    P->max_records_ = spec.max_records;
    P->freqs_ = spec.freqs;
    const int64_t npts = static_cast<int64_t>(spec.points.size() / 3);
    P->n_points_ = npts;

    // state offset of (element e, node i) for c = 0, b = 0
    auto node_off = [&](int64_t e, int i) -> int64_t {
        if (lay.fp32) return (static_cast<int64_t>(lay.inv_perm[e]) * 6 * Np + i) * lay.Bp;
        return e * Np + i;
    };
    std::vector<int32_t> item_ptr(1, 0);
    std::vector<int64_t> term_off;
    std::vector<double> term_w;

    // ---- point probes: locate (first element containing the point), interpolate
    const double* X = mesh.vertices.data();
    std::vector<double> phi(Np);
    for (int64_t p = 0; p < npts; ++p) {
        const double* x = &spec.points[3 * p];
        int64_t found = -1;
        double rst[3] = {0, 0, 0};
        for (int64_t e = 0; e < K && found < 0; ++e) {
            const double* v0 = X + 3 * mesh.elem_vertices[4 * e];
            const double* G = &mesh.geo[e * 9];
            const double d[3] = {x[0] - v0[0], x[1] - v0[1], x[2] - v0[2]};
            double r[3];
            for (int q = 0; q < 3; ++q) r[q] = -1.0 + G[3 * q] * d[0] + G[3 * q + 1] * d[1] + G[3 * q + 2] * d[2];
            const double tol = 1e-9;
            if (r[0] >= -1.0 - tol && r[1] >= -1.0 - tol && r[2] >= -1.0 - tol && r[0] + r[1] + r[2] <= -1.0 + tol) {
                found = e;
                rst[0] = r[0]; rst[1] = r[1]; rst[2] = r[2];
            }
        }
        if (found < 0)
            throw std::invalid_argument("probe point " + std::to_string(p) + " lies outside the mesh");
        nodal_basis_at(ref, rst[0], rst[1], rst[2], phi.data());
        for (int i = 0; i < Np; ++i) {
            term_off.push_back(node_off(found, i));
            term_w.push_back(phi[i]);
        }
        item_ptr.push_back(static_cast<int32_t>(term_off.size()));
    }

    // ---- near-to-far surface: the element on the inner side of each face, its face nodes
    const int64_t nfaces = static_cast<int64_t>(spec.surface_faces.size() / 3);
    if (nfaces > 0) {
        using Key = std::array<int32_t, 3>;
        std::map<Key, int64_t> want;
        for (int64_t q = 0; q < nfaces; ++q) {
            Key k{spec.surface_faces[3 * q], spec.surface_faces[3 * q + 1], spec.surface_faces[3 * q + 2]};
            std::sort(k.begin(), k.end());
            want[k] = q;
        }
        std::vector<std::vector<std::pair<int64_t, int>>> cand(nfaces);
        for (int64_t e = 0; e < K; ++e)
            for (int f = 0; f < 4; ++f) {
                Key k;
                int c = 0;
                for (int v = 0; v < 4; ++v)
                    if (v != f) k[c++] = mesh.elem_vertices[4 * e + v];
                std::sort(k.begin(), k.end());
                auto it = want.find(k);
                if (it != want.end()) cand[it->second].push_back({e, f});
            }
        for (int64_t q = 0; q < nfaces; ++q) {
            if (cand[q].empty()) throw std::invalid_argument("surface face " + std::to_string(q) + " is not a mesh face");
            const double* a = X + 3 * spec.surface_faces[3 * q];
            const double* bb = X + 3 * spec.surface_faces[3 * q + 1];
            const double* cc = X + 3 * spec.surface_faces[3 * q + 2];
            const double u[3] = {bb[0] - a[0], bb[1] - a[1], bb[2] - a[2]};
            const double w[3] = {cc[0] - a[0], cc[1] - a[1], cc[2] - a[2]};
            double n[3] = {u[1] * w[2] - u[2] * w[1], u[2] * w[0] - u[0] * w[2], u[0] * w[1] - u[1] * w[0]};
            const double twice_area = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
            if (!(twice_area > 0.0)) throw std::invalid_argument("degenerate surface face");
            for (double& v : n) v /= twice_area;
            std::pair<int64_t, int> pick = cand[q][0];
            for (const auto& ef : cand[q]) {
                const double* F = &mesh.fgeo[ef.first * 16 + ef.second * 4];
                if (F[0] * n[0] + F[1] * n[1] + F[2] * n[2] > 0.0) { pick = ef; break; }
            }
            const int64_t e = pick.first;
            const int f = pick.second;
            for (int a2 = 0; a2 < Nfp; ++a2) {
                const int i = ref.Fmask[f * Nfp + a2];
                term_off.push_back(node_off(e, i));
                term_w.push_back(1.0);
                item_ptr.push_back(static_cast<int32_t>(term_off.size()));
                const int64_t g = e * Np + i;
                P->surf_xyz_.insert(P->surf_xyz_.end(), {mesh.x[g], mesh.y[g], mesh.z[g]});
                P->surf_n_.insert(P->surf_n_.end(), {n[0], n[1], n[2]});
                P->surf_w_.push_back(ref.face_w[f * Nfp + a2] * 0.5 * twice_area / 2.0);
            }
        }
    }
    P->n_items_ = static_cast<int64_t>(item_ptr.size()) - 1;
    P->item_ptr_ = dev_copy(item_ptr, P->device_bytes_);
    P->term_off_ = dev_copy(term_off, P->device_bytes_);
    P->term_w_ = dev_copy(term_w, P->device_bytes_);
    const int64_t acc_len = static_cast<int64_t>(lay.B) * P->n_items_ * 6 * std::max<int64_t>(1, P->freqs_.size()) * 2;
    ckp(cudaMalloc(&P->acc_, acc_len * sizeof(double)), "cudaMalloc probe sums");
    P->device_bytes_ += acc_len * static_cast<int64_t>(sizeof(double));
    if (P->max_records_ > 0 && npts > 0) {
        const int64_t sl = static_cast<int64_t>(P->max_records_) * lay.B * npts * 6;
        ckp(cudaMalloc(&P->series_, sl * sizeof(double)), "cudaMalloc probe series");
        P->device_bytes_ += sl * static_cast<int64_t>(sizeof(double));
    }
    P->reset(nullptr);
    ckp(cudaStreamSynchronize(nullptr), "probe reset");
    return P;
}

ProbeSet::~ProbeSet()
{
    cudaFree(item_ptr_);
    cudaFree(term_off_);
    cudaFree(term_w_);
    cudaFree(acc_);
    cudaFree(series_);
}

void ProbeSet::reset(cudaStream_t s)
{
    const int64_t acc_len = static_cast<int64_t>(lay_.B) * n_items_ * 6 * std::max<int64_t>(1, freqs_.size()) * 2;
    ckp(cudaMemsetAsync(acc_, 0, acc_len * sizeof(double), s), "probe reset");
    n_samples_ = 0;
    n_records_ = 0;
    series_t_.clear();
}

void ProbeSet::sample(const void* d_state, double t, cudaStream_t s)
{
    if (n_items_ == 0) return;
    ProbeArgs a{};
    a.item_ptr = item_ptr_;
    a.term_off = term_off_;
    a.term_w = term_w_;
    a.acc = acc_;
    a.n_items = n_items_;
    a.n_points = n_points_;
    a.B = lay_.B;
    a.nf = static_cast<int>(freqs_.size());
    for (int f = 0; f < a.nf; ++f) {
        const double th = 2.0 * M_PI * freqs_[f] * t;
        a.cs[f] = std::cos(th);
        a.sn[f] = std::sin(th);
    }
    if (lay_.fp32) { a.cstride = static_cast<int64_t>(lay_.Np) * lay_.Bp; a.bstride = 1; }
    else { a.cstride = lay_.N; a.bstride = 6 * lay_.N; }
    a.series = nullptr;
    if (series_ != nullptr && n_records_ < max_records_) {
        a.series = series_;
        a.rec = n_records_;
        ++n_records_;
        series_t_.push_back(t);
    }
    dim3 grid(static_cast<unsigned>((n_items_ + 127) / 128), static_cast<unsigned>(lay_.B));
    if (lay_.fp32 || lay_.f32_ref) probe_sample_kernel<float><<<grid, 128, 0, s>>>(static_cast<const float*>(d_state), a);
    else probe_sample_kernel<double><<<grid, 128, 0, s>>>(static_cast<const double*>(d_state), a);
    ckp(cudaGetLastError(), "probe kernel");
    ++launches_;
    ++n_samples_;
}

void ProbeSet::read(double* point_dft, double* surface_dft, double* series, double* series_t, cudaStream_t s) const
{
    const int64_t per = 6 * static_cast<int64_t>(std::max<size_t>(1, freqs_.size())) * 2;
    const int nf = static_cast<int>(freqs_.size());
    std::vector<double> acc(static_cast<size_t>(lay_.B) * n_items_ * per);
    if (!acc.empty())
        ckp(cudaMemcpyAsync(acc.data(), acc_, acc.size() * sizeof(double), cudaMemcpyDeviceToHost, s), "probe read");
    std::vector<double> ser;
    if (series != nullptr && n_records_ > 0) {
        ser.resize(static_cast<size_t>(n_records_) * lay_.B * n_points_ * 6);
        ckp(cudaMemcpyAsync(ser.data(), series_, ser.size() * sizeof(double), cudaMemcpyDeviceToHost, s), "probe read");
    }
    ckp(cudaStreamSynchronize(s), "probe read");
    const int64_t nsurf = n_items_ - n_points_;
    const int64_t out_per = 6 * static_cast<int64_t>(nf) * 2;
    for (int b = 0; b < lay_.B; ++b)
        for (int64_t it = 0; it < n_items_; ++it) {
            const double* src = acc.data() + (static_cast<int64_t>(b) * n_items_ + it) * per;
            double* dst = nullptr;
            if (it < n_points_) { if (point_dft) dst = point_dft + (static_cast<int64_t>(b) * n_points_ + it) * out_per; }
            else if (surface_dft) dst = surface_dft + (static_cast<int64_t>(b) * nsurf + (it - n_points_)) * out_per;
            if (dst) std::copy(src, src + out_per, dst);
        }
    if (series != nullptr && !ser.empty()) std::copy(ser.begin(), ser.end(), series);
    if (series_t != nullptr) std::copy(series_t_.begin(), series_t_.end(), series_t);
}

}  // namespace dgtd
