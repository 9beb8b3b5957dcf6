// Continuous-batching request server for the DG Maxwell step.
//
// Each request is one independent solve (the reference's Solver::run over its
// own mesh, src/solver/Solver.cpp:483-533, driven by one JSON case,
// src/driver/driver.cpp:1545): plain FP64 operator, classical RK4, its own
// order, plane wave, step size and final time. The server keeps every admitted
// request's mesh tables and fields resident in one device region carved from a
// fixed memory budget, and advances all active requests of the same order in
// the same kernel launches: a launch's blocks are the concatenation of the
// requests' element blocks, and each block finds its request by a binary
// search over the per-request first-block table passed in the launch
// parameters. The per-block arithmetic is fp64::stage_body, the same code the
// single-operator kernels run, so a request's result does not depend on what
// else is in the launch.
//
// Threads:
//   admission  - builds the mesh tables on the host, waits (FIFO) until the
//                region fits in the budget, uploads tables + initial state;
//   engine     - admits uploaded requests into free slots between rounds and
//                launches the stage kernels (one stream per order, so launches
//                of different orders overlap on the device);
//   retirement - waits for a finished request's last kernel, downloads its
//                state and returns its region and slot.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <deque>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "../../include/dgtd_gb300.h"
#include "arena.hpp"
#include "skipbound.hpp"
#include "fp64_stage.cuh"
#include "mesh.hpp"
#include "refelem.hpp"

namespace {
constexpr double kUnstableNormHost = 1e20;   // reference Solver.cpp:500-516
}

namespace dgtd {

int set_last_error(int code, const std::string& msg);   // capi.cu

namespace serve {

constexpr int kMaxSlots = DGTD_SERVER_MAX_ACTIVE;
constexpr int kMaxWaves = 8;
constexpr int64_t kAlign = 256;
constexpr int kMaxOrder = 6;

__host__ __device__ inline int64_t al(int64_t v) { return (v + kAlign - 1) / kAlign * kAlign; }

// Byte offsets of one request's tables and state inside its device region, for
// real-number size `ws` (8: FP64 serving, 4: FP32 serving).
// [0, y0) is uploaded at admission (tables, sources, initial state x);
// y0, y1, z are the RK4 registers.
struct Layout {
    int64_t geo, fgeo, mat, vmap, fcode, xyz, tfsf, pw, x, y0, y1, z, total;
};

__host__ __device__ inline Layout layout(int64_t K, int Np, int Nfp, int64_t n_tfsf, int ws)
{
    Layout L{};
    const int64_t N = K * Np;
    int64_t o = 0;
    L.geo = o;   o = al(o + K * 9 * ws);
    L.fgeo = o;  o = al(o + K * 16 * ws);
    L.mat = o;   o = al(o + K * 3 * ws);
    L.vmap = o;  o = al(o + K * 4 * Nfp * 4);
    L.fcode = o; o = al(o + K * 4 * 4);
    L.xyz = o;   o = al(o + 3 * N * ws);
    L.tfsf = o;  o = al(o + (n_tfsf > 0 ? n_tfsf : 1) * 4);
    L.pw = o;    o = al(o + kMaxWaves * static_cast<int64_t>(sizeof(PlaneWaveDev)));
    L.x = o;     o = al(o + 6 * N * ws);
    L.y0 = o;    o = al(o + 6 * N * ws);
    L.y1 = o;    o = al(o + 6 * N * ws);
    L.z = o;     o = al(o + 6 * N * ws);
    L.total = o;
    return L;
}

struct SlotParam {
    char* base;        // device region
    int64_t K;
    int64_t block0;    // first block of this request in the launch grid
    int64_t n_tfsf;    // elements on the TF/SF submesh
    double t, dt;      // step start time and step size
    double alpha;
    int32_t n_pw;
    int32_t pos;       // slot index (skip flag)
    int32_t skip_known;// TF/SF skip flag decided on the host (0 / 1), or -1: test on the device
};

// Skip flags the stage reads when the host has decided the test.
__device__ const int kSkipFlags[2] = {0, 1};

struct LaunchParam {
    const void* DrT;    // reference-element operators in the serving precision
    const void* DsT;
    const void* DtT;
    const void* LIFTT;
    const int* Fmask;
    int* skip;         // [kMaxSlots] TF/SF skip flags
    double c;          // stage time = t + c * dt
    int mode;          // MODE_RK4_1..4
    int n;             // requests in this launch
    SlotParam s[kMaxSlots];
};

template <int P, typename R>
__device__ __forceinline__ void slot_views(const LaunchParam& L, const SlotParam& S, TablesT<R>& T, StageArgsT<R>& A)
{
    using O = fp64::Ord<P>;
    const Layout Y = layout(S.K, O::Np, O::Nfp, S.n_tfsf, static_cast<int>(sizeof(R)));
    T.p = P; T.Np = O::Np; T.Nfp = O::Nfp; T.K = S.K; T.N = S.K * O::Np;
    T.DrT = static_cast<const R*>(L.DrT); T.DsT = static_cast<const R*>(L.DsT);
    T.DtT = static_cast<const R*>(L.DtT); T.LIFTT = static_cast<const R*>(L.LIFTT); T.Fmask = L.Fmask;
    T.geo = reinterpret_cast<const R*>(S.base + Y.geo);
    T.fgeo = reinterpret_cast<const R*>(S.base + Y.fgeo);
    T.mat = reinterpret_cast<const R*>(S.base + Y.mat);
    T.vmapP = reinterpret_cast<const int32_t*>(S.base + Y.vmap);
    T.fcode = reinterpret_cast<const int32_t*>(S.base + Y.fcode);
    T.xyz = reinterpret_cast<const R*>(S.base + Y.xyz);
    T.tfsf_elems = reinterpret_cast<const int32_t*>(S.base + Y.tfsf);
    T.n_tfsf_elems = S.n_tfsf;
    T.alpha = static_cast<R>(S.alpha);
    T.curved = nullptr;
    R* x = reinterpret_cast<R*>(S.base + Y.x);
    R* y0 = reinterpret_cast<R*>(S.base + Y.y0);
    R* y1 = reinterpret_cast<R*>(S.base + Y.y1);
    R* z = reinterpret_cast<R*>(S.base + Y.z);
    A = StageArgsT<R>{};
    A.t = S.t + L.c * S.dt;
    A.dt = static_cast<R>(S.dt);
    A.mode = L.mode;
    A.batch = 1;
    A.x = x;
    A.z = z;
    switch (L.mode) {
    case MODE_RK4_1: A.in = x; A.yout = y0; break;
    case MODE_RK4_2: A.in = y0; A.yout = y1; break;
    case MODE_RK4_3: A.in = y1; A.yout = y0; break;
    default: A.in = y0; A.yout = nullptr; break;   // MODE_RK4_4
    }
    if (S.n_pw > 0 && S.n_tfsf > 0) {
        A.pw = reinterpret_cast<const PlaneWaveDev*>(S.base + Y.pw);
        A.n_pw = S.n_pw;
        A.skip = S.skip_known >= 0 ? &kSkipFlags[S.skip_known] : L.skip + S.pos;
    } else {
        A.pw = nullptr;
        A.n_pw = 0;
        A.skip = nullptr;
    }
}

// One RK4 stage of every request in the launch.
template <int P, typename R>
__global__ void __launch_bounds__(fp64::kBlock) serve_stage(const __grid_constant__ LaunchParam L)
{
    const int64_t bx = blockIdx.x;
    int lo = 0, hi = L.n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (L.s[mid].block0 <= bx) lo = mid; else hi = mid - 1;
    }
    const SlotParam& S = L.s[lo];
    TablesT<R> T{};
    StageArgsT<R> A{};
    slot_views<P, R>(L, S, T, A);
    fp64::stage_body<P, R>(T, A, (bx - S.block0) * fp64::Ord<P, R>::EPB, 0);
}

// TF/SF skip flag of every request with sources (one block each).
template <int P, typename R>
__global__ void __launch_bounds__(256) serve_skip(const __grid_constant__ LaunchParam L)
{
    const SlotParam& S = L.s[blockIdx.x];
    if (S.n_pw <= 0 || S.n_tfsf <= 0 || S.skip_known >= 0) return;
    TablesT<R> T{};
    StageArgsT<R> A{};
    slot_views<P, R>(L, S, T, A);
    fp64::tfsf_skip_body<R>(T, A.pw, A.n_pw, 0, A.t, L.skip + S.pos);
}

template <int P, typename R>
cudaError_t launch_round_stage(const LaunchParam& L, int64_t blocks, bool any_src, cudaStream_t s)
{
    if (any_src) {
        serve_skip<P, R><<<L.n, 256, 0, s>>>(L);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    serve_stage<P, R><<<static_cast<unsigned>(blocks), fp64::kBlock, 0, s>>>(L);
    return cudaGetLastError();
}

template <typename R>
cudaError_t launch_stage_r(int p, const LaunchParam& L, int64_t blocks, bool any_src, cudaStream_t s)
{
    switch (p) {
    case 1: return launch_round_stage<1, R>(L, blocks, any_src, s);
    case 2: return launch_round_stage<2, R>(L, blocks, any_src, s);
    case 3: return launch_round_stage<3, R>(L, blocks, any_src, s);
    case 4: return launch_round_stage<4, R>(L, blocks, any_src, s);
    case 5: return launch_round_stage<5, R>(L, blocks, any_src, s);
    case 6: return launch_round_stage<6, R>(L, blocks, any_src, s);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_stage(bool fp32, int p, const LaunchParam& L, int64_t blocks, bool any_src, cudaStream_t s)
{
    return fp32 ? launch_stage_r<float>(p, L, blocks, any_src, s) : launch_stage_r<double>(p, L, blocks, any_src, s);
}

template <typename R>
int elements_per_block_r(int p)
{
    switch (p) {
    case 1: return fp64::Ord<1, R>::EPB;
    case 2: return fp64::Ord<2, R>::EPB;
    case 3: return fp64::Ord<3, R>::EPB;
    case 4: return fp64::Ord<4, R>::EPB;
    case 5: return fp64::Ord<5, R>::EPB;
    default: return fp64::Ord<6, R>::EPB;
    }
}

int elements_per_block(int p, bool fp32)
{
    return fp32 ? elements_per_block_r<float>(p) : elements_per_block_r<double>(p);
}

struct ServeError : std::runtime_error {
    int code;
    ServeError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

void ck(cudaError_t e, const char* what)
{
    if (e != cudaSuccess) throw ServeError(DGTD_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

std::vector<double> transposed(const std::vector<double>& a, int rows, int cols)
{
    std::vector<double> t(a.size());
    for (int i = 0; i < rows; ++i)
        for (int j = 0; j < cols; ++j) t[static_cast<size_t>(j) * rows + i] = a[static_cast<size_t>(i) * cols + j];
    return t;
}

struct OrderTables {
    RefTet ref;
    void* DrT = nullptr;     // in the serving precision
    void* DsT = nullptr;
    void* DtT = nullptr;
    void* LIFTT = nullptr;
    int* Fmask = nullptr;
};

struct Req {
    int64_t id = 0;
    MeshInput mesh;
    int order = 0;
    double alpha = 1.0;
    std::vector<PlaneWaveDev> waves;
    std::vector<double> init;
    double t0 = 0, T = 0, dt = 0, cfl = 1;
    // derived at admission
    int64_t K = 0;
    int Np = 0, Nfp = 0;
    int64_t n_tfsf = 0;
    Layout lay{};
    dgtd::TfsfSkipBound skip_bound;   // one plain Gaussian wave: host bounds of the skip test
    int64_t off = -1;
    int pos = -1;
    // stepping
    double t = 0;
    int64_t steps = 0;
    bool launched = false;
    cudaEvent_t ev_last = nullptr;
    // outcome
    int status = DGTD_REQ_QUEUED;
    int err_code = 0;
    std::string err;
    std::vector<double> result;
    double t_submit = 0, t_admit = 0, t_first = 0, t_done = 0;
    int unstable = 0;   // the final state's norm was not finite or above 1e20
};

using ReqP = std::shared_ptr<Req>;

}  // namespace serve
}  // namespace dgtd

using dgtd::serve::ReqP;

struct dgtd_server {
    dgtd_server_opts opts{};
    bool fp32 = false;              // FP32 serving (single-instance FP32 form of the stage)
    std::chrono::steady_clock::time_point t_start;
    char* arena_base = nullptr;
    dgtd::RangeAllocator arena;
    int* skip = nullptr;
    dgtd::serve::OrderTables ord[dgtd::serve::kMaxOrder + 1];
    cudaStream_t adm_stream = nullptr, ret_stream = nullptr;
    cudaStream_t ord_stream[dgtd::serve::kMaxOrder + 1] = {};
    cudaEvent_t round_ev[2][dgtd::serve::kMaxOrder + 1] = {};

    std::mutex mu;                  // everything below
    std::condition_variable cv_submit, cv_ready, cv_mem, cv_retire, cv_done;
    std::deque<ReqP> submit_q, ready_q, retire_q;
    std::map<int64_t, ReqP> reqs;
    std::vector<int> free_pos;
    int64_t next_id = 1;
    bool stop = false;
    std::string fatal;
    dgtd_server_stats st{};

    std::thread th_admit, th_engine, th_retire;

    double now() const
    {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
    }
};

namespace {

int sfail(int code, const std::string& msg) { return dgtd::set_last_error(code, msg); }

using namespace dgtd::serve;

// Mark a request failed (caller holds s->mu).
void fail_locked(dgtd_server* s, const ReqP& r, int code, const std::string& msg)
{
    if (r->status == DGTD_REQ_DONE || r->status == DGTD_REQ_FAILED) return;
    r->status = DGTD_REQ_FAILED;
    r->err_code = code;
    r->err = msg;
    r->t_done = s->now();
    ++s->st.failed;
    s->cv_done.notify_all();
}

// Device error in the engine or retirement path: fail every request, stop.
void fatal_locked(dgtd_server* s, const std::string& msg)
{
    if (s->fatal.empty()) s->fatal = msg;
    s->stop = true;
    for (auto& kv : s->reqs) fail_locked(s, kv.second, DGTD_ERR_CUDA, "server stopped after a device error: " + msg);
    s->cv_submit.notify_all();
    s->cv_ready.notify_all();
    s->cv_mem.notify_all();
    s->cv_retire.notify_all();
}

// Host image of [0, lay.y0) of a request's region; real tables in R.
template <typename R>
std::vector<char> region_image(const Req& r, const dgtd::MeshTables& tab)
{
    const Layout& L = r.lay;
    std::vector<char> img(static_cast<size_t>(L.y0), 0);
    auto put = [&](int64_t off, const void* src, size_t bytes) {
        if (bytes) std::memcpy(img.data() + off, src, bytes);
    };
    auto put_real = [&](int64_t off, const double* src, size_t n) {
        R* dst = reinterpret_cast<R*>(img.data() + off);
        for (size_t i = 0; i < n; ++i) dst[i] = static_cast<R>(src[i]);
    };
    put_real(L.geo, tab.geo.data(), tab.geo.size());
    put_real(L.fgeo, tab.fgeo.data(), tab.fgeo.size());
    put_real(L.mat, tab.mat.data(), tab.mat.size());
    put(L.vmap, tab.vmapP.data(), tab.vmapP.size() * sizeof(int32_t));
    put(L.fcode, tab.fcode.data(), tab.fcode.size() * sizeof(int32_t));
    const size_t N = static_cast<size_t>(r.K) * r.Np;
    put_real(L.xyz, tab.x.data(), N);
    put_real(L.xyz + static_cast<int64_t>(N * sizeof(R)), tab.y.data(), N);
    put_real(L.xyz + static_cast<int64_t>(2 * N * sizeof(R)), tab.z.data(), N);
    put(L.tfsf, tab.tfsf_elems.data(), tab.tfsf_elems.size() * sizeof(int32_t));
    put(L.pw, r.waves.data(), r.waves.size() * sizeof(dgtd::PlaneWaveDev));
    if (!r.init.empty()) put_real(L.x, r.init.data(), r.init.size());
    return img;
}

void admission_loop(dgtd_server* s)
{
    cudaSetDevice(s->opts.device);
    for (;;) {
        ReqP r;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv_submit.wait(lk, [&] { return s->stop || !s->submit_q.empty(); });
            if (s->stop) return;
            r = s->submit_q.front();
            s->submit_q.pop_front();
        }
        try {
            const OrderTables& O = s->ord[r->order];
            dgtd::MeshTables tab = dgtd::build_tables(r->mesh, O.ref);
            r->mesh = dgtd::MeshInput();   // tables built; the raw mesh is no longer needed
            r->K = tab.K;
            r->Np = O.ref.Np;
            r->Nfp = O.ref.Nfp;
            r->n_tfsf = static_cast<int64_t>(tab.tfsf_elems.size());
            r->lay = layout(r->K, r->Np, r->Nfp, r->n_tfsf, s->fp32 ? 4 : 8);
            if (r->waves.size() == 1)
                r->skip_bound = dgtd::TfsfSkipBound(tab.x, tab.y, tab.z, tab.tfsf_elems, r->Np, r->waves[0]);
            if (!r->init.empty() && static_cast<int64_t>(r->init.size()) != 6 * r->K * r->Np)
                throw ServeError(DGTD_ERR_INVALID, "initial state has the wrong length for this mesh and order");
            if (!(r->dt > 0.0)) {
                // reference 3D Global estimator (Solver.cpp:289-300, 349-351), as dgtd_op_estimate_dt
                auto g = dgtd::gauss_lobatto(r->order);
                const double rmin = std::fabs(g[1] - g[0]);
                r->dt = tab.dt_scale_min * rmin * 2.0 / 3.0 * 0.75 * r->cfl / 0.8;
            }
            std::vector<char> img = s->fp32 ? region_image<float>(*r, tab) : region_image<double>(*r, tab);
            int64_t off = -1;
            {
                std::unique_lock<std::mutex> lk(s->mu);
                if (r->lay.total > s->arena.capacity())
                    throw ServeError(DGTD_ERR_NOMEM, "request needs " + std::to_string(r->lay.total) +
                                                         " device bytes, more than the server's whole budget of " +
                                                         std::to_string(s->arena.capacity()));
                for (;;) {
                    if (s->stop) return;
                    off = s->arena.alloc(r->lay.total);
                    if (off >= 0) break;
                    s->cv_mem.wait(lk);
                }
                s->st.bytes_in_use = s->arena.in_use();
                s->st.peak_bytes_in_use = std::max(s->st.peak_bytes_in_use, s->st.bytes_in_use);
            }
            r->off = off;
            ck(cudaMemcpyAsync(s->arena_base + off, img.data(), img.size(), cudaMemcpyHostToDevice, s->adm_stream),
               "request upload");
            ck(cudaStreamSynchronize(s->adm_stream), "request upload");
            std::lock_guard<std::mutex> lk(s->mu);
            r->t_admit = s->now();
            --s->st.queued;
            s->ready_q.push_back(r);
            s->cv_ready.notify_all();
        } catch (const ServeError& e) {
            std::lock_guard<std::mutex> lk(s->mu);
            if (r->off >= 0) { s->arena.release(r->off); r->off = -1; s->cv_mem.notify_all(); }
            --s->st.queued;
            fail_locked(s, r, e.code, e.what());
            if (e.code == DGTD_ERR_CUDA) { fatal_locked(s, e.what()); return; }
        } catch (const std::exception& e) {
            std::lock_guard<std::mutex> lk(s->mu);
            if (r->off >= 0) { s->arena.release(r->off); r->off = -1; s->cv_mem.notify_all(); }
            --s->st.queued;
            fail_locked(s, r, DGTD_ERR_INVALID, std::string("request rejected: ") + e.what());
        }
    }
}

bool running(const Req& r) { return r.t <= r.T - 1e-8 * r.dt; }

void engine_loop(dgtd_server* s)
{
    cudaSetDevice(s->opts.device);
    std::vector<ReqP> active;
    int round = 0;
    bool used[kMaxOrder + 1] = {};
    bool prev_used[kMaxOrder + 1] = {};
    auto params = std::make_unique<LaunchParam>();
    try {
        for (;;) {
            {
                std::unique_lock<std::mutex> lk(s->mu);
                auto can_admit = [&] {
                    return !s->ready_q.empty() && !s->free_pos.empty() &&
                           static_cast<int>(active.size()) < s->opts.max_active;
                };
                // idle: sleep until a request is uploaded and a slot is free (retirement frees slots)
                if (active.empty()) s->cv_ready.wait(lk, [&] { return s->stop || can_admit(); });
                if (s->stop) break;
                while (can_admit()) {
                    ReqP r = s->ready_q.front();
                    s->ready_q.pop_front();
                    r->pos = s->free_pos.back();
                    s->free_pos.pop_back();
                    r->t = r->t0;
                    r->status = DGTD_REQ_ACTIVE;
                    active.push_back(r);
                }
                s->st.active = static_cast<int64_t>(active.size());
                s->st.max_active_seen = std::max(s->st.max_active_seen, s->st.active);
            }
            // requests with nothing to do (final time already reached) retire at once
            for (int o = 0; o <= kMaxOrder; ++o) used[o] = false;
            for (int o = 1; o <= kMaxOrder; ++o) {
                std::vector<ReqP> grp;
                for (auto& r : active)
                    if (r->order == o) grp.push_back(r);
                if (grp.empty()) continue;
                cudaStream_t st = s->ord_stream[o];
                const OrderTables& O = s->ord[o];
                const int epb = elements_per_block(o, s->fp32);
                for (int k = 0; k < s->opts.steps_per_round; ++k) {
                    LaunchParam& L = *params;
                    L.DrT = O.DrT; L.DsT = O.DsT; L.DtT = O.DtT; L.LIFTT = O.LIFTT; L.Fmask = O.Fmask;
                    L.skip = s->skip;
                    L.n = 0;
                    int64_t blocks = 0;
                    bool any_src = false;
                    std::vector<Req*> in_launch;
                    for (auto& r : grp) {
                        if (!running(*r)) continue;
                        SlotParam& S = L.s[L.n++];
                        S.base = s->arena_base + r->off;
                        S.K = r->K;
                        S.block0 = blocks;
                        S.n_tfsf = r->n_tfsf;
                        S.t = r->t;
                        S.dt = std::min(r->dt, r->T - r->t);
                        S.alpha = r->alpha;
                        S.n_pw = static_cast<int32_t>(r->waves.size());
                        S.pos = r->pos;
                        any_src = any_src || (S.n_pw > 0 && S.n_tfsf > 0);
                        blocks += (r->K + epb - 1) / epb;
                        in_launch.push_back(r.get());
                    }
                    if (L.n == 0) break;
                    const int modes[4] = {dgtd::MODE_RK4_1, dgtd::MODE_RK4_2, dgtd::MODE_RK4_3, dgtd::MODE_RK4_4};
                    const double cs[4] = {0.0, 0.5, 0.5, 1.0};
                    for (int q = 0; q < 4; ++q) {
                        L.mode = modes[q];
                        L.c = cs[q];
                        bool any_device_test = false;
                        for (int i = 0; i < L.n; ++i) {
                            SlotParam& S = L.s[i];
                            S.skip_known = (S.n_pw > 0 && S.n_tfsf > 0) ? in_launch[i]->skip_bound.decide(S.t + cs[q] * S.dt) : 0;
                            any_device_test = any_device_test || (S.n_pw > 0 && S.n_tfsf > 0 && S.skip_known < 0);
                        }
                        ck(launch_stage(s->fp32, o, L, blocks, any_src && any_device_test, st), "serving stage kernel");
                    }
                    used[o] = true;
                    const double tnow = s->now();
                    std::lock_guard<std::mutex> lk(s->mu);
                    s->st.stage_launches += 4;
                    s->st.slot_stage_updates += 4 * static_cast<int64_t>(L.n);
                    for (int i = 0; i < L.n; ++i) {
                        Req* r = in_launch[i];
                        if (!r->launched) { r->launched = true; r->t_first = tnow; }
                        r->t += L.s[i].dt;
                        ++r->steps;
                        s->st.dof_updates += 6 * r->K * r->Np;
                    }
                }
                // finished requests: record their last kernel and hand them to retirement
                for (auto& r : grp) {
                    if (running(*r)) continue;
                    ck(cudaEventCreateWithFlags(&r->ev_last, cudaEventDisableTiming), "event");
                    ck(cudaEventRecord(r->ev_last, st), "event record");
                    std::lock_guard<std::mutex> lk(s->mu);
                    s->retire_q.push_back(r);
                    s->cv_retire.notify_all();
                }
            }
            active.erase(std::remove_if(active.begin(), active.end(), [](const ReqP& r) { return !running(*r); }),
                         active.end());
            // at most two rounds in flight: wait for the round before this one
            const int cur = round & 1, prv = cur ^ 1;
            for (int o = 1; o <= kMaxOrder; ++o)
                if (used[o]) ck(cudaEventRecord(s->round_ev[cur][o], s->ord_stream[o]), "round event");
            for (int o = 1; o <= kMaxOrder; ++o)
                if (prev_used[o]) ck(cudaEventSynchronize(s->round_ev[prv][o]), "round wait");
            for (int o = 0; o <= kMaxOrder; ++o) prev_used[o] = used[o];
            ++round;
        }
    } catch (const std::exception& e) {
        std::lock_guard<std::mutex> lk(s->mu);
        fatal_locked(s, e.what());
    }
}

void retire_loop(dgtd_server* s)
{
    cudaSetDevice(s->opts.device);
    for (;;) {
        ReqP r;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv_retire.wait(lk, [&] { return s->stop || !s->retire_q.empty(); });
            if (s->retire_q.empty()) return;   // stopping
            r = s->retire_q.front();
            s->retire_q.pop_front();
        }
        try {
            ck(cudaEventSynchronize(r->ev_last), "last kernel of a request");
            const size_t n = static_cast<size_t>(6 * r->K * r->Np);
            r->result.resize(n);
            if (s->fp32) {
                std::vector<float> f(n);
                ck(cudaMemcpyAsync(f.data(), s->arena_base + r->off + r->lay.x, n * sizeof(float),
                                   cudaMemcpyDeviceToHost, s->ret_stream),
                   "result download");
                ck(cudaStreamSynchronize(s->ret_stream), "result download");
                for (size_t i = 0; i < n; ++i) r->result[i] = f[i];
            } else {
                ck(cudaMemcpyAsync(r->result.data(), s->arena_base + r->off + r->lay.x, n * sizeof(double),
                                   cudaMemcpyDeviceToHost, s->ret_stream),
                   "result download");
                ck(cudaStreamSynchronize(s->ret_stream), "result download");
            }
            cudaEventDestroy(r->ev_last);
            r->ev_last = nullptr;
            // instability detector of the run loop (reference Solver::run, Solver.cpp:500-516)
            // on the downloaded final state: a norm that is not finite or above 1e20
            {
                double s2 = 0.0;
                for (size_t i = 0; i < n; ++i) s2 += r->result[i] * r->result[i];
                const double nrm = std::sqrt(s2);
                if (!(nrm <= kUnstableNormHost)) {
                    r->unstable = 1;
                    std::fprintf(stderr, "dgtd_gb300: WARNING: request %lld is potentially unstable (field norm = %g "
                                 "at t = %g, dt %g); verify the setup and consider a smaller time step\n",
                                 static_cast<long long>(r->id), nrm, r->T, r->dt);
                }
            }
            std::lock_guard<std::mutex> lk(s->mu);
            s->arena.release(r->off);
            r->off = -1;
            s->free_pos.push_back(r->pos);
            r->pos = -1;
            s->st.bytes_in_use = s->arena.in_use();
            if (r->status != DGTD_REQ_FAILED) {
                r->status = DGTD_REQ_DONE;
                r->t_done = s->now();
                ++s->st.completed;
            }
            s->cv_mem.notify_all();
            s->cv_ready.notify_all();
            s->cv_done.notify_all();
        } catch (const std::exception& e) {
            std::lock_guard<std::mutex> lk(s->mu);
            fatal_locked(s, e.what());
            return;
        }
    }
}

void fill_stats(const Req& r, dgtd_request_stats* o)
{
    std::memset(o, 0, sizeof(*o));
    o->status = r.status;
    o->order = r.order;
    o->n_elements = r.K;
    o->state_len = 6 * r.K * r.Np;
    o->steps = r.steps;
    o->region_bytes = r.lay.total;
    o->dt = r.dt;
    o->t_submit = r.t_submit;
    o->t_admit = r.t_admit;
    o->t_first_launch = r.t_first;
    o->t_done = r.t_done;
    o->unstable = r.unstable;
}

void destroy_server(dgtd_server* s)
{
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        s->cv_submit.notify_all();
        s->cv_ready.notify_all();
        s->cv_mem.notify_all();
        s->cv_retire.notify_all();
    }
    if (s->th_admit.joinable()) s->th_admit.join();
    if (s->th_engine.joinable()) s->th_engine.join();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->cv_retire.notify_all();
    }
    if (s->th_retire.joinable()) s->th_retire.join();
    cudaSetDevice(s->opts.device);
    for (int o = 1; o <= kMaxOrder; ++o)
        if (s->ord_stream[o]) cudaStreamSynchronize(s->ord_stream[o]);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        for (auto& kv : s->reqs) {
            if (kv.second->ev_last) { cudaEventDestroy(kv.second->ev_last); kv.second->ev_last = nullptr; }
            fail_locked(s, kv.second, DGTD_ERR_CUDA, "server destroyed before the request finished");
        }
    }
    for (int o = 1; o <= kMaxOrder; ++o) {
        OrderTables& O = s->ord[o];
        cudaFree(O.DrT); cudaFree(O.DsT); cudaFree(O.DtT); cudaFree(O.LIFTT); cudaFree(O.Fmask);
        if (s->ord_stream[o]) cudaStreamDestroy(s->ord_stream[o]);
        for (int k = 0; k < 2; ++k)
            if (s->round_ev[k][o]) cudaEventDestroy(s->round_ev[k][o]);
    }
    if (s->adm_stream) cudaStreamDestroy(s->adm_stream);
    if (s->ret_stream) cudaStreamDestroy(s->ret_stream);
    cudaFree(s->skip);
    cudaFree(s->arena_base);
    delete s;
}

template <typename T>
T* dev_upload(const std::vector<T>& v)
{
    T* d = nullptr;
    ck(cudaMalloc(&d, v.size() * sizeof(T)), "cudaMalloc");
    ck(cudaMemcpy(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice), "H2D");
    return d;
}

}  // namespace

extern "C" {

int dgtd_server_create(const dgtd_server_opts* opts, dgtd_server** out)
{
    if (!opts || !out) return sfail(DGTD_ERR_INVALID, "NULL argument");
    *out = nullptr;
    if (opts->memory_budget <= 0) return sfail(DGTD_ERR_INVALID, "memory_budget must be positive");
    if (opts->max_active < 1 || opts->max_active > kMaxSlots)
        return sfail(DGTD_ERR_INVALID, "max_active must be in [1, " + std::to_string(kMaxSlots) + "]");
    if (opts->steps_per_round < 1) return sfail(DGTD_ERR_INVALID, "steps_per_round must be >= 1");
    if (opts->precision != DGTD_FP64 && opts->precision != DGTD_FP32)
        return sfail(DGTD_ERR_INVALID, "server precision must be DGTD_FP64 or DGTD_FP32");
    dgtd_server* s = new dgtd_server();
    s->opts = *opts;
    s->fp32 = opts->precision == DGTD_FP32;
    s->t_start = std::chrono::steady_clock::now();
    try {
        ck(cudaSetDevice(opts->device), "cudaSetDevice");
        cudaError_t e = cudaMalloc(&s->arena_base, static_cast<size_t>(opts->memory_budget));
        if (e != cudaSuccess) {
            cudaGetLastError();
            s->arena_base = nullptr;
            throw ServeError(DGTD_ERR_NOMEM, std::string("cannot allocate the memory budget: ") + cudaGetErrorString(e));
        }
        s->arena.reset(opts->memory_budget, kAlign);
        ck(cudaMalloc(&s->skip, kMaxSlots * sizeof(int)), "cudaMalloc");
        ck(cudaMemset(s->skip, 0, kMaxSlots * sizeof(int)), "cudaMemset");
        for (int o = 1; o <= kMaxOrder; ++o) {
            OrderTables& O = s->ord[o];
            O.ref = dgtd::build_ref_tet(o);
            const int Np = O.ref.Np, NF = 4 * O.ref.Nfp;
            auto up_real = [&](const std::vector<double>& v) -> void* {
                if (s->fp32) return dev_upload(std::vector<float>(v.begin(), v.end()));
                return dev_upload(v);
            };
            O.DrT = up_real(transposed(O.ref.Dr, Np, Np));
            O.DsT = up_real(transposed(O.ref.Ds, Np, Np));
            O.DtT = up_real(transposed(O.ref.Dt, Np, Np));
            O.LIFTT = up_real(transposed(O.ref.LIFT, Np, NF));
            O.Fmask = dev_upload(O.ref.Fmask);
            ck(cudaStreamCreateWithFlags(&s->ord_stream[o], cudaStreamNonBlocking), "stream");
            for (int k = 0; k < 2; ++k) ck(cudaEventCreateWithFlags(&s->round_ev[k][o], cudaEventDisableTiming), "event");
        }
        ck(cudaStreamCreateWithFlags(&s->adm_stream, cudaStreamNonBlocking), "stream");
        ck(cudaStreamCreateWithFlags(&s->ret_stream, cudaStreamNonBlocking), "stream");
        for (int p = opts->max_active - 1; p >= 0; --p) s->free_pos.push_back(p);
        s->st.memory_budget = opts->memory_budget;
        s->th_admit = std::thread(admission_loop, s);
        s->th_engine = std::thread(engine_loop, s);
        s->th_retire = std::thread(retire_loop, s);
    } catch (const ServeError& e) {
        destroy_server(s);
        return sfail(e.code, e.what());
    } catch (const std::exception& e) {
        destroy_server(s);
        return sfail(DGTD_ERR_CUDA, e.what());
    }
    *out = s;
    return DGTD_OK;
}

void dgtd_server_destroy(dgtd_server* s)
{
    if (s) destroy_server(s);
}

int dgtd_server_submit(dgtd_server* s, const dgtd_request* q, int64_t* id_out)
{
    if (!s || !q || !id_out) return sfail(DGTD_ERR_INVALID, "NULL argument");
    const dgtd_mesh_desc* m = q->mesh;
    if (!m || m->dim != 3 || m->n_vertices <= 0 || !m->vertices || m->n_elements <= 0 || !m->elements)
        return sfail(DGTD_ERR_INVALID, "request mesh is missing or not a 3D tetrahedral mesh");
    if (q->order < 1 || q->order > kMaxOrder) return sfail(DGTD_ERR_UNSUPPORTED, "order must be in [1, 6]");
    if (q->n_waves < 0 || q->n_waves > kMaxWaves || (q->n_waves > 0 && !q->waves))
        return sfail(DGTD_ERR_INVALID, "a request takes 0.." + std::to_string(kMaxWaves) + " plane waves");
    if (!(q->final_time >= q->t0)) return sfail(DGTD_ERR_INVALID, "final_time must be >= t0");
    if (!(q->dt > 0.0) && !(q->cfl > 0.0)) return sfail(DGTD_ERR_INVALID, "give dt > 0 or cfl > 0");
    if (!(q->alpha >= 0.0)) return sfail(DGTD_ERR_INVALID, "alpha must be >= 0");
    auto r = std::make_shared<Req>();
    try {
        dgtd::MeshInput& in = r->mesh;
        in.dim = 3;
        in.vertices.assign(m->vertices, m->vertices + 3 * m->n_vertices);
        in.elements.assign(m->elements, m->elements + 4 * m->n_elements);
        if (m->eps_r) in.eps.assign(m->eps_r, m->eps_r + m->n_elements);
        if (m->mu_r) in.mu.assign(m->mu_r, m->mu_r + m->n_elements);
        if (m->sigma) in.sigma.assign(m->sigma, m->sigma + m->n_elements);
        if (m->n_bdr_faces > 0) {
            if (!m->bdr_faces || !m->bdr_codes) return sfail(DGTD_ERR_INVALID, "boundary faces without arrays");
            in.bdr_faces.assign(m->bdr_faces, m->bdr_faces + 3 * m->n_bdr_faces);
            in.bdr_codes.assign(m->bdr_codes, m->bdr_codes + m->n_bdr_faces);
        }
        if (m->n_tfsf_faces > 0) {
            if (!m->tfsf_faces) return sfail(DGTD_ERR_INVALID, "TF/SF faces without array");
            in.tfsf_faces.assign(m->tfsf_faces, m->tfsf_faces + 3 * m->n_tfsf_faces);
        }
        if (m->n_int_faces > 0) {
            if (!m->int_faces || !m->int_codes) return sfail(DGTD_ERR_INVALID, "interior faces without arrays");
            in.int_faces.assign(m->int_faces, m->int_faces + 3 * m->n_int_faces);
            in.int_codes.assign(m->int_codes, m->int_codes + m->n_int_faces);
            for (int32_t c : in.int_codes)
                if (c == DGTD_BC_SGBC)
                    return sfail(DGTD_ERR_UNSUPPORTED, "served requests do not take thin-layer (SGBC) faces");
        }
        if (m->n_curved != 0) return sfail(DGTD_ERR_UNSUPPORTED, "served requests do not take curved elements");
        for (int i = 0; i < q->n_waves; ++i) {
            const dgtd_planewave& w = q->waves[i];
            if (w.batch != 0) return sfail(DGTD_ERR_INVALID, "a served request is one incidence: wave batch must be 0");
            if (!(w.spread > 0.0)) return sfail(DGTD_ERR_INVALID, "source spread must be positive");
            const double kn = std::sqrt(w.propagation[0] * w.propagation[0] + w.propagation[1] * w.propagation[1] +
                                        w.propagation[2] * w.propagation[2]);
            const double pn = std::sqrt(w.polarization[0] * w.polarization[0] + w.polarization[1] * w.polarization[1] +
                                        w.polarization[2] * w.polarization[2]);
            if (!(kn > 0.0) || !(pn > 0.0)) return sfail(DGTD_ERR_INVALID, "zero propagation or polarization");
            dgtd::PlaneWaveDev d{};
            for (int c = 0; c < 3; ++c) { d.k[c] = w.propagation[c] / kn; d.pol[c] = w.polarization[c] / pn; }
            d.kxp[0] = d.k[1] * d.pol[2] - d.k[2] * d.pol[1];
            d.kxp[1] = d.k[2] * d.pol[0] - d.k[0] * d.pol[2];
            d.kxp[2] = d.k[0] * d.pol[1] - d.k[1] * d.pol[0];
            d.spread = w.spread;
            d.mean = w.mean;
            d.freq = w.frequency;
            d.batch = 0;
            r->waves.push_back(d);
        }
        r->order = q->order;
        r->K = m->n_elements;
        r->Np = dgtd::tet_np(q->order);
        r->alpha = q->alpha;
        r->t0 = q->t0;
        r->T = q->final_time;
        r->dt = q->dt > 0.0 ? q->dt : 0.0;
        r->cfl = q->cfl;
        if (q->h_init) {
            const int Np = dgtd::tet_np(q->order);
            r->init.assign(q->h_init, q->h_init + 6 * m->n_elements * static_cast<int64_t>(Np));
        }
    } catch (const std::bad_alloc&) {
        return sfail(DGTD_ERR_NOMEM, "host allocation failed");
    }
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) return sfail(DGTD_ERR_CUDA, s->fatal.empty() ? "server is stopping" : "server stopped: " + s->fatal);
    r->id = s->next_id++;
    r->t_submit = s->now();
    s->reqs[r->id] = r;
    s->submit_q.push_back(r);
    ++s->st.submitted;
    ++s->st.queued;
    s->cv_submit.notify_all();
    *id_out = r->id;
    return DGTD_OK;
}

int dgtd_server_wait(dgtd_server* s, int64_t id, double timeout_s, double* h_state, dgtd_request_stats* stats)
{
    if (!s) return sfail(DGTD_ERR_INVALID, "NULL server");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return sfail(DGTD_ERR_INVALID, "unknown request id " + std::to_string(id));
    ReqP r = it->second;
    auto done = [&] { return r->status == DGTD_REQ_DONE || r->status == DGTD_REQ_FAILED; };
    if (timeout_s < 0) {
        s->cv_done.wait(lk, done);
    } else if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), done)) {
        return sfail(DGTD_ERR_TIMEOUT, "request " + std::to_string(id) + " not finished within the timeout");
    }
    if (stats) fill_stats(*r, stats);
    s->reqs.erase(id);
    if (r->status == DGTD_REQ_FAILED) return sfail(r->err_code ? r->err_code : DGTD_ERR_CUDA, r->err);
    if (h_state && !r->result.empty()) std::memcpy(h_state, r->result.data(), r->result.size() * sizeof(double));
    return DGTD_OK;
}

int dgtd_server_query(dgtd_server* s, int64_t id, dgtd_request_stats* stats)
{
    if (!s || !stats) return sfail(DGTD_ERR_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return sfail(DGTD_ERR_INVALID, "unknown request id " + std::to_string(id));
    fill_stats(*it->second, stats);
    return DGTD_OK;
}

int dgtd_server_get_stats(dgtd_server* s, dgtd_server_stats* out)
{
    if (!s || !out) return sfail(DGTD_ERR_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->st;
    if (!s->fatal.empty()) return sfail(DGTD_ERR_CUDA, s->fatal);
    return DGTD_OK;
}

int dgtd_arena_create(int64_t capacity, int64_t align, dgtd_arena** out)
{
    if (!out) return sfail(DGTD_ERR_INVALID, "NULL argument");
    *out = nullptr;
    try {
        auto* a = new dgtd::RangeAllocator(capacity, align);
        *out = reinterpret_cast<dgtd_arena*>(a);
    } catch (const std::exception& e) {
        return sfail(DGTD_ERR_INVALID, e.what());
    }
    return DGTD_OK;
}

void dgtd_arena_destroy(dgtd_arena* a) { delete reinterpret_cast<dgtd::RangeAllocator*>(a); }

int64_t dgtd_arena_alloc(dgtd_arena* a, int64_t bytes)
{
    if (!a) return -1;
    return reinterpret_cast<dgtd::RangeAllocator*>(a)->alloc(bytes);
}

int dgtd_arena_release(dgtd_arena* a, int64_t offset)
{
    if (!a) return sfail(DGTD_ERR_INVALID, "NULL arena");
    return reinterpret_cast<dgtd::RangeAllocator*>(a)->release(offset) ? DGTD_OK
                                                                       : sfail(DGTD_ERR_INVALID, "not an allocated range");
}

int dgtd_arena_usage(const dgtd_arena* a, int64_t* in_use, int64_t* largest_free, int64_t* n_free)
{
    if (!a) return sfail(DGTD_ERR_INVALID, "NULL arena");
    const auto* r = reinterpret_cast<const dgtd::RangeAllocator*>(a);
    if (in_use) *in_use = r->in_use();
    if (largest_free) *largest_free = r->largest_free();
    if (n_free) *n_free = r->n_free_ranges();
    return DGTD_OK;
}

}  // extern "C"
