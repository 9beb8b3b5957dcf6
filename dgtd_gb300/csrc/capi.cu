// C ABI of the DG Maxwell step: operator life cycle, Mult, fused stepping.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "skipbound.hpp"

#include "../../include/dgtd_gb300.h"
#include "batched.hpp"
#include "kernels.hpp"
#include "mesh.hpp"
#include "probes.hpp"
#include "refelem.hpp"
#include "curved.hpp"
#include "curved_dev.hpp"
#include "sgbc_dev.hpp"
#include "single_tc.hpp"

namespace {

thread_local std::string g_err;
std::atomic<uint64_t> g_launches{0};   // kernels launched by this library (all threads)

// Skip flags a stage reads when the host has decided the TF/SF skip test.
__device__ const int kDecidedSkip[2] = {0, 1};

int fail(int code, const std::string& msg)
{
    g_err = msg;
    return code;
}

}  // namespace

namespace dgtd {
// Records the thread-local message dgtd_last_error() returns (also used by serve.cu).
int set_last_error(int code, const std::string& msg) { return fail(code, msg); }
}  // namespace dgtd

namespace {

struct CudaError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

void ck(cudaError_t e, const char* what)
{
    if (e != cudaSuccess) throw CudaError(std::string(what) + ": " + cudaGetErrorString(e));
}

template <typename T>
T* upload(const std::vector<T>& v, int64_t& bytes)
{
    if (v.empty()) return nullptr;
    T* d = nullptr;
    ck(cudaMalloc(&d, v.size() * sizeof(T)), "cudaMalloc");
    ck(cudaMemcpy(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice), "cudaMemcpy H2D");
    bytes += static_cast<int64_t>(v.size() * sizeof(T));
    return d;
}

// LSERK4 coefficients (Carpenter & Kennedy 1994, 5-stage, 4th order, 2N storage).
const double kRk4a[5] = {0.0, -567301805773.0 / 1357537059087.0, -2404267990393.0 / 2016746695238.0,
                         -3550918686646.0 / 2091501179385.0, -1275806237668.0 / 842570457699.0};
const double kRk4b[5] = {1432997174477.0 / 9575080441755.0, 5161836677717.0 / 13612068292357.0,
                         1720146321549.0 / 2090206949498.0, 3134564353537.0 / 4481467310338.0,
                         2277821191437.0 / 14882151754819.0};
const double kRk4c[5] = {0.0, 1432997174477.0 / 9575080441755.0, 2526269341429.0 / 6820363962896.0,
                         2006345519317.0 / 3224310063776.0, 2802321613138.0 / 2924317926251.0};

}  // namespace

struct dgtd_op {
    dgtd::RefTet ref;
    dgtd::MeshTables mesh;
    dgtd::TablesDev dev{};
    int batch = 1;
    int precision = DGTD_FP64;
    double alpha = 1.0;
    int64_t device_bytes = 0;
    int64_t state_len = 0;
    int64_t n_tfsf_faces = 0;
    std::vector<void*> allocs;
    // sources
    std::vector<dgtd::PlaneWaveDev> pw_host;
    dgtd::PlaneWaveDev* pw_dev = nullptr;
    int pw_cap = 0;
    int* skip_dev = nullptr;
    dgtd::SkipScratch skip_sc;          // split skip test: per-part sums and tickets
    dgtd::TfsfSkipBound skip_bound;     // one incidence, one plain wave: host bounds of the skip test
    const int* skip_const = nullptr;    // device flags {0, 1} a stage reads when the host decided
    double* norm_dev = nullptr;
    // instability detector of dgtd_op_run_host (reference Solver.cpp:500-516)
    dgtd::StabilityRecord* stab_dev = nullptr;
    int stab_every = 10;        // check every `stab_every` steps (0: off)
    int stab_stop = 0;          // 1: stop the run and return DGTD_ERR_UNSTABLE
    int n_sm = 152;
    // RK scratch (allocated on first dgtd_op_step)
    double* ws = nullptr;
    int64_t ws_len = 0;
    // change of nodal basis (dgtd_op_change_basis): [2][Np][Np], Gauss-Legendre -> Gauss-Lobatto
    // then back; allocated on first use, freed with `allocs`
    double* basis_dev = nullptr;
    // single-instance FP32 form: FP32 copies of the tables, RK scratch
    dgtd::TablesF32 dev32{};
    float* ws32 = nullptr;
    // single-instance FP32 form on the tensor cores: A-operand image, device error flag, and
    // the contraction path (0: tensor cores where supported, 1: FP32 SIMT)
    uint32_t* tc1_img = nullptr;
    int* tc1_status = nullptr;
    int contraction32 = 1;   // FP32 SIMT: 0.91 x the tensor-core stage's time at p = 6 on GB300
    // batched FP32 form
    std::unique_ptr<dgtd::BatchedOp> batched;
    // FP64 defect correction of the batched form: refresh period (steps, 0: off), steps since
    // the last refresh, the state buffer it was made from (nullptr: none valid), two scratch
    // buffers (each max(FP64 reference state, FP32 working state) bytes) and the bf16 term
    int defect_every = 0;
    int64_t defect_age = 0;
    const void* defect_state = nullptr;
    int64_t defect_refreshes = 0;
    void* defect_a = nullptr;
    void* defect_b = nullptr;
    uint16_t* defect_corr = nullptr;   // the applied correction c (bf16)
    float* defect_prev = nullptr;      // x_hi at the previous refresh (NaN: none)
    double* defect_sumsq = nullptr;    // per-incidence sum of squares of the state (refresh scratch)
    uint16_t* defect_inc = nullptr;    // c's classical-RK4 step increment for dt = defect_inc_dt (bf16)
    double defect_inc_dt = 0.0;
    bool defect_inc_stale = true;
    bool defect_prev_reset = true;     // clear defect_prev before the next refresh
    // point probes / DFT accumulators, sampled by dgtd_op_step every probes->every() steps
    std::unique_ptr<dgtd::ProbeSet> probes;
    int64_t probe_steps = 0;
    // thin-layer (SGBC) sub-solvers of the mesh's DGTD_BC_SGBC faces (dgtd_op_set_sgbc)
    std::unique_ptr<dgtd::SgbcOp> sgbc;
    // block rows of the mesh's curved (second-order) elements
    std::unique_ptr<dgtd::CurvedOp> curved;

    ~dgtd_op()
    {
        for (void* p : allocs) cudaFree(p);
        if (pw_dev) cudaFree(pw_dev);
        if (skip_dev) cudaFree(skip_dev);
        if (norm_dev) cudaFree(norm_dev);
        if (stab_dev) cudaFree(stab_dev);
        if (tc1_img) cudaFree(tc1_img);
        if (tc1_status) cudaFree(tc1_status);
        free_defect_buffers();
        if (ws) cudaFree(ws);
        if (ws32) cudaFree(ws32);
    }
    void free_defect_buffers()
    {
        if (defect_a) cudaFree(defect_a);
        if (defect_b) cudaFree(defect_b);
        if (defect_corr) cudaFree(defect_corr);
        if (defect_prev) cudaFree(defect_prev);
        if (defect_inc) cudaFree(defect_inc);
        if (defect_sumsq) cudaFree(defect_sumsq);
        defect_sumsq = nullptr;
        defect_a = defect_b = nullptr;
        defect_corr = defect_inc = nullptr;
        defect_prev = nullptr;
        defect_state = nullptr;
        defect_inc_stale = true;
    }
    template <typename T>
    T* up(const std::vector<T>& v)
    {
        T* d = upload(v, device_bytes);
        if (d) allocs.push_back(d);
        return d;
    }
};

namespace {

// Adds the batched form's kernel launches to the library-wide counter.
struct BatchedCount {
    dgtd_op* op;
    int64_t before;
    explicit BatchedCount(dgtd_op* o) : op(o), before(o->batched->kernel_launches()) {}
    ~BatchedCount() { g_launches.fetch_add(op->batched->kernel_launches() - before, std::memory_order_relaxed); }
};

// The reference-layout buffer of pack / unpack: device memory, or pinned host memory the device
// can address (the conversion kernel then reads or writes it over the host link, so the
// host-device transfer and the layout conversion are one pass). Anything else (pageable host
// memory) is rejected before a kernel could touch it.
const void* device_view(const void* p, bool* on_host = nullptr)
{
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        throw std::invalid_argument("pack/unpack: cannot query the reference-layout buffer");
    }
    if (on_host) *on_host = a.type == cudaMemoryTypeHost;
    if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) return p;
    if (a.type == cudaMemoryTypeHost && a.devicePointer != nullptr) return a.devicePointer;
    throw std::invalid_argument("pack/unpack: the reference-layout buffer must be device memory or pinned host "
                                "memory (pageable host memory is not addressable by the device)");
}

// Clears the instability record before a run (no check has tripped).
void reset_stability(dgtd_op* op)
{
    dgtd::StabilityRecord r{};
    r.first_step = -1;
    ck(cudaMemcpy(op->stab_dev, &r, sizeof(r), cudaMemcpyHostToDevice), "reset stability record");
}

dgtd::MeshInput to_input(const dgtd_mesh_desc* m)
{
    if (!m) throw std::invalid_argument("mesh descriptor is NULL");
    if (m->dim != 3) throw std::invalid_argument("only dim = 3 tetrahedral meshes are supported");
    if (m->n_vertices <= 0 || !m->vertices) throw std::invalid_argument("mesh has no vertices");
    if (m->n_elements <= 0 || !m->elements) throw std::invalid_argument("mesh has no elements");
    dgtd::MeshInput in;
    in.dim = 3;
    in.vertices.assign(m->vertices, m->vertices + 3 * m->n_vertices);
    in.elements.assign(m->elements, m->elements + 4 * m->n_elements);
    if (m->eps_r) in.eps.assign(m->eps_r, m->eps_r + m->n_elements);
    if (m->mu_r) in.mu.assign(m->mu_r, m->mu_r + m->n_elements);
    if (m->sigma) in.sigma.assign(m->sigma, m->sigma + m->n_elements);
    if (m->n_bdr_faces > 0) {
        if (!m->bdr_faces || !m->bdr_codes) throw std::invalid_argument("boundary faces without arrays");
        in.bdr_faces.assign(m->bdr_faces, m->bdr_faces + 3 * m->n_bdr_faces);
        in.bdr_codes.assign(m->bdr_codes, m->bdr_codes + m->n_bdr_faces);
    }
    if (m->n_tfsf_faces > 0) {
        if (!m->tfsf_faces) throw std::invalid_argument("TF/SF faces without array");
        in.tfsf_faces.assign(m->tfsf_faces, m->tfsf_faces + 3 * m->n_tfsf_faces);
    }
    if (m->n_int_faces > 0) {
        if (!m->int_faces || !m->int_codes) throw std::invalid_argument("interior faces without arrays");
        in.int_faces.assign(m->int_faces, m->int_faces + 3 * m->n_int_faces);
        in.int_codes.assign(m->int_codes, m->int_codes + m->n_int_faces);
    }
    if (m->n_curved < 0) throw std::invalid_argument("n_curved must be >= 0");
    if (m->n_curved > 0) {
        if (!m->curved_elems || !m->curved_nodes) throw std::invalid_argument("curved elements without arrays");
        in.curved_elems.assign(m->curved_elems, m->curved_elems + m->n_curved);
        in.curved_nodes.assign(m->curved_nodes, m->curved_nodes + 30 * m->n_curved);
    }
    return in;
}

std::vector<double> transpose(const std::vector<double>& a, int rows, int cols)
{
    std::vector<double> t(a.size());
    for (int i = 0; i < rows; ++i)
        for (int j = 0; j < cols; ++j) t[static_cast<size_t>(j) * rows + i] = a[static_cast<size_t>(i) * cols + j];
    return t;
}

void ensure_sources(dgtd_op* op)
{
    int n = static_cast<int>(op->pw_host.size());
    if (n > op->pw_cap) {
        if (op->pw_dev) cudaFree(op->pw_dev);
        op->pw_dev = nullptr;
        ck(cudaMalloc(&op->pw_dev, n * sizeof(dgtd::PlaneWaveDev)), "cudaMalloc sources");
        op->pw_cap = n;
    }
    if (n > 0)
        ck(cudaMemcpy(op->pw_dev, op->pw_host.data(), n * sizeof(dgtd::PlaneWaveDev), cudaMemcpyHostToDevice),
           "cudaMemcpy sources");
}

bool has_sources(const dgtd_op* op) { return op->mesh.tfsf_elems.size() > 0 && !op->pw_host.empty(); }

// One fused stage on the plain FP64 form (with the thin-layer coupling around it when the mesh
// has SGBC faces).
void run_stage(dgtd_op* op, dgtd::StageArgs A, double t, cudaStream_t s)
{
    A.t = t;
    A.batch = op->batch;
    if (!op->mesh.sgbc_faces.empty()) {
        if (!op->sgbc)
            throw std::invalid_argument("the mesh has thin-layer (SGBC) faces: give their stacks with dgtd_op_set_sgbc");
        const int64_t before = op->sgbc->launches();
        op->sgbc->before_stage(op->dev, A, t, s);
        g_launches.fetch_add(op->sgbc->launches() - before, std::memory_order_relaxed);
    }
    if (has_sources(op)) {
        const int known = op->skip_bound.decide(t);
        if (known < 0) {
            ck(dgtd::launch_tfsf_skip(op->dev, op->pw_dev, static_cast<int>(op->pw_host.size()), op->batch, t,
                                      op->skip_dev, op->skip_sc, s),
               "tfsf skip kernel");
            g_launches.fetch_add(1, std::memory_order_relaxed);
        }
        A.pw = op->pw_dev;
        A.n_pw = static_cast<int>(op->pw_host.size());
        A.skip = known < 0 ? op->skip_dev : op->skip_const + known;
    } else {
        A.pw = nullptr;
        A.n_pw = 0;
        A.skip = nullptr;
    }
    ck(dgtd::launch_stage_fp64(op->dev, A, s), "stage kernel");
    g_launches.fetch_add(1, std::memory_order_relaxed);
    if (op->curved) {
        op->curved->apply(op->dev, A, s);
        g_launches.fetch_add(1, std::memory_order_relaxed);
    }
    if (op->sgbc) {
        const int64_t before = op->sgbc->launches();
        op->sgbc->after_stage(op->dev, A, s);
        g_launches.fetch_add(op->sgbc->launches() - before, std::memory_order_relaxed);
    }
}

// FP64 defect correction of the batched form (dgtd_op_set_defect_correction): from the state in
// d_work at time t, c = L64(x) - L32(x_hi) in bf16, kept where the state has not moved since the
// previous refresh. Scratch a: x (reference layout, FP64), then L64(x) as a working state;
// scratch b: L64(x) (reference layout), then L32(x_hi). All on stream s, no host synchronisation.
void defect_refresh(dgtd_op* op, float* d_work, double t, cudaStream_t s)
{
    dgtd::BatchedOp& B = *op->batched;
    const int64_t L = B.state_len();
    if (!op->defect_a) {
        // all buffers or none: a failed allocation leaves the operator without any
        const size_t bytes = std::max(static_cast<size_t>(op->state_len) * sizeof(double),
                                      static_cast<size_t>(B.work_len()) * sizeof(float));
        try {
            ck(cudaMalloc(&op->defect_a, bytes), "cudaMalloc defect-correction scratch");
            ck(cudaMalloc(&op->defect_b, bytes), "cudaMalloc defect-correction scratch");
            ck(cudaMalloc(&op->defect_corr, static_cast<size_t>(L) * sizeof(uint16_t)), "cudaMalloc defect correction");
            ck(cudaMalloc(&op->defect_inc, static_cast<size_t>(L) * sizeof(uint16_t)), "cudaMalloc defect correction");
            ck(cudaMalloc(&op->defect_prev, static_cast<size_t>(L) * sizeof(float)), "cudaMalloc defect correction");
            ck(cudaMalloc(&op->defect_sumsq, static_cast<size_t>(B.batch_padded()) * sizeof(double)),
               "cudaMalloc defect correction");
        } catch (...) {
            op->free_defect_buffers();
            throw;
        }
        op->defect_prev_reset = true;
    }
    if (op->defect_prev_reset) {   // no earlier state to compare with: NaN never matches
        ck(cudaMemsetAsync(op->defect_prev, 0xff, static_cast<size_t>(L) * sizeof(float), s), "memset");
        op->defect_prev_reset = false;
    }
    double* x64 = static_cast<double*>(op->defect_a);
    double* l64 = static_cast<double*>(op->defect_b);
    B.unpack(d_work, x64, s);
    dgtd::StageArgs A{};
    A.mode = dgtd::MODE_MULT;
    A.in = x64;
    A.out = l64;
    run_stage(op, A, t, s);
    float* l64w = static_cast<float*>(op->defect_a);
    float* l32 = static_cast<float*>(op->defect_b);
    B.pack(l64, l64w, s);
    B.mult(d_work, l32, t, s);
    B.build_correction(l64w, l32, d_work, op->defect_prev, op->defect_sumsq, op->defect_corr, s);
    op->defect_state = d_work;
    op->defect_age = 0;
    op->defect_inc_stale = true;
    ++op->defect_refreshes;
}

// A new trajectory: refresh at the next step, with no earlier state to compare with (the
// previous-state buffer is reset on the refresh's own stream).
void defect_restart(dgtd_op* op)
{
    op->defect_state = nullptr;
    op->defect_age = 0;
    op->defect_prev_reset = true;
}

// nsteps steps of the batched form; with the defect correction on, one step at a time, each
// followed by the correction's increment, and the correction refreshed on its schedule
void batched_steps(dgtd_op* op, float* d_work, double t, double dt, int nsteps, int integrator, cudaStream_t s)
{
    dgtd::BatchedOp& B = *op->batched;
    if (op->defect_every <= 0) {
        B.step(d_work, t, dt, nsteps, integrator, s);
        return;
    }
    if (integrator != DGTD_RK4)
        throw std::invalid_argument("the defect correction is implemented for classical RK4 (DGTD_RK4)");
    for (int i = 0; i < nsteps; ++i) {
        if (op->defect_state != d_work || op->defect_age >= op->defect_every) defect_refresh(op, d_work, t, s);
        if (op->defect_inc_stale || op->defect_inc_dt != dt) {
            B.build_increment(op->defect_corr, static_cast<float*>(op->defect_a), static_cast<float*>(op->defect_b),
                              op->defect_inc, dt, s);
            op->defect_inc_dt = dt;
            op->defect_inc_stale = false;
        }
        B.step(d_work, t, dt, 1, integrator, s);
        B.add_increment(d_work, op->defect_inc, s);
        t += dt;
        ++op->defect_age;
    }
}

void ensure_ws(dgtd_op* op)
{
    int64_t need = 3 * op->state_len;
    if (op->ws_len >= need) return;
    if (op->ws) cudaFree(op->ws);
    op->ws = nullptr;
    op->ws_len = 0;
    ck(cudaMalloc(&op->ws, need * sizeof(double)), "cudaMalloc RK scratch");
    op->ws_len = need;
}

// One RK step of size dt at time t on d_x (device) using the op's scratch.
void rk_step(dgtd_op* op, double* d_x, double t, double dt, int integrator, double* lsrk_other, double*& cur,
             cudaStream_t s)
{
    const int64_t L = op->state_len;
    if (integrator == DGTD_RK4) {
        double* y0 = op->ws;
        double* y1 = op->ws + L;
        double* z = op->ws + 2 * L;
        dgtd::StageArgs A{};
        A.dt = dt;
        A.x = d_x;
        A.z = z;
        A.mode = dgtd::MODE_RK4_1; A.in = d_x; A.yout = y0; run_stage(op, A, t, s);
        A.mode = dgtd::MODE_RK4_2; A.in = y0; A.yout = y1; run_stage(op, A, t + dt / 2, s);
        A.mode = dgtd::MODE_RK4_3; A.in = y1; A.yout = y0; run_stage(op, A, t + dt / 2, s);
        A.mode = dgtd::MODE_RK4_4; A.in = y0; A.yout = nullptr; run_stage(op, A, t + dt, s);
    } else {
        double* res = op->ws + 2 * L;
        for (int st = 0; st < 5; ++st) {
            double* nxt = (cur == d_x) ? lsrk_other : d_x;
            dgtd::StageArgs A{};
            A.dt = dt;
            A.mode = dgtd::MODE_LSRK;
            A.in = cur;
            A.yout = nxt;
            A.res = res;
            A.a = kRk4a[st];
            A.b = kRk4b[st];
            run_stage(op, A, t + kRk4c[st] * dt, s);
            cur = nxt;
        }
    }
}

// ---- single-instance FP32 form: the same stage sequence on FP32 registers
bool uses_tc1(const dgtd_op* op) { return op->tc1_img != nullptr && op->contraction32 == 0; }

void run_stage32(dgtd_op* op, dgtd::StageArgsF32 A, double t, cudaStream_t s)
{
    A.t = t;
    A.batch = op->batch;
    if (has_sources(op)) {
        const int known = op->skip_bound.decide(t);
        if (known < 0) {
            ck(dgtd::launch_tfsf_skip_f32s(op->dev32, op->pw_dev, static_cast<int>(op->pw_host.size()), op->batch, t,
                                           op->skip_dev, op->skip_sc, s),
               "tfsf skip kernel");
            g_launches.fetch_add(1, std::memory_order_relaxed);
        }
        A.pw = op->pw_dev;
        A.n_pw = static_cast<int>(op->pw_host.size());
        A.skip = known < 0 ? op->skip_dev : op->skip_const + known;
    } else {
        A.pw = nullptr;
        A.n_pw = 0;
        A.skip = nullptr;
    }
    if (uses_tc1(op))
        dgtd::launch_stage_tc1(op->dev32, A, op->tc1_img, op->tc1_status, op->n_sm, s);
    else
        ck(dgtd::launch_stage_f32s(op->dev32, A, s), "FP32 stage kernel");
    g_launches.fetch_add(1, std::memory_order_relaxed);
}

void ensure_ws32(dgtd_op* op)
{
    if (op->ws32) return;
    ck(cudaMalloc(&op->ws32, 3 * op->state_len * sizeof(float)), "cudaMalloc RK scratch");
}

void rk_step32(dgtd_op* op, float* d_x, double t, double dt, int integrator, float* lsrk_other, float*& cur,
               cudaStream_t s)
{
    const int64_t L = op->state_len;
    const float dtf = static_cast<float>(dt);
    if (integrator == DGTD_RK4) {
        float* y0 = op->ws32;
        float* y1 = op->ws32 + L;
        float* z = op->ws32 + 2 * L;
        dgtd::StageArgsF32 A{};
        A.dt = dtf;
        A.x = d_x;
        A.z = z;
        A.mode = dgtd::MODE_RK4_1; A.in = d_x; A.yout = y0; run_stage32(op, A, t, s);
        A.mode = dgtd::MODE_RK4_2; A.in = y0; A.yout = y1; run_stage32(op, A, t + dt / 2, s);
        A.mode = dgtd::MODE_RK4_3; A.in = y1; A.yout = y0; run_stage32(op, A, t + dt / 2, s);
        A.mode = dgtd::MODE_RK4_4; A.in = y0; A.yout = nullptr; run_stage32(op, A, t + dt, s);
    } else {
        float* res = op->ws32 + 2 * L;
        for (int st = 0; st < 5; ++st) {
            float* nxt = (cur == d_x) ? lsrk_other : d_x;
            dgtd::StageArgsF32 A{};
            A.dt = dtf;
            A.mode = dgtd::MODE_LSRK;
            A.in = cur;
            A.yout = nxt;
            A.res = res;
            A.a = static_cast<float>(kRk4a[st]);
            A.b = static_cast<float>(kRk4b[st]);
            run_stage32(op, A, t + kRk4c[st] * dt, s);
            cur = nxt;
        }
    }
}

bool ref_layout_fp64(const dgtd_op* op) { return op->precision == DGTD_FP64; }

}  // namespace

extern "C" {

const char* dgtd_last_error(void) { return g_err.c_str(); }

uint64_t dgtd_kernel_launches(void) { return g_launches.load(std::memory_order_relaxed); }

int dgtd_op_create(const dgtd_mesh_desc* mesh, const dgtd_op_opts* opts, dgtd_op** out)
{
    if (!out) return fail(DGTD_ERR_INVALID, "out pointer is NULL");
    *out = nullptr;
    if (!opts) return fail(DGTD_ERR_INVALID, "options are NULL");
    if (opts->order < 1 || opts->order > 6) return fail(DGTD_ERR_UNSUPPORTED, "order must be in [1, 6]");
    if (opts->batch < 1) return fail(DGTD_ERR_INVALID, "batch must be >= 1");
    if (opts->precision != DGTD_FP64 && opts->precision != DGTD_FP32_3XTF32 && opts->precision != DGTD_FP32)
        return fail(DGTD_ERR_INVALID, "unknown precision form");
    if (!(opts->alpha >= 0.0)) return fail(DGTD_ERR_INVALID, "alpha must be >= 0");
    std::unique_ptr<dgtd_op> op;
    try {
        op = std::make_unique<dgtd_op>();
        op->ref = dgtd::build_ref_tet(opts->order);
        op->mesh = dgtd::build_tables(to_input(mesh), op->ref);
        op->batch = opts->batch;
        op->precision = opts->precision;
        op->alpha = opts->alpha;
        const int Np = op->ref.Np, Nfp = op->ref.Nfp;
        op->state_len = 6 * op->mesh.K * Np * static_cast<int64_t>(op->batch);
        if (!op->mesh.sgbc_faces.empty() && (op->precision != DGTD_FP64 || op->batch != 1))
            return fail(DGTD_ERR_UNSUPPORTED, "thin-layer (SGBC) faces need the FP64 form with one incidence");
        if (!op->mesh.curved_elems.empty() && op->precision != DGTD_FP64)
            return fail(DGTD_ERR_UNSUPPORTED, "curved (second-order) elements need the FP64 form");
        for (auto c : op->mesh.fcode)
            if (c == dgtd::FACE_TFSF_TF || c == dgtd::FACE_TFSF_SF) ++op->n_tfsf_faces;

        dgtd::TablesDev& T = op->dev;
        T.p = opts->order; T.Np = Np; T.Nfp = Nfp; T.K = op->mesh.K; T.N = op->mesh.K * Np;
        T.alpha = opts->alpha;
        T.DrT = op->up(transpose(op->ref.Dr, Np, Np));
        T.DsT = op->up(transpose(op->ref.Ds, Np, Np));
        T.DtT = op->up(transpose(op->ref.Dt, Np, Np));
        T.LIFTT = op->up(transpose(op->ref.LIFT, Np, 4 * Nfp));
        T.Fmask = op->up(op->ref.Fmask);
        T.geo = op->up(op->mesh.geo);
        T.fgeo = op->up(op->mesh.fgeo);
        T.mat = op->up(op->mesh.mat);
        T.vmapP = op->up(op->mesh.vmapP);
        T.fcode = op->up(op->mesh.fcode);
        std::vector<double> xyz;
        xyz.reserve(3 * T.N);
        xyz.insert(xyz.end(), op->mesh.x.begin(), op->mesh.x.end());
        xyz.insert(xyz.end(), op->mesh.y.begin(), op->mesh.y.end());
        xyz.insert(xyz.end(), op->mesh.z.begin(), op->mesh.z.end());
        T.xyz = op->up(xyz);
        T.tfsf_elems = op->up(op->mesh.tfsf_elems);
        T.n_tfsf_elems = static_cast<int64_t>(op->mesh.tfsf_elems.size());
        if (!op->mesh.curved_elems.empty()) {
            op->curved = std::make_unique<dgtd::CurvedOp>(op->mesh, op->ref, opts->alpha);
            T.curved = op->curved->flags();
            op->device_bytes += op->curved->device_bytes();
        }
        ck(cudaMalloc(&op->skip_dev, op->batch * sizeof(int)), "cudaMalloc skip");
        op->skip_sc.parts = dgtd::tfsf_skip_parts(T.n_tfsf_elems * T.Np);
        ck(cudaMalloc(&op->skip_sc.partial, static_cast<size_t>(op->batch) * op->skip_sc.parts * sizeof(double)),
           "cudaMalloc skip partials");
        op->allocs.push_back(op->skip_sc.partial);
        ck(cudaMalloc(&op->skip_sc.ticket, op->batch * sizeof(unsigned int)), "cudaMalloc skip tickets");
        op->allocs.push_back(op->skip_sc.ticket);
        ck(cudaMemset(op->skip_sc.ticket, 0, op->batch * sizeof(unsigned int)), "memset skip tickets");
        {
            void* a = nullptr;
            ck(cudaGetSymbolAddress(&a, kDecidedSkip), "skip flag symbol");
            op->skip_const = static_cast<const int*>(a);
        }
        ck(cudaMalloc(&op->norm_dev, (op->batch + 32) * sizeof(double)), "cudaMalloc norm");
        ck(cudaMalloc(&op->stab_dev, sizeof(dgtd::StabilityRecord)), "cudaMalloc stability record");
        reset_stability(op.get());
        {
            int dev = 0;
            ck(cudaGetDevice(&dev), "cudaGetDevice");
            ck(cudaDeviceGetAttribute(&op->n_sm, cudaDevAttrMultiProcessorCount, dev), "SM count");
        }
        if (op->precision == DGTD_FP32_3XTF32) op->batched = dgtd::BatchedOp::create(op->ref, op->mesh, op->dev, op->batch);
        if (op->precision == DGTD_FP32) {
            auto f32 = [](const std::vector<double>& v) { return std::vector<float>(v.begin(), v.end()); };
            dgtd::TablesF32& F = op->dev32;
            F.p = T.p; F.Np = T.Np; F.Nfp = T.Nfp; F.K = T.K; F.N = T.N;
            F.alpha = static_cast<float>(T.alpha);
            F.DrT = op->up(f32(transpose(op->ref.Dr, Np, Np)));
            F.DsT = op->up(f32(transpose(op->ref.Ds, Np, Np)));
            F.DtT = op->up(f32(transpose(op->ref.Dt, Np, Np)));
            F.LIFTT = op->up(f32(transpose(op->ref.LIFT, Np, 4 * Nfp)));
            F.Fmask = T.Fmask;
            F.geo = op->up(f32(op->mesh.geo));
            F.fgeo = op->up(f32(op->mesh.fgeo));
            F.mat = op->up(f32(op->mesh.mat));
            F.vmapP = T.vmapP;
            F.fcode = T.fcode;
            F.xyz = op->up(f32(xyz));
            F.tfsf_elems = T.tfsf_elems;
            F.n_tfsf_elems = T.n_tfsf_elems;
            if (dgtd::tc1_supported(T.p)) {
                const std::vector<uint32_t> img = dgtd::tc1_operator_image(op->ref);
                ck(cudaMalloc(&op->tc1_img, img.size() * sizeof(uint32_t)), "cudaMalloc tensor-core operator");
                ck(cudaMemcpy(op->tc1_img, img.data(), img.size() * sizeof(uint32_t), cudaMemcpyHostToDevice),
                   "upload tensor-core operator");
                op->device_bytes += static_cast<int64_t>(img.size() * sizeof(uint32_t));
                ck(cudaMalloc(&op->tc1_status, sizeof(int)), "cudaMalloc status");
                ck(cudaMemset(op->tc1_status, 0, sizeof(int)), "memset status");
            }
        }
    } catch (const CudaError& e) {
        return fail(DGTD_ERR_CUDA, e.what());
    } catch (const std::bad_alloc&) {
        return fail(DGTD_ERR_NOMEM, "host allocation failed");
    } catch (const std::exception& e) {
        return fail(DGTD_ERR_INVALID, e.what());
    }
    *out = op.release();
    return DGTD_OK;
}

void dgtd_op_destroy(dgtd_op* op) { delete op; }

int dgtd_op_get_info(const dgtd_op* op, dgtd_op_info* info)
{
    if (!op || !info) return fail(DGTD_ERR_INVALID, "NULL argument");
    info->n_elements = op->mesh.K;
    info->order = op->ref.p;
    info->np = op->ref.Np;
    info->nfp = op->ref.Nfp;
    info->batch = op->batch;
    info->precision = op->precision;
    info->ndofs = op->mesh.K * op->ref.Np;
    info->state_len = op->state_len;
    info->n_tfsf_faces = op->n_tfsf_faces;
    info->min_edge = op->mesh.min_edge;
    info->dt_scale_min = op->mesh.dt_scale_min;
    info->device_bytes = op->device_bytes + (op->batched ? op->batched->device_bytes() : 0);
    info->work_len = op->batched ? op->batched->work_len() : op->state_len;
    info->work_word_bytes = op->precision == DGTD_FP64 ? 8 : 4;
    info->batch_padded = op->batched ? static_cast<int32_t>(op->batched->state_len() / (op->mesh.K * 6 * op->ref.Np))
                                     : op->batch;
    return DGTD_OK;
}

int dgtd_op_node_coords(const dgtd_op* op, double* h_xyz)
{
    if (!op || !h_xyz) return fail(DGTD_ERR_INVALID, "NULL argument");
    const int64_t N = op->mesh.K * op->ref.Np;
    std::memcpy(h_xyz, op->mesh.x.data(), N * sizeof(double));
    std::memcpy(h_xyz + N, op->mesh.y.data(), N * sizeof(double));
    std::memcpy(h_xyz + 2 * N, op->mesh.z.data(), N * sizeof(double));
    return DGTD_OK;
}

int dgtd_op_set_planewaves(dgtd_op* op, const dgtd_planewave* pw, int32_t n)
{
    if (!op) return fail(DGTD_ERR_INVALID, "NULL operator");
    if (n < 0 || (n > 0 && !pw)) return fail(DGTD_ERR_INVALID, "bad source array");
    std::vector<dgtd::PlaneWaveDev> v;
    for (int i = 0; i < n; ++i) {
        const dgtd_planewave& s = pw[i];
        if (s.batch < 0 || s.batch >= op->batch) return fail(DGTD_ERR_INVALID, "source batch index out of range");
        if (!(s.spread > 0.0)) return fail(DGTD_ERR_INVALID, "source spread must be positive");
        double kn = std::sqrt(s.propagation[0] * s.propagation[0] + s.propagation[1] * s.propagation[1] +
                              s.propagation[2] * s.propagation[2]);
        double pn = std::sqrt(s.polarization[0] * s.polarization[0] + s.polarization[1] * s.polarization[1] +
                              s.polarization[2] * s.polarization[2]);
        if (!(kn > 0.0) || !(pn > 0.0)) return fail(DGTD_ERR_INVALID, "zero propagation or polarization");
        dgtd::PlaneWaveDev d{};
        for (int c = 0; c < 3; ++c) { d.k[c] = s.propagation[c] / kn; d.pol[c] = s.polarization[c] / pn; }
        d.kxp[0] = d.k[1] * d.pol[2] - d.k[2] * d.pol[1];
        d.kxp[1] = d.k[2] * d.pol[0] - d.k[0] * d.pol[2];
        d.kxp[2] = d.k[0] * d.pol[1] - d.k[1] * d.pol[0];
        d.spread = s.spread;
        d.mean = s.mean;
        d.freq = s.frequency;
        d.batch = s.batch;
        v.push_back(d);
    }
    try {
        op->pw_host = v;
        op->skip_bound = (op->batch == 1 && v.size() == 1)
                             ? dgtd::TfsfSkipBound(op->mesh.x, op->mesh.y, op->mesh.z, op->mesh.tfsf_elems, op->ref.Np, v[0])
                             : dgtd::TfsfSkipBound();
        ensure_sources(op);
        if (op->batched) op->batched->set_sources(op->pw_host);
        defect_restart(op);
    } catch (const std::exception& e) {
        return fail(DGTD_ERR_CUDA, e.what());
    }
    return DGTD_OK;
}

namespace {

// out = M in on every block of Np nodal values of the reference-layout state (incidence,
// component, element): a thread per output value, M and the block read through the read-only
// cache; a grid-stride loop over the n = state_len values
__global__ void basis_change_kernel(const double* __restrict__ M, int Np, int64_t n,
                                    const double* __restrict__ in, double* __restrict__ out)
{
    for (int64_t g = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; g < n;
         g += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t blk = g / Np;
        const int i = static_cast<int>(g - blk * Np);
        const double* x = in + blk * Np;
        const double* m = M + static_cast<int64_t>(i) * Np;
        double a = 0.0;
        for (int j = 0; j < Np; ++j) a = fma(__ldg(m + j), __ldg(x + j), a);
        out[g] = a;
    }
}

}  // namespace

int dgtd_op_change_basis(dgtd_op* op, const void* d_in, void* d_out, int32_t from_basis, int32_t to_basis,
                         void* stream)
{
    if (!op || !d_in || !d_out) return fail(DGTD_ERR_INVALID, "NULL argument");
    if (d_in == d_out) return fail(DGTD_ERR_INVALID, "in and out must not alias");
    if ((from_basis != DGTD_BASIS_GAUSS_LEGENDRE && from_basis != DGTD_BASIS_GAUSS_LOBATTO) ||
        (to_basis != DGTD_BASIS_GAUSS_LEGENDRE && to_basis != DGTD_BASIS_GAUSS_LOBATTO))
        return fail(DGTD_ERR_INVALID, "basis types are 0 (Gauss-Legendre) and 1 (Gauss-Lobatto)");
    if (op->batched || op->precision != DGTD_FP64)
        return fail(DGTD_ERR_UNSUPPORTED, "the change of basis works on the FP64 form's reference-layout state");
    try {
        const cudaStream_t st = static_cast<cudaStream_t>(stream);
        const int Np = op->ref.Np;
        const int64_t n = op->state_len;
        if (from_basis == to_basis) {
            ck(cudaMemcpyAsync(d_out, d_in, static_cast<size_t>(n) * sizeof(double), cudaMemcpyDeviceToDevice, st),
               "basis copy");
            return DGTD_OK;
        }
        if (!op->basis_dev) {
            std::vector<double> h = dgtd::tet_basis_change(op->ref.p, dgtd::kBasisGaussLegendre, dgtd::kBasisGaussLobatto);
            const std::vector<double> back =
                dgtd::tet_basis_change(op->ref.p, dgtd::kBasisGaussLobatto, dgtd::kBasisGaussLegendre);
            h.insert(h.end(), back.begin(), back.end());
            double* d = nullptr;
            ck(cudaMalloc(&d, h.size() * sizeof(double)), "cudaMalloc basis matrices");
            op->allocs.push_back(d);
            ck(cudaMemcpy(d, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice), "upload basis matrices");
            op->basis_dev = d;
        }
        const double* M = op->basis_dev + (from_basis == DGTD_BASIS_GAUSS_LEGENDRE ? 0 : static_cast<int64_t>(Np) * Np);
        const int threads = 256;
        const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>((n + threads - 1) / threads, 8 * op->n_sm));
        basis_change_kernel<<<static_cast<unsigned>(blocks), threads, 0, st>>>(
            M, Np, n, static_cast<const double*>(d_in), static_cast<double*>(d_out));
        ck(cudaGetLastError(), "basis change kernel");
        g_launches.fetch_add(1, std::memory_order_relaxed);
    } catch (const std::exception& e) {
        return fail(DGTD_ERR_CUDA, e.what());
    }
    return DGTD_OK;
}

int dgtd_op_mult(dgtd_op* op, const void* d_x, void* d_y, double t, void* stream)
{
    if (!op || !d_x || !d_y) return fail(DGTD_ERR_INVALID, "NULL argument");
    if (d_x == d_y) return fail(DGTD_ERR_INVALID, "x and y must not alias");
    try {
        if (op->batched) {
            BatchedCount bc(op);
            op->batched->mult(static_cast<const float*>(d_x), static_cast<float*>(d_y), t, static_cast<cudaStream_t>(stream));
            return DGTD_OK;
        }
        if (op->precision == DGTD_FP32) {
            dgtd::StageArgsF32 A{};
            A.mode = dgtd::MODE_MULT;
            A.in = static_cast<const float*>(d_x);
            A.out = static_cast<float*>(d_y);
            run_stage32(op, A, t, static_cast<cudaStream_t>(stream));
            return DGTD_OK;
        }
        dgtd::StageArgs A{};
        A.mode = dgtd::MODE_MULT;
        A.in = static_cast<const double*>(d_x);
        A.out = static_cast<double*>(d_y);
        run_stage(op, A, t, static_cast<cudaStream_t>(stream));
    } catch (const std::invalid_argument& e) {
        return fail(DGTD_ERR_UNSUPPORTED, e.what());
    } catch (const std::exception& e) {
        return fail(DGTD_ERR_CUDA, e.what());
    }
    return DGTD_OK;
}

int dgtd_op_pack(dgtd_op* op, const double* d_ref, void* d_work, void* stream)
{
    if (!op || !d_ref || !d_work) return fail(DGTD_ERR_INVALID, "NULL argument");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    try {
        bool host = false;
        d_ref = static_cast<const double*>(device_view(d_ref, &host));
        if (op->batched) {
            BatchedCount bc(op);
            op->batched->pack(d_ref, static_cast<float*>(d_work), s, host);
        } else if (op->precision == DGTD_FP32) {
            ck(dgtd::launch_convert_f64_to_f32(d_ref, static_cast<float*>(d_work), op->state_len, s), "pack kernel");
            g_launches.fetch_add(1, std::memory_order_relaxed);
        } else if (static_cast<const void*>(d_ref) != d_work) {
            ck(cudaMemcpyAsync(d_work, d_ref, op->state_len * sizeof(double), cudaMemcpyDefault, s), "copy");
        }
    } catch (const std::invalid_argument& e) {
        return fail(DGTD_ERR_INVALID, e.what());
    } catch (const std::exception& e) {
        return fail(DGTD_ERR_CUDA, e.what());
    }
    return DGTD_OK;
}

int dgtd_op_unpack(dgtd_op* op, const void* d_work, double* d_ref, void* stream)
{
    if (!op || !d_ref || !d_work) return fail(DGTD_ERR_INVALID, "NULL argument");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    try {
        bool host = false;
        d_ref = static_cast<double*>(const_cast<void*>(device_view(d_ref, &host)));
        if (op->batched) {
            BatchedCount bc(op);
            op->batched->unpack(static_cast<const float*>(d_work), d_ref, s, host);
        } else if (op->precision == DGTD_FP32) {
            ck(dgtd::launch_convert_f32_to_f64(static_cast<const float*>(d_work), d_ref, op->state_len, s), "unpack kernel");
            g_launches.fetch_add(1, std::memory_order_relaxed);
        } else if (d_work != static_cast<const void*>(d_ref)) {
            ck(cudaMemcpyAsync(d_ref, d_work, op->state_len * sizeof(double), cudaMemcpyDefault, s), "copy");
        }
    } catch (const std::invalid_argument& e) {
        return fail(DGTD_ERR_INVALID, e.what());
    } catch (const std::exception& e) {
        return fail(DGTD_ERR_CUDA, e.what());
    }
    return DGTD_OK;
}

int dgtd_op_mult_host(dgtd_op* op, const double* h_x, double* h_y, double t)
{
    if (!op || !h_x || !h_y) return fail(DGTD_ERR_INVALID, "NULL argument");
    double *dx = nullptr, *dy = nullptr;
    void *wx = nullptr, *wy = nullptr;
    const size_t bytes = op->state_len * sizeof(double);
    int rc = DGTD_OK;
    try {
        ck(cudaMalloc(&dx, bytes), "cudaMalloc");
        ck(cudaMalloc(&dy, bytes), "cudaMalloc");
        ck(cudaMemcpy(dx, h_x, bytes, cudaMemcpyHostToDevice), "H2D");
        if (op->precision != DGTD_FP64) {
            const size_t wb = (op->batched ? op->batched->work_len() : op->state_len) * sizeof(float);
            ck(cudaMalloc(&wx, wb), "cudaMalloc");
            ck(cudaMalloc(&wy, wb), "cudaMalloc");
            rc = dgtd_op_pack(op, dx, wx, nullptr);
            if (rc == DGTD_OK) rc = dgtd_op_mult(op, wx, wy, t, nullptr);
            if (rc == DGTD_OK) rc = dgtd_op_unpack(op, wy, dy, nullptr);
        } else {
            rc = dgtd_op_mult(op, dx, dy, t, nullptr);
        }
        if (rc == DGTD_OK) ck(cudaMemcpy(h_y, dy, bytes, cudaMemcpyDeviceToHost), "D2H");
    } catch (const std::exception& e) {
        rc = fail(DGTD_ERR_CUDA, e.what());
    }
    if (dx) cudaFree(dx);
    if (dy) cudaFree(dy);
    if (wx) cudaFree(wx);
    if (wy) cudaFree(wy);
    return rc;
}

int dgtd_op_step(dgtd_op* op, void* d_work, double t0, double dt, int32_t nsteps, int32_t integrator, void* stream)
{
    if (!op || !d_work) return fail(DGTD_ERR_INVALID, "NULL argument");
    if (nsteps < 0) return fail(DGTD_ERR_INVALID, "nsteps must be >= 0");
    if (integrator != DGTD_RK4 && integrator != DGTD_LSERK4) return fail(DGTD_ERR_INVALID, "unknown integrator");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    try {
        dgtd::ProbeSet* pr = op->probes.get();
        if (op->batched) {
            BatchedCount bc(op);
            if (!pr) {
                batched_steps(op, static_cast<float*>(d_work), t0, dt, nsteps, integrator, s);
                return DGTD_OK;
            }
            double t = t0;
            for (int i = 0; i < nsteps; ++i) {
                batched_steps(op, static_cast<float*>(d_work), t, dt, 1, integrator, s);
                t += dt;
                if (++op->probe_steps % pr->every() == 0) {
                    pr->sample(d_work, t, s);
                    g_launches.fetch_add(1, std::memory_order_relaxed);
                }
            }
            return DGTD_OK;
        }
        if (op->precision == DGTD_FP32) {
            float* d_state = static_cast<float*>(d_work);
            ensure_ws32(op);
            float* other = op->ws32;   // LSERK4 second state buffer
            float* cur = d_state;
            if (integrator == DGTD_LSERK4)
                ck(cudaMemsetAsync(op->ws32 + 2 * op->state_len, 0, op->state_len * sizeof(float), s), "memset");
            double t = t0;
            for (int i = 0; i < nsteps; ++i) {
                rk_step32(op, d_state, t, dt, integrator, other, cur, s);
                t += dt;
                if (pr && ++op->probe_steps % pr->every() == 0) {
                    pr->sample(cur, t, s);
                    g_launches.fetch_add(1, std::memory_order_relaxed);
                }
            }
            if (integrator == DGTD_LSERK4 && cur != d_state)
                ck(cudaMemcpyAsync(d_state, cur, op->state_len * sizeof(float), cudaMemcpyDeviceToDevice, s), "copy");
            return DGTD_OK;
        }
        double* d_state = static_cast<double*>(d_work);
        ensure_ws(op);
        double* other = op->ws;   // LSERK4 second state buffer
        double* cur = d_state;
        if (integrator == DGTD_LSERK4)
            ck(cudaMemsetAsync(op->ws + 2 * op->state_len, 0, op->state_len * sizeof(double), s), "memset");
        double t = t0;
        for (int i = 0; i < nsteps; ++i) {
            rk_step(op, d_state, t, dt, integrator, other, cur, s);
            t += dt;
            if (pr && ++op->probe_steps % pr->every() == 0) {
                pr->sample(cur, t, s);
                g_launches.fetch_add(1, std::memory_order_relaxed);
            }
        }
        if (integrator == DGTD_LSERK4 && cur != d_state)
            ck(cudaMemcpyAsync(d_state, cur, op->state_len * sizeof(double), cudaMemcpyDeviceToDevice, s), "copy");
    } catch (const std::invalid_argument& e) {
        return fail(DGTD_ERR_UNSUPPORTED, e.what());
    } catch (const std::exception& e) {
        return fail(DGTD_ERR_CUDA, e.what());
    }
    return DGTD_OK;
}

int dgtd_op_run_host(dgtd_op* op, double* h_state, double t0, double dt, double final_time, int32_t integrator,
                     int64_t* steps_out)
{
    if (!op || !h_state) return fail(DGTD_ERR_INVALID, "NULL argument");
    if (!(dt > 0.0)) return fail(DGTD_ERR_INVALID, "dt must be positive");
    double* d = nullptr;
    void* w = nullptr;
    const size_t bytes = op->state_len * sizeof(double);
    int rc = DGTD_OK;
    int64_t steps = 0;
    try {
        ck(cudaMalloc(&d, bytes), "cudaMalloc");
        ck(cudaMemcpy(d, h_state, bytes, cudaMemcpyHostToDevice), "H2D");
        if (op->precision != DGTD_FP64) {
            ck(cudaMalloc(&w, (op->batched ? op->batched->work_len() : op->state_len) * sizeof(float)), "cudaMalloc");
            defect_restart(op);   // a new trajectory: the defect correction refreshes at its first step
            rc = dgtd_op_pack(op, d, w, nullptr);
        } else {
            w = d;
        }
        // instability detector (reference Solver.cpp:500-516): a device check every
        // stab_every steps, its record read back every kStabReadEvery steps and at the end
        const bool f32 = op->precision != DGTD_FP64;
        const int64_t wlen = op->batched ? op->batched->state_len() : op->state_len;
        constexpr int64_t kStabReadEvery = 256;
        bool warned = false;
        auto stability_read = [&]() -> int {
            dgtd::StabilityRecord r{};
            ck(cudaMemcpy(&r, op->stab_dev, sizeof(r), cudaMemcpyDeviceToHost), "read stability record");
            if (r.first_step < 0) return DGTD_OK;
            const std::string msg = "simulation is potentially unstable: field norm = " + std::to_string(r.norm) +
                                    " at step " + std::to_string(r.first_step) + ", time " +
                                    std::to_string(r.t) + " / " + std::to_string(final_time) + ", dt " +
                                    std::to_string(dt) + "; verify the setup and consider a smaller time step";
            if (op->stab_stop) return fail(DGTD_ERR_UNSTABLE, msg);
            if (!warned) std::fprintf(stderr, "dgtd_gb300: WARNING: %s\n", msg.c_str());
            warned = true;
            return DGTD_OK;
        };
        if (op->stab_every > 0) reset_stability(op);
        double t = t0;
        while (rc == DGTD_OK && t <= final_time - 1e-8 * dt) {
            double truedt = std::min(dt, final_time - t);
            rc = dgtd_op_step(op, w, t, truedt, 1, integrator, nullptr);
            if (rc != DGTD_OK) break;
            t += truedt;
            ++steps;
            if (op->stab_every > 0 && steps % op->stab_every == 0) {
                ck(dgtd::launch_stability_check(w, wlen, f32, op->stab_dev, steps, t, op->n_sm, nullptr),
                   "stability check");
                g_launches.fetch_add(2, std::memory_order_relaxed);
                if (steps % kStabReadEvery == 0) rc = stability_read();
            }
        }
        if (rc == DGTD_OK && op->stab_every > 0) {
            if (steps % op->stab_every != 0) {   // the final state is always checked
                ck(dgtd::launch_stability_check(w, wlen, f32, op->stab_dev, steps, t, op->n_sm, nullptr),
                   "stability check");
                g_launches.fetch_add(2, std::memory_order_relaxed);
            }
            rc = stability_read();
        }
        if (rc == DGTD_OK && op->precision != DGTD_FP64) rc = dgtd_op_unpack(op, w, d, nullptr);
        if (rc == DGTD_OK) ck(cudaMemcpy(h_state, d, bytes, cudaMemcpyDeviceToHost), "D2H");
    } catch (const std::exception& e) {
        rc = fail(DGTD_ERR_CUDA, e.what());
    }
    if (w && w != d) cudaFree(w);
    if (d) cudaFree(d);
    if (steps_out) *steps_out = steps;
    return rc;
}

int dgtd_op_norm2(dgtd_op* op, const void* d_state, double* h_out, void* stream)
{
    if (!op || !d_state || !h_out) return fail(DGTD_ERR_INVALID, "NULL argument");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    try {
        if (op->batched) {
            BatchedCount bc(op);
            op->batched->norm2(static_cast<const float*>(d_state), op->norm_dev, s);
        } else if (op->precision == DGTD_FP32) {
            ck(dgtd::launch_norm2_f32s(static_cast<const float*>(d_state), op->state_len / op->batch, op->batch,
                                       op->norm_dev, s), "norm kernel");
            g_launches.fetch_add(1, std::memory_order_relaxed);
        } else {
            ck(dgtd::launch_norm2(static_cast<const double*>(d_state), op->state_len / op->batch, op->batch,
                                  op->norm_dev, s), "norm kernel");
            g_launches.fetch_add(1, std::memory_order_relaxed);
        }
        ck(cudaMemcpyAsync(h_out, op->norm_dev, op->batch * sizeof(double), cudaMemcpyDeviceToHost, s), "D2H");
        ck(cudaStreamSynchronize(s), "sync");
    } catch (const std::exception& e) {
        return fail(DGTD_ERR_CUDA, e.what());
    }
    return DGTD_OK;
}

int dgtd_op_set_stability_check(dgtd_op* op, int32_t every, int32_t stop)
{
    if (!op) return fail(DGTD_ERR_INVALID, "NULL argument");
    if (every < 0) return fail(DGTD_ERR_INVALID, "every must be >= 0");
    if (stop != 0 && stop != 1) return fail(DGTD_ERR_INVALID, "stop must be 0 or 1");
    op->stab_every = every;
    op->stab_stop = stop;
    return DGTD_OK;
}

int dgtd_op_stability_reset(dgtd_op* op)
{
    if (!op) return fail(DGTD_ERR_INVALID, "NULL argument");
    try {
        reset_stability(op);
    } catch (const std::exception& e) {
        return fail(DGTD_ERR_CUDA, e.what());
    }
    return DGTD_OK;
}

int dgtd_op_stability_check(dgtd_op* op, const void* d_state, int64_t step, double t, void* stream)
{
    if (!op || !d_state) return fail(DGTD_ERR_INVALID, "NULL argument");
    try {
        const bool f32 = op->precision != DGTD_FP64;
        const int64_t wlen = op->batched ? op->batched->state_len() : op->state_len;
        ck(dgtd::launch_stability_check(d_state, wlen, f32, op->stab_dev, step, t, op->n_sm,
                                        static_cast<cudaStream_t>(stream)),
           "stability check");
        g_launches.fetch_add(2, std::memory_order_relaxed);
    } catch (const std::exception& e) {
        return fail(DGTD_ERR_CUDA, e.what());
    }
    return DGTD_OK;
}

int dgtd_op_stability(const dgtd_op* op, int64_t* first_step, double* t, double* norm, int64_t* checks)
{
    if (!op) return fail(DGTD_ERR_INVALID, "NULL argument");
    dgtd::StabilityRecord r{};
    try {
        ck(cudaMemcpy(&r, op->stab_dev, sizeof(r), cudaMemcpyDeviceToHost), "read stability record");
    } catch (const std::exception& e) {
        return fail(DGTD_ERR_CUDA, e.what());
    }
    if (first_step) *first_step = r.first_step;
    if (t) *t = r.t;
    if (norm) *norm = r.norm;
    if (checks) *checks = r.checks;
    return DGTD_OK;
}

int dgtd_op_set_contraction(dgtd_op* op, int32_t mode)
{
    if (!op) return fail(DGTD_ERR_INVALID, "NULL operator");
    if (mode != 0 && mode != 1) return fail(DGTD_ERR_INVALID, "contraction mode must be 0 or 1");
    if (op->batched) op->batched->set_contraction(mode);
    op->contraction32 = mode;
    return DGTD_OK;
}

int dgtd_op_set_defect_correction(dgtd_op* op, int32_t every)
{
    if (!op) return fail(DGTD_ERR_INVALID, "NULL operator");
    if (every < 0) return fail(DGTD_ERR_INVALID, "defect-correction period must be >= 0");
    if (!op->batched) return fail(DGTD_ERR_UNSUPPORTED, "the defect correction is implemented for the batched FP32 form");
    try {
        op->defect_every = every;
        defect_restart(op);
        if (every == 0) op->free_defect_buffers();
    } catch (const std::exception& e) {
        return fail(DGTD_ERR_CUDA, e.what());
    }
    return DGTD_OK;
}

int dgtd_op_defect_refreshes(const dgtd_op* op, int64_t* refreshes)
{
    if (!op) return fail(DGTD_ERR_INVALID, "NULL operator");
    if (refreshes) *refreshes = op->defect_refreshes;
    return DGTD_OK;
}

int dgtd_op_set_graph_steps(dgtd_op* op, int32_t steps)
{
    if (!op) return fail(DGTD_ERR_INVALID, "NULL operator");
    if (steps < 0) return fail(DGTD_ERR_INVALID, "graph steps must be >= 0");
    if (!op->batched) return fail(DGTD_ERR_UNSUPPORTED, "CUDA-graph stepping is implemented for the batched FP32 form");
    try {
        op->batched->set_graph_steps(steps);
    } catch (const std::exception& e) {
        return fail(DGTD_ERR_CUDA, e.what());
    }
    return DGTD_OK;
}

int dgtd_op_autotune(dgtd_op* op, const void* d_work, void* stream, double* h_ms, int32_t* choice)
{
    if (!op || !d_work) return fail(DGTD_ERR_INVALID, "NULL argument");
    if (!op->batched) return fail(DGTD_ERR_UNSUPPORTED, "the autotuner chooses among the batched form's kernels");
    try {
        BatchedCount bc(op);
        double ms[4];
        const int c = op->batched->autotune(static_cast<const float*>(d_work), ms, static_cast<cudaStream_t>(stream));
        if (h_ms) std::copy(ms, ms + 4, h_ms);
        if (choice) *choice = c;
    } catch (const std::exception& e) {
        return fail(DGTD_ERR_CUDA, e.what());
    }
    return DGTD_OK;
}

int dgtd_op_uses_tensor_cores(const dgtd_op* op)
{
    if (!op) return 0;
    if (op->batched) return op->batched->uses_tensor_cores() ? 1 : 0;
    return (op->precision == DGTD_FP32 && uses_tc1(op)) ? 1 : 0;
}

int dgtd_op_check(dgtd_op* op, void* stream)
{
    if (!op) return fail(DGTD_ERR_INVALID, "NULL operator");
    try {
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        ck(cudaStreamSynchronize(s), "sync");
        if (op->batched && op->batched->take_status(s))
            return fail(DGTD_ERR_TIMEOUT, "a tensor-core completion wait inside the stage kernel timed out");
        if (op->tc1_status) {
            int st = 0;
            ck(cudaMemcpy(&st, op->tc1_status, sizeof(int), cudaMemcpyDeviceToHost), "read status");
            if (st) {
                ck(cudaMemset(op->tc1_status, 0, sizeof(int)), "clear status");
                return fail(DGTD_ERR_TIMEOUT, "a tensor-core completion wait inside the stage kernel timed out");
            }
        }
    } catch (const std::exception& e) {
        return fail(DGTD_ERR_CUDA, e.what());
    }
    return DGTD_OK;
}

int dgtd_op_estimate_dt(const dgtd_op* op, double cfl, double* dt_out)
{
    if (!op || !dt_out) return fail(DGTD_ERR_INVALID, "NULL argument");
    if (!(cfl > 0.0)) return fail(DGTD_ERR_INVALID, "cfl must be positive");
    *dt_out = dgtd::estimate_dt(op->mesh, op->ref.p, cfl, 1);   // the reference's default, global
    return DGTD_OK;
}

int dgtd_op_set_probes(dgtd_op* op, const dgtd_probe_spec* spec)
{
    if (!op || !spec) return fail(DGTD_ERR_INVALID, "NULL argument");
    if (spec->n_points < 0 || spec->n_surface_faces < 0 || spec->n_freqs < 0)
        return fail(DGTD_ERR_INVALID, "negative probe counts");
    if ((spec->n_points > 0 && !spec->points) || (spec->n_surface_faces > 0 && !spec->surface_faces) ||
        (spec->n_freqs > 0 && !spec->freqs))
        return fail(DGTD_ERR_INVALID, "probe arrays missing");
    try {
        dgtd::ProbeSpec ps;
        ps.points.assign(spec->points, spec->points + 3 * static_cast<int64_t>(spec->n_points));
        ps.surface_faces.assign(spec->surface_faces, spec->surface_faces + 3 * spec->n_surface_faces);
        ps.freqs.assign(spec->freqs, spec->freqs + spec->n_freqs);
        ps.every = spec->every;
        ps.max_records = spec->max_records;
        dgtd::ProbeStateLayout lay;
        lay.Np = op->ref.Np;
        lay.N = op->mesh.K * op->ref.Np;
        lay.B = op->batch;
        if (op->batched) {
            lay.fp32 = true;
            lay.Bp = op->batched->batch_padded();
            lay.inv_perm = op->batched->inv_perm().data();
        } else if (op->precision == DGTD_FP32) {
            lay.f32_ref = true;
        }
        op->probes.reset();
        op->probes = dgtd::ProbeSet::create(op->ref, op->mesh, ps, lay);
        op->probe_steps = 0;
    } catch (const std::invalid_argument& e) {
        return fail(DGTD_ERR_INVALID, e.what());
    } catch (const std::exception& e) {
        return fail(DGTD_ERR_CUDA, e.what());
    }
    return DGTD_OK;
}

int dgtd_op_clear_probes(dgtd_op* op)
{
    if (!op) return fail(DGTD_ERR_INVALID, "NULL operator");
    op->probes.reset();
    op->probe_steps = 0;
    return DGTD_OK;
}

int dgtd_op_probe_reset(dgtd_op* op, void* stream)
{
    if (!op) return fail(DGTD_ERR_INVALID, "NULL operator");
    if (!op->probes) return fail(DGTD_ERR_INVALID, "no probes installed");
    try {
        op->probes->reset(static_cast<cudaStream_t>(stream));
        op->probe_steps = 0;
    } catch (const std::exception& e) {
        return fail(DGTD_ERR_CUDA, e.what());
    }
    return DGTD_OK;
}

int dgtd_op_probe_info(const dgtd_op* op, int64_t* n_surface_nodes, int64_t* n_samples, int64_t* n_records)
{
    if (!op) return fail(DGTD_ERR_INVALID, "NULL operator");
    if (!op->probes) return fail(DGTD_ERR_INVALID, "no probes installed");
    if (n_surface_nodes) *n_surface_nodes = op->probes->n_surface_nodes();
    if (n_samples) *n_samples = op->probes->n_samples();
    if (n_records) *n_records = op->probes->n_records();
    return DGTD_OK;
}

int dgtd_op_probe_surface(const dgtd_op* op, double* h_xyz, double* h_normal, double* h_weight)
{
    if (!op) return fail(DGTD_ERR_INVALID, "NULL operator");
    if (!op->probes) return fail(DGTD_ERR_INVALID, "no probes installed");
    const auto& P = *op->probes;
    if (h_xyz) std::copy(P.surface_xyz().begin(), P.surface_xyz().end(), h_xyz);
    if (h_normal) std::copy(P.surface_normal().begin(), P.surface_normal().end(), h_normal);
    if (h_weight) std::copy(P.surface_weight().begin(), P.surface_weight().end(), h_weight);
    return DGTD_OK;
}

int dgtd_op_probe_sample(dgtd_op* op, const void* d_state, double t, void* stream)
{
    if (!op || !d_state) return fail(DGTD_ERR_INVALID, "NULL argument");
    if (!op->probes) return fail(DGTD_ERR_INVALID, "no probes installed");
    try {
        op->probes->sample(d_state, t, static_cast<cudaStream_t>(stream));
        g_launches.fetch_add(1, std::memory_order_relaxed);
    } catch (const std::exception& e) {
        return fail(DGTD_ERR_CUDA, e.what());
    }
    return DGTD_OK;
}

int dgtd_op_probe_read(dgtd_op* op, double* h_point_dft, double* h_surface_dft, double* h_series, double* h_series_t,
                       void* stream)
{
    if (!op) return fail(DGTD_ERR_INVALID, "NULL operator");
    if (!op->probes) return fail(DGTD_ERR_INVALID, "no probes installed");
    try {
        op->probes->read(h_point_dft, h_surface_dft, h_series, h_series_t, static_cast<cudaStream_t>(stream));
    } catch (const std::exception& e) {
        return fail(DGTD_ERR_CUDA, e.what());
    }
    return DGTD_OK;
}

namespace {

std::vector<dgtd::SgbcStackSpec> sgbc_specs(const dgtd_sgbc_stack* stacks, int32_t n)
{
    std::vector<dgtd::SgbcStackSpec> out;
    for (int32_t i = 0; i < n; ++i) {
        const dgtd_sgbc_stack& S = stacks[i];
        if (S.n_layers < 1 || !S.layers) throw std::invalid_argument("SGBC stack without layers");
        dgtd::SgbcStackSpec sp;
        for (int32_t l = 0; l < S.n_layers; ++l) {
            const dgtd_sgbc_layer& L = S.layers[l];
            sp.layers.push_back({L.eps_r, L.mu_r, L.sigma, L.width, L.segments, L.order});
        }
        sp.left_bc = S.left_bc;
        sp.right_bc = S.right_bc;
        sp.sub_dt = S.sub_dt;
        out.push_back(sp);
    }
    return out;
}

}  // namespace

int dgtd_op_set_sgbc(dgtd_op* op, const dgtd_sgbc_stack* stacks, int32_t n_stacks, const int32_t* face_stack)
{
    if (!op || !stacks || n_stacks < 1) return fail(DGTD_ERR_INVALID, "NULL argument or no stacks");
    const int64_t nf = static_cast<int64_t>(op->mesh.sgbc_faces.size() / 4);
    if (nf == 0) return fail(DGTD_ERR_INVALID, "the mesh has no thin-layer (SGBC) faces");
    if (!face_stack) return fail(DGTD_ERR_INVALID, "face_stack is NULL");
    try {
        std::vector<int32_t> fs(face_stack, face_stack + nf);
        auto S = std::make_unique<dgtd::SgbcOp>(op->mesh, op->ref, sgbc_specs(stacks, n_stacks), fs, op->alpha);
        op->sgbc = std::move(S);
    } catch (const std::invalid_argument& e) {
        return fail(DGTD_ERR_UNSUPPORTED, e.what());
    } catch (const std::exception& e) {
        return fail(DGTD_ERR_CUDA, e.what());
    }
    return DGTD_OK;
}

int dgtd_op_sgbc_commit(dgtd_op* op, const void* d_x, double t, double dt, void* stream)
{
    if (!op || !d_x) return fail(DGTD_ERR_INVALID, "NULL argument");
    if (!op->sgbc) return fail(DGTD_ERR_INVALID, "no thin-layer (SGBC) stacks are set");
    try {
        const int64_t before = op->sgbc->launches();
        op->sgbc->commit(op->dev, static_cast<const double*>(d_x), t, dt, static_cast<cudaStream_t>(stream));
        g_launches.fetch_add(op->sgbc->launches() - before, std::memory_order_relaxed);
    } catch (const std::exception& e) {
        return fail(DGTD_ERR_CUDA, e.what());
    }
    return DGTD_OK;
}

int dgtd_op_sgbc_finalize(dgtd_op* op, const void* d_x, void* stream)
{
    if (!op || !d_x) return fail(DGTD_ERR_INVALID, "NULL argument");
    if (!op->sgbc) return fail(DGTD_ERR_INVALID, "no thin-layer (SGBC) stacks are set");
    try {
        const int64_t before = op->sgbc->launches();
        op->sgbc->finalize(op->dev, static_cast<const double*>(d_x), static_cast<cudaStream_t>(stream));
        g_launches.fetch_add(op->sgbc->launches() - before, std::memory_order_relaxed);
    } catch (const std::invalid_argument& e) {
        return fail(DGTD_ERR_UNSUPPORTED, e.what());
    } catch (const std::exception& e) {
        return fail(DGTD_ERR_CUDA, e.what());
    }
    return DGTD_OK;
}

int dgtd_op_sgbc_states(const dgtd_op* op, int64_t* n_pairs, int64_t* state_len, double* h_states, int64_t cap)
{
    if (!op) return fail(DGTD_ERR_INVALID, "NULL argument");
    const int64_t np = op->sgbc ? op->sgbc->n_pairs() : 0, sl = op->sgbc ? op->sgbc->state_len() : 0;
    if (n_pairs) *n_pairs = np;
    if (state_len) *state_len = sl;
    if (h_states && op->sgbc) {
        if (cap < sl) return fail(DGTD_ERR_INVALID, "state buffer too small");
        try { op->sgbc->read_states(h_states); }
        catch (const std::exception& e) { return fail(DGTD_ERR_CUDA, e.what()); }
    }
    return DGTD_OK;
}

int dgtd_sgbc_stack_operator(const dgtd_sgbc_stack* stack, int64_t* n, int64_t* idx_left, int64_t* idx_right,
                             double* A, int64_t cap)
{
    if (!stack) return fail(DGTD_ERR_INVALID, "NULL argument");
    try {
        const dgtd::SgbcStack1D S = dgtd::build_sgbc_stack(sgbc_specs(stack, 1)[0]);
        if (n) *n = S.n;
        if (idx_left) *idx_left = S.idx_left;
        if (idx_right) *idx_right = S.idx_right;
        if (A) {
            if (cap < S.n * S.n) return fail(DGTD_ERR_INVALID, "operator buffer too small");
            std::memcpy(A, S.A.data(), S.A.size() * sizeof(double));
        }
    } catch (const std::invalid_argument& e) {
        return fail(DGTD_ERR_UNSUPPORTED, e.what());
    } catch (const std::exception& e) {
        return fail(DGTD_ERR_INVALID, e.what());
    }
    return DGTD_OK;
}

int dgtd_sgbc_stack_maps(const dgtd_sgbc_stack* stack, double span, int32_t nsteps, double* R, double* G, double* F,
                         double* Vo, double* Vn)
{
    if (!stack || nsteps < 1 || !(span > 0.0)) return fail(DGTD_ERR_INVALID, "NULL stack, nsteps < 1 or span <= 0");
    try {
        const dgtd::SgbcStack1D S = dgtd::build_sgbc_stack(sgbc_specs(stack, 1)[0]);
        if (R || G) {
            const dgtd::SgbcStageMap M = dgtd::sgbc_stage_map(S, span, nsteps);
            if (R) std::memcpy(R, M.R.data(), M.R.size() * sizeof(double));
            if (G) std::memcpy(G, M.G.data(), M.G.size() * sizeof(double));
        }
        if (F || Vo || Vn) {
            const dgtd::SgbcFinalMap M = dgtd::sgbc_final_map(S, span, nsteps);
            if (F)
                for (int64_t i = 0; i < S.n; ++i)
                    for (int64_t j = 0; j < S.n; ++j) F[i * S.n + j] = M.FT[j * S.n + i];
            if (Vo) std::memcpy(Vo, M.Vo.data(), M.Vo.size() * sizeof(double));
            if (Vn) std::memcpy(Vn, M.Vn.data(), M.Vn.size() * sizeof(double));
        }
    } catch (const std::invalid_argument& e) {
        return fail(DGTD_ERR_UNSUPPORTED, e.what());
    } catch (const std::exception& e) {
        return fail(DGTD_ERR_INVALID, e.what());
    }
    return DGTD_OK;
}

int dgtd_curved_block_rows(const dgtd_mesh_desc* mesh, int32_t order, double alpha, int32_t* elems, int32_t* nbr,
                           double* blocks, int64_t cap)
{
    if (!mesh) return fail(DGTD_ERR_INVALID, "NULL mesh");
    if (order < 1 || order > 6) return fail(DGTD_ERR_UNSUPPORTED, "order must be in [1, 6]");
    try {
        const dgtd::RefTet ref = dgtd::build_ref_tet(order);
        const dgtd::MeshTables T = dgtd::build_tables(to_input(mesh), ref);
        const dgtd::CurvedRows C = dgtd::build_curved_rows(T, ref, alpha);
        if (static_cast<int64_t>(C.blocks.size()) > cap) return fail(DGTD_ERR_INVALID, "block buffer too small");
        if (elems) std::copy(C.elems.begin(), C.elems.end(), elems);
        if (nbr) std::copy(C.nbr.begin(), C.nbr.end(), nbr);
        if (blocks) std::copy(C.blocks.begin(), C.blocks.end(), blocks);
    } catch (const std::exception& e) {
        return fail(DGTD_ERR_INVALID, e.what());
    }
    return DGTD_OK;
}

int dgtd_tet_nodes(int32_t order, int32_t basis_type, double* bary)
{
    if (!bary) return fail(DGTD_ERR_INVALID, "NULL argument");
    if (order < 1 || order > 6) return fail(DGTD_ERR_UNSUPPORTED, "order must be in [1, 6]");
    try {
        const std::vector<double> b = dgtd::tet_node_bary(order, basis_type);
        std::copy(b.begin(), b.end(), bary);
    } catch (const std::exception& e) {
        return fail(DGTD_ERR_INVALID, e.what());
    }
    return DGTD_OK;
}

int dgtd_tet_basis_change(int32_t order, int32_t from_basis, int32_t to_basis, double* m)
{
    if (!m) return fail(DGTD_ERR_INVALID, "NULL argument");
    if (order < 1 || order > 6) return fail(DGTD_ERR_UNSUPPORTED, "order must be in [1, 6]");
    try {
        const std::vector<double> M = dgtd::tet_basis_change(order, from_basis, to_basis);
        std::copy(M.begin(), M.end(), m);
    } catch (const std::exception& e) {
        return fail(DGTD_ERR_INVALID, e.what());
    }
    return DGTD_OK;
}

int dgtd_mesh_validate(const dgtd_mesh_desc* mesh, const dgtd_op_opts* opts, dgtd_op_info* info)
{
    if (!opts || !info) return fail(DGTD_ERR_INVALID, "NULL argument");
    if (opts->order < 1 || opts->order > 6) return fail(DGTD_ERR_UNSUPPORTED, "order must be in [1, 6]");
    try {
        auto ref = dgtd::build_ref_tet(opts->order);
        auto tab = dgtd::build_tables(to_input(mesh), ref);
        std::memset(info, 0, sizeof(*info));
        info->n_elements = tab.K;
        info->order = ref.p; info->np = ref.Np; info->nfp = ref.Nfp;
        info->batch = opts->batch; info->precision = opts->precision;
        info->ndofs = tab.K * ref.Np;
        info->state_len = 6 * tab.K * ref.Np * static_cast<int64_t>(std::max(1, opts->batch));
        for (auto c : tab.fcode)
            if (c == dgtd::FACE_TFSF_TF || c == dgtd::FACE_TFSF_SF) ++info->n_tfsf_faces;
        info->min_edge = tab.min_edge;
        info->dt_scale_min = tab.dt_scale_min;
    } catch (const std::exception& e) {
        return fail(DGTD_ERR_INVALID, e.what());
    }
    return DGTD_OK;
}

int dgtd_box_mesh_size(const dgtd_box_spec* spec, int64_t* nv, int64_t* ne, int64_t* nb, int64_t* nt)
{
    if (!spec) return fail(DGTD_ERR_INVALID, "NULL spec");
    try {
        dgtd::BoxSpec b;
        for (int d = 0; d < 3; ++d) {
            b.n[d] = spec->n[d]; b.lo[d] = spec->lo[d]; b.hi[d] = spec->hi[d];
            b.hole_lo[d] = spec->hole_lo[d]; b.hole_hi[d] = spec->hole_hi[d];
            b.tf_lo[d] = spec->tf_lo[d]; b.tf_hi[d] = spec->tf_hi[d];
        }
        b.outer_bc = spec->outer_bc; b.hole_bc = spec->hole_bc;
        auto m = dgtd::make_box(b);
        if (nv) *nv = static_cast<int64_t>(m.vertices.size() / 3);
        if (ne) *ne = static_cast<int64_t>(m.elements.size() / 4);
        if (nb) *nb = static_cast<int64_t>(m.bdr_codes.size());
        if (nt) *nt = static_cast<int64_t>(m.tfsf_faces.size() / 3);
    } catch (const std::exception& e) {
        return fail(DGTD_ERR_INVALID, e.what());
    }
    return DGTD_OK;
}

int dgtd_box_mesh_fill(const dgtd_box_spec* spec, double* vertices, int32_t* elements, int32_t* bdr_faces,
                       int32_t* bdr_codes, int32_t* tfsf_faces)
{
    if (!spec) return fail(DGTD_ERR_INVALID, "NULL spec");
    try {
        dgtd::BoxSpec b;
        for (int d = 0; d < 3; ++d) {
            b.n[d] = spec->n[d]; b.lo[d] = spec->lo[d]; b.hi[d] = spec->hi[d];
            b.hole_lo[d] = spec->hole_lo[d]; b.hole_hi[d] = spec->hole_hi[d];
            b.tf_lo[d] = spec->tf_lo[d]; b.tf_hi[d] = spec->tf_hi[d];
        }
        b.outer_bc = spec->outer_bc; b.hole_bc = spec->hole_bc;
        auto m = dgtd::make_box(b);
        if (vertices) std::memcpy(vertices, m.vertices.data(), m.vertices.size() * sizeof(double));
        if (elements) std::memcpy(elements, m.elements.data(), m.elements.size() * sizeof(int32_t));
        if (bdr_faces) std::memcpy(bdr_faces, m.bdr_faces.data(), m.bdr_faces.size() * sizeof(int32_t));
        if (bdr_codes) std::memcpy(bdr_codes, m.bdr_codes.data(), m.bdr_codes.size() * sizeof(int32_t));
        if (tfsf_faces) std::memcpy(tfsf_faces, m.tfsf_faces.data(), m.tfsf_faces.size() * sizeof(int32_t));
    } catch (const std::exception& e) {
        return fail(DGTD_ERR_INVALID, e.what());
    }
    return DGTD_OK;
}

int dgtd_ref_tet(int32_t order, double* r, double* s, double* t, double* Dr, double* Ds, double* Dt, double* Minv,
                 double* lift, int32_t* fmask)
{
    try {
        auto T = dgtd::build_ref_tet(order);
        auto cp = [](double* dst, const std::vector<double>& v) {
            if (dst) std::memcpy(dst, v.data(), v.size() * sizeof(double));
        };
        cp(r, T.r); cp(s, T.s); cp(t, T.t); cp(Dr, T.Dr); cp(Ds, T.Ds); cp(Dt, T.Dt); cp(Minv, T.Minv); cp(lift, T.LIFT);
        if (fmask) for (size_t i = 0; i < T.Fmask.size(); ++i) fmask[i] = T.Fmask[i];
    } catch (const std::exception& e) {
        return fail(DGTD_ERR_INVALID, e.what());
    }
    return DGTD_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Stepping without device allocation.
//
// dgtd_op_step allocates its three RK registers with cudaMalloc on first use.
// Some callers cannot allow that: a host that has reserved all device memory
// up front for its own pool, or a caller on a path where a cudaMalloc would
// synchronise the device and stall other streams. dgtd_op_step_noalloc runs the
// same fused stage kernels with the registers in one file-scope device array
// of fixed size instead, so the call itself allocates nothing.
//
// The array is shared by every operator and every call in the process and
// keeps the last call's contents; the parts that must start at zero (the
// LSERK4 residual) are cleared by each call. Calls that overlap on the GPU
// (two streams, or two host threads) use the same registers and race.
namespace {

// Largest reference-layout state (6 * K * Np * B entries) the scratch holds.
constexpr int64_t kNoAllocMaxState = int64_t(1) << 20;
// Three RK registers of FP64 state: 24 MiB.
static __device__ __align__(256) double g_noalloc_scratch[3 * kNoAllocMaxState];

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mutex;
double* g_noalloc_ptr[kNoAllocMaxDevices] = {};

// Address of the scratch array on the current device; looked up once per device
// (the first call on each device does this set-up).
double* noalloc_scratch()
{
    int dev = -1;
    ck(cudaGetDevice(&dev), "cudaGetDevice");
    if (dev < 0 || dev >= kNoAllocMaxDevices) throw CudaError("device ordinal out of range for the no-allocation scratch");
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
        double* ptr = nullptr;
        ck(cudaGetSymbolAddress(reinterpret_cast<void**>(&ptr), g_noalloc_scratch), "cudaGetSymbolAddress");
        g_noalloc_ptr[dev] = ptr;
    }
    return g_noalloc_ptr[dev];
}

// One RK step with the registers at ws (3 * state_len doubles); the same stage
// sequence as rk_step.
void rk_step_at(dgtd_op* op, double* ws, double* d_x, double t, double dt, int integrator, double* lsrk_other,
                double*& cur, cudaStream_t s)
{
    const int64_t L = op->state_len;
    if (integrator == DGTD_RK4) {
        double* y0 = ws;
        double* y1 = ws + L;
        double* z = ws + 2 * L;
        dgtd::StageArgs A{};
        A.dt = dt;
        A.x = d_x;
        A.z = z;
        A.mode = dgtd::MODE_RK4_1; A.in = d_x; A.yout = y0; run_stage(op, A, t, s);
        A.mode = dgtd::MODE_RK4_2; A.in = y0; A.yout = y1; run_stage(op, A, t + dt / 2, s);
        A.mode = dgtd::MODE_RK4_3; A.in = y1; A.yout = y0; run_stage(op, A, t + dt / 2, s);
        A.mode = dgtd::MODE_RK4_4; A.in = y0; A.yout = nullptr; run_stage(op, A, t + dt, s);
    } else {
        double* res = ws + 2 * L;
        for (int st = 0; st < 5; ++st) {
            double* nxt = (cur == d_x) ? lsrk_other : d_x;
            dgtd::StageArgs A{};
            A.dt = dt;
            A.mode = dgtd::MODE_LSRK;
            A.in = cur;
            A.yout = nxt;
            A.res = res;
            A.a = kRk4a[st];
            A.b = kRk4b[st];
            run_stage(op, A, t + kRk4c[st] * dt, s);
            cur = nxt;
        }
    }
}

}  // namespace

extern "C" {

int64_t dgtd_noalloc_max_state(void) { return kNoAllocMaxState; }

int dgtd_op_step_noalloc(dgtd_op* op, void* d_state, double t0, double dt, int32_t nsteps, int32_t integrator,
                         void* stream)
{
    if (!op || !d_state) return fail(DGTD_ERR_INVALID, "NULL argument");
    if (nsteps < 0) return fail(DGTD_ERR_INVALID, "nsteps must be >= 0");
    if (integrator != DGTD_RK4 && integrator != DGTD_LSERK4) return fail(DGTD_ERR_INVALID, "unknown integrator");
    if (op->precision != DGTD_FP64)
        return fail(DGTD_ERR_UNSUPPORTED, "dgtd_op_step_noalloc supports the FP64 form only");
    if (!op->mesh.sgbc_faces.empty())
        return fail(DGTD_ERR_UNSUPPORTED, "dgtd_op_step_noalloc does not step thin-layer (SGBC) faces "
                                          "(their sub-step maps are built on first use)");
    if (op->state_len > kNoAllocMaxState)
        return fail(DGTD_ERR_INVALID, "dgtd_op_step_noalloc: state of " + std::to_string(op->state_len) +
                                          " entries exceeds the fixed scratch limit of " +
                                          std::to_string(kNoAllocMaxState) + " entries (6*K*Np*B)");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    try {
        double* ws = noalloc_scratch();
        double* state = static_cast<double*>(d_state);
        double* other = ws;   // LSERK4 second state buffer
        double* cur = state;
        // installed probes are sampled exactly as dgtd_op_step samples them (same step
        // counter, so the two calls can be mixed); their buffers were allocated when the
        // probes were installed, so sampling allocates nothing
        dgtd::ProbeSet* pr = op->probes.get();
        if (integrator == DGTD_LSERK4)
            ck(cudaMemsetAsync(ws + 2 * op->state_len, 0, op->state_len * sizeof(double), s), "memset");
        double t = t0;
        for (int i = 0; i < nsteps; ++i) {
            rk_step_at(op, ws, state, t, dt, integrator, other, cur, s);
            t += dt;
            if (pr && ++op->probe_steps % pr->every() == 0) {
                pr->sample(cur, t, s);
                g_launches.fetch_add(1, std::memory_order_relaxed);
            }
        }
        if (integrator == DGTD_LSERK4 && cur != state)
            ck(cudaMemcpyAsync(state, cur, op->state_len * sizeof(double), cudaMemcpyDeviceToDevice, s), "copy");
    } catch (const std::exception& e) {
        return fail(DGTD_ERR_CUDA, e.what());
    }
    return DGTD_OK;
}

}  // extern "C"
