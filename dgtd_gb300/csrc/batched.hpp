// Batched FP32 form of the DG Maxwell step: B incidences share one mesh.
//
// Internal layout (private to this form): state[e'][c][i][b] in FP32 with the
// incidence index b fastest (B padded to a multiple of 32), elements e' in a
// space-filling-curve (Morton) order of their centroids so that face
// neighbours are processed close in time and their traces stay in L2.
// dgtd_op_pack / dgtd_op_unpack convert to and from the reference layout.
#pragma once
#include <cstdint>
#include <memory>
#include <vector>

#include <cuda_runtime.h>

#include "kernels.hpp"
#include "mesh.hpp"
#include "refelem.hpp"

namespace dgtd {

struct PlaneWaveF32 {
    float k[3], pol[3], kxp[3];
    float spread, mean, freq;
    int batch, pad;
};

struct BatchedTables {
    int p, Np, Nfp, B, Bpad;
    int64_t K;
    const float* D;        // [3][Np][Np]   Dr, Ds, Dt (row i, column j)
    const float* LIFT;     // [Np][4 Nfp]
    const int* Fmask;      // [4][Nfp]
    const float* geo;      // [K][9]
    const float* fgeo;     // [K][16]
    const float* mat;      // [K][3]
    const int32_t* vmapP;  // [K][4][Nfp]  neighbour (element' * Np + node), internal numbering
    const int32_t* fcode;  // [K][4]
    const float* fbc;      // [K][4][5] per face: jump coefficients cE1 cE2 cH1 cH2 (dE = cE1 E+ + cE2 E-,
                           // dH = cH1 H+ + cH2 H-) and the penalty coefficient of the face
    const float* fxyz;     // [K][4][Nfp][3] face-node coordinates (TF/SF source evaluation)
    const float* nxyz;     // [3][n_tfsf_nodes] coordinates of the TF/SF-submesh nodes (skip test)
    int64_t n_tfsf_nodes;
    float alpha;
};

// Classical RK4 in the batched form keeps the state register as an unevaluated sum of two FP32
// words, x = x_hi + x_lo (the working state is [x_hi block | x_lo block]), and the register z as
// the accumulated increment dt (k1/6 + k2/3 + k3/3) rather than x plus it. Stages read x_hi
// only; the last stage adds the increment to (x_hi, x_lo) with an error-free two-sum, so the
// state update itself does not round at FP32 precision every step.
struct BatchedStageArgs {
    const float* in;
    float* out;
    float* x;
    float* xl;               // x_lo (RK4 stage 4)
    float* yout;
    float* z;
    float* res;
    float t, dt, a, b;       // stage time: t, or *t_base + t when t_base is set (CUDA-graph replay)
    const double* t_base;    // device block start time (graph replay), else nullptr
    int mode;
    const PlaneWaveF32* pw;  // sources sorted by incidence
    const int* pw_off;       // [Bpad + 1]: sources of incidence b are pw[pw_off[b] .. pw_off[b+1])
    const int* skip;         // [Bpad]
};

#ifdef __CUDACC__
// (hi, lo) += inc with an error-free two-sum (Knuth) and a renormalisation: hi + lo carries
// the state to about 2^-48 relative, so the RK4 state update does not round each step.
// Explicitly rounded additions, so that nothing is contracted into a fused multiply-add.
__device__ __forceinline__ void add_compensated(float& hi, float& lo, float inc)
{
    const float s = __fadd_rn(hi, inc);
    const float bb = __fsub_rn(s, hi);
    const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(inc, bb));
    const float l2 = __fadd_rn(lo, err);
    const float h2 = __fadd_rn(s, l2);
    lo = __fsub_rn(l2, __fsub_rn(h2, s));
    hi = h2;
}

// bf16 bits -> FP32 (exact)
__device__ __forceinline__ float bf16_bits_to_float(uint16_t h) { return __uint_as_float(static_cast<uint32_t>(h) << 16); }
#endif

// Tensor-core stage kernel (batched_tc.cu).
bool tc_supported(int p, int Bpad);
std::vector<uint32_t> tc_operator_image(const RefTet& ref);
void launch_stage_tc(const BatchedTables& T, const BatchedStageArgs& A, const uint32_t* op_img, int* status, int n_sm,
                     cudaStream_t s);

class BatchedOp {
public:
    static std::unique_ptr<BatchedOp> create(const RefTet& ref, const MeshTables& mesh, const TablesDev& dev, int batch);
    ~BatchedOp();
    void set_sources(const std::vector<PlaneWaveDev>& pw);
    int64_t device_bytes() const { return device_bytes_; }
    int64_t state_len() const { return state_len_; }       // floats of one internal state (x_hi block)
    int64_t work_len() const { return 2 * state_len_; }    // floats of the working state: x_hi and x_lo
    int64_t kernel_launches() const { return launches_; }
    int batch_padded() const { return Bpad_; }
    // internal (Morton) index of each reference element, host copy
    const std::vector<int32_t>& inv_perm() const { return inv_perm_host_; }

    // reference layout (FP64, [b][c][e*Np+i]) <-> internal FP32 pair (x_hi = fl(x), x_lo = fl(x - x_hi))
    // ref_on_host: the reference-layout buffer is pinned host memory read or written over the
    // host link (larger tiles: longer contiguous runs per incidence row)
    void pack(const double* d_ref, float* d_state, cudaStream_t s, bool ref_on_host = false);
    void unpack(const float* d_state, double* d_ref, cudaStream_t s, bool ref_on_host = false);
    void mult(const float* d_in, float* d_out, double t, cudaStream_t s);
    void step(float* d_state, double t0, double dt, int nsteps, int integrator, cudaStream_t s);
    void norm2(const float* d_state, double* d_out_dev, cudaStream_t s);
    // contraction path: 0 = tensor cores (tcgen05, 3xTF32) when supported, 1 = FP32 SIMT
    void set_contraction(int mode) { contraction_ = mode; }
    // Times the candidate stage kernels (tensor cores where supported; FP32 SIMT with 4, 8
    // and 16 warps per block) on this operator's mesh with MODE_MULT launches on d_in and
    // keeps the fastest. ms[4] gets the mean launch time of each candidate (-1: not
    // applicable); returns the chosen index. The choice is cached per (order, Bpad, K).
    int autotune(const float* d_in, double* ms, cudaStream_t s);
    // RK4 steps per captured CUDA graph (0: launch every stage directly)
    void set_graph_steps(int g);
    bool uses_tensor_cores() const { return contraction_ == 0 && tc_supported(T_.p, Bpad_); }
    // reads and clears the device error flag (synchronises the stream)
    int take_status(cudaStream_t s);
    // FP64 defect correction (bf16 c and its step increment inc: state_len() entries each,
    // internal layout of one state block).
    // c = (ref_hi - l32) + ref_lo, where ref is a working state (pair) holding the FP64 operator's
    // product and l32 the hi block of this form's product of the state x (a working state), kept
    // only where x_hi has stayed within 0.1 of the incidence's RMS value of x_prev, its value at
    // the previous refresh (x_prev is then overwritten with x_hi; NaN entries never match).
    // sumsq: Bpad doubles of device scratch.
    void build_correction(const float* ref_pair, const float* l32, const float* x, float* x_prev, double* sumsq,
                          uint16_t* c, cudaStream_t s);
    // inc = one classical RK4 step of size dt from the zero state under the constant forcing c,
    // with the source-free operator A: dt/6 (k1 + 2 k2 + 2 k3 + k4), k1 = c, k2 = A (dt/2 k1) + c,
    // k3 = A (dt/2 k2) + c, k4 = A (dt k3) + c. The operator is linear, so a step of
    // u' = Au + s(t) + c equals the step of u' = Au + s(t) plus inc. scratch_a, scratch_b: working
    // states (2 state_len() floats each).
    void build_increment(const uint16_t* c, float* scratch_a, float* scratch_b, uint16_t* inc, double dt,
                         cudaStream_t s);
    // x_lo += inc over the working state x
    void add_increment(float* x, const uint16_t* inc, cudaStream_t s);

private:
    void stage(BatchedStageArgs A, double t, cudaStream_t s);
    unsigned stream_grid() const;   // grid of the elementwise kernels over one state block
    void ensure_ws();
    void rk4_steps_direct(float* d_x, double t, double dt, int nsteps, cudaStream_t s);
    void drop_graph();

    BatchedTables T_{};
    int64_t K_ = 0;
    int Np_ = 0, B_ = 0, Bpad_ = 0;
    int64_t state_len_ = 0;
    int64_t device_bytes_ = 0;
    int64_t launches_ = 0;
    std::vector<void*> allocs_;
    int32_t* inv_perm_ = nullptr;   // reference element -> internal element
    std::vector<int32_t> inv_perm_host_;
    PlaneWaveF32* pw_dev_ = nullptr;
    int* pw_off_ = nullptr;
    int n_pw_ = 0, pw_cap_ = 0;
    int* skip_ = nullptr;
    double* skip_partial_ = nullptr;      // [Bpad][parts] partial sums of the skip test
    unsigned int* skip_ticket_ = nullptr; // [Bpad] blocks finished per incidence
    float* ws_ = nullptr;
    bool has_tfsf_ = false;
    int contraction_ = 0;
    int simt_warps_ = 8;
    // CUDA graph of graph_steps_ RK4 steps (stage times relative to the device scalar t_dev_)
    int graph_steps_ = 0;
    double* t_dev_ = nullptr;
    cudaGraphExec_t gexec_ = nullptr;
    float* g_x_ = nullptr;
    double g_dt_ = 0.0;
    cudaStream_t g_stream_ = nullptr;
    int g_contraction_ = -1;
    int64_t g_graph_launches_ = 0;   // kernels in one replay
    bool no_sources_ = false;        // stages without the TF/SF sources (build_increment)
    const uint32_t* op_img_ = nullptr;
    int* status_ = nullptr;
    int n_sm_ = 152;
};

}  // namespace dgtd
