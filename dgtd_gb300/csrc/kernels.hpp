// Device-side data structures and kernel launchers of the DG Maxwell step.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace dgtd {

// One plane-wave source (reference: Planewave + Gaussian/ModulatedGaussian,
// src/math/Function.h:45-143, 329-416; built by driver.cpp:483-519).
// E = g(x.k - t) pol,  H = g(x.k - t) (k x pol),  g(s) = exp(-(s-mean)^2/(2 spread^2))
// [* cos(2 pi freq (s - mean)) when freq != 0].
struct PlaneWaveDev {
    double k[3];
    double pol[3];
    double kxp[3];
    double spread;
    double mean;
    double freq;
    int batch;      // incidence index the source belongs to
    int pad;
};

// Epilogue of the fused RHS kernel.
enum StageMode : int {
    MODE_MULT = 0,     // out = L(in)
    MODE_RK4_1 = 1,    // y_out = x + dt/2 k ; z = x + dt/6 k           (in = x)
    MODE_RK4_2 = 2,    // y_out = x + dt/2 k ; z += dt/3 k              (in = y)
    MODE_RK4_3 = 3,    // y_out = x + dt k   ; z += dt/3 k              (in = y)
    MODE_RK4_4 = 4,    // x = z + dt/6 k                                 (in = y)
    MODE_LSRK = 5,     // res = a res + dt k ; u_out = u_in + b res      (in = u_in)
};

// Per-mesh device tables of the plain (thread-per-node) form, in the arithmetic
// type R of that form: double for the FP64 form, float for the single-instance
// FP32 form.
template <typename R>
struct TablesT {
    int p, Np, Nfp;
    int64_t K;
    int64_t N;                 // K * Np
    const R* DrT;              // [Np][Np] transposed
    const R* DsT;
    const R* DtT;
    const R* LIFTT;            // [4 Nfp][Np] transposed
    const int* Fmask;          // [4][Nfp]
    const R* geo;              // [K][9]
    const R* fgeo;             // [K][16]
    const R* mat;              // [K][3]
    const int32_t* vmapP;      // [K][4][Nfp]
    const int32_t* fcode;      // [K][4]
    const R* xyz;              // [3][N]
    const int32_t* tfsf_elems; // [n_tfsf_elems]
    int64_t n_tfsf_elems;
    R alpha;
    const uint8_t* curved;     // [K] 1: the element's rows come from the curved-element kernel (the
                               // stage leaves its outputs alone); nullptr: no curved elements
};

template <typename R>
struct StageArgsT {
    const R* in;         // [B][6][N]
    R* out;              // MULT output
    R* x;                // RK4 base state
    R* yout;             // RK4 stage output
    R* z;                // RK4 accumulator
    R* res;              // LSRK residual
    double t;            // stage time
    R dt;
    R a, b;              // LSRK coefficients
    int mode;
    int batch;           // B
    const PlaneWaveDev* pw;
    int n_pw;
    const int* skip;     // [B] TF/SF skip flags (nullptr: never skip)
};

using TablesDev = TablesT<double>;
using StageArgs = StageArgsT<double>;
using TablesF32 = TablesT<float>;
using StageArgsF32 = StageArgsT<float>;

// Launch the fused FP64 RHS + stage-update kernel for one stage.
cudaError_t launch_stage_fp64(const TablesDev& T, const StageArgs& A, cudaStream_t s);

// Per-incidence TF/SF skip decision (reference GlobalEvolution.cpp:587-598):
// skip[b] = (sum over TF/SF-submesh nodes and components of (0.5 pw)^2 < 1e-16).
// The sum is split over `parts` blocks per incidence (partial: batch x parts doubles; ticket:
// batch counters, zero between launches).
struct SkipScratch {
    double* partial = nullptr;
    unsigned int* ticket = nullptr;
    int parts = 1;
};

// Blocks per incidence of the split skip test: about 8192 TF/SF nodes per block, 1..64.
inline int tfsf_skip_parts(int64_t tfsf_nodes)
{
    const int64_t p = (tfsf_nodes + 8191) / 8192;
    return static_cast<int>(p < 1 ? 1 : (p > 64 ? 64 : p));
}
cudaError_t launch_tfsf_skip(const TablesDev& T, const PlaneWaveDev* pw, int n_pw, int batch,
                             double t, int* skip, const SkipScratch& sc, cudaStream_t s);

// Squared L2 norm of each incidence's state: out[b] = sum_i in[b][i]^2.
cudaError_t launch_norm2(const double* in, int64_t n_per_batch, int batch, double* out, cudaStream_t s);

// Single-instance FP32 form (single_f32.cu): the same fused stage in FP32 on the
// reference layout, one thread per node.
cudaError_t launch_stage_f32s(const TablesF32& T, const StageArgsF32& A, cudaStream_t s);
cudaError_t launch_tfsf_skip_f32s(const TablesF32& T, const PlaneWaveDev* pw, int n_pw, int batch, double t, int* skip,
                                  const SkipScratch& sc, cudaStream_t s);
cudaError_t launch_norm2_f32s(const float* in, int64_t n_per_batch, int batch, double* out, cudaStream_t s);
cudaError_t launch_convert_f64_to_f32(const double* in, float* out, int64_t n, cudaStream_t s);
cudaError_t launch_convert_f32_to_f64(const float* in, double* out, int64_t n, cudaStream_t s);

// Instability detector of the run loop (stability.cu; reference Solver.cpp:500-516): a state
// whose L2 norm is not finite or above kUnstableNorm. The record lives in device memory;
// first_step < 0 while no check has tripped.
constexpr double kUnstableNorm = 1e20;
struct StabilityRecord {
    double sumsq;          // running sum of the current check (zero between checks)
    int64_t first_step;    // step count of the first check that tripped, or -1
    double t;              // its time
    double norm;           // its norm (NaN or infinity when the state was not finite)
    int64_t checks;        // checks run since the record was reset
};
// One check of n entries (FP32 or FP64) at step `step`, time t: two launches, no sync.
cudaError_t launch_stability_check(const void* state, int64_t n, bool f32, StabilityRecord* rec, int64_t step,
                                   double t, int n_sm, cudaStream_t s);

}  // namespace dgtd
