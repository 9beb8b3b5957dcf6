// Instability detector of the run loop (reference Solver::run, src/solver/Solver.cpp:500-516):
// the L2 norm of the whole state, flagged when it is not finite or above 1e20.
//
// Two launches per check, no host synchronisation: a grid-stride sum of squares that
// adds each block's partial sum into the record, then one thread that takes the square
// root, records the first check that tripped (step, time, norm) and clears the sum for
// the next check. The host reads the record when it chooses (every few hundred steps
// and at the end of a run). A NaN or an infinity anywhere in the state makes the sum
// NaN or infinite, so the one comparison !(norm <= 1e20) covers both conditions.
#include <cuda_runtime.h>

#include "kernels.hpp"

namespace dgtd {

namespace {

constexpr int kThreadsStab = 256;

template <typename T>
__global__ void __launch_bounds__(kThreadsStab) stability_sumsq(const T* __restrict__ x, int64_t n,
                                                                 StabilityRecord* rec)
{
    double acc = 0.0;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(kThreadsStab) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * kThreadsStab) {
        const double v = static_cast<double>(x[i]);
        acc += v * v;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    __shared__ double warp_sum[kThreadsStab / 32];
    if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < kThreadsStab / 32; ++w) s += warp_sum[w];
        atomicAdd(&rec->sumsq, s);
    }
}

__global__ void stability_record(StabilityRecord* rec, int64_t step, double t)
{
    const double norm = sqrt(rec->sumsq);
    rec->sumsq = 0.0;
    rec->checks += 1;
    if (!(norm <= kUnstableNorm) && rec->first_step < 0) {
        rec->first_step = step;
        rec->t = t;
        rec->norm = norm;
    }
}

}  // namespace

cudaError_t launch_stability_check(const void* state, int64_t n, bool f32, StabilityRecord* rec, int64_t step,
                                   double t, int n_sm, cudaStream_t s)
{
    const int64_t want = (n + kThreadsStab * 8 - 1) / (kThreadsStab * 8);
    const int64_t cap = static_cast<int64_t>(n_sm > 0 ? n_sm : 152) * 8;
    const unsigned grid = static_cast<unsigned>(want < 1 ? 1 : (want > cap ? cap : want));
    if (f32)
        stability_sumsq<float><<<grid, kThreadsStab, 0, s>>>(static_cast<const float*>(state), n, rec);
    else
        stability_sumsq<double><<<grid, kThreadsStab, 0, s>>>(static_cast<const double*>(state), n, rec);
    stability_record<<<1, 1, 0, s>>>(rec, step, t);
    return cudaGetLastError();
}

}  // namespace dgtd
