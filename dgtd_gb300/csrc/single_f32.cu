// Single-instance FP32 form: the plain form's fused stage (fp64_stage.cuh, one
// thread per node, elements staged in shared memory) instantiated in FP32 on
// the reference state layout [b][c][e*Np+i]. For single solves of high order
// (one incidence: the batched form's incidence lanes would stay empty), this
// runs the contractions on the FP32 pipe (about 50x the FP64 pipe of a GB300)
// and halves the bytes per DOF. Tables are built in FP64 on the host and rounded
// once.
#include "fp64_stage.cuh"

namespace dgtd {

namespace {

using fp64::kBlock;
using fp64::Ord;

template <int P>
__global__ void __launch_bounds__(kBlock) stage_f32s(TablesF32 T, StageArgsF32 A)
{
    fp64::stage_body<P, float>(T, A, static_cast<int64_t>(blockIdx.x) * Ord<P, float>::EPB, static_cast<int>(blockIdx.y));
}

__global__ void __launch_bounds__(256) tfsf_skip_f32s(TablesF32 T, const PlaneWaveDev* pw, int n_pw, double t,
                                                      double* partial, unsigned int* ticket, int* skip)
{
    fp64::tfsf_skip_part_body<float>(T, pw, n_pw, static_cast<int>(blockIdx.x), t, partial, ticket, skip);
}

__global__ void __launch_bounds__(256) norm2_f32s(const float* in, int64_t n, double* out)
{
    const int b = blockIdx.x;
    const float* p = in + static_cast<int64_t>(b) * n;
    double acc = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) acc += static_cast<double>(p[i]) * p[i];
    __shared__ double red[256];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[b] = red[0];
}

__global__ void f64_to_f32(const double* __restrict__ in, float* __restrict__ out, int64_t n)
{
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        out[i] = static_cast<float>(in[i]);
}

__global__ void f32_to_f64(const float* __restrict__ in, double* __restrict__ out, int64_t n)
{
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        out[i] = static_cast<double>(in[i]);
}

template <int P>
cudaError_t launch_p(const TablesF32& T, const StageArgsF32& A, cudaStream_t s)
{
    dim3 grid(static_cast<unsigned>((T.K + Ord<P, float>::EPB - 1) / Ord<P, float>::EPB), static_cast<unsigned>(A.batch));
    stage_f32s<P><<<grid, kBlock, 0, s>>>(T, A);
    return cudaGetLastError();
}

unsigned grid_for(int64_t n) { return static_cast<unsigned>(std::min<int64_t>((n + 255) / 256, 152 * 32)); }

}  // namespace

cudaError_t launch_stage_f32s(const TablesF32& T, const StageArgsF32& A, cudaStream_t s)
{
    switch (T.p) {
    case 1: return launch_p<1>(T, A, s);
    case 2: return launch_p<2>(T, A, s);
    case 3: return launch_p<3>(T, A, s);
    case 4: return launch_p<4>(T, A, s);
    case 5: return launch_p<5>(T, A, s);
    case 6: return launch_p<6>(T, A, s);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_tfsf_skip_f32s(const TablesF32& T, const PlaneWaveDev* pw, int n_pw, int batch, double t, int* skip,
                                  const SkipScratch& sc, cudaStream_t s)
{
    tfsf_skip_f32s<<<dim3(batch, sc.parts), 256, 0, s>>>(T, pw, n_pw, t, sc.partial, sc.ticket, skip);
    return cudaGetLastError();
}

cudaError_t launch_norm2_f32s(const float* in, int64_t n_per_batch, int batch, double* out, cudaStream_t s)
{
    norm2_f32s<<<batch, 256, 0, s>>>(in, n_per_batch, out);
    return cudaGetLastError();
}

cudaError_t launch_convert_f64_to_f32(const double* in, float* out, int64_t n, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    f64_to_f32<<<grid_for(n), 256, 0, s>>>(in, out, n);
    return cudaGetLastError();
}

cudaError_t launch_convert_f32_to_f64(const float* in, double* out, int64_t n, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    f32_to_f64<<<grid_for(n), 256, 0, s>>>(in, out, n);
    return cudaGetLastError();
}

}  // namespace dgtd
