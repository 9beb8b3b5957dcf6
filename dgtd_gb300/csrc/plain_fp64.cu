// Plain FP64 form of the DG Maxwell step: one fused kernel per RK stage over
// one operator's mesh (grid: element blocks x incidences), plus the TF/SF
// skip test and the per-incidence norm. The stage arithmetic (reference
// HesthavenEvolution::Mult, src/evolution/HesthavenEvolution.cpp:450-541, with
// the RK4 register updates of mfem::RK4Solver, src/solver/Solver.cpp:544) is
// in fp64_stage.cuh.
#include "fp64_stage.cuh"

namespace dgtd {

namespace {

using fp64::Ord;
using fp64::kBlock;

template <int P>
__global__ void __launch_bounds__(kBlock) stage_fp64(TablesDev T, StageArgs A)
{
    fp64::stage_body<P>(T, A, static_cast<int64_t>(blockIdx.x) * Ord<P>::EPB, static_cast<int>(blockIdx.y));
}

// Small meshes: blocks of about 64 threads, so that the grid spreads over every SM evenly
// (3,072 tets at p = 3 give 256 blocks of 240 threads, 0.56 waves, but 1,024 of 60).
// Orders 1-3 run the staged body (operators and face tables brought into shared memory by bulk
// copies, in-block face partners read from shared memory); it fits the static shared-memory limit
// with these small blocks.
template <int P>
__global__ void __launch_bounds__(Ord<P>::BLOCK_SMALL) stage_fp64_small(TablesDev T, StageArgs A)
{
    fp64::stage_body<P, double, Ord<P>::EPB_SMALL, (P <= 3)>(T, A, static_cast<int64_t>(blockIdx.x) * Ord<P>::EPB_SMALL,
                                                             static_cast<int>(blockIdx.y));
}

// below this many default blocks (4 per SM of a 152-SM GB300) the small-block variant is used
constexpr int64_t kSmallGridBlocks = 4 * 152;

__global__ void __launch_bounds__(256) tfsf_skip_kernel(TablesDev T, const PlaneWaveDev* pw, int n_pw, double t,
                                                        double* partial, unsigned int* ticket, int* skip)
{
    fp64::tfsf_skip_part_body(T, pw, n_pw, static_cast<int>(blockIdx.x), t, partial, ticket, skip);
}

__global__ void norm2_kernel(const double* in, int64_t n, double* out)
{
    const int b = blockIdx.x;
    const double* p = in + static_cast<int64_t>(b) * n;
    double acc = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) acc += p[i] * p[i];
    __shared__ double red[256];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[b] = red[0];
}

template <int P>
cudaError_t launch_p(const TablesDev& T, const StageArgs& A, cudaStream_t s)
{
    using O = Ord<P>;
    const int64_t blocks = (T.K + O::EPB - 1) / O::EPB;
    if (blocks * A.batch < kSmallGridBlocks) {
        dim3 grid(static_cast<unsigned>((T.K + O::EPB_SMALL - 1) / O::EPB_SMALL), static_cast<unsigned>(A.batch));
        stage_fp64_small<P><<<grid, O::BLOCK_SMALL, 0, s>>>(T, A);
        return cudaGetLastError();
    }
    dim3 grid(static_cast<unsigned>(blocks), static_cast<unsigned>(A.batch));
    stage_fp64<P><<<grid, kBlock, 0, s>>>(T, A);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_stage_fp64(const TablesDev& T, const StageArgs& A, cudaStream_t s)
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

cudaError_t launch_tfsf_skip(const TablesDev& T, const PlaneWaveDev* pw, int n_pw, int batch, double t, int* skip,
                             const SkipScratch& sc, cudaStream_t s)
{
    tfsf_skip_kernel<<<dim3(batch, sc.parts), 256, 0, s>>>(T, pw, n_pw, t, sc.partial, sc.ticket, skip);
    return cudaGetLastError();
}

cudaError_t launch_norm2(const double* in, int64_t n_per_batch, int batch, double* out, cudaStream_t s)
{
    norm2_kernel<<<batch, 256, 0, s>>>(in, n_per_batch, out);
    return cudaGetLastError();
}

}  // namespace dgtd
