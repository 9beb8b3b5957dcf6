// Second-order (curved) elements on the device: one block per curved element gathers its own
// state and its face neighbours' (5 x 6 Np values in shared memory) and applies the element's
// dense rows (transposed in memory: a thread per row reads consecutive entries), then writes the
// stage's register update exactly as the FP64 stage kernel writes it for straight elements.
#include "curved_dev.hpp"

#include <algorithm>
#include <stdexcept>
#include <string>

namespace dgtd {

namespace {

struct CurvedArgs {
    int64_t n;
    int Np;
    int64_t N;
    const int32_t* elems;
    const int32_t* nbr;
    const double* blocks;
};

__global__ void __launch_bounds__(256) curved_rows_kernel(CurvedArgs C, StageArgs A)
{
    extern __shared__ double xs[];   // [5][6 Np]
    const int Np = C.Np, R = 6 * Np;
    const int64_t N = C.N;
    const int64_t boff = static_cast<int64_t>(blockIdx.y) * 6 * N;   // incidence
    for (int64_t c = blockIdx.x; c < C.n; c += gridDim.x) {
        const int64_t e = C.elems[c];
        for (int w = threadIdx.x; w < 5 * R; w += blockDim.x) {
            const int blk = w / R, rr = w - blk * R, comp = rr / Np, j = rr - comp * Np;
            const int64_t src = (blk == 0) ? e : static_cast<int64_t>(C.nbr[4 * c + blk - 1]);
            xs[w] = (src >= 0) ? A.in[boff + comp * N + src * Np + j] : 0.0;
        }
        __syncthreads();
        for (int r = threadIdx.x; r < R; r += blockDim.x) {
            double k = 0.0;
            for (int blk = 0; blk < 5; ++blk) {
                if (blk > 0 && C.nbr[4 * c + blk - 1] < 0) continue;
                const double* BT = C.blocks + static_cast<size_t>(c * 5 + blk) * R * R;
                for (int col = 0; col < R; ++col) k = fma(BT[static_cast<size_t>(col) * R + r], xs[blk * R + col], k);
            }
            const int comp = r / Np, i = r - comp * Np;
            const int64_t o = boff + comp * N + e * Np + i;
            const double dt = A.dt;
            switch (A.mode) {
            case MODE_MULT: A.out[o] = k; break;
            case MODE_RK4_1: {
                const double xv = A.in[o];
                A.yout[o] = xv + 0.5 * dt * k;
                A.z[o] = xv + (dt / 6.0) * k;
                break;
            }
            case MODE_RK4_2: {
                const double xv = A.x[o];
                A.yout[o] = xv + 0.5 * dt * k;
                A.z[o] += (dt / 3.0) * k;
                break;
            }
            case MODE_RK4_3: {
                const double xv = A.x[o];
                A.yout[o] = xv + dt * k;
                A.z[o] += (dt / 3.0) * k;
                break;
            }
            case MODE_RK4_4: A.x[o] = A.z[o] + (dt / 6.0) * k; break;
            case MODE_LSRK: {
                const double rv = A.a * A.res[o] + dt * k;
                A.res[o] = rv;
                A.yout[o] = A.in[o] + A.b * rv;
                break;
            }
            default: break;
            }
        }
        __syncthreads();
    }
}

void ckc(cudaError_t e, const char* what)
{
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

}  // namespace

CurvedOp::CurvedOp(const MeshTables& T, const RefTet& ref, double alpha)
{
    const CurvedRows C = build_curved_rows(T, ref, alpha);
    Np_ = C.Np;
    n_ = static_cast<int64_t>(C.elems.size());
    // every index the kernel follows, checked once here
    if (static_cast<int64_t>(C.nbr.size()) != 4 * n_ ||
        static_cast<int64_t>(C.blocks.size()) != n_ * 5 * 36 * static_cast<int64_t>(Np_) * Np_ || Np_ != T.Np)
        throw std::runtime_error("curved rows: inconsistent tables");
    for (int32_t e : C.elems)
        if (e < 0 || e >= T.K) throw std::runtime_error("curved rows: element out of range");
    for (int32_t e : C.nbr)
        if (e < -1 || e >= T.K) throw std::runtime_error("curved rows: neighbour out of range");
    const int64_t R = 6 * static_cast<int64_t>(Np_);
    std::vector<double> bt(C.blocks.size());
    for (int64_t b = 0; b < 5 * n_; ++b)
        for (int64_t r = 0; r < R; ++r)
            for (int64_t col = 0; col < R; ++col) bt[(b * R + col) * R + r] = C.blocks[(b * R + r) * R + col];
    std::vector<uint8_t> fl(T.K, 0);
    for (int32_t e : C.elems) fl[e] = 1;
    try {
        ckc(cudaMalloc(&elems_, std::max<size_t>(1, C.elems.size()) * sizeof(int32_t)), "cudaMalloc curved");
        ckc(cudaMalloc(&nbr_, std::max<size_t>(1, C.nbr.size()) * sizeof(int32_t)), "cudaMalloc curved");
        ckc(cudaMalloc(&blocks_, std::max<size_t>(1, bt.size()) * sizeof(double)), "cudaMalloc curved rows");
        ckc(cudaMalloc(&flags_, std::max<size_t>(1, fl.size())), "cudaMalloc curved flags");
        ckc(cudaMemcpy(elems_, C.elems.data(), C.elems.size() * sizeof(int32_t), cudaMemcpyHostToDevice), "upload");
        ckc(cudaMemcpy(nbr_, C.nbr.data(), C.nbr.size() * sizeof(int32_t), cudaMemcpyHostToDevice), "upload");
        ckc(cudaMemcpy(blocks_, bt.data(), bt.size() * sizeof(double), cudaMemcpyHostToDevice), "upload");
        ckc(cudaMemcpy(flags_, fl.data(), fl.size(), cudaMemcpyHostToDevice), "upload");
    } catch (...) {
        release();
        throw;
    }
    bytes_ = static_cast<int64_t>(bt.size() * sizeof(double) + fl.size() + (C.elems.size() + C.nbr.size()) * 4);
}

CurvedOp::~CurvedOp() { release(); }

void CurvedOp::release()
{
    if (elems_) cudaFree(elems_);
    if (nbr_) cudaFree(nbr_);
    if (blocks_) cudaFree(blocks_);
    if (flags_) cudaFree(flags_);
    elems_ = nullptr; nbr_ = nullptr; blocks_ = nullptr; flags_ = nullptr;
}

void CurvedOp::apply(const TablesDev& T, const StageArgs& A, cudaStream_t s) const
{
    if (n_ == 0) return;
    CurvedArgs C{n_, Np_, T.N, elems_, nbr_, blocks_};
    const size_t shmem = static_cast<size_t>(5) * 6 * Np_ * sizeof(double);
    const dim3 grid(static_cast<unsigned>(std::min<int64_t>(n_, 4 * 152)), static_cast<unsigned>(std::max(1, A.batch)));
    curved_rows_kernel<<<grid, 256, shmem, s>>>(C, A);
    ckc(cudaGetLastError(), "curved-element kernel");
}

}  // namespace dgtd
