// Batched FP32 stage kernel with the contractions on the tensor cores (tcgen05, 3xTF32).
//
// For one element e and one chunk of 64 incidences the right-hand side of all
// six field components is a single tall-skinny product
//
//   RHS^T[(c,b), i] = sum_k W[(c,b), k] * Op[k, i],  Op = [Dr | Ds | Dt | LIFT]^T,
//
// with W the per-element operand built on the fly:
//   k in [0, 3Np)      : (g_r x F, g_s x F, g_t x F) at node k mod Np, where F is the
//                        partner field (H for E targets, -E for H targets) and g_r, g_s, g_t
//                        the element's geometric factors (rows of d(r,s,t)/dx) -- so the
//                        product is the curl (reference HesthavenEvolution.cpp:522-534);
//   k in [3Np, 3Np+4Nfp): Fscale/2 * upwind flux at face node k - 3Np (:509-520).
// Rows (c, b) are 6 components x 64 incidences = 3 M-tiles of 128; N = Np padded
// to 16; K = 3Np + 4Nfp padded to 8. The A operand is split into tf32 hi/lo and the
// constant Op is stored as hi/lo, giving A_hi Op_hi + A_lo Op_hi + A_hi Op_lo
// (3xTF32, FP32-level accuracy). The accumulators live in tensor memory; the
// epilogue applies 1/eps, 1/mu, the conductivity term and the RK stage update.
//
// Per CTA (persistent, 2 per SM): Op hi/lo resident in shared memory, a 2-slot
// ring of A-operand K-steps (producer threads write slot q%2 while the tensor
// core consumes the other), tcgen05.commit -> mbarrier per slot.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <vector>
#include <string>

#include "batched.hpp"
#include "tc_common.cuh"

namespace dgtd {

namespace {

constexpr int kThreads = 256;
constexpr int kChunk = 64;          // incidences per work item
constexpr int kTileBytes = 4096;    // 128 rows x 8 tf32

template <int P>
struct TcOrd {
    static constexpr int Np = (P + 1) * (P + 2) * (P + 3) / 6;
    static constexpr int Nfp = (P + 1) * (P + 2) / 2;
    static constexpr int NF = 4 * Nfp;
    static constexpr int KK = 3 * Np + NF;
    static constexpr int KKp = (KK + 7) / 8 * 8;
    static constexpr int NKS = KKp / 8;
    static constexpr int N = (Np + 15) / 16 * 16;
    static constexpr int OpStep = N * 32;                 // bytes of one K-step of Op (N rows x 8 tf32)
    static constexpr int OpBytes = NKS * OpStep;          // per hi / lo
    static constexpr int SlotBytes = 3 * kTileBytes;      // 3 M-tiles of one K-step, per hi / lo
    static constexpr int TmemCols = 256;
    static constexpr size_t smem = 2 * static_cast<size_t>(OpBytes) + 2 * 2 * SlotBytes;
};

__device__ __forceinline__ void pw_eval(const PlaneWaveF32* pw, const int* pw_off, int b, float px, float py, float pz, float t,
                                        float* e, float* h)
{
    e[0] = e[1] = e[2] = h[0] = h[1] = h[2] = 0.0f;
    const int q1 = pw_off[b + 1];
    for (int q = pw_off[b]; q < q1; ++q) {
        const PlaneWaveF32& w = pw[q];
        const float s = px * w.k[0] + py * w.k[1] + pz * w.k[2] - t;
        const float a = s - w.mean;
        float g = expf(-a * a / (2.0f * w.spread * w.spread));
        if (w.freq != 0.0f) g *= cosf(6.283185307179586f * w.freq * a);
        e[0] += g * w.pol[0]; e[1] += g * w.pol[1]; e[2] += g * w.pol[2];
        h[0] += g * w.kxp[0]; h[1] += g * w.kxp[1]; h[2] += g * w.kxp[2];
    }
}

__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float* v)
{
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

template <int P>
__global__ void __launch_bounds__(kThreads, 2) stage_tc(BatchedTables T, BatchedStageArgs A, const uint32_t* __restrict__ op_img,
                                                     int64_t n_work, int* status)
{
    using O = TcOrd<P>;
    constexpr int Np = O::Np, Nfp = O::Nfp, NF = O::NF, NKS = O::NKS, N = O::N;
    // no-swizzle descriptors need 16-byte aligned operands only
    extern __shared__ __align__(128) unsigned char sm[];
    unsigned char* op_hi = sm;
    unsigned char* op_lo = op_hi + O::OpBytes;
    unsigned char* ring = op_lo + O::OpBytes;               // [slot][hi/lo][3 tiles]
    __shared__ uint64_t bars[2];
    __shared__ uint32_t tbase;
    __shared__ int s_fmask[NF];
    __shared__ int s_err;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // producer mapping: incidence bl and a pair of K columns (kq); all six target components
    const int bl = tid & 63, kq = tid >> 6;
    const int64_t Bp = T.Bpad;
    const int nchunk = static_cast<int>(Bp / kChunk);
    const int CB = Np * static_cast<int>(Bp);          // stride of one component inside an element block
    const int64_t EB = 6 * static_cast<int64_t>(CB);   // stride of one element block

    // ---- prologue: operator image, face mask, barriers, tensor memory
    {
        const uint4* src = reinterpret_cast<const uint4*>(op_img);
        uint4* dst = reinterpret_cast<uint4*>(op_hi);
        for (int i = tid; i < 2 * O::OpBytes / 16; i += kThreads) dst[i] = src[i];
    }
    for (int i = tid; i < NF; i += kThreads) s_fmask[i] = T.Fmask[i];
    if (tid == 0) {
        tc::mbar_init(&bars[0], 1);
        tc::mbar_init(&bars[1], 1);
        tc::mbar_fence_init();
        s_err = 0;
    }
    if (warp == 0) {
        tc::tmem_alloc(&tbase, O::TmemCols);
        tc::tmem_relinquish();
    }
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t taddr = tbase;
    const uint32_t idesc = tc::idesc_tf32(128, N);
    uint32_t ncommit0 = 0, ncommit1 = 0;     // commits issued per ring slot (uniform in all threads)
    const float dtf = A.dt;

    for (int64_t w = blockIdx.x; w < n_work; w += gridDim.x) {
        const int64_t e = w / nchunk;
        const int g = static_cast<int>(w - e * nchunk);
        const int b = g * kChunk + bl;                   // incidence of this thread's row
        const int64_t eoff = e * EB + static_cast<int64_t>(g) * kChunk;
        const float* __restrict__ ue = A.in + eoff;      // element block of the stage input
        const float* gg = T.geo + e * 9;
        const float g0 = __ldg(gg + 0), g1 = __ldg(gg + 1), g2 = __ldg(gg + 2), g3 = __ldg(gg + 3),
                    g4 = __ldg(gg + 4), g5 = __ldg(gg + 5), g6 = __ldg(gg + 6), g7 = __ldg(gg + 7), g8 = __ldg(gg + 8);
        const bool skip_src = (A.skip == nullptr) || A.skip[b];

        for (int q = 0; q < NKS; ++q) {
            const int slot = q & 1;
            if (q >= 2) {
                const uint32_t nc = slot ? ncommit1 : ncommit0;
                if (!tc::mbar_wait(&bars[slot], (nc - 1) & 1u)) s_err = 1;
            }
            // ---- produce K-step q: columns k0, k0+1 for all six target components
            float v[6][2];
#pragma unroll
            for (int kk = 0; kk < 2; ++kk) {
                const int k = q * 8 + kq * 2 + kk;
                if (k < 3 * Np) {
                    const int type = k / Np, j = k - type * Np;
                    const float gx = type == 0 ? g0 : (type == 1 ? g3 : g6);
                    const float gy = type == 0 ? g1 : (type == 1 ? g4 : g7);
                    const float gz = type == 0 ? g2 : (type == 1 ? g5 : g8);
                    const int o = j * static_cast<int>(Bp) + bl;
                    const float Ex = __ldg(ue + o), Ey = __ldg(ue + o + CB), Ez = __ldg(ue + o + 2 * CB);
                    const float Hx = __ldg(ue + o + 3 * CB), Hy = __ldg(ue + o + 4 * CB), Hz = __ldg(ue + o + 5 * CB);
                    // E targets: g x H (curl H); H targets: -(g x E) (-curl E)
                    v[0][kk] = gy * Hz - gz * Hy;
                    v[1][kk] = gz * Hx - gx * Hz;
                    v[2][kk] = gx * Hy - gy * Hx;
                    v[3][kk] = gz * Ey - gy * Ez;
                    v[4][kk] = gx * Ez - gz * Ex;
                    v[5][kk] = gy * Ex - gx * Ey;
                } else if (k < 3 * Np + NF) {
                    const int m = k - 3 * Np, f = m / Nfp, a = m - f * Nfp;
                    const int vm = s_fmask[m];
                    const int code = __ldg(T.fcode + e * 4 + f);
                    const float* fg = T.fgeo + e * 16 + f * 4;
                    const float nx = __ldg(fg), ny = __ldg(fg + 1), nz = __ldg(fg + 2), fs = __ldg(fg + 3);
                    const int o = vm * static_cast<int>(Bp) + bl;
                    float uM[6];
#pragma unroll
                    for (int c = 0; c < 6; ++c) uM[c] = __ldg(ue + o + c * CB);
                    float dE[3], dH[3];
                    float aE = T.alpha, aH = T.alpha;
                    if (code == 0 || code == 4 || code == 5) {
                        const int32_t gp = __ldg(T.vmapP + (e * 4 + f) * Nfp + a);
                        const int32_t en = gp / Np, node = gp - en * Np;
                        const float* __restrict__ un = A.in + static_cast<int64_t>(en) * EB +
                                                       static_cast<int64_t>(g) * kChunk + node * static_cast<int>(Bp) + bl;
#pragma unroll
                        for (int c = 0; c < 3; ++c) {
                            dE[c] = __ldg(un + c * CB) - uM[c];
                            dH[c] = __ldg(un + (c + 3) * CB) - uM[c + 3];
                        }
                        if (code != 0 && !skip_src) {
                            const float* xq = T.fxyz + ((e * 4 + f) * Nfp + a) * 3;
                            float pe[3], ph[3];
                            pw_eval(A.pw, A.pw_off, b, __ldg(xq), __ldg(xq + 1), __ldg(xq + 2), A.t, pe, ph);
                            const float s2 = (code == 4) ? 1.0f : -1.0f;
#pragma unroll
                            for (int c = 0; c < 3; ++c) { dE[c] += s2 * pe[c]; dH[c] += s2 * ph[c]; }
                        }
                    } else if (code == 1 || code == 6) {
#pragma unroll
                        for (int c = 0; c < 3; ++c) { dE[c] = -2.0f * uM[c]; dH[c] = 0.0f; }
                    } else if (code == 2 || code == 7) {
#pragma unroll
                        for (int c = 0; c < 3; ++c) { dE[c] = 0.0f; dH[c] = -2.0f * uM[c + 3]; }
                    } else if (code == 3 || code == 8) {
#pragma unroll
                        for (int c = 0; c < 3; ++c) { dE[c] = -uM[c]; dH[c] = -uM[c + 3]; }
                        aE = 1.0f; aH = 1.0f;
                    } else {
#pragma unroll
                        for (int c = 0; c < 3; ++c) { dE[c] = 0.0f; dH[c] = 0.0f; }
                    }
                    const float hf = 0.5f * fs;
                    const float ndE = nx * dE[0] + ny * dE[1] + nz * dE[2];
                    const float ndH = nx * dH[0] + ny * dH[1] + nz * dH[2];
                    v[0][kk] = hf * ((ny * dH[2] - nz * dH[1]) + aE * (dE[0] - ndE * nx));
                    v[1][kk] = hf * ((nz * dH[0] - nx * dH[2]) + aE * (dE[1] - ndE * ny));
                    v[2][kk] = hf * ((nx * dH[1] - ny * dH[0]) + aE * (dE[2] - ndE * nz));
                    v[3][kk] = hf * (-(ny * dE[2] - nz * dE[1]) + aH * (dH[0] - ndH * nx));
                    v[4][kk] = hf * (-(nz * dE[0] - nx * dE[2]) + aH * (dH[1] - ndH * ny));
                    v[5][kk] = hf * (-(nx * dE[1] - ny * dE[0]) + aH * (dH[2] - ndH * nz));
                } else {
#pragma unroll
                    for (int c = 0; c < 6; ++c) v[c][kk] = 0.0f;
                }
            }
            unsigned char* shi = ring + slot * 2 * O::SlotBytes;
            unsigned char* slo = shi + O::SlotBytes;
#pragma unroll
            for (int c = 0; c < 6; ++c) {
                const int t = c >> 1, r = (c & 1) * 64 + bl;
                const uint32_t off = t * kTileBytes + tc::tile_offset(r, kq * 2);
                float2 h2, l2;
                h2.x = tc::to_tf32(v[c][0]); l2.x = tc::to_tf32(v[c][0] - h2.x);
                h2.y = tc::to_tf32(v[c][1]); l2.y = tc::to_tf32(v[c][1] - h2.y);
                *reinterpret_cast<float2*>(shi + off) = h2;
                *reinterpret_cast<float2*>(slo + off) = l2;
            }
            tc::fence_proxy_async();
            tc::fence_before_sync();
            __syncthreads();
            if (s_err) break;
            if (tid == 0) {
                tc::fence_after_sync();
                const uint32_t ah0 = tc::smem_u32(shi), al0 = tc::smem_u32(slo);
                const uint64_t bh = tc::smem_desc(tc::smem_u32(op_hi + q * O::OpStep));
                const uint64_t blo = tc::smem_desc(tc::smem_u32(op_lo + q * O::OpStep));
#pragma unroll
                for (int t = 0; t < 3; ++t) {
                    const uint32_t d = taddr + t * N;
                    const uint64_t ah = tc::smem_desc(ah0 + t * kTileBytes), al = tc::smem_desc(al0 + t * kTileBytes);
                    tc::mma_tf32(d, ah, bh, idesc, q > 0);
                    tc::mma_tf32(d, al, bh, idesc, true);
                    tc::mma_tf32(d, ah, blo, idesc, true);
                }
                tc::mma_commit(&bars[slot]);
            }
            if (slot) ++ncommit1; else ++ncommit0;
        }
        if (s_err) break;
        // ---- all MMAs of this work item done
        if (!tc::mbar_wait(&bars[(NKS - 1) & 1], (((NKS - 1) & 1 ? ncommit1 : ncommit0) - 1) & 1u)) s_err = 1;
        if (!tc::mbar_wait(&bars[NKS & 1], (((NKS & 1) ? ncommit1 : ncommit0) - 1) & 1u)) s_err = 1;
        tc::fence_after_sync();
        if (!__syncthreads_or(s_err)) {
            // ---- epilogue: warp (lane group lg, column half ch); rows of the tile are (c, incidence)
            const int lg = warp & 3, ch = warp >> 2;
            const int r = lg * 32 + lane;
            const float ie = __ldg(T.mat + e * 3 + 0), im = __ldg(T.mat + e * 3 + 1), se = __ldg(T.mat + e * 3 + 2);
            const int blr = r & 63;
#pragma unroll 1
            for (int t = 0; t < 3; ++t) {
                const int c = 2 * t + (r >> 6);
                const int rowoff = c * CB + blr;
#pragma unroll 1
                for (int c0 = ch * (N / 2); c0 < (ch + 1) * (N / 2); c0 += 8) {
                    float dv[8];
                    tmem_ld8(taddr + (static_cast<uint32_t>(lg * 32) << 16) + t * N + c0, dv);
                    tc::tmem_ld_wait();
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        const int i = c0 + u;
                        if (i >= Np) break;
                        const int64_t idx = eoff + rowoff + i * static_cast<int>(Bp);
                        const float uc = ue[rowoff + i * static_cast<int>(Bp)];
                        const float k = (c < 3) ? (ie * dv[u] - se * uc) : (im * dv[u]);
                        switch (A.mode) {
                        case MODE_MULT: A.out[idx] = k; break;
                        case MODE_RK4_1: A.yout[idx] = uc + 0.5f * dtf * k; A.z[idx] = uc + (dtf / 6.0f) * k; break;
                        case MODE_RK4_2: A.yout[idx] = A.x[idx] + 0.5f * dtf * k; A.z[idx] += (dtf / 3.0f) * k; break;
                        case MODE_RK4_3: A.yout[idx] = A.x[idx] + dtf * k; A.z[idx] += (dtf / 3.0f) * k; break;
                        case MODE_RK4_4: A.x[idx] = A.z[idx] + (dtf / 6.0f) * k; break;
                        case MODE_LSRK: {
                            const float rr = A.a * A.res[idx] + dtf * k;
                            A.res[idx] = rr;
                            A.yout[idx] = uc + A.b * rr;
                            break;
                        }
                        default: break;
                        }
                    }
                }
            }
        }
        tc::fence_before_sync();
        if (__syncthreads_or(s_err)) break;
    }
    if (s_err && tid == 0) atomicExch(status, 1);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(taddr, O::TmemCols);
}

uint32_t tf32_bits_rna(float x)
{
    uint32_t u;
    std::memcpy(&u, &x, 4);
    u += 0x1000u;          // round half away from zero on the magnitude
    u &= ~0x1FFFu;
    return u;
}

float bits_to_float(uint32_t u)
{
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

}  // namespace

bool tc_supported(int p, int Bpad) { return p >= 1 && p <= 4 && Bpad % kChunk == 0; }

// Host image of Op = [Dr | Ds | Dt | LIFT]^T as the kernel's K-major B operand, hi then lo.
std::vector<uint32_t> tc_operator_image(const RefTet& ref)
{
    const int p = ref.p;
    int Np = ref.Np, Nfp = ref.Nfp, NF = 4 * Nfp, KK = 3 * Np + NF, KKp = (KK + 7) / 8 * 8, NKS = KKp / 8;
    int N = (Np + 15) / 16 * 16;
    (void)p;
    const size_t words = static_cast<size_t>(NKS) * N * 8;
    std::vector<uint32_t> img(2 * words, 0u);
    for (int i = 0; i < Np; ++i)
        for (int k = 0; k < KK; ++k) {
            double v;
            if (k < Np) v = ref.Dr[i * Np + k];
            else if (k < 2 * Np) v = ref.Ds[i * Np + k - Np];
            else if (k < 3 * Np) v = ref.Dt[i * Np + k - 2 * Np];
            else v = ref.LIFT[static_cast<size_t>(i) * NF + (k - 3 * Np)];
            const float f = static_cast<float>(v);
            const uint32_t hb = tf32_bits_rna(f);
            const float lo = static_cast<float>(v - static_cast<double>(bits_to_float(hb)));
            const uint32_t lb = tf32_bits_rna(lo);
            const size_t off = (static_cast<size_t>(k / 8) * N * 32 + tc::tile_offset(i, k)) / 4;
            img[off] = hb;
            img[words + off] = lb;
        }
    return img;
}

void launch_stage_tc(const BatchedTables& T, const BatchedStageArgs& A, const uint32_t* op_img, int* status, int n_sm,
                     cudaStream_t s)
{
    const int64_t n_work = T.K * (T.Bpad / kChunk);
    auto go = [&](auto kernel, size_t smem) {
        static bool attr[8] = {};
        if (!attr[T.p]) {
            cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
            if (e != cudaSuccess) throw std::runtime_error(std::string("tc smem attribute: ") + cudaGetErrorString(e));
            attr[T.p] = true;
        }
        const int per_sm = (2 * smem <= 227 * 1024) ? 2 : 1;
        const int64_t grid = std::min<int64_t>(n_work, static_cast<int64_t>(n_sm) * per_sm);
        kernel<<<static_cast<unsigned>(grid), kThreads, smem, s>>>(T, A, op_img, n_work, status);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) throw std::runtime_error(std::string("tc stage kernel: ") + cudaGetErrorString(e));
    };
    switch (T.p) {
    case 1: go(stage_tc<1>, TcOrd<1>::smem); break;
    case 2: go(stage_tc<2>, TcOrd<2>::smem); break;
    case 3: go(stage_tc<3>, TcOrd<3>::smem); break;
    case 4: go(stage_tc<4>, TcOrd<4>::smem); break;
    default: throw std::runtime_error("tensor-core stage kernel supports orders 1..4");
    }
}

}  // namespace dgtd
