// Batched FP32 stage kernel with the contractions on the tensor cores (tcgen05, 3xTF32).
//
// For one element e and one chunk of 64 incidences the right-hand side of all
// six field components is a single tall-skinny product
//
//   RHS^T[(c,b), i] = sum_k W[(c,b), k] * Op[k, i],  Op = [LIFT | Dr | Ds | Dt]^T,
//
// with W the per-element operand built on the fly:
//   k in [0, 4Nfp)          : Fscale/2 * upwind flux at face node k
//                             (reference HesthavenEvolution.cpp:509-520);
//   k in [4Nfp, 4Nfp + 3Np) : (g_r x F, g_s x F, g_t x F) at node (k - 4Nfp) mod Np, where F is
//                             the partner field (H for E targets, -E for H targets) and g_r, g_s,
//                             g_t the element's geometric factors (rows of d(r,s,t)/dx), so the
//                             product is the curl (:522-534).
// Rows (c, b) are 6 components x 64 incidences = 3 M-tiles of 128; N = Np padded
// to 16; K padded to 8. W is split into a tf32 high part (mantissa truncated) and
// the FP32 remainder, the constant Op into round-to-nearest hi/lo parts, giving
// W_hi Op_hi + W_lo Op_hi + W_hi Op_lo (3xTF32, FP32-level accuracy). The
// accumulators live in tensor memory; the epilogue applies 1/eps, 1/mu, the
// conductivity term and the RK stage update.
//
// Per CTA (persistent, two per SM): the element's field block staged in shared
// memory once per work item; a 2-slot ring holding one K-step of W (written by
// all threads) and of Op (a 1D bulk async copy from L2 into the slot, completing
// on an mbarrier); tcgen05.commit -> mbarrier releases a slot once the tensor
// core has consumed it.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

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
    static constexpr int KK = NF + 3 * Np;
    static constexpr int KKp = (KK + 7) / 8 * 8;
    static constexpr int NKS = KKp / 8;
    static constexpr int N = (Np + 15) / 16 * 16;
    static constexpr int OpStep = N * 32;                   // bytes of one K-step of Op (N rows x 8 tf32)
    static constexpr int WBytes = 3 * kTileBytes;           // one K-step of W (3 M-tiles), per hi / lo
    static constexpr int SlotBytes = 2 * WBytes + 2 * OpStep;
    static constexpr int UBytes = 6 * Np * kChunk * 4;      // staged element block
    static constexpr int TmemCols = 256;
    static constexpr size_t smem = static_cast<size_t>(UBytes) + 2 * static_cast<size_t>(SlotBytes);
};

__device__ __forceinline__ void pw_eval(const PlaneWaveF32* pw, const int* pw_off, int b, float px, float py, float pz,
                                        float t, float* e, float* h)
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

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(tc::smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// 1D bulk async copy global -> shared, completing `bytes` of transaction count on `bar`.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     tc::smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(tc::smem_u32(bar))
                 : "memory");
}

// tf32 high part by mantissa truncation, and the FP32 remainder
__device__ __forceinline__ void split_tf32(float v, float& hi, float& lo)
{
    hi = __uint_as_float(__float_as_uint(v) & 0xFFFFE000u);
    lo = v - hi;
}

template <int P>
__global__ void __launch_bounds__(kThreads, 2) stage_tc(BatchedTables T, BatchedStageArgs A, const uint32_t* __restrict__ op_img,
                                                     int64_t n_work, int* status)
{
    using O = TcOrd<P>;
    constexpr int Np = O::Np, Nfp = O::Nfp, NF = O::NF, NKS = O::NKS, N = O::N;
    extern __shared__ __align__(128) unsigned char sm[];
    float* s_u = reinterpret_cast<float*>(sm);                // [6][Np][64]
    unsigned char* ring = sm + O::UBytes;                     // [slot]{W hi, W lo, Op hi, Op lo}
    __shared__ uint64_t mma_bar[2], op_bar[2];
    __shared__ uint32_t tbase;
    __shared__ int s_fmask[NF];
    __shared__ int32_t s_nbr[NF];        // neighbour (element * Np + node) of each face node, internal numbering
    __shared__ float s_fg[16];            // nx ny nz Fscale per face
    __shared__ int s_code[4];
    __shared__ int s_err;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int bl = tid & 63, kq = tid >> 6;      // producer: incidence and a pair of K columns
    const int Bp = static_cast<int>(T.Bpad);
    const int nchunk = Bp / kChunk;
    const int CB = Np * Bp;                      // component stride inside an element block (global)
    const int64_t EB = 6 * static_cast<int64_t>(CB);

    for (int i = tid; i < NF; i += kThreads) s_fmask[i] = T.Fmask[i];
    if (tid == 0) {
        for (int s = 0; s < 2; ++s) { tc::mbar_init(&mma_bar[s], 1); tc::mbar_init(&op_bar[s], 1); }
        tc::mbar_fence_init();
        s_err = 0;
    }
    if (warp == 0) {
        tc::tmem_alloc(&tbase, O::TmemCols);
        tc::tmem_relinquish();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t taddr = tbase;
    const uint32_t idesc = tc::idesc_tf32(128, N);
    uint32_t nmma0 = 0u, nmma1 = 0u, nop0 = 0u, nop1 = 0u;   // completions issued per ring slot (uniform)
    const float dtf = A.dt;

    for (int64_t w = blockIdx.x; w < n_work; w += gridDim.x) {
        const int64_t e = w / nchunk;
        const int g = static_cast<int>(w - e * nchunk);
        const int b = g * kChunk + bl;
        const int64_t eoff = e * EB + static_cast<int64_t>(g) * kChunk;
        // ---- stage the element block (6 Np rows of 64 incidences) and its face tables
        {
            const float* __restrict__ src = A.in + eoff;
            for (int idx = tid; idx < 6 * Np * 16; idx += kThreads) {
                const int row = idx >> 4, q4 = idx & 15;
                reinterpret_cast<float4*>(s_u)[idx] =
                    __ldg(reinterpret_cast<const float4*>(src + static_cast<int64_t>(row) * Bp) + q4);
            }
            for (int i = tid; i < NF; i += kThreads) s_nbr[i] = __ldg(T.vmapP + e * NF + i);
            if (tid < 16) s_fg[tid] = __ldg(T.fgeo + e * 16 + tid);
            if (tid < 4) s_code[tid] = __ldg(T.fcode + e * 4 + tid);
        }
        const float* gg = T.geo + e * 9;
        const float g0 = __ldg(gg + 0), g1 = __ldg(gg + 1), g2 = __ldg(gg + 2), g3 = __ldg(gg + 3),
                    g4 = __ldg(gg + 4), g5 = __ldg(gg + 5), g6 = __ldg(gg + 6), g7 = __ldg(gg + 7), g8 = __ldg(gg + 8);
        const bool skip_src = (A.skip == nullptr) || A.skip[b];
        __syncthreads();

        for (int q = 0; q < NKS; ++q) {
            const int slot = q & 1;
            unsigned char* sw = ring + slot * O::SlotBytes;
            unsigned char* w_hi = sw;
            unsigned char* w_lo = sw + O::WBytes;
            unsigned char* o_hi = sw + 2 * O::WBytes;
            if (q >= 2 && !tc::mbar_wait(&mma_bar[slot], ((slot ? nmma1 : nmma0) - 1) & 1u)) s_err = 1;
            if (tid == 0) {
                // Op K-step q (hi and lo contiguous) into the slot
                mbar_expect_tx(&op_bar[slot], 2 * O::OpStep);
                bulk_g2s(o_hi, op_img + static_cast<size_t>(q) * (2 * O::OpStep / 4), 2 * O::OpStep, &op_bar[slot]);
            }
            if (slot) ++nop1; else ++nop0;
            // ---- produce K-step q of W: columns k0, k0 + 1 for all six target components
            float v[6][2];
#pragma unroll
            for (int kk = 0; kk < 2; ++kk) {
                const int k = q * 8 + kq * 2 + kk;
                if (k < NF) {
                    const int m = k, f = m / Nfp;
                    const int vm = s_fmask[m];
                    const int code = s_code[f];
                    const float nx = s_fg[f * 4], ny = s_fg[f * 4 + 1], nz = s_fg[f * 4 + 2], fs = s_fg[f * 4 + 3];
                    float uM[6];
#pragma unroll
                    for (int c = 0; c < 6; ++c) uM[c] = s_u[(c * Np + vm) * kChunk + bl];
                    float dE[3], dH[3];
                    float aE = T.alpha, aH = T.alpha;
                    if (code == 0 || code == 4 || code == 5) {
                        const int32_t gp = s_nbr[m];
                        const int32_t en = gp / Np, node = gp - en * Np;
                        const float* __restrict__ un =
                            A.in + static_cast<int64_t>(en) * EB + static_cast<int64_t>(g) * kChunk + node * Bp + bl;
#pragma unroll
                        for (int c = 0; c < 3; ++c) {
                            dE[c] = __ldg(un + c * CB) - uM[c];
                            dH[c] = __ldg(un + (c + 3) * CB) - uM[c + 3];
                        }
                        if (code != 0 && !skip_src) {
                            const float* xq = T.fxyz + (e * NF + m) * 3;
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
                } else if (k < NF + 3 * Np) {
                    const int kc = k - NF, type = kc / Np, j = kc - type * Np;
                    const float gx = type == 0 ? g0 : (type == 1 ? g3 : g6);
                    const float gy = type == 0 ? g1 : (type == 1 ? g4 : g7);
                    const float gz = type == 0 ? g2 : (type == 1 ? g5 : g8);
                    const float* uj = s_u + j * kChunk + bl;
                    const float Ex = uj[0], Ey = uj[Np * kChunk], Ez = uj[2 * Np * kChunk];
                    const float Hx = uj[3 * Np * kChunk], Hy = uj[4 * Np * kChunk], Hz = uj[5 * Np * kChunk];
                    // E targets: g x H (curl H); H targets: -(g x E) (-curl E)
                    v[0][kk] = gy * Hz - gz * Hy;
                    v[1][kk] = gz * Hx - gx * Hz;
                    v[2][kk] = gx * Hy - gy * Hx;
                    v[3][kk] = gz * Ey - gy * Ez;
                    v[4][kk] = gx * Ez - gz * Ex;
                    v[5][kk] = gy * Ex - gx * Ey;
                } else {
#pragma unroll
                    for (int c = 0; c < 6; ++c) v[c][kk] = 0.0f;
                }
            }
#pragma unroll
            for (int c = 0; c < 6; ++c) {
                const int t = c >> 1, r = (c & 1) * 64 + bl;
                const uint32_t off = t * kTileBytes + tc::tile_offset(r, kq * 2);
                float2 h2, l2;
                split_tf32(v[c][0], h2.x, l2.x);
                split_tf32(v[c][1], h2.y, l2.y);
                *reinterpret_cast<float2*>(w_hi + off) = h2;
                *reinterpret_cast<float2*>(w_lo + off) = l2;
            }
            tc::fence_proxy_async();
            tc::fence_before_sync();
            __syncthreads();
            if (s_err) break;
            if (tid == 0 && !tc::mbar_wait(&op_bar[slot], ((slot ? nop1 : nop0) - 1) & 1u)) s_err = 1;
            if (tid == 0 && !s_err) {
                tc::fence_after_sync();
                const uint32_t ah0 = tc::smem_u32(w_hi), al0 = tc::smem_u32(w_lo);
                const uint64_t bh = tc::smem_desc(tc::smem_u32(o_hi));
                const uint64_t blo = tc::smem_desc(tc::smem_u32(o_hi + O::OpStep));
#pragma unroll
                for (int t = 0; t < 3; ++t) {
                    const uint32_t d = taddr + t * N;
                    const uint64_t ah = tc::smem_desc(ah0 + t * kTileBytes), al = tc::smem_desc(al0 + t * kTileBytes);
                    tc::mma_tf32(d, ah, bh, idesc, q > 0);
                    tc::mma_tf32(d, al, bh, idesc, true);
                    tc::mma_tf32(d, ah, blo, idesc, true);
                }
                tc::mma_commit(&mma_bar[slot]);
            }
            if (slot) ++nmma1; else ++nmma0;
        }
        if (s_err) break;
        // ---- all MMAs of this work item done
        if (!tc::mbar_wait(&mma_bar[0], (nmma0 - 1) & 1u)) s_err = 1;
        if (!tc::mbar_wait(&mma_bar[1], (nmma1 - 1) & 1u)) s_err = 1;
        tc::fence_after_sync();
        if (!__syncthreads_or(s_err)) {
            // ---- epilogue: warp (lane group lg, column half ch); tile rows are (c, incidence)
            const int lg = warp & 3, ch = warp >> 2;
            const int r = lg * 32 + lane;
            const float ie = __ldg(T.mat + e * 3 + 0), im = __ldg(T.mat + e * 3 + 1), se = __ldg(T.mat + e * 3 + 2);
            const int blr = r & 63;
#pragma unroll 1
            for (int t = 0; t < 3; ++t) {
                const int c = 2 * t + (r >> 6);
                const int rowoff = c * CB + blr;
                const float* su = s_u + c * Np * kChunk + blr;
#pragma unroll 1
                for (int c0 = ch * (N / 2); c0 < (ch + 1) * (N / 2); c0 += 8) {
                    float dv[8];
                    tmem_ld8(taddr + (static_cast<uint32_t>(lg * 32) << 16) + t * N + c0, dv);
                    tc::tmem_ld_wait();
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        const int i = c0 + u;
                        if (i >= Np) break;
                        const int64_t idx = eoff + rowoff + i * Bp;
                        const float uc = su[i * kChunk];
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

// Host image of Op = [LIFT | Dr | Ds | Dt]^T as the kernel's K-major B operand:
// per K-step q, N rows x 8 tf32 high parts followed by the N x 8 low parts.
std::vector<uint32_t> tc_operator_image(const RefTet& ref)
{
    const int Np = ref.Np, Nfp = ref.Nfp, NF = 4 * Nfp, KK = NF + 3 * Np, KKp = (KK + 7) / 8 * 8, NKS = KKp / 8;
    const int N = (Np + 15) / 16 * 16;
    const size_t step_words = static_cast<size_t>(N) * 8;        // one K-step, hi or lo
    std::vector<uint32_t> img(2 * step_words * NKS, 0u);
    for (int i = 0; i < Np; ++i)
        for (int k = 0; k < KK; ++k) {
            double v;
            if (k < NF) v = ref.LIFT[static_cast<size_t>(i) * NF + k];
            else {
                const int kc = k - NF, type = kc / Np, j = kc - type * Np;
                const std::vector<double>& D = type == 0 ? ref.Dr : (type == 1 ? ref.Ds : ref.Dt);
                v = D[static_cast<size_t>(i) * Np + j];
            }
            const float f = static_cast<float>(v);
            const uint32_t hb = tf32_bits_rna(f);
            const float lo = static_cast<float>(v - static_cast<double>(bits_to_float(hb)));
            const uint32_t lb = tf32_bits_rna(lo);
            const size_t base = static_cast<size_t>(k / 8) * 2 * step_words;
            const size_t off = tc::tile_offset(i, k) / 4;
            img[base + off] = hb;
            img[base + step_words + off] = lb;
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
        const int per_sm = (2 * (smem + 2048) <= 228 * 1024) ? 2 : 1;
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
