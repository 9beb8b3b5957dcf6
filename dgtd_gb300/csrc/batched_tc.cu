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
// Per CTA (persistent, one per SM, 512 threads): Op hi/lo resident in shared
// memory; the element's field block and face tables of the next work item
// prefetched by 1D bulk async copies into a second buffer (mbarrier
// completion) while the current item is processed; a 2-slot ring of W K-steps
// written by all threads; tcgen05.commit -> mbarrier releases a slot once the
// tensor core has consumed it.
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

constexpr int kThreads = 512;
constexpr int kChunk = 64;          // incidences per work item
constexpr int kWsbo = 288;                 // W operand: bytes between 8-row groups (bank-conflict-free stores)
constexpr int kTileBytes = 16 * kWsbo;      // W tile: 128 rows x 8 tf32

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
    static constexpr int OpBytes = NKS * OpStep;            // per hi / lo
    static constexpr int WBytes = 3 * kTileBytes;           // one K-step of W (3 M-tiles), per hi / lo
    static constexpr int UBytes = 6 * Np * kChunk * 4;      // staged element block
    static constexpr int NbrBytes = (4 * NF + 15) / 16 * 16;
    // U | neighbour table | face geometry (16 floats) | face codes (4 ints)
    static constexpr int UBufBytes = (UBytes + NbrBytes + 64 + 16 + 127) / 128 * 128;
    static constexpr int TmemCols = 256;
    static constexpr size_t smem = 2 * static_cast<size_t>(OpBytes) + 2 * static_cast<size_t>(UBufBytes) +
                                   2 * 2 * static_cast<size_t>(WBytes);
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

__device__ __forceinline__ void tmem_ld4(uint32_t taddr, float* v)
{
    uint32_t r[4];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(taddr));
#pragma unroll
    for (int i = 0; i < 4; ++i) v[i] = __uint_as_float(r[i]);
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

// Stage update of QC nodes (stride Bp) of one row of an element block: loads of the
// RK registers first, then the stores. `nv` = valid nodes (<= QC).
template <int QC>
__device__ __forceinline__ void epilogue_store(const BatchedStageArgs& A, int64_t base, int Bp, int nv, const float* kv,
                                               const float* uc, float dtf)
{
    float* __restrict__ out = A.out;
    float* __restrict__ x = A.x;
    float* __restrict__ y = A.yout;
    float* __restrict__ z = A.z;
    float* __restrict__ res = A.res;
    float a[QC], b[QC];
    switch (A.mode) {
    case MODE_MULT:
#pragma unroll
        for (int j = 0; j < QC; ++j)
            if (j < nv) out[base + j * Bp] = kv[j];
        break;
    case MODE_RK4_1:
#pragma unroll
        for (int j = 0; j < QC; ++j)
            if (j < nv) {
                y[base + j * Bp] = uc[j] + 0.5f * dtf * kv[j];
                z[base + j * Bp] = uc[j] + (dtf / 6.0f) * kv[j];
            }
        break;
    case MODE_RK4_2:
    case MODE_RK4_3: {
        const float cy = (A.mode == MODE_RK4_2) ? 0.5f * dtf : dtf;
#pragma unroll
        for (int j = 0; j < QC; ++j)
            if (j < nv) { a[j] = x[base + j * Bp]; b[j] = z[base + j * Bp]; }
#pragma unroll
        for (int j = 0; j < QC; ++j)
            if (j < nv) {
                y[base + j * Bp] = a[j] + cy * kv[j];
                z[base + j * Bp] = b[j] + (dtf / 3.0f) * kv[j];
            }
        break;
    }
    case MODE_RK4_4:
#pragma unroll
        for (int j = 0; j < QC; ++j)
            if (j < nv) b[j] = z[base + j * Bp];
#pragma unroll
        for (int j = 0; j < QC; ++j)
            if (j < nv) x[base + j * Bp] = b[j] + (dtf / 6.0f) * kv[j];
        break;
    case MODE_LSRK:
#pragma unroll
        for (int j = 0; j < QC; ++j)
            if (j < nv) a[j] = res[base + j * Bp];
#pragma unroll
        for (int j = 0; j < QC; ++j)
            if (j < nv) {
                const float rr = A.a * a[j] + dtf * kv[j];
                res[base + j * Bp] = rr;
                y[base + j * Bp] = uc[j] + A.b * rr;
            }
        break;
    default: break;
    }
}

// Issue the bulk copies of one work item's element block and face tables (one thread).
template <int P>
__device__ __forceinline__ void prefetch_item(const BatchedTables& T, const float* in, int64_t w, int nchunk, int Bp,
                                              unsigned char* buf, uint64_t* bar)
{
    using O = TcOrd<P>;
    constexpr int Np = O::Np, NF = O::NF;
    const int64_t e = w / nchunk;
    const int g = static_cast<int>(w - e * nchunk);
    const int64_t EB = 6 * static_cast<int64_t>(Np) * Bp;
    const float* src = in + e * EB + static_cast<int64_t>(g) * kChunk;
    mbar_expect_tx(bar, O::UBytes + 4 * NF + 64 + 16);
    if (Bp == kChunk) {
        bulk_g2s(buf, src, O::UBytes, bar);
    } else {
        for (int r = 0; r < 6 * Np; ++r)
            bulk_g2s(buf + r * kChunk * 4, src + static_cast<int64_t>(r) * Bp, kChunk * 4, bar);
    }
    bulk_g2s(buf + O::UBytes, T.vmapP + e * NF, 4 * NF, bar);
    bulk_g2s(buf + O::UBytes + O::NbrBytes, T.fgeo + e * 16, 64, bar);
    bulk_g2s(buf + O::UBytes + O::NbrBytes + 64, T.fcode + e * 4, 16, bar);
}

template <int P>
__global__ void __launch_bounds__(kThreads, 1) stage_tc(BatchedTables T, BatchedStageArgs A, const uint32_t* __restrict__ op_img,
                                                     int64_t n_work, int* status)
{
    using O = TcOrd<P>;
    constexpr int Np = O::Np, Nfp = O::Nfp, NF = O::NF, NKS = O::NKS, N = O::N;
    extern __shared__ __align__(128) unsigned char sm[];
    unsigned char* op_hi = sm;
    unsigned char* op_lo = sm + O::OpBytes;
    unsigned char* ubuf0 = sm + 2 * O::OpBytes;
    unsigned char* ring = ubuf0 + 2 * O::UBufBytes;           // [slot]{W hi, W lo}
    __shared__ uint64_t mma_bar[2], u_bar[2];
    __shared__ uint32_t tbase;
    __shared__ int s_fmask[NF];
    __shared__ int s_tj[3 * Np];          // combo column -> (type << 8) | node

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int bl = tid & 63, kc8 = tid >> 6;     // producer: incidence and one K column of each K-step
    const int Bp = static_cast<int>(T.Bpad);
    const int nchunk = Bp / kChunk;
    const int CB = Np * Bp;                      // component stride inside an element block (global)
    const int64_t EB = 6 * static_cast<int64_t>(CB);

    // ---- prologue: resident operator, lookup tables, barriers, tensor memory, first item
    {
        const uint4* src = reinterpret_cast<const uint4*>(op_img);
        uint4* dst = reinterpret_cast<uint4*>(op_hi);
        for (int i = tid; i < 2 * O::OpBytes / 16; i += kThreads) dst[i] = __ldg(src + i);
    }
    for (int i = tid; i < NF; i += kThreads) s_fmask[i] = T.Fmask[i];
    for (int i = tid; i < 3 * Np; i += kThreads) s_tj[i] = ((i / Np) << 8) | (i % Np);
    if (tid == 0) {
        for (int s = 0; s < 2; ++s) { tc::mbar_init(&mma_bar[s], 1); tc::mbar_init(&u_bar[s], 1); }
        tc::mbar_fence_init();
    }
    if (warp == 0) {
        tc::tmem_alloc(&tbase, O::TmemCols);
        tc::tmem_relinquish();
    }
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (tid == 0 && static_cast<int64_t>(blockIdx.x) < n_work)
        prefetch_item<P>(T, A.in, blockIdx.x, nchunk, Bp, ubuf0, &u_bar[0]);
    const uint32_t taddr = tbase;
    const uint32_t idesc = tc::idesc_tf32(128, N);
    // phases per barrier: MMA commits, item copies issued and consumed (uniform in all threads)
    uint32_t nmma0 = 0u, nmma1 = 0u, nu0 = 0u, nu1 = 0u, ni0 = 0u, ni1 = 0u;
    int err = 0;   // a bounded wait ran out; made uniform at the next barrier
    if (static_cast<int64_t>(blockIdx.x) < n_work) ++ni0;
    const float dtf = A.dt;
    // per-thread store offsets of the producer (row = (c & 1) * 64 + bl of tile c / 2, column kc8)
    uint32_t soff[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        const int r = (c & 1) * 64 + bl;
        soff[c] = (c >> 1) * kTileBytes + (r >> 3) * kWsbo + ((kc8 & 7) >> 2) * tc::kLBO + (r & 7) * 16 + (kc8 & 3) * 4;
    }

    int it = 0;
    for (int64_t w = blockIdx.x; w < n_work; w += gridDim.x, ++it) {
        const int ub = it & 1;
        unsigned char* buf = ubuf0 + ub * O::UBufBytes;
        const float* s_u = reinterpret_cast<const float*>(buf);          // [6][Np][64]
        const int32_t* s_nbr = reinterpret_cast<const int32_t*>(buf + O::UBytes);
        const float* s_fg = reinterpret_cast<const float*>(buf + O::UBytes + O::NbrBytes);
        const int* s_code = reinterpret_cast<const int*>(buf + O::UBytes + O::NbrBytes + 64);
        if (!tc::mbar_wait(&u_bar[ub], ((ub ? nu1 : nu0)) & 1u)) err = 1;
        if (ub) ++nu1; else ++nu0;
        // prefetch the next item into the other buffer (its previous user finished last iteration)
        if (w + gridDim.x < n_work) {
            if (tid == 0)
                prefetch_item<P>(T, A.in, w + gridDim.x, nchunk, Bp, ubuf0 + (ub ^ 1) * O::UBufBytes, &u_bar[ub ^ 1]);
            if (ub) ++ni0; else ++ni1;
        }

        const int64_t e = w / nchunk;
        const int g = static_cast<int>(w - e * nchunk);
        const int b = g * kChunk + bl;
        const int64_t eoff = e * EB + static_cast<int64_t>(g) * kChunk;
        const float* gg = T.geo + e * 9;
        const float g0 = __ldg(gg + 0), g1 = __ldg(gg + 1), g2 = __ldg(gg + 2), g3 = __ldg(gg + 3),
                    g4 = __ldg(gg + 4), g5 = __ldg(gg + 5), g6 = __ldg(gg + 6), g7 = __ldg(gg + 7), g8 = __ldg(gg + 8);
        const bool skip_src = (A.skip == nullptr) || A.skip[b];
        // neighbour traces of this thread's flux column, loaded one K-step ahead
        auto load_nbr = [&](int k, float* dst) {
            if (k < NF) {
                const int code = s_code[k / Nfp];
                if (code == 0 || code == 4 || code == 5) {
                    const int32_t gp = s_nbr[k];
                    const int32_t en = gp / Np, node = gp - en * Np;
                    const float* __restrict__ un =
                        A.in + static_cast<int64_t>(en) * EB + static_cast<int64_t>(g) * kChunk + node * Bp + bl;
#pragma unroll
                    for (int c = 0; c < 6; ++c) dst[c] = __ldg(un + c * CB);
                }
            }
        };
        float nb[6], nbn[6];
        load_nbr(kc8, nb);

        for (int q = 0; q < NKS; ++q) {
            load_nbr((q + 1) * 8 + kc8, nbn);
            const int slot = q & 1;
            unsigned char* w_hi = ring + slot * 2 * O::WBytes;
            unsigned char* w_lo = w_hi + O::WBytes;
            if (q >= 2 && !tc::mbar_wait(&mma_bar[slot], ((slot ? nmma1 : nmma0) - 1) & 1u)) err = 1;
            // ---- produce column k of K-step q for all six target components
            float v[6];
            const int k = q * 8 + kc8;
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
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        dE[c] = nb[c] - uM[c];
                        dH[c] = nb[c + 3] - uM[c + 3];
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
                v[0] = hf * ((ny * dH[2] - nz * dH[1]) + aE * (dE[0] - ndE * nx));
                v[1] = hf * ((nz * dH[0] - nx * dH[2]) + aE * (dE[1] - ndE * ny));
                v[2] = hf * ((nx * dH[1] - ny * dH[0]) + aE * (dE[2] - ndE * nz));
                v[3] = hf * (-(ny * dE[2] - nz * dE[1]) + aH * (dH[0] - ndH * nx));
                v[4] = hf * (-(nz * dE[0] - nx * dE[2]) + aH * (dH[1] - ndH * ny));
                v[5] = hf * (-(nx * dE[1] - ny * dE[0]) + aH * (dH[2] - ndH * nz));
            } else if (k < NF + 3 * Np) {
                const int tj = s_tj[k - NF], type = tj >> 8, j = tj & 255;
                const float gx = type == 0 ? g0 : (type == 1 ? g3 : g6);
                const float gy = type == 0 ? g1 : (type == 1 ? g4 : g7);
                const float gz = type == 0 ? g2 : (type == 1 ? g5 : g8);
                const float* uj = s_u + j * kChunk + bl;
                const float Ex = uj[0], Ey = uj[Np * kChunk], Ez = uj[2 * Np * kChunk];
                const float Hx = uj[3 * Np * kChunk], Hy = uj[4 * Np * kChunk], Hz = uj[5 * Np * kChunk];
                // E targets: g x H (curl H); H targets: -(g x E) (-curl E)
                v[0] = gy * Hz - gz * Hy;
                v[1] = gz * Hx - gx * Hz;
                v[2] = gx * Hy - gy * Hx;
                v[3] = gz * Ey - gy * Ez;
                v[4] = gx * Ez - gz * Ex;
                v[5] = gy * Ex - gx * Ey;
            } else {
#pragma unroll
                for (int c = 0; c < 6; ++c) v[c] = 0.0f;
            }
#pragma unroll
            for (int c = 0; c < 6; ++c) {
                float h, l;
                split_tf32(v[c], h, l);
                *reinterpret_cast<float*>(w_hi + soff[c]) = h;
                *reinterpret_cast<float*>(w_lo + soff[c]) = l;
            }
            tc::fence_proxy_async();
            tc::fence_before_sync();
            if (__syncthreads_or(err)) { err = 1; break; }
            if (tid == 0) {
                tc::fence_after_sync();
                const uint32_t ah0 = tc::smem_u32(w_hi), al0 = tc::smem_u32(w_lo);
                const uint64_t bh = tc::smem_desc(tc::smem_u32(op_hi + q * O::OpStep));
                const uint64_t blo = tc::smem_desc(tc::smem_u32(op_lo + q * O::OpStep));
#pragma unroll
                for (int t = 0; t < 3; ++t) {
                    const uint32_t d = taddr + t * N;
                    const uint64_t ah = tc::smem_desc_sbo(ah0 + t * kTileBytes, kWsbo);
                    const uint64_t al = tc::smem_desc_sbo(al0 + t * kTileBytes, kWsbo);
                    tc::mma_tf32(d, ah, bh, idesc, q > 0);
                    tc::mma_tf32(d, al, bh, idesc, true);
                    tc::mma_tf32(d, ah, blo, idesc, true);
                }
                tc::mma_commit(&mma_bar[slot]);
            }
            if (slot) ++nmma1; else ++nmma0;
#pragma unroll
            for (int c = 0; c < 6; ++c) nb[c] = nbn[c];
        }
        if (err) break;
        // ---- all MMAs of this work item done
        if (!tc::mbar_wait(&mma_bar[0], (nmma0 - 1) & 1u)) err = 1;
        if (!tc::mbar_wait(&mma_bar[1], (nmma1 - 1) & 1u)) err = 1;
        tc::fence_after_sync();
        if (__syncthreads_or(err)) { err = 1; break; }
        {
            // ---- epilogue: warp = (lane group lg, column quarter cq); tile rows are (c, incidence).
            // All operand loads of a tile are issued before its stores so that each thread
            // waits for one memory round trip per tile, not one per output.
            constexpr int QC = N / 4;
            const int lg = warp & 3, cq = warp >> 2;
            const int r = lg * 32 + lane;
            const float ie = __ldg(T.mat + e * 3 + 0), im = __ldg(T.mat + e * 3 + 1), se = __ldg(T.mat + e * 3 + 2);
            const int blr = r & 63;
            const int cb = cq * QC;
#pragma unroll 1
            for (int t = 0; t < 3; ++t) {
                const int c = 2 * t + (r >> 6);
                const int64_t base = eoff + c * CB + blr + static_cast<int64_t>(cb) * Bp;
                const float* su = s_u + (c * Np + cb) * kChunk + blr;
                float kv[QC], uc[QC];
#pragma unroll
                for (int j = 0; j < QC; j += 4)
                    tmem_ld4(taddr + (static_cast<uint32_t>(lg * 32) << 16) + t * N + cb + j, kv + j);
                tc::tmem_ld_wait();
                const float fe = (c < 3) ? ie : im, fs = (c < 3) ? se : 0.0f;
#pragma unroll
                for (int j = 0; j < QC; ++j) {
                    uc[j] = (cb + j < Np) ? su[j * kChunk] : 0.0f;
                    kv[j] = fe * kv[j] - fs * uc[j];
                }
                epilogue_store<QC>(A, base, Bp, Np - cb, kv, uc, dtf);
            }
        }
        tc::fence_before_sync();
        __syncthreads();
    }
    if (err) {
        // drain: wait (bounded) for this CTA's copies and MMAs still in flight before
        // the tensor memory and the shared buffers are released
        if (tid == 0) {
            atomicExch(status, 1);
            if (nmma0) tc::mbar_wait(&mma_bar[0], (nmma0 - 1) & 1u);
            if (nmma1) tc::mbar_wait(&mma_bar[1], (nmma1 - 1) & 1u);
            if (ni0) tc::mbar_wait(&u_bar[0], (ni0 - 1) & 1u);
            if (ni1) tc::mbar_wait(&u_bar[1], (ni1 - 1) & 1u);
        }
    }
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
// all K-steps of the tf32 high parts (N rows x 8 columns each), then all low parts.
std::vector<uint32_t> tc_operator_image(const RefTet& ref)
{
    const int Np = ref.Np, Nfp = ref.Nfp, NF = 4 * Nfp, KK = NF + 3 * Np, KKp = (KK + 7) / 8 * 8, NKS = KKp / 8;
    const int N = (Np + 15) / 16 * 16;
    const size_t words = static_cast<size_t>(NKS) * N * 8;        // one operator part (hi or lo)
    std::vector<uint32_t> img(2 * words, 0u);
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
    if (reinterpret_cast<uintptr_t>(A.in) % 16 != 0)
        throw std::runtime_error("tensor-core stage: the input state must be 16-byte aligned (bulk async copies)");
    auto go = [&](auto kernel, size_t smem) {
        static bool attr[8] = {};
        if (!attr[T.p]) {
            cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
            if (e != cudaSuccess) throw std::runtime_error(std::string("tc smem attribute: ") + cudaGetErrorString(e));
            attr[T.p] = true;
        }
        const int64_t grid = std::min<int64_t>(n_work, static_cast<int64_t>(n_sm));
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
