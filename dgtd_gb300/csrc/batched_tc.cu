// Batched FP32 stage kernel with the contractions on the tensor cores (tcgen05, 3xTF32).
//
// For one element e and one chunk of 64 incidences the right-hand side of all
// six field components is a single tall-skinny product
//
//   RHS^T[(c,b), i] = sum_k W[(c,b), k] * Op[k, i],  Op = [Dr | Ds | Dt | LIFT]^T,
//
// with W the per-element operand built on the fly:
//   k in [0, 3Np)           : g_d x F at node j, k = 3 j + d (d = r, s, t), where F is the
//                             partner field (H for E targets, -E for H targets) and g_r, g_s,
//                             g_t the element's geometric factors (rows of d(r,s,t)/dx), so the
//                             product is the curl (reference HesthavenEvolution.cpp:522-534);
//                             node-major, so a thread's 4 columns touch at most 2 nodes;
//   k in [3Np, 3Np + 4Nfp)  : Fscale/2 * upwind flux at face node k - 3Np (:509-520).
// The volume columns come first so that the neighbour traces the flux columns
// need are loaded while the volume columns are being built.
// Rows (c, b) are 6 components x 64 incidences = 3 M-tiles of 128; N = Np padded
// to 16; K padded to 8. W is split into a tf32 high part (rounded to nearest) and
// the rounded remainder, the constant Op into round-to-nearest hi/lo parts, giving
// W_hi Op_hi + W_lo Op_hi + W_hi Op_lo (3xTF32). The accumulators live in tensor
// memory: W_hi Op_hi in a double-buffered item accumulator (columns 0 and 160), the
// two small correction products in a separate accumulator (column 320) that the
// epilogue folds in with FP32 adds. Each MMA's accumulation truncates relative to the
// accumulator it adds into, so keeping the corrections apart cuts that error 3x.
// The epilogue applies 1/eps, 1/mu, the conductivity term and the RK stage update (classical
// RK4 with the state register kept as an FP32 pair and a compensated last-stage update,
// batched.hpp).
//
// One persistent CTA per SM, warp-specialised, no CTA-wide barrier in the
// steady state (all hand-offs are mbarriers, every wait bounded):
//   warps 0-7  producers, two groups of 128 threads: group g builds the K-steps
//              q = g, g + 2, ... of each work item into ring slot g. A thread
//              owns one incidence and 4 consecutive columns of its K-step and
//              computes all 6 component rows, stored as 16-byte vectors
//              (conflict-free in the K-major core-matrix layout);
//   warps 8-11 epilogue: fold the correction accumulator into the item's
//              accumulator and release it, then drain the item's accumulator
//              (tcgen05.ld) and apply the stage update, with the global
//              RK-register loads of the next 8 nodes in flight;
//   warp 12    tensor-memory owner and MMA issuer (one thread);
//   warp 13    copy issuer (one thread): 1D bulk async copies of the next work
//              item's element block and face tables into the free staging
//              buffer (mbarrier transaction counts).
// Op hi/lo stays resident in shared memory for the whole launch. The RK stage
// mode is a template parameter, so each instantiation carries one epilogue.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "batched.hpp"
#include "tc_common.cuh"

namespace dgtd {

namespace {

constexpr int kThreads = 448;
constexpr int kProducerThreads = 256;   // warps 0-7
constexpr int kEpiWarp0 = 8;            // warps 8-11 (TMEM lane quarters 0-3)
constexpr int kEpiThreads = 128;
constexpr int kMmaWarp = 12;
constexpr int kCopyWarp = 13;        // the last warp: copy issuer
constexpr int kChunk = 64;              // incidences per work item
constexpr int kTile = 4096;             // one W tile: 128 rows x 8 tf32, SBO 256, LBO 128
constexpr int kWStep = 3 * kTile;       // one K-step of W (3 M-tiles), hi or lo
constexpr int kSlot = 2 * kWStep;       // hi + lo
constexpr uint32_t kAccStride = 160;    // TMEM columns between the two accumulator buffers
constexpr uint32_t kCorrCol = 320;      // the correction accumulator (single buffer)
constexpr uint32_t kTmemCols = 512;

template <int P>
struct TcOrd {
    static constexpr int Np = (P + 1) * (P + 2) * (P + 3) / 6;
    static constexpr int Nfp = (P + 1) * (P + 2) / 2;
    static constexpr int NF = 4 * Nfp;
    static constexpr int KK = NF + 3 * Np;
    static constexpr int KKp = (KK + 7) / 8 * 8;
    static constexpr int NKS = KKp / 8;
    static constexpr int N = (Np + 15) / 16 * 16;
    static constexpr int NCH = (Np + 7) / 8;               // 8-column epilogue chunks per tile
    static constexpr int OpStep = N * 32;                   // bytes of one K-step of Op (N rows x 8 tf32)
    static constexpr int OpBytes = NKS * OpStep;            // per hi / lo
    static constexpr int UBytes = 6 * Np * kChunk * 4;      // staged element block
    static constexpr int NbrBytes = (4 * NF + 15) / 16 * 16;
    static constexpr int XyzBytes = NF * 12;                 // face-node coordinates (TF/SF source)
    // U | neighbour table | face geometry (16 floats) | face codes (4 ints) | jump coefficients (20 floats)
    // | face-node coordinates (NF x 3 floats)
    static constexpr int UBufBytes = (UBytes + NbrBytes + 64 + 16 + 80 + XyzBytes + 127) / 128 * 128;
    static constexpr size_t smem = 2 * static_cast<size_t>(OpBytes) + 2 * static_cast<size_t>(UBufBytes) +
                                   2 * static_cast<size_t>(kSlot);
    static_assert(3 * N <= static_cast<int>(kAccStride), "accumulator buffer too narrow");
    static_assert(kCorrCol + 3 * N <= kTmemCols, "correction accumulator past the allocation");
};

// Column metadata: kind in bits 28-29 (0 flux, 1 volume, 2 padding);
// flux: face node m in bits 16-27, its face in bits 12-15, its volume node in bits 0-11;
// volume: derivative direction (0 r, 1 s, 2 t) in bits 16-23, node in bits 0-15 (column 3 node + d).
constexpr int kColFlux = 0, kColVol = 1, kColPad = 2;

// Sum of the plane waves pw[q0, q1) (one incidence's) at point p and time t.
__device__ __forceinline__ void pw_eval(const PlaneWaveF32* pw, int q0, int q1, float px, float py, float pz,
                                        float t, float* e, float* h)
{
    e[0] = e[1] = e[2] = h[0] = h[1] = h[2] = 0.0f;
    for (int q = q0; q < q1; ++q) {
        const PlaneWaveF32& w = pw[q];
        const float s = px * w.k[0] + py * w.k[1] + pz * w.k[2] - t;
        const float a = s - w.mean;
        float g = expf(-a * a / (2.0f * w.spread * w.spread));
        if (w.freq != 0.0f) g *= cosf(6.283185307179586f * w.freq * a);
        e[0] += g * w.pol[0]; e[1] += g * w.pol[1]; e[2] += g * w.pol[2];
        h[0] += g * w.kxp[0]; h[1] += g * w.kxp[1]; h[2] += g * w.kxp[2];
    }
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

// Bring `bytes` (multiple of 16, 16-byte aligned) of global memory into L2 ahead of use.
__device__ __forceinline__ void prefetch_l2(const void* src, uint32_t bytes)
{
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}

__device__ __forceinline__ void st_shared_v4(uint32_t addr, float a, float b, float c, float d)
{
    asm volatile("st.shared.v4.f32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "f"(a), "f"(b), "f"(c), "f"(d) : "memory");
}

// tf32 high part by mantissa truncation, and the FP32 remainder
// v = hi + lo with hi the tf32 value nearest v (ties away from zero) and lo the remainder,
// itself rounded to the nearest tf32. Both then pass through the tensor core's tf32 operand
// path unchanged. |lo| <= 2^-11 |v| and its rounding error is <= 2^-11 |lo|; truncating either
// part instead doubles the error of the 3xTF32 product, which was measurable after a few
// hundred steps.
__device__ __forceinline__ void split_tf32(float v, float& hi, float& lo)
{
    hi = __uint_as_float((__float_as_uint(v) + 0x1000u) & 0xFFFFE000u);
    const float r = v - hi;
    lo = __uint_as_float((__float_as_uint(r) + 0x1000u) & 0xFFFFE000u);
}

__device__ __forceinline__ bool flag_set(const int* f) { return *reinterpret_cast<const volatile int*>(f) != 0; }

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
    mbar_expect_tx(bar, O::UBytes + 4 * NF + 64 + 16 + 80 + O::XyzBytes);
    if (Bp == kChunk) {
        bulk_g2s(buf, src, O::UBytes, bar);
    } else {
        for (int r = 0; r < 6 * Np; ++r)
            bulk_g2s(buf + r * kChunk * 4, src + static_cast<int64_t>(r) * Bp, kChunk * 4, bar);
    }
    bulk_g2s(buf + O::UBytes, T.vmapP + e * NF, 4 * NF, bar);
    bulk_g2s(buf + O::UBytes + O::NbrBytes, T.fgeo + e * 16, 64, bar);
    bulk_g2s(buf + O::UBytes + O::NbrBytes + 64, T.fcode + e * 4, 16, bar);
    bulk_g2s(buf + O::UBytes + O::NbrBytes + 80, T.fbc + e * 20, 80, bar);
    bulk_g2s(buf + O::UBytes + O::NbrBytes + 160, T.fxyz + e * NF * 3, O::XyzBytes, bar);
}

// The RK registers the epilogue of work item w reads, brought into L2 ahead of
// use so that its loads wait for L2 rather than HBM (the whole element block,
// once per element). Issued one item ahead: earlier, the lines are evicted by
// the other SMs' streams before they are read.
template <int MODE>
__device__ __forceinline__ void prefetch_rk_registers(const BatchedStageArgs& A, int64_t w, int nchunk, int64_t EB)
{
    const int64_t e = w / nchunk;
    if (w - e * nchunk != 0) return;
    const uint32_t eb = static_cast<uint32_t>(EB * sizeof(float));
    if (MODE == MODE_RK4_2 || MODE == MODE_RK4_3) {
        prefetch_l2(A.x + e * EB, eb);
        prefetch_l2(A.z + e * EB, eb);
    } else if (MODE == MODE_RK4_4) {
        prefetch_l2(A.z + e * EB, eb);
        prefetch_l2(A.x + e * EB, eb);
        prefetch_l2(A.xl + e * EB, eb);
    } else if (MODE == MODE_LSRK) {
        prefetch_l2(A.res + e * EB, eb);
    }
}

// Epilogue operand loads of one chunk of kEpiNodes nodes (global, stride Bp between nodes).
constexpr int kEpiNodes = 8;
struct EpiOps {
    float a[kEpiNodes];   // x_hi (RK4_2/3/4) or res (LSRK)
    float z[kEpiNodes];   // z (RK4_2/3/4)
    float u[kEpiNodes];   // stage input (RK4_1, LSRK, conductivity)
    float l[kEpiNodes];   // x_lo (RK4_4)
};

template <int MODE>
__device__ __forceinline__ void epi_load(const BatchedStageArgs& A, int64_t base, int Bp, int nv, bool need_u, EpiOps& o)
{
    constexpr bool need_a = (MODE == MODE_RK4_2 || MODE == MODE_RK4_3 || MODE == MODE_RK4_4 || MODE == MODE_LSRK);
    constexpr bool need_z = (MODE == MODE_RK4_2 || MODE == MODE_RK4_3 || MODE == MODE_RK4_4);
    constexpr bool need_l = (MODE == MODE_RK4_4);
    const float* __restrict__ px = (MODE == MODE_LSRK ? A.res : A.x) + base;
    const float* __restrict__ pz = A.z + base;
    const float* __restrict__ pu = A.in + base;
    const float* __restrict__ pl = A.xl + base;
#pragma unroll
    for (int j = 0; j < kEpiNodes; ++j) {
        if (j < nv) {
            if (need_a) o.a[j] = px[j * Bp];
            if (need_z) o.z[j] = pz[j * Bp];
            if (need_l) o.l[j] = pl[j * Bp];
            if (need_u) o.u[j] = __ldg(pu + j * Bp);
        }
    }
}

// Stage update of one chunk: k = fe * acc - fs * u, then the RK register writes.
template <int MODE>
__device__ __forceinline__ void epi_store(const BatchedStageArgs& A, int64_t base, int Bp, int nv, bool need_u,
                                          const float* kv, float fe, float fs, float dtf, const EpiOps& o)
{
#pragma unroll
    for (int j = 0; j < kEpiNodes; ++j) {
        if (j < nv) {
            const float uc = need_u ? o.u[j] : 0.0f;
            const float k = fe * kv[j] - fs * uc;
            const int64_t ix = base + static_cast<int64_t>(j) * Bp;
            if (MODE == MODE_MULT) {
                A.out[ix] = k;
            } else if (MODE == MODE_RK4_1) {
                A.yout[ix] = uc + 0.5f * dtf * k;
                A.z[ix] = (dtf / 6.0f) * k;
            } else if (MODE == MODE_RK4_2) {
                A.yout[ix] = o.a[j] + 0.5f * dtf * k;
                A.z[ix] = o.z[j] + (dtf / 3.0f) * k;
            } else if (MODE == MODE_RK4_3) {
                A.yout[ix] = o.a[j] + dtf * k;
                A.z[ix] = o.z[j] + (dtf / 3.0f) * k;
            } else if (MODE == MODE_RK4_4) {
                float hi = o.a[j], lo = o.l[j];
                add_compensated(hi, lo, o.z[j] + (dtf / 6.0f) * k);
                A.x[ix] = hi;
                A.xl[ix] = lo;
            } else {   // MODE_LSRK
                const float rr = A.a * o.a[j] + dtf * k;
                A.res[ix] = rr;
                A.yout[ix] = uc + A.b * rr;
            }
        }
    }
}

// Adds the incident field of waves pw[q0, q1) at one TF/SF face node (coordinates xq, staged in
// shared memory) and stage time ts to the jumps: + on the total-field side (code 4), - on the
// scattered-field side (reference GlobalEvolution.cpp:551-626).
__device__ __forceinline__ void tfsf_source(const BatchedStageArgs& A, const float* xq, int q0, int q1, float ts, int code,
                                            float* dE, float* dH)
{
    float pe[3], ph[3];
    pw_eval(A.pw, q0, q1, xq[0], xq[1], xq[2], ts, pe, ph);
    const float s2 = (code == 4) ? 1.0f : -1.0f;
#pragma unroll
    for (int c = 0; c < 3; ++c) { dE[c] += s2 * pe[c]; dH[c] += s2 * ph[c]; }
}

template <int P, int MODE>
__global__ void __launch_bounds__(kThreads, 1)
    stage_tc(BatchedTables T, BatchedStageArgs A, const uint32_t* __restrict__ op_img, int64_t n_work, int* status)
{
    using O = TcOrd<P>;
    constexpr int Np = O::Np, Nfp = O::Nfp, NF = O::NF, NKS = O::NKS, N = O::N;
    extern __shared__ __align__(128) unsigned char sm[];
    unsigned char* op_hi = sm;
    unsigned char* op_lo = sm + O::OpBytes;
    unsigned char* ubuf0 = sm + 2 * O::OpBytes;
    unsigned char* ring = ubuf0 + 2 * O::UBufBytes;
    __shared__ uint64_t u_full[2], u_empty[2], w_full[2], w_empty[2], acc_full[2], acc_empty[2];
    __shared__ uint64_t corr_empty, drain_bar;
    __shared__ uint32_t tbase;
    __shared__ int s_col[O::KKp];
    __shared__ int s_err;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int Bp = static_cast<int>(T.Bpad);
    const int nchunk = Bp / kChunk;
    const int CB = Np * Bp;                      // component stride inside an element block (global)
    const int64_t EB = 6 * static_cast<int64_t>(CB);

    // ---- prologue: resident operator, column table, barriers, tensor memory
    {
        const uint4* src = reinterpret_cast<const uint4*>(op_img);
        uint4* dst = reinterpret_cast<uint4*>(op_hi);
        for (int i = tid; i < 2 * O::OpBytes / 16; i += kThreads) dst[i] = __ldg(src + i);
    }
    for (int k = tid; k < O::KKp; k += kThreads) {
        int v;
        if (k < 3 * Np) v = (kColVol << 28) | ((k % 3) << 16) | (k / 3);
        else if (k < O::KK) v = (kColFlux << 28) | ((k - 3 * Np) << 16) | (((k - 3 * Np) / Nfp) << 12) | T.Fmask[k - 3 * Np];
        else v = kColPad << 28;
        s_col[k] = v;
    }
    if (tid == 0) {
        for (int s = 0; s < 2; ++s) {
            tc::mbar_init(&u_full[s], 1);
            tc::mbar_init(&u_empty[s], kProducerThreads);
            tc::mbar_init(&w_full[s], kProducerThreads / 2);
            tc::mbar_init(&w_empty[s], 1);
            tc::mbar_init(&acc_full[s], 1);
            tc::mbar_init(&acc_empty[s], kEpiThreads);
        }
        tc::mbar_init(&corr_empty, kEpiThreads);
        tc::mbar_init(&drain_bar, 1);
        s_err = 0;
        tc::mbar_fence_init();
    }
    if (warp == kMmaWarp) {
        tc::tmem_alloc(&tbase, kTmemCols);
        tc::tmem_relinquish();
    }
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tbase;
    bool err = false;

    if (warp < kEpiWarp0) {
        // ================================================================ producers
        const int pb = tid & 63;             // incidence within the chunk
        const int kh = (tid >> 6) & 1;       // which 4 columns of the K-step
        const int grp = tid >> 7;            // K-steps grp, grp + 2, ... -> ring slot grp
        uint32_t soff[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            const int row = (c & 1) * 64 + pb;
            soff[c] = tc::smem_u32(ring) + grp * kSlot + (c >> 1) * kTile + (row >> 3) * 256 + kh * 128 +
                      (row & 7) * 16;
        }
        int it = 0;
        int uses = 0;                        // uses of this group's ring slot so far
        for (int64_t w = blockIdx.x; w < n_work; w += gridDim.x, ++it) {
            const int ub = it & 1;
            const unsigned char* buf = ubuf0 + ub * O::UBufBytes;
            const float* s_u = reinterpret_cast<const float*>(buf);          // [6][Np][64]
            const int32_t* s_nbr = reinterpret_cast<const int32_t*>(buf + O::UBytes);
            const float* s_fg = reinterpret_cast<const float*>(buf + O::UBytes + O::NbrBytes);
            const int* s_code = reinterpret_cast<const int*>(buf + O::UBytes + O::NbrBytes + 64);
            const float* s_bc = reinterpret_cast<const float*>(buf + O::UBytes + O::NbrBytes + 80);
            const float* s_xyz = reinterpret_cast<const float*>(buf + O::UBytes + O::NbrBytes + 160);
            if (flag_set(&s_err) || !tc::mbar_wait(&u_full[ub], (it >> 1) & 1)) { err = true; break; }
            const int64_t e = w / nchunk;
            const int g = static_cast<int>(w - e * nchunk);
            const int b = g * kChunk + pb;
            const float* gg = T.geo + e * 9;
            float geo[9];
#pragma unroll
            for (int q = 0; q < 9; ++q) geo[q] = __ldg(gg + q);
            const bool skip_src = (A.skip == nullptr) || A.skip[b];
            // once per item: this incidence's waves, the stage time, and which faces of the element
            // take the TF/SF source (bit f of tf_faces; bit f of tf_total: total-field side)
            int pq0 = 0, pq1 = 0;
            float ts = A.t;
            uint32_t tf_faces = 0, tf_total = 0, nb_faces = 0;   // nb_faces: faces with a neighbour trace
#pragma unroll
            for (int f = 0; f < 4; ++f) {
                const int code = s_code[f];
                nb_faces |= static_cast<uint32_t>(code == 0 || code == 4 || code == 5) << f;
            }
            if (!skip_src) {
                pq0 = A.pw_off[b];
                pq1 = A.pw_off[b + 1];
                if (A.t_base) ts = static_cast<float>(*A.t_base + static_cast<double>(A.t));
#pragma unroll
                for (int f = 0; f < 4; ++f) {
                    const int code = s_code[f];
                    tf_faces |= static_cast<uint32_t>(code == 4 || code == 5) << f;
                    tf_total |= static_cast<uint32_t>(code == 4) << f;
                }
            }
            const float* __restrict__ nin = A.in + static_cast<int64_t>(g) * kChunk + pb;
            // neighbour traces of this thread's 4 columns of a K-step (flux columns of interior faces),
            // loaded one K-step of this group ahead
            float nb[4][6], nbn[4][6];
#define DGTD_LOAD_NBR(QQ, DST)                                                                          \
    _Pragma("unroll") for (int jj = 0; jj < 4; ++jj)                                                    \
    {                                                                                                   \
        const int ci_ = s_col[(QQ) * 8 + kh * 4 + jj];                                                   \
        if ((ci_ >> 28) == kColFlux) {                                                                  \
            const int m_ = (ci_ >> 16) & 0xfff;                                                         \
            if ((nb_faces >> ((ci_ >> 12) & 0xf)) & 1u) {                                               \
                const int32_t gp_ = s_nbr[m_];                                                          \
                const int32_t en_ = gp_ / Np, node_ = gp_ - en_ * Np;                                   \
                const float* __restrict__ un_ = nin + static_cast<int64_t>(en_) * EB + node_ * Bp;      \
                _Pragma("unroll") for (int c = 0; c < 6; ++c) DST[jj][c] = __ldg(un_ + c * CB);         \
            } else {                                                                                    \
                _Pragma("unroll") for (int c = 0; c < 6; ++c) DST[jj][c] = 0.0f;                        \
            }                                                                                           \
        }                                                                                               \
    }
            // a K-step holds flux columns when it reaches past the 3Np volume columns
            if (grp * 8 + 7 >= 3 * Np) { DGTD_LOAD_NBR(grp, nb) }
            for (int q = grp; q < NKS; q += 2) {
                if (q + 2 < NKS && (q + 2) * 8 + 7 >= 3 * Np) { DGTD_LOAD_NBR(q + 2, nbn) }
                float v[6][4];
                // fields at the (at most two) nodes this thread's volume columns use
                const int kq0 = q * 8 + kh * 4;
                const int jA = kq0 / 3;
                // Volume columns take F_j - F_0 (node 0 of the element): Dr, Ds and Dt annihilate
                // constants, so the product is unchanged in exact arithmetic, while the common part
                // of F no longer meets the rounding of the tf32 operator (each row of Dr sums to 0
                // with terms ~100x the result, so that error would otherwise be amplified).
                float FA[6], FB[6];
                if (kq0 < 3 * Np) {
                    float F0[6];
#pragma unroll
                    for (int c = 0; c < 6; ++c) F0[c] = s_u[(c * Np) * kChunk + pb];
#pragma unroll
                    for (int c = 0; c < 6; ++c) FA[c] = s_u[(c * Np + jA) * kChunk + pb] - F0[c];
                    if (jA + 1 < Np && kq0 + 3 < 3 * Np) {
#pragma unroll
                        for (int c = 0; c < 6; ++c) FB[c] = s_u[(c * Np + jA + 1) * kChunk + pb] - F0[c];
                    }
                }
#pragma unroll
                for (int jj = 0; jj < 4; ++jj) {
                    const int k = q * 8 + kh * 4 + jj;
                    const int ci = s_col[k];
                    const int kind = ci >> 28;
                    if (kind == kColFlux) {
                        const int m = (ci >> 16) & 0xfff, f = (ci >> 12) & 0xf, vm = ci & 0xfff;
                        const float4 fg = reinterpret_cast<const float4*>(s_fg)[f];
                        const float nx = fg.x, ny = fg.y, nz = fg.z;
                        const float hf = 0.5f * fg.w;
                        const float* bc = s_bc + f * 5;
                        const float cE1 = bc[0], cE2 = bc[1], cH1 = bc[2], cH2 = bc[3];
                        const float aE = bc[4], aH = bc[4];
                        float uM[6];
#pragma unroll
                        for (int c = 0; c < 6; ++c) uM[c] = s_u[(c * Np + vm) * kChunk + pb];
                        // jumps with the boundary rule of the face (branch-free: neighbour traces are
                        // zero where the coefficient is)
                        float dE[3], dH[3];
#pragma unroll
                        for (int c = 0; c < 3; ++c) {
                            dE[c] = cE1 * nb[jj][c] + cE2 * uM[c];
                            dH[c] = cH1 * nb[jj][c + 3] + cH2 * uM[c + 3];
                        }
                        if ((tf_faces >> f) & 1u)
                            tfsf_source(A, s_xyz + m * 3, pq0, pq1, ts, ((tf_total >> f) & 1u) ? 4 : 5, dE, dH);
                        const float ndE = nx * dE[0] + ny * dE[1] + nz * dE[2];
                        const float ndH = nx * dH[0] + ny * dH[1] + nz * dH[2];
                        v[0][jj] = hf * ((ny * dH[2] - nz * dH[1]) + aE * (dE[0] - ndE * nx));
                        v[1][jj] = hf * ((nz * dH[0] - nx * dH[2]) + aE * (dE[1] - ndE * ny));
                        v[2][jj] = hf * ((nx * dH[1] - ny * dH[0]) + aE * (dE[2] - ndE * nz));
                        v[3][jj] = hf * (-(ny * dE[2] - nz * dE[1]) + aH * (dH[0] - ndH * nx));
                        v[4][jj] = hf * (-(nz * dE[0] - nx * dE[2]) + aH * (dH[1] - ndH * ny));
                        v[5][jj] = hf * (-(nx * dE[1] - ny * dE[0]) + aH * (dH[2] - ndH * nz));
                    } else if (kind == kColVol) {
                        const int d = (ci >> 16) & 0xff, j = ci & 0xffff;
                        const float gx = d == 0 ? geo[0] : (d == 1 ? geo[3] : geo[6]);
                        const float gy = d == 0 ? geo[1] : (d == 1 ? geo[4] : geo[7]);
                        const float gz = d == 0 ? geo[2] : (d == 1 ? geo[5] : geo[8]);
                        const bool a = (j == jA);
                        const float Ex = a ? FA[0] : FB[0], Ey = a ? FA[1] : FB[1], Ez = a ? FA[2] : FB[2];
                        const float Hx = a ? FA[3] : FB[3], Hy = a ? FA[4] : FB[4], Hz = a ? FA[5] : FB[5];
                        // E rows: g x H (curl H); H rows: -(g x E) (-curl E)
                        v[0][jj] = gy * Hz - gz * Hy;
                        v[1][jj] = gz * Hx - gx * Hz;
                        v[2][jj] = gx * Hy - gy * Hx;
                        v[3][jj] = gz * Ey - gy * Ez;
                        v[4][jj] = gx * Ez - gz * Ex;
                        v[5][jj] = gy * Ex - gx * Ey;
                    } else {
#pragma unroll
                        for (int c = 0; c < 6; ++c) v[c][jj] = 0.0f;
                    }
                }
                // ---- hand the K-step to the tensor core through this group's ring slot
                if (uses >= 1 && (flag_set(&s_err) || !tc::mbar_wait(&w_empty[grp], (uses - 1) & 1))) {
                    err = true;
                    break;
                }
#pragma unroll
                for (int c = 0; c < 6; ++c) {
                    float h[4], l[4];
#pragma unroll
                    for (int jj = 0; jj < 4; ++jj) split_tf32(v[c][jj], h[jj], l[jj]);
                    st_shared_v4(soff[c], h[0], h[1], h[2], h[3]);
                    st_shared_v4(soff[c] + kWStep, l[0], l[1], l[2], l[3]);
                }
                tc::fence_proxy_async();
                tc::mbar_arrive(&w_full[grp]);
                ++uses;
#pragma unroll
                for (int jj = 0; jj < 4; ++jj)
#pragma unroll
                    for (int c = 0; c < 6; ++c) nb[jj][c] = nbn[jj][c];
            }
#undef DGTD_LOAD_NBR
            if (err) break;
            tc::mbar_arrive(&u_empty[ub]);        // this thread is done with the staged block
        }
    } else if (warp < kEpiWarp0 + 4) {
        // ================================================================ epilogue
        const int lq = warp & 3;                  // TMEM lane quarter of this warp
        const int r = lq * 32 + lane;             // accumulator row within each tile
        const int blr = r & 63;
        const float dtf = A.dt;
        constexpr int NCHT = 3 * O::NCH;          // 8-node chunks per item (3 tiles)
        int it = 0;
        for (int64_t w = blockIdx.x; w < n_work; w += gridDim.x, ++it) {
            const int64_t e = w / nchunk;
            const int g = static_cast<int>(w - e * nchunk);
            const int abuf = it & 1;
            const float ie = __ldg(T.mat + e * 3 + 0), im = __ldg(T.mat + e * 3 + 1), se = __ldg(T.mat + e * 3 + 2);
            const bool need_u = (MODE == MODE_RK4_1) || (MODE == MODE_LSRK) || (se != 0.0f);
            const int64_t eoff = e * EB + static_cast<int64_t>(g) * kChunk + blr;
            const uint32_t tacc = tmem + abuf * kAccStride + (static_cast<uint32_t>(lq * 32) << 16);
            auto chunk_base = [&](int n) {
                const int t = n / O::NCH, cb = (n % O::NCH) * kEpiNodes;
                return eoff + static_cast<int64_t>(2 * t + (r >> 6)) * CB + static_cast<int64_t>(cb) * Bp;
            };
            auto chunk_nv = [&](int n) { return min(kEpiNodes, Np - (n % O::NCH) * kEpiNodes); };
            // one chunk: accumulator columns -> registers, release the buffer after the last one, update
            auto process = [&](int n, const EpiOps& o) {
                const int t = n / O::NCH, cb = (n % O::NCH) * kEpiNodes;
                float kv[kEpiNodes];
                tc::tmem_ld8(tacc + t * N + cb, kv);
                tc::tmem_ld_wait();
                if (n == NCHT - 1) {
                    tc::fence_before_sync();
                    tc::mbar_arrive(&acc_empty[abuf]);
                }
                const int c = 2 * t + (r >> 6);
                const float fe = (c < 3) ? ie : im, fs = (c < 3) ? se : 0.0f;
                epi_store<MODE>(A, chunk_base(n), Bp, chunk_nv(n), need_u, kv, fe, fs, dtf, o);
            };
            if (warp == kEpiWarp0 && lane == 0 && w + gridDim.x < n_work)
                prefetch_rk_registers<MODE>(A, w + gridDim.x, nchunk, EB);
            EpiOps o0, o1;
            epi_load<MODE>(A, chunk_base(0), Bp, chunk_nv(0), need_u, o0);
            if (flag_set(&s_err) || !tc::mbar_wait(&acc_full[abuf], (it >> 1) & 1)) { err = true; break; }
            tc::fence_after_sync();
            // fold the correction accumulator into this item's accumulator (FP32, round to nearest)
            // and hand it back to the MMA issuer for the next item
            {
                const uint32_t tcorr = tmem + kCorrCol + (static_cast<uint32_t>(lq * 32) << 16);
#pragma unroll 1
                for (int n = 0; n < NCHT; ++n) {
                    const int t = n / O::NCH, cb = (n % O::NCH) * kEpiNodes;
                    float mv[kEpiNodes], cv[kEpiNodes];
                    tc::tmem_ld8(tacc + t * N + cb, mv);
                    tc::tmem_ld8(tcorr + t * N + cb, cv);
                    tc::tmem_ld_wait();
#pragma unroll
                    for (int q = 0; q < kEpiNodes; ++q) mv[q] += cv[q];
                    tc::tmem_st8(tacc + t * N + cb, mv);
                }
                tc::tmem_st_wait();
                tc::fence_before_sync();
                tc::mbar_arrive(&corr_empty);
            }
#pragma unroll 1
            for (int n = 0; n < NCHT; n += 2) {
                if (n + 1 < NCHT) epi_load<MODE>(A, chunk_base(n + 1), Bp, chunk_nv(n + 1), need_u, o1);
                process(n, o0);
                if (n + 1 < NCHT) {
                    if (n + 2 < NCHT) epi_load<MODE>(A, chunk_base(n + 2), Bp, chunk_nv(n + 2), need_u, o0);
                    process(n + 1, o1);
                }
            }
        }
    } else if (warp == kMmaWarp) {
        // ================================================================ MMA issuer
        if (lane == 0) {
            const uint32_t idesc = tc::idesc_tf32(128, N);
            const uint32_t ring_u32 = tc::smem_u32(ring);
            int it = 0;
            int uses0 = 0, uses1 = 0;        // consumed K-steps per ring slot
            for (int64_t w = blockIdx.x; w < n_work; w += gridDim.x, ++it) {
                const int abuf = it & 1, ause = it >> 1;
                if (ause >= 1 && (flag_set(&s_err) || !tc::mbar_wait(&acc_empty[abuf], (ause - 1) & 1))) {
                    err = true;
                    break;
                }
                tc::fence_after_sync();
                const uint32_t dacc = tmem + abuf * kAccStride;
                for (int q = 0; q < NKS; ++q) {
                    const int slot = q & 1;
                    const int use = slot ? uses1 : uses0;
                    if (flag_set(&s_err) || !tc::mbar_wait(&w_full[slot], use & 1)) { err = true; break; }
                    if (slot) ++uses1; else ++uses0;
                    tc::fence_after_sync();
                    const uint32_t ah0 = ring_u32 + slot * kSlot, al0 = ah0 + kWStep;
                    const uint64_t bh = tc::smem_desc(tc::smem_u32(op_hi + q * O::OpStep));
                    const uint64_t blo = tc::smem_desc(tc::smem_u32(op_lo + q * O::OpStep));
                    // W_hi Op_hi into the item's accumulator; the two small correction products into
                    // a separate one, so that the truncation in each accumulation is relative to the
                    // small correction sum, not to the full result
#pragma unroll
                    for (int t = 0; t < 3; ++t)
                        tc::mma_tf32(dacc + t * N, tc::smem_desc(ah0 + t * kTile), bh, idesc, q > 0);
                    if (q == 0 && it >= 1) {
                        // the epilogue has folded the previous item's corrections into its accumulator
                        if (flag_set(&s_err) || !tc::mbar_wait(&corr_empty, (it - 1) & 1)) { err = true; break; }
                        tc::fence_after_sync();
                    }
#pragma unroll
                    for (int t = 0; t < 3; ++t) {
                        const uint32_t dc = tmem + kCorrCol + t * N;
                        const uint64_t ah = tc::smem_desc(ah0 + t * kTile);
                        const uint64_t al = tc::smem_desc(al0 + t * kTile);
                        tc::mma_tf32(dc, al, bh, idesc, q > 0);
                        tc::mma_tf32(dc, ah, blo, idesc, true);
                    }
                    if (err) break;
                    tc::mma_commit(&w_empty[slot]);
                }
                if (err) break;
                tc::mma_commit(&acc_full[abuf]);
            }
            if (err) {
                // wait (bounded) for the MMAs already issued before the tensor memory is freed
                tc::mma_commit(&drain_bar);
                tc::mbar_wait(&drain_bar, 0);
            }
        }
    } else if (warp == kCopyWarp) {
        // ================================================================ copy issuer
        if (lane == 0) {
            int it = 0;
            int issued0 = 0, issued1 = 0;     // copies issued per staging buffer
            for (int64_t w = blockIdx.x; w < n_work; w += gridDim.x, ++it) {
                const int ub = it & 1, use = it >> 1;
                if (use >= 1 && (flag_set(&s_err) || !tc::mbar_wait(&u_empty[ub], (use - 1) & 1))) {
                    err = true;
                    break;
                }
                prefetch_item<P>(T, A.in, w, nchunk, Bp, ubuf0 + ub * O::UBufBytes, &u_full[ub]);
                if (ub) ++issued1; else ++issued0;
                if (it == 0) prefetch_rk_registers<MODE>(A, w, nchunk, EB);   // later items: the epilogue
            }
            if (err) {
                // wait (bounded) for this CTA's copies still in flight
                if (issued0) tc::mbar_wait(&u_full[0], (issued0 - 1) & 1);
                if (issued1) tc::mbar_wait(&u_full[1], (issued1 - 1) & 1);
            }
        }
    }

    if (err) atomicExch(&s_err, 1);
    tc::fence_before_sync();
    __syncthreads();
    if (tid == 0 && s_err) atomicExch(status, 1);
    if (warp == kMmaWarp) {
        tc::fence_after_sync();
        tc::tmem_dealloc(tmem, kTmemCols);
    }
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

// Host image of Op = [Dr | Ds | Dt | LIFT]^T as the kernel's K-major B operand:
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
            if (k >= 3 * Np) v = ref.LIFT[static_cast<size_t>(i) * NF + (k - 3 * Np)];
            else {
                const int type = k % 3, j = k / 3;
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

namespace {

// True the first time it is called for the current device (per call site): the
// dynamic shared-memory attribute of a kernel is set once per device, thread-safely.
inline bool first_use_on_device(std::atomic<uint64_t>& seen)
{
    int dev = 0;
    cudaGetDevice(&dev);
    const uint64_t bit = uint64_t(1) << (dev & 63);
    return (seen.fetch_or(bit) & bit) == 0;
}

template <int P, int MODE>
void launch_tc_instance(const BatchedTables& T, const BatchedStageArgs& A, const uint32_t* op_img, int* status,
                        int64_t grid, int64_t n_work, cudaStream_t s)
{
    static std::atomic<uint64_t> seen{0};
    if (first_use_on_device(seen)) {
        cudaError_t e = cudaFuncSetAttribute(stage_tc<P, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             static_cast<int>(TcOrd<P>::smem));
        if (e != cudaSuccess) throw std::runtime_error(std::string("tc smem attribute: ") + cudaGetErrorString(e));
    }
    stage_tc<P, MODE><<<static_cast<unsigned>(grid), kThreads, TcOrd<P>::smem, s>>>(T, A, op_img, n_work, status);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) throw std::runtime_error(std::string("tc stage kernel: ") + cudaGetErrorString(e));
}

template <int P>
void launch_tc_order(const BatchedTables& T, const BatchedStageArgs& A, const uint32_t* op_img, int* status,
                     int64_t grid, int64_t n_work, cudaStream_t s)
{
    switch (A.mode) {
    case MODE_MULT: launch_tc_instance<P, MODE_MULT>(T, A, op_img, status, grid, n_work, s); break;
    case MODE_RK4_1: launch_tc_instance<P, MODE_RK4_1>(T, A, op_img, status, grid, n_work, s); break;
    case MODE_RK4_2: launch_tc_instance<P, MODE_RK4_2>(T, A, op_img, status, grid, n_work, s); break;
    case MODE_RK4_3: launch_tc_instance<P, MODE_RK4_3>(T, A, op_img, status, grid, n_work, s); break;
    case MODE_RK4_4: launch_tc_instance<P, MODE_RK4_4>(T, A, op_img, status, grid, n_work, s); break;
    case MODE_LSRK: launch_tc_instance<P, MODE_LSRK>(T, A, op_img, status, grid, n_work, s); break;
    default: throw std::runtime_error("tensor-core stage: unknown stage mode");
    }
}

}  // namespace

void launch_stage_tc(const BatchedTables& T, const BatchedStageArgs& A, const uint32_t* op_img, int* status, int n_sm,
                     cudaStream_t s)
{
    const int64_t n_work = T.K * (T.Bpad / kChunk);
    if (reinterpret_cast<uintptr_t>(A.in) % 16 != 0)
        throw std::runtime_error("tensor-core stage: the input state must be 16-byte aligned (bulk async copies)");
    const int64_t grid = std::min<int64_t>(n_work, static_cast<int64_t>(n_sm));
    switch (T.p) {
    case 1: launch_tc_order<1>(T, A, op_img, status, grid, n_work, s); break;
    case 2: launch_tc_order<2>(T, A, op_img, status, grid, n_work, s); break;
    case 3: launch_tc_order<3>(T, A, op_img, status, grid, n_work, s); break;
    case 4: launch_tc_order<4>(T, A, op_img, status, grid, n_work, s); break;
    default: throw std::runtime_error("tensor-core stage kernel supports orders 1..4");
    }
}

}  // namespace dgtd
