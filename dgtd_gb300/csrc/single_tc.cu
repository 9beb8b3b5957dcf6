// Single-instance FP32 stage kernel with the contractions on the tensor cores (tcgen05, 3xTF32).
//
// The single-instance form keeps one solve (or a few stacked incidences) in the reference
// layout [b][c][e*Np+i] in FP32. There are no incidence lanes to fill an MMA tile, so the
// wide dimension is made of elements: a work item is kG = 8 consecutive elements of one
// incidence, and the right-hand side of its 48 (component, element) columns is
//
//   Dr F, Ds F, Dt F   (operator rows = nodes, K = Np source nodes)   and   LIFT Flux  (K = 4 Nfp),
//
// four products whose A operand is a reference-element matrix (M = 128 rows = nodes, Np <= 84
// used) and whose B operand holds the item's raw fields (minus each element's node-0 value:
// Dr, Ds and Dt annihilate constants) or its Fscale/2-scaled upwind fluxes. The chain rule
// (geometric factors), the curl, 1/eps, 1/mu, -sigma/eps E and the RK stage update run in the
// epilogue in FP32, with round-to-nearest, from four tensor-memory accumulators of 48 columns.
// That keeps each accumulator to at most max(Np, 4 Nfp)/8 K-steps (the tensor core's FP32
// accumulation truncates toward zero at every MMA) and leaves the producers only the split of
// the fields and the flux arithmetic (reference HesthavenEvolution::Mult,
// src/evolution/HesthavenEvolution.cpp:450-541; boundary rules of
// src/components/DGOperatorFactory.h:21-45; TF/SF source of src/evolution/GlobalEvolution.cpp:551-626).
//
// 3xTF32: operand v = hi + lo with hi the nearest tf32 value and lo the nearest tf32 value of the
// remainder; A_hi B_hi + A_lo B_hi + A_hi B_lo per K-step. The A operand (precomputed on the
// host) is the same for every work item; it is streamed from global memory (L2-resident, a few
// hundred KB) through a ring of shared-memory slots, one K-step of one matrix (hi and lo, 8 KB)
// per slot, as many slots as the order leaves room for.
//
// One persistent CTA per SM, warp-specialised, all hand-offs through mbarriers with bounded waits:
//   warps 0-7  producers: stage the item's fields, face geometry and face codes in shared memory
//              (coalesced loads), then build its whole B operand (volume then flux K-steps, hi
//              and lo) into one of two B buffers, 16-byte stores (conflict-free in the K-major
//              layout); only the neighbour traces of the flux come from global memory;
//   warps 8-11 epilogue (one per TMEM lane quarter: thread = node), with the item's RK-register
//              rows brought into L2 one item ahead;
//   warp 12    tensor-memory owner and MMA issuer (one thread);
//   warp 13    copy issuer (one thread): bulk copies of the A slots.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "fp64_stage.cuh"
#include "refelem.hpp"
#include "single_tc.hpp"
#include "tc_common.cuh"

namespace dgtd {

namespace {

constexpr int kG = 8;                    // elements per work item
constexpr int kNcol = 6 * kG;            // B rows / accumulator columns: n = c * kG + e
constexpr int kThreads = 448;
constexpr int kProducerThreads = 256;    // warps 0-7
constexpr int kEpiWarp0 = 8;             // warps 8-11
constexpr int kEpiThreads = 128;
constexpr int kMmaWarp = 12;
constexpr int kCopyWarp = 13;
constexpr int kBStep = kNcol * 32;       // one K-step of B (48 rows x 8 tf32), one part: 1536 B
constexpr int kATile = 128 * 32;         // one K-step of A (128 rows x 8 tf32), one part: 4 KB
constexpr int kASlot = 2 * kATile;       // hi + lo
constexpr int kMaxSlots = 16;            // A ring slots at most (the ring takes what shared memory is left)
// Copies of the A image in global memory; CTA i streams copy i % kReplicas. Every CTA reads the
// same slots at nearly the same time, and one copy makes those lines an L2 hot spot.
constexpr int kReplicas = 16;
constexpr uint32_t kAccCols = 4 * kNcol; // dr, ds, dt, lift: 192 columns per item
constexpr uint32_t kAccStride = 256;     // TMEM columns between the two item accumulator sets
constexpr uint32_t kTmemCols = 512;

template <int P>
struct Stc {
    static constexpr int Np = (P + 1) * (P + 2) * (P + 3) / 6;
    static constexpr int Nfp = (P + 1) * (P + 2) / 2;
    static constexpr int NF = 4 * Nfp;
    static constexpr int KV = (Np + 7) / 8 * 8;
    static constexpr int NKV = KV / 8;
    static constexpr int KF = (NF + 7) / 8 * 8;
    static constexpr int NKF = KF / 8;
    static constexpr int NA = 3 * NKV + NKF;                 // A slots per item
    static constexpr int BPart = (NKV + NKF) * kBStep;      // one part (hi or lo) of an item's B
    static constexpr int BBuf = 2 * BPart;
    static constexpr int FBuf = 6 * kG * Np * 4;              // the item's fields [c][e * Np + i]
    static constexpr int TBuf = kG * (16 + 4) * 4;            // its face geometry and face codes
    static constexpr int Fixed = 2 * BBuf + 2 * (FBuf + TBuf);
    // A ring: as many 8 KB slots as fit in 223 KB of dynamic shared memory (4 at p = 6, 16 at p <= 4)
    static constexpr int NSlot0 = (223 * 1024 - Fixed) / kASlot;
    static constexpr int NSlot = NSlot0 > kMaxSlots ? kMaxSlots : NSlot0;
    static constexpr size_t smem = static_cast<size_t>(Fixed) + static_cast<size_t>(NSlot) * kASlot;
    static_assert(NSlot >= 2, "A ring");
    static_assert(Np <= 128, "one M tile of nodes");
    static_assert(2 * kAccStride <= kTmemCols && kAccCols <= kAccStride, "tensor memory layout");
};

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(tc::smem_u32(bar)), "r"(bytes)
                 : "memory");
}

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

// v = hi + lo: hi the nearest tf32 value (ties away from zero), lo the remainder rounded the same way.
__device__ __forceinline__ void split_tf32(float v, float& hi, float& lo)
{
    hi = __uint_as_float((__float_as_uint(v) + 0x1000u) & 0xFFFFE000u);
    const float r = v - hi;
    lo = __uint_as_float((__float_as_uint(r) + 0x1000u) & 0xFFFFE000u);
}

__device__ __forceinline__ bool flag_set(const int* f) { return *reinterpret_cast<const volatile int*>(f) != 0; }

// Stores 4 consecutive K columns (k0 % 4 == 0) of B row n, hi and lo, into the item's B buffer.
__device__ __forceinline__ void store_b4(uint32_t bbase, int bpart, int ks, int n, int khalf, const float* v)
{
    float h[4], l[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) split_tf32(v[q], h[q], l[q]);
    const uint32_t off = static_cast<uint32_t>(ks * kBStep + (n >> 3) * 256 + khalf * 128 + (n & 7) * 16);
    st_shared_v4(bbase + off, h[0], h[1], h[2], h[3]);
    st_shared_v4(bbase + bpart + off, l[0], l[1], l[2], l[3]);
}

// Fscale/2-scaled upwind flux of the six components at face node a of face f of element e
// (the reference's jumps, boundary rules and TF/SF source; same arithmetic as the SIMT stage).
// The element's own fields, face geometry and face codes come from the item's staged copy in
// shared memory (sf: [c][el * Np + i]; sg: [el][16]; sc: [el][4]); the neighbour traces from
// global memory.
template <int P>
__device__ __forceinline__ void face_flux(const TablesF32& T, const StageArgsF32& A, const float* __restrict__ in,
                                          const float* sf, const float* sg, const int* sc, const int* sfm, int el,
                                          int64_t e, int f, int a, int b, bool skip_src, float* out)
{
    using O = Stc<P>;
    constexpr int Np = O::Np, Nfp = O::Nfp;
    const int64_t N = T.N;
    const int vm = sfm[f * Nfp + a];
    const int code = sc[el * 4 + f];
    const float4 fg = reinterpret_cast<const float4*>(sg + el * 16)[f];
    const float nx = fg.x, ny = fg.y, nz = fg.z, fs = fg.w;
    const int64_t gm = e * Np + vm;
    float uM[6], dE[3], dH[3];
#pragma unroll
    for (int c = 0; c < 6; ++c) uM[c] = sf[c * (kG * Np) + el * Np + vm];
    float aE = T.alpha, aH = T.alpha;
    if (code == 0 || code == 4 || code == 5) {
        const int64_t gp = __ldg(T.vmapP + (e * 4 + f) * Nfp + a);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            dE[c] = __ldg(in + c * N + gp) - uM[c];
            dH[c] = __ldg(in + (c + 3) * N + gp) - uM[c + 3];
        }
        if (code != 0 && !skip_src) {
            float pe[3], ph[3];
            fp64::eval_pw<float>(A.pw, A.n_pw, b, T.xyz[gm], T.xyz[N + gm], T.xyz[2 * N + gm], static_cast<float>(A.t),
                                 pe, ph);
            const float sg = (code == 4) ? 1.0f : -1.0f;
#pragma unroll
            for (int c = 0; c < 3; ++c) { dE[c] += sg * pe[c]; dH[c] += sg * ph[c]; }
        }
    } else if (code == 1 || code == 6) {           // PEC
#pragma unroll
        for (int c = 0; c < 3; ++c) { dE[c] = -2.0f * uM[c]; dH[c] = 0.0f; }
    } else if (code == 2 || code == 7) {           // PMC
#pragma unroll
        for (int c = 0; c < 3; ++c) { dE[c] = 0.0f; dH[c] = -2.0f * uM[c + 3]; }
    } else if (code == 3 || code == 8) {           // SMA: penalty 1 regardless of alpha
#pragma unroll
        for (int c = 0; c < 3; ++c) { dE[c] = -uM[c]; dH[c] = -uM[c + 3]; }
        aE = 1.0f; aH = 1.0f;
    } else {                                        // open: zero jump
#pragma unroll
        for (int c = 0; c < 3; ++c) { dE[c] = 0.0f; dH[c] = 0.0f; }
    }
    const float ndE = nx * dE[0] + ny * dE[1] + nz * dE[2];
    const float ndH = nx * dH[0] + ny * dH[1] + nz * dH[2];
    const float h = 0.5f * fs;
    out[0] = h * ((ny * dH[2] - nz * dH[1]) + aE * (dE[0] - ndE * nx));
    out[1] = h * ((nz * dH[0] - nx * dH[2]) + aE * (dE[1] - ndE * ny));
    out[2] = h * ((nx * dH[1] - ny * dH[0]) + aE * (dE[2] - ndE * nz));
    out[3] = h * (-(ny * dE[2] - nz * dE[1]) + aH * (dH[0] - ndH * nx));
    out[4] = h * (-(nz * dE[0] - nx * dE[2]) + aH * (dH[1] - ndH * ny));
    out[5] = h * (-(nx * dE[1] - ny * dE[0]) + aH * (dH[2] - ndH * nz));
}

template <int P, int MODE>
__global__ void __launch_bounds__(kThreads, 1)
    stage_tc1(TablesF32 T, StageArgsF32 A, const uint32_t* __restrict__ a_img, int64_t n_items, int64_t items_per_b,
              int* status)
{
    using O = Stc<P>;
    constexpr int Np = O::Np, Nfp = O::Nfp, NF = O::NF, NKV = O::NKV, NA = O::NA;
    extern __shared__ __align__(128) unsigned char sm[];
    unsigned char* bbuf0 = sm;
    unsigned char* aring = sm + 2 * O::BBuf;
    constexpr int kNSlot = O::NSlot;
    unsigned char* fbuf0 = aring + kNSlot * kASlot;             // [2] x (fields | face geometry | codes)
    __shared__ uint64_t bvol_full[2], bflux_full[2], b_empty[2], acc_full[2], acc_empty[2], geo_full[2];
    __shared__ uint64_t f_full[2];
    __shared__ int s_fmask[4 * Nfp];
    __shared__ uint64_t a_full[kMaxSlots], a_empty[kMaxSlots];
    __shared__ uint64_t drain_bar;
    __shared__ uint32_t tbase;
    __shared__ int s_err;
    __shared__ float s_geo[2][kG * 9], s_mat[2][kG * 3];   // epilogue: the item's element factors

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int64_t N = T.N;

    if (tid == 0) {
        for (int s = 0; s < 2; ++s) {
            tc::mbar_init(&bvol_full[s], kProducerThreads);
            tc::mbar_init(&bflux_full[s], kProducerThreads);
            tc::mbar_init(&b_empty[s], 1);
            tc::mbar_init(&acc_full[s], 1);
            tc::mbar_init(&acc_empty[s], kEpiThreads);
            tc::mbar_init(&geo_full[s], kEpiThreads);
            tc::mbar_init(&f_full[s], kProducerThreads);
        }
        for (int s = 0; s < kNSlot; ++s) {
            tc::mbar_init(&a_full[s], 1);
            tc::mbar_init(&a_empty[s], 1);
        }
        tc::mbar_init(&drain_bar, 1);
        s_err = 0;
        tc::mbar_fence_init();
    }
    for (int q = tid; q < 4 * Nfp; q += kThreads) s_fmask[q] = __ldg(T.Fmask + q);
    if (warp == kMmaWarp) {
        tc::tmem_alloc(&tbase, kTmemCols);
        tc::tmem_relinquish();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tbase;
    bool err = false;

    if (warp < kEpiWarp0) {
        // ================================================================ producers
        int it = 0;
        for (int64_t w = blockIdx.x; w < n_items; w += gridDim.x, ++it) {
            const int buf = it & 1, use = it >> 1;
            const int64_t b64 = w / items_per_b;
            const int b = static_cast<int>(b64);
            const int64_t e0 = (w - b64 * items_per_b) * kG;
            const int nel = static_cast<int>(min(static_cast<int64_t>(kG), T.K - e0));
            const float* __restrict__ in = A.in + b64 * 6 * N;
            const uint32_t bb = tc::smem_u32(bbuf0 + buf * O::BBuf);
            if (use >= 1 && (flag_set(&s_err) || !tc::mbar_wait(&b_empty[buf], (use - 1) & 1))) { err = true; break; }
            const bool skip_src = (A.skip != nullptr) && A.skip[b];
            // ---- stage the item's fields (6 contiguous runs of nel * Np values, coalesced loads),
            // face geometry and face codes; the buffer of this parity was last read for item it - 2,
            // which every producer finished before the MMA released its B buffer (b_empty above)
            float* sf = reinterpret_cast<float*>(fbuf0 + buf * (O::FBuf + O::TBuf));
            float* sgeo = sf + 6 * kG * Np;
            int* scode = reinterpret_cast<int*>(sgeo + kG * 16);
            for (int q = tid; q < 6 * kG * Np; q += kProducerThreads) {
                const int c = q / (kG * Np), r = q - c * (kG * Np);
                sf[q] = (r < nel * Np) ? __ldg(in + c * N + e0 * Np + r) : 0.0f;
            }
            for (int q = tid; q < kG * 20; q += kProducerThreads) {
                if (q < kG * 16) sgeo[q] = (q / 16 < nel) ? __ldg(T.fgeo + e0 * 16 + q) : 0.0f;
                else {
                    const int r = q - kG * 16;
                    scode[r] = (r / 4 < nel) ? __ldg(T.fcode + e0 * 4 + r) : 0;
                }
            }
            tc::mbar_arrive(&f_full[buf]);
            if (flag_set(&s_err) || !tc::mbar_wait(&f_full[buf], use & 1)) { err = true; break; }
            // ---- volume: B[(c, e), j] = F_c(e, j) - F_c(e, 0); task = (j quad, row n)
            for (int task = tid; task < (O::KV / 4) * kNcol; task += kProducerThreads) {
                const int jq = task / kNcol, n = task - jq * kNcol;
                const int c = n / kG, e = n - c * kG;
                float v[4] = {0.0f, 0.0f, 0.0f, 0.0f};
                if (e < nel) {
                    const float* p = sf + c * (kG * Np) + e * Np;
                    const float f0 = p[0];
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const int j = jq * 4 + q;
                        if (j < Np) v[q] = p[j] - f0;
                    }
                }
                store_b4(bb, O::BPart, jq >> 1, n, jq & 1, v);
            }
            tc::fence_proxy_async();
            tc::mbar_arrive(&bvol_full[buf]);
            // ---- flux: B[(c, e), m] = Fscale/2 * flux_c at face node m; task = (m quad, element)
            for (int task = tid; task < (O::KF / 4) * kG; task += kProducerThreads) {
                const int mq = task / kG, e = task - mq * kG;
                float v[6][4];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int m = mq * 4 + q;
                    float fl[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
                    if (e < nel && m < NF) {
                        const int f = m / Nfp, a = m - f * Nfp;
                        face_flux<P>(T, A, in, sf, sgeo, scode, s_fmask, e, e0 + e, f, a, b, skip_src, fl);
                    }
#pragma unroll
                    for (int c = 0; c < 6; ++c) v[c][q] = fl[c];
                }
#pragma unroll
                for (int c = 0; c < 6; ++c) store_b4(bb, O::BPart, NKV + (mq >> 1), c * kG + e, mq & 1, v[c]);
            }
            tc::fence_proxy_async();
            tc::mbar_arrive(&bflux_full[buf]);
        }
    } else if (warp < kEpiWarp0 + 4) {
        // ================================================================ epilogue
        const int lq = warp & 3;
        const int etid = tid - kEpiWarp0 * 32;      // 0..127
        const int i = lq * 32 + lane;              // node of this thread (TMEM lane)
        const bool active = i < Np;
        const float dtf = A.dt;
        constexpr bool kNeedX = (MODE == MODE_RK4_2 || MODE == MODE_RK4_3);
        constexpr bool kNeedZ = (MODE == MODE_RK4_2 || MODE == MODE_RK4_3 || MODE == MODE_RK4_4);
        constexpr bool kNeedU = (MODE == MODE_RK4_1 || MODE == MODE_LSRK);
        // RK-register rows of one item brought into L2 ahead of use (one item ahead), so that the
        // per-target loads below wait for L2 rather than HBM
        auto prefetch_item = [&](int64_t w) {
            const int64_t pb = w / items_per_b;
            const int64_t pe0 = (w - pb * items_per_b) * kG;
            if (pe0 + kG > T.K) return;              // a partial last item: not a 16-byte multiple
            const uint32_t bytes = static_cast<uint32_t>(kG * Np * sizeof(float));
            for (int c = 0; c < 6; ++c) {
                const int64_t off = pb * 6 * N + c * N + pe0 * Np;
                if (kNeedX) prefetch_l2(A.x + off, bytes);
                if (kNeedZ) prefetch_l2(A.z + off, bytes);
                if (kNeedU) prefetch_l2(A.in + off, bytes);
                if (MODE == MODE_LSRK) prefetch_l2(A.res + off, bytes);
            }
        };
        if (etid == 0 && blockIdx.x < n_items) prefetch_item(blockIdx.x);
        // the items' geometric factors and material scales, staged in shared memory for the 128
        // threads: item it's into s_geo[it & 1] (one value per thread), loaded during item it - 1
        auto factor = [&](int64_t w) -> float {
            const int64_t pb = w / items_per_b;
            const int64_t pe0 = (w - pb * items_per_b) * kG;
            const int pnel = static_cast<int>(min(static_cast<int64_t>(kG), T.K - pe0));
            if (etid < kG * 9) return (etid / 9 < pnel) ? __ldg(T.geo + pe0 * 9 + etid) : 0.0f;
            const int q = etid - kG * 9;
            if (q < kG * 3) return (q / 3 < pnel) ? __ldg(T.mat + pe0 * 3 + q) : 0.0f;
            return 0.0f;
        };
        auto put_factor = [&](int bufi, float v) {
            if (etid < kG * 9) s_geo[bufi][etid] = v;
            else if (etid < kG * 12) s_mat[bufi][etid - kG * 9] = v;
        };
        if (blockIdx.x < n_items) put_factor(0, factor(blockIdx.x));
        int it = 0;
        for (int64_t w = blockIdx.x; w < n_items; w += gridDim.x, ++it) {
            const int abuf = it & 1;
            const int64_t b64 = w / items_per_b;
            const int64_t e0 = (w - b64 * items_per_b) * kG;
            const int nel = static_cast<int>(min(static_cast<int64_t>(kG), T.K - e0));
            if (etid == 0 && w + gridDim.x < n_items) prefetch_item(w + gridDim.x);
            // hand-off among the 128 epilogue threads through an mbarrier with a bounded wait (a
            // thread that gave up on an earlier wait cannot leave the others blocked)
            tc::mbar_arrive(&geo_full[abuf]);
            if (flag_set(&s_err) || !tc::mbar_wait(&geo_full[abuf], (it >> 1) & 1)) { err = true; break; }
            const float* sg = s_geo[abuf];
            const float* smt = s_mat[abuf];
            // the RK-register operands of one target component for the 8 elements (all in flight)
            auto load_ops = [&](int ct, float* vx, float* vz, float* vu) {
                const int64_t base = b64 * 6 * N + ct * N + e0 * Np + i;
#pragma unroll
                for (int e = 0; e < kG; ++e) {
                    vx[e] = vz[e] = vu[e] = 0.0f;
                    if (active && e < nel) {
                        const int64_t ix = base + e * Np;
                        if (kNeedX) vx[e] = A.x[ix];
                        if (kNeedZ) vz[e] = A.z[ix];
                        if (MODE == MODE_LSRK) vx[e] = A.res[ix];
                        if (kNeedU || (ct < 3 && smt[e * 3 + 2] != 0.0f)) vu[e] = __ldg(A.in + ix);
                    }
                }
            };
            float ox[2][kG], oz[2][kG], ou[2][kG];
            load_ops(0, ox[0], oz[0], ou[0]);      // in flight while the accumulator completes
            const bool more = w + gridDim.x < n_items;
            const float fnext = more ? factor(w + gridDim.x) : 0.0f;
            if (flag_set(&s_err) || !tc::mbar_wait(&acc_full[abuf], (it >> 1) & 1)) { err = true; break; }
            tc::fence_after_sync();
            const uint32_t tacc = tmem + abuf * kAccStride + (static_cast<uint32_t>(lq * 32) << 16);
            // one target component at a time: its curl from the reference derivatives of the two
            // source components ([c * kG + e] columns of the dr, ds, dt accumulators) and its lift;
            // the next target's operands are loaded before this one is computed and stored
#pragma unroll
            for (int ct = 0; ct < 6; ++ct) {
                const int cur = ct & 1;
                if (ct + 1 < 6) load_ops(ct + 1, ox[cur ^ 1], oz[cur ^ 1], ou[cur ^ 1]);
                const int ax = ct % 3;                                 // target axis
                const int a1 = (ax + 1) % 3, a2 = (ax + 2) % 3;       // curl_ax = d/d(a1) F_a2 - d/d(a2) F_a1
                const int s1 = (ct < 3 ? 3 : 0) + a2;                  // E targets: curl H; H targets: -curl E
                const int s2 = (ct < 3 ? 3 : 0) + a1;
                // the curl in two passes over the accumulators, so that at most four 8-column
                // loads are held at a time: d/d(a1) of s1 with the lift, then d/d(a2) of s2
                float ra[kG], qa[kG], ta[kG], lf[kG], cu[kG];
                tc::tmem_ld8(tacc + 0 * kNcol + s1 * kG, ra);
                tc::tmem_ld8(tacc + 1 * kNcol + s1 * kG, qa);
                tc::tmem_ld8(tacc + 2 * kNcol + s1 * kG, ta);
                tc::tmem_ld8(tacc + 3 * kNcol + ct * kG, lf);
                tc::tmem_ld_wait();
#pragma unroll
                for (int e = 0; e < kG; ++e) {
                    const float* g = sg + e * 9;           // rx ry rz sx sy sz tx ty tz
                    cu[e] = g[a1] * ra[e] + g[3 + a1] * qa[e] + g[6 + a1] * ta[e];
                }
                tc::tmem_ld8(tacc + 0 * kNcol + s2 * kG, ra);
                tc::tmem_ld8(tacc + 1 * kNcol + s2 * kG, qa);
                tc::tmem_ld8(tacc + 2 * kNcol + s2 * kG, ta);
                tc::tmem_ld_wait();
                if (ct == 5) {
                    tc::fence_before_sync();
                    tc::mbar_arrive(&acc_empty[abuf]);
                }
                if (!active) continue;
                const float sgn = ct < 3 ? 1.0f : -1.0f;
                const int64_t base = b64 * 6 * N + ct * N + e0 * Np + i;
                const float* vx = ox[cur];
                const float* vz = oz[cur];
                const float* vu = ou[cur];
#pragma unroll
                for (int e = 0; e < kG; ++e) {
                    if (e >= nel) break;
                    const float* g = sg + e * 9;
                    const float d2 = g[a2] * ra[e] + g[3 + a2] * qa[e] + g[6 + a2] * ta[e];
                    const float curl = cu[e] - d2;
                    const float uc = vu[e];
                    const float k = ct < 3 ? smt[e * 3] * (sgn * curl + lf[e]) - smt[e * 3 + 2] * uc
                                           : smt[e * 3 + 1] * (sgn * curl + lf[e]);
                    const int64_t ix = base + e * Np;
                    if (MODE == MODE_MULT) {
                        A.out[ix] = k;
                    } else if (MODE == MODE_RK4_1) {
                        A.yout[ix] = uc + 0.5f * dtf * k;
                        A.z[ix] = uc + (dtf / 6.0f) * k;
                    } else if (MODE == MODE_RK4_2) {
                        A.yout[ix] = vx[e] + 0.5f * dtf * k;
                        A.z[ix] = vz[e] + (dtf / 3.0f) * k;
                    } else if (MODE == MODE_RK4_3) {
                        A.yout[ix] = vx[e] + dtf * k;
                        A.z[ix] = vz[e] + (dtf / 3.0f) * k;
                    } else if (MODE == MODE_RK4_4) {
                        A.x[ix] = vz[e] + (dtf / 6.0f) * k;
                    } else {   // MODE_LSRK
                        const float rr = A.a * vx[e] + dtf * k;
                        A.res[ix] = rr;
                        A.yout[ix] = uc + A.b * rr;
                    }
                }
            }
            // the next item's factors into the other buffer: its last readers (item it - 1) have
            // all passed this item's hand-off above
            if (more) put_factor(abuf ^ 1, fnext);
        }
    } else if (warp == kMmaWarp) {
        // ================================================================ MMA issuer
        if (lane == 0) {
            const uint32_t idesc = tc::idesc_tf32(128, kNcol);
            const uint32_t aring_u32 = tc::smem_u32(aring);
            int it = 0;
            int64_t g = 0;                            // A slots consumed so far
            for (int64_t w = blockIdx.x; w < n_items; w += gridDim.x, ++it) {
                const int buf = it & 1, abuf = it & 1;
                const int use = it >> 1;
                if (use >= 1 && (flag_set(&s_err) || !tc::mbar_wait(&acc_empty[abuf], (use - 1) & 1))) {
                    err = true;
                    break;
                }
                tc::fence_after_sync();
                const uint32_t dacc = tmem + abuf * kAccStride;
                const uint32_t bh0 = tc::smem_u32(bbuf0 + buf * O::BBuf);
                const uint32_t bl0 = bh0 + O::BPart;
                for (int t = 0; t < NA && !err; ++t) {
                    if (t == 0 && (flag_set(&s_err) || !tc::mbar_wait(&bvol_full[buf], use & 1))) { err = true; break; }
                    if (t == 3 * NKV && (flag_set(&s_err) || !tc::mbar_wait(&bflux_full[buf], use & 1))) {
                        err = true;
                        break;
                    }
                    const int slot = static_cast<int>(g % kNSlot);
                    if (flag_set(&s_err) || !tc::mbar_wait(&a_full[slot], static_cast<uint32_t>((g / kNSlot) & 1))) {
                        err = true;
                        break;
                    }
                    tc::fence_after_sync();
                    int ks, quantity;
                    if (t < 3 * NKV) { ks = t / 3; quantity = t - 3 * ks; }
                    else { ks = NKV + (t - 3 * NKV); quantity = 3; }
                    const int kq = quantity < 3 ? ks : ks - NKV;   // K-step within the quantity
                    const uint32_t d = dacc + quantity * kNcol;
                    const uint32_t ah = aring_u32 + slot * kASlot, al = ah + kATile;
                    const uint64_t bdh = tc::smem_desc(bh0 + ks * kBStep), bdl = tc::smem_desc(bl0 + ks * kBStep);
                    tc::mma_tf32(d, tc::smem_desc(ah), bdh, idesc, kq > 0);
                    tc::mma_tf32(d, tc::smem_desc(al), bdh, idesc, true);
                    tc::mma_tf32(d, tc::smem_desc(ah), bdl, idesc, true);
                    tc::mma_commit(&a_empty[slot]);
                    ++g;
                }
                if (err) break;
                tc::mma_commit(&b_empty[buf]);
                tc::mma_commit(&acc_full[abuf]);
            }
            if (err) {
                tc::mma_commit(&drain_bar);
                tc::mbar_wait(&drain_bar, 0);
            }
        }
    } else if (warp == kCopyWarp) {
        // ================================================================ copy issuer (A slots)
        if (lane == 0) {
            const unsigned char* a_mine = reinterpret_cast<const unsigned char*>(a_img) +
                                          static_cast<size_t>(blockIdx.x % kReplicas) * NA * kASlot;
            int64_t g = 0;
            int64_t n_mine = 0;
            for (int64_t w = blockIdx.x; w < n_items; w += gridDim.x) ++n_mine;
            const int64_t total = n_mine * NA;
            for (; g < total; ++g) {
                const int slot = static_cast<int>(g % kNSlot);
                if (g >= kNSlot && (flag_set(&s_err) ||
                                    !tc::mbar_wait(&a_empty[slot], static_cast<uint32_t>(((g / kNSlot) - 1) & 1)))) {
                    err = true;
                    break;
                }
                const int t = static_cast<int>(g % NA);
                mbar_expect_tx(&a_full[slot], kASlot);
                bulk_g2s(aring + slot * kASlot, a_mine + static_cast<size_t>(t) * kASlot, kASlot, &a_full[slot]);
            }
            if (err && g > 0) {
                // wait (bounded) for this CTA's last copy in flight
                const int64_t last = g - 1;
                tc::mbar_wait(&a_full[last % kNSlot], static_cast<uint32_t>((last / kNSlot) & 1));
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
    u += 0x1000u;
    u &= ~0x1FFFu;
    return u;
}

float bits_to_float(uint32_t u)
{
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

inline bool first_use_on_device(std::atomic<uint64_t>& seen)
{
    int dev = 0;
    cudaGetDevice(&dev);
    const uint64_t bit = uint64_t(1) << (dev & 63);
    return (seen.fetch_or(bit) & bit) == 0;
}

template <int P, int MODE>
void launch_instance(const TablesF32& T, const StageArgsF32& A, const uint32_t* a_img, int* status, int n_sm,
                     cudaStream_t s)
{
    static std::atomic<uint64_t> seen{0};
    if (first_use_on_device(seen)) {
        cudaError_t e = cudaFuncSetAttribute(stage_tc1<P, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             static_cast<int>(Stc<P>::smem));
        if (e != cudaSuccess) throw std::runtime_error(std::string("tc1 smem attribute: ") + cudaGetErrorString(e));
    }
    const int64_t items_per_b = (T.K + kG - 1) / kG;
    const int64_t n_items = items_per_b * A.batch;
    const int64_t grid = std::min<int64_t>(n_items, static_cast<int64_t>(n_sm));
    stage_tc1<P, MODE><<<static_cast<unsigned>(grid), kThreads, Stc<P>::smem, s>>>(T, A, a_img, n_items, items_per_b,
                                                                                    status);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) throw std::runtime_error(std::string("tc1 stage kernel: ") + cudaGetErrorString(e));
}

template <int P>
void launch_order(const TablesF32& T, const StageArgsF32& A, const uint32_t* a_img, int* status, int n_sm,
                  cudaStream_t s)
{
    switch (A.mode) {
    case MODE_MULT: launch_instance<P, MODE_MULT>(T, A, a_img, status, n_sm, s); break;
    case MODE_RK4_1: launch_instance<P, MODE_RK4_1>(T, A, a_img, status, n_sm, s); break;
    case MODE_RK4_2: launch_instance<P, MODE_RK4_2>(T, A, a_img, status, n_sm, s); break;
    case MODE_RK4_3: launch_instance<P, MODE_RK4_3>(T, A, a_img, status, n_sm, s); break;
    case MODE_RK4_4: launch_instance<P, MODE_RK4_4>(T, A, a_img, status, n_sm, s); break;
    case MODE_LSRK: launch_instance<P, MODE_LSRK>(T, A, a_img, status, n_sm, s); break;
    default: throw std::runtime_error("single-instance tensor-core stage: unknown stage mode");
    }
}

}  // namespace

bool tc1_supported(int p) { return p >= 1 && p <= 6; }

// Host image of the A operand in the order the kernel consumes it: for every volume K-step q,
// Dr, Ds, Dt (each one slot: the tf32 hi tile, then the lo tile, 128 rows x 8 columns K-major);
// then every K-step of LIFT. Row i = node (zero for i >= Np), column k = source node or face node.
// The image is repeated kReplicas times.
std::vector<uint32_t> tc1_operator_image(const RefTet& ref)
{
    const int Np = ref.Np, NF = 4 * ref.Nfp;
    const int NKV = (Np + 7) / 8, NKF = (NF + 7) / 8;
    const int NA = 3 * NKV + NKF;
    const size_t slot_words = kASlot / 4, tile_words = kATile / 4;
    std::vector<uint32_t> img(static_cast<size_t>(NA) * slot_words, 0u);
    auto put = [&](int t, const std::vector<double>& M, int cols, int q) {
        for (int i = 0; i < Np; ++i)
            for (int k = 0; k < 8; ++k) {
                const int col = q * 8 + k;
                if (col >= cols) continue;
                const double v = M[static_cast<size_t>(i) * cols + col];
                const uint32_t hb = tf32_bits_rna(static_cast<float>(v));
                const uint32_t lb = tf32_bits_rna(static_cast<float>(v - static_cast<double>(bits_to_float(hb))));
                const size_t off = static_cast<size_t>(t) * slot_words + tc::tile_offset(i, k) / 4;
                img[off] = hb;
                img[off + tile_words] = lb;
            }
    };
    int t = 0;
    for (int q = 0; q < NKV; ++q) {
        put(t++, ref.Dr, Np, q);
        put(t++, ref.Ds, Np, q);
        put(t++, ref.Dt, Np, q);
    }
    for (int q = 0; q < NKF; ++q) put(t++, ref.LIFT, NF, q);
    std::vector<uint32_t> all(img.size() * kReplicas);
    for (int r = 0; r < kReplicas; ++r) std::copy(img.begin(), img.end(), all.begin() + r * img.size());
    return all;
}

void launch_stage_tc1(const TablesF32& T, const StageArgsF32& A, const uint32_t* a_img, int* status, int n_sm,
                      cudaStream_t s)
{
    if (reinterpret_cast<uintptr_t>(a_img) % 16 != 0)
        throw std::runtime_error("single-instance tensor-core stage: operator image must be 16-byte aligned");
    switch (T.p) {
    case 1: launch_order<1>(T, A, a_img, status, n_sm, s); break;
    case 2: launch_order<2>(T, A, a_img, status, n_sm, s); break;
    case 3: launch_order<3>(T, A, a_img, status, n_sm, s); break;
    case 4: launch_order<4>(T, A, a_img, status, n_sm, s); break;
    case 5: launch_order<5>(T, A, a_img, status, n_sm, s); break;
    case 6: launch_order<6>(T, A, a_img, status, n_sm, s); break;
    default: throw std::runtime_error("single-instance tensor-core stage supports orders 1..6");
    }
}

}  // namespace dgtd
