// Device body of the plain FP64 stage: one block of 256 threads evaluates the
// fused DG Maxwell right-hand side and RK stage update of EPB consecutive
// elements of one incidence. Shared by the single-operator kernels
// (plain_fp64.cu) and the multi-request serving kernels (serve.cu), so both
// run the same arithmetic in the same order and give bit-identical results.
//
// Computes, per element (reference HesthavenEvolution::Mult,
// src/evolution/HesthavenEvolution.cpp:450-541, with the material scaling and
// boundary coefficients of the assembled operator, src/components/DGOperatorFactory.h:21-45,
// 413-424, 1061-1208):
//   dE/dt = (1/eps) [ curl H + LIFT (Fscale/2 * fluxE) ] - (sigma/eps) E
//   dH/dt = (1/mu)  [-curl E + LIFT (Fscale/2 * fluxH) ]
//   fluxE = n x dH + aE (dE - n (n.dE)),  fluxH = -n x dE + aH (dH - n (n.dH)),
// with d = u(neighbour) - u(own) and the boundary / TF-SF rules applied to d.
// The epilogue fuses the classical RK4 register updates of mfem::RK4Solver
// (called from src/solver/Solver.cpp:544) or a low-storage RK stage.
//
// Layout in HBM (reference src/evolution/Fields.h:48-65): state[b][c][e*Np+i],
// c = Ex,Ey,Ez,Hx,Hy,Hz; elements contiguous inside each component, so a block
// of consecutive elements reads six contiguous runs.
//
// The GB300 FP64 pipe is ~1.25 TFLOP/s, so this form is FP64-issue bound
// (arithmetic intensity ~6 flop/B >> ridge): the kernel is organised to keep
// the FP64 pipe fed (shared-memory broadcast of the element's fields,
// coalesced transposed operator rows from L1/L2) rather than to save bytes.
#pragma once
#include <type_traits>
#include <cmath>

#include "kernels.hpp"
#include "tc_common.cuh"

namespace dgtd {
namespace fp64 {

constexpr int kBlock = 256;

template <int P, typename R = double>
struct Ord {
    static constexpr int Np = (P + 1) * (P + 2) * (P + 3) / 6;
    static constexpr int Nfp = (P + 1) * (P + 2) / 2;
    static constexpr int NF = 4 * Nfp;
    // elements per block: fill 256 threads (one node each), capped so static shared memory
    // stays below 48 KB
    static constexpr int EPB0 = kBlock / Np > 0 ? kBlock / Np : 1;
    static constexpr int EPB = EPB0 > 32 ? 32 : EPB0;
    // small-block variant for meshes too small to fill the SMs with kBlock-thread blocks:
    // about 64 threads (one or two warps) per block
    static constexpr int EPB_SMALL = 64 / Np > 0 ? (64 / Np > 16 ? 16 : 64 / Np) : 1;
    static constexpr int BLOCK_SMALL = (EPB_SMALL * Np + 31) / 32 * 32;
};

// The body is written for an arithmetic type R: double (the FP64 form) or float
// (the single-instance FP32 form). Source parameters are stored in double and
// evaluated in R.
template <typename R>
__device__ __forceinline__ R pw_profile(const PlaneWaveDev& w, R s)
{
    R a = s - static_cast<R>(w.mean);
    const R sp = static_cast<R>(w.spread);
    R g = exp(-a * a / (R(2) * sp * sp));
    if (w.freq != 0.0) g *= cos(R(2) * static_cast<R>(M_PI) * static_cast<R>(w.freq) * a);
    return g;
}

// Sum of the plane waves of incidence b at point x and time t.
template <typename R>
__device__ __forceinline__ void eval_pw(const PlaneWaveDev* pw, int n_pw, int b, R px, R py, R pz, R t, R* e, R* h)
{
    e[0] = e[1] = e[2] = h[0] = h[1] = h[2] = R(0);
    for (int q = 0; q < n_pw; ++q) {
        const PlaneWaveDev& w = pw[q];
        if (w.batch != b) continue;
        R s = px * static_cast<R>(w.k[0]) + py * static_cast<R>(w.k[1]) + pz * static_cast<R>(w.k[2]) - t;
        R g = pw_profile<R>(w, s);
        e[0] += g * static_cast<R>(w.pol[0]); e[1] += g * static_cast<R>(w.pol[1]); e[2] += g * static_cast<R>(w.pol[2]);
        h[0] += g * static_cast<R>(w.kxp[0]); h[1] += g * static_cast<R>(w.kxp[1]); h[2] += g * static_cast<R>(w.kxp[2]);
    }
}

// Six components of one node (or face node) stored together in shared memory, so that a
// thread reads them with vector loads: 8 floats (32 B) or 6 doubles (48 B) per entry.
template <typename R>
struct Node6 {
    static constexpr int S = sizeof(R) == 4 ? 8 : 6;
};

template <typename R>
__device__ __forceinline__ void load6(const R* p, R* v)
{
    if constexpr (sizeof(R) == 4) {
        const float4 a = *reinterpret_cast<const float4*>(p);
        const float2 b = *reinterpret_cast<const float2*>(p + 4);
        v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y;
    } else {
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const double2 a = *reinterpret_cast<const double2*>(p + 2 * q);
            v[2 * q] = a.x; v[2 * q + 1] = a.y;
        }
    }
}

// Bulk (TMA-engine) copy of `bytes` (multiple of 16, both addresses 16-byte aligned) from global
// to shared memory, completing on the mbarrier's transaction count.
__device__ __forceinline__ void bulk_to_shared(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     tc::smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(tc::smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void expect_bytes(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(tc::smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// Shared-memory copies of the operator matrices and of a block's face tables (the staged
// variant of the FP64 stage): Dr, Ds, Dt and LIFT (transposed), and per element its face-partner
// indices, face codes and face geometry. Every piece is a multiple of 16 bytes for P <= 3.
template <int P, int EPB>
struct StagedOps {
    static constexpr int Np = (P + 1) * (P + 2) * (P + 3) / 6;
    static constexpr int NF = 4 * (P + 1) * (P + 2) / 2;
    double D[3 * Np * Np];
    double L[NF * Np];
    double fgeo[EPB * 16];
    int32_t vmapP[EPB * NF];
    int32_t fcode[EPB * 4];
    uint64_t bar;
};

// EPB_: elements per block (0: Ord's default); the block has at least EPB_ * Np threads.
// STAGE (FP64, P <= 3): the operator matrices and the block's face tables are brought into
// shared memory by bulk copies issued by one thread on one mbarrier (bounded wait; on expiry the
// block reads them from global memory instead), and a face node whose partner lies in the same
// block reads the partner's values from the block's staged fields instead of global memory.
// The arithmetic and its order are unchanged, so results are bit-identical to STAGE = false.
template <int P, typename R = double, int EPB_ = 0, bool STAGE = false>
__device__ __forceinline__ void stage_body(const TablesT<R>& T, const StageArgsT<R>& A, int64_t e0, int b)
{
    using O = Ord<P, R>;
    constexpr int Np = O::Np, Nfp = O::Nfp, NF = O::NF, EPB = EPB_ > 0 ? EPB_ : O::EPB;
    constexpr int S = Node6<R>::S;
    static_assert(!STAGE || (P <= 3 && sizeof(R) == 8), "staged operators: FP64, orders 1-3");
    __shared__ __align__(16) R s_u[EPB * Np * S];     // [node][component]
    __shared__ __align__(16) R s_f[EPB * NF * S];     // [face node][component]
    __shared__ int s_fmask[4 * Nfp];
    __shared__ __align__(16) StagedOps<STAGE ? P : 1, STAGE ? EPB : 1> s_ops;

    const int tid = threadIdx.x;
    const int64_t N = T.N;
    const R* __restrict__ in = A.in + static_cast<int64_t>(b) * 6 * N;
    const int nel = (T.K - e0) < EPB ? static_cast<int>(T.K - e0) : EPB;

    if (STAGE && tid == 0) {
        tc::mbar_init(&s_ops.bar, 1);
        tc::mbar_fence_init();
        const uint32_t dbytes = Np * Np * 8, lbytes = NF * Np * 8;
        const uint32_t vbytes = nel * NF * 4, cbytes = nel * 16, gbytes = nel * 128;
        expect_bytes(&s_ops.bar, 3 * dbytes + lbytes + vbytes + cbytes + gbytes);
        bulk_to_shared(s_ops.D, T.DrT, dbytes, &s_ops.bar);
        bulk_to_shared(s_ops.D + Np * Np, T.DsT, dbytes, &s_ops.bar);
        bulk_to_shared(s_ops.D + 2 * Np * Np, T.DtT, dbytes, &s_ops.bar);
        bulk_to_shared(s_ops.L, T.LIFTT, lbytes, &s_ops.bar);
        bulk_to_shared(s_ops.vmapP, T.vmapP + e0 * NF, vbytes, &s_ops.bar);
        bulk_to_shared(s_ops.fcode, T.fcode + e0 * 4, cbytes, &s_ops.bar);
        bulk_to_shared(s_ops.fgeo, T.fgeo + e0 * 16, gbytes, &s_ops.bar);
    }
    for (int i = tid; i < 4 * Nfp; i += blockDim.x) s_fmask[i] = T.Fmask[i];
    // coalesced load of the block's fields
    for (int c = 0; c < 6; ++c)
        for (int i = tid; i < nel * Np; i += blockDim.x) s_u[i * S + c] = in[c * N + e0 * Np + i];
    __syncthreads();
    const bool staged = STAGE && tc::mbar_wait(&s_ops.bar, 0);
    if (STAGE && !staged) tc::mbar_wait(&s_ops.bar, 0);   // copies still in flight: a second bounded
                                                          // wait before the tables are read from global

    // ---- face fluxes -----------------------------------------------------------
    const bool skip_src = (A.skip != nullptr) && A.skip[b];
    for (int w = tid; w < nel * NF; w += blockDim.x) {
        const int el = w / NF, fn = w - el * NF, f = fn / Nfp, a = fn - f * Nfp;
        const int64_t e = e0 + el;
        const int vm = s_fmask[f * Nfp + a];
        // face tables: the block's staged copies (indexed by the element's position in the block)
        // or global memory
        const int code = staged ? s_ops.fcode[el * 4 + f] : T.fcode[e * 4 + f];
        const R* fg = staged ? reinterpret_cast<const R*>(s_ops.fgeo) + el * 16 + f * 4 : T.fgeo + e * 16 + f * 4;
        const R nx = fg[0], ny = fg[1], nz = fg[2], fs = fg[3];
        R uM[6], dE[3], dH[3];
        load6(s_u + (el * Np + vm) * S, uM);
        R aE = T.alpha, aH = T.alpha;
        if (code == 0 || code == 4 || code == 5) {
            const int64_t gp = staged ? s_ops.vmapP[(el * 4 + f) * Nfp + a] : T.vmapP[(e * 4 + f) * Nfp + a];
            const int64_t lp = gp - e0 * Np;           // partner node within the block's elements
            if (STAGE && lp >= 0 && lp < nel * Np) {
                R uP[6];
                load6(s_u + lp * S, uP);
#pragma unroll
                for (int c = 0; c < 3; ++c) { dE[c] = uP[c] - uM[c]; dH[c] = uP[c + 3] - uM[c + 3]; }
            } else {
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    dE[c] = __ldg(in + c * N + gp) - uM[c];
                    dH[c] = __ldg(in + (c + 3) * N + gp) - uM[c + 3];
                }
            }
            if (code != 0 && !skip_src) {
                const int64_t gm = e * Np + vm;
                R pe[3], ph[3];
                eval_pw<R>(A.pw, A.n_pw, b, T.xyz[gm], T.xyz[N + gm], T.xyz[2 * N + gm], static_cast<R>(A.t), pe, ph);
                const R sg = (code == 4) ? R(1) : R(-1);
#pragma unroll
                for (int c = 0; c < 3; ++c) { dE[c] += sg * pe[c]; dH[c] += sg * ph[c]; }
            }
        } else if (code == 1 || code == 6) {           // PEC
#pragma unroll
            for (int c = 0; c < 3; ++c) { dE[c] = R(-2) * uM[c]; dH[c] = R(0); }
        } else if (code == 2 || code == 7) {           // PMC
#pragma unroll
            for (int c = 0; c < 3; ++c) { dE[c] = R(0); dH[c] = R(-2) * uM[c + 3]; }
        } else if (code == 3 || code == 8) {           // SMA: penalty 1 regardless of alpha
#pragma unroll
            for (int c = 0; c < 3; ++c) { dE[c] = -uM[c]; dH[c] = -uM[c + 3]; }
            aE = R(1); aH = R(1);
        } else {                                        // open: zero jump
#pragma unroll
            for (int c = 0; c < 3; ++c) { dE[c] = R(0); dH[c] = R(0); }
        }
        const R ndE = nx * dE[0] + ny * dE[1] + nz * dE[2];
        const R ndH = nx * dH[0] + ny * dH[1] + nz * dH[2];
        const R h = R(0.5) * fs;
        R* so = s_f + (el * NF + fn) * S;
        so[0] = h * ((ny * dH[2] - nz * dH[1]) + aE * (dE[0] - ndE * nx));
        so[1] = h * ((nz * dH[0] - nx * dH[2]) + aE * (dE[1] - ndE * ny));
        so[2] = h * ((nx * dH[1] - ny * dH[0]) + aE * (dE[2] - ndE * nz));
        so[3] = h * (-(ny * dE[2] - nz * dE[1]) + aH * (dH[0] - ndH * nx));
        so[4] = h * (-(nz * dE[0] - nx * dE[2]) + aH * (dH[1] - ndH * ny));
        so[5] = h * (-(nx * dE[1] - ny * dE[0]) + aH * (dH[2] - ndH * nz));
    }
    __syncthreads();

    // ---- volume terms + LIFT + epilogue ----------------------------------------
    if (tid >= nel * Np) return;
    const int el = tid / Np, i = tid - el * Np;
    const int64_t e = e0 + el;
    if constexpr (std::is_same<R, double>::value)      // curved elements exist on the FP64 form only
        if (T.curved != nullptr && T.curved[e]) return;   // rows from the curved-element kernel
    R ar[6], as[6], at[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) { ar[c] = R(0); as[c] = R(0); at[c] = R(0); }
    // operator entries: staged copies in shared memory, else the read-only cache
    auto op_ld = [&](const R* p) -> R {
        if (STAGE) return *p;
        return __ldg(p);
    };
    const R* __restrict__ DrT = staged ? reinterpret_cast<const R*>(s_ops.D) : T.DrT;
    const R* __restrict__ DsT = staged ? reinterpret_cast<const R*>(s_ops.D) + Np * Np : T.DsT;
    const R* __restrict__ DtT = staged ? reinterpret_cast<const R*>(s_ops.D) + 2 * Np * Np : T.DtT;
#pragma unroll 4
    for (int j = 0; j < Np; ++j) {
        const R dr = op_ld(DrT + j * Np + i), ds = op_ld(DsT + j * Np + i), dt = op_ld(DtT + j * Np + i);
        R uj[6];
        load6(s_u + (el * Np + j) * S, uj);
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            ar[c] = fma(dr, uj[c], ar[c]);
            as[c] = fma(ds, uj[c], as[c]);
            at[c] = fma(dt, uj[c], at[c]);
        }
    }
    R lf[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) lf[c] = R(0);
    const R* __restrict__ LT = staged ? reinterpret_cast<const R*>(s_ops.L) : T.LIFTT;
#pragma unroll 4
    for (int m = 0; m < NF; ++m) {
        const R L = op_ld(LT + m * Np + i);
        R fm[6];
        load6(s_f + (el * NF + m) * S, fm);
#pragma unroll
        for (int c = 0; c < 6; ++c) lf[c] = fma(L, fm[c], lf[c]);
    }
    const R* g = T.geo + e * 9;
    const R rx = g[0], ry = g[1], rz = g[2], sx = g[3], sy = g[4], sz = g[5], tx = g[6], ty = g[7], tz = g[8];
    auto dx = [&](int c) { return rx * ar[c] + sx * as[c] + tx * at[c]; };
    auto dy = [&](int c) { return ry * ar[c] + sy * as[c] + ty * at[c]; };
    auto dz = [&](int c) { return rz * ar[c] + sz * as[c] + tz * at[c]; };
    const R curlHx = dy(5) - dz(4), curlHy = dz(3) - dx(5), curlHz = dx(4) - dy(3);
    const R curlEx = dy(2) - dz(1), curlEy = dz(0) - dx(2), curlEz = dx(1) - dy(0);
    const R* mt = T.mat + e * 3;
    const R ie = mt[0], im = mt[1], se = mt[2];
    R uo[6];
    load6(s_u + tid * S, uo);
    R k[6];
    k[0] = ie * (curlHx + lf[0]) - se * uo[0];
    k[1] = ie * (curlHy + lf[1]) - se * uo[1];
    k[2] = ie * (curlHz + lf[2]) - se * uo[2];
    k[3] = im * (-curlEx + lf[3]);
    k[4] = im * (-curlEy + lf[4]);
    k[5] = im * (-curlEz + lf[5]);

    const int64_t base = static_cast<int64_t>(b) * 6 * N + e * Np + i;
    const R dt = A.dt;
    switch (A.mode) {
    case MODE_MULT:
#pragma unroll
        for (int c = 0; c < 6; ++c) A.out[base + c * N] = k[c];
        break;
    case MODE_RK4_1:
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            const R xv = uo[c];
            A.yout[base + c * N] = xv + R(0.5) * dt * k[c];
            A.z[base + c * N] = xv + (dt / R(6)) * k[c];
        }
        break;
    case MODE_RK4_2:
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            const R xv = A.x[base + c * N];
            A.yout[base + c * N] = xv + R(0.5) * dt * k[c];
            A.z[base + c * N] += (dt / R(3)) * k[c];
        }
        break;
    case MODE_RK4_3:
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            const R xv = A.x[base + c * N];
            A.yout[base + c * N] = xv + dt * k[c];
            A.z[base + c * N] += (dt / R(3)) * k[c];
        }
        break;
    case MODE_RK4_4:
#pragma unroll
        for (int c = 0; c < 6; ++c) A.x[base + c * N] = A.z[base + c * N] + (dt / R(6)) * k[c];
        break;
    case MODE_LSRK:
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            const R r = A.a * A.res[base + c * N] + dt * k[c];
            A.res[base + c * N] = r;
            A.yout[base + c * N] = uo[c] + A.b * r;
        }
        break;
    default:
        break;
    }
}

template <typename R = double>
__device__ __forceinline__ void tfsf_skip_body(const TablesT<R>& T, const PlaneWaveDev* pw, int n_pw, int b, double t,
                                              int* skip)
{
    const int64_t total = T.n_tfsf_elems * T.Np;
    double acc = 0.0;
    for (int64_t w = threadIdx.x; w < total; w += blockDim.x) {
        const int64_t e = T.tfsf_elems[w / T.Np];
        const int64_t gm = e * T.Np + (w % T.Np);
        R pe[3], ph[3];
        eval_pw<R>(pw, n_pw, b, T.xyz[gm], T.xyz[T.N + gm], T.xyz[2 * T.N + gm], static_cast<R>(t), pe, ph);
        for (int c = 0; c < 3; ++c) {
            const double a = 0.5 * static_cast<double>(pe[c]), h = 0.5 * static_cast<double>(ph[c]);
            acc += a * a + h * h;
        }
    }
    __shared__ double red[256];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) *skip = (red[0] < 1e-16) ? 1 : 0;
}

// The same sum split over gridDim.y blocks per incidence: block `part` adds its contiguous
// share of the TF/SF nodes, and the last block of the incidence to finish (ticket) adds the
// partial sums in part order, so the decision does not depend on block scheduling.
template <typename R = double>
__device__ __forceinline__ void tfsf_skip_part_body(const TablesT<R>& T, const PlaneWaveDev* pw, int n_pw, int b,
                                                   double t, double* partial, unsigned int* ticket, int* skip)
{
    const int part = blockIdx.y, nparts = gridDim.y;
    const int64_t total = T.n_tfsf_elems * T.Np;
    // node indices fit in 32 bits (vmapP is int32), so the index arithmetic is 32-bit
    const int lo = static_cast<int>(total * part / nparts), hi = static_cast<int>(total * (part + 1) / nparts);
    const int Np = T.Np;
    double acc = 0.0;
    for (int w = lo + static_cast<int>(threadIdx.x); w < hi; w += blockDim.x) {
        const int el = w / Np;
        const int64_t gm = static_cast<int64_t>(T.tfsf_elems[el]) * Np + (w - el * Np);
        R pe[3], ph[3];
        eval_pw<R>(pw, n_pw, b, T.xyz[gm], T.xyz[T.N + gm], T.xyz[2 * T.N + gm], static_cast<R>(t), pe, ph);
        for (int c = 0; c < 3; ++c) {
            const double a = 0.5 * static_cast<double>(pe[c]), h = 0.5 * static_cast<double>(ph[c]);
            acc += a * a + h * h;
        }
    }
    __shared__ double red[256];
    __shared__ bool last;
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        partial[static_cast<int64_t>(b) * nparts + part] = red[0];
        __threadfence();
        last = atomicAdd(&ticket[b], 1u) == static_cast<unsigned int>(nparts - 1);
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        __threadfence();
        const volatile double* pv = partial + static_cast<int64_t>(b) * nparts;
        double sum = 0.0;
        for (int q = 0; q < nparts; ++q) sum += pv[q];
        skip[b] = (sum < 1e-16) ? 1 : 0;
        ticket[b] = 0u;
    }
}

}  // namespace fp64
}  // namespace dgtd
