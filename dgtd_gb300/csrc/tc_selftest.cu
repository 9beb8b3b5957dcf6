// Self-check of the tcgen05 tf32 path: one CTA computes D[128 x 48] = A[128 x K] B[48 x K]^T
// with the 3xTF32 split (A_hi B_hi + A_lo B_hi + A_hi B_lo) through shared-memory
// descriptors, tensor-memory accumulation and tcgen05.ld, exactly as the batched
// stage kernel does. Exposed through the C ABI (dgtd_tc_selftest) so that tests can
// validate the tensor-core building blocks on the device before the solver uses them.
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "../../include/dgtd_gb300.h"
#include "tc_common.cuh"

namespace dgtd {
namespace {

constexpr int kM = 128, kN = 48;

__global__ void __launch_bounds__(128) tc_selftest_kernel(const float* __restrict__ A, const float* __restrict__ B,
                                                          float* __restrict__ D, int K, int* status)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    const int nks = K / 8;
    // layout: [A_hi | A_lo] tiles of 128x8 (4 KB each) per K-step, then [B_hi | B_lo] 48x8 (1.5 KB each)
    unsigned char* a_hi = smem;
    unsigned char* a_lo = a_hi + nks * 4096;
    unsigned char* b_hi = a_lo + nks * 4096;
    unsigned char* b_lo = b_hi + nks * 1536;
    __shared__ uint64_t bar;
    __shared__ uint32_t tbase;
    const int tid = threadIdx.x, warp = tid >> 5;

    for (int idx = tid; idx < kM * K; idx += blockDim.x) {
        const int r = idx / K, k = idx - r * K;
        const float v = A[idx];
        const float hi = tc::to_tf32(v), lo = tc::to_tf32(v - hi);
        const uint32_t off = (k / 8) * 4096 + tc::tile_offset(r, k);
        *reinterpret_cast<float*>(a_hi + off) = hi;
        *reinterpret_cast<float*>(a_lo + off) = lo;
    }
    for (int idx = tid; idx < kN * K; idx += blockDim.x) {
        const int r = idx / K, k = idx - r * K;
        const float v = B[idx];
        const float hi = tc::to_tf32(v), lo = tc::to_tf32(v - hi);
        const uint32_t off = (k / 8) * 1536 + tc::tile_offset(r, k);
        *reinterpret_cast<float*>(b_hi + off) = hi;
        *reinterpret_cast<float*>(b_lo + off) = lo;
    }
    tc::fence_proxy_async();
    if (tid == 0) { tc::mbar_init(&bar, 1); tc::mbar_fence_init(); }
    if (warp == 0) {
        tc::tmem_alloc(&tbase, 64);
        tc::tmem_relinquish();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t taddr = tbase;

    if (tid == 0) {
        const uint32_t idesc = tc::idesc_tf32(kM, kN);
        for (int q = 0; q < nks; ++q) {
            const uint64_t ah = tc::smem_desc(tc::smem_u32(a_hi + q * 4096));
            const uint64_t al = tc::smem_desc(tc::smem_u32(a_lo + q * 4096));
            const uint64_t bh = tc::smem_desc(tc::smem_u32(b_hi + q * 1536));
            const uint64_t bl = tc::smem_desc(tc::smem_u32(b_lo + q * 1536));
            tc::mma_tf32(taddr, ah, bh, idesc, q > 0);
            tc::mma_tf32(taddr, al, bh, idesc, true);
            tc::mma_tf32(taddr, ah, bl, idesc, true);
        }
        tc::mma_commit(&bar);
    }
    const bool ok = __syncthreads_and(tc::mbar_wait(&bar, 0)) != 0;
    if (!ok && tid == 0) atomicExch(status, 2);
    tc::fence_after_sync();
    if (ok) {
        float v[32];
        const uint32_t lane_base = static_cast<uint32_t>(warp * 32) << 16;
        tc::tmem_ld32(taddr + lane_base, v);
        tc::tmem_ld_wait();
        const int row = warp * 32 + (tid & 31);
        for (int c = 0; c < 32; ++c) D[row * kN + c] = v[c];
        tc::tmem_ld16(taddr + lane_base + 32, v);
        tc::tmem_ld_wait();
        for (int c = 0; c < 16; ++c) D[row * kN + 32 + c] = v[c];
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(taddr, 64);
}

}  // namespace
}  // namespace dgtd

extern "C" int dgtd_tc_selftest(const float* h_a, const float* h_b, float* h_d, int32_t k, int32_t* status)
{
    using namespace dgtd;
    if (!h_a || !h_b || !h_d || !status) return DGTD_ERR_INVALID;
    if (k <= 0 || k % 8 != 0 || k > 96) return DGTD_ERR_INVALID;
    *status = 0;
    float *a = nullptr, *b = nullptr, *d = nullptr;
    int* st = nullptr;
    int rc = DGTD_OK;
    const size_t smem = static_cast<size_t>(k / 8) * (2 * 4096 + 2 * 1536);
    auto ck = [&](cudaError_t e) { if (e != cudaSuccess && rc == DGTD_OK) rc = DGTD_ERR_CUDA; return e == cudaSuccess; };
    if (ck(cudaMalloc(&a, kM * k * sizeof(float))) && ck(cudaMalloc(&b, kN * k * sizeof(float))) &&
        ck(cudaMalloc(&d, kM * kN * sizeof(float))) && ck(cudaMalloc(&st, sizeof(int))) &&
        ck(cudaMemcpy(a, h_a, kM * k * sizeof(float), cudaMemcpyHostToDevice)) &&
        ck(cudaMemcpy(b, h_b, kN * k * sizeof(float), cudaMemcpyHostToDevice)) &&
        ck(cudaMemset(d, 0, kM * kN * sizeof(float))) && ck(cudaMemset(st, 0, sizeof(int))) &&
        ck(cudaFuncSetAttribute(tc_selftest_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)))) {
        tc_selftest_kernel<<<1, 128, smem>>>(a, b, d, k, st);
        if (ck(cudaGetLastError()) && ck(cudaDeviceSynchronize())) {
            ck(cudaMemcpy(h_d, d, kM * kN * sizeof(float), cudaMemcpyDeviceToHost));
            ck(cudaMemcpy(status, st, sizeof(int), cudaMemcpyDeviceToHost));
        }
    }
    cudaFree(a); cudaFree(b); cudaFree(d); cudaFree(st);
    return rc;
}
