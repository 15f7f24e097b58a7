// mlp.cu — the radiance-cache MLP on the tensor cores (tcgen05, BF16 operands,
// FP32 accumulators in tensor memory).
//
// This file starts with the probe of one tensor-core product, which pins the
// operand layouts and descriptors of tc.cuh against a CPU product.
#include <algorithm>
#include <string>

#include "common.cuh"
#include "internal.h"
#include "tc.cuh"

namespace mcrt {

namespace {

constexpr uint32_t kProbeM = 128;
constexpr uint32_t kProbeARegion = 64 * 1024;   // operand regions sized so that any stride of the
constexpr uint32_t kProbeBRegion = 16 * 1024;   // descriptors stays inside them
constexpr uint32_t kPollLimit = 1u << 22;

// D[128 x N] = A[128 x K] * B[N x K]^T with A, B bf16 (row-major in global
// memory), staged in shared memory K-major or MN-major (flags bit 0: A, bit 1: B).
// status[0]: 0 ok, 1 the MMA did not complete within the poll limit.
__global__ void __launch_bounds__(128) k_gemm_probe(const uint16_t *A, const uint16_t *B, uint32_t K, uint32_t N,
                                                    uint32_t flags, float *D, uint32_t *status) {
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t *sa = smem;
    uint8_t *sb = smem + kProbeARegion;
    uint64_t *mbar = reinterpret_cast<uint64_t *>(smem + kProbeARegion + kProbeBRegion);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(mbar + 1);
    const bool a_mn = flags & 1u, b_mn = flags & 2u;
    const uint32_t t = threadIdx.x, warp = t >> 5;
    for (uint32_t i = t; i < kProbeARegion / 4; i += blockDim.x) reinterpret_cast<uint32_t *>(sa)[i] = 0u;
    for (uint32_t i = t; i < kProbeBRegion / 4; i += blockDim.x) reinterpret_cast<uint32_t *>(sb)[i] = 0u;
    __syncthreads();
    for (uint32_t i = t; i < kProbeM * K; i += blockDim.x) {
        uint32_t m = i / K, k = i - m * K;
        uint32_t off = a_mn ? tc::op_offset(k, m, K) : tc::op_offset(m, k, kProbeM);
        *reinterpret_cast<uint16_t *>(sa + off) = A[i];
    }
    for (uint32_t i = t; i < N * K; i += blockDim.x) {
        uint32_t n = i / K, k = i - n * K;
        uint32_t off = b_mn ? tc::op_offset(k, n, K) : tc::op_offset(n, k, N);
        *reinterpret_cast<uint16_t *>(sb + off) = B[i];
    }
    tc::fence_proxy_async();
    uint32_t ncols = 32;
    while (ncols < N) ncols <<= 1;
    if (warp == 0) tc::tmem_alloc(tslot, ncols);
    if (t == 0) tc::mbar_init(mbar, 1);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t taddr = *tslot;
    if (t == 0) {
        const uint32_t idesc = tc::idesc_bf16(kProbeM, N, a_mn, b_mn);
        const uint32_t a_lbo = a_mn ? 128u : (kProbeM / 8) * 128u, a_sbo = a_mn ? (K / 8) * 128u : 128u;
        const uint32_t b_lbo = b_mn ? 128u : (N / 8) * 128u, b_sbo = b_mn ? (K / 8) * 128u : 128u;
        for (uint32_t kk = 0; kk < K / 16; ++kk) {
            const uint32_t a_step = a_mn ? 256u : 2u * (kProbeM / 8) * 128u;
            const uint32_t b_step = b_mn ? 256u : 2u * (N / 8) * 128u;
            uint64_t ad = tc::make_desc(tc::smem_u32(sa) + kk * a_step, a_lbo, a_sbo);
            uint64_t bd = tc::make_desc(tc::smem_u32(sb) + kk * b_step, b_lbo, b_sbo);
            tc::mma_bf16(taddr, ad, bd, idesc, kk > 0 ? 1u : 0u);
        }
        tc::commit(mbar);
    }
    const bool ok = tc::mbar_wait(mbar, 0, kPollLimit);
    tc::fence_after_sync();
    if (!ok) {
        if (t == 0) status[0] = 1u;
    } else {
        const uint32_t row = warp * 32 + (t & 31u);
        for (uint32_t c = 0; c < N; c += 16) {
            float v[16];
            tc::tmem_ld16(taddr + ((warp * 32u) << 16) + c, v);
            for (int j = 0; j < 16; ++j)
                if (c + j < N) D[(size_t)row * N + c + j] = v[j];
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tc::tmem_dealloc(taddr, ncols);
        tc::tmem_relinquish();
    }
}

}  // namespace

}  // namespace mcrt

extern "C" mcrt_status mcrt_mlp_gemm_probe(int device, const uint16_t *A, const uint16_t *B, uint32_t K, uint32_t N,
                                           uint32_t flags, float *D) {
    if (!A || !B || !D) { mcrt::set_global_error("NULL argument"); return MCRT_ERR_INVALID_ARG; }
    if (K == 0 || K % 16 || K > 64 || N < 16 || N > 64 || N % 16 || flags > 3) {
        mcrt::set_global_error("probe shape: K in 16..64 (multiple of 16), N in 16..64 (multiple of 16)");
        return MCRT_ERR_INVALID_ARG;
    }
    auto cuda_err = [](cudaError_t e, const char *what) {
        mcrt::set_global_error(std::string(what) + ": " + cudaGetErrorString(e));
        return MCRT_ERR_CUDA;
    };
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return cuda_err(e, "cudaSetDevice");
    const size_t na = (size_t)mcrt::kProbeM * K, nb = (size_t)N * K, nd = (size_t)mcrt::kProbeM * N;
    uint16_t *dA = nullptr, *dB = nullptr;
    float *dD = nullptr;
    uint32_t *dS = nullptr;
    mcrt_status rc = MCRT_OK;
    const size_t smem = mcrt::kProbeARegion + mcrt::kProbeBRegion + 64;
    if ((e = cudaMalloc(&dA, na * 2)) != cudaSuccess || (e = cudaMalloc(&dB, nb * 2)) != cudaSuccess ||
        (e = cudaMalloc(&dD, nd * 4)) != cudaSuccess || (e = cudaMalloc(&dS, 4)) != cudaSuccess) {
        rc = cuda_err(e, "allocate");
    } else if ((e = cudaMemcpy(dA, A, na * 2, cudaMemcpyHostToDevice)) != cudaSuccess ||
               (e = cudaMemcpy(dB, B, nb * 2, cudaMemcpyHostToDevice)) != cudaSuccess ||
               (e = cudaMemset(dD, 0, nd * 4)) != cudaSuccess || (e = cudaMemset(dS, 0, 4)) != cudaSuccess ||
               (e = cudaFuncSetAttribute(mcrt::k_gemm_probe, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem)) != cudaSuccess) {
        rc = cuda_err(e, "upload");
    } else {
        mcrt::k_gemm_probe<<<1, 128, smem>>>(dA, dB, K, N, flags, dD, dS);
        mcrt::note_launch();
        uint32_t st = 0;
        if ((e = cudaGetLastError()) != cudaSuccess || (e = cudaDeviceSynchronize()) != cudaSuccess ||
            (e = cudaMemcpy(&st, dS, 4, cudaMemcpyDeviceToHost)) != cudaSuccess ||
            (e = cudaMemcpy(D, dD, nd * 4, cudaMemcpyDeviceToHost)) != cudaSuccess) {
            rc = cuda_err(e, "probe");
        } else if (st) {
            mcrt::set_global_error("tensor-core product did not complete");
            rc = MCRT_ERR_TIMEOUT;
        }
    }
    cudaFree(dA);
    cudaFree(dB);
    cudaFree(dD);
    cudaFree(dS);
    return rc;
}
