// calibrate.cu -- integer-pipe throughput probe used to state the roofline of the
// bootstrap kernels (their bound is 32-bit multiply-class throughput, not HBM or tensor
// cores): many warps each run independent chains of 32-bit multiply-adds.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/yatfhe_gb300.h"

namespace {

constexpr int kChains = 8;

__global__ void imad_chains(uint32_t* sink, int iters, uint32_t seed) {
    uint32_t a[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c) a[c] = seed + threadIdx.x * 7 + c;
    const uint32_t b = seed | 1u, d = seed ^ 0x9e3779b9u;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < kChains; ++c) a[c] = a[c] * b + d;
    }
    uint32_t s = 0;
#pragma unroll
    for (int c = 0; c < kChains; ++c) s ^= a[c];
    if (s == 0x12345679u) sink[blockIdx.x] = s;  // keeps the chains live
}

}  // namespace

extern "C" int yg_probe_int32_rate(int device, double* ops_per_second) {
    if (!ops_per_second) return YG_ERR_INVALID;
    int prev = 0;
    cudaGetDevice(&prev);
    if (cudaSetDevice(device) != cudaSuccess) return YG_ERR_CUDA;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int blocks = sms * 8, threads = 256, iters = 1 << 14;
    uint32_t* sink = nullptr;
    cudaEvent_t e0, e1;
    int rc = YG_OK;
    if (cudaMalloc(&sink, blocks * sizeof(uint32_t)) != cudaSuccess) return YG_ERR_CUDA;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    imad_chains<<<blocks, threads>>>(sink, iters / 8, 3u);  // warm-up
    cudaEventRecord(e0);
    imad_chains<<<blocks, threads>>>(sink, iters, 5u);
    cudaEventRecord(e1);
    if (cudaEventSynchronize(e1) != cudaSuccess) rc = YG_ERR_CUDA;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    *ops_per_second = (double)blocks * threads * iters * kChains / (ms * 1e-3);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sink);
    cudaSetDevice(prev);
    return rc;
}
