// Hardware probes for bench.py (libnxm_probe.so, not part of the engine
// library or its C ABI).
//
// nxm_probe_fp32_peak: FP32 FMA throughput, the FP32-pipe peak that the pair
// kernel's roofline is measured against.  Every thread runs 8 independent
// chains of fused multiply-adds on float pairs, either as two scalar FFMAs or
// as one packed FP32x2 FFMA per pair (__ffma2_rn); the launch covers every SM
// many times over, and the rate is timed with CUDA events on its own stream.
//
// nxm_probe_stencil_atomics: global int32 atomic adds per second in the PME
// spread's pattern, the L2-atomic ceiling the spread kernel runs against.
//
// nxm_probe_shared_atomics: throughput of shared-memory integer atomic adds,
// 64-bit and 32-bit, at addresses drawn at random inside a 4,096-word array
// (what a half neighbour list would need to sum the j-side forces of a
// staged tile as fixed point in shared memory).
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#define NXM_PROBE_OK 0
#define NXM_PROBE_ERR_INVALID -1
#define NXM_PROBE_ERR_CUDA -2

namespace nxm {

constexpr int kProbeChains = 8;

template <bool PACKED>
__global__ void __launch_bounds__(256) k_fma_probe(float *out, int iters, float a, float b) {
    float2 acc[kProbeChains];
#pragma unroll
    for (int k = 0; k < kProbeChains; ++k) acc[k] = make_float2((float)(threadIdx.x + k), (float)(blockIdx.x + k));
    const float2 a2 = make_float2(a, a), b2 = make_float2(b, b);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < kProbeChains; ++k) {
            if (PACKED)
                acc[k] = __ffma2_rn(acc[k], a2, b2);
            else
                acc[k] = make_float2(fmaf(acc[k].x, a, b), fmaf(acc[k].y, a, b));
        }
    }
    float s = 0.0f;
#pragma unroll
    for (int k = 0; k < kProbeChains; ++k) s += acc[k].x + acc[k].y;
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

constexpr int kAtomWords = 4096;

__device__ __forceinline__ unsigned probe_hash(unsigned x) {
    x ^= x >> 16;
    x *= 0x7feb352dU;
    x ^= x >> 15;
    x *= 0x846ca68bU;
    x ^= x >> 16;
    return x;
}

// Each thread adds `iters` times into a 4,096-word shared array at
// hash-drawn addresses (every index masked into the array); the array is
// written out so the adds are kept.
template <bool WIDE>
__global__ void __launch_bounds__(512) k_atomic_probe(unsigned long long *out, int iters) {
    __shared__ unsigned long long a64[kAtomWords];
    unsigned *a32 = reinterpret_cast<unsigned *>(a64);
    for (int i = threadIdx.x; i < kAtomWords; i += blockDim.x) a64[i] = 0;
    __syncthreads();
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned long long v = threadIdx.x + 1;
    for (int it = 0; it < iters; ++it) {
        const int a = (int)(probe_hash(lane * 7919u + warp * 104729u + (unsigned)it * 15485863u) & (kAtomWords - 1));
        if (WIDE)
            atomicAdd(&a64[a], v);
        else
            atomicAdd(&a32[a], (unsigned)v);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kAtomWords; i += blockDim.x) out[(size_t)blockIdx.x * kAtomWords + i] = a64[i];
}

// The PME spread's global access pattern at full rate: each warp adds
// int32 words (the mixed engine's grid word) to the 32 consecutive points (x-major, z fastest) of one 5^3
// stencil of a K^3 grid, at a stencil base drawn at random with every point
// inside the grid.  One launch does `reps` stencils per warp.
__global__ void __launch_bounds__(256) k_stencil_atomic_probe(unsigned *grid, int K, int reps) {
    const unsigned lane = threadIdx.x & 31;
    const unsigned gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    for (int r = 0; r < reps; ++r) {
        const unsigned h = probe_hash(gw * 2654435761u + (unsigned)r * 40503u);
        const int bx = (int)(h % (unsigned)(K - 4)), by = (int)((h >> 8) % (unsigned)(K - 4)),
                  bz = (int)((h >> 16) % (unsigned)(K - 4));
        for (int p = (int)lane; p < 125; p += 32) {
            const int ix = p / 25, iy = (p / 5) % 5, iz = p % 5;
            atomicAdd(&grid[((size_t)(bx + ix) * K + (by + iy)) * K + (bz + iz)], 1u);
        }
    }
}

}  // namespace nxm

// Global int32 atomic adds per second in the spread's pattern (5^3 stencils
// at random places of a K^3 grid, consecutive stencil points per warp).
extern "C" int nxm_probe_stencil_atomics(int32_t device, int32_t K, double *atomics_per_s) {
    using namespace nxm;
    if (!atomics_per_s || K < 8 || K > 512) return NXM_PROBE_ERR_INVALID;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return NXM_PROBE_ERR_CUDA;
    cudaSetDevice(device);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const size_t pts = (size_t)K * K * K;
    unsigned *grid = nullptr;
    if (cudaMalloc(&grid, sizeof(unsigned) * pts) != cudaSuccess) return NXM_PROBE_ERR_CUDA;
    cudaMemset(grid, 0, sizeof(unsigned) * pts);
    cudaStream_t st;
    cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int threads = 256, blocks = std::max(1, sms) * 8, reps = 64;
    const double ops = (double)blocks * (threads / 32) * reps * 125;
    double best = 0.0;
    for (int rep = 0; rep < 4; ++rep) {  // the first launch warms up
        cudaEventRecord(e0, st);
        k_stencil_atomic_probe<<<blocks, threads, 0, st>>>(grid, K, reps);
        cudaEventRecord(e1, st);
        cudaEventSynchronize(e1);
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms > 0.0f) best = std::max(best, ops / (ms * 1e-3));
    }
    cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(st);
    cudaFree(grid);
    if (err != cudaSuccess) return NXM_PROBE_ERR_CUDA;
    *atomics_per_s = best;
    return NXM_PROBE_OK;
}

extern "C" int nxm_probe_shared_atomics(int32_t device, double *u64_per_clk_sm, double *u32_per_clk_sm) {
    using namespace nxm;
    if (!u64_per_clk_sm || !u32_per_clk_sm) return NXM_PROBE_ERR_INVALID;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return NXM_PROBE_ERR_CUDA;
    cudaSetDevice(device);
    int sms = 0, khz = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, device);
    const int threads = 512, blocks = std::max(1, sms) * 2, iters = 4096;
    unsigned long long *out = nullptr;
    if (cudaMalloc(&out, sizeof(unsigned long long) * (size_t)blocks * kAtomWords) != cudaSuccess)
        return NXM_PROBE_ERR_CUDA;
    cudaStream_t st;
    cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const double ops = (double)blocks * threads * iters;
    double best[2] = {0.0, 0.0};
    for (int wide = 0; wide < 2; ++wide) {
        for (int rep = 0; rep < 4; ++rep) {  // the first launch warms up
            cudaEventRecord(e0, st);
            if (wide)
                k_atomic_probe<true><<<blocks, threads, 0, st>>>(out, iters);
            else
                k_atomic_probe<false><<<blocks, threads, 0, st>>>(out, iters);
            cudaEventRecord(e1, st);
            cudaEventSynchronize(e1);
            float ms = 0.0f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (rep > 0 && ms > 0.0f) best[wide] = std::max(best[wide], ops / (ms * 1e-3));
        }
    }
    cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(st);
    cudaFree(out);
    if (err != cudaSuccess) return NXM_PROBE_ERR_CUDA;
    // per SM per clock at the device's nominal maximum clock
    const double per = (double)std::max(1, sms) * std::max(1, khz) * 1e3;
    *u64_per_clk_sm = best[1] / per;
    *u32_per_clk_sm = best[0] / per;
    return NXM_PROBE_OK;
}

extern "C" int nxm_probe_fp32_peak(int32_t device, double *tflops_scalar, double *tflops_packed) {
    using namespace nxm;
    if (!tflops_scalar || !tflops_packed) return NXM_PROBE_ERR_INVALID;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return NXM_PROBE_ERR_CUDA;
    cudaSetDevice(device);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int threads = 256, blocks = std::max(1, sms) * 8, iters = 4096;
    float *out = nullptr;
    if (cudaMalloc(&out, sizeof(float) * (size_t)blocks * threads) != cudaSuccess) return NXM_PROBE_ERR_CUDA;
    cudaStream_t st;
    cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    // flops per launch: 2 per FMA, 2 FMAs per chain step
    const double flops = 2.0 * 2.0 * kProbeChains * (double)iters * blocks * threads;
    double best[2] = {0.0, 0.0};
    for (int packed = 0; packed < 2; ++packed) {
        for (int rep = 0; rep < 6; ++rep) {  // the first launch warms up
            cudaEventRecord(e0, st);
            if (packed)
                k_fma_probe<true><<<blocks, threads, 0, st>>>(out, iters, 0.999f, 0.001f);
            else
                k_fma_probe<false><<<blocks, threads, 0, st>>>(out, iters, 0.999f, 0.001f);
            cudaEventRecord(e1, st);
            cudaEventSynchronize(e1);
            float ms = 0.0f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (rep > 0 && ms > 0.0f) best[packed] = std::max(best[packed], flops / (ms * 1e-3) / 1e12);
        }
    }
    cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(st);
    cudaFree(out);
    if (err != cudaSuccess) return NXM_PROBE_ERR_CUDA;
    *tflops_scalar = best[0];
    *tflops_packed = best[1];
    return NXM_PROBE_OK;
}
