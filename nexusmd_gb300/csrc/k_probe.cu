// FP32 FMA throughput probe: the FP32-pipe peak that the pair kernel's
// roofline is measured against.  Every thread runs 8 independent chains of
// fused multiply-adds on float pairs, either as two scalar FFMAs or as one
// packed FP32x2 FFMA per pair (__ffma2_rn); the launch covers every SM many
// times over, and the rate is timed with CUDA events on the caller's stream.
#include <cuda_runtime.h>

#include <algorithm>

#include "nxm.h"

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

}  // namespace nxm

extern "C" int nxm_fp32_peak(int32_t device, double *tflops_scalar, double *tflops_packed) {
    using namespace nxm;
    if (!tflops_scalar || !tflops_packed) return NXM_ERR_INVALID;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return NXM_ERR_CUDA;
    cudaSetDevice(device);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int threads = 256, blocks = std::max(1, sms) * 8, iters = 4096;
    float *out = nullptr;
    if (cudaMalloc(&out, sizeof(float) * (size_t)blocks * threads) != cudaSuccess) return NXM_ERR_CUDA;
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
    if (err != cudaSuccess) return NXM_ERR_CUDA;
    *tflops_scalar = best[0];
    *tflops_packed = best[1];
    return NXM_OK;
}
