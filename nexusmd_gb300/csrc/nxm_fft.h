// Plan of the batched 3-D real<->complex FFT used by PME.
#pragma once

#include <cuda_runtime.h>

#include <vector>

namespace nxm {

constexpr int kMaxPasses = 12;

// The Stockham passes of one axis of length n, each pass's constants worked
// out on the host: radix R, sub-transform size Ns before the pass,
// butterflies per line m = n / R, twiddle stride n / (Ns R), and the FP32
// reciprocals of m and Ns that the passes divide by.
struct FftPasses {
    int np;
    int R[kMaxPasses], Ns[kMaxPasses], m[kMaxPasses], step[kMaxPasses];
    float inv_m[kMaxPasses], inv_ns[kMaxPasses];
};

// Factors n = 2^a 3^b 5^c into passes of radix 10, 9, 8, 6, 4, 2, 3, 5 (the
// larger first: fewer passes through shared memory).
void fft_passes(int n, FftPasses &P);

// Per-system FFT geometry.  The real grid is row-major K0 x K1 x K2 (z
// fastest, NonbondedForce.cpp:253); the half spectrum is K0 x K1 x Kh with
// Kh = K2/2 + 1.
struct FftSysDev {
    int K[3];
    int Kh;
    long long roff;     // real grid offset (elements)
    long long coff;     // half-spectrum offset (elements)
    int tw[3];          // twiddle-table offset for the length of each axis
    FftPasses ax[3];    // passes per axis
};

struct FftWork {
    int sys;
    int unit;
};

struct FftPlan {
    int S = 0;
    FftSysDev *dsys = nullptr;
    std::vector<FftSysDev> hsys;
    FftWork *zwork = nullptr, *ywork = nullptr, *xwork = nullptr;
    void *buf = nullptr;  // one device buffer holding dsys and the work lists
    size_t cap = 0;       // its bytes
    void *ext = nullptr;  // a buffer the caller owns, used instead where the tables fit
    size_t ext_cap = 0;
    int nz = 0, ny = 0, nx = 0;
    int zlines = 16;    // real lines per block in the z passes (even)
    int cols = 8;       // z columns per block in the y and x passes
    size_t smem_z = 0, smem_y = 0, smem_x = 0;
    int kmax = 0;
    // Plane path: one block per (system, x-plane) runs z then y forward and
    // y then z inverse in shared memory (3 FFT launches instead of 5, the
    // same arithmetic).  plane_ok when every system's plane fits.
    FftWork *pwork = nullptr;
    int npl = 0;
    int plane = 0, plane_ok = 0;
    int plane_chunked = 0;  // a plane is larger than the scratch: the plane path works in chunks of lines
    int plane_threads = 512;
    int twcap = 0, qcap = 0, scr = 0;   // shared-memory regions, complex words
    size_t smem_plane = 0;
};

// Builds the plan; its device tables are copied in the order of stream st.
void fft_plan_build(FftPlan &plan, int mixed, cudaStream_t st);
void fft_plan_free(FftPlan &plan);
// Bytes of the plan's device tables for any z and column blocking the
// autotuner tries (hsys and S set).
size_t fft_plan_bytes_max(const FftPlan &plan);
// FFT kernel launches of one convolution with this plan.
int fft_launch_count(const FftPlan &plan);
// Shared memory of a line-path block: twiddles and two buffers of `lines`
// lines of up to kmax complex words.
size_t fft_line_smem(int lines, int kmax, size_t csz);

}  // namespace nxm
