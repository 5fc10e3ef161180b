// Plan of the batched 3-D real<->complex FFT used by PME.
#pragma once

#include <cuda_runtime.h>

#include <vector>

namespace nxm {

constexpr int kMaxPasses = 12;

// Per-system FFT geometry.  The real grid is row-major K0 x K1 x K2 (z
// fastest, NonbondedForce.cpp:253); the half spectrum is K0 x K1 x Kh with
// Kh = K2/2 + 1.
struct FftSysDev {
    int K[3];
    int Kh;
    long long roff;     // real grid offset (elements)
    long long coff;     // half-spectrum offset (elements)
    int tw[3];          // twiddle-table offset for the length of each axis
    int np[3];          // Stockham passes per axis
    int rad[3][kMaxPasses];
    double wscale;      // unused padding for alignment
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
    int nz = 0, ny = 0, nx = 0;
    int zlines = 16;    // real lines per block in the z passes (even)
    int cols = 8;       // z columns per block in the y and x passes
    size_t smem_z = 0, smem_y = 0, smem_x = 0;
    int kmax = 0;
};

void fft_plan_build(FftPlan &plan, int mixed);
void fft_plan_free(FftPlan &plan);

}  // namespace nxm
