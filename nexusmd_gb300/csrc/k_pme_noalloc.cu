// Reciprocal-space PME on caller-owned device buffers that allocates nothing:
// every intermediate (fixed-point charge grid, half spectrum, real grid,
// influence function, B-spline moduli, FFT twiddles and work lists, energy
// word) lives in one file-scope device array of fixed size, g_pme_scratch.
//
// The arithmetic is the engine's mixed-precision PME step (k_pme.cu spread
// and gather, k_fft.cu transforms, the influence function of nxm_engine.cu),
// all computed on the device so that one call is a sequence of kernel
// launches on the caller's stream and nothing else: no cudaMalloc, cudaFree,
// host<->device copy or library call that allocates.  It has no counterpart
// in the reference, whose PME (core/baseline/src/Forces/NonbondedForce.cpp
// :51-461) allocates its grids per evaluation.
//
// Limits: each grid axis K in [5, 64] with K = 2^a 3^b 5^c; any atom count.
// Scratch: about 3.7 MB of device memory per device, for the lifetime of
// the library.
//
// Set-up: the first call on a device (the device current at the call) looks
// up the array's device address with cudaGetSymbolAddress, once, and keeps
// it; that lookup may load the module, so the first call on each device
// should come before any stream capture.  The kept address belongs to the
// device's primary context of that time: after cudaDeviceReset (which
// destroys it) the library must be unloaded and loaded again before the
// next call.
//
// Sharing: every call on a device uses the same array, which keeps the
// previous call's contents.  Each call clears what must start at zero (the
// charge-grid accumulator and the energy word) and rewrites everything else
// before reading it.  Calls whose work overlaps on the GPU (two streams, or
// two host threads) race on the array and give wrong results; serialise them.
#include <algorithm>
#include <cstdio>
#include <mutex>
#include <string>

#include "../../include/nxm.h"
#include "nxm_fft.h"
#include "nxm_view.h"

namespace nxm {
int fail(int code, const std::string &msg);
}

namespace {

using namespace nxm;

constexpr int kStaticMaxK = 64;
constexpr int kStaticMaxKh = kStaticMaxK / 2 + 1;
constexpr int kZLines = 16;  // real lines per block in the z passes
constexpr int kCols = 8;     // columns per block in the y and x passes
constexpr int kMaxWork = kStaticMaxK * ((kStaticMaxKh + kCols - 1) / kCols);  // >= every work list

constexpr size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

// byte offsets of the regions of g_pme_scratch
constexpr size_t kOffE = 0;                                                   // long long[E_SLOTS]
constexpr size_t kOffSys = kOffE + align256(sizeof(long long) * E_SLOTS);     // FftSysDev
constexpr size_t kOffWork = kOffSys + align256(sizeof(FftSysDev));            // 3 x FftWork[kMaxWork]
constexpr size_t kOffTw = kOffWork + align256(3 * sizeof(FftWork) * kMaxWork);  // float2[3][K]
constexpr size_t kOffMod = kOffTw + align256(sizeof(float2) * 3 * kStaticMaxK);  // double[3][K]
constexpr size_t kOffAcc = kOffMod + align256(sizeof(double) * 3 * kStaticMaxK);
constexpr size_t kGridPts = (size_t)kStaticMaxK * kStaticMaxK * kStaticMaxK;
constexpr size_t kSpecPts = (size_t)kStaticMaxK * kStaticMaxK * kStaticMaxKh;
constexpr size_t kOffReal = kOffAcc + align256(sizeof(int) * kGridPts);
constexpr size_t kOffCplx = kOffReal + align256(sizeof(float) * kGridPts);
constexpr size_t kOffEterm = kOffCplx + align256(sizeof(float2) * kSpecPts);
constexpr size_t kScratchBytes = kOffEterm + align256(sizeof(float) * kSpecPts);

__device__ __align__(256) unsigned char g_pme_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
unsigned char *g_scratch_ptr[kMaxDevices] = {};

struct Geometry {
    int K[3];
    int Kh;
    double L[3], invL[3];
    double alpha;
};

template <typename T>
__device__ __forceinline__ T *region(unsigned char *base, size_t off) {
    return reinterpret_cast<T *>(base + off);
}

// B-spline weights and derivatives of order 5 at fraction dr, in the
// operation order of computeBSplineParameters (NonbondedForce.cpp:144-182).
__device__ __forceinline__ void spline5(float dr, float *th, float *dth) {
    th[4] = 0.f;
    th[1] = dr;
    th[0] = 1.f - dr;
#pragma unroll
    for (int k = 3; k < 5; k++) {
        float div = 1.f / (float)(k - 1);
        th[k - 1] = div * dr * th[k - 2];
#pragma unroll
        for (int l = 1; l < (k - 1); l++)
            th[k - l - 1] = div * ((dr + l) * th[k - l - 2] + ((float)(k - l) - dr) * th[k - l - 1]);
        th[0] = div * (1.f - dr) * th[0];
    }
    dth[0] = -th[0];
#pragma unroll
    for (int k = 1; k < 5; k++) dth[k] = th[k - 1] - th[k];
    float div = 0.25f;
    th[4] = div * dr * th[3];
#pragma unroll
    for (int l = 1; l < 4; l++) th[4 - l] = div * ((dr + l) * th[3 - l] + ((float)(5 - l) - dr) * th[4 - l]);
    th[0] = div * (1.f - dr) * th[0];
}

// Grid base index and fraction of one coordinate (NonbondedForce.cpp:51-71:
// the grid is anchored at the origin).
__device__ __forceinline__ void grid_coord(double p, double invL, int K, int &idx, float &fr) {
    double t = p * invL;
    t = (t - floor(t)) * K;
    int ti = (int)t;
    fr = (float)(t - ti);
    idx = ti % K;
}

// ---- set-up: clear the accumulator and the energy word, write the FFT
// geometry, work lists and twiddles; block 0 also computes the B-spline
// moduli |b(k)|^2 of the three axes with the neighbour average for values
// below 1e-7 (NonbondedForce.cpp:75-142).
__global__ void k_noalloc_setup(unsigned char *scr, FftSysDev F, int nz, int ny, int nx) {
    __shared__ double s_mod[3][kStaticMaxK];
    int *acc = region<int>(scr, kOffAcc);
    long long npts = (long long)F.K[0] * F.K[1] * F.K[2];
    long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long nthr = (long long)gridDim.x * blockDim.x;
    for (long long i = tid; i < npts; i += nthr) acc[i] = 0;
    if (tid < E_SLOTS) region<long long>(scr, kOffE)[tid] = 0;
    if (tid == 0) *region<FftSysDev>(scr, kOffSys) = F;
    FftWork *zw = region<FftWork>(scr, kOffWork);
    FftWork *yw = zw + kMaxWork, *xw = yw + kMaxWork;
    for (long long i = tid; i < kMaxWork; i += nthr) {
        int u = (int)i;
        if (u < nz) zw[u] = FftWork{0, u};
        if (u < ny) yw[u] = FftWork{0, u};
        if (u < nx) xw[u] = FftWork{0, u};
    }
    float2 *tw = region<float2>(scr, kOffTw);
    for (long long i = tid; i < F.K[0] + F.K[1] + F.K[2]; i += nthr) {
        int d = i < F.K[0] ? 0 : (i < F.K[0] + F.K[1] ? 1 : 2);
        int t = (int)i - F.tw[d];
        double a = -2.0 * kPi * (double)t / (double)F.K[d];
        double s, c;
        sincos(a, &s, &c);
        tw[i] = make_float2((float)c, (float)s);
    }
    if (blockIdx.x != 0) return;
    // spline values at the integer points, computed as the reference does
    double data[kOrder] = {0, 0, 0, 0, 0};
    data[0] = 1.0;
    for (int i = 3; i < kOrder; i++) {
        double div = 1.0 / (i - 1);
        data[i - 1] = 0.0;
        for (int j = 1; j < (i - 1); j++) data[i - j - 1] = div * (j * data[i - j - 2] + (i - j) * data[i - j - 1]);
        data[0] = div * data[0];
    }
    double div = 1.0 / (kOrder - 1);
    data[kOrder - 1] = div * data[kOrder - 2];
    for (int i = 1; i < (kOrder - 1); i++)
        data[kOrder - i - 1] = div * (i * data[kOrder - i - 2] + (kOrder - i) * data[kOrder - i - 1]);
    data[0] = div * data[0];
    for (int e = threadIdx.x; e < F.K[0] + F.K[1] + F.K[2]; e += blockDim.x) {
        int d = e < F.K[0] ? 0 : (e < F.K[0] + F.K[1] ? 1 : 2);
        int K = F.K[d], i = e - F.tw[d];
        double sc = 0.0, ss = 0.0;
        // b[j] = data[j - 1] for j = 1..order, zero elsewhere
        for (int j = 1; j <= kOrder && j < K; ++j) {
            double arg = (2 * kPi * i * j) / K;
            sc += data[j - 1] * cos(arg);
            ss += data[j - 1] * sin(arg);
        }
        s_mod[d][i] = sc * sc + ss * ss;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        int d = threadIdx.x, K = F.K[d];
        double *m = s_mod[d];
        for (int i = 0; i < K; i++)
            if (m[i] < 1e-7) m[i] = (m[(i - 1 + K) % K] + m[(i + 1) % K]) / 2.0;
        double *out = region<double>(scr, kOffMod) + d * kStaticMaxK;
        for (int i = 0; i < K; i++) out[i] = m[i];
    }
}

// ---- influence function on the half spectrum (NonbondedForce.cpp:323-388).
__global__ void k_noalloc_eterm(unsigned char *scr, Geometry g) {
    const double *mod = region<double>(scr, kOffMod);
    float *et = region<float>(scr, kOffEterm);
    int K0 = g.K[0], K1 = g.K[1], K2 = g.K[2], Kh = g.Kh;
    long long n = (long long)K0 * K1 * Kh;
    double factor = kPi * kPi / (g.alpha * g.alpha);
    double boxfactor = kPi * g.L[0] * g.L[1] * g.L[2];
    int maxkx = (K0 + 1) / 2, maxky = (K1 + 1) / 2, maxkz = (K2 + 1) / 2;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        int kz = (int)(i % Kh);
        long long r = i / Kh;
        int ky = (int)(r % K1), kx = (int)(r / K1);
        if (i == 0) {
            et[0] = 0.f;
            continue;
        }
        double mhx = ((kx < maxkx) ? kx : (kx - K0)) * (1 / g.L[0]);
        double mhy = ((ky < maxky) ? ky : (ky - K1)) * (1 / g.L[1]);
        double mhz = ((kz < maxkz) ? kz : (kz - K2)) * (1 / g.L[2]);
        double m2 = __dadd_rn(__dadd_rn(__dmul_rn(mhx, mhx), __dmul_rn(mhy, mhy)), __dmul_rn(mhz, mhz));
        double bx = boxfactor * mod[kx];
        double denom = m2 * bx * mod[kStaticMaxK + ky] * mod[2 * kStaticMaxK + kz];
        et[i] = (float)(kOne4PiEps0 * exp(-factor * m2) / denom);
    }
}

// ---- spread: one thread per atom, int32 fixed-point grid (2^-24 e units,
// the grid word the FFT's first pass reads).
__global__ void __launch_bounds__(128) k_noalloc_spread(unsigned char *scr, Geometry g, const double *xyz,
                                                        const double *charge, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int idx[3];
    float fr[3], th[3][5], dth[3][5];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        grid_coord(xyz[3 * (size_t)i + d], g.invL[d], g.K[d], idx[d], fr[d]);
        spline5(fr[d], th[d], dth[d]);
    }
    float q = (float)charge[i];
    int *acc = region<int>(scr, kOffAcc);
    int K0 = g.K[0], K1 = g.K[1], K2 = g.K[2];
    for (int ix = 0; ix < 5; ++ix) {
        int xi = idx[0] + ix;
        xi -= xi >= K0 ? K0 : 0;
        float qx = q * th[0][ix];
        for (int iy = 0; iy < 5; ++iy) {
            int yi = idx[1] + iy;
            yi -= yi >= K1 ? K1 : 0;
            float qxy = qx * th[1][iy];
            long long row = ((long long)xi * K1 + yi) * K2;
#pragma unroll
            for (int iz = 0; iz < 5; ++iz) {
                int zi = idx[2] + iz;
                zi -= zi >= K2 ? K2 : 0;
                atomicAdd(acc + row + zi, __float2int_rn(qxy * th[2][iz] * 16777216.0f));
            }
        }
    }
}

// ---- gather: one thread per atom; writes the force (kJ/mol/nm) and, from
// thread 0, the reciprocal energy.
__global__ void __launch_bounds__(128) k_noalloc_gather(unsigned char *scr, Geometry g, const double *xyz,
                                                        const double *charge, int n, double *force,
                                                        double *energy) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) *energy = (double)region<long long>(scr, kOffE)[E_RECIP] * kEnergyUnscale;
    if (i >= n) return;
    int idx[3];
    float fr[3], th[3][5], dth[3][5];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        grid_coord(xyz[3 * (size_t)i + d], g.invL[d], g.K[d], idx[d], fr[d]);
        spline5(fr[d], th[d], dth[d]);
    }
    const float *grid = region<float>(scr, kOffReal);
    int K0 = g.K[0], K1 = g.K[1], K2 = g.K[2];
    float fx = 0.f, fy = 0.f, fz = 0.f;
    for (int ix = 0; ix < 5; ++ix) {
        int xi = idx[0] + ix;
        xi -= xi >= K0 ? K0 : 0;
        for (int iy = 0; iy < 5; ++iy) {
            int yi = idx[1] + iy;
            yi -= yi >= K1 ? K1 : 0;
            const float *row = grid + ((long long)xi * K1 + yi) * K2;
            float txy = th[0][ix] * th[1][iy];
            float dxy = dth[0][ix] * th[1][iy];
            float tdy = th[0][ix] * dth[1][iy];
#pragma unroll
            for (int iz = 0; iz < 5; ++iz) {
                int zi = idx[2] + iz;
                zi -= zi >= K2 ? K2 : 0;
                float gv = row[zi];
                fx += dxy * th[2][iz] * gv;
                fy += tdy * th[2][iz] * gv;
                fz += txy * dth[2][iz] * gv;
            }
        }
    }
    float q = (float)charge[i];
    force[3 * (size_t)i] = (double)(-(q * (fx * (float)(K0 * g.invL[0]))));
    force[3 * (size_t)i + 1] = (double)(-(q * (fy * (float)(K1 * g.invL[1]))));
    force[3 * (size_t)i + 2] = (double)(-(q * (fz * (float)(K2 * g.invL[2]))));
}

bool smooth235(int n) {
    if (n < 1) return false;
    for (int p : {2, 3, 5})
        while (n % p == 0) n /= p;
    return n == 1;
}

// Device address of g_pme_scratch on the current device, looked up once.
int scratch_for_current_device(unsigned char **out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(NXM_ERR_CUDA, std::string("nxm_pme_reciprocal_noalloc: cudaGetDevice: ") +
                                                        cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return fail(NXM_ERR_CUDA, "nxm_pme_reciprocal_noalloc: device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_pme_scratch);
        if (e != cudaSuccess || !p)
            return fail(NXM_ERR_CUDA, std::string("nxm_pme_reciprocal_noalloc: cudaGetSymbolAddress: ") +
                                          cudaGetErrorString(e));
        g_scratch_ptr[dev] = static_cast<unsigned char *>(p);
    }
    *out = g_scratch_ptr[dev];
    return NXM_OK;
}

}  // namespace

extern "C" int nxm_pme_reciprocal_noalloc(const double *xyz, const double *charge, int32_t n_atoms,
                                          const double box_lb[3], const double box_ub[3],
                                          const int32_t grid[3], double alpha, double *force,
                                          double *energy, void *stream) {
    const char *fn = "nxm_pme_reciprocal_noalloc: ";
    if (n_atoms < 0 || !box_lb || !box_ub || !grid || !energy || (n_atoms > 0 && (!xyz || !charge || !force)))
        return fail(NXM_ERR_INVALID, std::string(fn) + "null argument or negative atom count");
    if (!(alpha > 0) || !(alpha < 1e300)) return fail(NXM_ERR_INVALID, std::string(fn) + "alpha must be positive");
    Geometry g{};
    for (int d = 0; d < 3; ++d) {
        if (grid[d] > kStaticMaxK) {
            char msg[160];
            std::snprintf(msg, sizeof msg, "%sgrid %dx%dx%d exceeds the static scratch limit of %d points per axis",
                          fn, grid[0], grid[1], grid[2], kStaticMaxK);
            return fail(NXM_ERR_CAPACITY, msg);
        }
        if (grid[d] < 5 || !smooth235(grid[d]))
            return fail(NXM_ERR_INVALID, std::string(fn) + "grid sizes must be 2^a 3^b 5^c and >= 5");
        g.K[d] = grid[d];
        g.L[d] = box_ub[d] - box_lb[d];
        if (g.L[d] < 0) g.L[d] = -g.L[d];
        if (!(g.L[d] > 0) || !(g.L[d] < 1e300)) return fail(NXM_ERR_INVALID, std::string(fn) + "empty box");
        g.invL[d] = 1 / g.L[d];
    }
    g.Kh = g.K[2] / 2 + 1;
    g.alpha = alpha;
    unsigned char *scr = nullptr;
    int rc = scratch_for_current_device(&scr);
    if (rc != NXM_OK) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);

    FftSysDev F{};
    int tw = 0;
    for (int d = 0; d < 3; ++d) {
        F.K[d] = g.K[d];
        F.tw[d] = tw;
        tw += g.K[d];
        fft_passes(g.K[d], F.ax[d]);
    }
    F.Kh = g.Kh;
    FftPlan plan;  // geometry only; every pointer is into g_pme_scratch
    plan.S = 1;
    plan.zlines = kZLines;
    plan.cols = kCols;
    int chunks = (g.Kh + kCols - 1) / kCols;
    plan.nz = (g.K[0] * g.K[1] + kZLines - 1) / kZLines;
    plan.ny = g.K[0] * chunks;
    plan.nx = g.K[1] * chunks;
    plan.kmax = std::max(g.K[0], std::max(g.K[1], g.K[2]));
    // line path (plan.plane = 0); at most 64 points per axis keeps every
    // block under the 48 KB that needs no shared-memory attribute
    plan.smem_z = fft_line_smem(kZLines / 2, plan.kmax, sizeof(float2));
    plan.smem_y = fft_line_smem(kCols, plan.kmax, sizeof(float2));
    plan.smem_x = plan.smem_y;
    plan.dsys = reinterpret_cast<FftSysDev *>(scr + kOffSys);
    plan.zwork = reinterpret_cast<FftWork *>(scr + kOffWork);
    plan.ywork = plan.zwork + kMaxWork;
    plan.xwork = plan.ywork + kMaxWork;

    DevView v{};
    v.N = n_atoms;
    v.S = 1;
    v.mixed = 1;
    v.force_mask = NXM_FORCE_NONBONDED;
    v.grid_acc = scr + kOffAcc;
    v.grid_real = scr + kOffReal;
    v.grid_cplx = scr + kOffCplx;
    v.eterm = scr + kOffEterm;
    v.twiddle = scr + kOffTw;
    v.E = reinterpret_cast<long long *>(scr + kOffE);
    v.total_grid = (long long)g.K[0] * g.K[1] * g.K[2];
    v.total_cgrid = (long long)g.K[0] * g.K[1] * g.Kh;

    // an error already pending on this thread belongs to the caller's earlier
    // work: report it and leave it pending rather than clear it
    cudaError_t pending = cudaPeekAtLastError();
    if (pending != cudaSuccess)
        return fail(NXM_ERR_CUDA, std::string(fn) + "a CUDA error was already pending: " +
                                      cudaGetErrorString(pending));
    k_noalloc_setup<<<152, 256, 0, st>>>(scr, F, plan.nz, plan.ny, plan.nx);
    k_noalloc_eterm<<<(int)std::min<long long>((v.total_cgrid + 255) / 256, 1216), 256, 0, st>>>(scr, g);
    if (n_atoms > 0) k_noalloc_spread<<<(n_atoms + 127) / 128, 128, 0, st>>>(scr, g, xyz, charge, n_atoms);
    launch_fft_convolve(v, plan, 1, st);
    k_noalloc_gather<<<std::max(1, (n_atoms + 127) / 128), 128, 0, st>>>(scr, g, xyz, charge, n_atoms, force,
                                                                          energy);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(NXM_ERR_CUDA, std::string(fn) + "launch failed: " + cudaGetErrorString(e));
    return NXM_OK;
}
