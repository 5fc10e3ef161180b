// Device-side definitions shared by every kernel of the NexusMD GB300 engine.
//
// Units follow the reference (nm, ps, kJ/mol, e).  Atoms of all systems of a
// batch live in one flattened "slot" space: system s owns slots
// [atom_off, atom_off + natoms) and, between neighbour-list rebuilds, slot
// order is the spatial (cell) order of that system.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

namespace nxm {

// Physical constants exactly as the reference spells them
// (core/baseline/headers/Forces/NonbondedForce.h:10-27).
constexpr double kPi = 3.14159265358979323846;
constexpr double kSqrtPi = 1.77245385090551602729;
constexpr double kTwoOverSqrtPi = 1.1283791670955126;
constexpr double kOne4PiEps0 = 138.93545764446428693393;

// Fixed-point scales (integer sums are order-independent, so
// bit-reproducible).  Forces: int64 multiples of 2^-32; the mixed-precision
// charge grid: int32 multiples of 2^-24 e; energies: int64 multiples of
// 2^-28 kJ/mol (|E| < 3.4e10).
constexpr double kForceScale = 4294967296.0;
constexpr double kForceUnscale = 1.0 / 4294967296.0;
constexpr double kGridScale = 16777216.0;
constexpr double kGridUnscale = 1.0 / 16777216.0;
constexpr double kEnergyScale = 268435456.0;
constexpr double kEnergyUnscale = 1.0 / 268435456.0;

constexpr int kOrder = 5;       // PME B-spline order (NonbondedForce.cpp:474)
constexpr int kCodeBits = 7;    // list entry = slot (25 bits) | cell-image code (7 bits)
constexpr uint32_t kSlotMask = (1u << 25) - 1u;
constexpr int kMaxExclFast = 32;
// cell-image displacement table per system: 5 (x) * 5 (y) * 12 (z) codes
constexpr int kDtabStride = 320;
constexpr int kMaxGroupCells = 8;  // cells per group of the tile kernels (5*5*(8+4) = 300 codes)
constexpr int kMaxGroupCellsWide = 4;  // the same with one 32-warp tile block per SM (FP32 tile extent)
constexpr int kMaxSmemDevices = 64;  // devices whose shared-memory attributes are tracked

// Energy slots per system.
enum EnergyTerm {
    E_BOND = 0,
    E_ANGLE,
    E_TORSION,
    E_RECIP,
    E_SELF,
    E_COUL,
    E_VDW,
    E_EXCL,
    E_KIN,
    E_EXCEPT,  // exception (scaled 1-4) pairs

    E_SLOTS = 16
};

// Device error bits (read by the host after each call).
enum ErrorBits {
    ERR_NLIST_OVERFLOW = 1,
    ERR_EXCL_OVERFLOW = 2,
    ERR_FORCE_RANGE = 4,
    ERR_NONFINITE = 8,
    ERR_SKIN_VIOLATION = 16,
    ERR_CELL = 32,
};

struct SysDev {
    double lb[3], ub[3], L[3], invL[3], halfL[3];
    double cutoff, cut2, alpha, rlist2, sw_dist;
    float Lf[3], halfLf[3], cut2f, cut2f_lo, cut2f_hi, alphaf, rlist2f, sw_distf, cutofff;
    int use_switch;
    int nb_on;                // nonbonded force enabled for this system
    int atom_off, natoms;
    int K[3], Kh;             // PME grid, Kh = K[2]/2 + 1
    long long grid_off;       // first element of this system's real grid
    long long cgrid_off;      // first element of this system's half complex grid
    int nc[3], cell_off;      // neighbour cells
    double cs[3];             // cell edge
    int tw_off[3];            // twiddle-table offsets for the three FFT lengths
    // FP32 pair-kernel constants: exp(-(alpha r)^2) = 2^(r^2 ex2c),
    // 0.4 alpha (erfc fit argument), 2 alpha / sqrt(pi); cell edges
    float ex2c, a04, k2a, csf[3];
    // PME grid coordinates from cell-relative positions (mixed precision):
    // cgrid[cg_off[d] + c] holds the grid coordinate of cell c's lower corner
    // along axis d (integer part, fraction); kl = K / L
    int cg_off[3];
    float kl[3];
    // box edge and half edge as multiples of 2^-40 nm (fix40), for the
    // minimum image of fixed-point displacements
    long long L40[3], halfL40[3];
    // order-preserving integer keys (dkey) of the box corners, for the
    // update's wrap test without FP64 comparisons
    long long lbkey[3], ubkey[3];
};

// Flags word layout in device memory.
struct Flags {
    int error;
    int rebuild;     // 1 = rebuild the neighbour list this step
    int since;       // steps since the last rebuild
    int interval;    // longest allowed gap between rebuilds
    int skin_hit;    // an atom moved more than skin/2 since the last rebuild
    int nrebuild;    // rebuilds so far
    int pad[2];
};

// ----------------------------------------------------------------- helpers

// Positions in fixed point.  This GPU issues FP64 instructions (arithmetic,
// comparisons and conversions alike) at a small fraction of its FP32 and
// integer rates, yet a displacement between two nearby atoms needs FP64
// precision only until it is rounded to FP32.  fix40(x) = x * 2^40 rounded
// to the nearest integer (half away from zero), formed from the bits of the
// double with integer instructions only; exact to 2^-41 nm for |x| < 2^22 nm.
// The difference of two such values is the displacement to 2^-40 nm, and
// its minimum image is an integer compare-and-add.
__host__ __device__ __forceinline__ long long fix40(double x) {
    long long b;
#ifdef __CUDA_ARCH__
    b = __double_as_longlong(x);
#else
    memcpy(&b, &x, sizeof b);
#endif
    const int e = (int)((b >> 52) & 0x7ff);
    const long long m = (b & 0xfffffffffffffLL) | 0x10000000000000LL;
    const int sh = 1035 - e;  // x * 2^40 = m * 2^(e - 1035)
    long long r = sh <= 0 ? (m << (-sh < 9 ? -sh : 9)) : (sh < 62 ? ((m >> (sh - 1)) + 1) >> 1 : 0);
    r = e == 0 ? 0 : r;
    return b < 0 ? -r : r;
}

// d * 2^-40 rounded once to FP32 (|d| < 2^45): d = hi 2^21 + lo with
// |hi| < 2^24 and 0 <= lo < 2^21, both exact in FP32, so the fused
// multiply-add rounds the exact value.
__device__ __forceinline__ float fix40_to_float(long long d) {
    const float hi = (float)(int)(d >> 21);
    const float lo = (float)(int)(d & 0x1fffff);
    return fmaf(hi, 1.9073486328125e-06f /* 2^-19 */, lo * 9.094947017729282e-13f /* 2^-40 */);
}

// The reference's single-shift minimum image (PeriodicBoundaryCondition.cpp
// :93-104) on a fixed-point displacement, rounded to FP32.
__device__ __forceinline__ float min_image40(long long d, long long L40, long long halfL40) {
    d = d > halfL40 ? d - L40 : (d < -halfL40 ? d + L40 : d);
    return fix40_to_float(d);
}

// An integer key with the order of the doubles it comes from (non-NaN):
// dkey(a) < dkey(b) exactly when a < b, -0 and +0 equal.
__host__ __device__ __forceinline__ long long dkey(double x) {
    long long b;
#ifdef __CUDA_ARCH__
    b = __double_as_longlong(x);
#else
    memcpy(&b, &x, sizeof b);
#endif
    return b < 0 ? (long long)((unsigned long long)0x8000000000000000ULL - (unsigned long long)b) : b;
}

__device__ __forceinline__ void atomic_add_fixed(long long *a, double v, double scale) {
    atomicAdd(reinterpret_cast<unsigned long long *>(a),
              static_cast<unsigned long long>(__double2ll_rn(v * scale)));
}

// float -> int64 fixed point in units of 2^-32, without the FP64 pipe (on
// this GPU double-precision and 64-bit conversion instructions issue far
// slower than FP32 and int32 ones): v = h + l with h = rint(v) and
// l = v - h in [-1/2, 1/2], both exact in FP32; h converts to int32 as is
// and l at 2^-31, so the result is round(v * 2^31) * 2 -- the 2^-32 grid
// less its last bit, for |v| < 2^31.
__device__ __forceinline__ unsigned long long to_fixed32(float v) {
    float h = rintf(v);
    float l = v - h;
    long long hi = __float2int_rn(h);
    long long lo = __float2int_rn(l * 2147483648.0f);
    return (static_cast<unsigned long long>(hi) << 32) + (static_cast<unsigned long long>(lo) << 1);
}

__device__ __forceinline__ void acc_add(long long *a, float v) {
    atomicAdd(reinterpret_cast<unsigned long long *>(a), to_fixed32(v));
}
__device__ __forceinline__ void acc_add(double *a, double v) { atomicAdd(a, v); }

__device__ __forceinline__ double acc_value(long long a) { return (double)a * kForceUnscale; }
__device__ __forceinline__ double acc_value(double a) { return a; }

// The reference's minimum image: one +-L shift when |d| > L/2
// (core/common/src/PeriodicBoundaryCondition.cpp:93-104).
__device__ __forceinline__ double min_image(double d, double L, double halfL) {
    if (d > halfL)
        d -= L;
    else if (d < -halfL)
        d += L;
    return d;
}

// The same single-shift minimum image for the mixed-precision paths: the FP64
// difference d is rounded to FP32 once and the shift is decided on that
// float (it can differ from the FP64 decision only for |d| within FP32
// rounding of L/2, which bonded and excluded pairs never approach); a
// shifted component is re-formed in FP64 before its rounding.
__device__ __forceinline__ float min_image_f(double d, double L, float halfLf) {
    float f = (float)d;
    if (f > halfLf)
        f = (float)(d - L);
    else if (f < -halfLf)
        f = (float)(d + L);
    return f;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Energy accumulation: a block-wide FP64 sum per (term, system), added once
// per block as fixed point when every thread of the block is in one system;
// otherwise each warp (or lane) adds its own share.  Deterministic.
__device__ __forceinline__ void energy_add(long long *E, int sys, int term, double v) {
    const unsigned full = 0xffffffffu;
    int s0 = __shfl_sync(full, sys, 0);
    if (__all_sync(full, sys == s0)) {
        v = warp_sum(v);
        if ((threadIdx.x & 31) == 0 && v != 0.0) atomic_add_fixed(&E[s0 * E_SLOTS + term], v, kEnergyScale);
    } else if (v != 0.0) {
        atomic_add_fixed(&E[sys * E_SLOTS + term], v, kEnergyScale);
    }
}

// v * 2^28 (the energy unit) rounded to an integer with FP32 and integer
// instructions only: v = h + l with h = rint(v) and l = v - h, both exact in
// FP32, so h 2^28 is exact and l 2^28 rounds once (|v| < 2^31).
__device__ __forceinline__ long long energy_fixed(float v) {
    const float h = rintf(v);
    const float l = v - h;
    return ((long long)__float2int_rn(h) << 28) + (long long)__float2int_rn(l * 268435456.0f);
}

// Energy accumulation of the FP32 kernels: each lane's FP32 partial is
// converted to fixed point (energy_fixed) and the warp sums the integers --
// no FP64 instruction, order-free, one atomic per warp when every lane is in
// one system (per lane otherwise).
__device__ __forceinline__ void energy_add_f(long long *E, int sys, int term, float v) {
    const unsigned full = 0xffffffffu;
    long long w = energy_fixed(v);
    const int s0 = __shfl_sync(full, sys, 0);
    if (__all_sync(full, sys == s0)) {
        for (int o = 16; o; o >>= 1) w += __shfl_xor_sync(full, w, o);
        if ((threadIdx.x & 31) == 0 && w != 0)
            atomicAdd(reinterpret_cast<unsigned long long *>(&E[s0 * E_SLOTS + term]), static_cast<unsigned long long>(w));
    } else if (w != 0) {
        atomicAdd(reinterpret_cast<unsigned long long *>(&E[sys * E_SLOTS + term]), static_cast<unsigned long long>(w));
    }
}

// The energy sum of either arithmetic: FP32 partials as fixed point, FP64
// partials by the FP64 warp sum.
__device__ __forceinline__ void energy_add_t(long long *E, int sys, int term, float v) { energy_add_f(E, sys, term, v); }
__device__ __forceinline__ void energy_add_t(long long *E, int sys, int term, double v) { energy_add(E, sys, term, v); }

// Adds one fixed-point energy per lane (units of 1 / kEnergyScale) of a
// warp whose lanes all belong to system `sys`: integer sums, so the total does
// not depend on how the contributions were grouped into lanes and warps.
__device__ __forceinline__ void energy_add_fixed(long long *E, int sys, int term, long long v) {
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0 && v != 0)
        atomicAdd(reinterpret_cast<unsigned long long *>(&E[sys * E_SLOTS + term]), static_cast<unsigned long long>(v));
}

// erfc(x) = exp(-x^2) * g(t), t = 1 / (1 + 0.4 x), x in [0, 4]: degree-6
// least-squares fit of the scaled complementary error function on Chebyshev
// nodes of t, max relative error 5e-7 in FP32 (derivation and error table:
// fit_erfcx.py next to this file).
__device__ __forceinline__ float erfcx_fit(float t) {
    float g = -2.164941738e-01f;
    g = fmaf(g, t, 7.803782561e-01f);
    g = fmaf(g, t, -4.985805536e-01f);
    g = fmaf(g, t, 5.875147125e-01f);
    g = fmaf(g, t, 1.009222009e-01f);
    g = fmaf(g, t, 2.479314205e-01f);
    g = fmaf(g, t, -1.671998421e-03f);
    return g;
}

__device__ __forceinline__ float fast_rcp(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

__device__ __forceinline__ float fast_rsqrt(float x) {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// (erf(x) - 2x exp(-x^2)/sqrt(pi)) without the cancellation at small x:
// for x < 0.6 the Maclaurin series of the difference,
//   (2/sqrt(pi)) * sum_{n>=1} (-1)^(n+1) x^(2n+1) 2n / (n! (2n+1)),
// otherwise the direct form.
__device__ __forceinline__ float erf_minus_gauss(float x, float e /* exp(-x^2) */) {
    if (x < 0.6f) {
        float x2 = x * x;
        float s = -1.0f / 42840.0f;                 // n = 8: 16 / (8! * 17)
        s = fmaf(s, x2, 1.0f / 5400.0f);            // n = 7
        s = fmaf(s, x2, -1.0f / 780.0f);            // n = 6
        s = fmaf(s, x2, 1.0f / 132.0f);             // n = 5
        s = fmaf(s, x2, -1.0f / 27.0f);             // n = 4
        s = fmaf(s, x2, 1.0f / 7.0f);               // n = 3
        s = fmaf(s, x2, -0.4f);                     // n = 2
        s = fmaf(s, x2, 2.0f / 3.0f);               // n = 1
        return (float)kTwoOverSqrtPi * x * x2 * s;
    }
    return erff(x) - (float)kTwoOverSqrtPi * x * e;
}

}  // namespace nxm
