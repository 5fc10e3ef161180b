// Per-pair terms of the nonbonded force that bypass the neighbour list: the
// exclusion correction of the Ewald sum and the exception (scaled 1-4)
// pairs, one call per pair.  The standalone kernels (k_nonbonded.cu) and the
// fused per-term kernel (k_bonded.cu) share them.
//
// Exclusion correction (one excluded pair):
// CalculateExclusionEnergyAndForces (core/baseline/src/Forces/
// NonbondedForce.cpp:590-630): for every excluded pair (i < j), at any
// separation, remove the erf (reciprocal-space) part of the pair; when
// erf(alpha r) <= 1e-6 only the r -> 0 energy limit alpha 2/sqrt(pi) q_i q_j
// is removed.  E_EXCL holds the positive total the reference subtracts from
// the potential energy.  Displacements are always formed from the FP64
// positions with the reference's minimum image (mixed mode: exactly, in
// 2^-40 nm fixed point with integer instructions, then rounded once to FP32);
// mixed mode then works in FP32, with the small-argument difference
// erf(x) - 2x exp(-x^2)/sqrt(pi) taken from its series so bonded neighbours
// (x ~ 0.25) do not lose digits to cancellation.
#pragma once

#include <type_traits>

#include "nxm_view.h"

namespace nxm {

// The energy type of a pair term: FP32 in mixed mode (summed as fixed point
// by energy_add_f), FP64 otherwise.
template <bool MIXED>
using TermE = typename std::conditional<MIXED, float, double>::type;

// Excluded pair t: adds its forces, returns its E_EXCL energy, sets sys.
template <bool MIXED>
__device__ __forceinline__ TermE<MIXED> exclusion_pair(const DevView &v, int t, int &sys) {
    TermE<MIXED> e = 0;
    int2 p = v.ex_slot[t];
    int ii = p.x, jj = p.y;
    sys = v.sys_of[ii];
    const SysDev &S = v.sys[sys];
    if (MIXED) {
        float fdx = min_image40(fix40(v.x[ii]) - fix40(v.x[jj]), S.L40[0], S.halfL40[0]);
        float fdy = min_image40(fix40(v.y[ii]) - fix40(v.y[jj]), S.L40[1], S.halfL40[1]);
        float fdz = min_image40(fix40(v.z[ii]) - fix40(v.z[jj]), S.L40[2], S.halfL40[2]);
        float r = sqrtf(fdx * fdx + fdy * fdy + fdz * fdz);
        float rinv = 1.0f / r;
        float xa = S.alphaf * r;
        float qq = v.pf[ii].w * v.pf[jj].w;
        float erfv = erff(xa);
        if (erfv > 1e-6f) {
            float ex = expf(-xa * xa);
            float dEdR = qq * rinv * rinv * rinv * erf_minus_gauss(xa, ex);
            acc_add(static_cast<long long *>(v.fx) + ii, -fdx * dEdR);
            acc_add(static_cast<long long *>(v.fy) + ii, -fdy * dEdR);
            acc_add(static_cast<long long *>(v.fz) + ii, -fdz * dEdR);
            acc_add(static_cast<long long *>(v.fx) + jj, fdx * dEdR);
            acc_add(static_cast<long long *>(v.fy) + jj, fdy * dEdR);
            acc_add(static_cast<long long *>(v.fz) + jj, fdz * dEdR);
            e = qq * rinv * erfv;
        } else {
            e = S.alphaf * (float)kTwoOverSqrtPi * qq;
        }
    } else {
        double dx = min_image(v.x[ii] - v.x[jj], S.L[0], S.halfL[0]);
        double dy = min_image(v.y[ii] - v.y[jj], S.L[1], S.halfL[1]);
        double dz = min_image(v.z[ii] - v.z[jj], S.L[2], S.halfL[2]);
        double r = sqrt(dx * dx + dy * dy + dz * dz);
        double rinv = 1.0 / r;
        double xa = S.alpha * r;
        double qq = v.qs[ii] * v.qs[jj];
        double erfv = erf(xa);
        if (erfv > 1e-6) {
            double dEdR = qq * rinv * rinv * rinv * (erfv - 2 * xa * exp(-xa * xa) / kSqrtPi);
            atomicAdd(static_cast<double *>(v.fx) + ii, -dx * dEdR);
            atomicAdd(static_cast<double *>(v.fy) + ii, -dy * dEdR);
            atomicAdd(static_cast<double *>(v.fz) + ii, -dz * dEdR);
            atomicAdd(static_cast<double *>(v.fx) + jj, dx * dEdR);
            atomicAdd(static_cast<double *>(v.fy) + jj, dy * dEdR);
            atomicAdd(static_cast<double *>(v.fz) + jj, dz * dEdR);
            e = qq * rinv * erfv;
        } else {
            e = S.alpha * kTwoOverSqrtPi * qq;
        }
    }
    return e;
}

// Exception pairs (scaled 1-4 interactions) in the semantics of OpenMM's
// NonbondedForce exceptions -- the reference parses them
// (core/common/src/SystemXMLParser.cpp:182-191) but applies none:
// E = ke chargeProd / r + 4 eps ((sig/r)^12 - (sig/r)^6) with plain
// Coulomb.  Every exception pair is also an exclusion, so the Ewald sum
// already left it out of the direct space and the exclusion correction
// removed its reciprocal part.  Displacement with the reference's minimum
// image (mixed: fixed point as above); FP32 arithmetic and parameters and
// fixed-point sums in mixed mode.
//
// Exception pair t: adds its forces, returns its E_EXCEPT energy, sets sys.
template <bool MIXED>
__device__ __forceinline__ TermE<MIXED> exception_pair(const DevView &v, int t, int &sys) {
    TermE<MIXED> e = 0;
    int2 p = v.xc_slot[t];
    int ii = p.x, jj = p.y;
    sys = v.sys_of[ii];
    const SysDev &S = v.sys[sys];
    if (MIXED) {
        const float4 prm = v.xc_prmf[t];
        float fdx = min_image40(fix40(v.x[ii]) - fix40(v.x[jj]), S.L40[0], S.halfL40[0]);
        float fdy = min_image40(fix40(v.y[ii]) - fix40(v.y[jj]), S.L40[1], S.halfL40[1]);
        float fdz = min_image40(fix40(v.z[ii]) - fix40(v.z[jj]), S.L40[2], S.halfL40[2]);
        float rinv2 = 1.0f / (fdx * fdx + fdy * fdy + fdz * fdz);
        float rinv = sqrtf(rinv2);
        float coul = prm.x * rinv;
        float sg = prm.y;
        float s2 = sg * sg * rinv2;
        float s6 = s2 * s2 * s2;
        float e4 = prm.z;
        float dEdR = (coul + e4 * (12.0f * s6 - 6.0f) * s6) * rinv2;
        acc_add(static_cast<long long *>(v.fx) + ii, fdx * dEdR);
        acc_add(static_cast<long long *>(v.fy) + ii, fdy * dEdR);
        acc_add(static_cast<long long *>(v.fz) + ii, fdz * dEdR);
        acc_add(static_cast<long long *>(v.fx) + jj, -fdx * dEdR);
        acc_add(static_cast<long long *>(v.fy) + jj, -fdy * dEdR);
        acc_add(static_cast<long long *>(v.fz) + jj, -fdz * dEdR);
        e = coul + e4 * (s6 - 1.0f) * s6;
    } else {
        const double4 prm = v.xc_prm[t];
        double dx = min_image(v.x[ii] - v.x[jj], S.L[0], S.halfL[0]);
        double dy = min_image(v.y[ii] - v.y[jj], S.L[1], S.halfL[1]);
        double dz = min_image(v.z[ii] - v.z[jj], S.L[2], S.halfL[2]);
        double r2 = dx * dx + dy * dy + dz * dz;
        double rinv = 1.0 / sqrt(r2);
        double coul = prm.x * rinv;
        double s2 = prm.y * rinv;
        s2 *= s2;
        double s6 = s2 * s2 * s2;
        double dEdR = (coul + prm.z * (12.0 * s6 - 6.0) * s6) * rinv * rinv;
        atomicAdd(static_cast<double *>(v.fx) + ii, dx * dEdR);
        atomicAdd(static_cast<double *>(v.fy) + ii, dy * dEdR);
        atomicAdd(static_cast<double *>(v.fz) + ii, dz * dEdR);
        atomicAdd(static_cast<double *>(v.fx) + jj, -dx * dEdR);
        atomicAdd(static_cast<double *>(v.fy) + jj, -dy * dEdR);
        atomicAdd(static_cast<double *>(v.fz) + jj, -dz * dEdR);
        e = coul + prm.z * (s6 - 1.0) * s6;
    }
    return e;
}

}  // namespace nxm
