// Real-space Ewald (erfc-Coulomb) + Lennard-Jones pair forces over the full
// per-atom neighbour list, one warp per atom, and the exclusion correction.
//
// Physics follows NonbondedForce::DirectForcesAndEnergy
// (core/baseline/src/Forces/NonbondedForce.cpp:530-585): sigma_ij =
// sigma_i/2 + sigma_j/2, eps_ij = (2 sqrt eps_i)(2 sqrt eps_j), no LJ shift,
// no dispersion correction; and CalculateExclusionEnergyAndForces (:590-630).
// The optional switching function is applied per pair (the reference never
// resets its switch state between pairs, :541; that order-dependent carry-over
// is not reproduced).  Pair membership is decided exactly as the reference's
// list does: FP64 single-shift minimum image, r^2 < cutoff^2
// (NeighborList.cpp:106-116); in mixed mode the FP32 r^2 settles all but the
// pairs within 1e-5 relative of the cutoff, which are re-tested in FP64.
#include "nxm_view.h"

namespace nxm {

// r^2 of the pair exactly as the reference forms it: d = p_j - p_i with one
// shift per component, then (dx*dx + dy*dy) + dz*dz with no fused multiply-add.
__device__ __forceinline__ double exact_r2(const DevView &v, const SysDev &S, int i, int j) {
    double dx = min_image(__dsub_rn(v.x[j], v.x[i]), S.L[0], S.halfL[0]);
    double dy = min_image(__dsub_rn(v.y[j], v.y[i]), S.L[1], S.halfL[1]);
    double dz = min_image(__dsub_rn(v.z[j], v.z[i]), S.L[2], S.halfL[2]);
    return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
}

template <bool ENERGY>
__global__ void __launch_bounds__(256) k_pairs_mixed(DevView v) {
    int lane = threadIdx.x & 31;
    int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < v.N; i += nwarps) {
        int sys = v.sys_of[i];
        const SysDev &S = v.sys[sys];
        const float lo = S.cut2f_lo, hi = S.cut2f_hi, alpha = S.alphaf;
        const float4 *dt = v.dtab + sys * 128;
        float4 pi = v.pf[i];
        float2 li = v.ljf[i];
        int cnt = v.ncount[i];
        const uint32_t *lst = v.nlist + (size_t)i * v.stride;
        float fx = 0.f, fy = 0.f, fz = 0.f, ec = 0.f, ev = 0.f;
        for (int k = lane; k < cnt; k += 32) {
            uint32_t e = __ldg(lst + k);
            int j = (int)(e & kSlotMask);
            float4 pj = __ldg(v.pf + j);
            float4 D = __ldg(dt + (e >> 25));
            float dx = pi.x - pj.x + D.x;
            float dy = pi.y - pj.y + D.y;
            float dz = pi.z - pj.z + D.z;
            float r2 = dx * dx + dy * dy + dz * dz;
            if (r2 >= hi) continue;
            if (r2 >= lo && !(exact_r2(v, S, i, j) < S.cut2)) continue;
            float2 lj = __ldg(v.ljf + j);
            float rinv = rsqrtf(r2);
            float rinv2 = rinv * rinv;
            float r = r2 * rinv;
            float xa = alpha * r;
            float ex = __expf(-xa * xa);
            float erfcv = ex * erfcx_fit(fast_rcp(fmaf(0.4f, xa, 1.0f)));
            float qq = pi.w * pj.w;
            float dEdR = qq * rinv * rinv2 * (erfcv + (float)kTwoOverSqrtPi * xa * ex);
            float sg = li.x + lj.x;
            float s2 = sg * sg * rinv2;
            float s6 = s2 * s2 * s2;
            float eps = li.y * lj.y;
            float evdw = eps * (s6 - 1.0f) * s6;
            float sw = 1.0f;
            if (S.use_switch && r > S.sw_distf) {
                float w = S.cutofff - S.sw_distf;
                float t = (r - S.sw_distf) / w;
                sw = 1.0f + t * t * t * (-10.0f + t * (15.0f - t * 6.0f));
                float dsw = t * t * (-30.0f + t * (60.0f - t * 30.0f)) / w;
                dEdR -= evdw * dsw * rinv;
            }
            dEdR += sw * eps * (12.0f * s6 - 6.0f) * s6 * rinv2;
            fx = fmaf(dx, dEdR, fx);
            fy = fmaf(dy, dEdR, fy);
            fz = fmaf(dz, dEdR, fz);
            if (ENERGY) {
                ec = fmaf(qq * rinv, erfcv, ec);
                ev = fmaf(sw, evdw, ev);
            }
        }
        fx = warp_sum(fx);
        fy = warp_sum(fy);
        fz = warp_sum(fz);
        if (lane == 0) {
            acc_add(static_cast<long long *>(v.fx) + i, fx);
            acc_add(static_cast<long long *>(v.fy) + i, fy);
            acc_add(static_cast<long long *>(v.fz) + i, fz);
        }
        if (ENERGY) {
            // each pair sits in both partners' lists
            energy_add(v.E, sys, E_COUL, 0.5 * (double)ec);
            energy_add(v.E, sys, E_VDW, 0.5 * (double)ev);
        }
    }
}

template <bool ENERGY>
__global__ void __launch_bounds__(256) k_pairs_fp64(DevView v) {
    int lane = threadIdx.x & 31;
    int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < v.N; i += nwarps) {
        int sys = v.sys_of[i];
        const SysDev &S = v.sys[sys];
        double xi = v.x[i], yi = v.y[i], zi = v.z[i];
        double qi = v.qs[i];
        double2 li = v.ljd[i];
        int cnt = v.ncount[i];
        const uint32_t *lst = v.nlist + (size_t)i * v.stride;
        double fx = 0, fy = 0, fz = 0, ec = 0, ev = 0;
        for (int k = lane; k < cnt; k += 32) {
            int j = (int)(lst[k] & kSlotMask);
            if (!(exact_r2(v, S, i, j) < S.cut2)) continue;
            // deltaR = minimumImageVector(p_i, p_j) (NonbondedForce.cpp:548)
            double dx = min_image(xi - v.x[j], S.L[0], S.halfL[0]);
            double dy = min_image(yi - v.y[j], S.L[1], S.halfL[1]);
            double dz = min_image(zi - v.z[j], S.L[2], S.halfL[2]);
            double r = sqrt(dx * dx + dy * dy + dz * dz);
            double rinv = 1.0 / r;
            double sw = 1.0, dsw = 0.0;
            if (S.use_switch && r > S.sw_dist) {
                double t = (r - S.sw_dist) / (S.cutoff - S.sw_dist);
                sw = 1 + t * t * t * (-10 + t * (15 - t * 6));
                dsw = t * t * (-30 + t * (60 - t * 30)) / (S.cutoff - S.sw_dist);
            }
            double xa = S.alpha * r;
            double qq = qi * v.qs[j];
            double erfcv = erfc(xa);
            double dEdR = qq * rinv * rinv * rinv * (erfcv + 2 * xa * exp(-xa * xa) / kSqrtPi);
            double2 lj = v.ljd[j];
            double sg = li.x + lj.x;
            double s2 = sg * rinv;
            s2 *= s2;
            double s6 = s2 * s2 * s2;
            double eps = li.y * lj.y;
            dEdR += sw * eps * (12.0 * s6 - 6.0) * s6 * rinv * rinv;
            double evdw = eps * (s6 - 1.0) * s6;
            if (S.use_switch) {
                dEdR -= evdw * dsw * rinv;
                evdw *= sw;
            }
            fx += dx * dEdR;
            fy += dy * dEdR;
            fz += dz * dEdR;
            if (ENERGY) {
                ec += qq * rinv * erfcv;
                ev += evdw;
            }
        }
        fx = warp_sum(fx);
        fy = warp_sum(fy);
        fz = warp_sum(fz);
        if (lane == 0) {
            atomicAdd(static_cast<double *>(v.fx) + i, fx);
            atomicAdd(static_cast<double *>(v.fy) + i, fy);
            atomicAdd(static_cast<double *>(v.fz) + i, fz);
        }
        if (ENERGY) {
            energy_add(v.E, sys, E_COUL, 0.5 * ec);
            energy_add(v.E, sys, E_VDW, 0.5 * ev);
        }
    }
}

// One thread per excluded pair (i < j by original index): subtract the erf
// (reciprocal-space) part of the pair, at any separation, as
// NonbondedForce.cpp:590-630 does.  E_EXCL holds the positive total that the
// reference subtracts from the potential energy.
template <bool MIXED>
__global__ void __launch_bounds__(256) k_exclusions(DevView v, int energy) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    double e = 0.0;
    int sys = 0;
    if (t < v.nex) {
        int2 p = v.ex_slot[t];
        int ii = p.x, jj = p.y;
        sys = v.sys_of[ii];
        const SysDev &S = v.sys[sys];
        double dx = min_image(v.x[ii] - v.x[jj], S.L[0], S.halfL[0]);
        double dy = min_image(v.y[ii] - v.y[jj], S.L[1], S.halfL[1]);
        double dz = min_image(v.z[ii] - v.z[jj], S.L[2], S.halfL[2]);
        if (MIXED) {
            float fdx = (float)dx, fdy = (float)dy, fdz = (float)dz;
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
                e = (double)(qq * rinv * erfv);
            } else {
                e = (double)S.alpha * kTwoOverSqrtPi * (double)qq;
            }
        } else {
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
    }
    if (energy) energy_add(v.E, sys, E_EXCL, e);
}

static int pair_grid(int N) {
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    long long need = ((long long)N * 32 + 255) / 256;
    long long cap = (long long)sms * 8;  // 8 resident 256-thread blocks per SM
    return (int)(need < cap ? need : cap);
}

void launch_pairs(const DevView &v, int energy, cudaStream_t st) {
    if (v.N == 0) return;
    int g = pair_grid(v.N);
    if (v.mixed) {
        if (energy)
            k_pairs_mixed<true><<<g, 256, 0, st>>>(v);
        else
            k_pairs_mixed<false><<<g, 256, 0, st>>>(v);
    } else {
        if (energy)
            k_pairs_fp64<true><<<g, 256, 0, st>>>(v);
        else
            k_pairs_fp64<false><<<g, 256, 0, st>>>(v);
    }
}

void launch_exclusions(const DevView &v, int energy, cudaStream_t st) {
    if (v.nex == 0) return;
    int nb = (v.nex + 255) / 256;
    if (v.mixed)
        k_exclusions<true><<<nb, 256, 0, st>>>(v, energy);
    else
        k_exclusions<false><<<nb, 256, 0, st>>>(v, energy);
}

// ---- test support: the neighbour pair set within the cutoff, exactly as
// the reference decides it, as (larger, smaller) original indices.
__global__ void k_collect(DevView v, int sys_sel, int *out, long long cap, unsigned long long *n) {
    int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (i >= v.N) return;
    int sys = v.sys_of[i];
    if (sys != sys_sel) return;
    const SysDev &S = v.sys[sys];
    int oi = v.orig[i];
    int cnt = v.ncount[i];
    for (int k = lane; k < cnt; k += 32) {
        int j = (int)(v.nlist[(size_t)i * v.stride + k] & kSlotMask);
        int oj = v.orig[j];
        if (oi <= oj) continue;
        if (!(exact_r2(v, S, i, j) < S.cut2)) continue;
        unsigned long long p = atomicAdd(n, 1ull);
        if ((long long)p < cap) {
            out[2 * p] = oi - S.atom_off;
            out[2 * p + 1] = oj - S.atom_off;
        }
    }
}

long long launch_collect_pairs(const DevView &v, int sys, int *out_pairs, long long cap,
                               cudaStream_t st) {
    unsigned long long *dn;
    cudaMallocAsync(&dn, sizeof(unsigned long long), st);
    cudaMemsetAsync(dn, 0, sizeof(unsigned long long), st);
    k_collect<<<(int)(((long long)v.N * 32 + 255) / 256), 256, 0, st>>>(v, sys, out_pairs, cap, dn);
    unsigned long long n = 0;
    cudaMemcpyAsync(&n, dn, sizeof(n), cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);
    cudaFreeAsync(dn, st);
    return (long long)n;
}

}  // namespace nxm
