// Leapfrog update, kinetic energy and report snapshot, one thread per slot.
// report: 0 none, 1 energies and the x/v/F snapshot, 2 energies and the
// positions only (a frame).
//
// VerletIntegration::Advance (core/baseline/src/VerletIntegration.cpp:49-89)
// with dt[0] = dt[1] = dt: v += invm F dt; x' = x + v dt; one +-L wrap into
// [lb, ub]; atoms with invm == 0 stay put.  On report steps the kinetic
// energy of the on-step velocity estimate v + F dt / (2m)
// (KineticEnergy.cpp:21-41) and a copy of x, v, F in original atom order are
// taken before the update, which is where Engine::Report sits
// (Engine.cpp:162-188).  The force accumulators are read, converted to FP64
// and cleared here, so the next step starts from zero without a memset.
#include "nxm_view.h"

namespace nxm {

template <typename Acc>
__global__ void __launch_bounds__(256) k_integrate(DevView v, double dt, int report) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    bool live = s < v.N;
    int sys = live ? v.sys_of[s] : 0;
    double ke = 0.0;   // FP64 engine
    float kef = 0.0f;  // mixed engine (summed as fixed point)
    if (live) {
        const SysDev &S = v.sys[sys];
        Acc *ax = static_cast<Acc *>(v.fx) + s;
        Acc *ay = static_cast<Acc *>(v.fy) + s;
        Acc *az = static_cast<Acc *>(v.fz) + s;
        const Acc w[3] = {*ax, *ay, *az};
        *ax = (Acc)0;
        *ay = (Acc)0;
        *az = (Acc)0;
        // forces in FP64 where they are needed (reports, FP64 update)
        auto F = [&](int c) { return acc_value(w[c]); };
        double p[3] = {v.x[s], v.y[s], v.z[s]};
        double u[3] = {v.vx[s], v.vy[s], v.vz[s]};
        if (report) {
            int o = v.orig[s];
            double m = v.mass[s];
            if (v.mixed) {
                // the same estimate in FP32 from the stored 1/m (the FP64 pipe is
                // narrow on this GPU); the force word converts exactly in two parts
                float vh[3];
                const float kf = m > 0 ? (float)(v.invm[s] * (0.5 * dt)) : 0.0f;
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const long long wc = static_cast<long long>(w[c]);
                    const float fc = __int2float_rn((int)(wc >> 24)) * 0.00390625f +                   // 2^-8
                                     __uint2float_rn((unsigned)(wc & 0xffffff)) * 2.3283064365386963e-10f;  // 2^-32
                    vh[c] = fmaf(fc, kf, (float)u[c]);
                }
                kef = 0.5f * (float)m * fmaf(vh[0], vh[0], fmaf(vh[1], vh[1], vh[2] * vh[2]));
            } else {
                double vh[3] = {u[0], u[1], u[2]};
                if (m > 0) {
                    double invMass = 1.0 / m;
                    double half = 0.5 * dt;
#pragma unroll
                    for (int c = 0; c < 3; ++c) vh[c] += F(c) * invMass * half;
                }
                ke = 0.5 * m * (vh[0] * vh[0] + vh[1] * vh[1] + vh[2] * vh[2]);
            }
            // report 1: positions, velocities and forces; report 2: a frame
            // (positions only, into the frame buffer the view points at)
#pragma unroll
            for (int c = 0; c < 3; ++c) v.snap_x[3 * (size_t)o + c] = p[c];
            if (report == 1) {
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    v.snap_v[3 * (size_t)o + c] = u[c];
                    v.snap_f[3 * (size_t)o + c] = F(c);
                }
            }
        }
        double im = v.invm[s];
        if (im != 0.0 && v.mixed) {
            // fixed-point forces: v += (invm dt 2^-32) * word, one multiply-add per
            // component on the FP64 pipe (the order of the two scalings differs
            // from the FP64 engine's only in the last bit).  The wrap test
            // compares order-preserving integer keys of the doubles (the same
            // outcome as the FP64 comparison, off the narrow FP64 pipe); the
            // shift itself is FP64 and is taken only when an atom crosses.
            const double c0 = im * (dt * kForceUnscale);
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                u[c] = fma(c0, (double)w[c], u[c]);
                double q = fma(u[c], dt, p[c]);
                const long long kq = dkey(q);
                const int out = kq < S.lbkey[c] ? 1 : (kq > S.ubkey[c] ? -1 : 0);
                if (__builtin_expect(out != 0, 0)) q += out > 0 ? S.L[c] : -S.L[c];
                p[c] = q;
            }
            v.x[s] = p[0];
            v.y[s] = p[1];
            v.z[s] = p[2];
            v.vx[s] = u[0];
            v.vy[s] = u[1];
            v.vz[s] = u[2];
        } else if (im != 0.0) {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                u[c] += im * F(c) * dt;
                double q = p[c] + u[c] * dt;
                if (q < S.lb[c])
                    q += S.L[c];
                else if (q > S.ub[c])
                    q -= S.L[c];
                p[c] = q;
            }
            v.x[s] = p[0];
            v.y[s] = p[1];
            v.z[s] = p[2];
            v.vx[s] = u[0];
            v.vy[s] = u[1];
            v.vz[s] = u[2];
        }
        if (v.mixed) {
            // One exact fixed-point displacement per component (integer
            // instructions on the positions' bits) serves both the FP32 cell
            // offset (offset at the last rebuild + displacement since) and
            // the skin check; shifts and squares in FP32, which keeps this
            // kernel off the slow FP64 pipe except for the update itself.
            float4 r = v.oref[s];
            float d[3], d2 = 0.0f;
            const long long *xref40 = reinterpret_cast<const long long *>(v.xref);
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                d[c] = min_image40(fix40(p[c]) - xref40[(size_t)c * v.N + s], S.L40[c], S.halfL40[c]);
                d2 = fmaf(d[c], d[c], d2);
            }
            v.pf[s] = make_float4(r.x + d[0], r.y + d[1], r.z + d[2], r.w);
            // a hair under skin/2: FP32 rounding can only trigger a rebuild early
            if (v.skin_half2 > 0.0 && d2 > (float)v.skin_half2 * 0.99999f) atomicOr(&v.flags->skin_hit, 1);
        } else {
            if (v.skin_half2 > 0.0) {
                double d2 = 0.0;
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    double d = min_image(p[c] - v.xref[(size_t)c * v.N + s], S.L[c], S.halfL[c]);
                    d2 += d * d;
                }
                if (d2 > v.skin_half2) atomicOr(&v.flags->skin_hit, 1);
            }
            // FP64 accumulators can hold a non-finite sum; int64 ones cannot
            if (!(isfinite(F(0)) && isfinite(F(1)) && isfinite(F(2)))) atomicOr(&v.flags->error, ERR_NONFINITE);
        }
    }
    if (report) {
        if (v.mixed)
            energy_add_f(v.E, sys, E_KIN, kef);
        else
            energy_add(v.E, sys, E_KIN, ke);
    }
}

// Copy positions, velocities and (optionally) the accumulated forces to the
// original-order snapshot; forces are cleared after the copy.
template <typename Acc>
__global__ void k_export(DevView v, int with_forces) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= v.N) return;
    int o = v.orig[s];
    v.snap_x[3 * (size_t)o] = v.x[s];
    v.snap_x[3 * (size_t)o + 1] = v.y[s];
    v.snap_x[3 * (size_t)o + 2] = v.z[s];
    v.snap_v[3 * (size_t)o] = v.vx[s];
    v.snap_v[3 * (size_t)o + 1] = v.vy[s];
    v.snap_v[3 * (size_t)o + 2] = v.vz[s];
    if (with_forces) {
        Acc *ax = static_cast<Acc *>(v.fx) + s;
        Acc *ay = static_cast<Acc *>(v.fy) + s;
        Acc *az = static_cast<Acc *>(v.fz) + s;
        v.snap_f[3 * (size_t)o] = acc_value(*ax);
        v.snap_f[3 * (size_t)o + 1] = acc_value(*ay);
        v.snap_f[3 * (size_t)o + 2] = acc_value(*az);
        *ax = (Acc)0;
        *ay = (Acc)0;
        *az = (Acc)0;
    }
}

void launch_integrate(const DevView &v, double dt, int report, cudaStream_t st) {
    int nb = (v.N + 255) / 256;
    if (v.mixed)
        k_integrate<long long><<<nb, 256, 0, st>>>(v, dt, report);
    else
        k_integrate<double><<<nb, 256, 0, st>>>(v, dt, report);
}

void launch_export(const DevView &v, int with_forces, cudaStream_t st) {
    int nb = (v.N + 255) / 256;
    if (v.mixed)
        k_export<long long><<<nb, 256, 0, st>>>(v, with_forces);
    else
        k_export<double><<<nb, 256, 0, st>>>(v, with_forces);
}

void launch_snapshot_forces(const DevView &v, cudaStream_t st) { launch_export(v, 1, st); }

}  // namespace nxm
