// Harmonic bond, harmonic angle and periodic torsion forces: one thread per
// term over the flattened index [bonds | angles | torsions].
//
// Formulas and evaluation order follow the reference
// (core/baseline/src/Forces/HarmonicBondForce.cpp:20-58,
//  HarmonicAngleForce.cpp:19-63, PeriodicTorsionForce.cpp:41-149).
// Displacements are always formed from the FP64 positions with the
// reference's single-shift minimum image.  In mixed mode they are formed
// exactly in 2^-40 nm fixed point from the bits of the FP64 positions with
// integer instructions (fix40: this GPU's FP64 pipe is narrow) and rounded
// once to FP32 (the stiff bond terms cannot afford FP32 positions); the rest
// of the term is FP32 with FP32 parameters and int64 fixed-point force
// accumulation.
#include "nxm_pairterms.cuh"
#include "nxm_view.h"

namespace nxm {

template <typename R>
struct V3 {
    R x, y, z;
};

template <typename R>
__device__ __forceinline__ V3<R> mk(R x, R y, R z) {
    return V3<R>{x, y, z};
}
template <typename R>
__device__ __forceinline__ R dot(const V3<R> &a, const V3<R> &b) {
    return a.x * b.x + a.y * b.y + a.z * b.z;
}
template <typename R>
__device__ __forceinline__ V3<R> cross(const V3<R> &a, const V3<R> &b) {
    return mk<R>(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
template <typename R>
__device__ __forceinline__ V3<R> scale(const V3<R> &a, R s) {
    return mk<R>(a.x * s, a.y * s, a.z * s);
}

// minimumImageVector(p[a], p[b]) = p[a] - p[b], one shift per component
template <typename R>
__device__ __forceinline__ V3<R> disp(const DevView &v, const SysDev &S, int a, int b) {
    if (sizeof(R) == 4) {
        // exact fixed-point difference, integer minimum image, one rounding
        return mk<R>((R)min_image40(fix40(v.x[a]) - fix40(v.x[b]), S.L40[0], S.halfL40[0]),
                     (R)min_image40(fix40(v.y[a]) - fix40(v.y[b]), S.L40[1], S.halfL40[1]),
                     (R)min_image40(fix40(v.z[a]) - fix40(v.z[b]), S.L40[2], S.halfL40[2]));
    }
    double dx = min_image(v.x[a] - v.x[b], S.L[0], S.halfL[0]);
    double dy = min_image(v.y[a] - v.y[b], S.L[1], S.halfL[1]);
    double dz = min_image(v.z[a] - v.z[b], S.L[2], S.halfL[2]);
    return mk<R>((R)dx, (R)dy, (R)dz);
}

// A term's two parameters in the arithmetic's precision (FP32 copies made
// at set-up in mixed mode).
template <typename R>
__device__ __forceinline__ void term_prm(const double2 *p64, const float2 *p32, int k, R &a, R &b) {
    if (sizeof(R) == 4) {
        const float2 p = p32[k];
        a = (R)p.x;
        b = (R)p.y;
    } else {
        const double2 p = p64[k];
        a = (R)p.x;
        b = (R)p.y;
    }
}

template <typename Acc, typename R>
__device__ __forceinline__ void add_force(const DevView &v, int s, const V3<R> &f) {
    acc_add(static_cast<Acc *>(v.fx) + s, f.x);
    acc_add(static_cast<Acc *>(v.fy) + s, f.y);
    acc_add(static_cast<Acc *>(v.fz) + s, f.z);
}

template <typename R>
__device__ __forceinline__ R r_sqrt(R a);
template <>
__device__ __forceinline__ float r_sqrt<float>(float a) { return sqrtf(a); }
template <>
__device__ __forceinline__ double r_sqrt<double>(double a) { return sqrt(a); }
template <typename R>
__device__ __forceinline__ R r_acos(R a);
template <>
__device__ __forceinline__ float r_acos<float>(float a) { return acosf(a); }
template <>
__device__ __forceinline__ double r_acos<double>(double a) { return acos(a); }
template <typename R>
__device__ __forceinline__ R r_asin(R a);
template <>
__device__ __forceinline__ float r_asin<float>(float a) { return asinf(a); }
template <>
__device__ __forceinline__ double r_asin<double>(double a) { return asin(a); }
template <typename R>
__device__ __forceinline__ void r_sincos(R a, R *s, R *c);
template <>
__device__ __forceinline__ void r_sincos<float>(float a, float *s, float *c) { sincosf(a, s, c); }
template <>
__device__ __forceinline__ void r_sincos<double>(double a, double *s, double *c) { sincos(a, s, c); }

template <typename R>
__device__ __forceinline__ V3<R> normalized(const V3<R> &a) {
    R len = r_sqrt<R>(a.x * a.x + a.y * a.y + a.z * a.z);
    if (len > (R)0) return mk<R>(a.x / len, a.y / len, a.z / len);
    return mk<R>(0, 0, 0);
}

// One thread per term over [bonds | angles | torsions], followed, when
// `pairs` is set, by [excluded pairs | exception pairs] (nxm_pairterms.cuh):
// every per-term force of a step in one launch.
template <typename R, typename Acc>
__global__ void __launch_bounds__(256) k_bonded(DevView v, int energy, int pairs) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int nbt = v.nb + v.na + v.nt;
    const int nx = pairs ? v.nex : 0, nc = pairs ? v.nxc : 0;
    int total = nbt;
    R e = 0;  // this thread's term energy (mixed: FP32, summed as fixed point)
    int term = -1, sys = 0;
    if (t >= nbt && t < nbt + nx) {
        term = E_EXCL;
        e = exclusion_pair<sizeof(R) == 4>(v, t - nbt, sys);
    } else if (t >= nbt + nx && t < nbt + nx + nc) {
        term = E_EXCEPT;
        e = exception_pair<sizeof(R) == 4>(v, t - nbt - nx, sys);
    }
    if (t < total) {
        if (t < v.nb) {
            // HarmonicBondForce.cpp:20-58
            term = E_BOND;
            int2 b = v.bond_slot[t];
            R p0, p1;  // d, k
            term_prm<R>(v.bond_prm, v.bond_prmf, t, p0, p1);
            sys = v.sys_of[b.x];
            const SysDev &S = v.sys[sys];
            V3<R> d = disp<R>(v, S, b.y, b.x);
            R r = r_sqrt<R>(dot(d, d));
            R dI = r - p0;
            if (energy) e = (R)0.5 * p1 * dI * dI;
            R dEdR = p1 * dI;
            d = r > (R)0 ? scale(d, dEdR / r) : mk<R>(0, 0, 0);
            add_force<Acc>(v, b.x, d);
            add_force<Acc>(v, b.y, scale(d, (R)-1));
        } else if (t < v.nb + v.na) {
            // HarmonicAngleForce.cpp:19-63
            term = E_ANGLE;
            int k = t - v.nb;
            int4 a = v.angle_slot[k];
            R p0, p1;  // a, k
            term_prm<R>(v.angle_prm, v.angle_prmf, k, p0, p1);
            sys = v.sys_of[a.x];
            const SysDev &S = v.sys[sys];
            V3<R> v0 = disp<R>(v, S, a.y, a.x);
            V3<R> v1 = disp<R>(v, S, a.y, a.z);
            V3<R> cp = cross(v0, v1);
            R q21 = dot(v0, v0), q23 = dot(v1, v1);
            R r21 = r_sqrt<R>(q21), r23 = r_sqrt<R>(q23);
            R c = dot(v0, v1) / (r21 * r23);
            c = c < (R)-1 ? (R)-1 : (c > (R)1 ? (R)1 : c);
            R theta = r_acos<R>(c);
            R dI = theta - p0;
            if (energy) e = (R)0.5 * p1 * dI * dI;
            R dEdA = p1 * dI;
            R rp = r_sqrt<R>(dot(cp, cp));
            rp = rp < (R)1.0e-06 ? (R)1.0e-06 : rp;
            V3<R> f1 = scale(cross(v0, cp), dEdA / (q21 * rp));
            V3<R> f3 = scale(cross(cp, v1), dEdA / (q23 * rp));
            V3<R> f2 = mk<R>(-f1.x - f3.x, -f1.y - f3.y, -f1.z - f3.z);
            add_force<Acc>(v, a.x, f1);
            add_force<Acc>(v, a.y, f2);
            add_force<Acc>(v, a.z, f3);
        } else {
            // PeriodicTorsionForce.cpp:41-149
            term = E_TORSION;
            int k = t - v.nb - v.na;
            int4 a = v.tors_slot[k];
            R p0, p1;  // k, phase
            term_prm<R>(v.tors_prm, v.tors_prmf, k, p0, p1);
            int per = v.tors_per[k];
            sys = v.sys_of[a.x];
            const SysDev &S = v.sys[sys];
            V3<R> v0 = disp<R>(v, S, a.x, a.y);
            V3<R> v1 = disp<R>(v, S, a.z, a.y);
            V3<R> v2 = disp<R>(v, S, a.z, a.w);
            V3<R> cp0 = cross(v0, v1), cp1 = cross(v1, v2);
            R cosang = dot(normalized(cp0), normalized(cp1));
            R ang;
            const R lim = (R)0.99f;  // the reference compares with the float literal 0.99f
            if (cosang > lim || cosang < -lim) {
                V3<R> cr = cross(cp0, cp1);
                R sc = dot(cp0, cp0) * dot(cp1, cp1);
                ang = r_asin<R>(r_sqrt<R>(dot(cr, cr) / sc));
                if (cosang < (R)0) ang = (R)kPi - ang;
            } else {
                ang = r_acos<R>(cosang);
            }
            ang = dot(v0, cp1) >= (R)0 ? ang : -ang;
            R dA = (R)per * ang - p1;
            R sn, cs;
            r_sincos<R>(dA, &sn, &cs);
            if (energy) e = p0 * ((R)1 + cs);
            R dEdPhi = -p0 * (R)per * sn;
            R nc1 = dot(cp0, cp0), nbc2 = dot(v1, v1), nc2 = dot(cp1, cp1);
            R nbc = r_sqrt<R>(nbc2);
            R dp = (R)1 / nbc2;
            R f1s = (-dEdPhi * nbc) / nc1;
            R fac2 = dot(v0, v1) * dp;
            R fac3 = dot(v2, v1) * dp;
            R f4s = (dEdPhi * nbc) / nc2;
            V3<R> f1 = scale(cp0, f1s), f4 = scale(cp1, f4s);
            V3<R> s = mk<R>(f1.x * fac2 - f4.x * fac3, f1.y * fac2 - f4.y * fac3, f1.z * fac2 - f4.z * fac3);
            add_force<Acc>(v, a.x, f1);
            add_force<Acc>(v, a.y, mk<R>(s.x - f1.x, s.y - f1.y, s.z - f1.z));
            add_force<Acc>(v, a.z, mk<R>(-s.x - f4.x, -s.y - f4.y, -s.z - f4.z));
            add_force<Acc>(v, a.w, f4);
        }
    }
    if (energy) {
        // each energy term reduced separately (all lanes participate)
        for (int k = E_BOND; k <= E_TORSION; ++k) energy_add_t(v.E, sys, k, term == k ? e : (R)0);
        if (pairs) {
            energy_add_t(v.E, sys, E_EXCL, term == E_EXCL ? e : (R)0);
            energy_add_t(v.E, sys, E_EXCEPT, term == E_EXCEPT ? e : (R)0);
        }
    }
}

// pairs != 0: the exclusion correction and the exception pairs too (the
// caller passes it only when the nonbonded force is on)
int launch_bonded(const DevView &v, int energy, cudaStream_t st, int pairs) {
    int n = v.nb + v.na + v.nt + (pairs ? v.nex + v.nxc : 0);  // disabled kinds arrive with a zero count
    if (n == 0) return 0;
    int nb = (n + 255) / 256;
    if (v.mixed)
        k_bonded<float, long long><<<nb, 256, 0, st>>>(v, energy, pairs);
    else
        k_bonded<double, double><<<nb, 256, 0, st>>>(v, energy, pairs);
    return 1;
}

}  // namespace nxm
