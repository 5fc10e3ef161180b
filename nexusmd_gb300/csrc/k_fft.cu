// Batched 3-D FFT for PME, written for shared memory: every block loads a
// tile of lines of one system's grid, transforms each line with mixed-radix
// (4/2/3/5) Stockham auto-sort passes in shared memory, and stores it back.
//
// It replaces the reference's FFTW call (NonbondedForce.cpp:264-290: complex
// in place, forward sign -1, backward +1, unnormalised).  Because the charge
// grid is real and the influence function is even, the same numbers come from
// a real-to-complex transform on the half spectrum (kz <= K2/2) and a
// complex-to-real inverse, which halves the work and the traffic.  The
// convolution with the influence function and the reciprocal energy sum
// (NonbondedForce.cpp:323-388) are fused into the x pass between its forward
// and inverse transforms, so the spectrum never makes an extra trip to memory.
//
// Two launch shapes with the same arithmetic (bit for bit):
//  * plane path (3 kernels): one block per x-plane does the z transforms and
//    then the y transforms of that plane in shared memory (forward), the x
//    kernel convolves, one block per x-plane does y and then z (inverse);
//  * line path (5 kernels): z, y, x, y, z, each kernel over tiles of lines --
//    for planes too large for shared memory, and for the no-allocation entry.
// Every pass has its radix fixed at compile time and reads its twiddles from
// a shared-memory copy of the axis's table; lines in shared memory have an odd
// stride (in complex words) so that column accesses do not conflict on banks.
#include <algorithm>
#include <cstring>
#include <mutex>

#include "nxm_fft.h"
#include "nxm_view.h"

namespace nxm {

template <typename C>
struct Cx;
template <>
struct Cx<float2> {
    using R = float;
    static __host__ __device__ __forceinline__ float2 mk(float a, float b) { return make_float2(a, b); }
};
template <>
struct Cx<double2> {
    using R = double;
    static __host__ __device__ __forceinline__ double2 mk(double a, double b) { return make_double2(a, b); }
};

template <typename C>
__host__ __device__ __forceinline__ C cadd(C a, C b) { return Cx<C>::mk(a.x + b.x, a.y + b.y); }
template <typename C>
__host__ __device__ __forceinline__ C csub(C a, C b) { return Cx<C>::mk(a.x - b.x, a.y - b.y); }
template <typename C>
__host__ __device__ __forceinline__ C cmul(C a, C b) { return Cx<C>::mk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
// i * s * a
template <typename C>
__host__ __device__ __forceinline__ C cis(C a, typename Cx<C>::R s) { return Cx<C>::mk(-s * a.y, s * a.x); }
template <typename C>
__host__ __device__ __forceinline__ C cscale(C a, typename Cx<C>::R s) { return Cx<C>::mk(a.x * s, a.y * s); }

// Length-R DFT with root exp(sign * 2 pi i / R), R in {2, 3, 4, 5, 6, 8, 9,
// 10}: 2, 3, 4, 5 directly; 6, 8 and 10 as two DFTs of half the length on the
// even and odd inputs, the odd ones twiddled by exp(sign * 2 pi i k / R), then
// R/2 DFTs of length 2; 9 as three DFTs of length 3 on the inputs n = n1 mod
// 3, twiddled by exp(sign * 2 pi i n1 k / 9), then three DFTs of length 3 --
// one pass in registers instead of two through shared memory.
template <typename C, int R>
__host__ __device__ __forceinline__ void small_dft(C *v, typename Cx<C>::R s) {
    using T = typename Cx<C>::R;
    if constexpr (R == 9) {
        const T c1 = (T)0.76604444311897803520, s1 = (T)0.64278760968653932632;   // 40 degrees
        const T c2 = (T)0.17364817766693034885, s2 = (T)0.98480775301220805936;   // 80 degrees
        const T c4 = (T)-0.93969262078590838405, s4 = (T)0.34202014332566873304;  // 160 degrees
        C y[3][3];
#pragma unroll
        for (int g = 0; g < 3; ++g) {
#pragma unroll
            for (int j = 0; j < 3; ++j) y[g][j] = v[g + 3 * j];
            small_dft<C, 3>(y[g], s);
        }
        y[1][1] = cmul(y[1][1], Cx<C>::mk(c1, s * s1));
        y[1][2] = cmul(y[1][2], Cx<C>::mk(c2, s * s2));
        y[2][1] = cmul(y[2][1], Cx<C>::mk(c2, s * s2));
        y[2][2] = cmul(y[2][2], Cx<C>::mk(c4, s * s4));
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            C z[3] = {y[0][k], y[1][k], y[2][k]};
            small_dft<C, 3>(z, s);
#pragma unroll
            for (int j = 0; j < 3; ++j) v[k + 3 * j] = z[j];
        }
    } else if constexpr (R == 6 || R == 8 || R == 10) {
        constexpr int H = R / 2;
        C e[H], o[H];
#pragma unroll
        for (int k = 0; k < H; ++k) {
            e[k] = v[2 * k];
            o[k] = v[2 * k + 1];
        }
        small_dft<C, H>(e, s);
        small_dft<C, H>(o, s);
        if constexpr (R == 6) {
            const T h = (T)0.86602540378443864676;  // sqrt(3)/2
            o[1] = cmul(o[1], Cx<C>::mk((T)0.5, s * h));
            o[2] = cmul(o[2], Cx<C>::mk((T)-0.5, s * h));
        } else if constexpr (R == 8) {
            const T h = (T)0.70710678118654752440;  // sqrt(2)/2
            o[1] = cmul(o[1], Cx<C>::mk(h, s * h));
            o[2] = cis(o[2], s);
            o[3] = cmul(o[3], Cx<C>::mk(-h, s * h));
        } else {
            const T c1 = (T)0.80901699437494742410, s1 = (T)0.58778525229247312917;  // 36 degrees
            const T c2 = (T)0.30901699437494742410, s2 = (T)0.95105651629515357212;  // 72 degrees
            o[1] = cmul(o[1], Cx<C>::mk(c1, s * s1));
            o[2] = cmul(o[2], Cx<C>::mk(c2, s * s2));
            o[3] = cmul(o[3], Cx<C>::mk(-c2, s * s2));
            o[4] = cmul(o[4], Cx<C>::mk(-c1, s * s1));
        }
#pragma unroll
        for (int k = 0; k < H; ++k) {
            v[k] = cadd(e[k], o[k]);
            v[k + H] = csub(e[k], o[k]);
        }
    } else if (R == 2) {
        C a = v[0], b = v[1];
        v[0] = cadd(a, b);
        v[1] = csub(a, b);
    } else if (R == 4) {
        C a0 = cadd(v[0], v[2]), a1 = csub(v[0], v[2]);
        C b0 = cadd(v[1], v[3]), b1 = csub(v[1], v[3]);
        v[0] = cadd(a0, b0);
        v[2] = csub(a0, b0);
        v[1] = cadd(a1, cis(b1, s));
        v[3] = csub(a1, cis(b1, s));
    } else if (R == 3) {
        const T h = (T)0.86602540378443864676;  // sqrt(3)/2
        C t1 = cadd(v[1], v[2]);
        C t2 = cis(csub(v[1], v[2]), s * h);
        C m = csub(v[0], cscale(t1, (T)0.5));
        v[0] = cadd(v[0], t1);
        v[1] = cadd(m, t2);
        v[2] = csub(m, t2);
    } else {  // R == 5
        const T c1 = (T)0.30901699437494742410, c2 = (T)-0.80901699437494742410;
        const T s1 = (T)0.95105651629515357212, s2 = (T)0.58778525229247312917;
        C t1 = cadd(v[1], v[4]), t2 = cadd(v[2], v[3]);
        C t3 = csub(v[1], v[4]), t4 = csub(v[2], v[3]);
        C a1 = cadd(v[0], cadd(cscale(t1, c1), cscale(t2, c2)));
        C a2 = cadd(v[0], cadd(cscale(t1, c2), cscale(t2, c1)));
        C b1 = cis(cadd(cscale(t3, s1), cscale(t4, s2)), s);
        C b2 = cis(csub(cscale(t3, s2), cscale(t4, s1)), s);
        v[0] = cadd(v[0], cadd(t1, t2));
        v[1] = cadd(a1, b1);
        v[4] = csub(a1, b1);
        v[2] = cadd(a2, b2);
        v[3] = csub(a2, b2);
    }
}

// floor(a / d) for 0 <= a < 2^22 and d <= 2^12 from a precomputed 1/d:
// (a + 1/2)/d is at least 1/(2d) away from an integer, far more than the
// float rounding of the product.
__device__ __forceinline__ int quot(int a, float inv_d) { return (int)(((float)a + 0.5f) * inv_d); }

// One Stockham pass of radix R after sub-transforms of size Ns, over nl
// lines of length n; line l of the source starts at src + l*lds, of the
// destination at dst + l*ldd.  Butterfly j (n/R per line) takes the
// elements j + r n/R, twiddles them by W_n^(r (j mod Ns) n/(Ns R)) (`tw`
// holds W_n^t = exp(-2 pi i t / n); conjugated for the inverse), and writes
// (j div Ns) Ns R + (j mod Ns) + r Ns.
template <typename C, int R, bool INV>
__device__ __forceinline__ void stockham(const C *src, int lds, C *dst, int ldd, int nl, const FftPasses &P, int p,
                                         const C *tw) {
    using T = typename Cx<C>::R;
    const int m = P.m[p], Ns = P.Ns[p], step = P.step[p], tot = nl * m;
    const float inv_m = P.inv_m[p], inv_ns = P.inv_ns[p];
    for (int bi = threadIdx.x; bi < tot; bi += blockDim.x) {
        int l = quot(bi, inv_m), j = bi - l * m;
        int jq = quot(j, inv_ns), k = j - jq * Ns;
        const C *s = src + l * lds + j;
        C v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) v[r] = s[r * m];
        if (k) {
#pragma unroll
            for (int r = 1; r < R; ++r) {
                C w = tw[r * k * step];
                if (INV) w.y = -w.y;
                v[r] = cmul(v[r], w);
            }
        }
        small_dft<C, R>(v, (T)(INV ? 1 : -1));
        C *d = dst + l * ldd + jq * Ns * R + k;
#pragma unroll
        for (int r = 0; r < R; ++r) d[r * Ns] = v[r];
    }
}

// All passes of one axis over nl lines of length n.  Pass 0 reads `in`
// (line stride ldi); the passes then alternate between the scratch buffers
// s0 and s1 (stride lds), s0 first; the last pass writes `out` (stride ldo)
// when it is given.  `in` must not be s0; it may be s1 (it is dead after
// pass 0) and it may be `out` (a single pass then goes through s0 and is
// copied).  Returns the buffer holding the result and sets *ldr to its line
// stride.  Ends with a barrier.
template <typename C, bool INV>
__device__ C *line_fft(C *in, int ldi, C *out, int ldo, C *s0, C *s1, int lds, int n, int nl, const FftPasses &P,
                       const C *tw, int *ldr) {
    C *src = in;
    int ls = ldi;
    const int np = P.np;
    for (int p = 0; p < np; ++p) {
        C *dst = (p & 1) ? s1 : s0;
        int ld = lds;
        if (out && p == np - 1 && !(p == 0 && out == in)) {
            dst = out;
            ld = ldo;
        }
        switch (P.R[p]) {
            case 10: stockham<C, 10, INV>(src, ls, dst, ld, nl, P, p, tw); break;
            case 9: stockham<C, 9, INV>(src, ls, dst, ld, nl, P, p, tw); break;
            case 6: stockham<C, 6, INV>(src, ls, dst, ld, nl, P, p, tw); break;
            case 8: stockham<C, 8, INV>(src, ls, dst, ld, nl, P, p, tw); break;
            case 4: stockham<C, 4, INV>(src, ls, dst, ld, nl, P, p, tw); break;
            case 2: stockham<C, 2, INV>(src, ls, dst, ld, nl, P, p, tw); break;
            case 3: stockham<C, 3, INV>(src, ls, dst, ld, nl, P, p, tw); break;
            default: stockham<C, 5, INV>(src, ls, dst, ld, nl, P, p, tw); break;
        }
        __syncthreads();
        src = dst;
        ls = ld;
    }
    if (out && src != out) {
        const float inv_n = 1.0f / (float)n;
        for (int e = threadIdx.x; e < nl * n; e += blockDim.x) {
            int l = quot(e, inv_n), i = e - l * n;
            out[l * ldo + i] = src[l * ls + i];
        }
        __syncthreads();
        src = out;
        ls = ldo;
    }
    *ldr = ls;
    return src;
}

// Moves `total` elements, U per thread per round: the U loads of a round
// are all issued before the first is used, so a thread waits for one memory
// latency per round instead of one per element.  load(e) must be valid for
// every e < total (a round's tail reloads element total - 1); store(e, value)
// runs for e < total only.
template <int U, typename Load, typename Store>
__device__ __forceinline__ void rounds(int total, Load load, Store store) {
    const int bd = blockDim.x;
    for (int e0 = threadIdx.x; e0 < total; e0 += U * bd) {
        decltype(load(0)) val[U];
#pragma unroll
        for (int u = 0; u < U; ++u) val[u] = load(min(e0 + u * bd, total - 1));
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (e0 + u * bd < total) store(e0 + u * bd, val[u]);
    }
}
constexpr int kRounds = 4;

// Fixed-point grid word (int32, units of 2^-24) to float: one rounding, the
// same float as (float)((double)g * 2^-24).
__device__ __forceinline__ float grid_value(int g) { return __int2float_rn(g) * 5.9604644775390625e-08f; }
__device__ __forceinline__ double grid_value(double g) { return g; }

// Copies the twiddle table of length n at `off` into shared memory (the
// caller's next barrier publishes it).
template <typename C>
__device__ __forceinline__ void load_tw(C *dst, const DevView &v, int off, int n) {
    const C *src = static_cast<const C *>(v.twiddle) + off;
    for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i];
}

// One spectrum element's reciprocal energy f |s|^2 (halved for an element
// the half spectrum holds once) in fixed point, units of 1 / kEnergyScale.
// FP64 engine: in FP64.  Mixed: in FP32, and converted without the FP64 pipe
// (narrow on this GPU): a = e * 2^8 splits exactly into the integer-valued
// h = rint(a) and l = a - h in [-1/2, 1/2], so round(e * 2^28) =
// h * 2^20 + round(l * 2^20), valid for |e| < 2^23.
__device__ __forceinline__ long long element_energy(double f, double2 s, bool once) {
    const double wgt = once ? 0.5 * kEnergyScale : kEnergyScale;
    return __double2ll_rn(wgt * f * (s.x * s.x + s.y * s.y));
}
__device__ __forceinline__ long long element_energy(float f, float2 s, bool once) {
    static_assert(kEnergyScale == 268435456.0, "the split below assumes units of 2^-28");
    const float e = (once ? 0.5f : 1.0f) * f * fmaf(s.x, s.x, s.y * s.y);
    const float a = e * 256.0f;
    const float h = rintf(a);
    const float l = a - h;
    return ((long long)__float2int_rn(h) << 20) + (long long)__float2int_rn(l * 1048576.0f);
}

// ---- z forward on nc real line pairs: line pair p (real lines ya = 2p and
// ya + 1 of `acc`, row length K2; the second may not exist) becomes one
// complex line, and after the transform they are separated with
// X_a[k] = (Z[k] + conj Z[n-k]) / 2, X_b[k] = (Z[k] - conj Z[n-k]) / 2i.
// `put(p, k, Xa, Xb, has_b)` stores the half spectra.
template <typename C, typename Acc, typename Put>
__device__ __forceinline__ void z_forward(const Acc *acc, int nreal, int nc, int n, int Kh, C *a, C *b, int ld,
                                          const FftSysDev &F, const C *tw, Put put) {
    using T = typename Cx<C>::R;
    const float inv_n = 1.0f / (float)n, inv_kh = 1.0f / (float)Kh;
    rounds<kRounds>(
        nc * n,
        [&](int e) {
            int p = quot(e, inv_n), z = e - p * n;
            int la = 2 * p, lb = min(la + 1, nreal - 1);
            Acc ga = __ldcs(acc + (long long)la * n + z);
            Acc gb = __ldcs(acc + (long long)lb * n + z);
            return Cx<C>::mk((T)grid_value(ga), la + 1 < nreal ? (T)grid_value(gb) : (T)0);
        },
        [&](int e, C val) {
            int p = quot(e, inv_n);
            a[p * ld + e - p * n] = val;
        });
    __syncthreads();
    int ldr;
    C *res = line_fft<C, false>(a, ld, nullptr, 0, b, a, ld, n, nc, F.ax[2], tw, &ldr);
    for (int e = threadIdx.x; e < nc * Kh; e += blockDim.x) {
        int p = quot(e, inv_kh), k = e - p * Kh;
        C z = res[p * ldr + k];
        C zc = res[p * ldr + (k == 0 ? 0 : n - k)];
        put(p, k, Cx<C>::mk((T)0.5 * (z.x + zc.x), (T)0.5 * (z.y - zc.y)),
            Cx<C>::mk((T)0.5 * (z.y + zc.y), (T)0.5 * (zc.x - z.x)), 2 * p + 1 < nreal);
    }
    __syncthreads();
}

// ---- z inverse on nc line pairs: the Hermitian lines A = get(p, kk, 0) and
// B = get(p, kk, 1) (kk <= n/2, completed by conjugation above) are combined
// as Z = A + iB; the real and imaginary parts of the inverse transform are
// the real output lines 2p and 2p + 1 of `out` (row length n).
template <typename C, typename Get>
__device__ __forceinline__ void z_inverse(typename Cx<C>::R *out, int nreal, int nc, int n, int Kh, C *a, C *b, int ld,
                                          const FftSysDev &F, const C *tw, Get get) {
    using T = typename Cx<C>::R;
    const float inv_n = 1.0f / (float)n;
    rounds<kRounds>(
        nc * n,
        [&](int e) {
            int p = quot(e, inv_n), k = e - p * n;
            bool upper = k >= Kh;
            int kk = upper ? n - k : k;
            C A = get(p, kk, 0);
            C B = get(p, kk, 2 * p + 1 < nreal ? 1 : 0);
            if (2 * p + 1 >= nreal) B = Cx<C>::mk((T)0, (T)0);
            if (upper) {
                A.y = -A.y;
                B.y = -B.y;
            }
            return Cx<C>::mk(A.x - B.y, A.y + B.x);
        },
        [&](int e, C val) {
            int p = quot(e, inv_n);
            a[p * ld + e - p * n] = val;
        });
    __syncthreads();
    int ldr;
    C *res = line_fft<C, true>(a, ld, nullptr, 0, b, a, ld, n, nc, F.ax[2], tw, &ldr);
    for (int e = threadIdx.x; e < nc * n; e += blockDim.x) {
        int p = quot(e, inv_n), z = e - p * n;
        C r = res[p * ldr + z];
        out[(long long)(2 * p) * n + z] = r.x;
        if (2 * p + 1 < nreal) out[(long long)(2 * p + 1) * n + z] = r.y;
    }
    __syncthreads();
}

// ================= plane path: one block per (system, x) =================
// Shared memory: twiddles of y and z (twcap), the plane Q as Kh columns of
// length K1 with odd stride ldq (qcap), two scratch buffers of `scr` words.

template <typename C, typename Acc>
__global__ void __launch_bounds__(1024) k_fft_plane_fwd(DevView v, const FftSysDev *fs, const FftWork *work,
                                                        int twcap, int qcap, int scr) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *twy = reinterpret_cast<C *>(smem_raw);
    FftWork w = work[blockIdx.x];
    const FftSysDev &F = fs[w.sys];
    const int K1 = F.K[1], K2 = F.K[2], Kh = F.Kh, x = w.unit;
    const int ldq = K1 | 1, ldz = K2 | 1;
    C *twz = twy + K1;
    C *Q = twy + twcap;
    C *A = Q + qcap;
    C *B = A + scr;
    load_tw(twy, v, F.tw[1], K1);
    load_tw(twz, v, F.tw[2], K2);
    const Acc *acc = static_cast<const Acc *>(v.grid_acc) + F.roff + (long long)x * K1 * K2;
    const int npairs = (K1 + 1) >> 1, zc = min(npairs, scr / ldz);
    for (int p0 = 0; p0 < npairs; p0 += zc) {
        const int nc = min(zc, npairs - p0), y0 = 2 * p0;
        z_forward<C, Acc>(acc + (long long)y0 * K2, K1 - y0, nc, K2, Kh, A, B, ldz, F, twz,
                          [&](int p, int k, C xa, C xb, bool hb) {
                              Q[k * ldq + y0 + 2 * p] = xa;
                              if (hb) Q[k * ldq + y0 + 2 * p + 1] = xb;
                          });
    }
    const int cc = min(Kh, scr / ldq);
    for (int c0 = 0; c0 < Kh; c0 += cc) {
        int ldr;
        line_fft<C, false>(Q + c0 * ldq, ldq, Q + c0 * ldq, ldq, A, B, ldq, K1, min(cc, Kh - c0), F.ax[1], twy,
                           &ldr);
    }
    C *out = static_cast<C *>(v.grid_cplx) + F.coff + (long long)x * K1 * Kh;
    const float inv_kh = 1.0f / (float)Kh;
    for (int e = threadIdx.x; e < K1 * Kh; e += blockDim.x) {
        int y = quot(e, inv_kh), kz = e - y * Kh;
        out[e] = Q[kz * ldq + y];
    }
}

template <typename C>
__global__ void __launch_bounds__(1024) k_fft_plane_inv(DevView v, const FftSysDev *fs, const FftWork *work,
                                                        int twcap, int qcap, int scr) {
    using T = typename Cx<C>::R;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *twy = reinterpret_cast<C *>(smem_raw);
    FftWork w = work[blockIdx.x];
    const FftSysDev &F = fs[w.sys];
    const int K1 = F.K[1], K2 = F.K[2], Kh = F.Kh, x = w.unit;
    const int ldq = K1 | 1, ldz = K2 | 1;
    C *twz = twy + K1;
    C *Q = twy + twcap;
    C *A = Q + qcap;
    C *B = A + scr;
    load_tw(twy, v, F.tw[1], K1);
    load_tw(twz, v, F.tw[2], K2);
    const C *in = static_cast<const C *>(v.grid_cplx) + F.coff + (long long)x * K1 * Kh;
    const float inv_kh = 1.0f / (float)Kh;
    rounds<kRounds>(
        K1 * Kh, [&](int e) { return in[e]; },
        [&](int e, C val) {
            int y = quot(e, inv_kh);
            Q[(e - y * Kh) * ldq + y] = val;
        });
    __syncthreads();
    const int cc = min(Kh, scr / ldq);
    for (int c0 = 0; c0 < Kh; c0 += cc) {
        int ldr;
        line_fft<C, true>(Q + c0 * ldq, ldq, Q + c0 * ldq, ldq, A, B, ldq, K1, min(cc, Kh - c0), F.ax[1], twy,
                          &ldr);
    }
    T *out = static_cast<T *>(v.grid_real) + F.roff + (long long)x * K1 * K2;
    const int npairs = (K1 + 1) >> 1, zc = min(npairs, scr / ldz);
    for (int p0 = 0; p0 < npairs; p0 += zc) {
        const int nc = min(zc, npairs - p0), y0 = 2 * p0;
        z_inverse<C>(out + (long long)y0 * K2, K1 - y0, nc, K2, Kh, A, B, ldz, F, twz,
                     [&](int p, int kk, int second) { return Q[kk * ldq + y0 + 2 * p + second]; });
    }
}

// ================= line path: tiles of lines per block =================
// Shared memory: the axis's twiddles (kmax words), two line buffers.

// z forward: L real lines (L/2 complex) per block.
template <typename C, typename Acc>
__global__ void __launch_bounds__(256) k_fft_z_fwd(DevView v, const FftSysDev *fs, const FftWork *work, int L,
                                                   int kmax) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *tw = reinterpret_cast<C *>(smem_raw);
    FftWork w = work[blockIdx.x];
    const FftSysDev &F = fs[w.sys];
    const int n = F.K[2], Kh = F.Kh, ld = n | 1;
    const int l0 = w.unit * L, nl = min(L, F.K[0] * F.K[1] - l0);
    C *a = tw + kmax;
    C *b = a + (L >> 1) * ld;
    load_tw(tw, v, F.tw[2], n);
    const Acc *acc = static_cast<const Acc *>(v.grid_acc) + F.roff + (long long)l0 * n;
    C *out = static_cast<C *>(v.grid_cplx) + F.coff + (long long)l0 * Kh;
    z_forward<C, Acc>(acc, nl, (nl + 1) >> 1, n, Kh, a, b, ld, F, tw, [&](int p, int k, C xa, C xb, bool hb) {
        out[(long long)(2 * p) * Kh + k] = xa;
        if (hb) out[(long long)(2 * p + 1) * Kh + k] = xb;
    });
}

// y: columns of the half spectrum for fixed x, `cols` consecutive kz.
template <typename C, bool INV>
__global__ void __launch_bounds__(256) k_fft_y(DevView v, const FftSysDev *fs, const FftWork *work, int cols,
                                               int kmax) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *tw = reinterpret_cast<C *>(smem_raw);
    FftWork w = work[blockIdx.x];
    const FftSysDev &F = fs[w.sys];
    const int n = F.K[1], Kh = F.Kh, ld = n | 1;
    const int chunks = (Kh + cols - 1) / cols;
    const int x = w.unit / chunks, z0 = (w.unit - x * chunks) * cols;
    const int nc = min(cols, Kh - z0);
    C *a = tw + kmax;
    C *b = a + cols * ld;
    load_tw(tw, v, F.tw[1], n);
    C *g = static_cast<C *>(v.grid_cplx) + F.coff + (long long)x * F.K[1] * Kh + z0;
    const float inv_c = 1.0f / (float)nc;
    // smem line c holds column z0 + c
    rounds<kRounds>(
        n * nc,
        [&](int e) {
            int y = quot(e, inv_c);
            return g[(long long)y * Kh + e - y * nc];
        },
        [&](int e, C val) {
            int y = quot(e, inv_c);
            a[(e - y * nc) * ld + y] = val;
        });
    __syncthreads();
    int ldr;
    C *res = line_fft<C, INV>(a, ld, nullptr, 0, b, a, ld, n, nc, F.ax[1], tw, &ldr);
    for (int e = threadIdx.x; e < n * nc; e += blockDim.x) {
        int y = quot(e, inv_c), c = e - y * nc;
        g[(long long)y * Kh + c] = res[c * ldr + y];
    }
}

// x: forward, convolution with the influence function, energy, inverse.
// Used by both paths.
template <typename C, typename ET>
__global__ void __launch_bounds__(256) k_fft_x_conv(DevView v, const FftSysDev *fs, const FftWork *work, int cols,
                                                    int kmax, int energy) {
    using T = typename Cx<C>::R;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *tw = reinterpret_cast<C *>(smem_raw);
    FftWork w = work[blockIdx.x];
    const FftSysDev &F = fs[w.sys];
    const int n = F.K[0], K1 = F.K[1], Kh = F.Kh, ld = n | 1;
    const int chunks = (Kh + cols - 1) / cols;
    const int y = w.unit / chunks, z0 = (w.unit - y * chunks) * cols;
    const int nc = min(cols, Kh - z0);
    C *a = tw + kmax;
    C *b = a + cols * ld;
    load_tw(tw, v, F.tw[0], n);
    const long long xstride = (long long)K1 * Kh;
    C *g = static_cast<C *>(v.grid_cplx) + F.coff + (long long)y * Kh + z0;
    const float inv_c = 1.0f / (float)nc, inv_n = 1.0f / (float)n;
    rounds<kRounds>(
        n * nc,
        [&](int e) {
            int x = quot(e, inv_c);
            return g[x * xstride + e - x * nc];
        },
        [&](int e, C val) {
            int x = quot(e, inv_c);
            a[(e - x * nc) * ld + x] = val;
        });
    __syncthreads();
    int ldr;
    C *res = line_fft<C, false>(a, ld, nullptr, 0, b, a, ld, n, nc, F.ax[0], tw, &ldr);
    C *other = res == a ? b : a;
    const ET *et = static_cast<const ET *>(v.eterm) + F.coff + (long long)y * Kh + z0;
    // the energy in fixed point per element: its sum is the same whatever
    // the column blocking (an autotuned launch shape) groups together
    long long esum = 0;
    rounds<kRounds>(
        n * nc,
        [&](int e) {
            int c = quot(e, inv_n);
            return (T)et[(e - c * n) * xstride + c];
        },
        [&](int e, T f) {
            int c = quot(e, inv_n), kx = e - c * n;
            int kz = z0 + c;
            C s = res[c * ldr + kx];
            if (energy) {
                // half spectrum: planes kz = 0 and kz = K2/2 (even K2) appear
                // once; E = sum / 2
                const bool once = kz == 0 || 2 * kz == F.K[2];
                esum += element_energy(f, s, once);
            }
            res[c * ldr + kx] = Cx<C>::mk(s.x * f, s.y * f);
        });
    __syncthreads();
    C *fin = line_fft<C, true>(res, ldr, nullptr, 0, other, res, ld, n, nc, F.ax[0], tw, &ldr);
    for (int e = threadIdx.x; e < n * nc; e += blockDim.x) {
        int x = quot(e, inv_c), c = e - x * nc;
        g[x * xstride + c] = fin[c * ldr + x];
    }
    if (energy) energy_add_fixed(v.E, w.sys, E_RECIP, esum);
}

// z inverse: L real output lines per block.
template <typename C>
__global__ void __launch_bounds__(256) k_fft_z_inv(DevView v, const FftSysDev *fs, const FftWork *work, int L,
                                                   int kmax) {
    using T = typename Cx<C>::R;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *tw = reinterpret_cast<C *>(smem_raw);
    FftWork w = work[blockIdx.x];
    const FftSysDev &F = fs[w.sys];
    const int n = F.K[2], Kh = F.Kh, ld = n | 1;
    const int l0 = w.unit * L, nl = min(L, F.K[0] * F.K[1] - l0);
    C *a = tw + kmax;
    C *b = a + (L >> 1) * ld;
    load_tw(tw, v, F.tw[2], n);
    const C *in = static_cast<const C *>(v.grid_cplx) + F.coff + (long long)l0 * Kh;
    T *out = static_cast<T *>(v.grid_real) + F.roff + (long long)l0 * n;
    z_inverse<C>(out, nl, (nl + 1) >> 1, n, Kh, a, b, ld, F, tw,
                 [&](int p, int kk, int second) { return in[(long long)(2 * p + second) * Kh + kk]; });
}

template <typename C, typename Acc, typename ET>
static void run(const DevView &v, const FftPlan &p, int energy, cudaStream_t st) {
    if (p.nz == 0) return;
    if (p.plane) {
        k_fft_plane_fwd<C, Acc><<<p.npl, p.plane_threads, p.smem_plane, st>>>(v, p.dsys, p.pwork, p.twcap, p.qcap,
                                                                            p.scr);
        k_fft_x_conv<C, ET><<<p.nx, 256, p.smem_x, st>>>(v, p.dsys, p.xwork, p.cols, p.kmax, energy);
        k_fft_plane_inv<C><<<p.npl, p.plane_threads, p.smem_plane, st>>>(v, p.dsys, p.pwork, p.twcap, p.qcap, p.scr);
        return;
    }
    k_fft_z_fwd<C, Acc><<<p.nz, 256, p.smem_z, st>>>(v, p.dsys, p.zwork, p.zlines, p.kmax);
    k_fft_y<C, false><<<p.ny, 256, p.smem_y, st>>>(v, p.dsys, p.ywork, p.cols, p.kmax);
    k_fft_x_conv<C, ET><<<p.nx, 256, p.smem_x, st>>>(v, p.dsys, p.xwork, p.cols, p.kmax, energy);
    k_fft_y<C, true><<<p.ny, 256, p.smem_y, st>>>(v, p.dsys, p.ywork, p.cols, p.kmax);
    k_fft_z_inv<C><<<p.nz, 256, p.smem_z, st>>>(v, p.dsys, p.zwork, p.zlines, p.kmax);
}

void launch_fft_convolve(const DevView &v, const FftPlan &p, int energy, cudaStream_t st) {
    if (v.mixed)
        run<float2, int, float>(v, p, energy, st);
    else
        run<double2, double, double>(v, p, energy, st);
}

int fft_launch_count(const FftPlan &p) { return p.nz == 0 ? 0 : (p.plane ? 3 : 5); }

size_t fft_line_smem(int lines, int kmax, size_t csz) {
    return ((size_t)kmax + 2 * (size_t)lines * (size_t)(kmax | 1)) * csz;
}

void fft_passes(int n, FftPasses &P) {
    P = FftPasses{};
    int k = 0, rest = n;
    for (int r : {10, 9, 8, 6, 4, 2, 3, 5})
        while (rest % r == 0 && k < kMaxPasses) {
            P.R[k++] = r;
            rest /= r;
        }
    P.np = k;
    int Ns = 1;
    for (int p = 0; p < k; ++p) {
        P.Ns[p] = Ns;
        P.m[p] = n / P.R[p];
        P.step[p] = n / (Ns * P.R[p]);
        P.inv_m[p] = 1.0f / (float)P.m[p];
        P.inv_ns[p] = 1.0f / (float)Ns;
        Ns *= P.R[p];
    }
}

// Raises a kernel's dynamic shared-memory limit.  The limit is a per-kernel
// attribute shared by every context (and plan) of the process on a device:
// it is only ever raised, so a plan with smaller lines cannot lower it under
// another one.  `slot` names the kernel (one per kernel and precision).
static void raise_smem(const void *kernel, int slot, size_t bytes) {
    static std::mutex mu;
    static size_t seen[16][kMaxSmemDevices] = {};
    if (bytes <= 48 * 1024) return;  // launches up to 48 KB need no attribute
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= kMaxSmemDevices) dev = 0;
    std::lock_guard<std::mutex> lock(mu);
    if (bytes <= seen[slot][dev]) return;
    seen[slot][dev] = bytes;
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

template <typename C, typename Acc, typename ET>
static void raise_all(const FftPlan &p, int base) {
    raise_smem((const void *)k_fft_z_fwd<C, Acc>, base + 0, p.smem_z);
    raise_smem((const void *)k_fft_z_inv<C>, base + 1, p.smem_z);
    raise_smem((const void *)k_fft_y<C, false>, base + 2, p.smem_y);
    raise_smem((const void *)k_fft_y<C, true>, base + 3, p.smem_y);
    raise_smem((const void *)k_fft_x_conv<C, ET>, base + 4, p.smem_x);
    if (p.plane_ok) {
        raise_smem((const void *)k_fft_plane_fwd<C, Acc>, base + 5, p.smem_plane);
        raise_smem((const void *)k_fft_plane_inv<C>, base + 6, p.smem_plane);
    }
}

void fft_plan_build(FftPlan &p, int mixed, cudaStream_t st) {
    // sizes and factorizations (lengths must be 2^a 3^b 5^c, checked by the caller)
    std::vector<FftWork> z, y, x, pl;
    p.kmax = 0;
    int twcap = 0, qcap = 0, scr = 0, minscr = 0;
    for (int s = 0; s < p.S; ++s) {
        FftSysDev &F = p.hsys[s];
        for (int d = 0; d < 3; ++d) {
            fft_passes(F.K[d], F.ax[d]);
            if (F.K[d] > p.kmax) p.kmax = F.K[d];
        }
        int nzb = (F.K[0] * F.K[1] + p.zlines - 1) / p.zlines;
        for (int u = 0; u < nzb; ++u) z.push_back({s, u});
        int chunks = (F.Kh + p.cols - 1) / p.cols;
        for (int u = 0; u < F.K[0] * chunks; ++u) y.push_back({s, u});
        for (int u = 0; u < F.K[1] * chunks; ++u) x.push_back({s, u});
        for (int u = 0; u < F.K[0]; ++u) pl.push_back({s, u});
        // plane path geometry: whole-plane scratch when it fits
        int ldq = F.K[1] | 1, ldz = F.K[2] | 1;
        twcap = std::max(twcap, F.K[1] + F.K[2]);
        qcap = std::max(qcap, F.Kh * ldq);
        scr = std::max(scr, std::max(F.Kh * ldq, ((F.K[1] + 1) / 2) * ldz));
        minscr = std::max(minscr, std::max(ldq, ldz));
    }
    size_t csz = mixed ? sizeof(float2) : sizeof(double2);
    p.smem_z = fft_line_smem(p.zlines / 2, p.kmax, csz);
    p.smem_y = fft_line_smem(p.cols, p.kmax, csz);
    p.smem_x = p.smem_y;
    // the plane path keeps a plane and two scratch buffers in shared memory;
    // the scratch shrinks to a chunk of lines when the plane is large
    const size_t budget = 200 * 1024 / csz;
    p.twcap = (twcap + 1) & ~1;  // keeps the next region 16-byte aligned
    p.qcap = qcap;
    long long room = (long long)budget - p.twcap - p.qcap;
    p.scr = (int)std::min<long long>(scr, room / 2);
    p.plane_ok = p.S > 0 && p.scr >= minscr;
    p.plane_chunked = p.plane_ok && p.scr < scr;
    if (!p.plane_ok) p.plane = 0;
    p.smem_plane = ((size_t)p.twcap + p.qcap + 2 * (size_t)std::max(p.scr, 0)) * csz;
    // The per-system geometry and the work lists share one device buffer,
    // kept across rebuilds of the plan (the autotuner rebuilds it per
    // candidate) and grown when too small; they are copied in the order of
    // the stream that runs the transforms.
    p.nz = (int)z.size();
    p.ny = (int)y.size();
    p.nx = (int)x.size();
    p.npl = (int)pl.size();
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t bs = al(sizeof(FftSysDev) * std::max(p.S, 1)), bz = al(sizeof(FftWork) * (p.nz + 1)),
                 by = al(sizeof(FftWork) * (p.ny + 1)), bx = al(sizeof(FftWork) * (p.nx + 1)),
                 bp = al(sizeof(FftWork) * (p.npl + 1)), need = bs + bz + by + bx + bp;
    char *b = static_cast<char *>(p.ext);
    if (need > p.ext_cap || !p.ext) {
        if (need > p.cap || !p.buf) {
            cudaFree(p.buf);
            p.buf = nullptr;
            p.cap = 0;
            if (cudaMalloc(&p.buf, need) == cudaSuccess) p.cap = need;
        }
        b = static_cast<char *>(p.buf);
    }
    p.dsys = reinterpret_cast<FftSysDev *>(b);
    p.zwork = reinterpret_cast<FftWork *>(b + bs);
    p.ywork = reinterpret_cast<FftWork *>(b + bs + bz);
    p.xwork = reinterpret_cast<FftWork *>(b + bs + bz + by);
    p.pwork = reinterpret_cast<FftWork *>(b + bs + bz + by + bx);
    if (b) {
        // one copy from a host image of the buffer
        std::vector<char> img(need, 0);
        std::memcpy(img.data(), p.hsys.data(), sizeof(FftSysDev) * p.S);
        std::memcpy(img.data() + bs, z.data(), sizeof(FftWork) * p.nz);
        std::memcpy(img.data() + bs + bz, y.data(), sizeof(FftWork) * p.ny);
        std::memcpy(img.data() + bs + bz + by, x.data(), sizeof(FftWork) * p.nx);
        std::memcpy(img.data() + bs + bz + by + bx, pl.data(), sizeof(FftWork) * p.npl);
        cudaMemcpyAsync(b, img.data(), need, cudaMemcpyHostToDevice, st);
    }
    if (mixed)
        raise_all<float2, int, float>(p, 0);
    else
        raise_all<double2, double, double>(p, 8);
}

size_t fft_plan_bytes_max(const FftPlan &p) {
    // the smallest blockings any build uses: 8 real lines per z block, 4 columns
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    size_t nz = 0, ny = 0, nx = 0, npl = 0;
    for (int s = 0; s < p.S; ++s) {
        const FftSysDev &F = p.hsys[s];
        const int Kh = F.K[2] / 2 + 1, chunks = (Kh + 3) / 4;
        nz += (F.K[0] * F.K[1] + 7) / 8;
        ny += (size_t)F.K[0] * chunks;
        nx += (size_t)F.K[1] * chunks;
        npl += F.K[0];
    }
    return al(sizeof(FftSysDev) * std::max(p.S, 1)) + al(sizeof(FftWork) * (nz + 1)) +
           al(sizeof(FftWork) * (ny + 1)) + al(sizeof(FftWork) * (nx + 1)) + al(sizeof(FftWork) * (npl + 1));
}

void fft_plan_free(FftPlan &p) {
    cudaFree(p.buf);
    p.buf = nullptr;
    p.cap = 0;
    p.dsys = nullptr;
    p.zwork = p.ywork = p.xwork = p.pwork = nullptr;
}

}  // namespace nxm
