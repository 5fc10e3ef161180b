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
#include <mutex>

#include "nxm_fft.h"
#include "nxm_view.h"

namespace nxm {

template <typename C>
struct Cx;
template <>
struct Cx<float2> {
    using R = float;
    static __device__ __forceinline__ float2 mk(float a, float b) { return make_float2(a, b); }
};
template <>
struct Cx<double2> {
    using R = double;
    static __device__ __forceinline__ double2 mk(double a, double b) { return make_double2(a, b); }
};

template <typename C>
__device__ __forceinline__ C cadd(C a, C b) { return Cx<C>::mk(a.x + b.x, a.y + b.y); }
template <typename C>
__device__ __forceinline__ C csub(C a, C b) { return Cx<C>::mk(a.x - b.x, a.y - b.y); }
template <typename C>
__device__ __forceinline__ C cmul(C a, C b) { return Cx<C>::mk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
// i * s * a
template <typename C>
__device__ __forceinline__ C cis(C a, typename Cx<C>::R s) { return Cx<C>::mk(-s * a.y, s * a.x); }
template <typename C>
__device__ __forceinline__ C cscale(C a, typename Cx<C>::R s) { return Cx<C>::mk(a.x * s, a.y * s); }

// Length-R DFT with root exp(sign * 2 pi i / R), R in {2, 3, 4, 5}.
template <typename C>
__device__ __forceinline__ void small_dft(C *v, int R, typename Cx<C>::R s) {
    using T = typename Cx<C>::R;
    if (R == 2) {
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

// Transform `nlines` contiguous lines of length n held in a (scratch b);
// returns the buffer that holds the result.  Stockham pass with radix R after
// sub-transforms of size Ns: element j + r*n/R, twiddled by
// W_n^(r (j mod Ns) n/(Ns R)), goes to (j div Ns) Ns R + (j mod Ns) + r Ns.
template <typename C>
__device__ C *fft_lines(C *a, C *b, int n, int nlines, const int *rad, int np, const C *tw,
                        int sign) {
    using T = typename Cx<C>::R;
    int Ns = 1;
    for (int p = 0; p < np; ++p) {
        int R = rad[p];
        int m = n / R;
        int step = n / (Ns * R);
        int tot = nlines * m;
        const float inv_m = 1.0f / (float)m, inv_ns = 1.0f / (float)Ns;
        for (int bi = threadIdx.x; bi < tot; bi += blockDim.x) {
            int l = quot(bi, inv_m), j = bi - l * m;
            const C *src = a + l * n;
            C *dst = b + l * n;
            int jq = quot(j, inv_ns);
            int k = j - jq * Ns;
            C v[5];
#pragma unroll
            for (int r = 0; r < 5; ++r)
                if (r < R) v[r] = src[j + r * m];
#pragma unroll
            for (int r = 1; r < 5; ++r) {
                if (r < R && k) {
                    C w = tw[r * k * step];
                    if (sign > 0) w.y = -w.y;
                    v[r] = cmul(v[r], w);
                }
            }
            small_dft(v, R, (T)sign);
            int idx = jq * Ns * R + k;
#pragma unroll
            for (int r = 0; r < 5; ++r)
                if (r < R) dst[idx + r * Ns] = v[r];
        }
        __syncthreads();
        C *t = a;
        a = b;
        b = t;
        Ns *= R;
    }
    return a;
}

// Fixed-point grid word (units of 2^-32) to float without the FP64 pipe:
// g = hi * 2^24 + lo with lo in [0, 2^24) splits it into two floats that are
// exact (|g| < 2^47), and their sum is rounded once -- the same float as
// (float)((double)g * 2^-32).
__device__ __forceinline__ float grid_value(long long g) {
    float hi = __int2float_rn((int)(g >> 24)) * 0.00390625f;                         // * 2^-8
    float lo = __uint2float_rn((unsigned)(g & 0xffffff)) * 2.3283064365386963e-10f;  // * 2^-32
    return hi + lo;
}
__device__ __forceinline__ double grid_value(double g) { return g; }

template <typename C>
__device__ __forceinline__ const C *tw_table(const DevView &v, int off) {
    return static_cast<const C *>(v.twiddle) + off;
}

// ---- z: real -> half spectrum.  Reads the spread accumulator (fixed point
// in mixed mode; the spread launch clears it first).  Two real lines go through
// one complex transform (line 2p as the real part, 2p+1 as the imaginary
// part) and are separated with X_a[k] = (Z[k] + conj Z[n-k]) / 2,
// X_b[k] = (Z[k] - conj Z[n-k]) / 2i.
template <typename C, typename Acc>
__global__ void k_fft_z_fwd(DevView v, const FftSysDev *fs, const FftWork *work, int L) {
    using T = typename Cx<C>::R;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *a = reinterpret_cast<C *>(smem_raw);
    FftWork w = work[blockIdx.x];
    const FftSysDev &F = fs[w.sys];
    int n = F.K[2], Kh = F.Kh;
    int nl_total = F.K[0] * F.K[1];
    int l0 = w.unit * L;
    int nl = min(L, nl_total - l0);
    int np2 = (nl + 1) >> 1;  // complex lines
    C *b = a + (L >> 1) * n;
    const Acc *acc = static_cast<const Acc *>(v.grid_acc) + F.roff + (long long)l0 * n;
    for (int e = threadIdx.x; e < np2 * n; e += blockDim.x) {
        int p = e / n, z = e - p * n;
        int la = 2 * p, lb = 2 * p + 1;
        Acc ga = __ldcs(acc + (long long)la * n + z);
        Acc gb = lb < nl ? __ldcs(acc + (long long)lb * n + z) : (Acc)0;
        a[e] = Cx<C>::mk((T)grid_value(ga), (T)grid_value(gb));
    }
    __syncthreads();
    C *res = fft_lines(a, b, n, np2, F.rad[2], F.np[2], tw_table<C>(v, F.tw[2]), -1);
    C *out = static_cast<C *>(v.grid_cplx) + F.coff + (long long)l0 * Kh;
    for (int e = threadIdx.x; e < np2 * Kh; e += blockDim.x) {
        int p = e / Kh, k = e - p * Kh;
        C z = res[p * n + k];
        C zc = res[p * n + (k == 0 ? 0 : n - k)];
        // A = (z + conj zc)/2, B = (z - conj zc)/(2i)
        out[(long long)(2 * p) * Kh + k] = Cx<C>::mk((T)0.5 * (z.x + zc.x), (T)0.5 * (z.y - zc.y));
        if (2 * p + 1 < nl)
            out[(long long)(2 * p + 1) * Kh + k] = Cx<C>::mk((T)0.5 * (z.y + zc.y), (T)0.5 * (zc.x - z.x));
    }
}

// ---- y: columns of the half spectrum for fixed x, `cols` consecutive kz.
template <typename C>
__global__ void k_fft_y(DevView v, const FftSysDev *fs, const FftWork *work, int cols, int sign) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *a = reinterpret_cast<C *>(smem_raw);
    FftWork w = work[blockIdx.x];
    const FftSysDev &F = fs[w.sys];
    int n = F.K[1], Kh = F.Kh;
    int chunks = (Kh + cols - 1) / cols;
    int x = w.unit / chunks, z0 = (w.unit - x * chunks) * cols;
    int nc = min(cols, Kh - z0);
    C *b = a + cols * n;
    C *g = static_cast<C *>(v.grid_cplx) + F.coff + (long long)x * F.K[1] * Kh + z0;
    // smem line c holds column z0 + c
    for (int e = threadIdx.x; e < n * cols; e += blockDim.x) {
        int y = e / cols, c = e - y * cols;
        if (c < nc) a[c * n + y] = g[(long long)y * Kh + c];
    }
    __syncthreads();
    C *res = fft_lines(a, b, n, nc, F.rad[1], F.np[1], tw_table<C>(v, F.tw[1]), sign);
    for (int e = threadIdx.x; e < n * cols; e += blockDim.x) {
        int y = e / cols, c = e - y * cols;
        if (c < nc) g[(long long)y * Kh + c] = res[c * n + y];
    }
}

// ---- x: forward, convolution with the influence function, energy, inverse.
template <typename C, typename ET>
__global__ void k_fft_x_conv(DevView v, const FftSysDev *fs, const FftWork *work, int cols,
                             int energy) {
    using T = typename Cx<C>::R;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *a = reinterpret_cast<C *>(smem_raw);
    FftWork w = work[blockIdx.x];
    const FftSysDev &F = fs[w.sys];
    int n = F.K[0], K1 = F.K[1], Kh = F.Kh;
    int chunks = (Kh + cols - 1) / cols;
    int y = w.unit / chunks, z0 = (w.unit - y * chunks) * cols;
    int nc = min(cols, Kh - z0);
    C *b = a + cols * n;
    long long xstride = (long long)K1 * Kh;
    C *g = static_cast<C *>(v.grid_cplx) + F.coff + (long long)y * Kh + z0;
    for (int e = threadIdx.x; e < n * cols; e += blockDim.x) {
        int x = e / cols, c = e - x * cols;
        if (c < nc) a[c * n + x] = g[x * xstride + c];
    }
    __syncthreads();
    C *res = fft_lines(a, b, n, nc, F.rad[0], F.np[0], tw_table<C>(v, F.tw[0]), -1);
    C *other = res == a ? b : a;
    const ET *et = static_cast<const ET *>(v.eterm) + F.coff + (long long)y * Kh + z0;
    double esum = 0.0;
    for (int e = threadIdx.x; e < n * nc; e += blockDim.x) {
        int c = e / n, kx = e - c * n;
        int kz = z0 + c;
        T f = (T)et[kx * xstride + c];
        C s = res[c * n + kx];
        if (energy) {
            // half spectrum: planes kz = 0 and kz = K2/2 (even K2) appear once
            double wgt = (kz == 0 || 2 * kz == F.K[2]) ? 1.0 : 2.0;
            esum += wgt * (double)f * ((double)s.x * (double)s.x + (double)s.y * (double)s.y);
        }
        res[c * n + kx] = Cx<C>::mk(s.x * f, s.y * f);
    }
    __syncthreads();
    C *fin = fft_lines(res, other, n, nc, F.rad[0], F.np[0], tw_table<C>(v, F.tw[0]), +1);
    for (int e = threadIdx.x; e < n * cols; e += blockDim.x) {
        int x = e / cols, c = e - x * cols;
        if (c < nc) g[x * xstride + c] = fin[c * n + x];
    }
    if (energy) energy_add(v.E, w.sys, E_RECIP, 0.5 * esum);
}

// ---- z inverse: half spectrum -> real grid.  Two Hermitian lines A, B are
// completed and combined as Z = A + iB; the real and imaginary parts of the
// inverse transform are the two real output lines.
template <typename C>
__global__ void k_fft_z_inv(DevView v, const FftSysDev *fs, const FftWork *work, int L) {
    using T = typename Cx<C>::R;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *a = reinterpret_cast<C *>(smem_raw);
    FftWork w = work[blockIdx.x];
    const FftSysDev &F = fs[w.sys];
    int n = F.K[2], Kh = F.Kh;
    int nl_total = F.K[0] * F.K[1];
    int l0 = w.unit * L;
    int nl = min(L, nl_total - l0);
    int np2 = (nl + 1) >> 1;
    C *b = a + (L >> 1) * n;
    const C *in = static_cast<const C *>(v.grid_cplx) + F.coff + (long long)l0 * Kh;
    for (int e = threadIdx.x; e < np2 * n; e += blockDim.x) {
        int p = e / n, k = e - p * n;
        bool upper = k >= Kh;
        int kk = upper ? n - k : k;
        C A = in[(long long)(2 * p) * Kh + kk];
        C B = (2 * p + 1 < nl) ? in[(long long)(2 * p + 1) * Kh + kk] : Cx<C>::mk((T)0, (T)0);
        if (upper) {
            A.y = -A.y;
            B.y = -B.y;
        }
        a[e] = Cx<C>::mk(A.x - B.y, A.y + B.x);
    }
    __syncthreads();
    C *res = fft_lines(a, b, n, np2, F.rad[2], F.np[2], tw_table<C>(v, F.tw[2]), +1);
    T *out = static_cast<T *>(v.grid_real) + F.roff + (long long)l0 * n;
    for (int e = threadIdx.x; e < np2 * n; e += blockDim.x) {
        int p = e / n, z = e - p * n;
        C r = res[e];
        out[(long long)(2 * p) * n + z] = r.x;
        if (2 * p + 1 < nl) out[(long long)(2 * p + 1) * n + z] = r.y;
    }
}

template <typename C, typename Acc, typename ET>
static void run(const DevView &v, const FftPlan &p, int energy, cudaStream_t st) {
    if (p.nz == 0) return;
    k_fft_z_fwd<C, Acc><<<p.nz, 256, p.smem_z, st>>>(v, p.dsys, p.zwork, p.zlines);
    k_fft_y<C><<<p.ny, 256, p.smem_y, st>>>(v, p.dsys, p.ywork, p.cols, -1);
    k_fft_x_conv<C, ET><<<p.nx, 256, p.smem_x, st>>>(v, p.dsys, p.xwork, p.cols, energy);
    k_fft_y<C><<<p.ny, 256, p.smem_y, st>>>(v, p.dsys, p.ywork, p.cols, +1);
    k_fft_z_inv<C><<<p.nz, 256, p.smem_z, st>>>(v, p.dsys, p.zwork, p.zlines);
}

void launch_fft_convolve(const DevView &v, const FftPlan &p, int energy, cudaStream_t st) {
    if (v.mixed)
        run<float2, long long, float>(v, p, energy, st);
    else
        run<double2, double, double>(v, p, energy, st);
}

static void factor(int n, int *rad, int *np) {
    int k = 0;
    while (n % 4 == 0) { rad[k++] = 4; n /= 4; }
    while (n % 2 == 0) { rad[k++] = 2; n /= 2; }
    while (n % 3 == 0) { rad[k++] = 3; n /= 3; }
    while (n % 5 == 0) { rad[k++] = 5; n /= 5; }
    *np = k;
}

void fft_plan_build(FftPlan &p, int mixed) {
    // sizes and factorizations (lengths must be 2^a 3^b 5^c, checked by the caller)
    std::vector<FftWork> z, y, x;
    p.kmax = 0;
    for (int s = 0; s < p.S; ++s) {
        FftSysDev &F = p.hsys[s];
        for (int d = 0; d < 3; ++d) {
            factor(F.K[d], F.rad[d], &F.np[d]);
            if (F.K[d] > p.kmax) p.kmax = F.K[d];
        }
        int nzb = (F.K[0] * F.K[1] + p.zlines - 1) / p.zlines;
        for (int u = 0; u < nzb; ++u) z.push_back({s, u});
        int chunks = (F.Kh + p.cols - 1) / p.cols;
        for (int u = 0; u < F.K[0] * chunks; ++u) y.push_back({s, u});
        for (int u = 0; u < F.K[1] * chunks; ++u) x.push_back({s, u});
    }
    size_t csz = mixed ? sizeof(float2) : sizeof(double2);
    p.smem_z = 2 * (size_t)(p.zlines / 2) * p.kmax * csz;
    p.smem_y = 2 * (size_t)p.cols * p.kmax * csz;
    p.smem_x = p.smem_y;
    cudaMalloc(&p.dsys, sizeof(FftSysDev) * p.S);
    cudaMemcpy(p.dsys, p.hsys.data(), sizeof(FftSysDev) * p.S, cudaMemcpyHostToDevice);
    p.nz = (int)z.size();
    p.ny = (int)y.size();
    p.nx = (int)x.size();
    cudaMalloc(&p.zwork, sizeof(FftWork) * (p.nz + 1));
    cudaMalloc(&p.ywork, sizeof(FftWork) * (p.ny + 1));
    cudaMalloc(&p.xwork, sizeof(FftWork) * (p.nx + 1));
    cudaMemcpy(p.zwork, z.data(), sizeof(FftWork) * p.nz, cudaMemcpyHostToDevice);
    cudaMemcpy(p.ywork, y.data(), sizeof(FftWork) * p.ny, cudaMemcpyHostToDevice);
    cudaMemcpy(p.xwork, x.data(), sizeof(FftWork) * p.nx, cudaMemcpyHostToDevice);
    // The dynamic shared-memory limit is a per-kernel attribute shared by
    // every context (and plan) of the process on a device: only ever raise
    // it, so a plan with smaller lines cannot lower it under another one.
    static std::mutex mu;
    static int seen[2][kMaxSmemDevices] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= kMaxSmemDevices) dev = 0;
    int big = (int)(p.smem_z > p.smem_y ? p.smem_z : p.smem_y);
    std::lock_guard<std::mutex> lock(mu);
    // launches up to 48 KB need no attribute
    if (big <= 48 * 1024 || big <= seen[mixed ? 1 : 0][dev]) return;
    seen[mixed ? 1 : 0][dev] = big;
    if (mixed) {
        cudaFuncSetAttribute(k_fft_z_fwd<float2, long long>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
        cudaFuncSetAttribute(k_fft_y<float2>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
        cudaFuncSetAttribute(k_fft_x_conv<float2, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
        cudaFuncSetAttribute(k_fft_z_inv<float2>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
    } else {
        cudaFuncSetAttribute(k_fft_z_fwd<double2, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
        cudaFuncSetAttribute(k_fft_y<double2>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
        cudaFuncSetAttribute(k_fft_x_conv<double2, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
        cudaFuncSetAttribute(k_fft_z_inv<double2>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
    }
}

void fft_plan_free(FftPlan &p) {
    cudaFree(p.dsys);
    cudaFree(p.zwork);
    cudaFree(p.ywork);
    cudaFree(p.xwork);
    p.dsys = nullptr;
    p.zwork = p.ywork = p.xwork = nullptr;
}

}  // namespace nxm
