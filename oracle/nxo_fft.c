/*
 * Double-precision complex FFT for the CPU oracle (test infrastructure only).
 *
 * The reference transforms its PME grid with FFTW 3.3.5 (a closed Windows
 * binary that cannot be used here): in-place complex-to-complex, row-major
 * n0 x n1 x n2, FFTW_FORWARD = sign -1, FFTW_BACKWARD = sign +1, no
 * normalisation (core/baseline/src/Forces/NonbondedForce.cpp:264-290).
 * This file restates that documented transform from the DFT definition
 *     X[k] = sum_j x[j] exp(sign * 2 pi i j k / n)
 * with a recursive mixed-radix Cooley-Tukey decomposition (radix 2/3/4/5
 * butterflies, a plain O(p^2) DFT for any other prime factor) and twiddles
 * evaluated directly with cos/sin (no recurrences).
 *
 * It is compiled twice: into the oracle library, and (with NXO_FFTW_SHIM)
 * as a stand-in exporting fftw_plan_dft_3d / fftw_execute /
 * fftw_destroy_plan so the reference's own NonbondedForce.cpp links.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "nxo_fft.h"

#define NXO_PI 3.14159265358979323846

typedef struct {
    int n;
    int nf;
    int f[40];
    double *tw; /* tw[2j], tw[2j+1] = cos, sin of sign*2*pi*j/n */
    double *scratch;
} plan1d;

static void factorize(int n, int *f, int *nf) {
    int k = 0;
    while (n % 4 == 0) { f[k++] = 4; n /= 4; }
    while (n % 2 == 0) { f[k++] = 2; n /= 2; }
    for (int p = 3; n > 1; p += 2) {
        while (n % p == 0) { f[k++] = p; n /= p; }
    }
    *nf = k;
}

static void plan_init(plan1d *p, int n, int sign) {
    p->n = n;
    factorize(n, p->f, &p->nf);
    p->tw = (double *)malloc(sizeof(double) * 2 * (size_t)n);
    p->scratch = (double *)malloc(sizeof(double) * 2 * (size_t)n);
    for (int j = 0; j < n; ++j) {
        double a = sign * 2.0 * NXO_PI * (double)j / (double)n;
        p->tw[2 * j] = cos(a);
        p->tw[2 * j + 1] = sin(a);
    }
}

static void plan_free(plan1d *p) {
    free(p->tw);
    free(p->scratch);
}

/* out[0..n) = DFT_n of in[0], in[is], ... ; twiddle index stride ts into the full table */
static void rec(const double *in, int is, double *out, int n, const int *f, const double *tw,
                int ts, int N) {
    if (n == 1) {
        out[0] = in[0];
        out[1] = in[1];
        return;
    }
    int p = f[0];
    int m = n / p;
    for (int r = 0; r < p; ++r)
        rec(in + 2 * (size_t)r * is, is * p, out + 2 * (size_t)r * m, m, f + 1, tw, ts * p, N);
    double t[2 * 64];
    double *tp = t;
    double *heap = NULL;
    if (p > 64) {
        heap = (double *)malloc(sizeof(double) * 2 * (size_t)p);
        tp = heap;
    }
    for (int k = 0; k < m; ++k) {
        /* twiddle the p sub-results */
        for (int r = 0; r < p; ++r) {
            double xr = out[2 * ((size_t)r * m + k)], xi = out[2 * ((size_t)r * m + k) + 1];
            long idx = ((long)r * k * ts) % N;
            double wr = tw[2 * idx], wi = tw[2 * idx + 1];
            tp[2 * r] = xr * wr - xi * wi;
            tp[2 * r + 1] = xr * wi + xi * wr;
        }
        /* length-p DFT with the root W_p = tw[N/p] */
        if (p == 2) {
            out[2 * k] = tp[0] + tp[2];
            out[2 * k + 1] = tp[1] + tp[3];
            out[2 * (k + m)] = tp[0] - tp[2];
            out[2 * (k + m) + 1] = tp[1] - tp[3];
        } else if (p == 4) {
            /* W_4 = tw[N/4] = (0, sign) */
            double s = tw[2 * (N / 4) + 1];
            double a0r = tp[0] + tp[4], a0i = tp[1] + tp[5];
            double a1r = tp[0] - tp[4], a1i = tp[1] - tp[5];
            double b0r = tp[2] + tp[6], b0i = tp[3] + tp[7];
            double b1r = tp[2] - tp[6], b1i = tp[3] - tp[7];
            /* (b1) * (0 + i s) = (-s b1i, s b1r) */
            out[2 * k] = a0r + b0r;
            out[2 * k + 1] = a0i + b0i;
            out[2 * (k + m)] = a1r - s * b1i;
            out[2 * (k + m) + 1] = a1i + s * b1r;
            out[2 * (k + 2 * m)] = a0r - b0r;
            out[2 * (k + 2 * m) + 1] = a0i - b0i;
            out[2 * (k + 3 * m)] = a1r + s * b1i;
            out[2 * (k + 3 * m) + 1] = a1i - s * b1r;
        } else {
            for (int q = 0; q < p; ++q) {
                double sr = 0.0, si = 0.0;
                for (int r = 0; r < p; ++r) {
                    long idx = ((long)r * q % p) * (N / p);
                    double wr = tw[2 * idx], wi = tw[2 * idx + 1];
                    sr += tp[2 * r] * wr - tp[2 * r + 1] * wi;
                    si += tp[2 * r] * wi + tp[2 * r + 1] * wr;
                }
                out[2 * ((size_t)k + (size_t)q * m)] = sr;
                out[2 * ((size_t)k + (size_t)q * m) + 1] = si;
            }
        }
    }
    free(heap);
}

static void exec1d(plan1d *p, double *line /* in place, contiguous */) {
    memcpy(p->scratch, line, sizeof(double) * 2 * (size_t)p->n);
    rec(p->scratch, 1, line, p->n, p->f, p->tw, 1, p->n);
}

void nxo_fft1d(double *data, int n, int sign) {
    plan1d p;
    plan_init(&p, n, sign);
    exec1d(&p, data);
    plan_free(&p);
}

void nxo_fft3d(double *data, int n0, int n1, int n2, int sign) {
    int dims[3] = {n0, n1, n2};
    size_t strides[3] = {(size_t)n1 * n2, (size_t)n2, 1};
    int nmax = n0 > n1 ? (n0 > n2 ? n0 : n2) : (n1 > n2 ? n1 : n2);
    double *line = (double *)malloc(sizeof(double) * 2 * (size_t)nmax);
    for (int ax = 2; ax >= 0; --ax) {
        plan1d p;
        plan_init(&p, dims[ax], sign);
        int a1 = (ax + 1) % 3, a2 = (ax + 2) % 3;
        for (int i = 0; i < dims[a1]; ++i) {
            for (int j = 0; j < dims[a2]; ++j) {
                size_t base = (size_t)i * strides[a1] + (size_t)j * strides[a2];
                for (int k = 0; k < dims[ax]; ++k) {
                    line[2 * k] = data[2 * (base + (size_t)k * strides[ax])];
                    line[2 * k + 1] = data[2 * (base + (size_t)k * strides[ax]) + 1];
                }
                exec1d(&p, line);
                for (int k = 0; k < dims[ax]; ++k) {
                    data[2 * (base + (size_t)k * strides[ax])] = line[2 * k];
                    data[2 * (base + (size_t)k * strides[ax]) + 1] = line[2 * k + 1];
                }
            }
        }
        plan_free(&p);
    }
    free(line);
}

#ifdef NXO_FFTW_SHIM
/* The three FFTW entry points NonbondedForce.cpp:271-289 calls. */
typedef double fftw_complex[2];
struct fftw_plan_s {
    int n0, n1, n2, sign;
    fftw_complex *in, *out;
};
typedef struct fftw_plan_s *fftw_plan;

fftw_plan fftw_plan_dft_3d(int n0, int n1, int n2, fftw_complex *in, fftw_complex *out, int sign,
                           unsigned flags) {
    (void)flags;
    fftw_plan p = (fftw_plan)malloc(sizeof(struct fftw_plan_s));
    p->n0 = n0;
    p->n1 = n1;
    p->n2 = n2;
    p->sign = sign;
    p->in = in;
    p->out = out;
    return p;
}

void fftw_execute(const fftw_plan p) {
    size_t n = (size_t)p->n0 * p->n1 * p->n2;
    if (p->out != p->in) memcpy(p->out, p->in, sizeof(fftw_complex) * n);
    nxo_fft3d((double *)p->out, p->n0, p->n1, p->n2, p->sign);
}

void fftw_destroy_plan(fftw_plan p) { free(p); }
#endif
