/* Double-precision complex FFT used by the CPU oracle (test infrastructure). */
#ifndef NXO_FFT_H
#define NXO_FFT_H
#ifdef __cplusplus
extern "C" {
#endif
/* In-place unnormalised 1-D / 3-D (row-major n0 x n1 x n2) DFT of interleaved
 * (re, im) doubles; sign -1 = forward, +1 = backward (FFTW's convention). */
void nxo_fft1d(double *data, int n, int sign);
void nxo_fft3d(double *data, int n0, int n1, int n2, int sign);
#ifdef __cplusplus
}
#endif
#endif
