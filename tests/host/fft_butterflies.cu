// Host-side check of the FFT's building blocks (compiled and run by
// tests/test_fft_host.py, no GPU): every radix's register DFT against the
// direct DFT in FP64 and FP32, both directions, and the per-pass constants
// of the plan's factorisation for every length 2^a 3^b 5^c <= 1024.
#include <cmath>
#include <cstdio>
#include <random>

#include "../../nexusmd_gb300/csrc/k_fft.cu"

using namespace nxm;

template <int R, typename C, typename T>
static double dft_error(T s) {
    std::mt19937 g(R);
    std::uniform_real_distribution<double> u(-1, 1);
    C v[R];
    double x[R][2];
    for (int i = 0; i < R; ++i) {
        x[i][0] = u(g);
        x[i][1] = u(g);
        v[i] = Cx<C>::mk((T)x[i][0], (T)x[i][1]);
    }
    small_dft<C, R>(v, s);
    double err = 0;
    for (int k = 0; k < R; ++k) {
        double re = 0, im = 0;
        for (int n = 0; n < R; ++n) {
            double a = (double)s * 2 * M_PI * n * k / R;
            re += x[n][0] * std::cos(a) - x[n][1] * std::sin(a);
            im += x[n][0] * std::sin(a) + x[n][1] * std::cos(a);
        }
        err = std::fmax(err, std::fmax(std::fabs(re - (double)v[k].x), std::fabs(im - (double)v[k].y)));
    }
    return err;
}

template <int R>
static bool check_radix() {
    bool ok = true;
    for (double s : {-1.0, 1.0}) {
        double ed = dft_error<R, double2>(s), ef = dft_error<R, float2>((float)s);
        std::printf("radix %2d sign %+.0f: double %.2e float %.2e\n", R, s, ed, ef);
        ok = ok && ed < 1e-13 && ef < 2e-6;
    }
    return ok;
}

int main() {
    bool ok = check_radix<2>() && check_radix<3>() && check_radix<4>() && check_radix<5>() && check_radix<6>() &&
              check_radix<8>() && check_radix<9>() && check_radix<10>();
    int lengths = 0;
    for (int n = 1; n <= 1024; ++n) {
        int r = n;
        for (int p : {2, 3, 5})
            while (r % p == 0) r /= p;
        if (r != 1) continue;
        FftPasses P;
        fft_passes(n, P);
        long long prod = 1;
        for (int p = 0; p < P.np; ++p) {
            bool good = P.Ns[p] == prod && P.m[p] * P.R[p] == n && P.step[p] * P.Ns[p] * P.R[p] == n &&
                        P.inv_m[p] == 1.0f / (float)P.m[p] && P.inv_ns[p] == 1.0f / (float)P.Ns[p];
            if (!good) {
                std::printf("length %d pass %d: inconsistent constants\n", n, p);
                ok = false;
            }
            prod *= P.R[p];
        }
        if (prod != n) {
            std::printf("length %d: radices multiply to %lld\n", n, prod);
            ok = false;
        }
        ++lengths;
    }
    std::printf("%d lengths factorised\n%s\n", lengths, ok ? "OK" : "FAILED");
    return ok ? 0 : 1;
}
