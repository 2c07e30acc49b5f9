// Host-side check of the PME DFT codelets (nb_fft.cuh): every radix transforms seeded complex
// inputs, in FP64 and FP32, and prints the largest deviation from a direct O(R^2) DFT summed
// in long double.  Built and run by test_fft_codelets.py.
#include <cmath>
#include <cstdio>
#include <cuda_runtime.h>

#include "nb_fft.cuh"

template <int R, typename C, typename T> double worst(unsigned seed)
{
    double err = 0.0;
    for (int trial = 0; trial < 64; ++trial) {
        C v[R];
        long double xr[R], xi[R];
        for (int n = 0; n < R; ++n) {
            seed = seed * 1664525u + 1013904223u;
            const T a = (T)((seed >> 8) * (1.0 / 16777216.0) - 0.5);
            seed = seed * 1664525u + 1013904223u;
            const T b = (T)((seed >> 8) * (1.0 / 16777216.0) - 0.5);
            v[n].x = a; v[n].y = b;
            xr[n] = a; xi[n] = b;
        }
        bfly<R>(v);
        for (int k = 0; k < R; ++k) {
            long double re = 0, im = 0;
            for (int n = 0; n < R; ++n) {
                const long double ang = -2.0L * 3.14159265358979323846264338327950288L * (long double)((n * k) % R) / R;
                re += xr[n] * cosl(ang) - xi[n] * sinl(ang);
                im += xr[n] * sinl(ang) + xi[n] * cosl(ang);
            }
            err = fmax(err, (double)fmaxl(fabsl(re - (long double)v[k].x), fabsl(im - (long double)v[k].y)));
        }
    }
    return err;
}

template <int R> void row()
{
    printf("%d %.3e %.3e\n", R, worst<R, double2, double>(12345u + R), worst<R, float2, float>(777u + R));
}

int main()
{
    row<2>(); row<3>(); row<4>(); row<5>(); row<6>(); row<8>(); row<9>(); row<10>();
    return 0;
}
