/*
 * fft64.h - FP64 complex FFT of any length, for the CPU oracle and for the
 * cuFFT stand-in of the reference emulation.  TEST INFRASTRUCTURE: only the
 * tests, the smoke check and bench.py's CPU baseline use it.
 *
 * Convention (cuFFT's): forward = sign -1, X[k] = sum_j x[j] exp(-2 pi i jk/n);
 * inverse = sign +1; neither is normalised.
 */
#ifndef OSE_FFT64_H
#define OSE_FFT64_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fft64_plan {
    int n;
    int nf;
    int fac[40];
    double* tw;     /* 2n doubles: exp(-2 pi i j / n), j < n */
} fft64_plan;

int fft64_plan_init(fft64_plan* p, int n);
void fft64_plan_free(fft64_plan* p);
/* In-place transform of n complex values (interleaved re, im). work holds 4n doubles. */
void fft64_exec(const fft64_plan* p, double* data, int sign, double* work);

/* 3-D transform of a [n2][n1][n0] array (n0 fastest), in place, all axes.
 * Uses every OpenMP thread. */
int fft64_3d(double* data, int n0, int n1, int n2, int sign);

#ifdef __cplusplus
}
#endif
#endif
