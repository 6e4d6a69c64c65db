/*
 * fft64.c - FP64 mixed-radix FFT (recursive decimation in time, any length;
 * prime factors above 5 use a direct DFT in the combine step).
 * TEST INFRASTRUCTURE ONLY (oracle and reference emulation).
 *
 * It stands in for cuFFT, which the reference calls as a closed library
 * (cufftXtExecDescriptorC2C, ose_3d_lib.cu:668-820; cufftExecR2C/C2R,
 * ose_3d_lib.cu:578-581).  cuFFT's published contract is the unnormalised DFT
 * with sign -1 forward, +1 inverse; that is what this computes, in double.
 */
#include "fft64.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

int fft64_plan_init(fft64_plan* p, int n)
{
    memset(p, 0, sizeof(*p));
    if (n < 1) return -1;
    p->n = n;
    int m = n;
    while (m % 4 == 0) { p->fac[p->nf++] = 4; m /= 4; }
    while (m % 2 == 0) { p->fac[p->nf++] = 2; m /= 2; }
    for (int f = 3; m > 1; f += 2) {
        while (m % f == 0) { p->fac[p->nf++] = f; m /= f; }
        if (f * f > m && m > 1) { p->fac[p->nf++] = m; m = 1; }
    }
    p->tw = (double*)malloc(sizeof(double) * 2 * (size_t)n);
    if (!p->tw) return -1;
    for (int j = 0; j < n; ++j) {
        /* reduce the angle to [-pi/4, pi/4] octants for accuracy */
        double a = -2.0 * M_PI * (double)j / (double)n;
        p->tw[2 * j] = cos(a);
        p->tw[2 * j + 1] = sin(a);
    }
    return 0;
}

void fft64_plan_free(fft64_plan* p)
{
    free(p->tw);
    p->tw = NULL;
}

/* out[k] = sum_j in[j*is] * W^(j*k) for a sub-length n = N / tstride, where
 * W = exp(sign * 2 pi i / n) = tw[tstride]^(+-1). */
static void rec(const fft64_plan* p, const double* in, long is, double* out, int n,
                int fi, int sign, long tstride)
{
    if (n == 1) { out[0] = in[0]; out[1] = in[1]; return; }
    const int r = p->fac[fi];
    const int m = n / r;
    for (int q = 0; q < r; ++q)
        rec(p, in + 2 * q * is, is * r, out + 2 * (long)q * m, m, fi + 1, sign, tstride * r);
    const long N = p->n;
    double yr[64], yi[64];
    double* ybig = NULL;
    double *Yr = yr, *Yi = yi;
    if (r > 64) {
        ybig = (double*)malloc(sizeof(double) * 2 * r);
        Yr = ybig;
        Yi = ybig + r;
    }
    for (int k = 0; k < m; ++k) {
        for (int q = 0; q < r; ++q) {
            double a = out[2 * ((long)q * m + k)], b = out[2 * ((long)q * m + k) + 1];
            long e = ((long)q * k % n) * tstride % N;
            double c = p->tw[2 * e], s = sign < 0 ? p->tw[2 * e + 1] : -p->tw[2 * e + 1];
            Yr[q] = a * c - b * s;
            Yi[q] = a * s + b * c;
        }
        if (r == 2) {
            out[2 * k] = Yr[0] + Yr[1];
            out[2 * k + 1] = Yi[0] + Yi[1];
            out[2 * (k + m)] = Yr[0] - Yr[1];
            out[2 * (k + m) + 1] = Yi[0] - Yi[1];
        } else if (r == 4) {
            double t0r = Yr[0] + Yr[2], t0i = Yi[0] + Yi[2];
            double t1r = Yr[0] - Yr[2], t1i = Yi[0] - Yi[2];
            double t2r = Yr[1] + Yr[3], t2i = Yi[1] + Yi[3];
            double t3r = Yr[1] - Yr[3], t3i = Yi[1] - Yi[3];
            /* multiply t3 by -i*sign... W_4 = exp(sign*2pi i/4) = sign*i */
            double ur = sign < 0 ? t3i : -t3i;
            double ui = sign < 0 ? -t3r : t3r;
            out[2 * k] = t0r + t2r;          out[2 * k + 1] = t0i + t2i;
            out[2 * (k + m)] = t1r + ur;     out[2 * (k + m) + 1] = t1i + ui;
            out[2 * (k + 2 * m)] = t0r - t2r; out[2 * (k + 2 * m) + 1] = t0i - t2i;
            out[2 * (k + 3 * m)] = t1r - ur; out[2 * (k + 3 * m) + 1] = t1i - ui;
        } else {
            for (int s = 0; s < r; ++s) {
                double accr = 0.0, acci = 0.0;
                for (int q = 0; q < r; ++q) {
                    long e = ((long)q * s % r) * (N / r) % N;
                    double c = p->tw[2 * e], sn = sign < 0 ? p->tw[2 * e + 1] : -p->tw[2 * e + 1];
                    accr += Yr[q] * c - Yi[q] * sn;
                    acci += Yr[q] * sn + Yi[q] * c;
                }
                out[2 * (k + (long)s * m)] = accr;
                out[2 * (k + (long)s * m) + 1] = acci;
            }
        }
    }
    free(ybig);
}

void fft64_exec(const fft64_plan* p, double* data, int sign, double* work)
{
    const int n = p->n;
    memcpy(work, data, sizeof(double) * 2 * (size_t)n);
    rec(p, work, 1, data, n, 0, sign, 1);
}

static int axis_pass(double* d, int n0, int n1, int n2, int axis, int sign)
{
    int n = axis == 0 ? n0 : axis == 1 ? n1 : n2;
    long stride = axis == 0 ? 1 : axis == 1 ? n0 : (long)n0 * n1;
    long nlines = (long)n0 * n1 * n2 / n;
    fft64_plan plan;
    if (fft64_plan_init(&plan, n)) return -1;
    int err = 0;
#pragma omp parallel
    {
        double* line = (double*)malloc(sizeof(double) * 2 * (size_t)n);
        double* work = (double*)malloc(sizeof(double) * 4 * (size_t)n);
        if (!line || !work) {
#pragma omp atomic write
            err = 1;
        } else {
#pragma omp for schedule(static)
            for (long l = 0; l < nlines; ++l) {
                long base;
                if (axis == 0) base = l * n0;
                else if (axis == 1) base = (l / n0) * (long)n0 * n1 + (l % n0);
                else base = l;
                for (int j = 0; j < n; ++j) {
                    line[2 * j] = d[2 * (base + j * stride)];
                    line[2 * j + 1] = d[2 * (base + j * stride) + 1];
                }
                fft64_exec(&plan, line, sign, work);
                for (int j = 0; j < n; ++j) {
                    d[2 * (base + j * stride)] = line[2 * j];
                    d[2 * (base + j * stride) + 1] = line[2 * j + 1];
                }
            }
        }
        free(line);
        free(work);
    }
    fft64_plan_free(&plan);
    return err ? -1 : 0;
}

int fft64_3d(double* data, int n0, int n1, int n2, int sign)
{
    if (axis_pass(data, n0, n1, n2, 0, sign)) return -1;
    if (axis_pass(data, n0, n1, n2, 1, sign)) return -1;
    if (axis_pass(data, n0, n1, n2, 2, sign)) return -1;
    return 0;
}
