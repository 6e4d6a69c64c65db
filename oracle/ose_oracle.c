/*
 * ose_oracle.c - FP64 CPU restatement of the reference's OSE modeling loop.
 *
 * TEST INFRASTRUCTURE (the checker, and the timed CPU baseline of bench.py).
 * The product library never links or calls this file.
 *
 * Restated from Littleke/3D-OSE:
 *   ose_3d.cu:85-122, 191-199      sizes, dk, R, dtR, M
 *   ose_3d_lib.cu:36-44             judge_odd
 *   ose_3d_lib.cu:887-1032          model read and sponge padding
 *   ose_3d_kernel.cu:3-13           Ricker
 *   ose_3d_kernel.cu:154-172 + ose_3d_lib.cu:578-581   Hilbert trace
 *   ose_3d_kernel.cu:242-261        sponge profile
 *   ose_3d_lib.cu:639-874           wavefield_extro_ori2, the time step
 *   ose_3d_kernel.cu:101-126, 345-359, 379-390, 263-288   |k|, v/R/N, Bessel, sponge
 *   ose_3d_kernel.cu:291-297, 412-436; ose_3d_lib.cu:610-633, 876-884   source, receivers
 *
 * Differences from the reference that are NOT rounding:
 *   - The reference transforms the p and q parts separately, each as a C2C
 *     transform of a real field (zero imaginary part).  The operator is real
 *     (|k| is even in k), so one transform of the packed p + i q gives both
 *     results exactly; this file does that.
 *   - Everything is double.  The reference mixes float fields with float
 *     Bessel values jnf(n, dtR) evaluated per element.
 */
#include "ose_oracle.h"
#include "fft64.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

int orc_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* judge_odd: bump the trailing pad when the padded size is odd. */
static void judge_odd(int* after, int* nb)
{
    if (*nb % 2 != 0) { *after += 1; *nb += 1; }
}

int orc_derive_dims(const ose_params* p, ose_derived* d)
{
    if (!p || !d) return -1;
    if (p->nx < 1 || p->ny < 1 || p->nz < 1) return -1;
    memset(d, 0, sizeof(*d));
    d->br = p->br; d->bb = p->bb; d->bd = p->bd;
    d->nxb = p->bl + p->nx + p->br;
    d->nyb = p->bf + p->ny + p->bb;
    d->nzb = p->bu + p->nz + p->bd;
    judge_odd(&d->br, &d->nxb);
    judge_odd(&d->bb, &d->nyb);
    judge_odd(&d->bd, &d->nzb);
    d->ng = p->nx * p->ny;
    d->dkx = 2.0 * M_PI / p->dx / (double)d->nxb;
    d->dky = 2.0 * M_PI / p->dy / (double)d->nyb;
    d->dkz = 2.0 * M_PI / p->dz / (double)d->nzb;
    return 0;
}

static int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

/* The padding loops of add_pml_layers_v_h (ose_3d_lib.cu:912-1032) copy the
 * nearest interior cell along x, then y, then z into the sponge; the result
 * is the interior value at the clamped coordinates. */
int orc_pad_model(const ose_params* p, const float* vel, float* vb)
{
    ose_derived d;
    if (orc_derive_dims(p, &d)) return -1;
    const int nx = p->nx, ny = p->ny, nz = p->nz;
    for (int z = 0; z < d.nzb; ++z)
        for (int y = 0; y < d.nyb; ++y)
            for (int x = 0; x < d.nxb; ++x) {
                int ix = clampi(x - p->bl, 0, nx - 1);
                int iy = clampi(y - p->bf, 0, ny - 1);
                int iz = clampi(z - p->bu, 0, nz - 1);
                vb[((long)z * d.nyb + y) * d.nxb + x] = vel[((long)ix * ny + iy) * nz + iz];
            }
    return 0;
}

int orc_series(const ose_params* p, float vmax, double* R, double* dtR, int* M)
{
    double r = (double)vmax * M_PI *
               sqrt(pow(1.0 / p->dx, 2.0) + pow(1.0 / p->dy, 2.0) + pow(1.0 / p->dz, 2.0));
    float rf = (float)r;             /* R is a float global in the reference */
    float dtrf = p->dt * rf;         /* dtR = dt*R in float                  */
    *R = r;
    *dtR = (double)p->dt * r;
    *M = p->M_override > 0 ? p->M_override : (int)dtrf + 6;
    return 0;
}

int orc_sponge(int before, int nn, int after, int mode, float factor, float* out)
{
    if (before < 0 || nn < 0 || after < 0) return -1;
    for (int i = 0; i < before; ++i) {
        if (mode == OSE_SPONGE_CERJAN) {
            double t = (double)factor * (double)(before - i);
            out[i] = (float)exp(-t * t);
        } else {
            double t = (float)(before - 1 - i) / (float)before;
            out[i] = (float)exp(-t * t);
        }
    }
    for (int i = before; i < before + nn; ++i) out[i] = 1.0f;
    for (int i = 0; i < after; ++i) {
        if (mode == OSE_SPONGE_CERJAN) {
            double t = (double)factor * (double)(i + 1);
            out[before + nn + i] = (float)exp(-t * t);
        } else {
            double t = (float)(i + 1) / (float)after;
            out[before + nn + i] = (float)exp(-t * t);
        }
    }
    return 0;
}

int orc_ricker(int nt, float fm, float dt, float amp, float* out)
{
    for (int i = 0; i < nt; ++i) {
        double t = M_PI * fm * ((double)(i - 40) * dt - 1.0 / fm);
        t = t * t;
        out[i] = (float)((double)amp * (1.0 - 2.0 * t) * exp(-t));
    }
    return 0;
}

/* R2C spectrum of the Ricker, bins k < nt/2 times -i, bins k >= nt/2 times +i
 * (hilbert_1d's test is tx < nt/2), then an unnormalised Hermitian C2R.  The
 * DC and (even nt) Nyquist bins become purely imaginary and drop out. */
int orc_hilbert(const float* w, int nt, int div_nt, float* out)
{
    int nb = nt / 2 + 1;
    double* xr = (double*)calloc((size_t)nb, sizeof(double));
    double* xi = (double*)calloc((size_t)nb, sizeof(double));
    if (!xr || !xi) { free(xr); free(xi); return -1; }
    for (int k = 0; k < nb; ++k) {
        double sr = 0, si = 0;
        for (int j = 0; j < nt; ++j) {
            long e = ((long)j * k) % nt;
            double a = -2.0 * M_PI * (double)e / nt;
            sr += w[j] * cos(a);
            si += w[j] * sin(a);
        }
        /* multiply by -i (k < nt/2) or +i */
        if (k < nt / 2) { xr[k] = si; xi[k] = -sr; }
        else { xr[k] = -si; xi[k] = sr; }
    }
    int kmax = (nt % 2 == 0) ? nt / 2 - 1 : (nt - 1) / 2;
    for (int n = 0; n < nt; ++n) {
        double acc = xr[0];
        if (nt % 2 == 0) acc += xr[nt / 2] * ((n % 2) ? -1.0 : 1.0);
        for (int k = 1; k <= kmax; ++k) {
            long e = ((long)k * n) % nt;
            double a = 2.0 * M_PI * (double)e / nt;
            acc += 2.0 * (xr[k] * cos(a) - xi[k] * sin(a));
        }
        out[n] = (float)(div_nt ? acc / nt : acc);
    }
    free(xr);
    free(xi);
    return 0;
}

int orc_bessel(int M, double dtR, double* J)
{
    for (int n = 0; n <= M + 1; ++n) J[n] = jn(n, dtR);
    return 0;
}

/* scale_kxkz_3D's wrapped wavenumber (ose_3d_kernel.cu:109-120). */
static double kwrap(int i, int n, double dk)
{
    return dk * (double)(i > n / 2 ? n - i : i);
}

int orc_apply_operator(const ose_params* p, const float* vb, double R,
                       const double* in, double* out)
{
    ose_derived d;
    if (orc_derive_dims(p, &d)) return -1;
    const int nxb = d.nxb, nyb = d.nyb, nzb = d.nzb;
    const long N = (long)nxb * nyb * nzb;
    if (out != in) memcpy(out, in, sizeof(double) * 2 * (size_t)N);
    if (fft64_3d(out, nxb, nyb, nzb, -1)) return -1;
#pragma omp parallel for schedule(static)
    for (int z = 0; z < nzb; ++z) {
        double kz = kwrap(z, nzb, d.dkz);
        for (int y = 0; y < nyb; ++y) {
            double ky = kwrap(y, nyb, d.dky);
            for (int x = 0; x < nxb; ++x) {
                double kx = kwrap(x, nxb, d.dkx);
                double k = sqrt(kx * kx + ky * ky + kz * kz);
                long id = ((long)z * nyb + y) * nxb + x;
                out[2 * id] *= k;
                out[2 * id + 1] *= k;
            }
        }
    }
    if (fft64_3d(out, nxb, nyb, nzb, +1)) return -1;
    const double s = 1.0 / (R * (double)N);
#pragma omp parallel for schedule(static)
    for (long id = 0; id < N; ++id) {
        double f = (double)vb[id] * s;
        out[2 * id] *= f;
        out[2 * id + 1] *= f;
    }
    return 0;
}

int orc_run(const ose_params* p, const float* vel, int is, int it0, int nsteps,
            double* P, double* Q, float* gather)
{
    ose_derived d;
    if (orc_derive_dims(p, &d)) return -1;
    if (it0 < 0 || nsteps < 0 || it0 + nsteps > p->nt) return -1;
    const int nxb = d.nxb, nyb = d.nyb, nzb = d.nzb;
    const long N = (long)nxb * nyb * nzb;
    const int nx = p->nx, ny = p->ny;
    int rc = -1;

    float* vb = (float*)malloc(sizeof(float) * N);
    float* ax = (float*)malloc(sizeof(float) * nxb);
    float* ay = (float*)malloc(sizeof(float) * nyb);
    float* az = (float*)malloc(sizeof(float) * nzb);
    float* ricker = (float*)malloc(sizeof(float) * p->nt);
    float* hil = (float*)malloc(sizeof(float) * p->nt);
    double* A0 = (double*)malloc(sizeof(double) * 2 * N);
    double* A1 = (double*)malloc(sizeof(double) * 2 * N);
    double* S = (double*)malloc(sizeof(double) * 2 * N);
    double* X = (double*)malloc(sizeof(double) * 2 * N);
    double* J = NULL;
    if (!vb || !ax || !ay || !az || !ricker || !hil || !A0 || !A1 || !S || !X) goto done;

    orc_pad_model(p, vel, vb);
    float vmax = -9999999.999f;                       /* find_max, ose_3d_lib.cu:544-555 */
    for (long i = 0; i < N; ++i) if (vb[i] > vmax) vmax = vb[i];
    double R, dtR;
    int M;
    orc_series(p, vmax, &R, &dtR, &M);
    J = (double*)malloc(sizeof(double) * (M + 2));
    if (!J) goto done;
    orc_bessel(M, dtR, J);
    orc_sponge(p->bl, nx, d.br, p->sponge_mode, p->cerjan_factor, ax);
    orc_sponge(p->bf, ny, d.bb, p->sponge_mode, p->cerjan_factor, ay);
    orc_sponge(p->bu, p->nz, d.bd, p->sponge_mode, p->cerjan_factor, az);
    orc_ricker(p->nt, p->fm, p->dt, p->amp, ricker);
    orc_hilbert(ricker, p->nt, p->hilbert_div_nt, hil);

    /* source cell: sg_init_host then the decode of Xt_add_wavelet_sxyz */
    int sx0 = p->sxbeg + is * p->jsx, sy0 = p->sybeg + is * p->jsy, sz0 = p->szbeg + is * p->jsz;
    long sxyz = (long)sz0 * nx * ny + (long)sy0 * nx + sx0;
    int sx = (int)(sxyz % ((long)nx * ny) % nx);
    int sy = (int)(sxyz % ((long)nx * ny) / nx);
    int sz = (int)(sxyz / ((long)nx * ny));
    long src = ((long)(p->bu + sz) * nyb + (p->bf + sy)) * nxb + (p->bl + sx);
    if (src < 0 || src >= N) goto done;
    const int gz = p->bu + p->gzbeg;
    if (gz < 0 || gz >= nzb) goto done;

    for (int it = it0; it < it0 + nsteps; ++it) {
        P[src] += ricker[it];
        Q[src] += hil[it];
        /* a0 = W = P + iQ */
#pragma omp parallel for schedule(static)
        for (long i = 0; i < N; ++i) { A0[2 * i] = P[i]; A0[2 * i + 1] = Q[i]; }
        /* a1 = -i L a0 ; S = J0 a0 + 2 J1 a1  (ose_3d_lib.cu:649-744) */
        if (orc_apply_operator(p, vb, R, A0, X)) goto done;
#pragma omp parallel for schedule(static)
        for (long i = 0; i < N; ++i) {
            A1[2 * i] = X[2 * i + 1];
            A1[2 * i + 1] = -X[2 * i];
            S[2 * i] = J[0] * A0[2 * i] + 2.0 * J[1] * A1[2 * i];
            S[2 * i + 1] = J[0] * A0[2 * i + 1] + 2.0 * J[1] * A1[2 * i + 1];
        }
        double *am1 = A0, *an = A1;
        for (int n = 1; n <= M; ++n) {     /* ose_3d_lib.cu:750-872 */
            if (orc_apply_operator(p, vb, R, an, X)) goto done;
            const double c = 2.0 * J[n + 1];
#pragma omp parallel for schedule(static)
            for (int z = 0; z < nzb; ++z)
                for (int y = 0; y < nyb; ++y) {
                    double ayz = (double)ay[y] * (double)az[z];
                    for (int x = 0; x < nxb; ++x) {
                        long i = ((long)z * nyb + y) * nxb + x;
                        /* a_{n+1} = a_{n-1} - 2i L a_n */
                        double re = am1[2 * i] + 2.0 * X[2 * i + 1];
                        double im = am1[2 * i + 1] - 2.0 * X[2 * i];
                        am1[2 * i] = re;
                        am1[2 * i + 1] = im;
                        double att = (double)ax[x] * ayz;
                        S[2 * i] = (S[2 * i] + c * re) * att;
                        S[2 * i + 1] = (S[2 * i + 1] + c * im) * att;
                    }
                }
            double* t = am1; am1 = an; an = t;
        }
#pragma omp parallel for schedule(static)
        for (long i = 0; i < N; ++i) { P[i] = S[2 * i]; Q[i] = S[2 * i + 1]; }
        if (gather) {
            float* row = gather + (long)(it - it0) * d.ng;
            for (int iy = 0; iy < ny; ++iy)
                for (int ix = 0; ix < nx; ++ix)
                    row[iy * nx + ix] =
                        (float)Q[((long)gz * nyb + (p->bf + iy)) * nxb + p->bl + ix];
        }
    }
    rc = 0;
done:
    free(vb); free(ax); free(ay); free(az); free(ricker); free(hil);
    free(A0); free(A1); free(S); free(X); free(J);
    return rc;
}
