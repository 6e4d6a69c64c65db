// ose_host.cpp - host-side setup of libose3d: sizes, model padding, sponge,
// source traces, series order, FFT radix plans and tables.  Everything is
// computed in double and rounded once to float for the device.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <complex>
#include <thread>
#include <string>
#include <vector>

#include "ose_internal.h"

namespace ose {

// judge_odd (ose_3d_lib.cu:36-44), applied per axis as ose_3d.cu:85-90 does.
int derive_dims(const ose_params& p, ose_derived* d, std::string* err)
{
    memset(d, 0, sizeof(*d));
    if (p.nx < 1 || p.ny < 1 || p.nz < 1) { *err = "nx, ny, nz must be >= 1"; return -1; }
    if (p.bu < 0 || p.bd < 0 || p.bl < 0 || p.br < 0 || p.bf < 0 || p.bb < 0) {
        *err = "sponge widths must be >= 0";
        return -1;
    }
    if (p.nt < 1) { *err = "nt must be >= 1"; return -1; }
    if (!(p.dt > 0.f) || !(p.dx > 0.f) || !(p.dy > 0.f) || !(p.dz > 0.f) || !(p.fm > 0.f)) {
        *err = "dt, dx, dy, dz and fm must be > 0";
        return -1;
    }
    auto fix = [](int b0, int n, int b1, int* b1out) {
        int nb = b0 + n + b1;
        *b1out = b1;
        if (nb % 2) { *b1out = b1 + 1; ++nb; }
        return nb;
    };
    d->nxb = fix(p.bl, p.nx, p.br, &d->br);
    d->nyb = fix(p.bf, p.ny, p.bb, &d->bb);
    d->nzb = fix(p.bu, p.nz, p.bd, &d->bd);
    d->ng = p.nx * p.ny;
    d->dkx = 2.0 * M_PI / p.dx / d->nxb;
    d->dky = 2.0 * M_PI / p.dy / d->nyb;
    d->dkz = 2.0 * M_PI / p.dz / d->nzb;
    return 0;
}

// R = vmax*pi*|(1/dx,1/dy,1/dz)|, dtR = dt*R, M = (int)dtR + 6 (ose_3d.cu:191-197).
// M is taken from the float product, as the reference's float globals give it.
void series_params(const ose_params& p, float vmax, ose_derived* d)
{
    double R = (double)vmax * M_PI *
               sqrt(1.0 / ((double)p.dx * p.dx) + 1.0 / ((double)p.dy * p.dy) +
                    1.0 / ((double)p.dz * p.dz));
    float rf = (float)R;
    float dtrf = p.dt * rf;
    d->vmax = vmax;
    d->R = R;
    d->dtR = (double)p.dt * R;
    d->M = p.M_override > 0 ? p.M_override : (int)dtrf + 6;
    d->bessel_tail = fabs(jn(d->M + 2, d->dtR));
}

// Model read + sponge padding (ose_3d_lib.cu:887-1032): every padded cell
// takes the interior value at the clamped coordinates.  Output [z][y][x].
void pad_model(const ose_params& p, const ose_derived& d, const float* vel, std::vector<float>& vb)
{
    vb.resize((size_t)d.nxb * d.nyb * d.nzb);
    for (int z = 0; z < d.nzb; ++z) {
        int iz = z < p.bu ? 0 : (z >= p.bu + p.nz ? p.nz - 1 : z - p.bu);
        for (int y = 0; y < d.nyb; ++y) {
            int iy = y < p.bf ? 0 : (y >= p.bf + p.ny ? p.ny - 1 : y - p.bf);
            float* row = &vb[((size_t)z * d.nyb + y) * d.nxb];
            for (int x = 0; x < d.nxb; ++x) {
                int ix = x < p.bl ? 0 : (x >= p.bl + p.nx ? p.nx - 1 : x - p.bl);
                row[x] = vel[((size_t)ix * p.ny + iy) * p.nz + iz];
            }
        }
    }
}

// generate_att (ose_3d_kernel.cu:242-261), or the Cerjan taper exp(-(a*d)^2)
// with d the distance into the sponge in cells.
void sponge_table(int before, int nn, int after, int mode, float factor, std::vector<float>& out)
{
    out.assign((size_t)before + nn + after, 1.0f);
    for (int i = 0; i < before; ++i) {
        double t = mode == OSE_SPONGE_CERJAN ? (double)factor * (before - i)
                                             : (double)((float)(before - 1 - i) / (float)before);
        out[i] = (float)exp(-t * t);
    }
    for (int i = 0; i < after; ++i) {
        double t = mode == OSE_SPONGE_CERJAN ? (double)factor * (i + 1)
                                             : (double)((float)(i + 1) / (float)after);
        out[(size_t)before + nn + i] = (float)exp(-t * t);
    }
}

// Ricker with the reference's hard 40-sample delay (ose_3d_kernel.cu:3-13).
void ricker_trace(int nt, float fm, float dt, float amp, std::vector<float>& out)
{
    out.resize(nt);
    for (int i = 0; i < nt; ++i) {
        double a = M_PI * (double)fm * ((double)(i - 40) * dt - 1.0 / fm);
        double a2 = a * a;
        out[i] = (float)((double)amp * (1.0 - 2.0 * a2) * exp(-a2));
    }
}

// The shot's Q trace (ose_3d_lib.cu:578-581): real DFT of the Ricker, bins
// k < nt/2 multiplied by -i and the rest by +i (hilbert_1d's test,
// ose_3d_kernel.cu:158), unnormalised inverse real DFT.  The DC and, for even
// nt, Nyquist bins turn purely imaginary and vanish from a real inverse.
// Runs f(i) for i in [0, n) over up to 16 host threads (one when n is small).
template <typename F>
static void parallel_for(int n, F f)
{
    const int hw = (int)std::thread::hardware_concurrency();
    const int nth = n < 256 ? 1 : std::max(1, std::min(16, hw));
    if (nth == 1) {
        for (int i = 0; i < n; ++i) f(i);
        return;
    }
    std::vector<std::thread> th;
    for (int t = 0; t < nth; ++t)
        th.emplace_back([&, t] {
            for (int i = t; i < n; i += nth) f(i);
        });
    for (auto& x : th) x.join();
}

// Direct DFTs in double with the exponent index advanced by addition
// (j k mod nt), split over host threads by output index; the same
// arithmetic for every thread count.
void hilbert_trace(const std::vector<float>& w, int div_nt, std::vector<float>& out)
{
    const int nt = (int)w.size();
    const int nb = nt / 2 + 1;
    std::vector<std::complex<double>> X(nb);
    std::vector<double> c(nt), s(nt);
    for (int j = 0; j < nt; ++j) {
        c[j] = cos(2.0 * M_PI * j / nt);
        s[j] = sin(2.0 * M_PI * j / nt);
    }
    parallel_for(nb, [&](int k) {
        double re = 0, im = 0;
        for (int j = 0, e = 0; j < nt; ++j) {
            re += w[j] * c[e];
            im -= w[j] * s[e];
            e += k;
            if (e >= nt) e -= nt;
        }
        std::complex<double> v(re, im);
        X[k] = k < nt / 2 ? v * std::complex<double>(0, -1) : v * std::complex<double>(0, 1);
    });
    const int kmax = nt % 2 == 0 ? nt / 2 - 1 : (nt - 1) / 2;
    out.resize(nt);
    parallel_for(nt, [&](int n) {
        double acc = X[0].real();
        if (nt % 2 == 0) acc += X[nt / 2].real() * ((n & 1) ? -1.0 : 1.0);
        for (int k = 1, e = n % nt; k <= kmax; ++k) {
            acc += 2.0 * (X[k].real() * c[e] - X[k].imag() * s[e]);
            e += n;
            if (e >= nt) e -= nt;
        }
        out[n] = (float)(div_nt ? acc / nt : acc);
    });
}

// Radix plan: a prime factor >= 11 (when the length has one, taken once), then
// 4s, 2, 3, 5, 7 and any remaining prime.
int plan_axis(int n, AxisPlan* p)
{
    memset(p, 0, sizeof(*p));
    p->n = n;
    if (n < 1 || n > kMaxAxis) return -1;
    int m = n;
    auto push = [&](int r) {
        if (p->ns >= kMaxStages) return false;
        p->radix[p->ns++] = r;
        return true;
    };
    // a prime factor >= 11 goes first: the first stage has no input twiddles,
    // which the paired direct DFT of ose_kernels.cu needs
    int big = 0;
    {
        int t = m;
        for (int f = 2; f * f <= t; ++f)
            while (t % f == 0) t /= f;   // t = the largest prime factor
        if (t >= 11) big = t;
    }
    if (big) { if (!push(big)) return -1; m /= big; }
    while (m % 4 == 0) { if (!push(4)) return -1; m /= 4; }
    while (m % 2 == 0) { if (!push(2)) return -1; m /= 2; }
    for (int f = 3; m > 1; f += 2) {
        while (m % f == 0) { if (!push(f)) return -1; m /= f; }
        if (f * f > m && m > 1) { if (!push(m)) return -1; m = 1; }
    }
    return 0;
}

// W_n^t = exp(-2 pi i t / n), t < n: nearest floats, and (if lo) the
// remainders, so hi + lo carries the twiddle to about 48 bits.
void twiddle_table(int n, std::vector<float2>& out, std::vector<float2>* lo)
{
    out.resize(n);
    if (lo) lo->resize(n);
    for (int t = 0; t < n; ++t) {
        const double a = -2.0 * M_PI * (double)t / n;
        const double c = cos(a), s = sin(a);
        float ch, cl, sh, sl;
        split_float(c, &ch, &cl);
        split_float(s, &sh, &sl);
        out[t] = make_float2(ch, sh);
        if (lo) (*lo)[t] = make_float2(cl, sl);
    }
}

// (dk * wrapped index)^2 as scale_kxkz_3D wraps it (ose_3d_kernel.cu:109-120),
// nearest floats and (if lo) the remainders.
void k2_table(int n, double dk, std::vector<float>& out, std::vector<float>* lo)
{
    out.resize(n);
    if (lo) lo->resize(n);
    for (int i = 0; i < n; ++i) {
        const double k = dk * (i > n / 2 ? n - i : i);
        float h, l;
        split_float(k * k, &h, &l);
        out[i] = h;
        if (lo) (*lo)[i] = l;
    }
}

}  // namespace ose
