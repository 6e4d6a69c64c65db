// ose_epilogue.cuh - the pointwise work of one operator application, shared
// by the shared-memory row kernels (ose_kernels.cu) and the register row
// kernels (ose_cols.cu): scal_vr_3d, the recurrence, add_bessel_3d,
// apply_ABC_Xt and the receiver row of ose_3d_lib.cu:651-874, fused.
#pragma once

#include <cuda_runtime.h>

#include "ose_internal.h"

namespace ose {

// EPI_SCALE_VEL: out = X * vel[i] * scale (the allocation-free entry point)
// EPI_FIRST_FWD, EPI_MID_FWD (row launches only): FIRST / MID followed by the
// next application's forward x transform of the new term.
enum { EPI_NONE = -1, EPI_SCALE_VEL = 4, EPI_FIRST_FWD = 5, EPI_MID_FWD = 6 };

// The partial-sum update of one cell at a FIRST/MID/LAST application, by the
// schedule's weights (EpiArgs::wS, wP, wN): s = the stored S (zero unless
// it is read), am = a_{n-1}, an = a_{n+1}, att = the cell's sponge factor.
// Branch-free; a zero weight adds exactly nothing, so each factor is the
// rounded product of one coefficient and one power of att.
__device__ __forceinline__ float2 sum_update(const EpiArgs& e, float att, float2 s, float2 am, float2 an)
{
    const float a2 = att * att, a3 = a2 * att;
    const float fS = fmaf(e.wS[2], a3, fmaf(e.wS[1], a2, e.wS[0] * att));
    const float fP = fmaf(e.wP[2], a3, fmaf(e.wP[1], a2, e.wP[0] * att));
    const float fN = e.wN * att;
    float2 r = make_float2(s.x * fS, s.y * fS);
    if (kCompensatedConstants) {
        const float lP = fmaf(e.wPl[2], a3, fmaf(e.wPl[1], a2, e.wPl[0] * att)), lN = e.wNl * att;
        r.x = fmaf(lP, am.x, fmaf(lN, an.x, r.x));
        r.y = fmaf(lP, am.y, fmaf(lN, an.y, r.y));
    }
    r.x = fmaf(fP, am.x, fmaf(fN, an.x, r.x));
    r.y = fmaf(fP, am.y, fmaf(fN, an.y, r.y));
    return r;
}

// The pointwise work of one application on cell i = (x, y, z); X is the
// unnormalised inverse transform, e.vs the velocity, (e.sch + e.scl) = 1/(R N).
template <int EPI>
__device__ __forceinline__ void epilogue(long long i, int x, int y, int z, float2 X, const EpiArgs& e)
{
    const float v = __ldg(e.vs + i);
    float2 Lx = make_float2(X.x * v, X.y * v);
    // compensated: vs holds v and (sch + scl) = 1/(R N); else vs holds v/(R N)
    if (kCompensatedConstants || EPI == EPI_SCALE_VEL)
        Lx = make_float2(fmaf(Lx.x, e.sch, Lx.x * e.scl), fmaf(Lx.y, e.sch, Lx.y * e.scl));
    if (EPI == EPI_SCALE || EPI == EPI_SCALE_VEL) {
        e.prev[i] = Lx;
    } else if (EPI == EPI_FIRST) {
        // a_1 = -i L a_0   (ose_3d_lib.cu:651-731); S by the schedule
        const float2 a1 = make_float2(Lx.y, -Lx.x);
        e.prev[i] = a1;
        if (e.sp.touch) e.S[i] = sum_update(e, 1.f, make_float2(0.f, 0.f), a1, a1);
    } else {
        // a_{n+1} = a_{n-1} - 2i L a_n   (ose_3d_lib.cu:750-833); the partial
        // sum and sponge of ose_3d_lib.cu:839-860 by the schedule
        const float2 am = e.prev[i];
        const float2 an = make_float2(fmaf(2.f, Lx.y, am.x), fmaf(-2.f, Lx.x, am.y));
        if (EPI == EPI_MID && !e.sp.touch) {
            e.prev[i] = an;
            return;
        }
        const float att = __ldg(e.ax + x) * __ldg(e.ay + y) * __ldg(e.az + z);
        const float2 s = sum_update(e, att, e.sp.s_read ? e.S[i] : make_float2(0.f, 0.f), am, an);
        if (EPI == EPI_MID) {
            e.prev[i] = an;
            e.S[i] = s;
        } else {
            e.wout[i] = s;
            if (z == e.gz) {
                const int ix = x - e.bl, iy = y - e.bf;
                if (ix >= 0 && ix < e.nx && iy >= 0 && iy < e.ny) {
                    const int c = *e.cur;
                    if (c >= 0 && c < e.nt) e.gather[(long long)c * e.nx * e.ny + iy * e.nx + ix] = s.y;
                }
            }
        }
    }
}

// The same work for cnt cells of one row held by one thread, x = x0 + k * xs,
// i = i0 + k * xs: every load of a chunk of 8 cells is issued before the
// first store, so the loads overlap (the per-cell arithmetic is epilogue's).
// KEEP (FIRST, MID): v also receives the new term a_{n+1}, for the next
// application's forward transform in the same kernel.  Only the first
// `valid` cells exist (a row shorter than CNT * xs); the others are left alone.
// COH: a_{n-1} and S are read with loads that bypass the SM's L1 (for a
// persistent kernel that reads fields other CTAs wrote in the same launch).
template <int EPI, int CNT, bool KEEP = false, bool COH = false>
__device__ __forceinline__ void epilogue_row(float2 (&v)[CNT], long long i0, int x0, int xs, int y, int z,
                                             const EpiArgs& e, int valid = CNT)
{
    constexpr int CH = 8;
    static_assert(CNT % CH == 0, "whole chunks");
#pragma unroll
    for (int h = 0; h < CNT / CH; ++h) {
        float vv[CH], axv[CH];
        float2 am[CH], sm[CH];
#pragma unroll
        for (int q = 0; q < CH; ++q) {
            const int k = CH * h + q;
            const long long i = i0 + (long long)k * xs;
            if (k >= valid) continue;
            vv[q] = __ldg(e.vs + i);
            if (EPI == EPI_MID || EPI == EPI_LAST) {
                am[q] = COH ? __ldcg(e.prev + i) : e.prev[i];
                sm[q] = e.sp.s_read ? (COH ? __ldcg(e.S + i) : e.S[i]) : make_float2(0.f, 0.f);
                axv[q] = e.sp.touch ? __ldg(e.ax + x0 + k * xs) : 1.f;
            }
        }
        float ayz0 = 0.f, ayz1 = 0.f;
        if ((EPI == EPI_MID || EPI == EPI_LAST) && e.sp.touch) {
            ayz0 = __ldg(e.ay + y);
            ayz1 = __ldg(e.az + z);
        }
#pragma unroll
        for (int q = 0; q < CH; ++q) {
            const int k = CH * h + q;
            const long long i = i0 + (long long)k * xs;
            const int x = x0 + k * xs;
            if (k >= valid) continue;
            const float2 X = v[k];
            float2 Lx = make_float2(X.x * vv[q], X.y * vv[q]);
            if (kCompensatedConstants || EPI == EPI_SCALE_VEL)
                Lx = make_float2(fmaf(Lx.x, e.sch, Lx.x * e.scl), fmaf(Lx.y, e.sch, Lx.y * e.scl));
            if (EPI == EPI_SCALE || EPI == EPI_SCALE_VEL) {
                e.prev[i] = Lx;
            } else if (EPI == EPI_FIRST) {
                const float2 a1 = make_float2(Lx.y, -Lx.x);
                e.prev[i] = a1;
                if (e.sp.touch) e.S[i] = sum_update(e, 1.f, make_float2(0.f, 0.f), a1, a1);
                if (KEEP) v[k] = a1;
            } else {
                const float2 an = make_float2(fmaf(2.f, Lx.y, am[q].x), fmaf(-2.f, Lx.x, am[q].y));
                if (EPI == EPI_MID) {
                    e.prev[i] = an;
                    if (e.sp.touch) e.S[i] = sum_update(e, axv[q] * ayz0 * ayz1, sm[q], am[q], an);
                    if (KEEP) v[k] = an;
                } else {
                    const float2 s = sum_update(e, axv[q] * ayz0 * ayz1, sm[q], am[q], an);
                    e.wout[i] = s;
                    if (z == e.gz) {
                        const int ix = x - e.bl, iy = y - e.bf;
                        if (ix >= 0 && ix < e.nx && iy >= 0 && iy < e.ny) {
                            const int c = *e.cur;
                            if (c >= 0 && c < e.nt) e.gather[(long long)c * e.nx * e.ny + iy * e.nx + ix] = s.y;
                        }
                    }
                }
            }
        }
    }
}

// The epilogue arguments of batched shot S at application n.
__device__ __forceinline__ EpiArgs batch_epi(const BatchShot& S, int n)
{
    EpiArgs e{};
    e.vs = S.vs;
    e.ax = S.ax;
    e.ay = S.ay;
    e.az = S.az;
    e.S = S.S;
    e.wout = S.W;
    e.prev = n == 0 ? S.A : ((n & 1) ? S.W : S.A);
    e.sch = S.sch;
    e.scl = S.scl;
    e.c1 = S.c[n];
    e.c1l = S.cl[n];
    e.cp = n == 1 ? S.c0 : (n >= 2 ? S.c[n - 2] : 0.f);
    e.cpl = n == 1 ? S.c0l : (n >= 2 ? S.cl[n - 2] : 0.f);
    e.sp = sum_plan(n, S.M);
    set_sum_weights(e);
    e.gather = S.gather;
    e.cur = S.ctr + 1;
    e.gz = S.gz;
    e.bl = S.bl;
    e.bf = S.bf;
    e.nx = S.nx;
    e.ny = S.ny;
    e.nt = S.nt;
    return e;
}

}  // namespace ose
