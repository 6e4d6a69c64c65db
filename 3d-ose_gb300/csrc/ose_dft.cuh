// ose_dft.cuh - in-register DFT building blocks of the four-step transforms
// (ose_cols.cu, ose_bluestein.cu): complex helpers and DFT-C of a
// compile-time length by mixed radix (radix 4 first, then the smallest prime
// factor; paired direct sums for primes), twiddles from a shared table.
#pragma once

#include <cuda_runtime.h>

namespace ose {
namespace cols {

__host__ __device__ constexpr bool is_prime(int n)
{
    if (n < 2) return false;
    for (int d = 2; d * d <= n; ++d)
        if (n % d == 0) return false;
    return true;
}

__host__ __device__ constexpr int first_factor(int n)
{
    if (n % 4 == 0) return 4;
    for (int d = 2; d <= n; ++d)
        if (n % d == 0) return d;
    return n;
}

// A complex add or subtract is one packed two-lane FP32 instruction
// (add/sub.rn.f32x2: the same IEEE results as two scalar ones, never
// contracted with a preceding multiply).
__device__ __forceinline__ float2 cadd(float2 a, float2 b)
{
    unsigned long long d, x, y;
    asm("mov.b64 %0, {%1, %2};" : "=l"(x) : "f"(a.x), "f"(a.y));
    asm("mov.b64 %0, {%1, %2};" : "=l"(y) : "f"(b.x), "f"(b.y));
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(x), "l"(y));
    float2 r;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(d));
    return r;
}
__device__ __forceinline__ float2 csub(float2 a, float2 b)
{
    unsigned long long d, x, y;
    asm("mov.b64 %0, {%1, %2};" : "=l"(x) : "f"(a.x), "f"(a.y));
    asm("mov.b64 %0, {%1, %2};" : "=l"(y) : "f"(b.x), "f"(b.y));
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(x), "l"(y));
    float2 r;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(d));
    return r;
}
__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}

template <bool INV>
__device__ __forceinline__ float2 tw(const float2* W, int e)
{
    const float2 w = W[e];
    return INV ? make_float2(w.x, -w.y) : w;
}

// times -i (forward) or +i (inverse)
template <bool INV>
__device__ __forceinline__ float2 rot(float2 a)
{
    return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

// v[0..C) <- DFT_C(v[0..C)) in natural order; W_C^t = W[ST * t] (forward
// twiddles; conjugated for INV).
template <int C, int ST, bool INV, int L>
__device__ __forceinline__ void dftc(float2 (&v)[L], const float2* __restrict__ W)
{
    static_assert(C <= L, "array too short");
    if constexpr (C == 1) {
    } else if constexpr (C == 2) {
        const float2 a = v[0], b = v[1];
        v[0] = cadd(a, b);
        v[1] = csub(a, b);
    } else if constexpr (C == 4) {
        const float2 t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]), t2 = cadd(v[1], v[3]);
        const float2 t3 = rot<INV>(csub(v[1], v[3]));
        v[0] = cadd(t0, t2);
        v[2] = csub(t0, t2);
        // +-i (v1 - v3): a swapped pair, added lane by lane
        v[1] = make_float2(t1.x + t3.x, t1.y + t3.y);
        v[3] = make_float2(t1.x - t3.x, t1.y - t3.y);
    } else if constexpr (is_prime(C)) {
        // direct sums, pairing j and C - j: X_k = x0 + sum_j (x_j + x_{C-j}) cos
        //                                        -/+ i (x_j - x_{C-j}) sin
        constexpr int H = (C - 1) / 2;
        float2 s[H], d[H];
#pragma unroll
        for (int j = 1; j <= H; ++j) {
            s[j - 1] = cadd(v[j], v[C - j]);
            d[j - 1] = csub(v[j], v[C - j]);
        }
        float2 o[C];
        float2 sum = v[0];
#pragma unroll
        for (int j = 0; j < H; ++j) sum = cadd(sum, s[j]);
        o[0] = sum;
#pragma unroll
        for (int k = 1; k <= H; ++k) {
            float2 re = v[0], im = make_float2(0.f, 0.f);
#pragma unroll
            for (int j = 1; j <= H; ++j) {
                const float2 w = W[ST * ((j * k) % C)];   // (cos, -sin) of 2 pi j k / C
                re.x = fmaf(s[j - 1].x, w.x, re.x);
                re.y = fmaf(s[j - 1].y, w.x, re.y);
                im.x = fmaf(d[j - 1].x, w.y, im.x);
                im.y = fmaf(d[j - 1].y, w.y, im.y);
            }
            // forward: X_k = re + i im_term with im_term = sum d_j (-sin) -> i * (d * w.y)
            const float2 ii = INV ? make_float2(im.y, -im.x) : make_float2(-im.y, im.x);
            o[k] = cadd(re, ii);
            o[C - k] = csub(re, ii);
        }
#pragma unroll
        for (int k = 0; k < C; ++k) v[k] = o[k];
    } else {
        constexpr int A = first_factor(C), B = C / A;
        float2 t[A][B];
#pragma unroll
        for (int r = 0; r < A; ++r)
#pragma unroll
            for (int m = 0; m < B; ++m) t[r][m] = v[A * m + r];
#pragma unroll
        for (int r = 0; r < A; ++r) dftc<B, ST * A, INV, B>(t[r], W);
#pragma unroll
        for (int k2 = 0; k2 < B; ++k2) {
            float2 u[A];
#pragma unroll
            for (int r = 0; r < A; ++r) u[r] = (r * k2) ? cmul(t[r][k2], tw<INV>(W, ST * r * k2)) : t[r][k2];
            dftc<A, ST * B, INV, A>(u, W);
#pragma unroll
            for (int k1 = 0; k1 < A; ++k1) v[k2 + B * k1] = u[k1];
        }
    }
}

}  // namespace cols
}  // namespace ose
