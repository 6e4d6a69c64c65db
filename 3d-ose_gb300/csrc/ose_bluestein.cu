// ose_bluestein.cu - axis transforms of lengths that have no register
// four-step kernel of their own (142 = 2 x 71 in config 1, 152 = 8 x 19 in
// the reference's default grid), by Bluestein's chirp-z identity on the
// register four-step transforms of a longer length L = 16 C >= 2 n - 1.
//
// With the chirp c_m = exp(-i pi m^2 / n), W_n^(m k) = c_m c_k conj(c_(k-m)),
// so the forward DFT of a line x of length n is
//   X_k = c_k sum_m (x_m c_m) conj(c_(k-m)) = c_k (a * b)_k,   k < n,
// a circular convolution of length L of a = x c (zero-padded) with
// b_j = conj(c_|j|) for |j| < n (b at j mod L).  It is computed as
//   y = IFFT_L( FFT_L(a) . B ),   B = FFT_L(b) / L  (from the host, FP64),
// both transforms in registers by the same two phases as ose_cols.cu
// (a line is a 16 x C matrix: DFT-16, twiddle, shared-memory transpose,
// DFT-C).  The inverse DFT is conj(forward(conj(X))).  A thread of phase 1
// holds positions m = C n1 + p, n1 < 16; the data occupy n1 < 8 (n <= 8 C).
//
// Kernels: the y and z passes (forward, inverse, forward * |k| inverse) on
// TX neighbouring x columns per CTA, and the x passes on RW rows per CTA
// (forward, or inverse + the step's epilogue + the forward transform of the
// new term, as the register row kernels).  Tables per axis: the chirp (n),
// B (L) and W_L^t (L), uploaded at create.
#include <cuda_runtime.h>
#include <math.h>

#include <complex>
#include <vector>

#include "ose_dft.cuh"
#include "ose_epilogue.cuh"
#include "ose_internal.h"
#include "ose_pdl.cuh"

namespace ose {
namespace blue {

using cols::cadd;
using cols::cmul;
using cols::csub;
using cols::dftc;

__device__ __forceinline__ float2 conjf2(float2 a) { return make_float2(a.x, -a.y); }

// DFT-16 as dftc<16, ST> (4 x 4: DFT-4 over m of v[4 m + r], twiddle, DFT-4
// over r), for the halves Bluestein leaves: LOW_IN = inputs v[8..15] are zero
// (the first DFT-4s see (a, b, 0, 0)); LOW_OUT = only v[0..7] is wanted
// (the last DFT-4s give outputs 0 and 1).  Same arithmetic on the rest.
template <int ST, bool INV, bool LOW_IN, bool LOW_OUT>
__device__ __forceinline__ void dft16_half(float2 (&v)[16], const float2* __restrict__ W)
{
    float2 t[4][4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        if (LOW_IN) {
            const float2 a = v[r], b = v[4 + r], rb = cols::rot<INV>(b);
            t[r][0] = cadd(a, b);
            t[r][1] = cadd(a, rb);
            t[r][2] = csub(a, b);
            t[r][3] = csub(a, rb);
        } else {
#pragma unroll
            for (int m = 0; m < 4; ++m) t[r][m] = v[4 * m + r];
            dftc<4, ST * 4, INV, 4>(t[r], W);
        }
    }
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) {
        float2 u[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) u[r] = (r * k2) ? cmul(t[r][k2], cols::tw<INV>(W, ST * r * k2)) : t[r][k2];
        if (LOW_OUT) {
            const float2 t0 = cadd(u[0], u[2]), t1 = csub(u[0], u[2]), t2 = cadd(u[1], u[3]);
            const float2 t3 = cols::rot<INV>(csub(u[1], u[3]));
            v[k2] = cadd(t0, t2);
            v[k2 + 4] = cadd(t1, t3);
        } else {
            dftc<4, ST * 4, INV, 4>(u, W);
#pragma unroll
            for (int k1 = 0; k1 < 4; ++k1) v[k2 + 4 * k1] = u[k1];
        }
    }
}

template <int C>
struct Cfg {
    static constexpr int L = 16 * C;
    static constexpr int P = C > 16 ? C : 16;      // line threads
    // columns per CTA (y, z passes): 16 up to C = 20 (288 or 320 threads,
    // two CTAs per SM; for C = 18 this measured 1.77 -> 1.55 ms per step of
    // the padded 142^3 grid against 8 columns at three CTAs of 144 threads),
    // 8 for C = 24 (16 would spill)
    static constexpr int TX = P > 20 ? 8 : 16;
    static constexpr bool CWIDE = TX * P > 256;    // launched two per SM: registers capped
    // rows per CTA (x passes); 16 rows at C = 18 measured slower (spills)
    static constexpr int RW = P > 16 ? 8 : 16;
    // row CTAs per SM the registers must allow: 4 at C = 18 (96 registers, no
    // spill; 1.52 -> 1.48 ms per step of the padded 142^3 grid against three
    // CTAs at 125 registers); C = 20 and 24 would spill
    static constexpr int RMINB = C == 18 ? 4 : 0;
    static constexpr int CTHREADS = TX * P;
    static constexpr int RTHREADS = RW * P;
    static constexpr int NP = 17 * C;              // padded row of the row transpose buffer
    static constexpr int NMAX = 8 * C;             // longest n: 2 n - 1 <= L
    // W_L (L) + B (L) + chirp (NMAX) + transpose buffer
    static constexpr size_t CSMEM = sizeof(float2) * ((size_t)2 * L + NMAX + (size_t)L * TX);
    static constexpr size_t RSMEM = sizeof(float2) * ((size_t)2 * L + NMAX + (size_t)RW * NP);
};

// Element (a, b) of the transpose buffer of this thread's line: a = line
// thread of phase 1, b = the 16-point index.
struct ColIdx {
    int c, tx;
    __device__ int operator()(int a, int b) const { return (a * 16 + b) * tx + c; }
};
struct RowIdx {
    int base;
    __device__ int operator()(int a, int b) const { return base + a * 17 + b; }
};

// One length-n DFT (INV: inverse, unnormalised) of the line whose phase-1
// values this thread holds: v[n1] = x[C n1 + p] (zero where C n1 + p >= n) in,
// the transform in the same positions out.  Every thread of the CTA calls it
// (two CTA barriers inside).
template <int C, bool INV, typename IDX>
__device__ __forceinline__ void bs_line(float2 (&v)[8], int p, IDX idx, float2* T, const float2* W,
                                        const float2* chirp, const float2* spec, int n)
{
    float2 w[16];
    if (p < C) {
#pragma unroll
        for (int n1 = 0; n1 < 8; ++n1) {
            const int m = C * n1 + p;
            w[n1] = m < n ? cmul(INV ? conjf2(v[n1]) : v[n1], chirp[m]) : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int n1 = 8; n1 < 16; ++n1) w[n1] = make_float2(0.f, 0.f);
        dft16_half<C, false, true, false>(w, W);
#pragma unroll
        for (int k1 = 0; k1 < 16; ++k1) T[idx(p, k1)] = k1 ? cmul(w[k1], W[p * k1]) : w[k1];
    }
    __syncthreads();
    if (p < 16) {
        float2 u[C];
#pragma unroll
        for (int j = 0; j < C; ++j) u[j] = T[idx(j, p)];
        dftc<C, 16, false>(u, W);   // u[k2] = FFT_L(a)[p + 16 k2]
#pragma unroll
        for (int k2 = 0; k2 < C; ++k2) u[k2] = cmul(u[k2], spec[p + 16 * k2]);
        dftc<C, 16, true>(u, W);
#pragma unroll
        for (int j = 0; j < C; ++j) {
            const float2 t = W[j * p];
            T[idx(j, p)] = (j * p) ? cmul(u[j], conjf2(t)) : u[j];
        }
    }
    __syncthreads();
    if (p < C) {
#pragma unroll
        for (int k1 = 0; k1 < 16; ++k1) w[k1] = T[idx(p, k1)];
        dft16_half<C, true, false, true>(w, W);    // w[n1] = (a * b)[C n1 + p], n1 < 8
#pragma unroll
        for (int n1 = 0; n1 < 8; ++n1) {
            const int m = C * n1 + p;
            const float2 r = m < n ? cmul(w[n1], chirp[m]) : make_float2(0.f, 0.f);
            v[n1] = INV ? conjf2(r) : r;
        }
    }
}

__device__ __forceinline__ void load_tables(float2* W, float2* B, float2* ch, const float2* gw, const float2* gb,
                                            const float2* gc, int L, int n)
{
    for (int i = threadIdx.x; i < L; i += blockDim.x) {
        W[i] = gw[i];
        B[i] = gb[i];
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) ch[i] = gc[i];
}

// y lines (AXIS 1) or z lines (AXIS 2) of TX columns; MODE as ose_cols.cu:
// 0 forward, 1 inverse, 2 forward * |k| inverse.
template <int C, int MODE>
__global__ void __launch_bounds__(Cfg<C>::CTHREADS, Cfg<C>::CWIDE ? 2 : 0) k_col_bs(float2* __restrict__ X, int nxb, long long stride,
                                                             long long ostride, int n, int axis, Tables tb)
{
    using K = Cfg<C>;
    extern __shared__ float4 smem4[];
    float2* W = reinterpret_cast<float2*>(smem4);
    float2* B = W + K::L;
    float2* ch = B + K::L;
    float2* T = ch + K::NMAX;
    load_tables(W, B, ch, tb.btw[axis], tb.bsp[axis], tb.bch[axis], K::L, n);
    griddep_launch();   // launched with launch_pdl: only the constant tables are read before the wait
    griddep_wait();
    const int c = threadIdx.x % K::TX, p = threadIdx.x / K::TX;
    const int x = blockIdx.x * K::TX + c, other = blockIdx.y;
    const bool ok = x < nxb && p < C;
    float2* line = X + (size_t)other * ostride + x;
    __syncthreads();
    float2 v[8];
#pragma unroll
    for (int n1 = 0; n1 < 8; ++n1) {
        const int m = C * n1 + p;
        v[n1] = (ok && m < n) ? line[(size_t)m * stride] : make_float2(0.f, 0.f);
    }
    const ColIdx idx{c, K::TX};
    if (MODE == 1) {
        bs_line<C, true>(v, p, idx, T, W, ch, B, n);
    } else {
        bs_line<C, false>(v, p, idx, T, W, ch, B, n);
        if (MODE == 2) {
            // spectral index m along z: * |k| (scale_kxkz_3D between the z transforms)
            const float kxy = ok ? __ldg(tb.kx2 + x) + __ldg(tb.ky2 + other) : 0.f;
#pragma unroll
            for (int n1 = 0; n1 < 8; ++n1) {
                const int m = C * n1 + p;
                if (ok && m < n) {
                    const float k = sqrtf(kxy + __ldg(tb.kz2 + m));
                    v[n1].x *= k;
                    v[n1].y *= k;
                }
            }
            bs_line<C, true>(v, p, idx, T, W, ch, B, n);
        }
    }
#pragma unroll
    for (int n1 = 0; n1 < 8; ++n1) {
        const int m = C * n1 + p;
        if (ok && m < n) line[(size_t)m * stride] = v[n1];
    }
}

// x rows (contiguous, row = z * nyb + y), RW per CTA.  EPI_NONE: forward
// transform of src into dst.  Otherwise the inverse transform of src, the
// step's epilogue and (FWD) the forward transform of the new term into dst.
template <int C, int EPI, bool FWD>
__global__ void __launch_bounds__(Cfg<C>::RTHREADS, Cfg<C>::RMINB) k_row_bs(const float2* __restrict__ src, float2* __restrict__ dst,
                                                             int n, int nyb, long long nrows, Tables tb, EpiArgs e)
{
    using K = Cfg<C>;
    extern __shared__ float4 smem4[];
    float2* W = reinterpret_cast<float2*>(smem4);
    float2* B = W + K::L;
    float2* ch = B + K::L;
    float2* T = ch + K::NMAX;
    load_tables(W, B, ch, tb.btw[0], tb.bsp[0], tb.bch[0], K::L, n);
    griddep_launch();
    griddep_wait();
    const int r = threadIdx.x / K::P, q = threadIdx.x % K::P;
    const long long row = (long long)blockIdx.x * K::RW + r;
    const bool ok = row < nrows && q < C;
    const RowIdx idx{r * K::NP};
    __syncthreads();
    float2 v[8];
#pragma unroll
    for (int n1 = 0; n1 < 8; ++n1) {
        const int m = C * n1 + q;
        v[n1] = (ok && m < n) ? src[row * n + m] : make_float2(0.f, 0.f);
    }
    if (EPI == EPI_NONE) {
        bs_line<C, false>(v, q, idx, T, W, ch, B, n);
    } else {
        bs_line<C, true>(v, q, idx, T, W, ch, B, n);
        if (ok) {
            // cells x = q + C k, k < valid: the rest of the line is beyond the row
            const int valid = q < n ? (n - q + C - 1) / C : 0;
            const int y = (int)(row % nyb), z = (int)(row / nyb);
            epilogue_row<EPI, 8, FWD>(v, row * n + q, q, C, y, z, e, valid < 8 ? valid : 8);
        }
        if (!FWD) return;   // uniform: no barrier follows
        bs_line<C, false>(v, q, idx, T, W, ch, B, n);
    }
#pragma unroll
    for (int n1 = 0; n1 < 8; ++n1) {
        const int m = C * n1 + q;
        if (ok && m < n) dst[row * n + m] = v[n1];
    }
}

// L = 16 C >= 2 n - 1 for 128 <= n <= 192: C from 16; 18, 20 and 24 cover it
#define OSE_BS_SIZES(X) X(18) X(20) X(24)

template <int C>
cudaError_t configure_one()
{
    using K = Cfg<C>;
    cudaError_t e;
#define SETC(k) if ((e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)K::CSMEM)) != cudaSuccess) return e
#define SETR(k) if ((e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)K::RSMEM)) != cudaSuccess) return e
    SETC((k_col_bs<C, 0>));
    SETC((k_col_bs<C, 1>));
    SETC((k_col_bs<C, 2>));
    SETR((k_row_bs<C, EPI_NONE, false>));
    SETR((k_row_bs<C, EPI_FIRST, true>));
    SETR((k_row_bs<C, EPI_MID, true>));
    SETR((k_row_bs<C, EPI_LAST, false>));
    SETR((k_row_bs<C, EPI_SCALE, false>));
#undef SETC
#undef SETR
    return cudaSuccess;
}

template <int C>
cudaError_t launch_col_c(cudaStream_t s, int mode, int n, float2* X, int nxb, int nother, long long stride,
                         long long ostride, int axis, const Tables& t)
{
    using K = Cfg<C>;
    const dim3 grid((nxb + K::TX - 1) / K::TX, nother);
    if (mode == 0) return launch_pdl(k_col_bs<C, 0>, grid, dim3(K::CTHREADS), K::CSMEM, s, X, nxb, stride, ostride, n, axis, t);
    if (mode == 1) return launch_pdl(k_col_bs<C, 1>, grid, dim3(K::CTHREADS), K::CSMEM, s, X, nxb, stride, ostride, n, axis, t);
    return launch_pdl(k_col_bs<C, 2>, grid, dim3(K::CTHREADS), K::CSMEM, s, X, nxb, stride, ostride, n, axis, t);
}

template <int C>
cudaError_t launch_row_c(cudaStream_t s, int epi, int n, const float2* src, float2* dst, int nyb, long long nrows,
                         const Tables& t, const EpiArgs& e)
{
    using K = Cfg<C>;
    const dim3 grid((unsigned)((nrows + K::RW - 1) / K::RW)), block(K::RTHREADS);
    switch (epi) {
    case EPI_NONE:
        return launch_pdl(k_row_bs<C, EPI_NONE, false>, grid, block, K::RSMEM, s, src, dst, n, nyb, nrows, t, e);
    case EPI_FIRST_FWD:
        return launch_pdl(k_row_bs<C, EPI_FIRST, true>, grid, block, K::RSMEM, s, src, dst, n, nyb, nrows, t, e);
    case EPI_MID_FWD:
        return launch_pdl(k_row_bs<C, EPI_MID, true>, grid, block, K::RSMEM, s, src, dst, n, nyb, nrows, t, e);
    case EPI_LAST:
        return launch_pdl(k_row_bs<C, EPI_LAST, false>, grid, block, K::RSMEM, s, src, dst, n, nyb, nrows, t, e);
    case EPI_SCALE:
        return launch_pdl(k_row_bs<C, EPI_SCALE, false>, grid, block, K::RSMEM, s, src, dst, n, nyb, nrows, t, e);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace blue

// Bluestein length for an axis of length n: the smallest L = 16 C, C in the
// instantiated set, with L >= 2 n - 1; 0 = the axis keeps its own kernels
// (a register four-step length, shorter than 128 — where the Stockham
// stages, paired direct DFTs included, cost little — longer than 192, or no
// prime factor >= 11, where the Stockham radices 2..7 already serve it).
// The batched form has no Bluestein kernels: its shots keep the Stockham
// passes on such lengths.
int bluestein_length(int n)
{
    if (n < 128 || n > 192 || col_supported(n)) return 0;
    int t = n, big = 1;
    for (int f = 2; f <= t; ++f)
        while (t % f == 0) { t /= f; big = f; }
    if (big < 11) return 0;
    static const int cs[] = {18, 20, 24};
    for (int c : cs)
        if (16 * c >= 2 * n - 1) return 16 * c;
    return 0;
}

// Tables of one axis (double precision, rounded once): chirp c_m =
// exp(-i pi m^2 / n), m < n; B = FFT_L(b) / L with b_j = conj(c_|j|) at j mod
// L; W_L^t = exp(-2 pi i t / L).
void bluestein_tables(int n, int L, std::vector<float2>& chirp, std::vector<float2>& spec,
                      std::vector<float2>& twl)
{
    using cd = std::complex<double>;
    const double pi = 3.14159265358979323846;
    std::vector<cd> c(n), b(L, cd(0.0, 0.0));
    for (int m = 0; m < n; ++m) {
        const long long q = ((long long)m * m) % (2LL * n);   // exp(-i pi q / n) has period 2 n in q
        c[m] = std::polar(1.0, -pi * (double)q / n);
    }
    for (int j = 0; j < n; ++j) {
        b[j] = std::conj(c[j]);
        if (j) b[L - j] = std::conj(c[j]);
    }
    chirp.resize(n);
    for (int m = 0; m < n; ++m) chirp[m] = make_float2((float)c[m].real(), (float)c[m].imag());
    spec.resize(L);
    for (int k = 0; k < L; ++k) {
        cd acc(0.0, 0.0);
        for (int j = 0; j < L; ++j) acc += b[j] * std::polar(1.0, -2.0 * pi * (double)(((long long)j * k) % L) / L);
        acc /= (double)L;
        spec[k] = make_float2((float)acc.real(), (float)acc.imag());
    }
    twl.resize(L);
    for (int t = 0; t < L; ++t) {
        const cd w = std::polar(1.0, -2.0 * pi * (double)t / L);
        twl[t] = make_float2((float)w.real(), (float)w.imag());
    }
}

cudaError_t configure_bluestein_kernels()
{
    cudaError_t e = cudaSuccess;
#define CONF(C) if ((e = blue::configure_one<C>()) != cudaSuccess) return e;
    OSE_BS_SIZES(CONF)
#undef CONF
    return e;
}

// mode: 0 forward, 1 inverse, 2 forward * |k| inverse; axis 1 (y) or 2 (z).
cudaError_t launch_col_bluestein(cudaStream_t s, int mode, int n, float2* X, int nxb, int nother, long long stride,
                                 long long ostride, int axis, const Tables& t)
{
    switch (t.bl[axis] / 16) {
#define LAUNCH(C) case C: return blue::launch_col_c<C>(s, mode, n, X, nxb, nother, stride, ostride, axis, t);
        OSE_BS_SIZES(LAUNCH)
#undef LAUNCH
    default: return cudaErrorInvalidValue;
    }
}

// epi: EPI_NONE (forward), EPI_FIRST_FWD, EPI_MID_FWD, EPI_LAST or EPI_SCALE.
cudaError_t launch_row_bluestein(cudaStream_t s, int epi, int n, const float2* src, float2* dst, int nyb,
                                 long long nrows, const Tables& t, const EpiArgs& e)
{
    switch (t.bl[0] / 16) {
#define LAUNCH(C) case C: return blue::launch_row_c<C>(s, epi, n, src, dst, nyb, nrows, t, e);
        OSE_BS_SIZES(LAUNCH)
#undef LAUNCH
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace ose
