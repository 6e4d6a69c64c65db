// ose_kernels.cu - generic-size kernels of one OSE operator application
// (any even padded size, axes up to 1024 with radices 4, 2, 3, 5, 7 and a
// direct DFT for other primes).
//
// One application of L = v * IFFT3(|k| FFT3(.)) / (R N) to the packed field
// a_n = p + i q (wavefield_extro_ori2, ose_3d_lib.cu:665-687 for one part) is
// five passes over HBM:
//   1. x rows   forward   a_n -> X
//   2. y lines  forward   X in place
//   3. z lines  forward, * |k|, inverse   X in place (scale_kxkz_3D fused
//      between the two z transforms)
//   4. y lines  inverse   X in place
//   5. x rows   inverse + the step's pointwise work: v/(R N) (scal_vr_3d),
//      recurrence a_{n+1} = a_{n-1} - 2i L a_n, S += 2 J_{n+1} a_{n+1}
//      (add_bessel_3d), S *= sponge (apply_ABC_Xt), and on the last term the
//      new state and the receiver row (rec_shotdata_3d).
// Each pass stages a tile of lines in shared memory and runs a Stockham
// autosort FFT there (natural order in, natural order out).
#include <cuda_runtime.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "ose_internal.h"
#include "ose_pdl.cuh"
#include "ose_epilogue.cuh"

namespace ose {

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }

template <bool INV>
__device__ __forceinline__ float2 twiddle(const float2* tw, int e)
{
    float2 w = tw[e];
    return INV ? make_float2(w.x, -w.y) : w;
}

// times W_4 = -i (forward) or +i (inverse)
template <bool INV>
__device__ __forceinline__ float2 rot4(float2 a)
{
    return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

// One Stockham stage of radix r on L lines: element e of line l sits at
// buf[l*LS + e*ES].  p = product of the radices already applied.
template <bool INV>
__device__ void fft_stage(const float2* __restrict__ in, float2* __restrict__ out, int L, int LS,
                          int ES, bool line_fastest, int n, int r, int p, const float2* tw)
{
    const int m = n / r;
    const int tstep = n / (p * r);
    const int total = L * m;
    if (r > 4 && p == 1 && (r & 1)) {
        // odd radix r >= 5 as the first stage (no input twiddles): the paired
        // direct DFT.  With s_j = x_j + x_{r-j}, d_j = x_j - x_{r-j} and
        // W_r^(j q) = c - i s, for q = 1 .. (r-1)/2
        //   y_q, y_{r-q} = x_0 + sum_j s_j c  -/+ i sum_j d_j s
        // (signs swapped for the inverse), so one work item computes two
        // outputs from (r-1)/2 terms: a quarter of the multiply-adds of the
        // direct sum.  Item q = 0 computes y_0 = x_0 + sum_j s_j.
        const int h = (r - 1) / 2, nr = n / r;
        for (int b = threadIdx.x; b < total * (h + 1); b += blockDim.x) {
            const int q = b % (h + 1), bb = b / (h + 1);
            int l, i;
            if (line_fastest) { l = bb % L; i = bb / L; }
            else { l = bb / m; i = bb - l * m; }
            const float2* src = in + l * LS + i * ES;
            const int ms = m * ES;
            const float2 x0 = src[0];
            float2 A = make_float2(0.f, 0.f), B = make_float2(0.f, 0.f);
            int jq = 0;
            for (int j = 1; j <= h; ++j) {
                jq += q;
                if (jq >= r) jq -= r;
                const float2 xa = src[j * ms], xb = src[(r - j) * ms];
                const float2 w = tw[jq * nr];   // (cos, -sin) of 2 pi j q / r
                A.x = fmaf(xa.x + xb.x, w.x, A.x);
                A.y = fmaf(xa.y + xb.y, w.x, A.y);
                B.x = fmaf(xa.x - xb.x, w.y, B.x);
                B.y = fmaf(xa.y - xb.y, w.y, B.y);
            }
            // forward: y_q = x0 + A + i B, y_{r-q} = x0 + A - i B; inverse swapped
            const float2 base = make_float2(x0.x + A.x, x0.y + A.y);
            const float2 iB = INV ? make_float2(B.y, -B.x) : make_float2(-B.y, B.x);
            float2* dst = out + l * LS + i * r * ES;
            if (q == 0) {
                dst[0] = base;
            } else {
                dst[q * ES] = cadd(base, iB);
                dst[(r - q) * ES] = csub(base, iB);
            }
        }
        return;
    }
    if (r > 4) {
        // radix 5, 7 and larger primes: one output q of one butterfly per work
        // item, y_q = sum_j x_j W_n^(j te) W_r^(j q), the two exponents
        // combined into one table index e_j = j te + (j q mod r) n / r < 2n
        const int nr = n / r;
        for (int b = threadIdx.x; b < total * r; b += blockDim.x) {
            const int q = b % r, bb = b / r;
            int l, i;
            if (line_fastest) { l = bb % L; i = bb / L; }
            else { l = bb / m; i = bb - l * m; }
            const int k = i % p;
            const int te = k * tstep;
            const float2* src = in + l * LS + i * ES;
            const int ms = m * ES;
            float2 acc = make_float2(0.f, 0.f);
            int jte = 0, jq = 0;
            for (int j = 0; j < r; ++j) {
                int e = jte + jq * nr;
                if (e >= n) e -= n;
                acc = cadd(acc, cmul(src[j * ms], twiddle<INV>(tw, e)));
                jte += te;
                jq += q;
                if (jq >= r) jq -= r;
            }
            out[l * LS + ((i - k) * r + k + q * p) * ES] = acc;
        }
        return;
    }
    for (int b = threadIdx.x; b < total; b += blockDim.x) {
        int l, i;
        if (line_fastest) { l = b % L; i = b / L; }
        else { l = b / m; i = b - l * m; }
        const int k = i % p;
        const int te = k * tstep;
        const float2* src = in + l * LS + i * ES;
        float2* dst = out + l * LS + ((i - k) * r + k) * ES;
        const int ms = m * ES, ps = p * ES;
        if (r == 4) {
            float2 x0 = src[0], x1 = src[ms], x2 = src[2 * ms], x3 = src[3 * ms];
            if (te) {
                x1 = cmul(x1, twiddle<INV>(tw, te));
                x2 = cmul(x2, twiddle<INV>(tw, 2 * te));
                x3 = cmul(x3, twiddle<INV>(tw, 3 * te));
            }
            float2 a0 = cadd(x0, x2), a1 = csub(x0, x2), a2 = cadd(x1, x3), a3 = rot4<INV>(csub(x1, x3));
            dst[0] = cadd(a0, a2);
            dst[ps] = cadd(a1, a3);
            dst[2 * ps] = csub(a0, a2);
            dst[3 * ps] = csub(a1, a3);
        } else if (r == 2) {
            float2 x0 = src[0], x1 = src[ms];
            if (te) x1 = cmul(x1, twiddle<INV>(tw, te));
            dst[0] = cadd(x0, x1);
            dst[ps] = csub(x0, x1);
        } else if (r == 3) {
            float2 x0 = src[0], x1 = src[ms], x2 = src[2 * ms];
            if (te) {
                x1 = cmul(x1, twiddle<INV>(tw, te));
                x2 = cmul(x2, twiddle<INV>(tw, 2 * te));
            }
            const float h = 0.866025403784438647f;   // sqrt(3)/2
            float2 s = cadd(x1, x2), d = csub(x1, x2);
            float2 t = make_float2(x0.x - 0.5f * s.x, x0.y - 0.5f * s.y);
            // forward: y1 = t - i h d, y2 = t + i h d
            float2 ihd = INV ? make_float2(-h * d.y, h * d.x) : make_float2(h * d.y, -h * d.x);
            dst[0] = cadd(x0, s);
            dst[ps] = cadd(t, ihd);
            dst[2 * ps] = csub(t, ihd);
        }
    }
}

// Full transform of L lines held in a; returns the buffer holding the result.
template <bool INV>
__device__ float2* fft_lines(float2* a, float2* b, int L, int LS, int ES, bool line_fastest,
                             const AxisPlan& pl, const float2* tw)
{
    int p = 1;
    for (int s = 0; s < pl.ns; ++s) {
        const int r = pl.radix[s];
        fft_stage<INV>(a, b, L, LS, ES, line_fastest, pl.n, r, p, tw);
        __syncthreads();
        p *= r;
        float2* t = a; a = b; b = t;
    }
    return a;
}

// Pass over x rows: rows_per_cta consecutive rows (one contiguous block).
template <bool INV, int EPI>
__global__ void __launch_bounds__(kThreads) k_rows(const float2* __restrict__ src, float2* __restrict__ dst,
                                                   Geometry g, AxisPlan pl, const float2* __restrict__ twg,
                                                   int rows_per_cta, EpiArgs e)
{
    extern __shared__ float4 smem4[];
    float2* sm = reinterpret_cast<float2*>(smem4);
    const int n = pl.n;
    const long long nrows = (long long)g.nyb * g.nzb;
    const long long row0 = (long long)blockIdx.x * rows_per_cta;
    const int rows = (int)min((long long)rows_per_cta, nrows - row0);
    float2* tw = sm;
    float2* A = sm + n;
    float2* B = A + (size_t)rows_per_cta * n;
    for (int t = threadIdx.x; t < n; t += blockDim.x) tw[t] = twg[t];
    const int nv = rows * n / 2;   // float4 = two complex values; n is even
    const float4* s4 = reinterpret_cast<const float4*>(src + row0 * n);
    float4* A4 = reinterpret_cast<float4*>(A);
    for (int t = threadIdx.x; t < nv; t += blockDim.x) A4[t] = s4[t];
    __syncthreads();
    float2* R = fft_lines<INV>(A, B, rows, n, 1, false, pl, tw);
    if (EPI == EPI_NONE) {
        float4* d4 = reinterpret_cast<float4*>(dst + row0 * n);
        const float4* R4 = reinterpret_cast<const float4*>(R);
        for (int t = threadIdx.x; t < nv; t += blockDim.x) d4[t] = R4[t];
    } else {
        for (int t = threadIdx.x; t < rows * n; t += blockDim.x) {
            const int r = t / n, x = t - r * n;
            const long long row = row0 + r;
            const int y = (int)(row % g.nyb), z = (int)(row / g.nyb);
            epilogue<EPI>(row0 * n + t, x, y, z, R[t], e);
        }
    }
}

// Pass over lines of stride `stride` (y: nxb, z: nxb*nyb); a CTA takes TX
// neighbouring x columns so every global access is a TX-wide row segment.
// KSCALE: forward, * |k|, inverse (the z pass).
template <bool INV, bool KSCALE>
__global__ void __launch_bounds__(kThreads) k_lines(float2* __restrict__ data, Geometry g, AxisPlan pl,
                                                    const float2* __restrict__ twg, int TX,
                                                    long long stride, Tables tb)
{
    extern __shared__ float4 smem4[];
    float2* sm = reinterpret_cast<float2*>(smem4);
    const int n = pl.n;
    float2* tw = sm;
    float2* A = sm + n;
    float2* B = A + (size_t)n * TX;
    const int x0 = blockIdx.x * TX;
    const int cols = min(TX, g.nxb - x0);
    // blockIdx.y: the other index (z for the y pass, y for the z pass)
    const long long base = KSCALE ? (long long)blockIdx.y * g.nxb + x0
                                  : (long long)blockIdx.y * g.nyb * g.nxb + x0;
    for (int t = threadIdx.x; t < n; t += blockDim.x) tw[t] = twg[t];
    for (int t = threadIdx.x; t < n * TX; t += blockDim.x) {
        const int e = t / TX, c = t - e * TX;
        A[t] = c < cols ? data[base + e * stride + c] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    float2* R;
    if (KSCALE) {
        R = fft_lines<false>(A, B, TX, 1, TX, true, pl, tw);
        float2* O = R == A ? B : A;
        const float ky2 = tb.ky2[blockIdx.y];
        for (int t = threadIdx.x; t < n * TX; t += blockDim.x) {
            const int z = t / TX, c = t - z * TX;
            const float kx2 = c < cols ? tb.kx2[x0 + c] : 0.f;
            R[t] = cscale(R[t], sqrtf(kx2 + ky2 + tb.kz2[z]));
        }
        __syncthreads();
        R = fft_lines<true>(R, O, TX, 1, TX, true, pl, tw);
    } else {
        R = fft_lines<INV>(A, B, TX, 1, TX, true, pl, tw);
    }
    for (int t = threadIdx.x; t < n * TX; t += blockDim.x) {
        const int e = t / TX, c = t - e * TX;
        if (c < cols) data[base + e * stride + c] = R[t];
    }
}

int rows_per_cta(int n) { return n >= 2048 ? 1 : 2048 / n; }
// 8 columns (64-byte row segments): on 384 x 384 x 256 and 320 x 288 x 256
// the autotuner of the batched form picks 8 over 16 for both column passes.
int tile_x(int) { return 8; }

// The register column kernels (ose_cols.cu) where the length allows, unless
// OSE3D_COLS=stockham asks for the shared-memory Stockham passes (comparison).
bool use_col_kernels()
{
    static int v = -1;
    if (v < 0) {
        const char* e = getenv("OSE3D_COLS");
        v = (e && strcmp(e, "stockham") == 0) ? 0 : 1;
    }
    return v == 1;
}
size_t rows_smem(int n) { return sizeof(float2) * ((size_t)n + 2 * (size_t)rows_per_cta(n) * n); }
size_t lines_smem(int n) { return sizeof(float2) * ((size_t)n + 2 * (size_t)n * tile_x(n)); }

template <typename K>
cudaError_t allow_smem(K k)
{
    return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
}

struct Timer {
    KernelTiming* t;
    cudaStream_t s;
    int cls;
    Timer(KernelTiming* tt, cudaStream_t ss, int c) : t(tt), s(ss), cls(c)
    {
        if (t) cudaEventRecord(t->ev[0], s);
    }
    void done()
    {
        if (!t) return;
        cudaEventRecord(t->ev[1], s);
        cudaEventSynchronize(t->ev[1]);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, t->ev[0], t->ev[1]);
        t->ms[cls] += ms;
        t->count[cls] += 1;
    }
};

}  // namespace

cudaError_t configure_kernels()
{
    cudaError_t e;
#define ALLOW(k) if ((e = allow_smem(k)) != cudaSuccess) return e
    ALLOW((k_rows<false, EPI_NONE>));
    ALLOW((k_rows<true, EPI_FIRST>));
    ALLOW((k_rows<true, EPI_MID>));
    ALLOW((k_rows<true, EPI_LAST>));
    ALLOW((k_rows<true, EPI_SCALE>));
    ALLOW((k_rows<true, EPI_SCALE_VEL>));
    ALLOW((k_lines<false, false>));
    ALLOW((k_lines<true, false>));
    ALLOW((k_lines<false, true>));
#undef ALLOW
    return cudaSuccess;
}

// Timing classes of the generic path.
// T_XI_NOSUM: the x inverse + epilogue passes that leave the partial sum alone.
enum { T_XF = 0, T_YF = 1, T_ZK = 2, T_YI = 3, T_XI = 4, T_INJ = 5, T_XI_NOSUM = 8 };

// x_ready: X already holds the forward x transform of a_n (written by the
// previous application's fused row pass), so pass 1 is skipped.
static cudaError_t passes_1_to_4(cudaStream_t s, const Geometry& g, const AxisPlan& px,
                                 const AxisPlan& py, const AxisPlan& pz, const Tables& t,
                                 const float2* an, float2* X, KernelTiming* tm, bool x_ready = false)
{
    EpiArgs none{};
    const long long nrows = (long long)g.nyb * g.nzb;
    if (!x_ready) {
        Timer T(tm, s, T_XF);
        if (t.bl[0]) {
            cudaError_t e = launch_row_bluestein(s, EPI_NONE, px.n, an, X, g.nyb, nrows, t, none);
            if (e != cudaSuccess) return e;
        } else if (use_col_kernels() && col_supported(px.n)) {
            cudaError_t e = launch_row(s, EPI_NONE, px.n, an, X, g.nyb, nrows, t.twx, none);
            if (e != cudaSuccess) return e;
        } else {
            const int rpc = rows_per_cta(px.n);
            k_rows<false, EPI_NONE><<<(unsigned)((nrows + rpc - 1) / rpc), kThreads, rows_smem(px.n), s>>>(
                an, X, g, px, t.twx, rpc, none);
        }
        T.done();
    }
    const long long plane = (long long)g.nxb * g.nyb;
    const bool ycols = use_col_kernels() && col_supported(py.n);
    const bool zcols = use_col_kernels() && col_supported(pz.n);
    {
        Timer T(tm, s, T_YF);
        if (t.bl[1]) {
            cudaError_t e = launch_col_bluestein(s, 0, py.n, X, g.nxb, g.nzb, g.nxb, plane, 1, t);
            if (e != cudaSuccess) return e;
        } else if (ycols) {
            cudaError_t e = launch_col(s, 0, py.n, X, g.nxb, g.nzb, g.nxb, plane, t.twy, t);
            if (e != cudaSuccess) return e;
        } else {
            const int tx = tile_x(py.n);
            dim3 grid((g.nxb + tx - 1) / tx, g.nzb);
            k_lines<false, false><<<grid, kThreads, lines_smem(py.n), s>>>(X, g, py, t.twy, tx, g.nxb, t);
        }
        T.done();
    }
    {
        Timer T(tm, s, T_ZK);
        if (t.tcvar != OSE_PRECISION_FP32) {
            cudaError_t e = launch_tensor_zpass(s, X, g, t);
            if (e != cudaSuccess) return e;
        } else if (use_col_kernels() && zpass256_supported(g)) {
            cudaError_t e = launch_zpass256(s, X, g, t);
            if (e != cudaSuccess) return e;
        } else if (t.bl[2]) {
            cudaError_t e = launch_col_bluestein(s, 2, pz.n, X, g.nxb, g.nyb, plane, g.nxb, 2, t);
            if (e != cudaSuccess) return e;
        } else if (zcols) {
            cudaError_t e = launch_col(s, 2, pz.n, X, g.nxb, g.nyb, plane, g.nxb, t.twz, t);
            if (e != cudaSuccess) return e;
        } else {
            const int tx = tile_x(pz.n);
            dim3 grid((g.nxb + tx - 1) / tx, g.nyb);
            k_lines<false, true><<<grid, kThreads, lines_smem(pz.n), s>>>(X, g, pz, t.twz, tx, plane, t);
        }
        T.done();
    }
    {
        Timer T(tm, s, T_YI);
        if (t.bl[1]) {
            cudaError_t e = launch_col_bluestein(s, 1, py.n, X, g.nxb, g.nzb, g.nxb, plane, 1, t);
            if (e != cudaSuccess) return e;
        } else if (ycols) {
            cudaError_t e = launch_col(s, 1, py.n, X, g.nxb, g.nzb, g.nxb, plane, t.twy, t);
            if (e != cudaSuccess) return e;
        } else {
            const int tx = tile_x(py.n);
            dim3 grid((g.nxb + tx - 1) / tx, g.nzb);
            k_lines<true, false><<<grid, kThreads, lines_smem(py.n), s>>>(X, g, py, t.twy, tx, g.nxb, t);
        }
        T.done();
    }
    return cudaGetLastError();
}

bool generic_fuses_x(const AxisPlan& px, const Tables& t)
{
    return t.bl[0] != 0 || (use_col_kernels() && col_supported(px.n));
}

cudaError_t launch_generic_application(cudaStream_t s, const Geometry& g, const AxisPlan& px,
                                       const AxisPlan& py, const AxisPlan& pz, const Tables& t,
                                       const float2* an, float2* X, EpiMode mode, const EpiArgs& e,
                                       KernelTiming* tm, bool x_ready, bool fwd_next)
{
    const bool fuse = generic_fuses_x(px, t);
    cudaError_t err = passes_1_to_4(s, g, px, py, pz, t, an, X, tm, fuse && x_ready);
    if (err != cudaSuccess) return err;
    const long long nrows = (long long)g.nyb * g.nzb;
    const int rpc = rows_per_cta(px.n);
    const unsigned nb = (unsigned)((nrows + rpc - 1) / rpc);
    Timer T(tm, s, (mode != EPI_LAST && !e.sp.touch) ? T_XI_NOSUM : T_XI);
    if (fuse) {
        int epi = (int)mode;
        if (fwd_next && mode == EPI_FIRST) epi = EPI_FIRST_FWD;
        if (fwd_next && mode == EPI_MID) epi = EPI_MID_FWD;
        err = t.bl[0] ? launch_row_bluestein(s, epi, px.n, X, X, g.nyb, nrows, t, e)
                      : launch_row(s, epi, px.n, X, X, g.nyb, nrows, t.twx, e);
        T.done();
        return err;
    }
    switch (mode) {
    case EPI_FIRST:
        k_rows<true, EPI_FIRST><<<nb, kThreads, rows_smem(px.n), s>>>(X, nullptr, g, px, t.twx, rpc, e);
        break;
    case EPI_MID:
        k_rows<true, EPI_MID><<<nb, kThreads, rows_smem(px.n), s>>>(X, nullptr, g, px, t.twx, rpc, e);
        break;
    default:
        k_rows<true, EPI_LAST><<<nb, kThreads, rows_smem(px.n), s>>>(X, nullptr, g, px, t.twx, rpc, e);
        break;
    }
    T.done();
    return cudaGetLastError();
}

cudaError_t launch_apply_operator(cudaStream_t s, const Geometry& g, const AxisPlan& px,
                                  const AxisPlan& py, const AxisPlan& pz, const Tables& t,
                                  const float2* in, float2* X, float2* out, const float* vs,
                                  float sch, float scl)
{
    cudaError_t err = passes_1_to_4(s, g, px, py, pz, t, in, X, nullptr);
    if (err != cudaSuccess) return err;
    EpiArgs e{};
    e.prev = out;
    e.vs = vs;
    e.sch = sch;
    e.scl = scl;
    const long long nrows = (long long)g.nyb * g.nzb;
    if (t.bl[0]) return launch_row_bluestein(s, EPI_SCALE, px.n, X, nullptr, g.nyb, nrows, t, e);
    if (use_col_kernels() && col_supported(px.n)) return launch_row(s, EPI_SCALE, px.n, X, nullptr, g.nyb, nrows, t.twx, e);
    const int rpc = rows_per_cta(px.n);
    k_rows<true, EPI_SCALE><<<(unsigned)((nrows + rpc - 1) / rpc), kThreads, rows_smem(px.n), s>>>(
        X, nullptr, g, px, t.twx, rpc, e);
    return cudaGetLastError();
}

// Source injection of one step (Xt_add_wavelet_sxyz x2, ose_3d_lib.cu:610-633):
// the step index lives in device memory (ctr[0] = next step, ctr[1] = current)
// so a captured graph can replay it.
__global__ void k_inject(float2* W, long long src, const float* ricker, const float* hil, int* ctr, int nt)
{
    // launched with launch_pdl: the step's first transform may start its
    // table loads meanwhile; everything here comes after the wait
    griddep_launch();
    griddep_wait();
    const int it = ctr[0];
    ctr[1] = it;
    ctr[0] = it + 1;
    if (it >= 0 && it < nt) {
        float2 w = W[src];
        w.x += ricker[it];
        w.y += hil[it];
        W[src] = w;
    }
}

cudaError_t launch_inject(cudaStream_t s, float2* W, long long src, const float* ricker,
                          const float* hil, int* ctr, int nt)
{
    return launch_pdl(k_inject, dim3(1), dim3(1), 0, s, W, src, ricker, hil, ctr, nt);
}

/* ---- batched shots ---------------------------------------------------------
 * The same passes for many shots of different sizes in one launch per pass:
 * CTA b works on block work[b].y of shot work[b].x and reads that shot's
 * geometry, radix plans, tables and buffers from the BatchShot array.  The
 * device code per block is the single-shot code above, so a batched shot
 * computes exactly what a single-shot handle with the same plans computes. */

namespace {

// x rows of application n: forward (a_n -> X) or inverse + the series update.
template <bool INV>
__global__ void __launch_bounds__(kThreads) kb_rows(const BatchShot* __restrict__ shots,
                                                    const int2* __restrict__ work, int n)
{
    extern __shared__ float4 smem4[];
    float2* sm = reinterpret_cast<float2*>(smem4);
    const int2 wk = work[blockIdx.x];
    const BatchShot& S = shots[wk.x];
    const int nn = S.px.n, rpc = S.rpc;
    const long long nrows = (long long)S.g.nyb * S.g.nzb;
    const long long row0 = (long long)wk.y * rpc;
    const int rows = (int)min((long long)rpc, nrows - row0);
    float2* tw = sm;
    float2* A = sm + nn;
    float2* B = A + (size_t)rpc * nn;
    for (int t = threadIdx.x; t < nn; t += blockDim.x) tw[t] = S.twx[t];
    const float2* src = INV ? S.X : (n == 0 ? S.W : ((n & 1) ? S.A : S.W));
    const int nv = rows * nn / 2;
    const float4* s4 = reinterpret_cast<const float4*>(src + row0 * nn);
    float4* A4 = reinterpret_cast<float4*>(A);
    for (int t = threadIdx.x; t < nv; t += blockDim.x) A4[t] = s4[t];
    __syncthreads();
    float2* R = fft_lines<INV>(A, B, rows, nn, 1, false, S.px, tw);
    if (!INV) {
        float4* d4 = reinterpret_cast<float4*>(S.X + row0 * nn);
        const float4* R4 = reinterpret_cast<const float4*>(R);
        for (int t = threadIdx.x; t < nv; t += blockDim.x) d4[t] = R4[t];
        return;
    }
    const EpiArgs e = batch_epi(S, n);
    const int mode = n == 0 ? EPI_FIRST : (n == S.M ? EPI_LAST : EPI_MID);
    for (int t = threadIdx.x; t < rows * nn; t += blockDim.x) {
        const int r = t / nn, x = t - r * nn;
        const long long row = row0 + r;
        const int y = (int)(row % S.g.nyb), z = (int)(row / S.g.nyb);
        const long long i = row0 * nn + t;
        if (mode == EPI_FIRST) epilogue<EPI_FIRST>(i, x, y, z, R[t], e);
        else if (mode == EPI_MID) epilogue<EPI_MID>(i, x, y, z, R[t], e);
        else epilogue<EPI_LAST>(i, x, y, z, R[t], e);
    }
}

// y lines (AXIS 1) or z lines (AXIS 2, forward * |k| inverse) of one shot's
// x tile; block = x tile + (number of x tiles) * (z for y lines, y for z lines).
template <int AXIS, bool INV>
__global__ void __launch_bounds__(kThreads) kb_lines(const BatchShot* __restrict__ shots,
                                                     const int2* __restrict__ work)
{
    extern __shared__ float4 smem4[];
    float2* sm = reinterpret_cast<float2*>(smem4);
    const int2 wk = work[blockIdx.x];
    const BatchShot& S = shots[wk.x];
    const AxisPlan& pl = AXIS == 1 ? S.py : S.pz;
    const int n = pl.n;
    const int TX = AXIS == 1 ? S.txy : S.txz;
    const int ntx = (S.g.nxb + TX - 1) / TX;
    const int xt = wk.y % ntx, other = wk.y / ntx;
    const int x0 = xt * TX;
    const int cols = min(TX, S.g.nxb - x0);
    const long long stride = AXIS == 1 ? (long long)S.g.nxb : (long long)S.g.nxb * S.g.nyb;
    const long long base = AXIS == 1 ? (long long)other * S.g.nyb * S.g.nxb + x0 : (long long)other * S.g.nxb + x0;
    const float2* twg = AXIS == 1 ? S.twy : S.twz;
    float2* tw = sm;
    float2* A = sm + n;
    float2* B = A + (size_t)n * TX;
    float2* data = S.X;
    for (int t = threadIdx.x; t < n; t += blockDim.x) tw[t] = twg[t];
    for (int t = threadIdx.x; t < n * TX; t += blockDim.x) {
        const int el = t / TX, c = t - el * TX;
        A[t] = c < cols ? data[base + el * stride + c] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    float2* R;
    if (AXIS == 2) {
        R = fft_lines<false>(A, B, TX, 1, TX, true, pl, tw);
        float2* O = R == A ? B : A;
        const float ky2 = S.ky2[other];
        for (int t = threadIdx.x; t < n * TX; t += blockDim.x) {
            const int z = t / TX, c = t - z * TX;
            const float kx2 = c < cols ? S.kx2[x0 + c] : 0.f;
            R[t] = cscale(R[t], sqrtf(kx2 + ky2 + S.kz2[z]));
        }
        __syncthreads();
        R = fft_lines<true>(R, O, TX, 1, TX, true, pl, tw);
    } else {
        R = fft_lines<INV>(A, B, TX, 1, TX, true, pl, tw);
    }
    for (int t = threadIdx.x; t < n * TX; t += blockDim.x) {
        const int el = t / TX, c = t - el * TX;
        if (c < cols) data[base + el * stride + c] = R[t];
    }
}

__global__ void kb_inject(const BatchShot* __restrict__ shots, int nshots)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nshots) return;
    const BatchShot& S = shots[s];
    const int it = S.ctr[0];
    S.ctr[1] = it;
    S.ctr[0] = it + 1;
    if (it >= 0 && it < S.nt) {
        float2 w = S.W[S.src];
        w.x += S.ricker[it];
        w.y += S.hil[it];
        S.W[S.src] = w;
    }
}

}  // namespace

size_t batch_rows_smem(int n, int rpc) { return sizeof(float2) * ((size_t)n + 2 * (size_t)rpc * n); }
size_t batch_lines_smem(int n, int tx) { return sizeof(float2) * ((size_t)n + 2 * (size_t)n * tx); }

cudaError_t configure_batch_kernels()
{
    cudaError_t e;
#define ALLOW(k) if ((e = allow_smem(k)) != cudaSuccess) return e
    ALLOW((kb_rows<false>));
    ALLOW((kb_rows<true>));
    ALLOW((kb_lines<1, false>));
    ALLOW((kb_lines<1, true>));
    ALLOW((kb_lines<2, false>));
#undef ALLOW
    return cudaSuccess;
}

cudaError_t launch_batch_inject(cudaStream_t s, const BatchShot* shots, int nshots)
{
    kb_inject<<<(nshots + 127) / 128, 128, 0, s>>>(shots, nshots);
    return cudaGetLastError();
}

cudaError_t launch_batch_stockham_pass(cudaStream_t s, const BatchShot* shots, int n, const BatchPass& p)
{
    if (p.nblocks <= 0) return cudaSuccess;
    switch (p.kind) {
    case 0: kb_rows<false><<<p.nblocks, kThreads, p.smem, s>>>(shots, p.work, n); break;
    case 1: kb_lines<1, false><<<p.nblocks, kThreads, p.smem, s>>>(shots, p.work); break;
    case 2: kb_lines<2, false><<<p.nblocks, kThreads, p.smem, s>>>(shots, p.work); break;
    case 3: kb_lines<1, true><<<p.nblocks, kThreads, p.smem, s>>>(shots, p.work); break;
    default: kb_rows<true><<<p.nblocks, kThreads, p.smem, s>>>(shots, p.work, n); break;
    }
    return cudaGetLastError();
}

// The generic operator for callers that hold a plain velocity array and pass
// the scale: out = vel * scale * IFFT3(|k| FFT3(in)).
// X is caller-provided scratch of one field.
cudaError_t launch_apply_operator_vel(cudaStream_t s, const Geometry& g, const AxisPlan& px,
                                      const AxisPlan& py, const AxisPlan& pz, const Tables& t,
                                      const float2* in, float2* X, float2* out, const float* vel,
                                      double scale)
{
    cudaError_t err = passes_1_to_4(s, g, px, py, pz, t, in, X, nullptr);
    if (err != cudaSuccess) return err;
    EpiArgs e{};
    e.prev = out;
    e.vs = vel;
    split_float(scale, &e.sch, &e.scl);
    const long long nrows = (long long)g.nyb * g.nzb;
    if (use_col_kernels() && col_supported(px.n))
        return launch_row(s, EPI_SCALE_VEL, px.n, X, nullptr, g.nyb, nrows, t.twx, e);
    const int rpc = rows_per_cta(px.n);
    k_rows<true, EPI_SCALE_VEL><<<(unsigned)((nrows + rpc - 1) / rpc), kThreads, rows_smem(px.n), s>>>(
        X, nullptr, g, px, t.twx, rpc, e);
    return cudaGetLastError();
}

}  // namespace ose
