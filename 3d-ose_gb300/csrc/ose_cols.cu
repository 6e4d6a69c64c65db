// ose_cols.cu - column transforms of the generic path held in registers: the
// y passes (forward, inverse) and the z pass (forward, * |k|, inverse) for a
// line length N = 16 C, C in OSE_COL_SIZES (below).
//
// A line is a 16 x C matrix (four-step, n = C n1 + j, k = p + 16 k2):
//   phase 1  thread j < C holds x[C n1 + j], n1 < 16: DFT-16, twiddle W_N^(j p)
//   transpose through shared memory
//   phase 2  thread p < 16 holds the j < C values: DFT-C -> X[p + 16 k2]
// and the inverse runs the same steps backwards.  The DFTs are in registers:
// DFT-C by compile-time mixed radix (radix 4 first, then the smallest prime
// factor; direct sums for primes), its twiddles W_N^t from a table in shared
// memory.  A CTA holds TX neighbouring x columns of one line family, so every
// global access is a TX-wide row segment.  The x passes (k_row) use the same
// two phases on contiguous rows, RW rows per CTA; the inverse x pass ends in
// the step's pointwise epilogue.  These replace the shared-memory Stockham
// passes (ose_kernels.cu) on these sizes.
#include <cuda_runtime.h>

#include <algorithm>
#include <math.h>

#include "ose_dft.cuh"
#include "ose_epilogue.cuh"
#include "ose_internal.h"

namespace ose {
namespace cols {

enum { COL_FWD = 0, COL_INV = 1, COL_KSCALE = 2 };

template <int C>
struct ColCfg {
    static constexpr int N = 16 * C;
    static constexpr int P = C > 16 ? C : 16;      // line threads
    static constexpr int TX = P > 16 ? 8 : 16;     // columns per CTA
    static constexpr int THREADS = TX * P;
    static constexpr size_t SMEM = sizeof(float2) * ((size_t)N + (size_t)N * TX);
    // CTAs per SM asked of the register allocator: about 80 registers a thread
    static constexpr int MINB = C == 23 ? 1 : 65536 / (THREADS * 80);
};

// Lines at base + n * stride of the columns x0 .. x0 + TX - 1 (x tile xt);
// `other` = the other index (z for the y passes, y for the z pass).
// W: shared twiddle table (N), T: shared transpose buffer (N x TX).
// COHERENT: column loads bypass the SM's L1 (as row_body's).
template <int C, int MODE, bool COHERENT = false>
__device__ __forceinline__ void col_body(float2* __restrict__ X, int nxb, long long stride, long long ostride,
                                         const float2* __restrict__ twg, const float* __restrict__ kx2,
                                         const float* __restrict__ ky2, const float* __restrict__ kz2, int xt,
                                         int other, float2* W, float2* T)
{
    using K = ColCfg<C>;
    constexpr int N = K::N, TX = K::TX;
    for (int i = threadIdx.x; i < N; i += K::THREADS) W[i] = twg[i];
    const int c = threadIdx.x % TX, p = threadIdx.x / TX;
    const int x = xt * TX + c;
    const bool col_ok = x < nxb;
    float2* line = X + (size_t)other * ostride + x;
    __syncthreads();

    if (MODE == COL_FWD || MODE == COL_KSCALE) {
        if (p < C) {   // phase 1: thread j = p, DFT-16 over n1
            float2 v[16];
#pragma unroll
            for (int n1 = 0; n1 < 16; ++n1) {
                const float2* a = line + (size_t)(C * n1 + p) * stride;
                v[n1] = col_ok ? (COHERENT ? __ldcg(a) : *a) : make_float2(0.f, 0.f);
            }
            dftc<16, C, false>(v, W);
#pragma unroll
            for (int k1 = 0; k1 < 16; ++k1) T[(p * 16 + k1) * TX + c] = k1 ? cmul(v[k1], W[p * k1]) : v[k1];
        }
        __syncthreads();
    }
    float2 u[C];
    if (p < 16) {
        if (MODE == COL_INV) {
#pragma unroll
            for (int k2 = 0; k2 < C; ++k2) {
                const float2* a = line + (size_t)(p + 16 * k2) * stride;
                u[k2] = col_ok ? (COHERENT ? __ldcg(a) : *a) : make_float2(0.f, 0.f);
            }
        } else {
#pragma unroll
            for (int j = 0; j < C; ++j) u[j] = T[(j * 16 + p) * TX + c];
            dftc<C, 16, false>(u, W);   // u[k2] = X[p + 16 k2]
        }
        if (MODE == COL_FWD) {
            if (col_ok)
#pragma unroll
                for (int k2 = 0; k2 < C; ++k2) line[(size_t)(p + 16 * k2) * stride] = u[k2];
        } else {
            if (MODE == COL_KSCALE) {
                // z pass: other is y, x the column
                const float kxy = col_ok ? __ldg(kx2 + x) + __ldg(ky2 + other) : 0.f;
#pragma unroll
                for (int k2 = 0; k2 < C; ++k2) {
                    const float k = sqrtf(kxy + __ldg(kz2 + p + 16 * k2));
                    u[k2].x *= k;
                    u[k2].y *= k;
                }
            }
            dftc<C, 16, true>(u, W);   // u[j] = Z[p][j]
#pragma unroll
            for (int j = 0; j < C; ++j) {
                const float2 w = W[j * p];
                T[(j * 16 + p) * TX + c] = (j * p) ? cmul(u[j], make_float2(w.x, -w.y)) : u[j];
            }
        }
    }
    if (MODE == COL_FWD) return;
    __syncthreads();
    if (p < C) {   // inverse phase 1: thread j = p, DFT-16 over p'
        float2 v[16];
#pragma unroll
        for (int k1 = 0; k1 < 16; ++k1) v[k1] = T[(p * 16 + k1) * TX + c];
        dftc<16, C, true>(v, W);
        if (col_ok)
#pragma unroll
            for (int n1 = 0; n1 < 16; ++n1) line[(size_t)(C * n1 + p) * stride] = v[n1];
    }
}

template <int C, int MODE>
__global__ void __launch_bounds__(ColCfg<C>::THREADS, ColCfg<C>::MINB) k_col(float2* __restrict__ X, int nxb, long long stride,
                                                            long long ostride, const float2* __restrict__ twg,
                                                            Tables tb)
{
    extern __shared__ float4 smem4[];
    float2* W = reinterpret_cast<float2*>(smem4);
    col_body<C, MODE>(X, nxb, stride, ostride, twg, tb.kx2, tb.ky2, tb.kz2, blockIdx.x, blockIdx.y, W,
                      W + ColCfg<C>::N);
}

// Batched: CTA b works on block work[b].y = x tile + (x tiles) * other of
// shot work[b].x; AXIS 1 = y lines, 2 = z lines.
template <int C, int MODE, int AXIS, bool COHERENT = false>
__device__ __forceinline__ void kb_col_item(const BatchShot* __restrict__ shots, int2 wk, float2* W)
{
    const BatchShot& S = shots[wk.x];
    const int ntx = (S.g.nxb + ColCfg<C>::TX - 1) / ColCfg<C>::TX;
    const int xt = wk.y % ntx, other = wk.y / ntx;
    const long long plane = (long long)S.g.nxb * S.g.nyb;
    if (AXIS == 1)
        col_body<C, MODE, COHERENT>(S.X, S.g.nxb, S.g.nxb, plane, S.twy, S.kx2, S.ky2, S.kz2, xt, other, W,
                                    W + ColCfg<C>::N);
    else
        col_body<C, MODE, COHERENT>(S.X, S.g.nxb, plane, S.g.nxb, S.twz, S.kx2, S.ky2, S.kz2, xt, other, W,
                                    W + ColCfg<C>::N);
}

template <int C, int MODE, int AXIS>
__global__ void __launch_bounds__(ColCfg<C>::THREADS, ColCfg<C>::MINB) kb_col(const BatchShot* __restrict__ shots,
                                                             const int2* __restrict__ work)
{
    extern __shared__ float4 smem4[];
    kb_col_item<C, MODE, AXIS>(shots, work[blockIdx.x], reinterpret_cast<float2*>(smem4));
}

template <int C>
struct RowCfg {
    static constexpr int N = 16 * C;
    static constexpr int P = C > 16 ? C : 16;      // line threads
    static constexpr int RW = P > 16 ? 8 : 16;     // rows per CTA
    static constexpr int THREADS = RW * P;
    static constexpr int NP = 17 * C;              // padded row of the transpose buffer
    static constexpr size_t SMEM = sizeof(float2) * ((size_t)N + (size_t)RW * NP);
    // CTAs per SM asked of the register allocator: 4 where a CTA has at most
    // 160 threads (C = 18, 20: 96 registers, a few spilled in the epilogue
    // instances; 320 x 288 x 256 measured 4.41 -> 4.36 ms per step against
    // three CTAs at 111-115 registers); none otherwise
    static constexpr int MINB = THREADS <= 160 ? 4 : 0;
};

// x rows (contiguous, row = z * nyb + y) of row block rb.  EPI_NONE: forward
// transform of src into dst.  Otherwise: inverse transform of src followed by
// epilogue<EPI>; FWD (FIRST, MID): then the forward transform of the new term
// a_{n+1}, still in registers, into dst (the next application's x pass; each
// row is read before it is written, by the same CTA).
// COHERENT: the rows are read with loads that bypass the SM's L1 (the
// persistent kernel reads fields other CTAs wrote earlier in the same launch).
template <int C, int EPI, bool FWD = false, bool COHERENT = false>
__device__ __forceinline__ void row_body(const float2* __restrict__ src, float2* __restrict__ dst, int nyb,
                                         long long nrows, const float2* __restrict__ twg, const EpiArgs& e,
                                         long long rb, float2* W, float2* T)
{
    using K = RowCfg<C>;
    constexpr int N = K::N, P = K::P, NP = K::NP;
    for (int i = threadIdx.x; i < N; i += K::THREADS) W[i] = twg[i];
    const int r = threadIdx.x / P, q = threadIdx.x % P;
    const long long row = rb * K::RW + r;
    const bool ok = row < nrows;
    float2* Tr = T + r * NP;
    __syncthreads();
    if (EPI == EPI_NONE) {
        if (q < C) {   // phase 1: thread j = q, DFT-16 over n1
            float2 v[16];
            const float2* in = src + row * N + q;
#pragma unroll
            for (int n1 = 0; n1 < 16; ++n1)
                v[n1] = ok ? (COHERENT ? __ldcg(in + C * n1) : in[C * n1]) : make_float2(0.f, 0.f);
            dftc<16, C, false>(v, W);
#pragma unroll
            for (int k1 = 0; k1 < 16; ++k1) Tr[q * 17 + k1] = k1 ? cmul(v[k1], W[q * k1]) : v[k1];
        }
        __syncthreads();
        if (q < 16 && ok) {   // phase 2: thread p = q, DFT-C over j
            float2 u[C];
#pragma unroll
            for (int j = 0; j < C; ++j) u[j] = Tr[j * 17 + q];
            dftc<C, 16, false>(u, W);
            float2* out = dst + row * N + q;
#pragma unroll
            for (int k2 = 0; k2 < C; ++k2) out[16 * k2] = u[k2];
        }
    } else {
        if (q < 16) {   // inverse phase 2: thread p = q holds X[p + 16 k2]
            float2 u[C];
            const float2* in = src + row * N + q;
#pragma unroll
            for (int k2 = 0; k2 < C; ++k2)
                u[k2] = ok ? (COHERENT ? __ldcg(in + 16 * k2) : in[16 * k2]) : make_float2(0.f, 0.f);
            dftc<C, 16, true>(u, W);
#pragma unroll
            for (int j = 0; j < C; ++j) {
                const float2 w = W[j * q];
                Tr[j * 17 + q] = (j * q) ? cmul(u[j], make_float2(w.x, -w.y)) : u[j];
            }
        }
        __syncthreads();
        if (q < C && ok) {   // inverse phase 1: thread j = q -> x[C n1 + j]
            float2 v[16];
#pragma unroll
            for (int k1 = 0; k1 < 16; ++k1) v[k1] = Tr[q * 17 + k1];
            dftc<16, C, true>(v, W);
            const int y = (int)(row % nyb), z = (int)(row / nyb);
            epilogue_row<EPI, 16, FWD, COHERENT>(v, row * N + q, q, C, y, z, e);
            if (FWD) {   // forward phase 1 of a_{n+1} (v[n1] = a[C n1 + j]); thread q owns Tr row q
                dftc<16, C, false>(v, W);
#pragma unroll
                for (int k1 = 0; k1 < 16; ++k1) Tr[q * 17 + k1] = k1 ? cmul(v[k1], W[q * k1]) : v[k1];
            }
        }
        if (FWD) {
            __syncthreads();
            if (q < 16 && ok) {   // forward phase 2
                float2 u[C];
#pragma unroll
                for (int j = 0; j < C; ++j) u[j] = Tr[j * 17 + q];
                dftc<C, 16, false>(u, W);
                float2* out = dst + row * N + q;
#pragma unroll
                for (int k2 = 0; k2 < C; ++k2) out[16 * k2] = u[k2];
            }
        }
    }
}

template <int C, int EPI, bool FWD = false>
__global__ void __launch_bounds__(RowCfg<C>::THREADS, RowCfg<C>::MINB) k_row(const float2* __restrict__ src, float2* __restrict__ dst,
                                                            int nyb, long long nrows, const float2* __restrict__ twg,
                                                            EpiArgs e)
{
    extern __shared__ float4 smem4[];
    float2* W = reinterpret_cast<float2*>(smem4);
    row_body<C, EPI, FWD>(src, dst, nyb, nrows, twg, e, blockIdx.x, W, W + RowCfg<C>::N);
}

// Batched x rows of application n: forward (a_n -> X) or inverse + the series
// update (FIRST, MID or LAST by the shot's series order M).
template <int C, bool INV, bool COHERENT = false>
__device__ __forceinline__ void kb_row_item(const BatchShot* __restrict__ shots, int2 wk, int n, float2* W)
{
    float2* T = W + RowCfg<C>::N;
    const BatchShot& S = shots[wk.x];
    const long long nrows = (long long)S.g.nyb * S.g.nzb;
    if (!INV) {
        const float2* src = n == 0 ? S.W : ((n & 1) ? S.A : S.W);
        row_body<C, EPI_NONE, false, COHERENT>(src, S.X, S.g.nyb, nrows, S.twx, EpiArgs{}, wk.y, W, T);
        return;
    }
    const EpiArgs e = batch_epi(S, n);
    if (n == 0) row_body<C, EPI_FIRST, false, COHERENT>(S.X, nullptr, S.g.nyb, nrows, S.twx, e, wk.y, W, T);
    else if (n == S.M) row_body<C, EPI_LAST, false, COHERENT>(S.X, nullptr, S.g.nyb, nrows, S.twx, e, wk.y, W, T);
    else row_body<C, EPI_MID, false, COHERENT>(S.X, nullptr, S.g.nyb, nrows, S.twx, e, wk.y, W, T);
}

template <int C, bool INV>
__global__ void __launch_bounds__(RowCfg<C>::THREADS) kb_row(const BatchShot* __restrict__ shots,
                                                             const int2* __restrict__ work, int n)
{
    extern __shared__ float4 smem4[];
    kb_row_item<C, INV>(shots, work[blockIdx.x], n, reinterpret_cast<float2*>(smem4));
}

// ---- the batched step as one persistent cooperative launch ----
//
// Every CTA walks the same list of phases (the batched passes in launch
// order: per shot group, application and pass kind, one entry per axis-length
// class); inside a phase it takes work items (shot, block) strided by the
// grid, and between phases all CTAs meet at a grid barrier.  Only lengths
// 16 C with C <= 16 take part (their row and column kernels all have 256
// threads).  The barrier is a counter and a generation word in global
// memory; a CTA waits at most kBarrierLimitNs for the others, then sets
// *err and leaves the kernel, so a failed step ends instead of hanging.
constexpr int kPersistThreads = 256;
constexpr unsigned long long kBarrierLimitNs = 2000000000ull;

__device__ __forceinline__ unsigned long long now_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// bar[0] = arrivals, bar[1] = generation.  Returns false after a timeout.
// expected = the CTAs that arrive (the grid; the self test asks for more).
__device__ bool grid_barrier(unsigned* bar, int* err, unsigned long long limit_ns = kBarrierLimitNs,
                             unsigned expected = 0)
{
    if (expected == 0) expected = gridDim.x;
    __syncthreads();
    int ok = 1;
    if (threadIdx.x == 0) {
        volatile unsigned* gen = bar + 1;
        const unsigned g = *gen;
        __threadfence();
        if (atomicAdd(bar, 1u) + 1u == expected) {
            atomicExch(bar, 0u);
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            const unsigned long long t0 = now_ns();
            while (*gen == g) {
                if (now_ns() - t0 > limit_ns) {
                    ok = 0;
                    atomicExch(err, 1);
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
    }
    const bool all = __syncthreads_and(ok) != 0;
    __threadfence();   // every thread orders its later loads after the barrier
    return all;
}

// Self test of the bounded grid barrier: one CTA waits for a second one that
// is never launched, so the wait runs out after limit_ns and sets *err.
__global__ void k_selftest_grid_barrier(unsigned* bar, int* err, unsigned long long limit_ns)
{
    grid_barrier(bar, err, limit_ns, gridDim.x + 1);
}

template <int C>
__device__ __forceinline__ void persist_item(const BatchShot* shots, int kind, int2 wk, int n, float2* W)
{
    switch (kind) {
    case 0: kb_row_item<C, false, true>(shots, wk, n, W); break;
    case 1: kb_col_item<C, COL_FWD, 1, true>(shots, wk, W); break;
    case 2: kb_col_item<C, COL_KSCALE, 2, true>(shots, wk, W); break;
    case 3: kb_col_item<C, COL_INV, 1, true>(shots, wk, W); break;
    default: kb_row_item<C, true, true>(shots, wk, n, W); break;
    }
}

#define OSE_PERSIST_SIZES(X) X(4) X(6) X(7) X(8) X(9) X(10) X(11) X(12) X(16)

__global__ void __launch_bounds__(kPersistThreads, 2) kb_persistent(const BatchShot* __restrict__ shots,
                                                                    const PersistPass* __restrict__ passes,
                                                                    int npass, unsigned* bar, int* err)
{
    extern __shared__ float4 smem4[];
    float2* W = reinterpret_cast<float2*>(smem4);
    for (int pi = 0; pi < npass; ++pi) {
        const PersistPass P = passes[pi];
        for (int w = blockIdx.x; w < P.nblocks; w += gridDim.x) {
            const int2 wk = P.work[w];
            switch (P.n_axis / 16) {
#define ITEM(C) case C: persist_item<C>(shots, P.kind, wk, P.n, W); break;
                OSE_PERSIST_SIZES(ITEM)
#undef ITEM
            default: break;
            }
            __syncthreads();   // the next item overwrites the twiddle table and the transpose buffer
        }
        if (P.barrier_after && !grid_barrier(bar, err)) return;
    }
}

template <int C, int EPI, bool FWD = false>
cudaError_t launch_row_one(cudaStream_t s, const float2* src, float2* dst, int nyb, long long nrows,
                           const float2* twg, const EpiArgs& e)
{
    using K = RowCfg<C>;
    const unsigned grid = (unsigned)((nrows + K::RW - 1) / K::RW);
    k_row<C, EPI, FWD><<<grid, K::THREADS, K::SMEM, s>>>(src, dst, nyb, nrows, twg, e);
    return cudaGetLastError();
}

template <int C>
cudaError_t launch_row_c(cudaStream_t s, int epi, const float2* src, float2* dst, int nyb, long long nrows,
                         const float2* twg, const EpiArgs& e)
{
    switch (epi) {
    case EPI_NONE: return launch_row_one<C, EPI_NONE>(s, src, dst, nyb, nrows, twg, e);
    case EPI_FIRST: return launch_row_one<C, EPI_FIRST>(s, src, dst, nyb, nrows, twg, e);
    case EPI_MID: return launch_row_one<C, EPI_MID>(s, src, dst, nyb, nrows, twg, e);
    case EPI_LAST: return launch_row_one<C, EPI_LAST>(s, src, dst, nyb, nrows, twg, e);
    case EPI_SCALE: return launch_row_one<C, EPI_SCALE>(s, src, dst, nyb, nrows, twg, e);
    case EPI_SCALE_VEL: return launch_row_one<C, EPI_SCALE_VEL>(s, src, dst, nyb, nrows, twg, e);
    case EPI_FIRST_FWD: return launch_row_one<C, EPI_FIRST, true>(s, src, dst, nyb, nrows, twg, e);
    case EPI_MID_FWD: return launch_row_one<C, EPI_MID, true>(s, src, dst, nyb, nrows, twg, e);
    default: return cudaErrorInvalidValue;
    }
}

template <int C>
cudaError_t configure_one()
{
    cudaError_t e;
    if ((e = cudaFuncSetAttribute(k_col<C, COL_FWD>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)ColCfg<C>::SMEM)) != cudaSuccess)
        return e;
    if ((e = cudaFuncSetAttribute(k_col<C, COL_INV>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)ColCfg<C>::SMEM)) != cudaSuccess)
        return e;
    return cudaFuncSetAttribute(k_col<C, COL_KSCALE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)ColCfg<C>::SMEM);
}

template <int C>
cudaError_t launch_one(cudaStream_t s, int mode, float2* X, int nxb, int nother, long long stride, long long ostride,
                       const float2* twg, const Tables& t)
{
    using K = ColCfg<C>;
    const dim3 grid((nxb + K::TX - 1) / K::TX, nother);
    if (mode == COL_FWD) k_col<C, COL_FWD><<<grid, K::THREADS, K::SMEM, s>>>(X, nxb, stride, ostride, twg, t);
    else if (mode == COL_INV) k_col<C, COL_INV><<<grid, K::THREADS, K::SMEM, s>>>(X, nxb, stride, ostride, twg, t);
    else k_col<C, COL_KSCALE><<<grid, K::THREADS, K::SMEM, s>>>(X, nxb, stride, ostride, twg, t);
    return cudaGetLastError();
}

#define OSE_COL_SIZES(X) X(4) X(6) X(7) X(8) X(9) X(10) X(11) X(12) X(16) X(18) X(20) X(23) X(24)

template <int C>
cudaError_t launch_batch_one(cudaStream_t s, int kind, const BatchShot* shots, const int2* work, int nblocks, int n)
{
    if (nblocks <= 0) return cudaSuccess;
    switch (kind) {
    case 0: kb_row<C, false><<<nblocks, RowCfg<C>::THREADS, RowCfg<C>::SMEM, s>>>(shots, work, n); break;
    case 1: kb_col<C, COL_FWD, 1><<<nblocks, ColCfg<C>::THREADS, ColCfg<C>::SMEM, s>>>(shots, work); break;
    case 2: kb_col<C, COL_KSCALE, 2><<<nblocks, ColCfg<C>::THREADS, ColCfg<C>::SMEM, s>>>(shots, work); break;
    case 3: kb_col<C, COL_INV, 1><<<nblocks, ColCfg<C>::THREADS, ColCfg<C>::SMEM, s>>>(shots, work); break;
    default: kb_row<C, true><<<nblocks, RowCfg<C>::THREADS, RowCfg<C>::SMEM, s>>>(shots, work, n); break;
    }
    return cudaGetLastError();
}

}  // namespace cols

bool col_supported(int n)
{
    if (n % 16) return false;
    switch (n / 16) {
#define CASE(C) case C:
        OSE_COL_SIZES(CASE)
#undef CASE
        return true;
    default: return false;
    }
}

cudaError_t configure_col_kernels()
{
    cudaError_t e = cudaSuccess;
#define CONF(C) if ((e = cols::configure_one<C>()) != cudaSuccess) return e;
    OSE_COL_SIZES(CONF)
#undef CONF
    return e;
}

// Batched pass `kind` (0 x forward, 1 y forward, 2 z, 3 y inverse, 4 x inverse +
// update) of application n over the blocks of the shots whose length on that
// axis is n_axis = 16 C.
cudaError_t launch_batch_col_pass(cudaStream_t s, int kind, int n_axis, const BatchShot* shots, const int2* work,
                                  int nblocks, int n)
{
    switch (n_axis / 16) {
#define LAUNCH(C) case C: return cols::launch_batch_one<C>(s, kind, shots, work, nblocks, n);
        OSE_COL_SIZES(LAUNCH)
#undef LAUNCH
    default: return cudaErrorInvalidValue;
    }
}

bool persist_supported(int n_axis)
{
    switch (n_axis / 16) {
#define CASE(C) case C:
        OSE_PERSIST_SIZES(CASE)
#undef CASE
        return n_axis % 16 == 0;
    default: return false;
    }
}

size_t persist_smem()
{
    size_t m = 0;
#define SM(C) m = std::max(m, std::max(cols::ColCfg<C>::SMEM, cols::RowCfg<C>::SMEM));
    OSE_PERSIST_SIZES(SM)
#undef SM
    return m;
}

int persist_grid()
{
    int dev = 0, sms = 0, per = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    if (cudaFuncSetAttribute(cols::kb_persistent, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)persist_smem()) !=
        cudaSuccess)
        return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, cols::kb_persistent, cols::kPersistThreads,
                                                      persist_smem()) != cudaSuccess)
        return 0;
    return sms * per;
}

cudaError_t launch_batch_persistent(cudaStream_t s, const BatchShot* shots, const PersistPass* passes, int npass,
                                    unsigned* bar, int* err, int grid)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(cols::kPersistThreads);
    cfg.dynamicSmemBytes = persist_smem();
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, cols::kb_persistent, shots, passes, npass, bar, err);
}

int col_tile(int n_axis) { return n_axis / 16 > 16 ? 8 : 16; }
int row_tile(int n_axis) { return n_axis / 16 > 16 ? 8 : 16; }

// x rows of length n: epi = EPI_NONE forward src -> dst, else inverse of src
// and the epilogue.
cudaError_t launch_row(cudaStream_t s, int epi, int n, const float2* src, float2* dst, int nyb, long long nrows,
                       const float2* twg, const EpiArgs& e)
{
    switch (n / 16) {
#define LAUNCH(C) case C: return cols::launch_row_c<C>(s, epi, src, dst, nyb, nrows, twg, e);
        OSE_COL_SIZES(LAUNCH)
#undef LAUNCH
    default: return cudaErrorInvalidValue;
    }
}

// mode: 0 forward, 1 inverse, 2 forward * |k| inverse (z pass).
cudaError_t launch_col(cudaStream_t s, int mode, int n, float2* X, int nxb, int nother, long long stride,
                       long long ostride, const float2* twg, const Tables& t)
{
    switch (n / 16) {
#define LAUNCH(C) case C: return cols::launch_one<C>(s, mode, X, nxb, nother, stride, ostride, twg, t);
        OSE_COL_SIZES(LAUNCH)
#undef LAUNCH
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t selftest_grid_barrier(cudaStream_t s, unsigned* bar, int* err, unsigned long long limit_ns)
{
    cols::k_selftest_grid_barrier<<<1, 32, 0, s>>>(bar, err, limit_ns);
    return cudaGetLastError();
}

}  // namespace ose
