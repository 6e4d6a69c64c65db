// ose_tensor.cu - the precision form: the z pass of one operator application
// (FFT_z -> * |k| -> IFFT_z, the part of scale_kxkz_3D's round trip that runs
// along z, ose_3d_kernel.cu:101-126 and ose_3d_lib.cu:665-687) for a padded
// z axis of 256, as four batched DFT-16 matmuls on the tcgen05 tensor cores.
//
// A column of 256 values is a 16 x 16 matrix (four-step factorisation,
// n = n1 + 16 n2, k = k2 + 16 k1):
//   stage 1  Y[n1][k2]  = sum_n2 x[n1 + 16 n2] W16^(n2 k2)       (matmul)
//            Y[n1][k2] *= W256^(n1 k2)                          (CUDA cores)
//   stage 2  X[k2+16k1] = sum_n1 Y[n1][k2] W16^(n1 k1)           (matmul)
//            X *= |k|                                           (CUDA cores)
//   stage 3  Z[n1][k2]  = sum_k1 X[k2+16k1] W16^(-n1 k1)         (matmul)
//            Z[n1][k2] *= W256^(-n1 k2)                         (CUDA cores)
//   stage 4  x[n1+16n2] = sum_k2 Z[n1][k2] W16^(-n2 k2)          (matmul)
// Each matmul is D[256 x 32] = A[256 x 32] * B[32 x 32] in real arithmetic:
// the 256 rows are (16 columns of the tile) x (16 values of the index that is
// not transformed), the 32 K entries are 16 complex inputs (re, im), and B is
// the real 32 x 32 form of the complex DFT-16 matrix, built in FP64 on the
// host.  D is two M = 128 tiles in TMEM; each thread owns one row, reads it
// back with tcgen05.ld, applies the twiddle (or |k|) and writes the next
// stage's A row (transposed between stages 1-2 and 3-4) into shared memory.
//
// Variants (arithmetic of the products; accumulation is FP32 throughout):
//   OSE_PRECISION_TF32    one pass, operands rounded to TF32
//   OSE_PRECISION_TF32X3  a = hi + lo in TF32, D = lo*Bhi + hi*Blo + hi*Bhi
//   OSE_PRECISION_BF16X3  the same three products with BF16 hi/lo parts
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "ose_internal.h"
#include "tcgen05.cuh"

namespace ose {

namespace tcz {

constexpr int NZ = 256;
constexpr int TX = 16;              // x columns per CTA
constexpr int ROWS = 16 * TX;       // matmul rows per stage: two M = 128 tiles
constexpr int THREADS = ROWS;       // one row per thread
constexpr int KR = 32;              // real K and N of one DFT-16 matmul
constexpr uint32_t TMEM_COLS = 64;  // two tiles x 32 FP32 columns
constexpr uint64_t kWaitLimitNs = 1000000000ull;

template <int VAR>
struct Cfg {
    static constexpr bool bf16 = VAR == OSE_PRECISION_BF16X3;
    static constexpr bool split = VAR != OSE_PRECISION_TF32;
    static constexpr int es = bf16 ? 2 : 4;                  // operand element bytes
    static constexpr int row_bytes = KR * es;                // one operand row
    static constexpr uint32_t sbo = 8 * row_bytes;           // 8-row group stride
    static constexpr uint32_t lbo = 128;                     // K core stride
    static constexpr int ksteps = row_bytes / 32;            // MMAs per K = 32
    static constexpr int a_bytes = ROWS * row_bytes;         // one A operand
    static constexpr int b_bytes = KR * row_bytes;           // one B operand
    static constexpr int off_alo = a_bytes;
    static constexpr int off_b = split ? 2 * a_bytes : a_bytes;   // [Fhi][Flo][Ihi][Ilo]
    static constexpr int off_tw = off_b + 4 * b_bytes;
    static constexpr int off_bar = off_tw + NZ * 8;
    static constexpr int smem = off_bar + 16;
    static constexpr uint32_t id = tc5::idesc(bf16 ? tc5::kTypeBF16 : tc5::kTypeTF32, 128, KR);
};

// Byte offset of complex entry kp (K columns 2kp, 2kp+1) of operand row r.
template <int VAR>
__device__ __forceinline__ uint32_t opnd_off(int r, int kp)
{
    using C = Cfg<VAR>;
    if (C::bf16) return (r >> 3) * C::sbo + (kp >> 2) * C::lbo + (r & 7) * 16 + (kp & 3) * 4;
    return (r >> 3) * C::sbo + (kp >> 1) * C::lbo + (r & 7) * 16 + (kp & 1) * 8;
}

template <int VAR>
__device__ __forceinline__ void put(uint8_t* sm, int r, int kp, float2 v)
{
    using C = Cfg<VAR>;
    const uint32_t o = opnd_off<VAR>(r, kp);
    if (C::bf16) {
        const __nv_bfloat16 hx = __float2bfloat16_rn(v.x), hy = __float2bfloat16_rn(v.y);
        const __nv_bfloat16 lx = __float2bfloat16_rn(v.x - __bfloat162float(hx));
        const __nv_bfloat16 ly = __float2bfloat16_rn(v.y - __bfloat162float(hy));
        *reinterpret_cast<__nv_bfloat162*>(sm + o) = __halves2bfloat162(hx, hy);
        *reinterpret_cast<__nv_bfloat162*>(sm + C::off_alo + o) = __halves2bfloat162(lx, ly);
    } else {
        const float hx = tc5::to_tf32(v.x), hy = tc5::to_tf32(v.y);
        *reinterpret_cast<float2*>(sm + o) = make_float2(hx, hy);
        if (C::split)
            *reinterpret_cast<float2*>(sm + C::off_alo + o) =
                make_float2(tc5::to_tf32(v.x - hx), tc5::to_tf32(v.y - hy));
    }
}

// One stage: D_tile = A * B for both tiles (bsel 0 forward, 1 inverse).
template <int VAR>
__device__ __forceinline__ void issue(uint32_t sbase, uint32_t tmem, int bsel, uint64_t* bar)
{
    using C = Cfg<VAR>;
    const uint32_t bhi = sbase + C::off_b + (2 * bsel) * C::b_bytes;
    const uint32_t blo = bhi + C::b_bytes;
    const uint32_t ahi = sbase, alo = sbase + C::off_alo;
#pragma unroll
    for (int t = 0; t < ROWS / 128; ++t) {
        const uint32_t d = tmem + t * KR;
        const uint32_t at = t * 16 * C::sbo;
        uint32_t acc = 0;
        // products in increasing size: lo*Bhi, hi*Blo, hi*Bhi
        const int np = C::split ? 3 : 1;
#pragma unroll
        for (int p = 0; p < np; ++p) {
            const uint32_t a = (C::split && p == 0) ? alo : ahi;
            const uint32_t b = (C::split && p == 1) ? blo : bhi;
#pragma unroll
            for (int k = 0; k < C::ksteps; ++k) {
                const uint64_t da = tc5::smem_desc(a + at + k * 2 * C::lbo, C::lbo, C::sbo);
                const uint64_t db = tc5::smem_desc(b + k * 2 * C::lbo, C::lbo, C::sbo);
                if (C::bf16) tc5::mma_f16(d, da, db, C::id, acc);
                else tc5::mma_tf32(d, da, db, C::id, acc);
                acc = 1;
            }
        }
    }
    tc5::mma_commit(bar);
}

__device__ __forceinline__ float2 cmulf(float2 a, float2 w)
{
    return make_float2(fmaf(a.x, w.x, -a.y * w.y), fmaf(a.x, w.y, a.y * w.x));
}
__device__ __forceinline__ float2 cmulf_conj(float2 a, float2 w)
{
    return make_float2(fmaf(a.x, w.x, a.y * w.y), fmaf(a.y, w.x, -a.x * w.y));
}

// grid (nxb / TX, nyb); X is [z][y][x] with nzb = 256, transformed in place.
// CTAs per SM asked of the register allocator (85 registers a thread for
// three; shared memory allows three for TF32 and BF16X3, two for TF32X3)
template <int VAR>
constexpr int ztc_min_blocks() { return Cfg<VAR>::smem * 3 <= 227 * 1024 ? 3 : 2; }

template <int VAR>
__global__ void __launch_bounds__(THREADS, ztc_min_blocks<VAR>()) k_ztc(float2* __restrict__ X, int nxb, int nyb,
                                                 const uint8_t* __restrict__ bmat, Tables t, int* err)
{
    using C = Cfg<VAR>;
    extern __shared__ __align__(1024) uint8_t sm[];
    float2* tw = reinterpret_cast<float2*>(sm + C::off_tw);
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm + C::off_bar);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + C::off_bar + 8);
    const uint32_t sbase = tc5::smem_u32(sm);
    const int r = threadIdx.x, j = r >> 4, c = r & (TX - 1), warp = r >> 5;
    const int y = blockIdx.y, x = blockIdx.x * TX + c;
    const size_t zs = (size_t)nxb * nyb;
    float2* col = X + (size_t)y * nxb + x;

    if (warp == 0) tc5::tmem_alloc(tslot, TMEM_COLS);
    if (r == 0) tc5::mbar_init(bar, 1);
    {   // DFT operands and twiddles
        const int4* s4 = reinterpret_cast<const int4*>(bmat);
        int4* d4 = reinterpret_cast<int4*>(sm + C::off_b);
        for (int i = r; i < 4 * C::b_bytes / 16; i += THREADS) d4[i] = s4[i];
        tw[r] = t.twz[r];
    }
    // stage 1 operand: row (n1 = j, c), K = n2
    float2 v[16];
#pragma unroll
    for (int n2 = 0; n2 < 16; ++n2) v[n2] = col[(size_t)(j + 16 * n2) * zs];
#pragma unroll
    for (int n2 = 0; n2 < 16; ++n2) put<VAR>(sm, r, n2, v[n2]);
    tc5::fence_async_smem();
    tc5::fence_before_sync();
    __syncthreads();
    tc5::fence_after_sync();
    const uint32_t tmem = *tslot;
    // this thread's TMEM row: tile r / 128, lane r % 128
    const uint32_t trow = tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)((r >> 7) * KR);
    const float kxy = __ldg(t.kx2 + x) + __ldg(t.ky2 + y);

    int failed = 0, stage = 0;
    float d[32];
    for (; stage < 4; ++stage) {
        const int s = stage;
        if (r == 0) issue<VAR>(sbase, tmem, s >= 2, bar);
        int bad = 0;
        if (r == 0) bad = !tc5::mbar_wait(bar, (uint32_t)(s & 1), kWaitLimitNs);
        failed = __syncthreads_or(bad);
        if (failed) break;
        tc5::fence_after_sync();
        tc5::tmem_ld32(trow, d);
        if (s == 3) break;
        if (s == 0) {
            // row (n1 = j, c) holds Y[n1][k2]: twiddle, then row (k2, c) at K = n1
#pragma unroll
            for (int k2 = 0; k2 < 16; ++k2) {
                const float2 yv = make_float2(d[2 * k2], d[2 * k2 + 1]);
                put<VAR>(sm, k2 * TX + c, j, k2 ? cmulf(yv, tw[j * k2]) : yv);
            }
        } else if (s == 1) {
            // row (k2 = j, c) holds X[j + 16 k1]: scale by |k|, same row for stage 3
#pragma unroll
            for (int k1 = 0; k1 < 16; ++k1) {
                const float kk = sqrtf(kxy + __ldg(t.kz2 + j + 16 * k1));
                put<VAR>(sm, r, k1, make_float2(d[2 * k1] * kk, d[2 * k1 + 1] * kk));
            }
        } else {
            // row (k2 = j, c) holds Z[n1][k2]: conjugate twiddle, row (n1, c) at K = k2
#pragma unroll
            for (int n1 = 0; n1 < 16; ++n1) {
                const float2 zv = make_float2(d[2 * n1], d[2 * n1 + 1]);
                put<VAR>(sm, n1 * TX + c, j, n1 ? cmulf_conj(zv, tw[j * n1]) : zv);
            }
        }
        tc5::fence_async_smem();
        tc5::fence_before_sync();
        __syncthreads();
        tc5::fence_after_sync();
    }
    if (!failed) {
        // row (n1 = j, c) holds x[j + 16 n2]
#pragma unroll
        for (int n2 = 0; n2 < 16; ++n2) col[(size_t)(j + 16 * n2) * zs] = make_float2(d[2 * n2], d[2 * n2 + 1]);
    } else if (r == 0) {
        atomicExch(err, 1);
        // give the MMAs still in flight one more limited wait before the
        // columns are released
        tc5::mbar_wait(bar, (uint32_t)(stage & 1), kWaitLimitNs);
    }
    tc5::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tc5::fence_after_sync();
        tc5::tmem_dealloc(tmem, TMEM_COLS);
    }
}

template <int VAR>
cudaError_t launch(cudaStream_t s, float2* X, const Geometry& g, const Tables& t, const void* bmat, int* err)
{
    dim3 grid(g.nxb / TX, g.nyb);
    k_ztc<VAR><<<grid, THREADS, Cfg<VAR>::smem, s>>>(X, g.nxb, g.nyb, static_cast<const uint8_t*>(bmat), t,
                                                     err);
    return cudaGetLastError();
}

// Host rounding of a double to the operand types (nearest, ties to even).
uint32_t f32_bits(float f)
{
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
}
float bits_f32(uint32_t u)
{
    float f;
    memcpy(&f, &u, 4);
    return f;
}
float round_bits(double v, int drop)
{
    const uint32_t u = f32_bits((float)v);
    const uint32_t half = 1u << (drop - 1), mask = (1u << drop) - 1;
    const uint32_t lsb = (u >> drop) & 1u;
    return bits_f32((u + half - 1 + lsb) & ~mask);
}

}  // namespace tcz

bool tensor_zpass_supported(int nxb, int nyb, int nzb)
{
    (void)nyb;
    return nzb == tcz::NZ && nxb % tcz::TX == 0;
}

size_t tensor_operand_bytes(int var)
{
    return var == OSE_PRECISION_BF16X3 ? 4 * tcz::Cfg<OSE_PRECISION_BF16X3>::b_bytes
                                       : 4 * tcz::Cfg<OSE_PRECISION_TF32>::b_bytes;
}

// The four B operands [F hi][F lo][I hi][I lo] of a variant in their shared
// memory byte layout.  Row n = 2k + c' (output k, c' = re/im), K column
// m = 2j + c (input j, c = re/im) of the real form of W16^(+-jk).
void tensor_operands(int var, std::vector<uint8_t>& out)
{
    const bool bf16 = var == OSE_PRECISION_BF16X3;
    const int es = bf16 ? 2 : 4;
    const int drop = bf16 ? 16 : 13;
    const int bb = tcz::KR * tcz::KR * es;
    out.assign(4 * (size_t)bb, 0);
    const double pi = 3.14159265358979323846;
    for (int inv = 0; inv < 2; ++inv)
        for (int n = 0; n < tcz::KR; ++n)
            for (int m = 0; m < tcz::KR; ++m) {
                const int k = n >> 1, cp = n & 1, jj = m >> 1, cc = m & 1;
                const double th = 2.0 * pi * (double)((jj * k) % 16) / 16.0;
                const double cs = cos(th), sn = inv ? -sin(th) : sin(th);
                // forward: re' = re cos + im sin, im' = im cos - re sin
                const double val = cp == 0 ? (cc == 0 ? cs : sn) : (cc == 0 ? -sn : cs);
                const float hi = tcz::round_bits(val, drop);
                const float lo = tcz::round_bits(val - (double)hi, drop);
                size_t off;
                if (bf16) off = (n >> 3) * 512 + (m >> 3) * 128 + (n & 7) * 16 + (m & 7) * 2;
                else off = (n >> 3) * 1024 + (m >> 2) * 128 + (n & 7) * 16 + (m & 3) * 4;
                uint8_t* base = out.data() + (size_t)(2 * inv) * bb;
                if (bf16) {
                    const uint16_t h = (uint16_t)(tcz::f32_bits(hi) >> 16), l = (uint16_t)(tcz::f32_bits(lo) >> 16);
                    memcpy(base + off, &h, 2);
                    memcpy(base + bb + off, &l, 2);
                } else {
                    memcpy(base + off, &hi, 4);
                    memcpy(base + bb + off, &lo, 4);
                }
            }
}

cudaError_t configure_tensor_kernels()
{
    cudaError_t e;
    if ((e = cudaFuncSetAttribute(tcz::k_ztc<OSE_PRECISION_TF32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  tcz::Cfg<OSE_PRECISION_TF32>::smem)) != cudaSuccess)
        return e;
    if ((e = cudaFuncSetAttribute(tcz::k_ztc<OSE_PRECISION_TF32X3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  tcz::Cfg<OSE_PRECISION_TF32X3>::smem)) != cudaSuccess)
        return e;
    return cudaFuncSetAttribute(tcz::k_ztc<OSE_PRECISION_BF16X3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                tcz::Cfg<OSE_PRECISION_BF16X3>::smem);
}

cudaError_t launch_tensor_zpass(cudaStream_t s, float2* X, const Geometry& g, const Tables& t)
{
    switch (t.tcvar) {
    case OSE_PRECISION_TF32: return tcz::launch<OSE_PRECISION_TF32>(s, X, g, t, t.tcb, t.tcerr);
    case OSE_PRECISION_TF32X3: return tcz::launch<OSE_PRECISION_TF32X3>(s, X, g, t, t.tcb, t.tcerr);
    case OSE_PRECISION_BF16X3: return tcz::launch<OSE_PRECISION_BF16X3>(s, X, g, t, t.tcb, t.tcerr);
    default: return cudaErrorInvalidValue;
    }
}

// Self test of the bounded MMA-completion wait (tc5::mbar_wait, as the
// tensor z pass and the corrector use it): a barrier no commit ever reaches.
__global__ void k_selftest_mma_wait(int* err, unsigned long long limit_ns)
{
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) tc5::mbar_init(&bar, 1);
    __syncthreads();
    if (threadIdx.x == 0 && !tc5::mbar_wait(&bar, 0u, limit_ns)) atomicExch(err, 1);
}

cudaError_t selftest_mma_wait(cudaStream_t s, int* err, unsigned long long limit_ns)
{
    k_selftest_mma_wait<<<1, 32, 0, s>>>(err, limit_ns);
    return cudaGetLastError();
}

}  // namespace ose
