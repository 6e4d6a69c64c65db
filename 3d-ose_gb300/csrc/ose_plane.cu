// ose_plane.cu - the fast path for 256 x 256 x 256 padded grids.
//
// One operator application L = v * IFFT3(|k| FFT3(.)) / (R N) costs two HBM
// passes here instead of five:
//   k_zpass            z lines: forward FFT, * |k|, inverse FFT (in place)
//   k_plane_inv<...>   one z plane per 8-CTA thread-block cluster: inverse y
//                      and x FFTs, the step's pointwise update (the same
//                      epilogue as the generic path: scal_vr_3d, the
//                      recurrence, add_bessel_3d, apply_ABC_Xt, receivers),
//                      then the NEXT application's forward x and y FFTs of the
//                      new term, written as its spectrum.
// plus k_plane_fwd (forward x and y FFTs of the state) once per step.
//
// Plane work is split over the cluster: CTA r owns rows y in [32r, 32r+32) for
// the x transforms and columns x in [32r, 32r+32) for the y transforms; the
// 512 KiB plane changes hands between the two through distributed shared
// memory: each CTA pushes the 32 x 32 blocks it holds into their owners'
// receive buffers with st.async, whose bytes complete a transaction count on
// the receiver's mbarrier, so a receiver waits on its own barrier.  One
// cluster barrier per exchange tells the senders that the receive buffers
// (which overlay the transpose buffer) are free: a release arrive, so this
// CTA's reads of the buffer are ordered before the other CTAs' pushes (a
// relaxed arrive after a __syncthreads measured faster but let pushes overtake
// reads still in flight).
//
// Every 256-point transform is a four-step 16 x 16 FFT: a line is held by 16
// threads with 16 values each, a radix-16 DFT runs in registers, twiddles
// W_256^(j k) come from a shared table, and one transpose through shared
// memory connects the two radix-16 stages.
#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <stdlib.h>
#include <string.h>

#include "ose_internal.h"
#include "ose_epilogue.cuh"
#include "ose_pdl.cuh"
#include "tcgen05.cuh"

namespace cg = cooperative_groups;

namespace ose {
namespace plane {

constexpr int N = 256;          // line length on all three axes
using ose::kCompensatedTwiddles;
constexpr int CL = 8;           // CTAs per cluster (one plane per cluster)
constexpr int SL = N / CL;      // rows / columns per CTA = 32
// Line slots per thread: 2 (256 threads, up to 128 registers) or 1 (512
// threads, up to 64 registers); either way two CTAs per SM.
constexpr int NS = 2;
constexpr int THREADS = 512 / NS;
constexpr int WARPS = THREADS / 32;
constexpr int ECH = NS == 1 ? 4 : 8;   // epilogue cells loaded ahead of their stores
#ifndef OSE_PLANE_ECH_SUM
#define OSE_PLANE_ECH_SUM 8
#endif
constexpr int ECH_SUM = OSE_PLANE_ECH_SUM;   // the same where S is read and written too
#ifndef OSE_PLANE_ECH_LAST
#define OSE_PLANE_ECH_LAST 8
#endif
constexpr int ECH_LAST = OSE_PLANE_ECH_LAST;  // the last application (S read, the state written)
constexpr int TPAD = 17;        // padded stride of the row-transpose buffer
constexpr int TROWS = SL * 16 * TPAD;  // complex values in the row exchange buffer
constexpr int ABUF = SL * N;           // complex values of one CTA's plane slice
constexpr int MAIN = TROWS > ABUF ? TROWS : ABUF;   // transpose buffer = receive buffer
// + twiddle table (hi, lo) + the x sponge factor's powers ax, ax^2, ax^3 (3 N floats)
constexpr int SMEM_COMPLEX = MAIN + 2 * N + 3 * N / 2;
// + the exchange's mbarrier
constexpr size_t SMEM_BYTES = sizeof(float2) * SMEM_COMPLEX + 16;

// times -i (forward) or +i (inverse)
template <bool INV>
__device__ __forceinline__ float2 rot(float2 a)
{
    return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

// Complex add and subtract as one packed two-lane FP32 instruction each
// (add/sub.rn.f32x2: the same IEEE results as two scalar operations).
__device__ __forceinline__ uint64_t pk2(float2 a)
{
    uint64_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a.x), "f"(a.y));
    return r;
}
__device__ __forceinline__ float2 upk2(uint64_t r)
{
    float2 a;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a.x), "=f"(a.y) : "l"(r));
    return a;
}
__device__ __forceinline__ float2 padd(float2 a, float2 b)
{
    uint64_t d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(pk2(a)), "l"(pk2(b)));
    return upk2(d);
}
__device__ __forceinline__ float2 psub(float2 a, float2 b)
{
    uint64_t d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(pk2(a)), "l"(pk2(b)));
    return upk2(d);
}

template <bool INV>
__device__ __forceinline__ void dft4(float2& a0, float2& a1, float2& a2, float2& a3)
{
    // the +-i (a1 - a3) terms stay scalar: a swapped pair is no packed operand
    const float2 t0 = padd(a0, a2), t1 = psub(a0, a2), t2 = padd(a1, a3), d = psub(a1, a3);
    a0 = padd(t0, t2);
    a2 = psub(t0, t2);
    const float2 t3 = rot<INV>(d);
    a1 = make_float2(t1.x + t3.x, t1.y + t3.y);
    a3 = make_float2(t1.x - t3.x, t1.y - t3.y);
}

// times W_16^E (forward) or its conjugate (inverse); E in {0,1,2,3,4,6,9}.
// With kCompensatedTwiddles the constants are float pairs hi + lo (cos(pi/8),
// sin(pi/8), sqrt(1/2) to about 48 bits), so no rounded constant perturbs every
// transform the same way.
template <int E, bool INV>
__device__ __forceinline__ float2 w16(float2 a)
{
    constexpr double C1d = 0.92387953251128675612818318939678828682;   // cos(pi/8)
    constexpr double S1d = 0.38268343236508977172845998403039886676;   // sin(pi/8)
    constexpr double Hd = 0.70710678118654752440084436210484903928;    // sqrt(1/2)
    constexpr float C1 = (float)C1d, C1l = (float)(C1d - (double)(float)C1d);
    constexpr float S1 = (float)S1d, S1l = (float)(S1d - (double)(float)S1d);
    constexpr float H = (float)Hd, Hl = (float)(Hd - (double)(float)Hd);
    constexpr float s = INV ? 1.f : -1.f;         // sign of the sine part
    if (E == 0) return a;
    if (E == 4) return rot<INV>(a);
    float c, cl, sn, snl;
    if (E == 1) { c = C1; cl = C1l; sn = s * S1; snl = s * S1l; }
    else if (E == 2) { c = H; cl = Hl; sn = s * H; snl = s * Hl; }
    else if (E == 3) { c = S1; cl = S1l; sn = s * C1; snl = s * C1l; }
    else if (E == 6) { c = -H; cl = -Hl; sn = s * H; snl = s * Hl; }
    else { c = -C1; cl = -C1l; sn = -s * S1; snl = -s * S1l; }   // E == 9
    if (!kCompensatedTwiddles) return make_float2(fmaf(a.x, c, -a.y * sn), fmaf(a.x, sn, a.y * c));
    const float tx = fmaf(a.x, cl, -a.y * snl), ty = fmaf(a.x, snl, a.y * cl);
    return make_float2(fmaf(a.x, c, fmaf(-a.y, sn, tx)), fmaf(a.x, sn, fmaf(a.y, c, ty)));
}

// a * (w + wl) with w, wl the two halves of a twiddle (conj for INV)
template <bool INV>
__device__ __forceinline__ float2 cmul_ff(float2 a, float2 w, float2 wl)
{
    if (INV) { w.y = -w.y; wl.y = -wl.y; }
    if (!kCompensatedTwiddles) return make_float2(fmaf(a.x, w.x, -a.y * w.y), fmaf(a.x, w.y, a.y * w.x));
    const float tx = fmaf(a.x, wl.x, -a.y * wl.y), ty = fmaf(a.x, wl.y, a.y * wl.x);
    return make_float2(fmaf(a.x, w.x, fmaf(-a.y, w.y, tx)), fmaf(a.x, w.y, fmaf(a.y, w.x, ty)));
}

// In-register 16-point DFT, natural order in and out (4 x 4 split).
template <bool INV>
__device__ __forceinline__ void dft16(float2 (&v)[16])
{
    // DFT4 over m1 for each m2 (elements m2, m2+4, m2+8, m2+12)
#pragma unroll
    for (int m2 = 0; m2 < 4; ++m2) dft4<INV>(v[m2], v[m2 + 4], v[m2 + 8], v[m2 + 12]);
    // now v[m2 + 4 k1] = Y[m2][k1]; twiddle by W16^(m2 k1)
    v[5] = w16<1, INV>(v[5]);
    v[9] = w16<2, INV>(v[9]);
    v[13] = w16<3, INV>(v[13]);
    v[6] = w16<2, INV>(v[6]);
    v[10] = w16<4, INV>(v[10]);
    v[14] = w16<6, INV>(v[14]);
    v[7] = w16<3, INV>(v[7]);
    v[11] = w16<6, INV>(v[11]);
    v[15] = w16<9, INV>(v[15]);
    // DFT4 over m2 for each k1 (elements 4k1 .. 4k1+3) -> X[k1 + 4 k2] at v[4 k1 + k2]
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) dft4<INV>(v[4 * k1], v[4 * k1 + 1], v[4 * k1 + 2], v[4 * k1 + 3]);
    // transpose the 4 x 4 index (v[4 k1 + k2] -> v[k1 + 4 k2])
    float2 t;
    t = v[1]; v[1] = v[4]; v[4] = t;
    t = v[2]; v[2] = v[8]; v[8] = t;
    t = v[3]; v[3] = v[12]; v[12] = t;
    t = v[6]; v[6] = v[9]; v[9] = t;
    t = v[7]; v[7] = v[13]; v[13] = t;
    t = v[11]; v[11] = v[14]; v[14] = t;
}

// bytes each CTA receives per exchange: a 32 x 32 block from each other CTA
constexpr unsigned PUSH_BYTES = (CL - 1) * SL * SL * sizeof(float2);
constexpr uint64_t PUSH_WAIT_NS = 2000000000ull;   // then the error word is set
constexpr int ERR_PLANE_EXCHANGE = 3;

// Arrive with release semantics: this thread's earlier reads of its shared
// memory (and the barrier initialisation) are ordered before the other CTAs'
// pushes that follow their wait.
__device__ __forceinline__ void cluster_arrive() { asm volatile("barrier.cluster.arrive.release;" ::: "memory"); }
__device__ __forceinline__ void cluster_wait() { asm volatile("barrier.cluster.wait;" ::: "memory"); }

// The shared::cluster address of shared-memory address a in CTA `rank`.
__device__ __forceinline__ uint32_t map_rank(uint32_t a, int rank)
{
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
    return r;
}

// 8 bytes into another CTA's shared memory; completes 8 transaction bytes on
// that CTA's barrier.
__device__ __forceinline__ void push8(uint32_t addr, float2 v, uint32_t bar)
{
    asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v2.f32 [%0], {%1, %2}, [%3];" ::"r"(addr),
                 "f"(v.x), "f"(v.y), "r"(bar)
                 : "memory");
}

// Waits for the phase with the given parity to complete, with acquire
// semantics at cluster scope (the bytes come from other CTAs' st.async);
// false after limit_ns nanoseconds.
__device__ __forceinline__ bool wait_pushed(uint64_t* bar, uint32_t parity, uint64_t limit_ns)
{
    const uint32_t a = tc5::smem_u32(bar);
    uint64_t t0 = 0;
    for (bool first = true;; first = false) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
        if (first) t0 = tc5::global_ns();
        else if (tc5::global_ns() - t0 > limit_ns) return false;
    }
}

// Receiving side of the exchanges of one kernel: the mbarrier (one arrival,
// by thread 0 with the expected bytes, per exchange), the phase, and whether
// every wait so far completed.
struct Exchange {
    uint64_t* bar;
    int* err;
    uint32_t phase;
    bool ok;
};

__device__ __forceinline__ void arm(uint64_t* bar)
{
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(
                     tc5::smem_u32(bar)),
                 "r"(PUSH_BYTES)
                 : "memory");
}

// Thread 0 initialises the barrier and arms the first exchange; the other
// CTAs see the initialisation through the relaxed cluster barrier that comes
// before any push.
__device__ __forceinline__ Exchange exchange_init(float2* smem, int* err)
{
    Exchange x{reinterpret_cast<uint64_t*>(smem + SMEM_COMPLEX), err, 0u, true};
    if (threadIdx.x == 0) {
        tc5::mbar_init(x.bar, 1);
        arm(x.bar);
    }
    return x;
}

// Waits (bounded) until every pushed block of this exchange has landed, arms
// the next exchange (more) and makes this CTA's own block, written with plain
// stores, visible to all its threads.  A wait that runs out of time sets the
// error word; the kernel still passes every later barrier, so nothing hangs.
__device__ __forceinline__ void receive(Exchange& x, bool more)
{
    if (x.ok && !wait_pushed(x.bar, x.phase & 1u, PUSH_WAIT_NS)) {
        x.ok = false;
        if (x.err) atomicExch(x.err, ERR_PLANE_EXCHANGE);
    }
    ++x.phase;
    if (more && x.ok && threadIdx.x == 0) arm(x.bar);
    __syncthreads();
}

// Self test of the bounded exchange wait: the barrier is armed for an
// exchange that no CTA ever pushes, so every thread's wait runs out after
// limit_ns and the error word is set.
__global__ void k_selftest_exchange_wait(int* err, unsigned long long limit_ns)
{
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        tc5::mbar_init(&bar, 1);
        arm(&bar);
    }
    __syncthreads();
    if (!wait_pushed(&bar, 0u, limit_ns)) atomicExch(err, ERR_PLANE_EXCHANGE);
}

// Rows context (x transforms): slot s of thread t handles row
// (warp + WARPS s) * 2 + lane / 16 and line thread j = lane % 16.
struct RowSlot {
    int row, j;
};
__device__ __forceinline__ RowSlot row_slot(int s)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    return {(warp + WARPS * s) * 2 + (lane >> 4), lane & 15};
}
// Columns context (y and z transforms): column c = lane, line thread j = warp + WARPS s.
struct ColSlot {
    int c, j;
};
__device__ __forceinline__ ColSlot col_slot(int s)
{
    return {(int)(threadIdx.x & 31), (int)(threadIdx.x >> 5) + WARPS * s};
}

// Exchange between the two radix-16 stages for both slots of every thread.
// rows: buffer [row][a][TPAD]; cols: buffer [a][b][SL] (column fastest).
template <bool ROWS>
__device__ __forceinline__ void exchange(float2* T, float2 (&v0)[16], float2 (&v1)[16])
{
#pragma unroll
    for (int s = 0; s < NS; ++s) {
        float2(&v)[16] = s ? v1 : v0;
        if (ROWS) {
            const RowSlot q = row_slot(s);
            float2* b = T + q.row * (16 * TPAD) + q.j * TPAD;
#pragma unroll
            for (int k = 0; k < 16; ++k) b[k] = v[k];
        } else {
            const ColSlot q = col_slot(s);
#pragma unroll
            for (int k = 0; k < 16; ++k) T[(q.j * 16 + k) * SL + q.c] = v[k];
        }
    }
    __syncthreads();
#pragma unroll
    for (int s = 0; s < NS; ++s) {
        float2(&v)[16] = s ? v1 : v0;
        if (ROWS) {
            const RowSlot q = row_slot(s);
            const float2* b = T + q.row * (16 * TPAD) + q.j;
#pragma unroll
            for (int a = 0; a < 16; ++a) v[a] = b[a * TPAD];
        } else {
            const ColSlot q = col_slot(s);
#pragma unroll
            for (int a = 0; a < 16; ++a) v[a] = T[(a * 16 + q.j) * SL + q.c];
        }
    }
    __syncthreads();
}

// Four-step 256-point transform.  Forward: v[n1] = x[16 n1 + j] in,
// v[k2] = X[j + 16 k2] out.  Inverse: the reverse.  LOCAL_IN: v0/v1 were
// read from a receive buffer that T overlays, so all threads finish reading
// before T is written.  ARRIVE: arrive at the cluster barrier once this CTA's
// reads of T are done, so the other CTAs may push into it.
template <bool INV, bool ROWS, bool LOCAL_IN = false, bool ARRIVE = false>
__device__ __forceinline__ void fft256(float2* T, const float2* tw, float2 (&v0)[16], float2 (&v1)[16])
{
#pragma unroll
    for (int s = 0; s < NS; ++s) {
        float2(&v)[16] = s ? v1 : v0;
        const int j = ROWS ? row_slot(s).j : col_slot(s).j;
        dft16<INV>(v);
#pragma unroll
        for (int k = 1; k < 16; ++k) v[k] = cmul_ff<INV>(v[k], tw[j * k], tw[N + j * k]);
    }
    if (LOCAL_IN) __syncthreads();
    exchange<ROWS>(T, v0, v1);
    if (ARRIVE) cluster_arrive();
    dft16<INV>(v0);
    if (NS > 1) dft16<INV>(v1);
}

struct Args {
    const float2* src;     // k_plane_fwd: state rows.  k_plane_inv: spectrum after k_zpass
    float2* dst;           // spectrum of the next application (forward output)
    const float2* tw;      // W_256^t, t < 256 (nearest floats)
    const float2* twl;     // remainders of the twiddles
    const float* kx2;
    const float* ky2;
    const float* kz2;
    int* err;              // error word (an exchange wait that ran out of time)
    EpiArgs e;
};

// W_256^t, t < 256, at tw[t] (nearest floats) and tw[256 + t] (remainders)
__device__ __forceinline__ void load_twiddles(float2* tw, const float2* g, const float2* gl)
{
    for (int t = threadIdx.x; t < N; t += blockDim.x) {
        tw[t] = g[t];
        if (kCompensatedTwiddles) tw[N + t] = gl[t];
    }
}

// Bulk prefetch of a contiguous range into L2 (no registers, no shared
// memory); p 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void prefetch_l2(const void* p, unsigned bytes)
{
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

// Columns to rows: this CTA (columns x in [32r, 32r+32)) sends the value at
// (y = 16 n1 + j, x = 32 r + c) to the owner of row y, R[(y & 31) N + x].
__device__ __forceinline__ void push_cols_to_rows(float2* R, const Exchange& xc, float2 (&v0)[16],
                                                  float2 (&v1)[16], int r)
{
    const uint32_t rb = tc5::smem_u32(R), bar = tc5::smem_u32(xc.bar);
#pragma unroll
    for (int s = 0; s < NS; ++s) {
        const ColSlot q = col_slot(s);
        float2(&v)[16] = s ? v1 : v0;
#pragma unroll
        for (int n1 = 0; n1 < 16; ++n1) {
            const int d = n1 >> 1;
            const int off = (16 * (n1 & 1) + q.j) * N + SL * r + q.c;
            if (d == r) R[off] = v[n1];
            else push8(map_rank(rb + 8u * off, d), v[n1], map_rank(bar, d));
        }
    }
}

// Rows to columns: this CTA (rows y in [32r, 32r+32)) sends the value at
// (y = 32 r + row, x = j + 16 k2) to the owner of column x, R[y 32 + (x & 31)].
__device__ __forceinline__ void push_rows_to_cols(float2* R, const Exchange& xc, float2 (&v0)[16],
                                                  float2 (&v1)[16], int r)
{
    const uint32_t rb = tc5::smem_u32(R), bar = tc5::smem_u32(xc.bar);
#pragma unroll
    for (int s = 0; s < NS; ++s) {
        const RowSlot q = row_slot(s);
        float2(&v)[16] = s ? v1 : v0;
        const int y = SL * r + q.row;
#pragma unroll
        for (int k2 = 0; k2 < 16; ++k2) {
            const int d = k2 >> 1;
            const int off = y * SL + q.j + 16 * (k2 & 1);
            if (d == r) R[off] = v[k2];
            else push8(map_rank(rb + 8u * off, d), v[k2], map_rank(bar, d));
        }
    }
}

// Forward x FFT of this CTA's 32 rows (values in v0/v1, spatial order) then
// forward y FFT of its 32 columns; spectrum stored to dst plane z.
__device__ __forceinline__ void forward_xy(float2* smem, const float2* tw,
                                           float2 (&v0)[16], float2 (&v1)[16], float2* dst, int z, int r,
                                           Exchange& xc)
{
    float2* T = smem;
    fft256<false, true, false, true>(T, tw, v0, v1);
    cluster_wait();   // every CTA's transpose buffer is free
    push_rows_to_cols(smem, xc, v0, v1, r);
    receive(xc, false);
#pragma unroll
    for (int s = 0; s < NS; ++s) {
        const ColSlot q = col_slot(s);
        float2(&v)[16] = s ? v1 : v0;
#pragma unroll
        for (int n1 = 0; n1 < 16; ++n1) v[n1] = smem[(16 * n1 + q.j) * SL + q.c];
    }
    fft256<false, false, true>(T, tw, v0, v1);
    float2* out = dst + (size_t)z * N * N + SL * r;
#pragma unroll
    for (int s = 0; s < NS; ++s) {
        const ColSlot q = col_slot(s);
        float2(&v)[16] = s ? v1 : v0;
#pragma unroll
        for (int k2 = 0; k2 < 16; ++k2) out[(size_t)(q.j + 16 * k2) * N + q.c] = v[k2];
    }
}

__global__ void __cluster_dims__(CL, 1, 1) __launch_bounds__(THREADS, 2) k_plane_fwd(Args a)
{
    extern __shared__ float4 smem4[];
    float2* smem = reinterpret_cast<float2*>(smem4);
    float2* tw = smem + (SMEM_COMPLEX - 2 * N - 3 * N / 2);
    cg::cluster_group cluster = cg::this_cluster();
    const int r = (int)cluster.block_rank();
    const int z = blockIdx.y;
    load_twiddles(tw, a.tw, a.twl);
    Exchange xc = exchange_init(smem, a.err);
    griddep_launch();
    griddep_wait();
    float2 v0[16], v1[16];
    const float2* in = a.src + ((size_t)z * N + SL * r) * N;
#pragma unroll
    for (int s = 0; s < NS; ++s) {
        const RowSlot q = row_slot(s);
        float2(&v)[16] = s ? v1 : v0;
#pragma unroll
        for (int n1 = 0; n1 < 16; ++n1) v[n1] = in[(size_t)q.row * N + 16 * n1 + q.j];
    }
    __syncthreads();
    forward_xy(smem, tw, v0, v1, a.dst, z, r, xc);
}

// The pointwise update of one row slot (x = 16 n1 + j): scal_vr_3d, the
// recurrence, and add_bessel_3d / apply_ABC_Xt of ose_3d_lib.cu:651-870 by
// the partial-sum schedule e.sp (SumPlan), fused.  v holds the unnormalised
// inverse transform on entry and the new term a_{n+1} (FIRST: a_1) on exit.
// Loads are issued ECH cells at a time ahead of any store; the buffers never
// overlap at different cells, so the restrict qualifiers are exact.
// SUM: 0 = S left alone, 1 = S written (its first update of the step),
// 2 = S read and written (SumPlan: touch, s_read); LAST always has 2.
// The partial-sum update in this kernel takes the sponge as att = ax[x] *
// (ay[y] az[z]): the powers of ax come from the shared table axp (axp[(k-1)
// N + x] = ax[x]^k), those of ay az, times the coefficients, are per row.
template <int EPI, int SUM>
__device__ __forceinline__ void epilogue_slot(float2 (&v)[16], const EpiArgs& e, const float* axp, int y, int z,
                                              int j)
{
    float2* __restrict__ prev = e.prev;
    float2* __restrict__ S = e.S;
    float2* __restrict__ wout = e.wout;
    const float* __restrict__ vs = e.vs;
    const size_t rowbase = ((size_t)z * N + y) * N + j;
    constexpr bool upd = EPI == EPI_LAST || (EPI == EPI_MID && SUM > 0);
    // cells whose loads are in flight together (8 everywhere: measured
    // fastest, with a few spilled registers in the last application)
    constexpr int CH = SUM == 2 ? (EPI == EPI_MID ? ECH_SUM : (EPI == EPI_LAST ? ECH_LAST : ECH)) : ECH;
    constexpr bool sread = upd && SUM == 2;
    const float attyz = upd ? __ldg(e.ay + y) * __ldg(e.az + z) : 1.f;
    // row factors of the schedule (SumPlan): S times ax^kS qS, a_{n-1} times
    // ax^kP (qP + qPl), a_{n+1} times ax (qN + qNl)
    const SumPlan& sp = e.sp;
    const float y2 = attyz * attyz, y3 = y2 * attyz;
    auto ypow = [&](int k) { return k <= 1 ? attyz : (k == 2 ? y2 : y3); };
    const float qS = sread ? ypow(sp.kS) : 0.f;
    const float yP = sp.add_prev ? ypow(sp.kP) : 0.f;
    const float qP = e.cp * yP, qPl = e.cpl * yP;
    const float qN = sp.add_new ? e.c1 * attyz : 0.f, qNl = sp.add_new ? e.c1l * attyz : 0.f;
    const float* axS = axp + (sp.kS > 1 ? sp.kS - 1 : 0) * N;
    const float* axP = axp + (sp.kP > 1 ? sp.kP - 1 : 0) * N;
    auto update = [&](float2 s, float2 am, float2 an, int x) {
        const float ax = axp[x], fS = axS[x] * qS, aP = axP[x];
        const float fP = aP * qP, fN = ax * qN;
        float2 r = make_float2(s.x * fS, s.y * fS);
        if (kCompensatedConstants) {
            const float lP = aP * qPl, lN = ax * qNl;
            r.x = fmaf(lP, am.x, fmaf(lN, an.x, r.x));
            r.y = fmaf(lP, am.y, fmaf(lN, an.y, r.y));
        }
        r.x = fmaf(fP, am.x, fmaf(fN, an.x, r.x));
        r.y = fmaf(fP, am.y, fmaf(fN, an.y, r.y));
        return r;
    };
#pragma unroll
    for (int h = 0; h < 16 / CH; ++h) {
        float vv[CH];
        float2 am[CH], sm[CH];
#pragma unroll
        for (int q = 0; q < CH; ++q) {
            const size_t i = rowbase + 16 * (CH * h + q);
            vv[q] = __ldg(vs + i);
            if (EPI == EPI_MID || EPI == EPI_LAST) am[q] = prev[i];
            sm[q] = sread ? S[i] : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int q = 0; q < CH; ++q) {
            const int n1 = CH * h + q;
            const int x = 16 * n1 + j;
            const size_t i = rowbase + 16 * n1;
            // L a_n = v * X * (sch + scl)  (vv = v / (R N) when not compensated)
            float2 Lx = make_float2(v[n1].x * vv[q], v[n1].y * vv[q]);
            if (kCompensatedConstants)
                Lx = make_float2(fmaf(Lx.x, e.sch, Lx.x * e.scl), fmaf(Lx.y, e.sch, Lx.y * e.scl));
            if (EPI == EPI_SCALE) {
                prev[i] = Lx;
            } else if (EPI == EPI_FIRST) {
                // a_1 = -i L a_0
                const float2 a1 = make_float2(Lx.y, -Lx.x);
                prev[i] = a1;
                if (SUM) S[i] = sum_update(e, 1.f, make_float2(0.f, 0.f), a1, a1);
                v[n1] = a1;
            } else {
                // a_{n+1} = a_{n-1} - 2i L a_n
                const float2 an = make_float2(fmaf(2.f, Lx.y, am[q].x), fmaf(-2.f, Lx.x, am[q].y));
                if (EPI == EPI_MID) {
                    prev[i] = an;
                    if (upd) S[i] = update(sm[q], am[q], an, x);
                    v[n1] = an;
                } else {
                    const float2 s = update(sm[q], am[q], an, x);
                    wout[i] = s;
                    if (z == e.gz) {
                        const int ix = x - e.bl, iy = y - e.bf;
                        if (ix >= 0 && ix < e.nx && iy >= 0 && iy < e.ny) {
                            const int c = *e.cur;
                            if (c >= 0 && c < e.nt) e.gather[(size_t)c * e.nx * e.ny + iy * e.nx + ix] = s.y;
                        }
                    }
                }
            }
        }
    }
}

// Inverse y and x FFTs of plane z, the pointwise update, and (FWD) the
// forward x and y FFTs of the new term.
template <int EPI, bool FWD, int SUM = 2>
__global__ void __cluster_dims__(CL, 1, 1) __launch_bounds__(THREADS, 2) k_plane_inv(Args a)
{
    extern __shared__ float4 smem4[];
    float2* smem = reinterpret_cast<float2*>(smem4);
    float2* tw = smem + (SMEM_COMPLEX - 2 * N - 3 * N / 2);
    float* axp = reinterpret_cast<float*>(tw + 2 * N);
    cg::cluster_group cluster = cg::this_cluster();
    const int r = (int)cluster.block_rank();
    const int z = blockIdx.y;
    if (EPI == EPI_MID || EPI == EPI_LAST) {
        for (int t = threadIdx.x; t < N; t += blockDim.x) {
            const float ax = __ldg(a.e.ax + t);
            axp[t] = ax;
            axp[N + t] = ax * ax;
            axp[2 * N + t] = ax * ax * ax;
        }
    }
    // The epilogue's operands of this CTA's 32 rows are contiguous: start
    // pulling them into L2 now, so the epilogue's loads hit L2 (v is constant;
    // a_{n-1} and S only once the kernels that wrote them have completed).
    const size_t row0 = ((size_t)z * N + SL * r) * N;
    if (threadIdx.x == 0 && EPI != EPI_SCALE) prefetch_l2(a.e.vs + row0, SL * N * sizeof(float));
    load_twiddles(tw, a.tw, a.twl);
    Exchange xc = exchange_init(smem, a.err);
    griddep_launch();
    griddep_wait();
    if (threadIdx.x == 0 && EPI != EPI_SCALE && EPI != EPI_FIRST) {
        prefetch_l2(a.e.prev + row0, SL * N * sizeof(float2));
        if (SUM == 2) prefetch_l2(a.e.S + row0, SL * N * sizeof(float2));
    }
    float2 v0[16], v1[16];
    // spectrum columns 32r..: thread (c, j) takes ky = j + 16 k2
    const float2* in = a.src + (size_t)z * N * N + SL * r;
#pragma unroll
    for (int s = 0; s < NS; ++s) {
        const ColSlot q = col_slot(s);
        float2(&v)[16] = s ? v1 : v0;
#pragma unroll
        for (int k2 = 0; k2 < 16; ++k2) v[k2] = in[(size_t)(q.j + 16 * k2) * N + q.c];
    }
    __syncthreads();
    float2* T = smem;
    fft256<true, false, false, true>(T, tw, v0, v1);
    cluster_wait();   // every CTA's transpose buffer is free, its barrier initialised
    push_cols_to_rows(smem, xc, v0, v1, r);
    receive(xc, FWD);
    // rows 32r..: thread (row, j) takes kx = j + 16 k2
#pragma unroll
    for (int s = 0; s < NS; ++s) {
        const RowSlot q = row_slot(s);
        float2(&v)[16] = s ? v1 : v0;
#pragma unroll
        for (int k2 = 0; k2 < 16; ++k2) v[k2] = smem[q.row * N + q.j + 16 * k2];
    }
    fft256<true, true, true>(T, tw, v0, v1);
    // pointwise update on (x = 16 n1 + j, y, z)
    epilogue_slot<EPI, SUM>(v0, a.e, axp, SL * r + row_slot(0).row, z, row_slot(0).j);
    if (NS > 1) epilogue_slot<EPI, SUM>(v1, a.e, axp, SL * r + row_slot(1).row, z, row_slot(1).j);
    if (FWD) forward_xy(smem, tw, v0, v1, a.dst, z, r, xc);
}

// z lines of a 16-wide kx tile at one ky: forward, * |k|, inverse, in place.
// One line slot per thread (column c = t % 16, line thread j = t / 16) keeps
// registers near 64 so four CTAs share an SM.
#ifndef OSE_ZPASS_MINB
#define OSE_ZPASS_MINB 4
#endif
constexpr int ZW = 16;
constexpr int ZTHREADS = 256;
constexpr size_t ZSMEM_BYTES = sizeof(float2) * (16 * 16 * ZW + 2 * N);

// (hi, lo) + (hi, lo) as a float pair (Knuth's two-sum on the high parts)
__device__ __forceinline__ void ff_add(float ah, float al, float bh, float bl, float& h, float& l)
{
    const float s = ah + bh;
    const float bb = s - ah;
    const float e = (ah - (s - bb)) + (bh - bb);
    h = s;
    l = e + al + bl;
}

// GRID: any grid with 256 z planes and nxb a multiple of 16 (row stride
// nxb, plane stride nxb * nyb as arguments: the generic path's z pass);
// otherwise the 256^3 plane path's, with the strides as constants (runtime
// strides cost registers: the GRID form spills a little at this bound, which
// measured faster than three CTAs per SM without most of the spills).
template <bool GRID>
__global__ void __launch_bounds__(ZTHREADS, OSE_ZPASS_MINB) k_zpass16(float2* __restrict__ X, const float2* __restrict__ gtw,
                                                         Tables t, int nxb_arg, long long plane_arg)
{
    extern __shared__ float4 smem4[];
    float2* T = reinterpret_cast<float2*>(smem4);
    float2* tw = T + 16 * 16 * ZW;
    load_twiddles(tw, gtw, t.twl);
    griddep_launch();
    griddep_wait();
    const int c = threadIdx.x & (ZW - 1), j = threadIdx.x / ZW;
    const int ky = blockIdx.y, kx = ZW * blockIdx.x + c;
    const int nxb = GRID ? nxb_arg : N;
    const size_t plane = GRID ? (size_t)plane_arg : (size_t)N * N;
    float2* base = X + (size_t)ky * nxb + kx;
    float2 v[16];
#pragma unroll
    for (int n1 = 0; n1 < 16; ++n1) v[n1] = base[(size_t)(16 * n1 + j) * plane];
    __syncthreads();
    // forward: DFT16 over n1, twiddle, transpose, DFT16 over n2
    dft16<false>(v);
#pragma unroll
    for (int k = 1; k < 16; ++k) v[k] = cmul_ff<false>(v[k], tw[j * k], tw[N + j * k]);
#pragma unroll
    for (int k = 0; k < 16; ++k) T[(j * 16 + k) * ZW + c] = v[k];
    __syncthreads();
#pragma unroll
    for (int a = 0; a < 16; ++a) v[a] = T[(a * 16 + j) * ZW + c];
    __syncthreads();
    dft16<false>(v);
    // v[k2] = spectrum at kz = j + 16 k2.  Compensated: |k| to about 44 bits
    // (k^2 as a float pair, sqrt of its high part, one Newton correction).
    if (kCompensatedConstants) {
        float kxyh, kxyl;
        ff_add(__ldg(t.kx2 + kx), __ldg(t.kx2l + kx), __ldg(t.ky2 + ky), __ldg(t.ky2l + ky), kxyh, kxyl);
#pragma unroll
        for (int k2 = 0; k2 < 16; ++k2) {
            const int kz = j + 16 * k2;
            float sh, sl;
            ff_add(kxyh, kxyl, __ldg(t.kz2 + kz), __ldg(t.kz2l + kz), sh, sl);
            const float r = sqrtf(sh);
            const float e = fmaf(-r, r, sh) + sl;
            const float rl = r > 0.f ? 0.5f * e / r : 0.f;
            v[k2] = make_float2(fmaf(v[k2].x, r, v[k2].x * rl), fmaf(v[k2].y, r, v[k2].y * rl));
        }
    } else {
        const float kxy = __ldg(t.kx2 + kx) + __ldg(t.ky2 + ky);
#pragma unroll
        for (int k2 = 0; k2 < 16; ++k2) {
            const float k = sqrtf(kxy + __ldg(t.kz2 + j + 16 * k2));
            v[k2].x *= k;
            v[k2].y *= k;
        }
    }
    // inverse: IDFT16 over k2, twiddle, transpose, IDFT16 over k1
    dft16<true>(v);
#pragma unroll
    for (int k = 1; k < 16; ++k) v[k] = cmul_ff<true>(v[k], tw[j * k], tw[N + j * k]);
#pragma unroll
    for (int k = 0; k < 16; ++k) T[(j * 16 + k) * ZW + c] = v[k];
    __syncthreads();
#pragma unroll
    for (int a = 0; a < 16; ++a) v[a] = T[(a * 16 + j) * ZW + c];
    dft16<true>(v);
#pragma unroll
    for (int n1 = 0; n1 < 16; ++n1) base[(size_t)(16 * n1 + j) * plane] = v[n1];
}

}  // namespace plane

bool plane_path_supported(int nxb, int nyb, int nzb)
{
    return nxb == plane::N && nyb == plane::N && nzb == plane::N;
}

cudaError_t configure_plane_kernels()
{
    cudaError_t e;
    const int bytes = (int)plane::SMEM_BYTES;
#define ALLOW(k)                                                                              \
    if ((e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes)) != \
        cudaSuccess)                                                                          \
        return e
    ALLOW(plane::k_plane_fwd);
    ALLOW((plane::k_plane_inv<EPI_FIRST, true, 0>));
    ALLOW((plane::k_plane_inv<EPI_FIRST, true, 1>));
    ALLOW((plane::k_plane_inv<EPI_MID, true, 0>));
    ALLOW((plane::k_plane_inv<EPI_MID, true, 1>));
    ALLOW((plane::k_plane_inv<EPI_MID, true, 2>));
    ALLOW((plane::k_plane_inv<EPI_MID, false, 0>));
    ALLOW((plane::k_plane_inv<EPI_MID, false, 1>));
    ALLOW((plane::k_plane_inv<EPI_LAST, false>));
    ALLOW((plane::k_plane_inv<EPI_MID, false>));
    ALLOW((plane::k_plane_inv<EPI_SCALE, false>));
    ALLOW(plane::k_zpass16<false>);
    ALLOW(plane::k_zpass16<true>);
#undef ALLOW
    return cudaSuccess;
}

cudaError_t launch_plane_fwd(cudaStream_t s, const float2* state, float2* X, const Tables& t)
{
    plane::Args a{};
    a.src = state;
    a.dst = X;
    a.tw = t.twx;
    a.twl = t.twl;
    a.err = t.tcerr;
    return launch_pdl(plane::k_plane_fwd, dim3(plane::CL, plane::N), dim3(plane::THREADS), plane::SMEM_BYTES, s, a);
}

cudaError_t launch_zpass(cudaStream_t s, float2* X, const Tables& t)
{
    if (t.tcvar != OSE_PRECISION_FP32) {
        Geometry g{plane::N, plane::N, plane::N, (long long)plane::N * plane::N * plane::N};
        return launch_tensor_zpass(s, X, g, t);
    }
    return launch_pdl(plane::k_zpass16<false>, dim3(plane::N / plane::ZW, plane::N), dim3(plane::ZTHREADS),
                      plane::ZSMEM_BYTES, s, X, (const float2*)t.twx, t, (int)plane::N,
                      (long long)plane::N * plane::N);
}

cudaError_t selftest_exchange_wait(cudaStream_t s, int* err, unsigned long long limit_ns)
{
    plane::k_selftest_exchange_wait<<<1, 64, 0, s>>>(err, limit_ns);
    return cudaGetLastError();
}

bool zpass256_supported(const Geometry& g) { return g.nzb == plane::N && g.nxb % plane::ZW == 0; }

cudaError_t launch_zpass256(cudaStream_t s, float2* X, const Geometry& g, const Tables& t)
{
    // a plain launch: with programmatic serialisation the generic path's
    // passes measured slower (320 x 288 x 256: 4.57 -> 4.78 ms/step)
    plane::k_zpass16<true><<<dim3(g.nxb / plane::ZW, g.nyb), plane::ZTHREADS, plane::ZSMEM_BYTES, s>>>(
        X, t.twz, t, g.nxb, (long long)g.nxb * g.nyb);
    return cudaGetLastError();
}

// mode: EPI_FIRST / EPI_MID with the next forward fused (fwd = true), or
// EPI_LAST without it.  Xin: spectrum after the z pass; Xout: next spectrum.
cudaError_t launch_plane_inv(cudaStream_t s, EpiMode mode, bool fwd, const float2* Xin, float2* Xout,
                             const Tables& t, const EpiArgs& e)
{
    plane::Args a{};
    a.src = Xin;
    a.dst = Xout;
    a.tw = t.twx;
    a.twl = t.twl;
    a.err = t.tcerr;
    a.e = e;
    const dim3 grid(plane::CL, plane::N), block(plane::THREADS);
    const size_t sm = plane::SMEM_BYTES;
    const int sum = e.sp.touch ? (e.sp.s_read ? 2 : 1) : 0;
    if (mode == EPI_FIRST)   // the first application never reads S
        return sum ? launch_pdl(plane::k_plane_inv<EPI_FIRST, true, 1>, grid, block, sm, s, a)
                   : launch_pdl(plane::k_plane_inv<EPI_FIRST, true, 0>, grid, block, sm, s, a);
    if (mode == EPI_MID && fwd)
        return sum == 2 ? launch_pdl(plane::k_plane_inv<EPI_MID, true, 2>, grid, block, sm, s, a)
               : sum == 1 ? launch_pdl(plane::k_plane_inv<EPI_MID, true, 1>, grid, block, sm, s, a)
                          : launch_pdl(plane::k_plane_inv<EPI_MID, true, 0>, grid, block, sm, s, a);
    if (mode == EPI_MID)
        return sum == 2 ? launch_pdl(plane::k_plane_inv<EPI_MID, false, 2>, grid, block, sm, s, a)
               : sum == 1 ? launch_pdl(plane::k_plane_inv<EPI_MID, false, 1>, grid, block, sm, s, a)
                          : launch_pdl(plane::k_plane_inv<EPI_MID, false, 0>, grid, block, sm, s, a);
    // LAST always reads S: an earlier application of every step stores it
    if (sum != 2) return cudaErrorInvalidValue;
    return launch_pdl(plane::k_plane_inv<EPI_LAST, false, 2>, grid, block, sm, s, a);
}

// out = v * IFFT3(|k| FFT3(in)) * (sch + scl) with the plane kernels.
cudaError_t launch_plane_apply_operator(cudaStream_t s, const float2* in, float2* X, float2* out,
                                        const float* vs, float sch, float scl, const Tables& t)
{
    cudaError_t e = launch_plane_fwd(s, in, X, t);
    if (e != cudaSuccess) return e;
    if ((e = launch_zpass(s, X, t)) != cudaSuccess) return e;
    plane::Args a{};
    a.src = X;
    a.tw = t.twx;
    a.twl = t.twl;
    a.err = t.tcerr;
    a.e.prev = out;
    a.e.vs = vs;
    a.e.sch = sch;
    a.e.scl = scl;
    plane::k_plane_inv<EPI_SCALE, false><<<dim3(plane::CL, plane::N), plane::THREADS, plane::SMEM_BYTES, s>>>(a);
    return cudaGetLastError();
}

int plane_max_active_clusters()
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(plane::CL, plane::N);
    cfg.blockDim = dim3(plane::THREADS);
    cfg.dynamicSmemBytes = plane::SMEM_BYTES;
    cudaLaunchAttribute attr;
    attr.id = cudaLaunchAttributeClusterDimension;
    attr.val.clusterDim.x = plane::CL;
    attr.val.clusterDim.y = 1;
    attr.val.clusterDim.z = 1;
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, (void*)(plane::k_plane_inv<EPI_MID, true>), &cfg) != cudaSuccess)
        return -1;
    return n;
}

}  // namespace ose
