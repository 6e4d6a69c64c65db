// ose_learn_tc.cu - inference of the boundary corrector on the tcgen05 tensor
// cores: each 3x3x3 convolution layer is an implicit GEMM with BF16 weights
// and activations and an FP32 accumulator in TMEM.
//
// A CTA walks a column of output planes: 8 (x) x 16 (y) cells, the M rows of
// the MMA (row m = y * 8 + x), for up to ZL consecutive z.  It streams the
// input halo planes (10 x 18 cells, all input channels) through two shared-
// memory slots, each in the layout [y 18][channel chunk][x 10][8 channels x
// 2 bytes]: for an in-plane tap (dx, dy) the 128 x Cin operand is a plain
// K-major descriptor into the slot (rows 16 bytes apart, y groups SBO apart,
// channel chunks LBO apart, start shifted by dx * 16 bytes), so no im2col
// copy is made.  A halo plane at z feeds the outputs at z + 1, z and z - 1
// (taps dz = -1, 0, +1), so the B operand of a tap (dx, dy) holds the three
// dz weight blocks side by side and one MMA of N = 3 Cout updates the three
// output planes' accumulators, which sit next to one another in a ring of
// accumulators in TMEM (an MMA is split in two where the run wraps): each
// halo plane is read by the tensor core 9 times instead of 27.  The global
// loads of the next halo plane are in flight while the CTA writes out the
// plane that the last MMAs completed.
//
// Layer 0's halo is built from the state and the velocity (the 8 features;
// K = 16 pairs two x taps, see LayerCfg); hidden activations are BF16 [cell][32];
// the output layer adds s(x) (dP, dQ) to the state at the write cells.  Inputs
// outside the shell are zero, as in the FP32 kernels (ose_learn.cu).
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "ose_internal.h"
#include "ose_learn.h"
#include "tcgen05.cuh"

namespace ose {
namespace learn {

namespace {

constexpr int TXW = 8, TYW = 16;              // output tile (x, y) of one z plane
constexpr int HX = TXW + 2, HY = TYW + 2;
constexpr int ZL = 16;                        // output planes per column at most
constexpr int SLOTS = 2;                      // halo plane slots per pipeline
constexpr int TMEM_PER_PIPE = 128;            // TMEM columns per pipeline (4 pipelines per SM)
constexpr int kMinSmem = 80 * 1024;           // at most two CTAs per SM (their TMEM)
constexpr int PIPE_THREADS = 128;             // one output row (cell) per thread
constexpr int PIPES = 2;                      // independent columns per CTA (shared weights)
constexpr int THREADS = PIPES * PIPE_THREADS;
constexpr uint64_t kWaitLimitNs = 1000000000ull;

__device__ __forceinline__ int wrapi(int v, int n) { return v < 0 ? v + n : (v >= n ? v - n : v); }

__device__ __forceinline__ bool in_shell(const NetGeom& g, int x, int y, int z)
{
    const int d = min(min(min(x, g.nx - 1 - x), min(y, g.ny - 1 - y)), min(z, g.nz - 1 - z));
    return d < g.shell;
}

__device__ __forceinline__ bool is_write(const NetGeom& g, int x, int y, int z)
{
    return in_shell(g, x, y, z) && x >= g.sp[0] && x < g.nx - g.sp[1] && y >= g.sp[2] &&
           y < g.ny - g.sp[3] && z >= g.sp[4] && z < g.nz - g.sp[5];
}

__device__ __forceinline__ float face_coord(int v, int n, int shell)
{
    const int lo = v, hi = n - 1 - v;
    if (lo < shell && lo <= hi) return -(float)(shell - lo) / (float)shell;
    if (hi < shell) return (float)(shell - hi) / (float)shell;
    return 0.f;
}

__device__ __forceinline__ uint32_t pack2(float a, float b)
{
    __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    uint32_t u;
    memcpy(&u, &h, 4);
    return u;
}

// Layer 0 (CIN = 16: 8 features + 8 zero channels) uses PAIR taps: its halo
// has one 16-byte chunk per cell in rows of 11 cells (the 11th zero), and an
// A descriptor with LBO = 16 bytes reads K channels 8..15 from the next cell
// in x, so one K = 16 MMA applies two x taps (dx, dx + 1): 3 dy x 2 pairs
// ((-1, 0) and (+1, +2 with zero weights)) instead of 9 taps.
template <int CIN, int NPAD>
struct LayerCfg {
    static constexpr bool pair = CIN == 16;
    static constexpr int chunks = pair ? 1 : CIN / 8;            // 16-byte chunks per halo cell
    static constexpr int hxp = pair ? HX + 1 : HX;               // halo row length in cells
    static constexpr int plane_bytes = HY * chunks * hxp * 16;   // one halo plane
    static constexpr int halo_bytes = PIPES * SLOTS * plane_bytes;
    static constexpr uint32_t lbo = pair ? 16 : hxp * 16;        // A: K chunk stride
    static constexpr uint32_t sbo = chunks * hxp * 16;           // A: y stride
    static constexpr int kchunks = CIN / 8;                      // B: K chunks
    static constexpr int ntaps = pair ? 6 : 9;                   // B blocks: (dy, pair) or (dx, dy)
    static constexpr int ngroups = 3 * NPAD / 8;                 // B rows: dz = +1, 0, -1 blocks
    static constexpr int tap_bytes = ngroups * kchunks * 128;    // B operand of one tap
    static constexpr int w_bytes = ntaps * tap_bytes;
    static constexpr uint32_t wsbo = kchunks * 128;              // B: n-group stride
    static constexpr int ksteps = CIN / 16;
    static constexpr int off_w = halo_bytes;
    static constexpr int off_bias = off_w + w_bytes;
    static constexpr int off_bar = off_bias + NPAD * 4;          // 2 mbarriers per pipeline, TMEM address
    static constexpr int used = off_bar + 8 * 2 * PIPES + 8;
    static constexpr int smem = used > kMinSmem ? used : kMinSmem;
    // ring of accumulators (output planes) per pipeline: 4 of 32 columns, or
    // 8 of 16 for the output layer (a run of three wraps less often)
    static constexpr int ring = TMEM_PER_PIPE / NPAD;
    static constexpr int tmem_cols = PIPES * TMEM_PER_PIPE;
    // staged loads of one halo plane per thread: cells (layer 0) or 16-byte units
    static constexpr int cells = HY * HX;
    static constexpr int units = cells * chunks;
    static constexpr int per = ((pair ? cells : units) + PIPE_THREADS - 1) / PIPE_THREADS;
};

// One halo plane in registers: layer 0 keeps the state, velocity and scale of
// each cell; the other layers keep 16-byte units of BF16 activations.
template <int MODE, int PER>
struct Staged {
    float2 w[MODE == 0 ? PER : 1];
    float v[MODE == 0 ? PER : 1], s[MODE == 0 ? PER : 1];
    uint4 u[MODE == 0 ? 1 : PER];
    bool ok[PER];
};

template <int CIN, int NPAD, int MODE>
__device__ __forceinline__ void load_plane(Staged<MODE, LayerCfg<CIN, NPAD>::per>& st, const uint16_t* act_in,
                                           const float2* Win, const float* vel, const float* scal,
                                           const NetGeom& g, int x0, int y0, int z, int t)
{
    using C = LayerCfg<CIN, NPAD>;
#pragma unroll
    for (int k = 0; k < C::per; ++k) {
        const int u = t + k * PIPE_THREADS;
        const int ch = MODE == 0 ? 0 : u % C::chunks, cell = MODE == 0 ? u : u / C::chunks;
        const int hx = cell % HX, hy = cell / HX;
        const int x = wrapi(x0 + hx - 1, g.nx), y = wrapi(y0 + hy - 1, g.ny);
        const bool ok = u < (MODE == 0 ? C::cells : C::units) && in_shell(g, x, y, z);
        const size_t c = ((size_t)z * g.ny + y) * g.nx + x;
        st.ok[k] = ok;
        if (MODE == 0) {
            st.w[k] = ok ? __ldg(Win + c) : make_float2(0.f, 0.f);
            st.v[k] = ok ? __ldg(vel + c) : 0.f;
            st.s[k] = ok ? __ldg(scal + c) : 1.f;
        } else {
            st.u[k] = ok ? __ldg(reinterpret_cast<const uint4*>(act_in + c * CIN + ch * 8)) : make_uint4(0, 0, 0, 0);
        }
    }
}

template <int CIN, int NPAD, int MODE>
__device__ __forceinline__ void store_plane(const Staged<MODE, LayerCfg<CIN, NPAD>::per>& st, uint8_t* slot,
                                            const NetGeom& g, int x0, int y0, int z, int t)
{
    using C = LayerCfg<CIN, NPAD>;
#pragma unroll
    for (int k = 0; k < C::per; ++k) {
        const int u = t + k * PIPE_THREADS;
        if (u >= (MODE == 0 ? C::cells : C::units)) break;
        const int ch = MODE == 0 ? 0 : u % C::chunks, cell = MODE == 0 ? u : u / C::chunks;
        const int hx = cell % HX, hy = cell / HX;
        uint4 v = MODE == 0 ? make_uint4(0, 0, 0, 0) : st.u[k];
        if (MODE == 0 && st.ok[k]) {
            const int x = wrapi(x0 + hx - 1, g.nx), y = wrapi(y0 + hy - 1, g.ny);
            const float inv = 1.f / st.s[k];
            v.x = pack2(st.w[k].x * inv, st.w[k].y * inv);
            v.y = pack2(st.v[k] * (1.f / 4500.f), face_coord(x, g.nx, g.shell));
            v.z = pack2(face_coord(y, g.ny, g.shell), face_coord(z, g.nz, g.shell));
        }
        *reinterpret_cast<uint4*>(slot + ((hy * C::chunks + ch) * C::hxp + hx) * 16) = v;
    }
}

// Barrier of one pipeline's 128 threads (named barrier 1 + pipe); returns
// whether any of them passed v != 0.
__device__ __forceinline__ int pipe_sync_or(int pipe, int v)
{
    int r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.s32 p, %1, 0;\n\t"
        "bar.red.or.pred q, %2, %3, p;\n\t"
        "selp.s32 %0, 1, 0, q;\n\t}"
        : "=r"(r)
        : "r"(v), "r"(1 + pipe), "n"(PIPE_THREADS)
        : "memory");
    return r;
}

// MODE 0: layer 0 (features from state + velocity), hidden output (ReLU, BF16)
// MODE 1: hidden layer, BF16 in, hidden output
// MODE 2: output layer, BF16 in, state += s(x) (o0, o1) at the write cells
// (scal = the local scale s(x) per cell).  cols: (x tile | y tile << 10,
// z0 | planes << 16) per column.
//
// The CTA runs two independent pipelines (threads 0-127 and 128-255), each
// with its own halo slots, mbarriers and TMEM accumulators, over alternate
// columns; the weights in shared memory serve both.  Halo plane p of a
// column (p = 0 .. len + 1, z = z0 - 1 + p) feeds outputs q = p - 2
// (dz = +1), p - 1 (dz = 0) and p (dz = -1), q in [0, len); output q is
// complete after plane q + 2.  Iteration p: barrier (plane p in slot p & 1),
// MMAs of plane p, loads of plane p + 1, wait for the MMAs of plane p - 1,
// write output p - 3, store plane p + 1 into the slot plane p - 1 left.
template <int CIN, int NPAD, int MODE>
__global__ void __launch_bounds__(THREADS, 2) k_conv_tc(const uint16_t* __restrict__ act_in,
                                                        const float2* __restrict__ Win, const float* __restrict__ vel,
                                                        const uint8_t* __restrict__ wts, const float* __restrict__ bias,
                                                        uint16_t* __restrict__ act_out, float2* __restrict__ state,
                                                        const float* __restrict__ scal, NetGeom g,
                                                        const int2* __restrict__ cols, int ncols, int* err)
{
    using C = LayerCfg<CIN, NPAD>;
    extern __shared__ __align__(1024) uint8_t sm[];
    const int t = threadIdx.x, warp = t >> 5, pipe = t / PIPE_THREADS, tl = t % PIPE_THREADS;
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm + C::off_bar) + 2 * pipe;   // this pipeline's two
    uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + C::off_bar + 16 * PIPES);
    float* sb = reinterpret_cast<float*>(sm + C::off_bias);
    uint8_t* halo = sm + pipe * SLOTS * C::plane_bytes;
    const uint32_t hbase = tc5::smem_u32(halo);
    const uint32_t wbase = tc5::smem_u32(sm + C::off_w);

    if (warp == 0) tc5::tmem_alloc(tslot, C::tmem_cols);
    if (tl == 0) {
        tc5::mbar_init(bar, 1);
        tc5::mbar_init(bar + 1, 1);
    }
    {
        const int4* s4 = reinterpret_cast<const int4*>(wts);
        int4* d4 = reinterpret_cast<int4*>(sm + C::off_w);
        for (int i = t; i < C::w_bytes / 16; i += THREADS) d4[i] = s4[i];
        for (int i = t; i < NPAD; i += THREADS) sb[i] = bias[i];
        if (C::pair)   // the 11th cell of every halo row: read by the (+1, +2) pair, never loaded
            for (int i = t; i < PIPES * SLOTS * HY; i += THREADS)
                *reinterpret_cast<uint4*>(sm + (size_t)i * C::hxp * 16 + HX * 16) = make_uint4(0, 0, 0, 0);
    }
    tc5::fence_before_sync();
    __syncthreads();
    tc5::fence_after_sync();
    const uint32_t tmem = *tslot + (uint32_t)(pipe * TMEM_PER_PIPE);
    const uint32_t trow = tmem + ((uint32_t)((warp & 3) * 32) << 16);
    int failed = 0;
    uint32_t ph = 0u;   // bit b: the parity to wait for on bar[b]
    Staged<MODE, C::per> st;

    // outputs of plane z from accumulator `slot` (after its MMAs completed)
    auto epilogue = [&](int x0, int y0, int z, int slot) {
        const int x = x0 + (tl & 7), y = y0 + (tl >> 3);
        const bool valid = x < g.nx && y < g.ny && in_shell(g, x, y, z);
        const size_t c = ((size_t)z * g.ny + y) * g.nx + x;
        const uint32_t ta = trow + (uint32_t)(slot * NPAD);
        if (MODE == 2) {
            float o[16];
            tc5::tmem_ld16(ta, o);
            if (valid && is_write(g, x, y, z)) {
                const float sc = scal[c];
                float2 w = state[c];
                w.x = fmaf(sc, o[0] + sb[0], w.x);
                w.y = fmaf(sc, o[1] + sb[1], w.y);
                state[c] = w;
            }
        } else {
            float o[32];
            tc5::tmem_ld32(ta, o);
            if (valid) {
                uint4* dst = reinterpret_cast<uint4*>(act_out + c * 32);
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const float* r = o + 8 * q;
                    const float* b = sb + 8 * q;
                    dst[q] = make_uint4(pack2(fmaxf(r[0] + b[0], 0.f), fmaxf(r[1] + b[1], 0.f)),
                                        pack2(fmaxf(r[2] + b[2], 0.f), fmaxf(r[3] + b[3], 0.f)),
                                        pack2(fmaxf(r[4] + b[4], 0.f), fmaxf(r[5] + b[5], 0.f)),
                                        pack2(fmaxf(r[6] + b[6], 0.f), fmaxf(r[7] + b[7], 0.f)));
                }
            }
        }
    };

    // MMAs of one (dx, dy, k step) of halo plane p into the accumulators of
    // outputs qa..qb (contiguous ring runs; B rows of output q start at block
    // q - (p - 2))
    auto issue = [&](int p, int qa, int qb, uint64_t da, uint32_t b0, uint32_t acc) {
        while (qa <= qb) {
            const int s = qa & (C::ring - 1);
            const int cnt = min(qb - qa + 1, C::ring - s);
            const int blk = qa - (p - 2);
            const uint64_t db = tc5::smem_desc(b0 + blk * (NPAD / 8) * C::wsbo, 128, C::wsbo);
            tc5::mma_f16(tmem + (uint32_t)(s * NPAD), da, db, tc5::idesc(tc5::kTypeBF16, 128, cnt * NPAD), acc);
            qa += cnt;
        }
    };

    for (int col = blockIdx.x * PIPES + pipe; col < ncols && !failed; col += gridDim.x * PIPES) {
        const int2 cd = cols[col];
        const int x0 = (cd.x & 1023) * TXW, y0 = ((cd.x >> 10) & 1023) * TYW;
        const int z0 = cd.y & 0xFFFF, len = cd.y >> 16;
        {
            const int z = wrapi(z0 - 1, g.nz);
            load_plane<CIN, NPAD, MODE>(st, act_in, Win, vel, scal, g, x0, y0, z, tl);
            store_plane<CIN, NPAD, MODE>(st, halo, g, x0, y0, z, tl);
        }
        int bad = 0;
#pragma unroll 1
        for (int p = 0; p <= len + 1; ++p) {
            tc5::fence_async_smem();
            tc5::fence_before_sync();
            failed = pipe_sync_or(pipe, bad);
            if (failed) break;
            if (tl == 0) {
                tc5::fence_after_sync();
                const int qa = max(p - 2, 0), qb = min(p, len - 1);
                const bool fresh = p <= len - 1;   // output p starts here
                const uint32_t slot = hbase + (p & 1) * C::plane_bytes;
                for (int tap = 0; tap < C::ntaps; ++tap) {
                    // halo x of the A rows' first tap: dx + 1, or 0 / 2 for the pairs
                    const int dy = C::pair ? tap / 2 - 1 : tap / 3 - 1;
                    const int hx0 = C::pair ? 2 * (tap & 1) : tap % 3;
                    const uint32_t a0 = slot + (1 + dy) * C::sbo + hx0 * 16;
                    const uint32_t b0 = wbase + tap * C::tap_bytes;
#pragma unroll
                    for (int k = 0; k < C::ksteps; ++k) {
                        const uint64_t da = tc5::smem_desc(a0 + 2 * k * C::lbo, C::lbo, C::sbo);
                        if (fresh && tap == 0 && k == 0) {
                            issue(p, qa, p - 1, da, b0 + 2 * k * 128, 1u);
                            issue(p, p, p, da, b0 + 2 * k * 128, 0u);
                        } else {
                            issue(p, qa, qb, da, b0 + 2 * k * 128, 1u);
                        }
                    }
                }
                tc5::mma_commit(bar + (p & 1));
            }
            const int zn = wrapi(z0 + p, g.nz);   // halo plane p + 1
            if (p <= len) load_plane<CIN, NPAD, MODE>(st, act_in, Win, vel, scal, g, x0, y0, zn, tl);
            if (p >= 1) {
                const int b = (p - 1) & 1;
                bad = !tc5::mbar_wait(bar + b, (ph >> b) & 1u, kWaitLimitNs);
                if (!bad) ph ^= 1u << b;
                tc5::fence_after_sync();
                if (!bad && p >= 3) epilogue(x0, y0, z0 + p - 3, (p - 3) & (C::ring - 1));
            }
            if (p <= len) store_plane<CIN, NPAD, MODE>(st, halo + ((p + 1) & 1) * C::plane_bytes, g, x0, y0, zn, tl);
        }
        if (failed) break;
        // the column's last plane, after the MMAs of halo plane len + 1
        {
            const int b = (len + 1) & 1;
            bad = !tc5::mbar_wait(bar + b, (ph >> b) & 1u, kWaitLimitNs);
            if (!bad) ph ^= 1u << b;
            tc5::fence_after_sync();
            if (!bad) epilogue(x0, y0, z0 + len - 1, (len - 1) & (C::ring - 1));
        }
        tc5::fence_before_sync();
        failed = pipe_sync_or(pipe, bad);
    }
    if (failed && tl == 0) {
        atomicExch(err, 2);
        tc5::mbar_wait(bar, ph & 1u, kWaitLimitNs);
        tc5::mbar_wait(bar + 1, (ph >> 1) & 1u, kWaitLimitNs);
    }
    tc5::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tc5::fence_after_sync();
        tc5::tmem_dealloc(*tslot, C::tmem_cols);
    }
}

uint16_t bf16_bits(float f)
{
    uint32_t u;
    memcpy(&u, &f, 4);
    u += 0x7FFFu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}

}  // namespace

// Host: BF16 B operands of one layer in the kernel's shared-memory layout
// [tap][n group][channel chunk][8 rows][8 channels], row n = blk * npad +
// output channel with blk 0, 1, 2 the taps dz = +1, 0, -1; zero beyond
// (cin, cout).  Taps: (dx, dy) = tap % 3 - 1, tap / 3 - 1, or for layer 0
// (cin_pad 16, pairs) dy = tap / 2 - 1 with K 0..7 the x tap dx_a = -1 or
// +1 (tap & 1) and K 8..15 the tap dx_a + 1 (zero for +2).
// w: [tap = (dz + 1) 9 + (dy + 1) 3 + dx + 1][cin][cout].
void tc_layer_weights(const float* w, int cin, int cout, int cin_pad, int npad, std::vector<uint8_t>& out)
{
    const bool pair = cin_pad == 16;
    const int kchunks = cin_pad / 8, ngroups = 3 * npad / 8, ntaps = pair ? 6 : 9;
    out.assign((size_t)ntaps * ngroups * kchunks * 128, 0);
    for (int tap = 0; tap < ntaps; ++tap)
        for (int n = 0; n < 3 * npad; ++n)
            for (int k = 0; k < cin_pad; ++k) {
                const int blk = n / npad, co = n % npad, dz = 1 - blk;
                int dx, dy, ci;
                if (pair) {
                    dy = tap / 2 - 1;
                    dx = 2 * (tap & 1) - 1 + k / 8;
                    ci = k % 8;
                } else {
                    dx = tap % 3 - 1;
                    dy = tap / 3 - 1;
                    ci = k;
                }
                const bool live = co < cout && ci < cin && dx <= 1;
                const int src = (dz + 1) * 9 + (dy + 1) * 3 + (dx + 1);
                const float v = live ? w[((size_t)src * cin + ci) * cout + co] : 0.f;
                const uint16_t b = bf16_bits(v);
                const size_t o = (((size_t)tap * ngroups + n / 8) * kchunks + k / 8) * 128 + (n % 8) * 16 + (k % 8) * 2;
                memcpy(out.data() + o, &b, 2);
            }
}

// Columns of output planes: for each 8 x 16 (x, y) tile, the runs of
// consecutive z planes holding shell cells, cut into pieces of at most ZL;
// two ints per column (x tile | y tile << 10, z0 | planes << 16).
void tc_tiles(const NetGeom& g, std::vector<int>& cols)
{
    cols.clear();
    const int tx = (g.nx + TXW - 1) / TXW, ty = (g.ny + TYW - 1) / TYW;
    for (int j = 0; j < ty; ++j)
        for (int i = 0; i < tx; ++i) {
            int run0 = -1;
            for (int z = 0; z <= g.nz; ++z) {
                bool any = false;
                for (int y = j * TYW; z < g.nz && y < std::min(g.ny, j * TYW + TYW) && !any; ++y)
                    for (int x = i * TXW; x < std::min(g.nx, i * TXW + TXW) && !any; ++x) {
                        const int d = std::min(std::min(std::min(x, g.nx - 1 - x), std::min(y, g.ny - 1 - y)),
                                               std::min(z, g.nz - 1 - z));
                        any = d < g.shell;
                    }
                if (any && run0 < 0) run0 = z;
                if ((!any || z - run0 == ZL) && run0 >= 0) {
                    cols.push_back(i | (j << 10));
                    cols.push_back(run0 | ((z - run0) << 16));
                    run0 = any ? z : -1;
                }
            }
        }
}

cudaError_t configure_tc()
{
    cudaError_t e;
    if ((e = cudaFuncSetAttribute(k_conv_tc<16, 32, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  LayerCfg<16, 32>::smem)) != cudaSuccess)
        return e;
    if ((e = cudaFuncSetAttribute(k_conv_tc<32, 32, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  LayerCfg<32, 32>::smem)) != cudaSuccess)
        return e;
    return cudaFuncSetAttribute(k_conv_tc<32, 16, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                LayerCfg<32, 16>::smem);
}

cudaError_t forward_tc(cudaStream_t s, const Net& n, const TcNet& tc, float2* W, const float* vel, bool scale)
{
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 148;
    }
    const unsigned grid = (unsigned)std::max(1, std::min((tc.ntiles + PIPES - 1) / PIPES, 2 * sms));
    const int2* cols = reinterpret_cast<const int2*>(tc.tiles);
    cudaError_t e = scale ? shell_scale(s, n, W) : cudaSuccess;
    if (e != cudaSuccess) return e;
    k_conv_tc<16, 32, 0><<<grid, THREADS, LayerCfg<16, 32>::smem, s>>>(
        nullptr, W, vel, tc.w[0], tc.b[0], tc.act[0], nullptr, n.sloc, n.g, cols, tc.ntiles, tc.err);
    k_conv_tc<32, 32, 1><<<grid, THREADS, LayerCfg<32, 32>::smem, s>>>(
        tc.act[0], nullptr, nullptr, tc.w[1], tc.b[1], tc.act[1], nullptr, n.scal, n.g, cols, tc.ntiles, tc.err);
    k_conv_tc<32, 32, 1><<<grid, THREADS, LayerCfg<32, 32>::smem, s>>>(
        tc.act[1], nullptr, nullptr, tc.w[2], tc.b[2], tc.act[0], nullptr, n.scal, n.g, cols, tc.ntiles, tc.err);
    k_conv_tc<32, 16, 2><<<grid, THREADS, LayerCfg<32, 16>::smem, s>>>(
        tc.act[0], nullptr, nullptr, tc.w[3], tc.b[3], nullptr, W, n.sloc, n.g, cols, tc.ntiles, tc.err);
    return cudaGetLastError();
}

}  // namespace learn
}  // namespace ose
