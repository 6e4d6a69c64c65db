// ose_learn.cu - the learned-boundary form: a small 3D convolutional network
// that corrects the wavefield next to a thin sponge once per time step, with
// its own training kernels (forward, gradients, Adam).  No counterpart in the
// reference, whose sponge is the only boundary treatment (apply_ABC_Xt,
// ose_3d_kernel.cu:263-288).
//
// Network (fixed architecture, 64,034 parameters):
//   input  8 channels per cell: P/s, Q/s, v/4500, ex, ey, ez, 0, 0
//          s = s(x), the local RMS of (P, Q): sqrt(m/2 + f^2), m the mean of
//          P^2 + Q^2 over the 17^3 box around the cell (shell cells only), f
//          = 1e-3 x the RMS over the whole shell (a floor for empty regions);
//          e. = signed closeness to the nearest face of that axis inside the
//          shell, -1 .. 1, 0 beyond it
//   conv 3x3x3  8 -> 32, ReLU
//   conv 3x3x3 32 -> 32, ReLU
//   conv 3x3x3 32 -> 32, ReLU
//   conv 3x3x3 32 ->  2      output (dP, dQ) / s(x)
// The network lives on the SHELL: cells within `shell` cells of a face of the
// padded grid (periodic, like the FFT grid, so opposite faces are neighbours).
// Every layer reads zeros outside the shell.  The correction s(x) (dP, dQ)
// is added to the state at the WRITE cells: shell cells outside the sponge.
//
// Layout: activations are dense channels-last float arrays [cell][C] over the
// padded grid, cell = (z * nyb + y) * nxb + x; only shell cells are computed
// or read.  Work is a list of 8^3 tiles that meet the shell.  Parameters are
// one FP32 vector: per layer W[27][Cin][Cout] (tap = (dz+1)*9 + (dy+1)*3 +
// (dx+1)) then b[Cout].
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "ose_internal.h"
#include "ose_learn.h"

namespace ose {
namespace learn {

namespace {

constexpr int T = 8;            // tile edge
constexpr int kThreads = 256;   // conv: 2 cells of a 512-cell tile per thread

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

__device__ __forceinline__ void tile_origin(int tp, int& x0, int& y0, int& z0)
{
    x0 = (tp & 1023) * T;
    y0 = ((tp >> 10) & 1023) * T;
    z0 = (tp >> 20) * T;
}

// Local scale s(x): three periodic box sums of P^2 + Q^2 (shell cells) with
// half-width kBoxR, x then y then z over the whole padded grid.  Each pass
// stages whole lines in shared memory (coalesced global reads and writes)
// and every output is a 17-term sum from shared memory.
constexpr int kBoxR = 8;
constexpr int kBoxTX = 32;   // x columns per block of the y and z passes

// Which box sums are needed: s(x) only at shell cells, so the z pass writes
// shell cells and reads the y pass where `need_y` holds, which reads the x
// pass where `need_x` holds (each set holds the +-kBoxR neighbours the next
// pass reads along its axis, periodic).
__device__ __forceinline__ int edge_dist(int v, int n) { return min(v, n - 1 - v); }
__device__ __forceinline__ bool need_y(const NetGeom& g, int x, int y, int z)
{
    return edge_dist(x, g.nx) < g.shell || edge_dist(y, g.ny) < g.shell || edge_dist(z, g.nz) < g.shell + kBoxR;
}
__device__ __forceinline__ bool need_x(const NetGeom& g, int x, int y, int z)
{
    return edge_dist(x, g.nx) < g.shell || edge_dist(y, g.ny) < g.shell + kBoxR ||
           edge_dist(z, g.nz) < g.shell + kBoxR;
}

// rows of the x pass per block (shared memory <= 48 KiB)
static int box_rows(const NetGeom& g) { return std::max(1, std::min(8, 12288 / (g.nx + 2 * kBoxR))); }
static int box_blocks(const NetGeom& g)
{
    const int r = box_rows(g);
    return (g.ny * g.nz + r - 1) / r;
}

// x pass over `rows` (y, z) rows per block, e[x] with its periodic halo in
// shared memory; also the block's sum of e over its rows -> part[block].
__global__ void __launch_bounds__(256) k_box_x(const float2* __restrict__ W, float* __restrict__ out,
                                               float* __restrict__ part, NetGeom g, int rows)
{
    extern __shared__ float box_e[];   // [rows][nx + 2 kBoxR]
    __shared__ float red[8];
    const int L = g.nx + 2 * kBoxR;
    const int row0 = blockIdx.x * rows, nr = min(rows, g.ny * g.nz - row0);
    float sum = 0.f;
#pragma unroll 4
    for (int i = threadIdx.x; i < nr * L; i += blockDim.x) {
        const int r = i / L, j = i - r * L;
        const int row = row0 + r, y = row % g.ny, z = row / g.ny;
        const int x = wrapi(j - kBoxR, g.nx);
        const bool sh = in_shell(g, x, y, z);
        const float2 v = sh ? W[(size_t)row * g.nx + x] : make_float2(0.f, 0.f);
        const float e = sh ? fmaf(v.x, v.x, v.y * v.y) : 0.f;
        box_e[i] = e;
        if (j >= kBoxR && j < g.nx + kBoxR) sum += e;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nr * g.nx; i += blockDim.x) {
        const int r = i / g.nx, x = i - r * g.nx;
        const int row = row0 + r;
        if (!need_x(g, x, row % g.ny, row / g.ny)) continue;
        const float* e = box_e + r * L + x;
        float acc = 0.f;
#pragma unroll
        for (int d = 0; d <= 2 * kBoxR; ++d) acc += e[d];
        out[(size_t)(row0 + r) * g.nx + x] = acc;
    }
    for (int o = 16; o; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = sum;
    __syncthreads();
    if (threadIdx.x == 0) {
        float b = 0.f;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) b += red[w];
        part[blockIdx.x] = b;
    }
}

// scal[0] = sum of P^2 + Q^2 over the shell (the x pass's block sums, added
// in a fixed order), scal[1] = s = sqrt(scal[0] / (2 n)), scal[2] = 1/s (0 for
// a zero field).
__global__ void __launch_bounds__(1024) k_shell_scale(float* scal, const float* __restrict__ part, int nparts,
                                                      float inv_count2)
{
    __shared__ double red[32];
    double a = 0.0;
    for (int i = threadIdx.x; i < nparts; i += blockDim.x) a += part[i];
    for (int o = 16; o; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = a;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
        const float sum = (float)t;
        const float s = sqrtf(sum * inv_count2);
        scal[0] = sum;
        scal[1] = s;
        scal[2] = s > 0.f ? 1.f / s : 0.f;
    }
}

__device__ __forceinline__ int modi(int v, int n) { return ((v % n) + n) % n; }

// block per (x tile, plane index, chunk of kBoxL outputs): lines of length n
// at stride `stride` (y pass: n = ny, stride nx, plane = z; z pass: n = nz,
// stride nx ny, plane = y); the chunk and its periodic halo sit in shared
// memory.  Only the sums the next step needs are read and written (need_x ->
// need_y -> shell cells).  FINAL (the z pass): s = sqrt(m / 2 + f^2), m the
// box mean, f = 1e-3 x the shell RMS.
constexpr int kBoxL = 256;

template <bool FINAL>
__global__ void __launch_bounds__(256) k_box_lines(const float* __restrict__ in, float* __restrict__ out,
                                                   const float* __restrict__ scal, int n, long long stride,
                                                   long long pstride, NetGeom g)
{
    __shared__ float box_e[(kBoxL + 2 * kBoxR) * kBoxTX];
    const int c = threadIdx.x, x = blockIdx.x * kBoxTX + c;
    const int i0 = blockIdx.z * kBoxL, len = min(kBoxL, n - i0);
    const int pl = blockIdx.y;
    const size_t base = (size_t)pl * pstride + x;
    const bool ok = x < g.nx;
    for (int j = threadIdx.y; j < len + 2 * kBoxR; j += blockDim.y) {
        const int i = modi(i0 + j - kBoxR, n);
        const bool need = ok && (FINAL ? need_y(g, x, pl, i) : need_x(g, x, i, pl));
        box_e[j * kBoxTX + c] = need ? in[base + (size_t)i * stride] : 0.f;
    }
    __syncthreads();
    if (!ok) return;
    const float f = FINAL ? 1e-3f * scal[1] : 0.f;
    const float inv_vol = 1.f / (float)((2 * kBoxR + 1) * (2 * kBoxR + 1) * (2 * kBoxR + 1));
    for (int j = threadIdx.y; j < len; j += blockDim.y) {
        const int i = i0 + j;
        if (!(FINAL ? in_shell(g, x, pl, i) : need_y(g, x, i, pl))) continue;
        float acc = 0.f;
        for (int d = 0; d <= 2 * kBoxR; ++d) acc += box_e[(j + d) * kBoxTX + c];
        out[base + (size_t)i * stride] = FINAL ? sqrtf(0.5f * fmaxf(acc, 0.f) * inv_vol + f * f) : acc;
    }
}

__global__ void k_features(const float2* __restrict__ W, const float* __restrict__ vel, const float* __restrict__ sloc,
                           float* __restrict__ F, NetGeom g, const int* __restrict__ tiles, int ntiles)
{
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        int x0, y0, z0;
        tile_origin(tiles[tile], x0, y0, z0);
        for (int t = threadIdx.x; t < T * T * T; t += blockDim.x) {
            const int x = x0 + (t & 7), y = y0 + ((t >> 3) & 7), z = z0 + (t >> 6);
            if (x >= g.nx || y >= g.ny || z >= g.nz || !in_shell(g, x, y, z)) continue;
            const size_t c = ((size_t)z * g.ny + y) * g.nx + x;
            const float2 w = W[c];
            const float inv = 1.f / sloc[c];
            float4* f = reinterpret_cast<float4*>(F + c * 8);
            f[0] = make_float4(w.x * inv, w.y * inv, vel[c] * (1.f / 4500.f), face_coord(x, g.nx, g.shell));
            f[1] = make_float4(face_coord(y, g.ny, g.shell), face_coord(z, g.nz, g.shell), 0.f, 0.f);
        }
    }
}

// out[c][co] = sum_{tap, ci} w[tap][ci][co] * in[c + off(tap)][ci] (+ b[co]) for
// the shell cells c, inputs outside the shell read as zero.
//   MODE_RELU   out = max(0, acc)
//   MODE_LINEAR out = acc
//   MODE_MASK   out = acc * (mask[c][co] > 0)   (data gradient through a ReLU)
//   MODE_APPLY  state[c] += s(c) * (acc0, acc1) at the write cells (COUT = 2)
enum { MODE_RELU = 0, MODE_LINEAR = 1, MODE_MASK = 2, MODE_APPLY = 3 };

template <int CIN, int COUT, int MODE>
__global__ void __launch_bounds__(kThreads) k_conv(const float* __restrict__ in, const float* __restrict__ w,
                                                  const float* __restrict__ bias, float* __restrict__ out,
                                                  const float* __restrict__ mask, float2* __restrict__ state,
                                                  const float* __restrict__ scal, NetGeom g,
                                                  const int* __restrict__ tiles, int ntiles)
{
    extern __shared__ float4 smem4[];
    float* sw = reinterpret_cast<float*>(smem4);
    for (int i = threadIdx.x; i < 27 * CIN * COUT; i += kThreads) sw[i] = w[i];
    __syncthreads();
    const int t = threadIdx.x;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        int x0, y0, z0;
        tile_origin(tiles[tile], x0, y0, z0);
        const int x = x0 + (t & 7), y = y0 + ((t >> 3) & 7);
        const int za = z0 + (t >> 6), zb = za + 4;
        const bool inxy = x < g.nx && y < g.ny;
        const bool va = inxy && za < g.nz && in_shell(g, x, y, za);
        const bool vb = inxy && zb < g.nz && in_shell(g, x, y, zb);
        if (!va && !vb) continue;
        float a[COUT], b[COUT];
#pragma unroll
        for (int co = 0; co < COUT; ++co) {
            const float b0 = (MODE == MODE_MASK) ? 0.f : bias[co];
            a[co] = b0;
            b[co] = b0;
        }
        for (int tap = 0; tap < 27; ++tap) {
            const int dx = tap % 3 - 1, dy = (tap / 3) % 3 - 1, dz = tap / 9 - 1;
            const int xn = wrapi(x + dx, g.nx), yn = wrapi(y + dy, g.ny);
            const int zna = wrapi(za + dz, g.nz), znb = wrapi(zb + dz, g.nz);
            const bool oka = va && in_shell(g, xn, yn, zna);
            const bool okb = vb && in_shell(g, xn, yn, znb);
            const float* ia = in + (((size_t)zna * g.ny + yn) * g.nx + xn) * CIN;
            const float* ib = in + (((size_t)znb * g.ny + yn) * g.nx + xn) * CIN;
            const float* wt = sw + tap * CIN * COUT;
            if (CIN % 4 == 0) {
#pragma unroll 2
                for (int ci = 0; ci < CIN; ci += 4) {
                    const float4 p = oka ? __ldg(reinterpret_cast<const float4*>(ia + ci)) : make_float4(0, 0, 0, 0);
                    const float4 q = okb ? __ldg(reinterpret_cast<const float4*>(ib + ci)) : make_float4(0, 0, 0, 0);
                    const float pv[4] = {p.x, p.y, p.z, p.w}, qv[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        const float* wr = wt + (ci + j) * COUT;
#pragma unroll
                        for (int co = 0; co < COUT; ++co) {
                            a[co] = fmaf(pv[j], wr[co], a[co]);
                            b[co] = fmaf(qv[j], wr[co], b[co]);
                        }
                    }
                }
            } else {
                for (int ci = 0; ci < CIN; ++ci) {
                    const float pv = oka ? __ldg(ia + ci) : 0.f, qv = okb ? __ldg(ib + ci) : 0.f;
                    const float* wr = wt + ci * COUT;
#pragma unroll
                    for (int co = 0; co < COUT; ++co) {
                        a[co] = fmaf(pv, wr[co], a[co]);
                        b[co] = fmaf(qv, wr[co], b[co]);
                    }
                }
            }
        }
        const size_t ca = ((size_t)za * g.ny + y) * g.nx + x, cb = ((size_t)zb * g.ny + y) * g.nx + x;
        if (MODE == MODE_APPLY) {
            if (va && is_write(g, x, y, za)) {
                const float s = scal[ca];
                float2 v = state[ca];
                v.x = fmaf(s, a[0], v.x);
                v.y = fmaf(s, a[1], v.y);
                state[ca] = v;
            }
            if (vb && is_write(g, x, y, zb)) {
                const float s = scal[cb];
                float2 v = state[cb];
                v.x = fmaf(s, b[0], v.x);
                v.y = fmaf(s, b[1], v.y);
                state[cb] = v;
            }
        } else {
#pragma unroll
            for (int co = 0; co < COUT; ++co) {
                float ra = a[co], rb = b[co];
                if (MODE == MODE_RELU) { ra = fmaxf(ra, 0.f); rb = fmaxf(rb, 0.f); }
                if (MODE == MODE_MASK) {
                    ra = va && mask[ca * COUT + co] > 0.f ? ra : 0.f;
                    rb = vb && mask[cb * COUT + co] > 0.f ? rb : 0.f;
                }
                if (va) out[ca * COUT + co] = ra;
                if (vb) out[cb * COUT + co] = rb;
            }
        }
    }
}

// gw[tap][ci][co] += sum_c in[c + off(tap)][ci] * gout[c][co] over shell cells
// (inputs outside the shell are zero).  Thread (tap, ci), 27 * CIN threads.
template <int CIN, int COUT>
__global__ void __launch_bounds__(27 * CIN) k_wgrad(const float* __restrict__ in, const float* __restrict__ gout,
                                                    float* __restrict__ gw, NetGeom g,
                                                    const int* __restrict__ tiles, int ntiles)
{
    extern __shared__ float4 smem4[];
    float* halo = reinterpret_cast<float*>(smem4);            // [10^3][CIN]
    float* go = halo + 1000 * CIN;                            // [512][COUT]
    const int tid = threadIdx.x, nth = 27 * CIN;
    const int tap = tid / CIN, ci = tid - tap * CIN;
    const int dx = tap % 3 - 1, dy = (tap / 3) % 3 - 1, dz = tap / 9 - 1;
    float acc[COUT];
#pragma unroll
    for (int co = 0; co < COUT; ++co) acc[co] = 0.f;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        int x0, y0, z0;
        tile_origin(tiles[tile], x0, y0, z0);
        __syncthreads();
        for (int i = tid; i < 1000 * CIN; i += nth) {
            const int h = i / CIN, c = i - h * CIN;
            const int hx = h % 10, hy = (h / 10) % 10, hz = h / 100;
            const int x = x0 + hx - 1, y = y0 + hy - 1, z = z0 + hz - 1;
            // neighbours wrap periodically (x is in [-1, nx + 7], inside one period)
            const int xw = wrapi(x, g.nx), yw = wrapi(y, g.ny), zw = wrapi(z, g.nz);
            halo[i] = in_shell(g, xw, yw, zw) ? in[(((size_t)zw * g.ny + yw) * g.nx + xw) * CIN + c] : 0.f;
        }
        for (int i = tid; i < 512 * COUT; i += nth) {
            const int l = i / COUT, c = i - l * COUT;
            const int x = x0 + (l & 7), y = y0 + ((l >> 3) & 7), z = z0 + (l >> 6);
            float v = 0.f;
            if (x < g.nx && y < g.ny && z < g.nz && in_shell(g, x, y, z))
                v = gout[(((size_t)z * g.ny + y) * g.nx + x) * COUT + c];
            go[i] = v;
        }
        __syncthreads();
        for (int l = 0; l < 512; ++l) {
            const int lx = l & 7, ly = (l >> 3) & 7, lz = l >> 6;
            const float v = halo[(((lz + 1 + dz) * 10 + (ly + 1 + dy)) * 10 + (lx + 1 + dx)) * CIN + ci];
            const float* gr = go + l * COUT;
#pragma unroll
            for (int co = 0; co < COUT; ++co) acc[co] = fmaf(v, gr[co], acc[co]);
        }
    }
#pragma unroll
    for (int co = 0; co < COUT; ++co) atomicAdd(gw + (tap * CIN + ci) * COUT + co, acc[co]);
}

// gb[co] += sum over shell cells of gout[c][co].
template <int COUT>
__global__ void k_bgrad(const float* __restrict__ gout, float* __restrict__ gb, NetGeom g,
                        const int* __restrict__ tiles, int ntiles)
{
    __shared__ float red[COUT];
    for (int i = threadIdx.x; i < COUT; i += blockDim.x) red[i] = 0.f;
    __syncthreads();
    float acc[COUT];
#pragma unroll
    for (int co = 0; co < COUT; ++co) acc[co] = 0.f;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        int x0, y0, z0;
        tile_origin(tiles[tile], x0, y0, z0);
        for (int t = threadIdx.x; t < 512; t += blockDim.x) {
            const int x = x0 + (t & 7), y = y0 + ((t >> 3) & 7), z = z0 + (t >> 6);
            if (x >= g.nx || y >= g.ny || z >= g.nz || !in_shell(g, x, y, z)) continue;
            const float* r = gout + (((size_t)z * g.ny + y) * g.nx + x) * COUT;
#pragma unroll
            for (int co = 0; co < COUT; ++co) acc[co] += r[co];
        }
    }
#pragma unroll
    for (int co = 0; co < COUT; ++co) {
        float v = acc[co];
        for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) atomicAdd(red + co, v);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < COUT; i += blockDim.x) atomicAdd(gb + i, red[i]);
}

// Loss of one sample: r = (target - state) / s(x) at the write cells, the
// network output o (normalised units); g = 2 (o - r) / nw, loss += |o - r|^2 / nw.
__global__ void k_loss(const float* __restrict__ o, const float2* __restrict__ state, const float2* __restrict__ tgt,
                       const float* __restrict__ sloc, float* __restrict__ gout, float* loss, float inv_nw, NetGeom g,
                       const int* __restrict__ tiles, int ntiles)
{
    float l = 0.f;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        int x0, y0, z0;
        tile_origin(tiles[tile], x0, y0, z0);
        for (int t = threadIdx.x; t < 512; t += blockDim.x) {
            const int x = x0 + (t & 7), y = y0 + ((t >> 3) & 7), z = z0 + (t >> 6);
            if (x >= g.nx || y >= g.ny || z >= g.nz || !in_shell(g, x, y, z)) continue;
            const size_t c = ((size_t)z * g.ny + y) * g.nx + x;
            float gx = 0.f, gy = 0.f;
            if (is_write(g, x, y, z)) {
                const float inv = 1.f / sloc[c];
                const float2 u = state[c], v = tgt[c];
                const float ex = o[2 * c] - (v.x - u.x) * inv, ey = o[2 * c + 1] - (v.y - u.y) * inv;
                gx = 2.f * ex * inv_nw;
                gy = 2.f * ey * inv_nw;
                l += (ex * ex + ey * ey) * inv_nw;
            }
            gout[2 * c] = gx;
            gout[2 * c + 1] = gy;
        }
    }
    for (int off = 16; off; off >>= 1) l += __shfl_xor_sync(0xffffffffu, l, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, l);
}

// wt[tap'][co][ci] = w[26 - tap'][ci][co]: the data-gradient weights.
__global__ void k_flip(const float* __restrict__ w, float* __restrict__ wt, int cin, int cout)
{
    const int n = 27 * cin * cout;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int tp = i / (cin * cout), r = i - tp * cin * cout;
        const int co = r / cin, ci = r - co * cin;
        wt[i] = w[((26 - tp) * cin + ci) * cout + co];
    }
}

__global__ void k_adam(float* __restrict__ p, float* __restrict__ gr, float* __restrict__ m, float* __restrict__ v,
                       int n, float lr, float b1, float b2, float eps, float c1, float c2, float gscale)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float g = gr[i] * gscale;
        const float mi = b1 * m[i] + (1.f - b1) * g;
        const float vi = b2 * v[i] + (1.f - b2) * g * g;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
        gr[i] = 0.f;
    }
}

template <typename K>
cudaError_t smem_attr(K k, size_t bytes)
{
    return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

}  // namespace

const int kCin[kLayers] = {8, 32, 32, 32};
const int kCout[kLayers] = {32, 32, 32, 2};

size_t param_offset(int layer)
{
    size_t o = 0;
    for (int l = 0; l < layer; ++l) o += (size_t)27 * kCin[l] * kCout[l] + kCout[l];
    return o;
}

size_t param_count() { return param_offset(kLayers); }

void shell_tiles(const NetGeom& g, std::vector<int>& tiles, long long* ncells, long long* nwrite)
{
    tiles.clear();
    long long nc = 0, nw = 0;
    const int tx = (g.nx + T - 1) / T, ty = (g.ny + T - 1) / T, tz = (g.nz + T - 1) / T;
    auto shell = [&](int x, int y, int z) {
        const int d = std::min(std::min(std::min(x, g.nx - 1 - x), std::min(y, g.ny - 1 - y)),
                               std::min(z, g.nz - 1 - z));
        return d < g.shell;
    };
    for (int k = 0; k < tz; ++k)
        for (int j = 0; j < ty; ++j)
            for (int i = 0; i < tx; ++i) {
                bool any = false;
                for (int z = k * T; z < std::min(g.nz, k * T + T); ++z)
                    for (int y = j * T; y < std::min(g.ny, j * T + T); ++y)
                        for (int x = i * T; x < std::min(g.nx, i * T + T); ++x)
                            if (shell(x, y, z)) {
                                any = true;
                                ++nc;
                                if (x >= g.sp[0] && x < g.nx - g.sp[1] && y >= g.sp[2] && y < g.ny - g.sp[3] &&
                                    z >= g.sp[4] && z < g.nz - g.sp[5])
                                    ++nw;
                            }
                if (any) tiles.push_back(i | (j << 10) | (k << 20));
            }
    if (ncells) *ncells = nc;
    if (nwrite) *nwrite = nw;
}

cudaError_t configure()
{
    cudaError_t e;
    if ((e = smem_attr(k_conv<8, 32, MODE_RELU>, 27 * 8 * 32 * 4)) != cudaSuccess) return e;
    if ((e = smem_attr(k_conv<32, 32, MODE_RELU>, 27 * 32 * 32 * 4)) != cudaSuccess) return e;
    if ((e = smem_attr(k_conv<32, 2, MODE_LINEAR>, 27 * 32 * 2 * 4)) != cudaSuccess) return e;
    if ((e = smem_attr(k_conv<32, 2, MODE_APPLY>, 27 * 32 * 2 * 4)) != cudaSuccess) return e;
    if ((e = smem_attr(k_conv<2, 32, MODE_MASK>, 27 * 2 * 32 * 4)) != cudaSuccess) return e;
    if ((e = smem_attr(k_conv<32, 32, MODE_MASK>, 27 * 32 * 32 * 4)) != cudaSuccess) return e;
    if ((e = smem_attr(k_wgrad<8, 32>, (1000 * 8 + 512 * 32) * 4)) != cudaSuccess) return e;
    if ((e = smem_attr(k_wgrad<32, 32>, (1000 * 32 + 512 * 32) * 4)) != cudaSuccess) return e;
    if ((e = smem_attr(k_wgrad<32, 2>, (1000 * 32 + 512 * 2) * 4)) != cudaSuccess) return e;
    return cudaSuccess;
}

static unsigned grid_for(int ntiles, int per_sm)
{
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 148;
    }
    return (unsigned)std::max(1, std::min(ntiles, per_sm * sms));
}

cudaError_t shell_scale(cudaStream_t s, const Net& n, const float2* W)
{
    const NetGeom& g = n.g;
    const long long plane = (long long)g.nx * g.ny;
    const unsigned xt = (unsigned)((g.nx + kBoxTX - 1) / kBoxTX);
    const int rows = box_rows(g), nb = box_blocks(g);
    float* part = n.scal + 4;
    k_box_x<<<nb, 256, sizeof(float) * rows * (g.nx + 2 * kBoxR), s>>>(W, n.sloc, part, g, rows);
    k_shell_scale<<<1, 1024, 0, s>>>(n.scal, part, nb, (float)(0.5 / (double)std::max(1LL, n.ncells)));
    k_box_lines<false><<<dim3(xt, g.nz, (g.ny + kBoxL - 1) / kBoxL), dim3(kBoxTX, 8), 0, s>>>(
        n.sloc, n.stmp, n.scal, g.ny, g.nx, plane, g);
    k_box_lines<true><<<dim3(xt, g.ny, (g.nz + kBoxL - 1) / kBoxL), dim3(kBoxTX, 8), 0, s>>>(
        n.stmp, n.sloc, n.scal, g.nz, plane, g.nx, g);
    return cudaGetLastError();
}

cudaError_t forward(cudaStream_t s, const Net& n, const float2* W, const float* vel, bool apply, float2* state_out,
                    bool scale)
{
    const NetGeom& g = n.g;
    const float* p = n.params;
    const unsigned gr = grid_for(n.ntiles, 2);
    cudaError_t e0 = scale ? shell_scale(s, n, W) : cudaSuccess;
    if (e0 != cudaSuccess) return e0;
    k_features<<<gr, 256, 0, s>>>(W, vel, n.sloc, n.F, g, n.tiles, n.ntiles);
    const float* w0 = p + param_offset(0);
    const float* w1 = p + param_offset(1);
    const float* w2 = p + param_offset(2);
    const float* w3 = p + param_offset(3);
    k_conv<8, 32, MODE_RELU><<<gr, kThreads, 27 * 8 * 32 * 4, s>>>(n.F, w0, w0 + 27 * 8 * 32, n.A[0], nullptr,
                                                                   nullptr, n.scal, g, n.tiles, n.ntiles);
    k_conv<32, 32, MODE_RELU><<<gr, kThreads, 27 * 32 * 32 * 4, s>>>(n.A[0], w1, w1 + 27 * 32 * 32, n.A[1], nullptr,
                                                                     nullptr, n.scal, g, n.tiles, n.ntiles);
    k_conv<32, 32, MODE_RELU><<<gr, kThreads, 27 * 32 * 32 * 4, s>>>(n.A[1], w2, w2 + 27 * 32 * 32, n.A[2], nullptr,
                                                                     nullptr, n.scal, g, n.tiles, n.ntiles);
    if (apply)
        k_conv<32, 2, MODE_APPLY><<<gr, kThreads, 27 * 32 * 2 * 4, s>>>(n.A[2], w3, w3 + 27 * 32 * 2, nullptr,
                                                                        nullptr, state_out, n.sloc, g, n.tiles,
                                                                        n.ntiles);
    else
        k_conv<32, 2, MODE_LINEAR><<<gr, kThreads, 27 * 32 * 2 * 4, s>>>(n.A[2], w3, w3 + 27 * 32 * 2, n.O, nullptr,
                                                                         nullptr, n.scal, g, n.tiles, n.ntiles);
    return cudaGetLastError();
}

cudaError_t train_sample(cudaStream_t s, const Net& n, const float2* W, const float* vel, const float2* tgt)
{
    cudaError_t e = forward(s, n, W, vel, false, nullptr);
    if (e != cudaSuccess) return e;
    const NetGeom& g = n.g;
    const unsigned gr = grid_for(n.ntiles, 2);
    const unsigned gw = grid_for(n.ntiles, 1);
    k_loss<<<gr, 256, 0, s>>>(n.O, W, tgt, n.sloc, n.G4, n.loss, (float)(1.0 / (double)std::max(1LL, n.nwrite)), g,
                              n.tiles, n.ntiles);
    float* gp = n.grads;
    // data-gradient weights of layers 1..3 (layer 0's input needs none)
    for (int l = 1; l < kLayers; ++l)
        k_flip<<<64, 256, 0, s>>>(n.params + param_offset(l), n.wt[l], kCin[l], kCout[l]);
    // layer 3 (32 -> 2)
    k_wgrad<32, 2><<<gw, 27 * 32, (1000 * 32 + 512 * 2) * 4, s>>>(n.A[2], n.G4, gp + param_offset(3), g, n.tiles,
                                                                   n.ntiles);
    k_bgrad<2><<<gw, 256, 0, s>>>(n.G4, gp + param_offset(3) + 27 * 32 * 2, g, n.tiles, n.ntiles);
    k_conv<2, 32, MODE_MASK><<<gr, kThreads, 27 * 2 * 32 * 4, s>>>(n.G4, n.wt[3], nullptr, n.GA[2], n.A[2], nullptr,
                                                                   n.scal, g, n.tiles, n.ntiles);
    // layer 2 (32 -> 32)
    k_wgrad<32, 32><<<gw, 27 * 32, (1000 * 32 + 512 * 32) * 4, s>>>(n.A[1], n.GA[2], gp + param_offset(2), g,
                                                                     n.tiles, n.ntiles);
    k_bgrad<32><<<gw, 256, 0, s>>>(n.GA[2], gp + param_offset(2) + 27 * 32 * 32, g, n.tiles, n.ntiles);
    k_conv<32, 32, MODE_MASK><<<gr, kThreads, 27 * 32 * 32 * 4, s>>>(n.GA[2], n.wt[2], nullptr, n.GA[1], n.A[1],
                                                                     nullptr, n.scal, g, n.tiles, n.ntiles);
    // layer 1 (32 -> 32)
    k_wgrad<32, 32><<<gw, 27 * 32, (1000 * 32 + 512 * 32) * 4, s>>>(n.A[0], n.GA[1], gp + param_offset(1), g,
                                                                     n.tiles, n.ntiles);
    k_bgrad<32><<<gw, 256, 0, s>>>(n.GA[1], gp + param_offset(1) + 27 * 32 * 32, g, n.tiles, n.ntiles);
    k_conv<32, 32, MODE_MASK><<<gr, kThreads, 27 * 32 * 32 * 4, s>>>(n.GA[1], n.wt[1], nullptr, n.GA[0], n.A[0],
                                                                     nullptr, n.scal, g, n.tiles, n.ntiles);
    // layer 0 (8 -> 32)
    k_wgrad<8, 32><<<gw, 27 * 8, (1000 * 8 + 512 * 32) * 4, s>>>(n.F, n.GA[0], gp + param_offset(0), g, n.tiles,
                                                                 n.ntiles);
    k_bgrad<32><<<gw, 256, 0, s>>>(n.GA[0], gp + param_offset(0) + 27 * 8 * 32, g, n.tiles, n.ntiles);
    return cudaGetLastError();
}

cudaError_t adam(cudaStream_t s, const Net& n, float lr, float b1, float b2, float eps, int step, float gscale)
{
    const float c1 = 1.f / (1.f - powf(b1, (float)step));
    const float c2 = 1.f / (1.f - powf(b2, (float)step));
    k_adam<<<64, 256, 0, s>>>(n.params, n.grads, n.m, n.v, (int)param_count(), lr, b1, b2, eps, c1, c2, gscale);
    return cudaGetLastError();
}

}  // namespace learn
}  // namespace ose

// ---------------------------------------------------------------- C ABI ----

struct ose_corrector {
    ose::learn::Net net{};
    ose::learn::TcNet tc{};
    bool has_tc = false;
    std::vector<void*> bufs;
    std::string err;
    int step = 0;
};

namespace {

std::string g_corr_error;

ose_status corr_fail(ose_corrector* c, ose_status s, const std::string& m)
{
    if (c) c->err = m;
    else g_corr_error = m;
    return s;
}

template <typename T>
cudaError_t corr_alloc(ose_corrector* c, T** p, size_t count, bool zero = true)
{
    cudaError_t e = cudaMalloc((void**)p, sizeof(T) * std::max<size_t>(count, 1));
    if (e != cudaSuccess) return e;
    c->bufs.push_back(*p);
    return zero ? cudaMemset(*p, 0, sizeof(T) * std::max<size_t>(count, 1)) : cudaSuccess;
}

void corr_free(ose_corrector* c)
{
    for (void* b : c->bufs) cudaFree(b);
    c->bufs.clear();
}

}  // namespace

namespace ose {
namespace learn {

// Allocates a network for a grid; training = also gradients, Adam moments
// and backward buffers.
cudaError_t create_net(ose_corrector* c, const NetGeom& g, bool training, bool fp32_forward)
{
    Net& n = c->net;
    n.g = g;
    std::vector<int> tiles;
    shell_tiles(g, tiles, &n.ncells, &n.nwrite);
    n.ntiles = (int)tiles.size();
    const size_t cells = (size_t)g.nx * g.ny * g.nz;
    const size_t np = param_count();
    cudaError_t e;
#define A_(p, cnt) if ((e = corr_alloc(c, &(p), (cnt))) != cudaSuccess) return e
    A_(n.tiles, tiles.size());
    if ((e = cudaMemcpy(n.tiles, tiles.data(), sizeof(int) * tiles.size(), cudaMemcpyHostToDevice)) != cudaSuccess)
        return e;
    A_(n.params, np);
    A_(n.scal, 4 + (size_t)box_blocks(g));   // + the x pass's block sums
    A_(n.loss, 1);
    A_(n.sloc, cells);
    A_(n.stmp, cells);
    if (training || fp32_forward) {   // the tensor-core forward keeps its own BF16 activations
        A_(n.F, cells * 8);
        for (int l = 0; l < 3; ++l) A_(n.A[l], cells * 32);
    }
    if (training) {
        A_(n.grads, np);
        A_(n.m, np);
        A_(n.v, np);
        for (int l = 1; l < kLayers; ++l) A_(n.wt[l], (size_t)27 * kCin[l] * kCout[l]);
        A_(n.O, cells * 2);
        A_(n.G4, cells * 2);
        for (int l = 0; l < 3; ++l) A_(n.GA[l], cells * 32);
    }
#undef A_
    return configure();
}

cudaError_t create_tc(ose_corrector* c, const float* params_host, int* err)
{
    TcNet& t = c->tc;
    std::vector<int> tiles;
    tc_tiles(c->net.g, tiles);
    t.ntiles = (int)tiles.size() / 2;   // columns of (x, y) tile, z0, planes
    const size_t cells = (size_t)c->net.g.nx * c->net.g.ny * c->net.g.nz;
    cudaError_t e;
    if ((e = corr_alloc(c, &t.tiles, tiles.size(), false)) != cudaSuccess) return e;
    if ((e = cudaMemcpy(t.tiles, tiles.data(), sizeof(int) * tiles.size(), cudaMemcpyHostToDevice)) != cudaSuccess)
        return e;
    const int cin_pad[kLayers] = {16, 32, 32, 32};
    const int npad[kLayers] = {32, 32, 32, 16};
    for (int l = 0; l < kLayers; ++l) {
        const float* w = params_host + param_offset(l);
        std::vector<uint8_t> wb;
        tc_layer_weights(w, kCin[l], kCout[l], cin_pad[l], npad[l], wb);
        std::vector<float> bb(npad[l], 0.f);
        for (int i = 0; i < kCout[l]; ++i) bb[i] = w[(size_t)27 * kCin[l] * kCout[l] + i];
        if ((e = corr_alloc(c, &t.w[l], wb.size(), false)) != cudaSuccess) return e;
        if ((e = cudaMemcpy(t.w[l], wb.data(), wb.size(), cudaMemcpyHostToDevice)) != cudaSuccess) return e;
        if ((e = corr_alloc(c, &t.b[l], bb.size(), false)) != cudaSuccess) return e;
        if ((e = cudaMemcpy(t.b[l], bb.data(), sizeof(float) * bb.size(), cudaMemcpyHostToDevice)) != cudaSuccess)
            return e;
    }
    for (int i = 0; i < 2; ++i)
        if ((e = corr_alloc(c, &t.act[i], cells * 32, false)) != cudaSuccess) return e;
    t.err = err;
    c->has_tc = true;
    return configure_tc();
}

const TcNet* tc_of(const ose_corrector* c) { return c && c->has_tc ? &c->tc : nullptr; }

ose_corrector* new_corrector() { return new ose_corrector(); }
void delete_corrector(ose_corrector* c)
{
    if (!c) return;
    corr_free(c);
    delete c;
}
const Net& net_of(const ose_corrector* c) { return c->net; }

}  // namespace learn
}  // namespace ose

extern "C" {

size_t ose_corrector_param_count(void) { return ose::learn::param_count(); }

ose_status ose_corrector_create(int nxb, int nyb, int nzb, int shell, const int* sponge, ose_corrector** out)
{
    if (!out || !sponge) return corr_fail(nullptr, OSE_ERR_INVALID, "null argument");
    *out = nullptr;
    if (nxb < 8 || nyb < 8 || nzb < 8 || nxb > 8192 || nyb > 8192 || nzb > 8192 || shell < 1)
        return corr_fail(nullptr, OSE_ERR_INVALID, "grid sizes must be 8..8192 and shell >= 1");
    for (int i = 0; i < 6; ++i)
        if (sponge[i] < 0 || sponge[i] > shell) return corr_fail(nullptr, OSE_ERR_INVALID, "sponge widths must be 0..shell");
    ose_corrector* c = new ose_corrector();
    ose::learn::NetGeom g{nxb, nyb, nzb, shell, {sponge[0], sponge[1], sponge[2], sponge[3], sponge[4], sponge[5]}};
    cudaError_t e = ose::learn::create_net(c, g, true, true);
    if (e != cudaSuccess) {
        ose_status s = corr_fail(nullptr, e == cudaErrorMemoryAllocation ? OSE_ERR_NOMEM : OSE_ERR_CUDA,
                                 std::string("corrector allocation: ") + cudaGetErrorString(e));
        ose::learn::delete_corrector(c);
        return s;
    }
    *out = c;
    return OSE_OK;
}

ose_status ose_corrector_destroy(ose_corrector* c)
{
    ose::learn::delete_corrector(c);
    return OSE_OK;
}

const char* ose_corrector_last_error(const ose_corrector* c) { return c ? c->err.c_str() : g_corr_error.c_str(); }

ose_status ose_corrector_info(const ose_corrector* c, long long* shell_cells, long long* write_cells, int* tiles)
{
    if (!c) return OSE_ERR_INVALID;
    if (shell_cells) *shell_cells = c->net.ncells;
    if (write_cells) *write_cells = c->net.nwrite;
    if (tiles) *tiles = c->net.ntiles;
    return OSE_OK;
}

ose_status ose_corrector_set_params(ose_corrector* c, const float* params)
{
    if (!c || !params) return OSE_ERR_INVALID;
    cudaError_t e = cudaMemcpy(c->net.params, params, sizeof(float) * ose::learn::param_count(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(c->net.m, 0, sizeof(float) * ose::learn::param_count());
    if (e == cudaSuccess) e = cudaMemset(c->net.v, 0, sizeof(float) * ose::learn::param_count());
    if (e == cudaSuccess) e = cudaMemset(c->net.grads, 0, sizeof(float) * ose::learn::param_count());
    c->step = 0;
    return e == cudaSuccess ? OSE_OK : corr_fail(c, OSE_ERR_CUDA, cudaGetErrorString(e));
}

ose_status ose_corrector_get_params(ose_corrector* c, float* params)
{
    if (!c || !params) return OSE_ERR_INVALID;
    cudaError_t e = cudaMemcpy(params, c->net.params, sizeof(float) * ose::learn::param_count(), cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? OSE_OK : corr_fail(c, OSE_ERR_CUDA, cudaGetErrorString(e));
}

ose_status ose_corrector_get_grads(ose_corrector* c, float* grads)
{
    if (!c || !grads) return OSE_ERR_INVALID;
    cudaError_t e = cudaMemcpy(grads, c->net.grads, sizeof(float) * ose::learn::param_count(), cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? OSE_OK : corr_fail(c, OSE_ERR_CUDA, cudaGetErrorString(e));
}

ose_status ose_corrector_forward(ose_corrector* c, const void* state_dev, const float* vel_dev, float* out_dev,
                                 float* scale_out)
{
    if (!c || !state_dev || !vel_dev) return OSE_ERR_INVALID;
    const ose::learn::Net& n = c->net;
    cudaError_t e = ose::learn::forward(0, n, static_cast<const float2*>(state_dev), vel_dev, false, nullptr);
    const size_t cells = (size_t)n.g.nx * n.g.ny * n.g.nz;
    if (e == cudaSuccess && out_dev)
        e = cudaMemcpyAsync(out_dev, n.O, sizeof(float) * 2 * cells, cudaMemcpyDeviceToDevice, 0);
    float scal[4] = {0, 0, 0, 0};
    if (e == cudaSuccess) e = cudaMemcpy(scal, n.scal, sizeof(scal), cudaMemcpyDeviceToHost);
    if (scale_out) *scale_out = scal[1];
    return e == cudaSuccess ? OSE_OK : corr_fail(c, OSE_ERR_CUDA, cudaGetErrorString(e));
}

ose_status ose_corrector_apply(ose_corrector* c, void* state_dev, const float* vel_dev)
{
    if (!c || !state_dev || !vel_dev) return OSE_ERR_INVALID;
    cudaError_t e = ose::learn::forward(0, c->net, static_cast<const float2*>(state_dev), vel_dev, true,
                                        static_cast<float2*>(state_dev));
    if (e == cudaSuccess) e = cudaStreamSynchronize(0);
    return e == cudaSuccess ? OSE_OK : corr_fail(c, OSE_ERR_CUDA, cudaGetErrorString(e));
}

ose_status ose_corrector_train_sample(ose_corrector* c, const void* state_dev, const float* vel_dev,
                                      const void* target_dev)
{
    if (!c || !state_dev || !vel_dev || !target_dev) return OSE_ERR_INVALID;
    cudaError_t e = ose::learn::train_sample(0, c->net, static_cast<const float2*>(state_dev), vel_dev,
                                             static_cast<const float2*>(target_dev));
    return e == cudaSuccess ? OSE_OK : corr_fail(c, OSE_ERR_CUDA, cudaGetErrorString(e));
}

ose_status ose_corrector_adam(ose_corrector* c, float lr, int batch, float* mean_loss)
{
    if (!c || batch < 1) return OSE_ERR_INVALID;
    c->step += 1;
    cudaError_t e = ose::learn::adam(0, c->net, lr, 0.9f, 0.999f, 1e-8f, c->step, 1.f / (float)batch);
    float l = 0.f;
    if (e == cudaSuccess) e = cudaMemcpy(&l, c->net.loss, sizeof(float), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemset(c->net.loss, 0, sizeof(float));
    if (mean_loss) *mean_loss = l / (float)batch;
    return e == cudaSuccess ? OSE_OK : corr_fail(c, OSE_ERR_CUDA, cudaGetErrorString(e));
}

ose_status ose_corrector_loss(ose_corrector* c, float* loss, int reset)
{
    if (!c || !loss) return OSE_ERR_INVALID;
    cudaError_t e = cudaMemcpy(loss, c->net.loss, sizeof(float), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && reset) e = cudaMemset(c->net.loss, 0, sizeof(float));
    if (e == cudaSuccess && reset) e = cudaMemset(c->net.grads, 0, sizeof(float) * ose::learn::param_count());
    return e == cudaSuccess ? OSE_OK : corr_fail(c, OSE_ERR_CUDA, cudaGetErrorString(e));
}

}  // extern "C"
