// ose_capi.cu - the C ABI of libose3d.so (include/ose3d.h): handle lifetime,
// device memory, the step sequence and its CUDA-graph replay.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <complex>
#include <string>
#include <thread>
#include <vector>

#include "ose_internal.h"
#include "ose_io.h"
#include "ose_learn.h"

using ose::AxisPlan;

struct ose_handle {
    ose_params p{};
    ose_derived d{};
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string err;

    AxisPlan px{}, py{}, pz{};
    ose::Geometry g{};
    ose::Tables tables{};

    // device memory (all owned)
    float2* W = nullptr;     // state: P in .x, Q in .y  (a_0, and a_even during a step)
    float2* A = nullptr;     // a_odd
    float2* S = nullptr;     // partial sum
    float2* X = nullptr;     // FFT scratch
    float* vs = nullptr;     // velocity v per cell (padded model)
    float *ax = nullptr, *ay = nullptr, *az = nullptr;
    float *kx2 = nullptr, *ky2 = nullptr, *kz2 = nullptr;
    float *kx2l = nullptr, *ky2l = nullptr, *kz2l = nullptr;   // low parts
    float2* twxl = nullptr;                                     // low parts of W_nxb
    float2* bluetab[3] = {};                                    // Bluestein tables per axis
    float sch = 0.f, scl = 0.f;                                 // 1 / (R N) as hi + lo
    float2 *twx = nullptr, *twy = nullptr, *twz = nullptr;
    float *ricker = nullptr, *hil = nullptr;
    float* gather = nullptr; // [nt][ng]
    // receiver list (ose_set_receivers): padded-grid cell index per receiver
    // on the device, interior (x, y, z) on the host; empty = the receiver plane
    long long* rec_idx = nullptr;
    std::vector<int> rec_xyz;
    int* ctr = nullptr;      // [0] next step, [1] current step
    size_t bytes = 0;
    // fault injection for tests: the fail_alloc_at-th device allocation of
    // ose_create fails as if the device were out of memory (0 = never; from
    // OSE3D_FAIL_DEVICE_ALLOC in the environment)
    int fail_alloc_at = 0;
    int nalloc = 0;
    // precision form: mode, DFT operands of the tensor-core z pass, error word
    int precision = OSE_PRECISION_FP32;
    void* tcb = nullptr;
    int* tcerr = nullptr;
    // learned boundary corrector (inference buffers) and the velocity it reads
    ose_corrector* corr = nullptr;
    float* corr_vel = nullptr;

    // host copies
    std::vector<float> vb, h_ax, h_ay, h_az, h_ricker, h_hil;
    std::vector<float> vel_in;   // the model as given ([x][y][z] interior); vb is padded from it on demand
    std::vector<double> J;

    long long src = 0;
    int shot = -1;
    int it = 0;
    bool shot_ready = false;
    cudaGraphExec_t graph = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    ose::KernelTiming timing{};

    // receiver rows on their way to the host (ose_run_record): two pinned
    // chunks of kRecChunk rows and the events that mark them filled
    float* rec_stage = nullptr;
    int rec_stage_ng = 0;        // ng at allocation
    cudaEvent_t rec_ev[2] = {nullptr, nullptr};

    // snapshots (allocated on first use): device copy of the state, two
    // pinned host buffers, a copy stream and its events
    float2* Wsnap = nullptr;
    float2* hsnap[2] = {nullptr, nullptr};
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t snap_ready = nullptr;
    cudaEvent_t snap_done[2] = {nullptr, nullptr};
};

namespace {

std::string g_create_error;

ose_status fail(ose_handle* h, ose_status s, const std::string& msg)
{
    if (h) h->err = msg;
    else g_create_error = msg;
    return s;
}

ose_status cuda_fail(ose_handle* h, cudaError_t e, const char* what)
{
    return fail(h, OSE_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(h, call)                                                          \
    do {                                                                     \
        cudaError_t e_ = (call);                                             \
        if (e_ != cudaSuccess) return cuda_fail((h), e_, #call);             \
    } while (0)

template <typename T>
cudaError_t dalloc(ose_handle* h, T** p, size_t count)
{
    size_t b = sizeof(T) * count;
    if (h->fail_alloc_at > 0 && ++h->nalloc == h->fail_alloc_at) return cudaErrorMemoryAllocation;
    cudaError_t e = cudaMalloc((void**)p, b);
    if (e == cudaSuccess) h->bytes += b;
    return e;
}

template <typename T>
cudaError_t upload(ose_handle* h, T* dst, const std::vector<T>& src)
{
    return cudaMemcpyAsync(dst, src.data(), sizeof(T) * src.size(), cudaMemcpyHostToDevice, h->stream);
}

void free_all(ose_handle* h)
{
    if (h->graph) cudaGraphExecDestroy(h->graph);
    void* bufs[] = {h->W, h->A, h->S, h->X, h->vs, h->ax, h->ay, h->az, h->kx2, h->ky2, h->kz2,
                    h->twx, h->twy, h->twz, h->ricker, h->hil, h->gather, h->ctr,
                    h->kx2l, h->ky2l, h->kz2l, h->twxl, h->tcb, h->tcerr, h->rec_idx};
    for (void* b : bufs)
        if (b) cudaFree(b);
    for (float2* b : h->bluetab)
        if (b) cudaFree(b);
    if (h->ev0) cudaEventDestroy(h->ev0);
    if (h->ev1) cudaEventDestroy(h->ev1);
    if (h->timing.ev[0]) cudaEventDestroy(h->timing.ev[0]);
    if (h->timing.ev[1]) cudaEventDestroy(h->timing.ev[1]);
    if (h->Wsnap) cudaFree(h->Wsnap);
    for (int b = 0; b < 2; ++b) {
        if (h->hsnap[b]) cudaFreeHost(h->hsnap[b]);
        if (h->snap_done[b]) cudaEventDestroy(h->snap_done[b]);
    }
    if (h->snap_ready) cudaEventDestroy(h->snap_ready);
    if (h->rec_stage) cudaFreeHost(h->rec_stage);
    for (int b = 0; b < 2; ++b)
        if (h->rec_ev[b]) cudaEventDestroy(h->rec_ev[b]);
    if (h->copy_stream) cudaStreamDestroy(h->copy_stream);
    if (h->corr) ose::learn::delete_corrector(h->corr);
    if (h->corr_vel) cudaFree(h->corr_vel);
    if (h->stream) cudaStreamDestroy(h->stream);
}

// Runs one launch; with a timing record, brackets it with events and adds
// its duration and algorithmic bytes to class cls.
template <typename F>
cudaError_t timed(ose::KernelTiming* tm, cudaStream_t s, int cls, double bytes, F launch)
{
    if (tm) cudaEventRecord(tm->ev[0], s);
    cudaError_t e = launch();
    if (tm && e == cudaSuccess) {
        cudaEventRecord(tm->ev[1], s);
        e = cudaEventSynchronize(tm->ev[1]);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, tm->ev[0], tm->ev[1]);
        tm->ms[cls] += ms;
        tm->count[cls] += 1;
        tm->bytes[cls] += bytes;
    }
    return e;
}

// Receiver list: Q of step ctr[1] at the listed cells (rec_shotdata_3d's
// gxyz form, ose_3d_kernel.cu:412-421).
__global__ void k_record_list(const float2* __restrict__ W, const long long* __restrict__ idx, int n,
                              float* __restrict__ gather, const int* __restrict__ ctr, int nt)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int c = ctr[1];
    if (i < n && c >= 0 && c < nt) gather[(size_t)c * n + i] = W[idx[i]].y;
}

cudaError_t enqueue_receivers(ose_handle* h, ose::KernelTiming* tm)
{
    if (h->rec_xyz.empty()) return cudaSuccess;
    const int n = h->d.ng;
    return timed(tm, h->stream, 5, 12.0 * n, [&] {
        k_record_list<<<(n + 255) / 256, 256, 0, h->stream>>>(h->W, h->rec_idx, n, h->gather, h->ctr, h->p.nt);
        return cudaGetLastError();
    });
}

// The learned boundary correction at the end of a step: timing class 6 the
// local scale (shell sum of squares, three box passes over the grid), class 7
// the four layers (bytes: layer 0 reads state + velocity + scale and writes
// 32 BF16 channels, two hidden layers read and write them, the output layer
// reads them and updates the state).
cudaError_t enqueue_corrector(ose_handle* h, ose::KernelTiming* tm)
{
    if (!h->corr) return cudaSuccess;
    const ose::learn::Net& n = ose::learn::net_of(h->corr);
    const ose::learn::TcNet* tc = ose::learn::tc_of(h->corr);
    const double grid = (double)n.g.nx * n.g.ny * n.g.nz;
    cudaError_t e = timed(tm, h->stream, 6, (double)n.ncells * 8.0 + grid * (8.0 + 5 * 4.0), [&] {
        return ose::learn::shell_scale(h->stream, n, h->W);
    });
    if (e != cudaSuccess) return e;
    const double bytes = (double)n.ncells * (8.0 + 12.0 + 64.0 + 2 * 128.0 + 64.0 + 16.0);
    return timed(tm, h->stream, 7, bytes, [&] {
        return tc ? ose::learn::forward_tc(h->stream, n, *tc, h->W, h->corr_vel, false)
                  : ose::learn::forward(h->stream, n, h->W, h->corr_vel, true, h->W, false);
    });
}

// Plane path step: 2 HBM passes per operator application (ose_plane.cu).
// Timing classes: 0 plane_fwd, 1 zpass, 2 plane_inv_first, 3 plane_inv_mid,
// 4 plane_inv_last, 5 inject.
cudaError_t enqueue_step_plane(ose_handle* h, ose::KernelTiming* tm, bool source)
{
    cudaStream_t s = h->stream;
    const double N = (double)h->g.ncell;
    cudaError_t e = source ? timed(tm, s, 5, 16.0, [&] {
        return ose::launch_inject(s, h->W, h->src, h->ricker, h->hil, h->ctr, h->p.nt);
    }) : cudaSuccess;
    if (e != cudaSuccess) return e;
    const int M = h->d.M;
    ose::EpiArgs ea{};
    ea.vs = h->vs;
    ea.sch = h->sch;
    ea.scl = h->scl;
    ea.ax = h->ax;
    ea.ay = h->ay;
    ea.az = h->az;
    ea.S = h->S;
    ea.wout = h->W;
    ea.gather = h->gather;
    ea.cur = h->ctr + 1;
    ea.gz = h->rec_xyz.empty() ? h->p.bu + h->p.gzbeg : -1;   // a receiver list records separately
    ea.bl = h->p.bl;
    ea.bf = h->p.bf;
    ea.nx = h->p.nx;
    ea.ny = h->p.ny;
    ea.nt = h->p.nt;
    e = timed(tm, s, 0, 16.0 * N, [&] { return ose::launch_plane_fwd(s, h->W, h->X, h->tables); });
    if (e != cudaSuccess) return e;
    for (int n = 0; n <= M; ++n) {
        e = timed(tm, s, 1, 16.0 * N, [&] { return ose::launch_zpass(s, h->X, h->tables); });
        if (e != cudaSuccess) return e;
        const ose::EpiMode mode = n == 0 ? ose::EPI_FIRST : (n == M ? ose::EPI_LAST : ose::EPI_MID);
        ea.prev = n == 0 ? h->A : ((n & 1) ? h->W : h->A);
        ose::set_application(ea, n, M, h->J.data());
        const bool fwd = n < M;
        const double bytes = ose::epilogue_bytes(mode, ea.sp, fwd) * N;
        // classes: 3 MID reading and writing S, 9 MID starting S, 8 MID leaving S alone
        const int cls = mode == ose::EPI_FIRST ? 2
                        : (mode == ose::EPI_LAST ? 4 : (ea.sp.touch ? (ea.sp.s_read ? 3 : 9) : 8));
        e = timed(tm, s, cls, bytes, [&] { return ose::launch_plane_inv(s, mode, fwd, h->X, h->X, h->tables, ea); });
        if (e != cudaSuccess) return e;
    }
    if (source && (e = enqueue_receivers(h, tm)) != cudaSuccess) return e;
    return enqueue_corrector(h, tm);
}

// Enqueue one whole time step on h->stream (no synchronisation).
// source = false leaves out the source injection (reverse-time propagation).
cudaError_t enqueue_step(ose_handle* h, ose::KernelTiming* tm, bool source = true)
{
    if (h->d.path == OSE_PATH_PLANE) return enqueue_step_plane(h, tm, source);
    cudaError_t e = source ? timed(tm, h->stream, 5, 16.0, [&] {
        return ose::launch_inject(h->stream, h->W, h->src, h->ricker, h->hil, h->ctr, h->p.nt);
    }) : cudaSuccess;
    if (e != cudaSuccess) return e;
    const int M = h->d.M;
    ose::EpiArgs ea{};
    ea.vs = h->vs;
    ea.sch = h->sch;
    ea.scl = h->scl;
    ea.ax = h->ax;
    ea.ay = h->ay;
    ea.az = h->az;
    ea.S = h->S;
    ea.wout = h->W;
    ea.gather = h->gather;
    ea.cur = h->ctr + 1;
    ea.gz = h->rec_xyz.empty() ? h->p.bu + h->p.gzbeg : -1;   // a receiver list records separately
    ea.bl = h->p.bl;
    ea.bf = h->p.bf;
    ea.nx = h->p.nx;
    ea.ny = h->p.ny;
    ea.nt = h->p.nt;
    const double N = (double)h->g.ncell;
    // with the register row kernels, the row pass of application n also
    // writes the x transform of a_{n+1}, so application n + 1 skips its x pass
    const bool fuse = ose::generic_fuses_x(h->px, h->tables);
    for (int n = 0; n <= M; ++n) {
        // n = 0: a_1 = -i L a_0 from a_0 = W
        const float2* an = n == 0 ? h->W : ((n & 1) ? h->A : h->W);
        const ose::EpiMode mode = n == 0 ? ose::EPI_FIRST : (n == M ? ose::EPI_LAST : ose::EPI_MID);
        ea.prev = n == 0 ? h->A : ((n & 1) ? h->W : h->A);
        ose::set_application(ea, n, M, h->J.data());
        const bool fwd = fuse && n < M;
        e = ose::launch_generic_application(h->stream, h->g, h->px, h->py, h->pz, h->tables, an, h->X, mode, ea,
                                            tm, fuse && n > 0, fwd);
        if (tm) {
            for (int c = (fuse && n > 0) ? 1 : 0; c < 4; ++c) tm->bytes[c] += 16.0 * N;
            const bool skip = mode != ose::EPI_LAST && !ea.sp.touch;
            tm->bytes[skip ? 8 : 4] += ose::epilogue_bytes(mode, ea.sp, fwd) * N;
        }
        if (e != cudaSuccess) return e;
    }
    if (source && (e = enqueue_receivers(h, tm)) != cudaSuccess) return e;
    return enqueue_corrector(h, tm);
}

ose_status build_graph(ose_handle* h)
{
    if (h->graph) return OSE_OK;
    cudaGraph_t graph = nullptr;
    CK(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = enqueue_step(h, nullptr);
    cudaError_t e2 = cudaStreamEndCapture(h->stream, &graph);
    if (e != cudaSuccess) { if (graph) cudaGraphDestroy(graph); return cuda_fail(h, e, "capture step"); }
    if (e2 != cudaSuccess) return cuda_fail(h, e2, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&h->graph, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) { h->graph = nullptr; return cuda_fail(h, e, "cudaGraphInstantiate"); }
    return OSE_OK;
}

// After the stream is idle: kernels with bounded waits (tensor-core z pass,
// corrector, the plane kernels' exchanges) record a wait that ran out of time
// in the handle's error word.
ose_status tensor_status(ose_handle* h)
{
    if (!h->tcerr) return OSE_OK;
    int v = 0;
    CK(h, cudaMemcpy(&v, h->tcerr, sizeof(int), cudaMemcpyDeviceToHost));
    if (v) {
        CK(h, cudaMemset(h->tcerr, 0, sizeof(int)));
        return fail(h, OSE_ERR_TIMEOUT, v == 3 ? "plane kernels: a DSMEM exchange wait ran out of time"
                                     : v == 2 ? "boundary corrector: an MMA completion wait ran out of time"
                                              : "tensor-core z pass: an MMA completion wait ran out of time");
    }
    return OSE_OK;
}

// The padded model [z][y][x] from the interior [x][y][z] (edge values
// replicated into the sponge, as pad_model on the host), scaled by sc in
// double and rounded to float (scale = false: v itself).
__global__ void k_pad_model(const float* __restrict__ vin, float* __restrict__ vs, ose_params p, int nxb, int nyb,
                            int nzb, double sc, bool scale)
{
    const long long n = (long long)nxb * nyb * nzb;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(i % nxb), y = (int)((i / nxb) % nyb), z = (int)(i / ((long long)nxb * nyb));
        const int ix = x < p.bl ? 0 : (x >= p.bl + p.nx ? p.nx - 1 : x - p.bl);
        const int iy = y < p.bf ? 0 : (y >= p.bf + p.ny ? p.ny - 1 : y - p.bf);
        const int iz = z < p.bu ? 0 : (z >= p.bu + p.nz ? p.nz - 1 : z - p.bu);
        const float v = vin[((size_t)ix * p.ny + iy) * p.nz + iz];
        vs[i] = scale ? (float)((double)v * sc) : v;
    }
}

// P (which = 0) or Q (1) of the state, deinterleaved
__global__ void k_take_component(const float2* __restrict__ W, float* __restrict__ out, long long n, int which)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float2 w = W[i];
        out[i] = which ? w.y : w.x;
    }
}

// The padded model on the host (pad_model of the model as given), made on
// first use.
const std::vector<float>& padded_model(ose_handle* h)
{
    if (h->vb.empty()) ose::pad_model(h->p, h->d, h->vel_in.data(), h->vb);
    return h->vb;
}

void to_layout(const ose_handle* h, const float* zyx, float* out, int layout)
{
    const int nxb = h->d.nxb, nyb = h->d.nyb, nzb = h->d.nzb;
    if (layout == OSE_LAYOUT_ZYX) {
        memcpy(out, zyx, sizeof(float) * (size_t)nxb * nyb * nzb);
        return;
    }
    size_t o = 0;   // [y][x][z] (write_3dfile_from_1darray_ci, ose_3d_lib.cu:374-377)
    for (int y = 0; y < nyb; ++y)
        for (int x = 0; x < nxb; ++x)
            for (int z = 0; z < nzb; ++z) out[o++] = zyx[((size_t)z * nyb + y) * nxb + x];
}

void from_layout(const ose_handle* h, const float* in, float* zyx, int layout)
{
    const int nxb = h->d.nxb, nyb = h->d.nyb, nzb = h->d.nzb;
    if (layout == OSE_LAYOUT_ZYX) {
        memcpy(zyx, in, sizeof(float) * (size_t)nxb * nyb * nzb);
        return;
    }
    size_t o = 0;
    for (int y = 0; y < nyb; ++y)
        for (int x = 0; x < nxb; ++x)
            for (int z = 0; z < nzb; ++z) zyx[((size_t)z * nyb + y) * nxb + x] = in[o++];
}

}  // namespace

extern "C" {

const char* ose_version(void) { return "ose3d-gb300 0.1 (sm_103a)"; }

ose_status ose_default_params(ose_params* p)
{
    if (!p) return OSE_ERR_INVALID;
    memset(p, 0, sizeof(*p));
    p->nx = p->ny = p->nz = 101;
    p->bu = p->bd = p->bl = p->br = p->bf = p->bb = 25;
    p->nt = 300;
    p->fm = 40.0f;
    p->dt = 0.001f;
    p->amp = 100.0f;
    p->dx = p->dy = p->dz = 10.0f;
    p->nshot = 1;
    p->sxbeg = p->nx / 2;
    p->sybeg = p->ny / 2;
    p->szbeg = 0;
    p->jsx = p->jsy = p->jsz = 1;
    p->jgx = p->jgy = p->jgz = 1;
    return OSE_OK;
}

ose_status ose_padded_dims(const ose_params* p, int* nxb, int* nyb, int* nzb)
{
    if (!p || !nxb || !nyb || !nzb) return OSE_ERR_INVALID;
    ose_derived d;
    std::string err;
    if (ose::derive_dims(*p, &d, &err)) return fail(nullptr, OSE_ERR_INVALID, err);
    *nxb = d.nxb;
    *nyb = d.nyb;
    *nzb = d.nzb;
    return OSE_OK;
}

const char* ose_last_error(const ose_handle* h) { return h ? h->err.c_str() : g_create_error.c_str(); }

ose_status ose_self_test_waits(double limit_ms, int* expired)
{
    if (!expired || !(limit_ms > 0.0 && limit_ms <= 100.0))
        return fail(nullptr, OSE_ERR_INVALID, "ose_self_test_waits: limit_ms must be in (0, 100]");
    *expired = 0;
    int* d = nullptr;   // error words [0..2], grid barrier words [4..5]
    cudaStream_t s = nullptr;
    const unsigned long long ns = (unsigned long long)(limit_ms * 1e6);
    int w[3] = {0, 0, 0};
    cudaError_t e = cudaMalloc((void**)&d, 8 * sizeof(int));
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMemsetAsync(d, 0, 8 * sizeof(int), s);
    if (e == cudaSuccess) e = ose::selftest_exchange_wait(s, d + 0, ns);
    if (e == cudaSuccess) e = ose::selftest_grid_barrier(s, reinterpret_cast<unsigned*>(d + 4), d + 1, ns);
    if (e == cudaSuccess) e = ose::selftest_mma_wait(s, d + 2, ns);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e == cudaSuccess) e = cudaMemcpy(w, d, sizeof w, cudaMemcpyDeviceToHost);
    if (s) cudaStreamDestroy(s);
    if (d) cudaFree(d);
    if (e != cudaSuccess) return fail(nullptr, OSE_ERR_CUDA, std::string("ose_self_test_waits: ") + cudaGetErrorString(e));
    *expired = (w[0] ? 1 : 0) | (w[1] ? 2 : 0) | (w[2] ? 4 : 0);
    return OSE_OK;
}

ose_status ose_get_derived(const ose_handle* h, ose_derived* d)
{
    if (!h || !d) return OSE_ERR_INVALID;
    *d = h->d;
    d->device_bytes = h->bytes;
    return OSE_OK;
}

ose_status ose_create(const ose_params* pin, const float* vel, ose_handle** out)
{
    if (!pin || !vel || !out) return fail(nullptr, OSE_ERR_INVALID, "null argument");
    *out = nullptr;
    ose_handle* h = new (std::nothrow) ose_handle();
    if (!h) return fail(nullptr, OSE_ERR_NOMEM, "host allocation failed");
    if (const char* fa = getenv("OSE3D_FAIL_DEVICE_ALLOC")) h->fail_alloc_at = atoi(fa);
    h->p = *pin;
    std::string err;
    if (ose::derive_dims(h->p, &h->d, &err)) { delete h; return fail(nullptr, OSE_ERR_INVALID, err); }
    const ose_params& p = h->p;
    ose_derived& d = h->d;
    if (p.sponge_mode != OSE_SPONGE_REFERENCE && p.sponge_mode != OSE_SPONGE_CERJAN) {
        delete h;
        return fail(nullptr, OSE_ERR_INVALID, "unknown sponge_mode");
    }
    if (ose::plan_axis(d.nxb, &h->px) || ose::plan_axis(d.nyb, &h->py) || ose::plan_axis(d.nzb, &h->pz)) {
        delete h;
        return fail(nullptr, OSE_ERR_UNSUPPORTED, "padded axis longer than 1024 or not factorable");
    }
    if (p.gzbeg < 0 || p.gzbeg >= p.nz) {
        delete h;
        return fail(nullptr, OSE_ERR_INVALID, "receiver depth gzbeg outside the interior");
    }
    h->g.nxb = d.nxb;
    h->g.nyb = d.nyb;
    h->g.nzb = d.nzb;
    h->g.ncell = (long long)d.nxb * d.nyb * d.nzb;
    const size_t N = (size_t)h->g.ncell;

    // the padded model repeats the interior's values, so its maximum and its
    // validity are the interior's
    const size_t nin = (size_t)p.nx * p.ny * p.nz;
    h->vel_in.assign(vel, vel + nin);
    float vmax = -9999999.999f;    // find_max (ose_3d_lib.cu:544-555)
    bool valid = true;
    for (float v : h->vel_in) {
        vmax = v > vmax ? v : vmax;
        valid = valid && v > 0.f && std::isfinite(v);
    }
    if (!valid || !(vmax > 0.f) || !std::isfinite(vmax)) {
        delete h;
        return fail(nullptr, OSE_ERR_INVALID, "velocity model must be positive and finite");
    }
    ose::series_params(p, vmax, &d);
    h->J.resize(d.M + 2);
    for (int n = 0; n <= d.M + 1; ++n) h->J[n] = jn(n, d.dtR);
    ose::sponge_table(p.bl, p.nx, d.br, p.sponge_mode, p.cerjan_factor, h->h_ax);
    ose::sponge_table(p.bf, p.ny, d.bb, p.sponge_mode, p.cerjan_factor, h->h_ay);
    ose::sponge_table(p.bu, p.nz, d.bd, p.sponge_mode, p.cerjan_factor, h->h_az);
    std::vector<float> kx2, ky2, kz2, kx2l, ky2l, kz2l;
    ose::k2_table(d.nxb, d.dkx, kx2, &kx2l);
    ose::k2_table(d.nyb, d.dky, ky2, &ky2l);
    ose::k2_table(d.nzb, d.dkz, kz2, &kz2l);
    std::vector<float2> twx, twy, twz, twxl;
    ose::twiddle_table(d.nxb, twx, &twxl);
    ose::twiddle_table(d.nyb, twy);
    ose::twiddle_table(d.nzb, twz);
    // L = v * IFFT3(|k| FFT3(.)) * (1 / (R N)): the device keeps v itself and
    // applies 1/(R N) as a float pair
    ose::split_float(1.0 / (d.R * (double)N), &h->sch, &h->scl);

    cudaError_t e = cudaGetDevice(&h->device);
    if (e != cudaSuccess) { ose_status s = cuda_fail(nullptr, e, "cudaGetDevice"); delete h; return s; }
#define CKC(call)                                                                   \
    do {                                                                            \
        cudaError_t e_ = (call);                                                    \
        if (e_ != cudaSuccess) {                                                    \
            ose_status s_ = cuda_fail(nullptr, e_, #call);                          \
            if (e_ == cudaErrorMemoryAllocation) s_ = OSE_ERR_NOMEM;                \
            free_all(h);                                                            \
            delete h;                                                               \
            return s_;                                                              \
        }                                                                           \
    } while (0)
    CKC(ose::configure_kernels());
    CKC(ose::configure_plane_kernels());
    CKC(ose::configure_tensor_kernels());
    CKC(ose::configure_bluestein_kernels());
    CKC(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    CKC(cudaEventCreate(&h->ev0));
    CKC(cudaEventCreate(&h->ev1));
    CKC(cudaEventCreate(&h->timing.ev[0]));
    CKC(cudaEventCreate(&h->timing.ev[1]));
    CKC(dalloc(h, &h->W, N));
    CKC(dalloc(h, &h->A, N));
    CKC(dalloc(h, &h->S, N));
    CKC(dalloc(h, &h->X, N));
    CKC(dalloc(h, &h->vs, N));
    CKC(dalloc(h, &h->ax, d.nxb));
    CKC(dalloc(h, &h->ay, d.nyb));
    CKC(dalloc(h, &h->az, d.nzb));
    CKC(dalloc(h, &h->kx2, d.nxb));
    CKC(dalloc(h, &h->ky2, d.nyb));
    CKC(dalloc(h, &h->kz2, d.nzb));
    CKC(dalloc(h, &h->twx, d.nxb));
    CKC(dalloc(h, &h->twy, d.nyb));
    CKC(dalloc(h, &h->twz, d.nzb));
    CKC(dalloc(h, &h->twxl, d.nxb));
    CKC(dalloc(h, &h->kx2l, d.nxb));
    CKC(dalloc(h, &h->ky2l, d.nyb));
    CKC(dalloc(h, &h->kz2l, d.nzb));
    CKC(dalloc(h, &h->ricker, (size_t)p.nt));
    CKC(dalloc(h, &h->hil, (size_t)p.nt));
    CKC(dalloc(h, &h->gather, (size_t)p.nt * d.ng));
    CKC(dalloc(h, &h->ctr, 4));
    CKC(dalloc(h, &h->tcerr, 1));
    CKC(cudaMemset(h->tcerr, 0, sizeof(int)));
    // the model as given goes up once (X is free scratch here) and is padded
    // on the device; vs = v (compensated constants) or v / (R N)
    CKC(cudaMemcpyAsync(h->X, h->vel_in.data(), sizeof(float) * nin, cudaMemcpyHostToDevice, h->stream));
    k_pad_model<<<4096, 256, 0, h->stream>>>(reinterpret_cast<const float*>(h->X), h->vs, p, d.nxb, d.nyb, d.nzb,
                                             1.0 / (d.R * (double)N), !ose::kCompensatedConstants);
    CKC(cudaGetLastError());
    CKC(upload(h, h->twxl, twxl));
    CKC(upload(h, h->kx2l, kx2l));
    CKC(upload(h, h->ky2l, ky2l));
    CKC(upload(h, h->kz2l, kz2l));
    CKC(upload(h, h->ax, h->h_ax));
    CKC(upload(h, h->ay, h->h_ay));
    CKC(upload(h, h->az, h->h_az));
    CKC(upload(h, h->kx2, kx2));
    CKC(upload(h, h->ky2, ky2));
    CKC(upload(h, h->kz2, kz2));
    CKC(upload(h, h->twx, twx));
    CKC(upload(h, h->twy, twy));
    CKC(upload(h, h->twz, twz));
    // axes without register kernels of their own: Bluestein tables (chirp,
    // spectrum, W_L) in one buffer per axis (none for a 256-long axis)
    std::vector<float2> blue_all[3];
    {
        const int ns[3] = {d.nxb, d.nyb, d.nzb};
        for (int a = 0; a < 3; ++a) {
            const int L = ose::bluestein_length(ns[a]);
            h->tables.bl[a] = L;
            if (!L) continue;
            std::vector<float2> ch, sp, tw;
            ose::bluestein_tables(ns[a], L, ch, sp, tw);
            blue_all[a] = ch;
            blue_all[a].insert(blue_all[a].end(), sp.begin(), sp.end());
            blue_all[a].insert(blue_all[a].end(), tw.begin(), tw.end());
            CKC(dalloc(h, &h->bluetab[a], blue_all[a].size()));
            CKC(upload(h, h->bluetab[a], blue_all[a]));
            h->tables.bch[a] = h->bluetab[a];
            h->tables.bsp[a] = h->bluetab[a] + ns[a];
            h->tables.btw[a] = h->bluetab[a] + ns[a] + L;
        }
    }
    CKC(cudaMemsetAsync(h->W, 0, sizeof(float2) * N, h->stream));
    CKC(cudaMemsetAsync(h->ctr, 0, sizeof(int) * 4, h->stream));
    CKC(cudaStreamSynchronize(h->stream));
#undef CKC
    h->tables.twx = h->twx;
    h->tables.twy = h->twy;
    h->tables.twz = h->twz;
    h->tables.kx2 = h->kx2;
    h->tables.ky2 = h->ky2;
    h->tables.kz2 = h->kz2;
    h->tables.twl = h->twxl;
    h->tables.tcerr = h->tcerr;
    h->tables.kx2l = h->kx2l;
    h->tables.ky2l = h->ky2l;
    h->tables.kz2l = h->kz2l;

    d.path = ose::plane_path_supported(d.nxb, d.nyb, d.nzb) ? OSE_PATH_PLANE : OSE_PATH_GENERIC;
    if (const char* env = getenv("OSE3D_PATH"))
        if (!strcmp(env, "generic")) d.path = OSE_PATH_GENERIC;
    d.device_bytes = h->bytes;
    *out = h;
    return OSE_OK;
}

ose_status ose_create_from_file(const ose_params* p, const char* path, ose_handle** out)
{
    if (!p || !path || !out) return fail(nullptr, OSE_ERR_INVALID, "null argument");
    FILE* f = fopen(path, "rb");
    if (!f) return fail(nullptr, OSE_ERR_IO, std::string("cannot open ") + path);
    const size_t n = (size_t)p->nx * p->ny * p->nz;
    std::vector<float> v(n);
    size_t got = fread(v.data(), sizeof(float), n, f);
    fclose(f);
    if (got != n) return fail(nullptr, OSE_ERR_IO, std::string("short model file ") + path);
    return ose_create(p, v.data(), out);
}

ose_status ose_destroy(ose_handle* h)
{
    if (!h) return OSE_OK;
    if (h->stream) cudaStreamSynchronize(h->stream);
    free_all(h);
    delete h;
    return OSE_OK;
}

// Source cell and source traces of shot `is` (no change to the wavefield).
static ose_status prepare_shot(ose_handle* h, int is)
{
    const ose_params& p = h->p;
    if (is < 0) return fail(h, OSE_ERR_INVALID, "negative shot index");
    // source: sg_init_host then the decode of Xt_add_wavelet_sxyz (ose_3d_lib.cu:598-616)
    const long long nxy = (long long)p.nx * p.ny;
    const long long sx0 = p.sxbeg + (long long)is * p.jsx, sy0 = p.sybeg + (long long)is * p.jsy,
                    sz0 = p.szbeg + (long long)is * p.jsz;
    const long long sxyz = sz0 * nxy + sy0 * p.nx + sx0;
    if (sxyz < 0) return fail(h, OSE_ERR_INVALID, "source outside the model");
    const long long sx = sxyz % nxy % p.nx, sy = sxyz % nxy / p.nx, sz = sxyz / nxy;
    const long long X = p.bl + sx, Y = p.bf + sy, Z = p.bu + sz;
    if (X >= h->d.nxb || Y >= h->d.nyb || Z >= h->d.nzb)
        return fail(h, OSE_ERR_INVALID, "source outside the padded grid");
    h->src = (Z * h->d.nyb + Y) * h->d.nxb + X;
    // Alloc_wavelet (ose_3d_lib.cu:557-586)
    ose::ricker_trace(p.nt, p.fm, p.dt, p.amp, h->h_ricker);
    ose::hilbert_trace(h->h_ricker, p.hilbert_div_nt, h->h_hil);
    CK(h, upload(h, h->ricker, h->h_ricker));
    CK(h, upload(h, h->hil, h->h_hil));
    if (h->graph) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; }   // src may have moved
    h->shot = is;
    return OSE_OK;
}

ose_status ose_reset_shot(ose_handle* h, int is)
{
    if (!h) return OSE_ERR_INVALID;
    ose_status st = prepare_shot(h, is);
    if (st != OSE_OK) return st;
    const ose_params& p = h->p;
    const size_t N = (size_t)h->g.ncell;
    // Xtdata_value: the state starts at rest
    CK(h, cudaMemsetAsync(h->W, 0, sizeof(float2) * N, h->stream));
    CK(h, cudaMemsetAsync(h->gather, 0, sizeof(float) * (size_t)p.nt * h->d.ng, h->stream));
    CK(h, cudaMemsetAsync(h->ctr, 0, sizeof(int) * 4, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    h->it = 0;
    h->shot_ready = true;
    return OSE_OK;
}

ose_status ose_step(ose_handle* h)
{
    if (!h) return OSE_ERR_INVALID;
    if (!h->shot_ready) return fail(h, OSE_ERR_STATE, "ose_reset_shot must come first");
    if (h->it >= h->p.nt) return fail(h, OSE_ERR_STATE, "all nt steps of the shot are done");
    CK(h, enqueue_step(h, nullptr));
    CK(h, cudaStreamSynchronize(h->stream));
    h->it += 1;
    return tensor_status(h);
}

static ose_status run_graph(ose_handle* h, int nsteps)
{
    if (!h->shot_ready) return fail(h, OSE_ERR_STATE, "ose_reset_shot must come first");
    if (nsteps < 0 || h->it + nsteps > h->p.nt) return fail(h, OSE_ERR_INVALID, "nsteps beyond nt");
    ose_status s = build_graph(h);
    if (s != OSE_OK) return s;
    for (int i = 0; i < nsteps; ++i) CK(h, cudaGraphLaunch(h->graph, h->stream));
    return OSE_OK;
}

ose_status ose_run(ose_handle* h, int nsteps, float* gather_out)
{
    if (!h) return OSE_ERR_INVALID;
    ose_status s = run_graph(h, nsteps);
    if (s != OSE_OK) return s;
    CK(h, cudaStreamSynchronize(h->stream));
    h->it += nsteps;
    if ((s = tensor_status(h)) != OSE_OK) return s;
    if (gather_out) return ose_get_gather(h, gather_out);
    return OSE_OK;
}

// Steps are enqueued in chunks of kRecChunk without waiting on the host; each
// chunk's receiver rows go to one of two pinned buffers by an asynchronous
// copy, and the host moves chunk c into rows_out while chunk c + 1 runs.
constexpr int kRecChunk = 32;

ose_status ose_run_record(ose_handle* h, int nsteps, float* rows_out)
{
    if (!h || !rows_out || nsteps < 0) return OSE_ERR_INVALID;
    if (!h->shot_ready) return fail(h, OSE_ERR_STATE, "ose_reset_shot must come first");
    if (h->it + nsteps > h->p.nt) return fail(h, OSE_ERR_INVALID, "nsteps beyond nt");
    const int ng = h->d.ng;
    if (!h->rec_stage || h->rec_stage_ng != ng) {
        if (h->rec_stage) cudaFreeHost(h->rec_stage);
        h->rec_stage = nullptr;
        CK(h, cudaMallocHost((void**)&h->rec_stage, sizeof(float) * 2 * kRecChunk * (size_t)ng));
        h->rec_stage_ng = ng;
    }
    for (int b = 0; b < 2; ++b)
        if (!h->rec_ev[b]) CK(h, cudaEventCreateWithFlags(&h->rec_ev[b], cudaEventDisableTiming));
    const size_t chunk = (size_t)kRecChunk * ng;
    int pending_k = 0, pending_b = 0;
    float* pending_out = nullptr;
    auto drain = [&]() -> ose_status {
        if (!pending_k) return OSE_OK;
        CK(h, cudaEventSynchronize(h->rec_ev[pending_b]));
        memcpy(pending_out, h->rec_stage + pending_b * chunk, sizeof(float) * (size_t)pending_k * ng);
        pending_k = 0;
        return OSE_OK;
    };
    for (int done = 0, c = 0; done < nsteps; ++c) {
        const int k = std::min(kRecChunk, nsteps - done), b = c & 1;
        const int it0 = h->it;
        ose_status s = run_graph(h, k);
        if (s != OSE_OK) return s;
        CK(h, cudaMemcpyAsync(h->rec_stage + b * chunk, h->gather + (size_t)it0 * ng, sizeof(float) * (size_t)k * ng,
                              cudaMemcpyDeviceToHost, h->stream));
        CK(h, cudaEventRecord(h->rec_ev[b], h->stream));
        h->it += k;
        // chunk c - 1 (the other buffer) is complete or about to be
        if ((s = drain()) != OSE_OK) return s;
        pending_k = k;
        pending_b = b;
        pending_out = rows_out + (size_t)done * ng;
        done += k;
    }
    ose_status s = drain();
    if (s != OSE_OK) return s;
    return tensor_status(h);
}

ose_status ose_run_timed(ose_handle* h, int nsteps, float* ms)
{
    if (!h || !ms) return OSE_ERR_INVALID;
    if (!h->shot_ready) return fail(h, OSE_ERR_STATE, "ose_reset_shot must come first");
    ose_status s = build_graph(h);
    if (s != OSE_OK) return s;
    CK(h, cudaStreamSynchronize(h->stream));
    CK(h, cudaEventRecord(h->ev0, h->stream));
    s = run_graph(h, nsteps);
    if (s != OSE_OK) return s;
    CK(h, cudaEventRecord(h->ev1, h->stream));
    CK(h, cudaEventSynchronize(h->ev1));
    CK(h, cudaEventElapsedTime(ms, h->ev0, h->ev1));
    h->it += nsteps;
    return tensor_status(h);
}

ose_status ose_select_path(ose_handle* h, int path)
{
    if (!h) return OSE_ERR_INVALID;
    if (path == OSE_PATH_PLANE && !ose::plane_path_supported(h->d.nxb, h->d.nyb, h->d.nzb))
        return fail(h, OSE_ERR_UNSUPPORTED, "the plane path needs a 256 x 256 x 256 padded grid");
    if (path != OSE_PATH_PLANE && path != OSE_PATH_GENERIC) return fail(h, OSE_ERR_INVALID, "unknown path");
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->graph) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; }
    h->d.path = path;
    return OSE_OK;
}

ose_status ose_set_precision(ose_handle* h, int mode)
{
    if (!h) return OSE_ERR_INVALID;
    if (mode < OSE_PRECISION_FP32 || mode > OSE_PRECISION_BF16X3) return fail(h, OSE_ERR_INVALID, "unknown precision mode");
    if (mode != OSE_PRECISION_FP32 && !ose::tensor_zpass_supported(h->d.nxb, h->d.nyb, h->d.nzb))
        return fail(h, OSE_ERR_UNSUPPORTED, "the tensor-core z pass needs nzb = 256 and nxb a multiple of 16");
    CK(h, cudaStreamSynchronize(h->stream));
    if (mode != OSE_PRECISION_FP32) {
        if (!h->tcb) CK(h, dalloc(h, (uint8_t**)&h->tcb, ose::tensor_operand_bytes(OSE_PRECISION_TF32)));
        if (!h->tcerr) {
            CK(h, dalloc(h, &h->tcerr, 1));
            CK(h, cudaMemset(h->tcerr, 0, sizeof(int)));
        }
        std::vector<uint8_t> ops;
        ose::tensor_operands(mode, ops);
        CK(h, cudaMemcpy(h->tcb, ops.data(), ops.size(), cudaMemcpyHostToDevice));
    }
    if (h->graph) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; }
    h->precision = mode;
    h->tables.tcvar = mode;
    h->tables.tcb = h->tcb;
    h->tables.tcerr = h->tcerr;
    return OSE_OK;
}

ose_status ose_get_precision(const ose_handle* h, int* mode)
{
    if (!h || !mode) return OSE_ERR_INVALID;
    *mode = h->precision;
    return OSE_OK;
}

ose_status ose_set_receivers(ose_handle* h, int n, const int* xyz)
{
    if (!h || n < 0 || (n > 0 && !xyz)) return OSE_ERR_INVALID;
    const ose_params& p = h->p;
    for (int i = 0; i < n; ++i) {
        const int x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
        if (x < 0 || x >= p.nx || y < 0 || y >= p.ny || z < 0 || z >= p.nz)
            return fail(h, OSE_ERR_INVALID, "receiver " + std::to_string(i) + " outside the model interior");
    }
    CK(h, cudaStreamSynchronize(h->stream));
    if (h->graph) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; }
    const int ng = n > 0 ? n : p.nx * p.ny;
    if (ng != h->d.ng) {
        float* g = nullptr;
        CK(h, cudaMalloc((void**)&g, sizeof(float) * (size_t)p.nt * ng));
        cudaFree(h->gather);
        h->gather = g;
        h->d.ng = ng;
    }
    CK(h, cudaMemset(h->gather, 0, sizeof(float) * (size_t)p.nt * ng));
    if (h->rec_idx) { cudaFree(h->rec_idx); h->rec_idx = nullptr; }
    h->rec_xyz.assign(xyz, xyz + 3 * (size_t)n);
    if (n > 0) {
        std::vector<long long> idx(n);
        for (int i = 0; i < n; ++i)
            idx[i] = ((long long)(p.bu + xyz[3 * i + 2]) * h->d.nyb + (p.bf + xyz[3 * i + 1])) * h->d.nxb +
                     (p.bl + xyz[3 * i]);
        CK(h, cudaMalloc((void**)&h->rec_idx, sizeof(long long) * n));
        CK(h, cudaMemcpy(h->rec_idx, idx.data(), sizeof(long long) * n, cudaMemcpyHostToDevice));
    }
    return OSE_OK;
}

ose_status ose_set_corrector(ose_handle* h, const float* params, int shell)
{
    if (!h) return OSE_ERR_INVALID;
    CK(h, cudaStreamSynchronize(h->stream));
    if (h->graph) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; }
    if (h->corr) { ose::learn::delete_corrector(h->corr); h->corr = nullptr; }
    if (!params) return OSE_OK;
    const int sp[6] = {h->p.bl, h->d.br, h->p.bf, h->d.bb, h->p.bu, h->d.bd};
    for (int i = 0; i < 6; ++i)
        if (shell < 1 || sp[i] > shell) return fail(h, OSE_ERR_INVALID, "the shell must be at least as wide as every sponge");
    ose::learn::NetGeom g{h->d.nxb, h->d.nyb, h->d.nzb, shell, {sp[0], sp[1], sp[2], sp[3], sp[4], sp[5]}};
    // the tensor-core kernels unless OSE3D_CORRECTOR=fp32 asks for the FP32 ones
    const char* mode = getenv("OSE3D_CORRECTOR");
    const bool fp32 = mode && strcmp(mode, "fp32") == 0;
    h->corr = ose::learn::new_corrector();
    cudaError_t e = ose::learn::create_net(h->corr, g, false, fp32);
    if (e == cudaSuccess)
        e = cudaMemcpy(ose::learn::net_of(h->corr).params, params, sizeof(float) * ose::learn::param_count(),
                       cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !h->corr_vel) {
        const std::vector<float>& vb = padded_model(h);
        e = cudaMalloc((void**)&h->corr_vel, sizeof(float) * vb.size());
        if (e == cudaSuccess) e = cudaMemcpy(h->corr_vel, vb.data(), sizeof(float) * vb.size(), cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess && !h->tcerr) {
        e = cudaMalloc((void**)&h->tcerr, sizeof(int));
        if (e == cudaSuccess) e = cudaMemset(h->tcerr, 0, sizeof(int));
    }
    if (e == cudaSuccess && !fp32) e = ose::learn::create_tc(h->corr, params, h->tcerr);
    if (e != cudaSuccess) {
        ose::learn::delete_corrector(h->corr);
        h->corr = nullptr;
        return cuda_fail(h, e, "ose_set_corrector");
    }
    return OSE_OK;
}

namespace {
__global__ void k_box(const float2* __restrict__ src, int snx, int sny, int sx0, int sy0, int sz0,
                      float2* __restrict__ dst, int dnx, int dny, int dx0, int dy0, int dz0, int nx, int ny, int nz)
{
    const long long n = (long long)nx * ny * nz;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(i % nx), y = (int)((i / nx) % ny), z = (int)(i / ((long long)nx * ny));
        dst[((size_t)(z + dz0) * dny + (y + dy0)) * dnx + (x + dx0)] =
            src[((size_t)(z + sz0) * sny + (y + sy0)) * snx + (x + sx0)];
    }
}
}  // namespace

ose_status ose_state_box(ose_handle* h, int dir, const int* box, void* buf_dev, const int* buf)
{
    if (!h || !box || !buf || !buf_dev || (dir != 0 && dir != 1)) return OSE_ERR_INVALID;
    const int x0 = box[0], y0 = box[1], z0 = box[2], nx = box[3], ny = box[4], nz = box[5];
    const int bnx = buf[0], bny = buf[1], bx0 = buf[2], by0 = buf[3], bz0 = buf[4];
    if (nx < 1 || ny < 1 || nz < 1 || x0 < 0 || y0 < 0 || z0 < 0 || x0 + nx > h->d.nxb || y0 + ny > h->d.nyb ||
        z0 + nz > h->d.nzb || bx0 < 0 || by0 < 0 || bz0 < 0 || bx0 + nx > bnx || by0 + ny > bny)
        return fail(h, OSE_ERR_INVALID, "box outside the grid or the buffer");
    float2* b = static_cast<float2*>(buf_dev);
    const unsigned blocks = (unsigned)std::min<long long>(4096, ((long long)nx * ny * nz + 255) / 256);
    if (dir == 0)
        k_box<<<blocks, 256, 0, h->stream>>>(h->W, h->d.nxb, h->d.nyb, x0, y0, z0, b, bnx, bny, bx0, by0, bz0, nx, ny, nz);
    else
        k_box<<<blocks, 256, 0, h->stream>>>(b, bnx, bny, bx0, by0, bz0, h->W, h->d.nxb, h->d.nyb, x0, y0, z0, nx, ny, nz);
    CK(h, cudaGetLastError());
    CK(h, cudaStreamSynchronize(h->stream));
    return OSE_OK;
}

namespace {

// P of the state -> snap (the source wavefield of reverse-time migration).
__global__ void k_take_p(const float2* __restrict__ W, float* __restrict__ snap, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        snap[i] = W[i].x;
}

// Reverse-time injection of one gather row at the receivers (the cells the
// LAST epilogue records): P += p[ig], Q += q[ig].
__global__ void k_inject_row(float2* __restrict__ W, const float* __restrict__ p, const float* __restrict__ q, int gz,
                             int bl, int bf, int nx, int ny, int nxb, int nyb, const long long* __restrict__ idx, int ng)
{
    const int ig = blockIdx.x * blockDim.x + threadIdx.x;
    if (ig >= ng) return;
    const int iy = ig / nx, ix = ig - iy * nx;
    float2& w = W[idx ? idx[ig] : ((size_t)gz * nyb + (bf + iy)) * nxb + (bl + ix)];
    w.x += p[ig];
    w.y += q[ig];
}

// Zero-lag cross-correlation imaging condition: image += P_source * P_receiver,
// and the source illumination ill += P_source^2.
__global__ void k_image(float* __restrict__ img, float* __restrict__ ill, const float* __restrict__ snap,
                        const float2* __restrict__ W, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float s = snap[i];
        img[i] = fmaf(s, W[i].x, img[i]);
        ill[i] = fmaf(s, s, ill[i]);
    }
}

// In-place radix-2 FFT of length n (a power of two), sign -1 forward.
void fft_pow2(std::vector<std::complex<double>>& a, int sign)
{
    const size_t n = a.size();
    for (size_t i = 1, j = 0; i < n; ++i) {
        size_t bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) std::swap(a[i], a[j]);
    }
    const double pi = 3.14159265358979323846;
    for (size_t len = 2; len <= n; len <<= 1) {
        const std::complex<double> wl(cos(2 * pi / (double)len), sign * sin(2 * pi / (double)len));
        for (size_t i = 0; i < n; i += len) {
            std::complex<double> w(1.0, 0.0);
            for (size_t k = 0; k < len / 2; ++k) {
                const std::complex<double> u = a[i + k], v = a[i + k + len / 2] * w;
                a[i + k] = u + v;
                a[i + k + len / 2] = u - v;
                w *= wl;
            }
        }
    }
}

// Hilbert transform of every receiver trace of rows [nsteps][ng] (zero padded
// to a power of two >= 2 nsteps, so the transform does not wrap around):
// h = IFFT(-i sgn(f) FFT(d)).  Spread over the host threads.
void hilbert_rows(const float* rows, int nsteps, int ng, std::vector<float>& out)
{
    out.assign((size_t)nsteps * ng, 0.f);
    size_t L = 1;
    while (L < 2 * (size_t)nsteps) L <<= 1;
    const int nth = std::max(1, std::min(16, (int)std::thread::hardware_concurrency()));
    auto work = [&](int t0) {
        std::vector<std::complex<double>> a(L);
        for (int ig = t0; ig < ng; ig += nth) {
            for (size_t i = 0; i < L; ++i) a[i] = i < (size_t)nsteps ? rows[i * ng + ig] : 0.0;
            fft_pow2(a, -1);
            for (size_t k = 0; k < L; ++k) {
                if (k == 0 || k == L / 2) a[k] = 0.0;
                else if (k < L / 2) a[k] *= std::complex<double>(0.0, -1.0);
                else a[k] *= std::complex<double>(0.0, 1.0);
            }
            fft_pow2(a, +1);
            for (int i = 0; i < nsteps; ++i) out[(size_t)i * ng + ig] = (float)(a[i].real() / (double)L);
        }
    };
    std::vector<std::thread> th;
    for (int t = 0; t < nth; ++t) th.emplace_back(work, t);
    for (auto& x : th) x.join();
}

}  // namespace

ose_status ose_rtm(ose_handle* h, const float* rows, int nsteps, int every, float* image, float* illum)
{
    if (!h || !rows || !image || nsteps < 1 || every < 1) return OSE_ERR_INVALID;
    if (nsteps > h->p.nt) return fail(h, OSE_ERR_INVALID, "nsteps beyond nt");
    const size_t N = (size_t)h->g.ncell;
    const int ng = h->d.ng;
    const int nsnap = nsteps / every + 1;
    size_t free_b = 0, total_b = 0;
    CK(h, cudaMemGetInfo(&free_b, &total_b));
    const size_t need = sizeof(float) * (N * (size_t)(nsnap + 2) + 2 * (size_t)nsteps * ng);
    if (need + ((size_t)1 << 30) > free_b)
        return fail(h, OSE_ERR_NOMEM, "reverse-time migration needs " + std::to_string(need >> 20) +
                                          " MiB of device memory for its snapshots");
    std::vector<float> hil;
    hilbert_rows(rows, nsteps, ng, hil);
    // The step is W(t + dt) = exp(-i v|k| dt) W(t), so a free wave has
    // P = H[Q] along time (H: the Hilbert transform, -i on positive
    // frequencies).  The receivers record Q = d, hence P = h = H[d].  Run
    // backwards, W_rev(tau) = conj(W(T - tau)) obeys the same step with the
    // source -conj(P + iQ): inject P += -h(t), Q += +d(t) at t = T - tau.
    // (Checked by refocusing a recorded point source at its position.)
    std::vector<float> pin((size_t)nsteps * ng), qin((size_t)nsteps * ng);
    for (size_t i = 0; i < pin.size(); ++i) {
        pin[i] = -hil[i];
        qin[i] = rows[i];
    }
    float *snaps = nullptr, *img = nullptr, *ill = nullptr, *dp = nullptr, *dq = nullptr;
    auto release = [&] {
        for (float* b : {snaps, img, ill, dp, dq})
            if (b) cudaFree(b);
    };
#define CKR(call)                                                    \
    do {                                                             \
        cudaError_t e_ = (call);                                     \
        if (e_ != cudaSuccess) { release(); return cuda_fail(h, e_, #call); } \
    } while (0)
    CKR(cudaMalloc((void**)&snaps, sizeof(float) * N * nsnap));
    CKR(cudaMalloc((void**)&img, sizeof(float) * N));
    CKR(cudaMalloc((void**)&ill, sizeof(float) * N));
    CKR(cudaMemsetAsync(ill, 0, sizeof(float) * N, h->stream));
    CKR(cudaMalloc((void**)&dp, sizeof(float) * pin.size()));
    CKR(cudaMalloc((void**)&dq, sizeof(float) * qin.size()));
    CKR(cudaMemcpyAsync(dp, pin.data(), sizeof(float) * pin.size(), cudaMemcpyHostToDevice, h->stream));
    CKR(cudaMemcpyAsync(dq, qin.data(), sizeof(float) * qin.size(), cudaMemcpyHostToDevice, h->stream));
    CKR(cudaMemsetAsync(img, 0, sizeof(float) * N, h->stream));
    CKR(cudaMemsetAsync(snaps, 0, sizeof(float) * N, h->stream));   // time 0: at rest
    const unsigned blocks = (unsigned)std::min<size_t>(8192, (N + 255) / 256);
    // forward: the source wavefield, P kept every `every` steps
    ose_status st = ose_reset_shot(h, h->shot >= 0 ? h->shot : 0);
    if (st != OSE_OK) { release(); return st; }
    st = build_graph(h);
    if (st != OSE_OK) { release(); return st; }
    for (int it = 0; it < nsteps; ++it) {
        CKR(cudaGraphLaunch(h->graph, h->stream));
        if ((it + 1) % every == 0)
            k_take_p<<<blocks, 256, 0, h->stream>>>(h->W, snaps + N * (size_t)((it + 1) / every), (long long)N);
    }
    // backward: receiver wavefield from the time-reversed rows, no source, no recording
    CKR(cudaMemsetAsync(h->W, 0, sizeof(float2) * N, h->stream));
    const int no_record[2] = {0, -1};
    CKR(cudaMemcpyAsync(h->ctr, no_record, sizeof(no_record), cudaMemcpyHostToDevice, h->stream));
    const int gz = h->p.bu + h->p.gzbeg;
    for (int it = nsteps - 1; it >= 0; --it) {
        k_inject_row<<<(ng + 255) / 256, 256, 0, h->stream>>>(h->W, dp + (size_t)it * ng, dq + (size_t)it * ng, gz,
                                                                h->p.bl, h->p.bf, h->p.nx, h->p.ny, h->d.nxb, h->d.nyb,
                                                                h->rec_xyz.empty() ? nullptr : h->rec_idx, ng);
        CKR(enqueue_step(h, nullptr, false));
        if (it % every == 0)
            k_image<<<blocks, 256, 0, h->stream>>>(img, ill, snaps + N * (size_t)(it / every), h->W, (long long)N);
    }
    CKR(cudaGetLastError());
    CKR(cudaMemcpyAsync(image, img, sizeof(float) * N, cudaMemcpyDeviceToHost, h->stream));
    if (illum) CKR(cudaMemcpyAsync(illum, ill, sizeof(float) * N, cudaMemcpyDeviceToHost, h->stream));
    CKR(cudaStreamSynchronize(h->stream));
#undef CKR
    release();
    // the state now holds the receiver wavefield: a new shot must be started
    h->shot_ready = false;
    h->it = 0;
    return tensor_status(h);
}

ose_status ose_get_it(const ose_handle* h, int* it)
{
    if (!h || !it) return OSE_ERR_INVALID;
    *it = h->it;
    return OSE_OK;
}

ose_status ose_get_gather(ose_handle* h, float* out)
{
    if (!h || !out) return OSE_ERR_INVALID;
    const int nt = h->p.nt, ng = h->d.ng;
    std::vector<float> g((size_t)nt * ng);
    CK(h, cudaMemcpyAsync(g.data(), h->gather, sizeof(float) * g.size(), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    for (int it = 0; it < nt; ++it)        // [it][ig] -> [ig][it] (ose_3d_lib.cu:327-343)
        for (int ig = 0; ig < ng; ++ig) out[(size_t)ig * nt + it] = g[(size_t)it * ng + ig];
    return OSE_OK;
}

ose_status ose_get_wavefield(ose_handle* h, int which, float* out, int layout)
{
    if (!h || !out) return OSE_ERR_INVALID;
    if (layout != OSE_LAYOUT_ZYX && layout != OSE_LAYOUT_YXZ) return fail(h, OSE_ERR_INVALID, "bad layout");
    const size_t N = (size_t)h->g.ncell;
    if (which == OSE_FIELD_V) {
        to_layout(h, padded_model(h).data(), out, layout);
        return OSE_OK;
    }
    if (which != OSE_FIELD_P && which != OSE_FIELD_Q) return fail(h, OSE_ERR_INVALID, "bad field");
    // one component, deinterleaved on the device into the scratch spectrum
    // buffer (free between steps), then one copy of N floats
    float* comp = reinterpret_cast<float*>(h->X);
    k_take_component<<<4096, 256, 0, h->stream>>>(h->W, comp, (long long)N, which == OSE_FIELD_Q);
    CK(h, cudaGetLastError());
    if (layout == OSE_LAYOUT_ZYX) {
        CK(h, cudaMemcpyAsync(out, comp, sizeof(float) * N, cudaMemcpyDeviceToHost, h->stream));
        CK(h, cudaStreamSynchronize(h->stream));
        return OSE_OK;
    }
    std::vector<float> zyx(N);
    CK(h, cudaMemcpyAsync(zyx.data(), comp, sizeof(float) * N, cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    to_layout(h, zyx.data(), out, layout);
    return OSE_OK;
}

ose_status ose_set_wavefield(ose_handle* h, int which, const float* in, int layout)
{
    if (!h || !in) return OSE_ERR_INVALID;
    if (which != OSE_FIELD_P && which != OSE_FIELD_Q) return fail(h, OSE_ERR_INVALID, "only P or Q can be set");
    if (layout != OSE_LAYOUT_ZYX && layout != OSE_LAYOUT_YXZ) return fail(h, OSE_ERR_INVALID, "bad layout");
    const size_t N = (size_t)h->g.ncell;
    std::vector<float> zyx(N);
    from_layout(h, in, zyx.data(), layout);
    std::vector<float2> w(N);
    CK(h, cudaMemcpyAsync(w.data(), h->W, sizeof(float2) * N, cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    for (size_t i = 0; i < N; ++i) (which == OSE_FIELD_P ? w[i].x : w[i].y) = zyx[i];
    CK(h, cudaMemcpyAsync(h->W, w.data(), sizeof(float2) * N, cudaMemcpyHostToDevice, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    return OSE_OK;
}

ose_status ose_get_wavelets(const ose_handle* h, float* ricker, float* hilbert)
{
    if (!h) return OSE_ERR_INVALID;
    if (!h->shot_ready) return OSE_ERR_STATE;
    if (ricker) memcpy(ricker, h->h_ricker.data(), sizeof(float) * h->p.nt);
    if (hilbert) memcpy(hilbert, h->h_hil.data(), sizeof(float) * h->p.nt);
    return OSE_OK;
}

ose_status ose_get_sponge(const ose_handle* h, float* ax, float* ay, float* az)
{
    if (!h) return OSE_ERR_INVALID;
    if (ax) memcpy(ax, h->h_ax.data(), sizeof(float) * h->h_ax.size());
    if (ay) memcpy(ay, h->h_ay.data(), sizeof(float) * h->h_ay.size());
    if (az) memcpy(az, h->h_az.data(), sizeof(float) * h->h_az.size());
    return OSE_OK;
}

ose_status ose_apply_operator(ose_handle* h, const float* in, float* out)
{
    if (!h || !in || !out) return OSE_ERR_INVALID;
    const size_t N = (size_t)h->g.ncell;
    // A and S carry no state between steps, so they serve as in/out here.
    CK(h, cudaMemcpyAsync(h->A, in, sizeof(float2) * N, cudaMemcpyHostToDevice, h->stream));
    if (h->d.path == OSE_PATH_PLANE)
        CK(h, ose::launch_plane_apply_operator(h->stream, h->A, h->X, h->S, h->vs, h->sch, h->scl, h->tables));
    else
        CK(h, ose::launch_apply_operator(h->stream, h->g, h->px, h->py, h->pz, h->tables, h->A, h->X, h->S, h->vs,
                                         h->sch, h->scl));
    CK(h, cudaMemcpyAsync(out, h->S, sizeof(float2) * N, cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    return tensor_status(h);
}

ose_status ose_profile_step(ose_handle* h, int reps, int cap, int* count, const char** names,
                            float* ms, double* bytes, int* launches)
{
    if (!h || !count || reps < 1) return OSE_ERR_INVALID;
    if (!h->shot_ready) return fail(h, OSE_ERR_STATE, "ose_reset_shot must come first");
    if (h->it + reps > h->p.nt) return fail(h, OSE_ERR_INVALID, "reps beyond nt");
    ose::KernelTiming& t = h->timing;
    // class 8: the epilogue passes that leave the partial sum alone (SumPlan)
    static const char* kGeneric[] = {"fft_x_fwd", "fft_y_fwd", "fft_z_kscale", "fft_y_inv",
                                     "fft_x_inv_epilogue", "inject", "corrector_scale", "corrector",
                                     "fft_x_inv_epilogue_nosum", "unused"};
    static const char* kPlane[] = {"plane_fwd", "zpass", "plane_inv_first", "plane_inv_mid",
                                   "plane_inv_last", "inject", "corrector_scale", "corrector",
                                   "plane_inv_mid_nosum", "plane_inv_mid_sumstart"};
    const char** kNames = h->d.path == OSE_PATH_PLANE ? kPlane : kGeneric;
    for (int c = 0; c < ose::KernelTiming::kClasses; ++c) { t.ms[c] = 0.f; t.count[c] = 0; t.bytes[c] = 0.0; }
    for (int r = 0; r < reps; ++r) {
        CK(h, enqueue_step(h, &t));
        CK(h, cudaStreamSynchronize(h->stream));
        h->it += 1;
    }
    // the classes that launched (inject always, the corrector when set)
    int nc = 0;
    for (int c = 0; c < ose::KernelTiming::kClasses; ++c) {
        if (!t.count[c] && c != 5) continue;
        if (nc < cap) {
            if (names) names[nc] = kNames[c];
            if (ms) ms[nc] = t.count[c] ? t.ms[c] / t.count[c] : 0.f;
            if (bytes) bytes[nc] = t.count[c] ? t.bytes[c] / t.count[c] : 0.0;
            if (launches) launches[nc] = t.count[c] / reps;
        }
        ++nc;
    }
    *count = nc;
    return OSE_OK;
}

ose_status ose_write_outputs(ose_handle* h, const char* gather_path, const char* par_path)
{
    if (!h) return OSE_ERR_INVALID;
    const ose_params& p = h->p;
    if (gather_path) {
        std::vector<float> g((size_t)p.nt * h->d.ng);
        ose_status s = ose_get_gather(h, g.data());
        if (s != OSE_OK) return s;
        FILE* f = fopen(gather_path, "wb");
        if (!f) return fail(h, OSE_ERR_IO, std::string("cannot write ") + gather_path);
        size_t w = fwrite(g.data(), sizeof(float), g.size(), f);
        fclose(f);
        if (w != g.size()) return fail(h, OSE_ERR_IO, std::string("short write ") + gather_path);
    }
    if (par_path) {
        // output_par (ose_3d_lib.cu:255-319): label line, value line, same labels
        FILE* f = fopen(par_path, "wb");
        if (!f) return fail(h, OSE_ERR_IO, std::string("cannot write ") + par_path);
        struct { const char* label; int iv; float fv; bool is_f; } rows[] = {
            {"X dimension size----> nx\n", p.nx, 0, false},
            {"Y dimension size----> ny\n", p.ny, 0, false},
            {"Z dimension size----> ny\n", p.nz, 0, false},
            {"The interval of samples in space domain X dimension ----> dx (the units is 'mile')\n", 0, p.dx, true},
            {"The interval of samples in space domain Y dimension ----> dy (the units is 'mile')\n", 0, p.dy, true},
            {"The interval of samples in space domain Z dimension ----> dz (the units is 'mile')\n", 0, p.dz, true},
            {"The number of samples in time domain ----> nt\n", p.nt, 0, false},
            {"The number of receivers gather ----> ng\n", h->d.ng, 0, false},
            {"The number of sources ----> ns\n", p.nshot, 0, false},
            {"The interval of samples in time domain (the units is 's') ----> dt\n", 0, p.dt, true},
            {"The amplitude of wavelet ----> amp\n", 0, p.amp, true},
            {"The main frequency of wavelet ----> fm\n", 0, p.fm, true},
            {"The beginning location of sources in X-axis ----> sxbeg\n", p.sxbeg, 0, false},
            {"The beginning location of sources in Y-axis ----> sxbeg\n", p.sybeg, 0, false},
            {"The beginning location of sources in Z-axis ----> szbeg\n", p.szbeg, 0, false},
            {"The beginning location of receivers in X-axis ----> gxbeg\n", p.gxbeg, 0, false},
            {"The beginning location of receivers in Y-axis ----> gybeg\n", p.gybeg, 0, false},
            {"The beginning location of receivers in Z-axis ----> gzbeg\n", p.gzbeg, 0, false},
            {"Sources X-axis  jump interval ----> jsx\n", p.jsx, 0, false},
            {"Sources Y-axis  jump interval ----> jsy\n", p.jsy, 0, false},
            {"Sources Z-axis  jump interval ----> jsz\n", p.jsz, 0, false},
            {"Receivers X-axis  jump interval ----> jgx\n", p.jgx, 0, false},
            {"Receivers Y-axis  jump interval ----> jgy\n", p.jgy, 0, false},
            {"Receivers Z-axis  jump interval ----> jgzn", p.jgz, 0, false},
            {"Default, common shot-gather; if n, record at every point\n", p.csdgather, 0, false},
        };
        for (auto& r : rows) {
            fputs(r.label, f);
            if (r.is_f) fprintf(f, "%f\n", r.fv);
            else fprintf(f, "%d\n", r.iv);
        }
        fclose(f);
    }
    return OSE_OK;
}

/* ---- checkpoint / resume ------------------------------------------------- */

namespace {
const char kCkMagic[8] = {'O', 'S', 'E', '3', 'D', 'C', 'K', '1'};
struct CkHeader {
    char magic[8];
    int32_t version, params_bytes;
    int32_t nxb, nyb, nzb, nt, ng, shot, it;
};
}  // namespace

ose_status ose_checkpoint_save(ose_handle* h, const char* path)
{
    if (!h || !path) return OSE_ERR_INVALID;
    if (!h->shot_ready) return fail(h, OSE_ERR_STATE, "ose_reset_shot must come first");
    const size_t N = (size_t)h->g.ncell;
    std::vector<float2> w(N);
    std::vector<float> g((size_t)h->it * h->d.ng);
    CK(h, cudaMemcpyAsync(w.data(), h->W, sizeof(float2) * N, cudaMemcpyDeviceToHost, h->stream));
    if (!g.empty())
        CK(h, cudaMemcpyAsync(g.data(), h->gather, sizeof(float) * g.size(), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    CkHeader hd;
    memcpy(hd.magic, kCkMagic, 8);
    hd.version = 1;
    hd.params_bytes = (int32_t)sizeof(ose_params);
    hd.nxb = h->d.nxb; hd.nyb = h->d.nyb; hd.nzb = h->d.nzb;
    hd.nt = h->p.nt; hd.ng = h->d.ng; hd.shot = h->shot; hd.it = h->it;
    FILE* f = fopen(path, "wb");
    if (!f) return fail(h, OSE_ERR_IO, std::string("cannot write ") + path);
    bool ok = fwrite(&hd, sizeof hd, 1, f) == 1 && fwrite(&h->p, sizeof(ose_params), 1, f) == 1 &&
              fwrite(w.data(), sizeof(float2), N, f) == N &&
              (g.empty() || fwrite(g.data(), sizeof(float), g.size(), f) == g.size());
    if (fclose(f) != 0) ok = false;
    return ok ? OSE_OK : fail(h, OSE_ERR_IO, std::string("short write ") + path);
}

ose_status ose_checkpoint_load(ose_handle* h, const char* path)
{
    if (!h || !path) return OSE_ERR_INVALID;
    FILE* f = fopen(path, "rb");
    if (!f) return fail(h, OSE_ERR_IO, std::string("cannot open ") + path);
    CkHeader hd;
    ose_params p;
    bool ok = fread(&hd, sizeof hd, 1, f) == 1;
    if (!ok || memcmp(hd.magic, kCkMagic, 8) != 0 || hd.version != 1 || hd.params_bytes != (int32_t)sizeof(ose_params)) {
        fclose(f);
        return fail(h, OSE_ERR_IO, std::string("not an ose3d checkpoint: ") + path);
    }
    ok = fread(&p, sizeof p, 1, f) == 1;
    if (!ok || memcmp(&p, &h->p, sizeof p) != 0 || hd.nxb != h->d.nxb || hd.nyb != h->d.nyb ||
        hd.nzb != h->d.nzb || hd.it < 0 || hd.it > h->p.nt) {
        fclose(f);
        return fail(h, OSE_ERR_INVALID, "checkpoint was written with other parameters");
    }
    const size_t N = (size_t)h->g.ncell;
    std::vector<float2> w(N);
    std::vector<float> g((size_t)hd.it * h->d.ng);
    ok = fread(w.data(), sizeof(float2), N, f) == N &&
         (g.empty() || fread(g.data(), sizeof(float), g.size(), f) == g.size());
    fclose(f);
    if (!ok) return fail(h, OSE_ERR_IO, std::string("truncated checkpoint ") + path);
    ose_status st = prepare_shot(h, hd.shot);
    if (st != OSE_OK) return st;
    CK(h, cudaMemcpyAsync(h->W, w.data(), sizeof(float2) * N, cudaMemcpyHostToDevice, h->stream));
    CK(h, cudaMemsetAsync(h->gather, 0, sizeof(float) * (size_t)h->p.nt * h->d.ng, h->stream));
    if (!g.empty())
        CK(h, cudaMemcpyAsync(h->gather, g.data(), sizeof(float) * g.size(), cudaMemcpyHostToDevice, h->stream));
    int ctr[4] = {hd.it, hd.it > 0 ? hd.it - 1 : 0, 0, 0};
    CK(h, cudaMemcpyAsync(h->ctr, ctr, sizeof ctr, cudaMemcpyHostToDevice, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    h->it = hd.it;
    h->shot_ready = true;
    return OSE_OK;
}

/* ---- snapshots ------------------------------------------------------------ */

ose_status ose_run_snapshots(ose_handle* h, int nsteps, int every, int layout, ose_snapshot_fn fn, void* user)
{
    if (!h || !fn || every < 1 || nsteps < 0) return OSE_ERR_INVALID;
    if (layout != OSE_LAYOUT_ZYX && layout != OSE_LAYOUT_YXZ) return fail(h, OSE_ERR_INVALID, "bad layout");
    if (!h->shot_ready) return fail(h, OSE_ERR_STATE, "ose_reset_shot must come first");
    if (h->it + nsteps > h->p.nt) return fail(h, OSE_ERR_INVALID, "nsteps beyond nt");
    const size_t N = (size_t)h->g.ncell;
    if (!h->Wsnap) {
        CK(h, dalloc(h, &h->Wsnap, N));
        for (int b = 0; b < 2; ++b) {
            CK(h, cudaMallocHost((void**)&h->hsnap[b], sizeof(float2) * N));
            CK(h, cudaEventCreateWithFlags(&h->snap_done[b], cudaEventDisableTiming));
        }
        CK(h, cudaEventCreateWithFlags(&h->snap_ready, cudaEventDisableTiming));
        CK(h, cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking));
    }
    ose_status st = build_graph(h);
    if (st != OSE_OK) return st;
    const int K = (nsteps + every - 1) / every;
    std::vector<int> its(K);
    std::vector<float> P(N), Q(N), tmp(N);
    // batch k: its steps, then W -> Wsnap (device) and Wsnap -> hsnap[k % 2] on
    // the copy stream; the host hands snapshot k to fn while batch k+1 runs.
    auto enqueue = [&](int k) -> ose_status {
        const int n = std::min(every, nsteps - k * every);
        for (int i = 0; i < n; ++i) CK(h, cudaGraphLaunch(h->graph, h->stream));
        h->it += n;
        its[k] = h->it - 1;
        if (k > 0) CK(h, cudaStreamWaitEvent(h->stream, h->snap_done[(k - 1) % 2], 0));
        CK(h, cudaMemcpyAsync(h->Wsnap, h->W, sizeof(float2) * N, cudaMemcpyDeviceToDevice, h->stream));
        CK(h, cudaEventRecord(h->snap_ready, h->stream));
        CK(h, cudaStreamWaitEvent(h->copy_stream, h->snap_ready, 0));
        CK(h, cudaMemcpyAsync(h->hsnap[k % 2], h->Wsnap, sizeof(float2) * N, cudaMemcpyDeviceToHost,
                              h->copy_stream));
        CK(h, cudaEventRecord(h->snap_done[k % 2], h->copy_stream));
        return OSE_OK;
    };
    if (K > 0 && (st = enqueue(0)) != OSE_OK) return st;
    for (int k = 0; k < K; ++k) {
        if (k + 1 < K && (st = enqueue(k + 1)) != OSE_OK) return st;
        CK(h, cudaEventSynchronize(h->snap_done[k % 2]));
        const float2* w = h->hsnap[k % 2];
        for (size_t i = 0; i < N; ++i) { P[i] = w[i].x; Q[i] = w[i].y; }
        if (layout == OSE_LAYOUT_YXZ) {
            to_layout(h, P.data(), tmp.data(), layout);
            P.swap(tmp);
            to_layout(h, Q.data(), tmp.data(), layout);
            Q.swap(tmp);
        }
        fn(its[k], P.data(), Q.data(), user);
    }
    CK(h, cudaStreamSynchronize(h->stream));
    return OSE_OK;
}

/* ---- SU / SEG-Y ------------------------------------------------------------ */

static ose_status write_traces(ose_handle* h, const char* path, bool segy)
{
    if (!h || !path) return OSE_ERR_INVALID;
    if (!h->shot_ready) return fail(h, OSE_ERR_STATE, "ose_reset_shot must come first");
    const ose_params& p = h->p;
    std::vector<float> g((size_t)p.nt * h->d.ng);
    ose_status st = ose_get_gather(h, g.data());
    if (st != OSE_OK) return st;
    ose::TraceGeometry tg{};
    tg.ng = h->d.ng;
    tg.nt = p.nt;
    tg.nx = p.nx;
    tg.shot = h->shot;
    tg.dx = p.dx;
    tg.dy = p.dy;
    tg.sx = (double)(p.sxbeg + h->shot * p.jsx) * p.dx;
    tg.sy = (double)(p.sybeg + h->shot * p.jsy) * p.dy;
    tg.sz = (double)(p.szbeg + h->shot * p.jsz) * p.dz;
    tg.gz = (double)p.gzbeg * p.dz;
    tg.dt_us = (int)lround((double)p.dt * 1e6);
    tg.rxyz = h->rec_xyz.empty() ? nullptr : h->rec_xyz.data();
    tg.dz = p.dz;
    const int rc = ose::write_gather_traces(path, g.data(), tg, segy);
    if (rc == -2) return fail(h, OSE_ERR_UNSUPPORTED, "nt or dt does not fit the 16-bit trace header fields");
    if (rc != 0) return fail(h, OSE_ERR_IO, std::string("cannot write ") + path);
    return OSE_OK;
}

ose_status ose_write_su(ose_handle* h, const char* path) { return write_traces(h, path, false); }
ose_status ose_write_segy(ose_handle* h, const char* path) { return write_traces(h, path, true); }

}  // extern "C"
