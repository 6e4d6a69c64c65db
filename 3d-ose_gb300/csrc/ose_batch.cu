// ose_batch.cu - many shots, each on its own window of a larger model, advanced
// together: every pass of a time step is one launch across all shots (the
// batched kernels of ose_kernels.cu), and the whole step is one CUDA graph.
//
// The reference runs its shots one after another on the full model
// (for(is...) in ose_3d.cu:242-279); here each shot gets a window around its
// source cut from the model (edge cells replicated where the window leaves
// the model), its own sponge, series order and tables, and all windows of
// the batch share the device.  ose_batch_autotune picks the tile widths and
// radix orders by timing candidates on the batch and caches the choice.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <string>
#include <vector>

#include "ose_internal.h"

namespace {

struct ShotHost {
    ose_params p;          // window parameters (nx, ny, nz = window interior)
    ose_derived d;
    ose::AxisPlan px, py, pz;
    std::vector<float> vb;
    std::vector<double> J;
    long long src = 0;
    size_t off = 0;        // first byte of the shot in the arena
};

}  // namespace

struct ose_batch {
    ose_params base{};
    int nshots = 0;
    int Mmax = 0;
    std::vector<ShotHost> shots;
    std::vector<ose::BatchShot> desc;      // host copy of the device descriptors
    ose::BatchShot* d_shots = nullptr;
    int2* d_work = nullptr;
    size_t work_cap = 0;
    std::vector<ose::BatchPass> passes;    // every pass of every application, in launch order
    char* arena = nullptr;
    size_t arena_bytes = 0;
    cudaStream_t stream = nullptr;
    cudaGraphExec_t graph = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    int it = 0;
    int rows_scale = 2048, txy = 16, txz = 16, radix_order = 0;   // tunables of the Stockham kernels
    int group_mb = 0;      // shots per group: working set up to this many MB (0: one group)
    // lanes = 0: batched launches (one per pass and length class).  lanes = k
    // > 0: every shot's own single-shot launches, shots spread round-robin
    // over k streams that run concurrently inside the captured step.
    // lanes = -1: the whole step (after the source injection) as one
    // persistent cooperative launch over the batched passes, grid barriers
    // between passes (ose_cols.cu kb_persistent).
    int lanes = 0;
    static constexpr int kMaxLanes = 8;
    ose::PersistPass* d_ppass = nullptr;
    int nppass = 0;
    size_t ppass_cap = 0;
    bool persist_ok = false;   // every pass of the batch has a persistent kernel
    unsigned* d_bar = nullptr; // [0] arrivals, [1] generation, [2] error word
    int pgrid = 0;
    cudaStream_t lane[kMaxLanes] = {};
    cudaEvent_t fork = nullptr, join[kMaxLanes] = {};
    std::string err;
};

namespace {

std::string g_batch_create_error;

ose_status bfail(ose_batch* b, ose_status s, const std::string& m)
{
    if (b) b->err = m;
    else g_batch_create_error = m;
    return s;
}

#define BCK(b, call)                                                                   \
    do {                                                                               \
        cudaError_t e_ = (call);                                                       \
        if (e_ != cudaSuccess)                                                         \
            return bfail((b), OSE_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// radix order variants: 0 = 4s first (plan_axis), 1 = 2s and odd radices first
void order_plan(ose::AxisPlan& pl, int variant)
{
    if (variant == 1) std::reverse(pl.radix, pl.radix + pl.ns);
}

void fill_descriptors(ose_batch* b)
{
    for (int s = 0; s < b->nshots; ++s) {
        const ShotHost& sh = b->shots[s];
        ose::BatchShot& D = b->desc[s];
        D.px = sh.px;
        D.py = sh.py;
        D.pz = sh.pz;
        order_plan(D.px, b->radix_order);
        order_plan(D.py, b->radix_order);
        order_plan(D.pz, b->radix_order);
        D.rpc = std::max(1, b->rows_scale / sh.d.nxb);
        D.txy = b->txy;
        D.txz = b->txz;
    }
}

// Work lists.  The shots are cut into groups whose working set (36 bytes per
// cell: W, A, S, X, v) stays within group_mb MB, so that a group's fields can
// stay in L2 through its whole step (0: all shots in one group).  For each
// group, every application n runs five passes (x forward, y forward, z,
// y inverse, x inverse + update), each split by the axis length of the
// group's shots: one launch per length the register kernels have
// (ose_cols.cu), one launch of the Stockham kernels for all other lengths.
ose_status build_passes(ose_batch* b)
{
    std::vector<int2> all;
    struct Range { size_t off, count, smem; int kind, n_axis, n; };
    std::vector<Range> ranges;
    b->passes.clear();
    std::vector<std::vector<int>> groups(1);
    double gbytes = 0.0;
    for (int s = 0; s < b->nshots; ++s) {
        const ose::Geometry& g = b->desc[s].g;
        const double sb = 36.0 * (double)g.nxb * g.nyb * g.nzb;
        if (b->group_mb > 0 && !groups.back().empty() && gbytes + sb > b->group_mb * 1048576.0) {
            groups.emplace_back();
            gbytes = 0.0;
        }
        groups.back().push_back(s);
        gbytes += sb;
    }
    for (const std::vector<int>& grp : groups) {
        int Mg = 0;
        for (int s : grp) Mg = std::max(Mg, b->desc[s].M);
        for (int n = 0; n <= Mg; ++n) {
            for (int kind = 0; kind < 5; ++kind) {
                auto axis_len = [&](const ose::BatchShot& D) {
                    return kind == 0 || kind == 4 ? D.g.nxb : (kind == 2 ? D.g.nzb : D.g.nyb);
                };
                std::vector<int> lens;   // register classes present, 0 = Stockham
                for (int s : grp) {
                    const ose::BatchShot& D = b->desc[s];
                    if (D.M < n) continue;
                    const int L = ose::col_supported(axis_len(D)) ? axis_len(D) : 0;
                    if (std::find(lens.begin(), lens.end(), L) == lens.end()) lens.push_back(L);
                }
                std::sort(lens.begin(), lens.end(), [](int a, int c) { return a > c; });
                for (int L : lens) {
                    const size_t off = all.size();
                    size_t sm = 0;
                    for (int s : grp) {
                        const ose::BatchShot& D = b->desc[s];
                        if (D.M < n) continue;
                        const int len = axis_len(D);
                        if ((ose::col_supported(len) ? len : 0) != L) continue;
                        long long nb;
                        if (L > 0) {
                            if (kind == 0 || kind == 4)
                                nb = ((long long)D.g.nyb * D.g.nzb + ose::row_tile(L) - 1) / ose::row_tile(L);
                            else
                                nb = (long long)((D.g.nxb + ose::col_tile(L) - 1) / ose::col_tile(L)) *
                                     (kind == 2 ? D.g.nyb : D.g.nzb);
                        } else if (kind == 0 || kind == 4) {
                            nb = ((long long)D.g.nyb * D.g.nzb + D.rpc - 1) / D.rpc;
                            sm = std::max(sm, ose::batch_rows_smem(D.g.nxb, D.rpc));
                        } else if (kind == 2) {
                            nb = (long long)(D.g.nxb + D.txz - 1) / D.txz * D.g.nyb;
                            sm = std::max(sm, ose::batch_lines_smem(D.g.nzb, D.txz));
                        } else {
                            nb = (long long)(D.g.nxb + D.txy - 1) / D.txy * D.g.nzb;
                            sm = std::max(sm, ose::batch_lines_smem(D.g.nyb, D.txy));
                        }
                        for (long long k = 0; k < nb; ++k) all.push_back(make_int2(s, (int)k));
                    }
                    if (sm > 227 * 1024) return bfail(b, OSE_ERR_UNSUPPORTED, "a tile does not fit shared memory");
                    ranges.push_back({off, all.size() - off, sm, kind, L, n});
                }
            }
        }
    }
    if (all.size() > b->work_cap) {
        if (b->d_work) cudaFree(b->d_work);
        b->d_work = nullptr;
        BCK(b, cudaMalloc((void**)&b->d_work, sizeof(int2) * all.size()));
        b->work_cap = all.size();
    }
    BCK(b, cudaMemcpyAsync(b->d_work, all.data(), sizeof(int2) * all.size(), cudaMemcpyHostToDevice, b->stream));
    BCK(b, cudaMemcpyAsync(b->d_shots, b->desc.data(), sizeof(ose::BatchShot) * b->nshots,
                           cudaMemcpyHostToDevice, b->stream));
    BCK(b, cudaStreamSynchronize(b->stream));
    for (const Range& r : ranges)
        b->passes.push_back({b->d_work + r.off, (int)r.count, r.smem, r.kind, r.n_axis, r.n});
    // the same passes for the persistent launch: a grid barrier after the
    // last length class of every (group, application, kind)
    b->persist_ok = !ranges.empty();
    std::vector<ose::PersistPass> pp;
    for (size_t i = 0; i < ranges.size(); ++i) {
        const Range& r = ranges[i];
        if (!ose::persist_supported(r.n_axis)) b->persist_ok = false;
        const bool last = i + 1 == ranges.size() || ranges[i + 1].kind != r.kind || ranges[i + 1].n != r.n ||
                          ranges[i + 1].off < r.off;
        pp.push_back({b->d_work + r.off, (int)r.count, r.kind, r.n_axis, r.n, last ? 1 : 0});
    }
    // a new group restarts at application 0, kind 0: that change of (n, kind)
    // already puts a barrier between groups
    if (b->persist_ok) {
        if (pp.size() > b->ppass_cap) {
            if (b->d_ppass) cudaFree(b->d_ppass);
            b->d_ppass = nullptr;
            BCK(b, cudaMalloc((void**)&b->d_ppass, sizeof(ose::PersistPass) * pp.size()));
            b->ppass_cap = pp.size();
        }
        BCK(b, cudaMemcpy(b->d_ppass, pp.data(), sizeof(ose::PersistPass) * pp.size(), cudaMemcpyHostToDevice));
        b->nppass = (int)pp.size();
        if (!b->d_bar) {
            BCK(b, cudaMalloc((void**)&b->d_bar, 4 * sizeof(unsigned)));
            BCK(b, cudaMemset(b->d_bar, 0, 4 * sizeof(unsigned)));
        }
        if (!b->pgrid) b->pgrid = ose::persist_grid();
        if (b->pgrid <= 0) b->persist_ok = false;
    }
    if (b->graph) { cudaGraphExecDestroy(b->graph); b->graph = nullptr; }
    return OSE_OK;
}

// One shot's whole step with the single-shot launch sequence (source
// injection, then M + 1 applications of the generic passes) on stream st.
cudaError_t enqueue_shot_step(ose_batch* b, int s, cudaStream_t st)
{
    const ose::BatchShot& D = b->desc[s];
    cudaError_t e = ose::launch_inject(st, D.W, D.src, D.ricker, D.hil, D.ctr, D.nt);
    if (e != cudaSuccess) return e;
    ose::Tables t{};
    t.twx = D.twx;
    t.twy = D.twy;
    t.twz = D.twz;
    t.kx2 = D.kx2;
    t.ky2 = D.ky2;
    t.kz2 = D.kz2;
    ose::EpiArgs ea{};
    ea.vs = D.vs;
    ea.ax = D.ax;
    ea.ay = D.ay;
    ea.az = D.az;
    ea.S = D.S;
    ea.wout = D.W;
    ea.sch = D.sch;
    ea.scl = D.scl;
    ea.gather = D.gather;
    ea.cur = D.ctr + 1;
    ea.gz = D.gz;
    ea.bl = D.bl;
    ea.bf = D.bf;
    ea.nx = D.nx;
    ea.ny = D.ny;
    ea.nt = D.nt;
    const bool fuse = ose::generic_fuses_x(D.px, t);   // as the single-shot step
    for (int n = 0; n <= D.M; ++n) {
        const float2* an = n == 0 ? D.W : ((n & 1) ? D.A : D.W);
        ea.prev = n == 0 ? D.A : ((n & 1) ? D.W : D.A);
        ea.c1 = D.c[n];
        ea.c1l = D.cl[n];
        ea.cp = n == 1 ? D.c0 : (n >= 2 ? D.c[n - 2] : 0.f);
        ea.cpl = n == 1 ? D.c0l : (n >= 2 ? D.cl[n - 2] : 0.f);
        ea.sp = ose::sum_plan(n, D.M);
        ose::set_sum_weights(ea);
        const ose::EpiMode mode = n == 0 ? ose::EPI_FIRST : (n == D.M ? ose::EPI_LAST : ose::EPI_MID);
        e = ose::launch_generic_application(st, D.g, D.px, D.py, D.pz, t, an, D.X, mode, ea, nullptr,
                                            fuse && n > 0, fuse && n < D.M);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t enqueue_lanes(ose_batch* b)
{
    cudaError_t e;
    for (int k = 0; k < b->lanes; ++k) {
        if (!b->lane[k] && (e = cudaStreamCreateWithFlags(&b->lane[k], cudaStreamNonBlocking)) != cudaSuccess)
            return e;
        if (!b->join[k] && (e = cudaEventCreateWithFlags(&b->join[k], cudaEventDisableTiming)) != cudaSuccess)
            return e;
    }
    if (!b->fork && (e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming)) != cudaSuccess) return e;
    if ((e = cudaEventRecord(b->fork, b->stream)) != cudaSuccess) return e;
    for (int k = 0; k < b->lanes; ++k)
        if ((e = cudaStreamWaitEvent(b->lane[k], b->fork, 0)) != cudaSuccess) return e;
    for (int s = 0; s < b->nshots; ++s)
        if ((e = enqueue_shot_step(b, s, b->lane[s % b->lanes])) != cudaSuccess) return e;
    for (int k = 0; k < b->lanes; ++k) {
        if ((e = cudaEventRecord(b->join[k], b->lane[k])) != cudaSuccess) return e;
        if ((e = cudaStreamWaitEvent(b->stream, b->join[k], 0)) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t enqueue_batch_step(ose_batch* b)
{
    if (b->lanes > 0) return enqueue_lanes(b);
    cudaError_t e = ose::launch_batch_inject(b->stream, b->d_shots, b->nshots);
    if (e != cudaSuccess) return e;
    if (b->lanes < 0) {
        // barrier counter back to zero (the error word stays until read)
        if ((e = cudaMemsetAsync(b->d_bar, 0, 2 * sizeof(unsigned), b->stream)) != cudaSuccess) return e;
        return ose::launch_batch_persistent(b->stream, b->d_shots, b->d_ppass, b->nppass, b->d_bar,
                                            reinterpret_cast<int*>(b->d_bar + 2), b->pgrid);
    }
    for (const ose::BatchPass& p : b->passes) {
        e = p.n_axis > 0 ? ose::launch_batch_col_pass(b->stream, p.kind, p.n_axis, b->d_shots, p.work, p.nblocks, p.n)
                         : ose::launch_batch_stockham_pass(b->stream, b->d_shots, p.n, p);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

ose_status batch_graph(ose_batch* b)
{
    if (b->graph) return OSE_OK;
    cudaGraph_t g = nullptr;
    BCK(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = enqueue_batch_step(b);
    cudaError_t e2 = cudaStreamEndCapture(b->stream, &g);
    if (e != cudaSuccess || e2 != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return bfail(b, OSE_ERR_CUDA, std::string("capture batch step: ") +
                                          cudaGetErrorString(e != cudaSuccess ? e : e2));
    }
    e = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        b->graph = nullptr;
        return bfail(b, OSE_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
    }
    return OSE_OK;
}

void free_batch(ose_batch* b)
{
    if (b->graph) cudaGraphExecDestroy(b->graph);
    for (int k = 0; k < ose_batch::kMaxLanes; ++k) {
        if (b->lane[k]) cudaStreamDestroy(b->lane[k]);
        if (b->join[k]) cudaEventDestroy(b->join[k]);
    }
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->d_work) cudaFree(b->d_work);
    if (b->d_ppass) cudaFree(b->d_ppass);
    if (b->d_bar) cudaFree(b->d_bar);
    if (b->d_shots) cudaFree(b->d_shots);
    if (b->arena) cudaFree(b->arena);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->stream) cudaStreamDestroy(b->stream);
}

}  // namespace

extern "C" {

ose_status ose_batch_create(const ose_params* p, const float* model, int mnx, int mny, int mnz, int nshots,
                            const ose_shot_window* win, ose_batch** out)
{
    if (!p || !model || !win || !out || nshots < 1 || mnx < 1 || mny < 1 || mnz < 1)
        return bfail(nullptr, OSE_ERR_INVALID, "bad argument");
    *out = nullptr;
    ose_batch* b = new ose_batch();
    b->base = *p;
    b->nshots = nshots;
    b->shots.resize(nshots);
    b->desc.resize(nshots);
    size_t total = 0;
    std::string err;
    for (int s = 0; s < nshots; ++s) {
        const ose_shot_window& w = win[s];
        ShotHost& sh = b->shots[s];
        sh.p = *p;
        sh.p.nx = w.nx;
        sh.p.ny = w.ny;
        sh.p.nz = w.nz;
        sh.p.sxbeg = w.sx;
        sh.p.sybeg = w.sy;
        sh.p.szbeg = w.sz;
        sh.p.jsx = sh.p.jsy = sh.p.jsz = 0;
        if (w.sx < 0 || w.sy < 0 || w.sz < 0 || w.sx >= w.nx || w.sy >= w.ny || w.sz >= w.nz ||
            p->gzbeg < 0 || p->gzbeg >= w.nz) {
            delete b;
            return bfail(nullptr, OSE_ERR_INVALID, "source or receiver depth outside window " + std::to_string(s));
        }
        if (ose::derive_dims(sh.p, &sh.d, &err) || ose::plan_axis(sh.d.nxb, &sh.px) ||
            ose::plan_axis(sh.d.nyb, &sh.py) || ose::plan_axis(sh.d.nzb, &sh.pz)) {
            delete b;
            return bfail(nullptr, OSE_ERR_UNSUPPORTED, "window " + std::to_string(s) + ": " + (err.empty() ? "axis too long" : err));
        }
        // the window's interior [x][y][z], cut from the model with clamping
        std::vector<float> wv((size_t)w.nx * w.ny * w.nz);
        for (int ix = 0; ix < w.nx; ++ix)
            for (int iy = 0; iy < w.ny; ++iy)
                for (int iz = 0; iz < w.nz; ++iz) {
                    const int X = std::min(std::max(w.x0 + ix, 0), mnx - 1);
                    const int Y = std::min(std::max(w.y0 + iy, 0), mny - 1);
                    const int Z = std::min(std::max(w.z0 + iz, 0), mnz - 1);
                    wv[((size_t)ix * w.ny + iy) * w.nz + iz] = model[((size_t)X * mny + Y) * mnz + Z];
                }
        ose::pad_model(sh.p, sh.d, wv.data(), sh.vb);
        float vmax = -9999999.999f;
        for (float v : sh.vb) vmax = std::max(vmax, v);
        for (float v : sh.vb)
            if (!(v > 0.f) || !std::isfinite(v)) {
                delete b;
                return bfail(nullptr, OSE_ERR_INVALID, "velocity model must be positive and finite");
            }
        ose::series_params(sh.p, vmax, &sh.d);
        if (sh.d.M + 1 > ose::kMaxTerms) {
            delete b;
            return bfail(nullptr, OSE_ERR_UNSUPPORTED, "series order too high for a batched shot");
        }
        sh.J.resize(sh.d.M + 2);
        for (int n = 0; n <= sh.d.M + 1; ++n) sh.J[n] = jn(n, sh.d.dtR);
        b->Mmax = std::max(b->Mmax, sh.d.M);
        const long long Z = p->bu + w.sz, Y = p->bf + w.sy, X = p->bl + w.sx;
        sh.src = (Z * sh.d.nyb + Y) * sh.d.nxb + X;
        const size_t N = (size_t)sh.d.nxb * sh.d.nyb * sh.d.nzb;
        sh.off = total;
        total += 4 * align256(sizeof(float2) * N) + align256(sizeof(float) * N) +
                 align256(sizeof(float) * (size_t)p->nt * w.nx * w.ny) + 2 * align256(sizeof(float) * p->nt) +
                 align256(64) + 3 * align256(sizeof(float2) * 1024) + 6 * align256(sizeof(float) * 1024);
    }
    cudaError_t e;
#define BCKC(call)                                                                                 \
    do {                                                                                           \
        e = (call);                                                                                \
        if (e != cudaSuccess) {                                                                    \
            ose_status s_ = e == cudaErrorMemoryAllocation ? OSE_ERR_NOMEM : OSE_ERR_CUDA;         \
            bfail(nullptr, s_, std::string(#call) + ": " + cudaGetErrorString(e));                 \
            free_batch(b);                                                                         \
            delete b;                                                                              \
            return s_;                                                                             \
        }                                                                                          \
    } while (0)
    BCKC(ose::configure_kernels());
    BCKC(ose::configure_batch_kernels());
    BCKC(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    BCKC(cudaEventCreate(&b->ev0));
    BCKC(cudaEventCreate(&b->ev1));
    BCKC(cudaMalloc((void**)&b->arena, total));
    b->arena_bytes = total;
    BCKC(cudaMalloc((void**)&b->d_shots, sizeof(ose::BatchShot) * nshots));
    std::vector<float> ricker, hil;
    ose::ricker_trace(p->nt, p->fm, p->dt, p->amp, ricker);
    ose::hilbert_trace(ricker, p->hilbert_div_nt, hil);
    for (int s = 0; s < nshots; ++s) {
        ShotHost& sh = b->shots[s];
        ose::BatchShot& D = b->desc[s];
        const ose_derived& d = sh.d;
        const size_t N = (size_t)d.nxb * d.nyb * d.nzb;
        char* q = b->arena + sh.off;
        auto take = [&](size_t bytes) { char* r = q; q += align256(bytes); return r; };
        D.g = {d.nxb, d.nyb, d.nzb, (long long)N};
        D.W = (float2*)take(sizeof(float2) * N);
        D.A = (float2*)take(sizeof(float2) * N);
        D.S = (float2*)take(sizeof(float2) * N);
        D.X = (float2*)take(sizeof(float2) * N);
        float* vs = (float*)take(sizeof(float) * N);
        D.vs = vs;
        D.gather = (float*)take(sizeof(float) * (size_t)p->nt * sh.p.nx * sh.p.ny);
        float* rk = (float*)take(sizeof(float) * p->nt);
        float* hl = (float*)take(sizeof(float) * p->nt);
        D.ricker = rk;
        D.hil = hl;
        D.ctr = (int*)take(64);
        float2* tw[3];
        float* k2[3];
        float* att[3];
        for (int a = 0; a < 3; ++a) tw[a] = (float2*)take(sizeof(float2) * 1024);
        for (int a = 0; a < 3; ++a) k2[a] = (float*)take(sizeof(float) * 1024);
        for (int a = 0; a < 3; ++a) att[a] = (float*)take(sizeof(float) * 1024);
        D.twx = tw[0]; D.twy = tw[1]; D.twz = tw[2];
        D.kx2 = k2[0]; D.ky2 = k2[1]; D.kz2 = k2[2];
        D.ax = att[0]; D.ay = att[1]; D.az = att[2];
        std::vector<float2> t0, t1, t2;
        std::vector<float> k0, k1, kk2, a0, a1, a2;
        ose::twiddle_table(d.nxb, t0);
        ose::twiddle_table(d.nyb, t1);
        ose::twiddle_table(d.nzb, t2);
        ose::k2_table(d.nxb, d.dkx, k0);
        ose::k2_table(d.nyb, d.dky, k1);
        ose::k2_table(d.nzb, d.dkz, kk2);
        ose::sponge_table(sh.p.bl, sh.p.nx, d.br, sh.p.sponge_mode, sh.p.cerjan_factor, a0);
        ose::sponge_table(sh.p.bf, sh.p.ny, d.bb, sh.p.sponge_mode, sh.p.cerjan_factor, a1);
        ose::sponge_table(sh.p.bu, sh.p.nz, d.bd, sh.p.sponge_mode, sh.p.cerjan_factor, a2);
        auto up = [&](void* dst, const void* src, size_t bytes) {
            return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, b->stream);
        };
        std::vector<float> vsc(sh.vb);
        if (!ose::kCompensatedConstants)
            for (size_t i = 0; i < N; ++i) vsc[i] = (float)((double)sh.vb[i] / (d.R * (double)N));
        BCKC(up(vs, vsc.data(), sizeof(float) * N));
        BCKC(up(rk, ricker.data(), sizeof(float) * p->nt));
        BCKC(up(hl, hil.data(), sizeof(float) * p->nt));
        BCKC(up(tw[0], t0.data(), sizeof(float2) * d.nxb));
        BCKC(up(tw[1], t1.data(), sizeof(float2) * d.nyb));
        BCKC(up(tw[2], t2.data(), sizeof(float2) * d.nzb));
        BCKC(up(k2[0], k0.data(), sizeof(float) * d.nxb));
        BCKC(up(k2[1], k1.data(), sizeof(float) * d.nyb));
        BCKC(up(k2[2], kk2.data(), sizeof(float) * d.nzb));
        BCKC(up(att[0], a0.data(), sizeof(float) * d.nxb));
        BCKC(up(att[1], a1.data(), sizeof(float) * d.nyb));
        BCKC(up(att[2], a2.data(), sizeof(float) * d.nzb));
        D.src = sh.src;
        D.M = d.M;
        D.gz = sh.p.bu + sh.p.gzbeg;
        D.bl = sh.p.bl;
        D.bf = sh.p.bf;
        D.nx = sh.p.nx;
        D.ny = sh.p.ny;
        D.nt = p->nt;
        ose::split_float(1.0 / (d.R * (double)N), &D.sch, &D.scl);
        ose::split_float(sh.J[0], &D.c0, &D.c0l);
        for (int n = 0; n <= d.M; ++n) ose::split_float(2.0 * sh.J[n + 1], &D.c[n], &D.cl[n]);
        sh.d.path = OSE_PATH_GENERIC;
    }
#undef BCKC
    fill_descriptors(b);
    ose_status st = build_passes(b);
    if (st != OSE_OK) {
        g_batch_create_error = b->err;
        free_batch(b);
        delete b;
        return st;
    }
    st = ose_batch_reset(b);
    if (st != OSE_OK) {
        g_batch_create_error = b->err;
        free_batch(b);
        delete b;
        return st;
    }
    *out = b;
    return OSE_OK;
}

ose_status ose_batch_destroy(ose_batch* b)
{
    if (!b) return OSE_OK;
    if (b->stream) cudaStreamSynchronize(b->stream);
    free_batch(b);
    delete b;
    return OSE_OK;
}

const char* ose_batch_last_error(const ose_batch* b) { return b ? b->err.c_str() : g_batch_create_error.c_str(); }

ose_status ose_batch_reset(ose_batch* b)
{
    if (!b) return OSE_ERR_INVALID;
    for (int s = 0; s < b->nshots; ++s) {
        const ose::BatchShot& D = b->desc[s];
        BCK(b, cudaMemsetAsync(D.W, 0, sizeof(float2) * (size_t)D.g.ncell, b->stream));
        BCK(b, cudaMemsetAsync(D.gather, 0, sizeof(float) * (size_t)D.nt * D.nx * D.ny, b->stream));
        BCK(b, cudaMemsetAsync(D.ctr, 0, 64, b->stream));
    }
    BCK(b, cudaStreamSynchronize(b->stream));
    b->it = 0;
    return OSE_OK;
}

// A persistent step whose grid barrier timed out leaves a nonzero error word.
static ose_status persist_status(ose_batch* b)
{
    if (b->lanes >= 0 || !b->d_bar) return OSE_OK;
    unsigned w = 0;
    BCK(b, cudaMemcpy(&w, b->d_bar + 2, sizeof w, cudaMemcpyDeviceToHost));
    if (w) {
        cudaMemset(b->d_bar + 2, 0, sizeof w);
        return bfail(b, OSE_ERR_TIMEOUT, "persistent batched step: a grid barrier timed out");
    }
    return OSE_OK;
}

ose_status ose_batch_run(ose_batch* b, int nsteps)
{
    if (!b || nsteps < 0) return OSE_ERR_INVALID;
    if (b->it + nsteps > b->base.nt) return bfail(b, OSE_ERR_INVALID, "nsteps beyond nt");
    ose_status st = batch_graph(b);
    if (st != OSE_OK) return st;
    for (int i = 0; i < nsteps; ++i) BCK(b, cudaGraphLaunch(b->graph, b->stream));
    BCK(b, cudaStreamSynchronize(b->stream));
    b->it += nsteps;
    return persist_status(b);
}

ose_status ose_batch_run_timed(ose_batch* b, int nsteps, float* ms)
{
    if (!b || !ms || nsteps < 0) return OSE_ERR_INVALID;
    if (b->it + nsteps > b->base.nt) return bfail(b, OSE_ERR_INVALID, "nsteps beyond nt");
    ose_status st = batch_graph(b);
    if (st != OSE_OK) return st;
    BCK(b, cudaStreamSynchronize(b->stream));
    BCK(b, cudaEventRecord(b->ev0, b->stream));
    for (int i = 0; i < nsteps; ++i) BCK(b, cudaGraphLaunch(b->graph, b->stream));
    BCK(b, cudaEventRecord(b->ev1, b->stream));
    BCK(b, cudaEventSynchronize(b->ev1));
    BCK(b, cudaEventElapsedTime(ms, b->ev0, b->ev1));
    b->it += nsteps;
    return persist_status(b);
}

ose_status ose_batch_info(const ose_batch* b, int shot, ose_derived* d, long long* cells)
{
    if (!b || shot < 0 || shot >= b->nshots) return OSE_ERR_INVALID;
    if (d) *d = b->shots[shot].d;
    if (cells) *cells = b->desc[shot].g.ncell;
    return OSE_OK;
}

ose_status ose_batch_get_gather(ose_batch* b, int shot, float* out)
{
    if (!b || !out || shot < 0 || shot >= b->nshots) return OSE_ERR_INVALID;
    const ose::BatchShot& D = b->desc[shot];
    const int nt = D.nt, ng = D.nx * D.ny;
    std::vector<float> g((size_t)nt * ng);
    BCK(b, cudaMemcpyAsync(g.data(), D.gather, sizeof(float) * g.size(), cudaMemcpyDeviceToHost, b->stream));
    BCK(b, cudaStreamSynchronize(b->stream));
    for (int it = 0; it < nt; ++it)
        for (int ig = 0; ig < ng; ++ig) out[(size_t)ig * nt + it] = g[(size_t)it * ng + ig];
    return OSE_OK;
}

ose_status ose_batch_get_wavefield(ose_batch* b, int shot, int which, float* out)
{
    if (!b || !out || shot < 0 || shot >= b->nshots || (which != OSE_FIELD_P && which != OSE_FIELD_Q))
        return OSE_ERR_INVALID;
    const ose::BatchShot& D = b->desc[shot];
    std::vector<float2> w((size_t)D.g.ncell);
    BCK(b, cudaMemcpyAsync(w.data(), D.W, sizeof(float2) * w.size(), cudaMemcpyDeviceToHost, b->stream));
    BCK(b, cudaStreamSynchronize(b->stream));
    for (size_t i = 0; i < w.size(); ++i) out[i] = which == OSE_FIELD_P ? w[i].x : w[i].y;
    return OSE_OK;
}

// Coordinate search over the tunables (rows per x-pass CTA, y and z column
// tiles, radix order), each candidate timed over `steps` batched steps from a
// fresh state; the best setting is kept, written to cache_path (when given)
// and read back from it for a batch with the same window sizes.
ose_status ose_batch_autotune(ose_batch* b, int steps, const char* cache_path, float* best_ms)
{
    if (!b || steps < 1) return OSE_ERR_INVALID;
    std::string sig;
    for (int s = 0; s < b->nshots; ++s) {
        const ose::Geometry& g = b->desc[s].g;
        sig += std::to_string(g.nxb) + "x" + std::to_string(g.nyb) + "x" + std::to_string(g.nzb) + "/" +
               std::to_string(b->desc[s].M) + ";";
    }
    if (cache_path) {
        FILE* f = fopen(cache_path, "r");
        if (f) {
            char line[1 << 16];
            while (fgets(line, sizeof line, f)) {
                char key[1 << 15];
                int rs, ty, tz, ro, gm = 0, ln = 0;
                const int nf = sscanf(line, "%32767s %d %d %d %d %d %d", key, &rs, &ty, &tz, &ro, &gm, &ln);
                if (nf >= 5 && sig == key) {
                    b->rows_scale = rs; b->txy = ty; b->txz = tz; b->radix_order = ro; b->group_mb = gm;
                    b->lanes = std::min(std::max(ln, -1), (int)ose_batch::kMaxLanes);
                    if (b->graph) { cudaGraphExecDestroy(b->graph); b->graph = nullptr; }
                    fclose(f);
                    fill_descriptors(b);
                    ose_status st = build_passes(b);
                    if (st == OSE_OK && b->lanes < 0 && !b->persist_ok) b->lanes = 0;
                    if (best_ms) *best_ms = -1.f;
                    return st != OSE_OK ? st : ose_batch_reset(b);
                }
            }
            fclose(f);
        }
    }
    if (steps > b->base.nt) steps = b->base.nt;
    auto measure = [&](float* ms) -> ose_status {
        fill_descriptors(b);
        ose_status st = build_passes(b);
        if (st != OSE_OK) return st;
        if ((st = ose_batch_reset(b)) != OSE_OK) return st;
        if ((st = ose_batch_run(b, 1)) != OSE_OK) return st;   // warm up
        return ose_batch_run_timed(b, std::min(steps, b->base.nt - 1), ms);
    };
    float best = 1e30f, ms = 0.f;
    ose_status st = measure(&best);
    if (st != OSE_OK) return st;
    // batching strategy first: per-shot launches on 1, 2, 4 or 8 concurrent
    // streams against batched launches (lanes = 0)
    for (int ln : {1, 2, 4, 8}) {
        const int keep = b->lanes;
        b->lanes = ln;
        if (measure(&ms) == OSE_OK && ms < best) best = ms;
        else b->lanes = keep;
    }
    // the persistent launch over the batched passes, with shot groups sized
    // for L2 or one group
    {
        fill_descriptors(b);
        if (build_passes(b) == OSE_OK && b->persist_ok) {
            const int keep_l = b->lanes, keep_g = b->group_mb;
            int best_g = -1;
            for (int gm : {0, 96, 48}) {
                b->lanes = -1;
                b->group_mb = gm;
                if (measure(&ms) == OSE_OK && ms < best) {
                    best = ms;
                    best_g = gm;
                }
            }
            if (best_g >= 0) {
                b->lanes = -1;
                b->group_mb = best_g;
            } else {
                b->lanes = keep_l;
                b->group_mb = keep_g;
            }
        }
    }
    // then the group size of batched launches: it decides whether fields stay
    // in L2 (1 MB: one shot per group, since every shot is larger)
    for (int gm : {1024, 256, 96, 1}) {
        if (b->lanes != 0) break;
        const int keep = b->group_mb;
        b->group_mb = gm;
        if (measure(&ms) == OSE_OK && ms < best) best = ms;
        else b->group_mb = keep;
    }
    const int rs_c[] = {1024, 2048, 4096};
    const int tx_c[] = {8, 16, 32};
    for (int rs : rs_c) {
        const int keep = b->rows_scale;
        if (rs == keep) continue;
        b->rows_scale = rs;
        if (measure(&ms) == OSE_OK && ms < best) best = ms;
        else b->rows_scale = keep;
    }
    for (int axis = 0; axis < 2; ++axis)
        for (int tx : tx_c) {
            int& knob = axis == 0 ? b->txy : b->txz;
            const int keep = knob;
            if (tx == keep) continue;
            knob = tx;
            if (measure(&ms) == OSE_OK && ms < best) best = ms;
            else knob = keep;
        }
    {
        const int keep = b->radix_order;
        b->radix_order = 1 - keep;
        if (measure(&ms) == OSE_OK && ms < best) best = ms;
        else b->radix_order = keep;
    }
    fill_descriptors(b);
    if ((st = build_passes(b)) != OSE_OK) return st;
    if ((st = ose_batch_reset(b)) != OSE_OK) return st;
    if (best_ms) *best_ms = best;
    if (cache_path) {
        FILE* f = fopen(cache_path, "a");
        if (!f) return bfail(b, OSE_ERR_IO, std::string("cannot write ") + cache_path);
        fprintf(f, "%s %d %d %d %d %d %d\n", sig.c_str(), b->rows_scale, b->txy, b->txz, b->radix_order, b->group_mb,
                b->lanes);
        fclose(f);
    }
    return OSE_OK;
}

ose_status ose_batch_set_tuning(ose_batch* b, int rows_scale, int txy, int txz, int radix_order, int group_mb,
                                int lanes)
{
    if (!b || rows_scale < 1 || txy < 1 || txz < 1 || radix_order < 0 || radix_order > 1 || group_mb < 0 ||
        lanes < -1 || lanes > ose_batch::kMaxLanes)
        return OSE_ERR_INVALID;
    b->lanes = lanes;
    b->rows_scale = rows_scale;
    b->txy = txy;
    b->txz = txz;
    b->radix_order = radix_order;
    b->group_mb = group_mb;
    fill_descriptors(b);
    ose_status st = build_passes(b);
    if (st != OSE_OK) return st;
    if (lanes < 0 && !b->persist_ok) {
        b->lanes = 0;
        return bfail(b, OSE_ERR_UNSUPPORTED, "the persistent step needs axis lengths 16 C with C <= 16 and a "
                                             "cooperative launch");
    }
    return ose_batch_reset(b);
}

ose_status ose_batch_get_tuning(const ose_batch* b, int* rows_scale, int* txy, int* txz, int* radix_order,
                                int* group_mb, int* lanes)
{
    if (!b) return OSE_ERR_INVALID;
    if (group_mb) *group_mb = b->group_mb;
    if (lanes) *lanes = b->lanes;
    if (rows_scale) *rows_scale = b->rows_scale;
    if (txy) *txy = b->txy;
    if (txz) *txz = b->txz;
    if (radix_order) *radix_order = b->radix_order;
    return OSE_OK;
}

}  // extern "C"
