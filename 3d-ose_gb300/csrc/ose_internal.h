// ose_internal.h - declarations shared by the host and device parts of libose3d.
#pragma once

#include <cuda_runtime.h>
#include <assert.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/ose3d.h"

namespace ose {

constexpr int kMaxStages = 16;
constexpr int kMaxAxis = 1024;   // longest padded axis the generic kernels accept

// Radix plan of one FFT axis: n = prod(radix[0..ns)).
struct AxisPlan {
    int n;
    int ns;
    int radix[kMaxStages];
};

// Everything the per-application kernels read; passed by value.
struct Geometry {
    int nxb, nyb, nzb;
    long long ncell;
};

// Epilogue selection of the last pass of one operator application
// (wavefield_extro_ori2, ose_3d_lib.cu:651-870, fused).
enum EpiMode { EPI_FIRST = 0, EPI_MID = 1, EPI_LAST = 2, EPI_SCALE = 3 };

// Schedule of the Chebyshev partial sum S over the applications of one step.
// The reference adds a_{n+1} to S at application n and multiplies S by the
// sponge att after every addition (ose_3d_lib.cu:736-744, 839-860), so after
// application n the term a_j carries att^e(j, n), e = n for j <= 1 and
// n - j + 2 for j >= 2, and the new state is S after application M.  Here
// every term a_j is added exactly once, at an application where the epilogue
// holds it anyway: application j - 1 (it is the new term a_{n+1}) or j + 1
// (it is a_{n-1}, read for the recurrence), with the power of att it carries
// there; S itself is multiplied by att^(n - n') where n' is the application
// that last stored it.  Terms are taken in pairs (a_{4k}, a_{4k+2}) at
// application 4k + 1 and (a_{4k+1}, a_{4k+3}) at 4k + 2, so S is read and
// written at 6 of the 11 applications of M = 10 instead of at all of them
// (the other applications write only the recurrence term), and the first
// application reads neither the state nor S.  Same sum, same sponge powers;
// only the rounding order differs.
struct SumPlan {
    int add_prev;   // add c_{n-1} att^kP a_{n-1}
    int add_new;    // add c_{n+1} att^kN a_{n+1}
    int s_read;     // S holds earlier terms (else this application starts it)
    int touch;      // S is updated here (MID: S written; LAST: always, writes the state)
    int kS, kP, kN; // powers of att on the stored S, a_{n-1} and a_{n+1}
};

// Application at which term a_j (j = 0 .. M + 1) is added.
__host__ __device__ inline int sum_term_app(int j, int M)
{
    if ((j & 3) < 2) return j + 1 <= M ? j + 1 : j - 1;
    return j - 1;
}

__host__ __device__ inline bool sum_touches(int n, int M)
{
    return n == M || sum_term_app(n + 1, M) == n || (n >= 1 && sum_term_app(n - 1, M) == n);
}

__host__ __device__ inline SumPlan sum_plan(int n, int M)
{
    SumPlan p{};
    p.add_prev = n >= 1 && sum_term_app(n - 1, M) == n;
    p.add_new = sum_term_app(n + 1, M) == n;
    p.touch = sum_touches(n, M);
    int last = -1;
    for (int k = n - 1; k >= 0; --k)
        if (sum_touches(k, M)) { last = k; break; }
    p.s_read = p.touch && last >= 0;
    p.kS = p.s_read ? n - last : 0;
    const int jp = n - 1, jn = n + 1;
    p.kP = jp <= 1 ? n : n - jp + 2;
    p.kN = jn <= 1 ? n : n - jn + 2;
    return p;
}

// The powers a SumPlan uses are 0 .. 3 for every series order M up to
// kMaxTerms (kS, kP in 1 .. 3; kN = 1, or 0 at the first application where
// att = 1), which the three weights of EpiArgs cover.
constexpr int kSumMaxPow = 3;

struct EpiArgs {
    float2* prev;         // FIRST: a_1 out.  MID/LAST: a_{n-1} in, a_{n+1} out (MID)
    float2* S;            // partial sum
    float2* wout;         // LAST: new state (P, Q)
    const float* vs;      // velocity v per cell (the model value itself)
    const float* ax;      // sponge, x
    const float* ay;      // sponge, y
    const float* az;      // sponge, z
    // Constants as unevaluated float pairs hi + lo (about 48 significant
    // bits), so that no rounded constant biases every step the same way:
    float c1, c1l;        // coefficient of the new term a_{n+1}: 2 J_{n+1}
    float cp, cpl;        // coefficient of a_{n-1}: J0 (n = 1) or 2 J_{n-1}
    SumPlan sp;           // what this application adds to S
    // The schedule as weights of att, att^2, att^3 (set_sum_weights): the
    // stored S is multiplied by sum_k wS[k] att^(k+1), a_{n-1} by
    // sum_k (wP[k] + wPl[k]) att^(k+1) (one weight nonzero, the coefficient
    // folded in), a_{n+1} by (wN + wNl) att (its power is 1; the first
    // application passes att = 1).
    float wS[3], wP[3], wPl[3], wN, wNl;
    float sch, scl;       // 1 / (R N), the scale of v * IFFT3(|k| FFT3(.))
    // receivers (LAST)
    float* gather;        // [nt][ng]
    const int* cur;       // current step index
    int gz, bl, bf, nx, ny, nt;
};

struct Tables {
    const float2* twx;    // W_n^t, t < n, per axis
    const float2* twy;
    const float2* twz;
    const float* kx2;     // squared wrapped wavenumbers
    const float* ky2;
    const float* kz2;
    const float2* twl;    // plane path: low parts of W_256^t (twx = high parts)
    const float* kx2l;    // plane path: low parts of the squared wavenumbers
    const float* ky2l;
    const float* kz2l;
    // precision form (ose_tensor.cu): OSE_PRECISION_* of the z pass, its DFT
    // operands in shared-memory layout and the device error word
    int tcvar;
    const void* tcb;
    int* tcerr;
    // Bluestein transforms (ose_bluestein.cu), per axis x, y, z: length L of
    // the register transforms (0 = the axis has its own kernels), chirp (n),
    // B = FFT_L(b) / L and W_L^t (L each)
    int bl[3];
    const float2* bch[3];
    const float2* bsp[3];
    const float2* btw[3];
};

// Compensated constants: when true, the Bessel coefficients, 1/(R N) and |k|
// enter the kernels as float pairs (about 48 bits) and the velocity buffer
// holds v itself; when false, single floats and the buffer holds v/(R N).
// Measured on the 256^3 workload over 2000 steps the pairs change the error
// against FP64 only slightly (gather 9.9e-6 -> 8.5e-6, final Q 1.9e-4 ->
// 1.86e-4) and cost about 6% of the step, so they are off.
constexpr bool kCompensatedConstants = false;

// Twiddles as float pairs (hi + lo) in every 256-point transform of the plane
// kernels (ose_plane.cu, k_zpass16 included).  Off: the measured 2000-step
// error of the 256^3 workload is the same either way (round-off, not twiddle
// bias, dominates) and the pairs cost about 8% of the step.
constexpr bool kCompensatedTwiddles = false;

// hi + lo split of a double: hi = nearest float, lo = nearest float to the rest.
inline void split_float(double v, float* hi, float* lo)
{
    *hi = (float)v;
    *lo = kCompensatedConstants ? (float)(v - (double)*hi) : 0.f;
}

// Coefficients and partial-sum schedule of application n of M + 1 (J = the
// Bessel values J_0 .. J_{M+1} of the step, in double).
// The weights of EpiArgs from its schedule and coefficients (host and device
// build the same values: no arithmetic, only placement).
__host__ __device__ inline void set_sum_weights(EpiArgs& e)
{
    const SumPlan& p = e.sp;
    for (int k = 0; k < 3; ++k) {
        e.wS[k] = (p.s_read && p.kS == k + 1) ? 1.f : 0.f;
        e.wP[k] = (p.add_prev && p.kP == k + 1) ? e.cp : 0.f;
        e.wPl[k] = (p.add_prev && p.kP == k + 1) ? e.cpl : 0.f;
    }
    e.wN = p.add_new ? e.c1 : 0.f;
    e.wNl = p.add_new ? e.c1l : 0.f;
}

inline void set_application(EpiArgs& e, int n, int M, const double* J)
{
    split_float(2.0 * J[n + 1], &e.c1, &e.c1l);
    split_float(n == 1 ? J[0] : (n >= 2 ? 2.0 * J[n - 1] : 0.0), &e.cp, &e.cpl);
    e.sp = sum_plan(n, M);
    assert(e.sp.kS <= kSumMaxPow && e.sp.kP <= kSumMaxPow && e.sp.kN <= 1);
    set_sum_weights(e);
}

// HBM bytes per cell of the epilogue of application n (FIRST, MID, LAST):
// reads X, v and (MID, LAST) a_{n-1}; writes the new term (or, LAST, the
// state); S read and written as the schedule says; fwd: the fused forward
// transform of the new term also writes X.
inline double epilogue_bytes(EpiMode mode, const SumPlan& sp, bool fwd)
{
    double b = 8.0 + 4.0 + 8.0 + (fwd ? 8.0 : 0.0);
    if (mode != EPI_FIRST) b += 8.0;
    if (sp.s_read) b += 8.0;
    if (sp.touch && mode != EPI_LAST) b += 8.0;
    return b;
}

// Host-side launch helpers (ose_kernels.cu).
struct KernelTiming;
// One operator application with the series update (5 passes).  With the
// register row kernels (generic_fuses_x): x_ready = X already holds the x
// transform of an (pass 1 skipped); fwd_next (FIRST, MID) = the row pass also
// writes the x transform of the new term into X for the next application.
bool generic_fuses_x(const AxisPlan& px, const Tables& t);
cudaError_t launch_generic_application(cudaStream_t s, const Geometry& g, const AxisPlan& px,
                                       const AxisPlan& py, const AxisPlan& pz, const Tables& t,
                                       const float2* an, float2* X, EpiMode mode,
                                       const EpiArgs& e, KernelTiming* timing, bool x_ready = false,
                                       bool fwd_next = false);
cudaError_t launch_inject(cudaStream_t s, float2* W, long long src, const float* ricker,
                          const float* hil, int* ctr, int nt);
cudaError_t launch_apply_operator(cudaStream_t s, const Geometry& g, const AxisPlan& px,
                                  const AxisPlan& py, const AxisPlan& pz, const Tables& t,
                                  const float2* in, float2* X, float2* out, const float* vs,
                                  float sch, float scl);
cudaError_t configure_kernels();

struct BatchShot;

// Register column transforms for lengths 16 C (ose_cols.cu).
bool col_supported(int n);
cudaError_t configure_col_kernels();
cudaError_t launch_col(cudaStream_t s, int mode, int n, float2* X, int nxb, int nother, long long stride,
                       long long ostride, const float2* twg, const Tables& t);
// Batched register passes (kind 0 x fwd, 1 y fwd, 2 z, 3 y inv, 4 x inv + update)
// over the shots whose axis length is n_axis; x tile of the column passes
// and rows per CTA of the row passes for that length.
cudaError_t launch_batch_col_pass(cudaStream_t s, int kind, int n_axis, const BatchShot* shots, const int2* work,
                                  int nblocks, int n);
int col_tile(int n_axis);
int row_tile(int n_axis);
// epi: -1 = forward src -> dst, else an EpiMode (or 4 = scale by a velocity array)
cudaError_t launch_row(cudaStream_t s, int epi, int n, const float2* src, float2* dst, int nyb, long long nrows,
                       const float2* twg, const EpiArgs& e);

// 256^3 fast path (ose_plane.cu).
bool plane_path_supported(int nxb, int nyb, int nzb);
cudaError_t configure_plane_kernels();
cudaError_t launch_plane_fwd(cudaStream_t s, const float2* state, float2* X, const Tables& t);
cudaError_t launch_zpass(cudaStream_t s, float2* X, const Tables& t);
// The same z pass (forward, |k|, inverse of 256-point z lines) on any grid
// with 256 z planes and nxb a multiple of 16.
bool zpass256_supported(const Geometry& g);
cudaError_t launch_zpass256(cudaStream_t s, float2* X, const Geometry& g, const Tables& t);
cudaError_t launch_plane_inv(cudaStream_t s, EpiMode mode, bool fwd, const float2* Xin, float2* Xout,
                             const Tables& t, const EpiArgs& e);
cudaError_t launch_plane_apply_operator(cudaStream_t s, const float2* in, float2* X, float2* out,
                                        const float* vs, float sch, float scl, const Tables& t);
int plane_max_active_clusters();

// Self tests of the bounded waits (one CTA each; nothing ever completes the
// wait, so it runs out after limit_ns and the kernel sets *err, non-zero):
// the plane kernels' DSMEM exchange wait, the persistent batch's grid barrier
// (bar: two zeroed words) and the tensor-core MMA completion wait.
cudaError_t selftest_exchange_wait(cudaStream_t s, int* err, unsigned long long limit_ns);
cudaError_t selftest_grid_barrier(cudaStream_t s, unsigned* bar, int* err, unsigned long long limit_ns);
cudaError_t selftest_mma_wait(cudaStream_t s, int* err, unsigned long long limit_ns);

// Axis transforms by Bluestein's chirp-z identity (ose_bluestein.cu).
int bluestein_length(int n);
void bluestein_tables(int n, int L, std::vector<float2>& chirp, std::vector<float2>& spec,
                      std::vector<float2>& twl);
cudaError_t configure_bluestein_kernels();
cudaError_t launch_col_bluestein(cudaStream_t s, int mode, int n, float2* X, int nxb, int nother, long long stride,
                                 long long ostride, int axis, const Tables& t);
cudaError_t launch_row_bluestein(cudaStream_t s, int epi, int n, const float2* src, float2* dst, int nyb,
                                 long long nrows, const Tables& t, const EpiArgs& e);

// Precision form: tensor-core z pass (ose_tensor.cu).
bool tensor_zpass_supported(int nxb, int nyb, int nzb);
size_t tensor_operand_bytes(int var);
void tensor_operands(int var, std::vector<uint8_t>& out);
cudaError_t configure_tensor_kernels();
cudaError_t launch_tensor_zpass(cudaStream_t s, float2* X, const Geometry& g, const Tables& t);

// ---- batched shots (ose_batch.cu host side, kernels in ose_kernels.cu) ----
constexpr int kMaxTerms = 48;   // series terms M + 1 a batched shot may use

// Everything one shot of a batch needs on the device; an array of these lives
// in device memory and each CTA reads the entry of the shot it works on.
struct BatchShot {
    Geometry g;
    AxisPlan px, py, pz;
    int rpc, txy, txz;              // rows per CTA (x pass), column tiles (y, z passes)
    float2 *W, *A, *S, *X;
    const float* vs;
    const float *ax, *ay, *az;
    const float2 *twx, *twy, *twz;
    const float *kx2, *ky2, *kz2;
    float* gather;                  // [nt][nx*ny]
    int* ctr;                       // [0] next step, [1] current step
    const float* ricker;
    const float* hil;
    long long src;
    int M, gz, bl, bf, nx, ny, nt;
    float sch, scl, c0, c0l;
    float c[kMaxTerms], cl[kMaxTerms];   // 2 J_{n+1} (hi, lo), n = 0..M
};

// One batched pass: work[b] = (shot, block of that shot), b < nblocks.
// kind: 0 x forward, 1 y forward, 2 z (forward * |k| inverse), 3 y inverse,
// 4 x inverse + series update.  n_axis > 0: the register kernels for that
// axis length (ose_cols.cu); 0: the shared-memory Stockham kernels.
struct BatchPass {
    const int2* work;
    int nblocks;
    size_t smem;
    int kind;
    int n_axis;
    int n;        // operator application
};

cudaError_t configure_batch_kernels();

// The batched step as one persistent cooperative launch (ose_cols.cu): one
// entry per batched pass in launch order; barrier_after = the grid meets
// before the next entry (after the last length class of a pass).
struct PersistPass {
    const int2* work;
    int nblocks;
    int kind;
    int n_axis;
    int n;
    int barrier_after;
};
bool persist_supported(int n_axis);
size_t persist_smem();
int persist_grid();   // CTAs of a co-resident grid on the current device (0 = unavailable)
cudaError_t launch_batch_persistent(cudaStream_t s, const BatchShot* shots, const PersistPass* passes, int npass,
                                    unsigned* bar, int* err, int grid);
cudaError_t launch_batch_inject(cudaStream_t s, const BatchShot* shots, int nshots);
// One pass of operator application n (shared-memory Stockham kernels).
cudaError_t launch_batch_stockham_pass(cudaStream_t s, const BatchShot* shots, int n, const BatchPass& p);
size_t batch_rows_smem(int n, int rpc);
size_t batch_lines_smem(int n, int tx);

// Per-kernel-class timing used by ose_profile_step.
struct KernelTiming {
    static constexpr int kClasses = 10;
    cudaEvent_t ev[2];
    float ms[kClasses];
    int count[kClasses];
    double bytes[kClasses];
    const char* name[kClasses];
    int nclass;
};

// Host setup (ose_host.cpp), all in double.
int plan_axis(int n, AxisPlan* p);
void pad_model(const ose_params& p, const ose_derived& d, const float* vel_xyz, std::vector<float>& vb);
void sponge_table(int before, int nn, int after, int mode, float factor, std::vector<float>& out);
void ricker_trace(int nt, float fm, float dt, float amp, std::vector<float>& out);
void hilbert_trace(const std::vector<float>& w, int div_nt, std::vector<float>& out);
void twiddle_table(int n, std::vector<float2>& out, std::vector<float2>* lo = nullptr);
void k2_table(int n, double dk, std::vector<float>& out, std::vector<float>* lo = nullptr);
int derive_dims(const ose_params& p, ose_derived* d, std::string* err);
void series_params(const ose_params& p, float vmax, ose_derived* d);

}  // namespace ose
