// ose_internal.h - declarations shared by the host and device parts of libose3d.
#pragma once

#include <cuda_runtime.h>
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

struct EpiArgs {
    float2* prev;         // FIRST: a_1 out.  MID/LAST: a_{n-1} in, a_{n+1} out (MID)
    const float2* w;      // FIRST: a_0 = W
    float2* S;            // partial sum
    float2* wout;         // LAST: new state (P, Q)
    const float* vs;      // v / (R N), per cell
    const float* ax;      // sponge, x
    const float* ay;      // sponge, y
    const float* az;      // sponge, z
    float c0, c1;         // FIRST: J0, 2 J1.  MID/LAST: c1 = 2 J_{n+1}
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
};

// Host-side launch helpers (ose_kernels.cu).
struct KernelTiming;
cudaError_t launch_generic_application(cudaStream_t s, const Geometry& g, const AxisPlan& px,
                                       const AxisPlan& py, const AxisPlan& pz, const Tables& t,
                                       const float2* an, float2* X, EpiMode mode,
                                       const EpiArgs& e, KernelTiming* timing);
cudaError_t launch_inject(cudaStream_t s, float2* W, long long src, const float* ricker,
                          const float* hil, int* ctr, int nt);
cudaError_t launch_apply_operator(cudaStream_t s, const Geometry& g, const AxisPlan& px,
                                  const AxisPlan& py, const AxisPlan& pz, const Tables& t,
                                  const float2* in, float2* X, float2* out, const float* vs);
cudaError_t configure_kernels();

// 256^3 fast path (ose_plane.cu).
bool plane_path_supported(int nxb, int nyb, int nzb);
cudaError_t configure_plane_kernels();
cudaError_t launch_plane_fwd(cudaStream_t s, const float2* state, float2* X, const float2* tw);
cudaError_t launch_zpass(cudaStream_t s, float2* X, const float2* tw, const Tables& t);
cudaError_t launch_plane_inv(cudaStream_t s, EpiMode mode, bool fwd, const float2* Xin, float2* Xout,
                             const float2* tw, const EpiArgs& e);
cudaError_t launch_plane_apply_operator(cudaStream_t s, const float2* in, float2* X, float2* out,
                                        const float* vs, const float2* tw, const Tables& t);
int plane_max_active_clusters();

// Per-kernel-class timing used by ose_profile_step.
struct KernelTiming {
    static constexpr int kClasses = 8;
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
void twiddle_table(int n, std::vector<float2>& out);
void k2_table(int n, double dk, std::vector<float>& out);
int derive_dims(const ose_params& p, ose_derived* d, std::string* err);
void series_params(const ose_params& p, float vmax, ose_derived* d);

}  // namespace ose
