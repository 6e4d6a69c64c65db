// ose_noalloc.cu - an operator entry point that allocates nothing.
//
// Some callers cannot call cudaMalloc: code that runs where another framework
// owns the device allocator (a custom-call or plugin inside an ML runtime that
// forbids allocations behind its back), real-time or embedded hosts that must
// not allocate after start-up, and callers that already hold every buffer they
// want the library to touch.  For them, ose_apply_operator_noalloc applies the
// normalised OSE operator to device buffers the caller passes in, and keeps
// its one-field FFT scratch and its twiddle/wavenumber tables in a fixed
// file-scope device array instead of allocating them.
//
// Limits and rules (also stated in include/ose3d.h):
//   - at most OSE_NOALLOC_MAX_CELLS = 262144 padded cells (for example 64^3);
//     each axis even, at most 1024 long;
//   - the array (about 2 MiB) lives on every GPU that loads the library until
//     the process exits;
//   - every call shares it and it keeps the last call's contents, so calls
//     that overlap on the GPU (two streams, two host threads) race and give
//     wrong results: serialise them;
//   - nothing in it has to start at zero: each call rewrites the tables and
//     the whole scratch field before reading them;
//   - the first call on a device looks up the array's device address (and
//     sets kernel attributes); make that first call before any stream capture.
#include <cuda_runtime.h>
#include <math.h>

#include <mutex>

#include "ose_internal.h"

namespace ose {

cudaError_t launch_apply_operator_vel(cudaStream_t s, const Geometry& g, const AxisPlan& px,
                                      const AxisPlan& py, const AxisPlan& pz, const Tables& t,
                                      const float2* in, float2* X, float2* out, const float* vel,
                                      double scale);

namespace {

// The tables below hold single-float twiddles and squared wavenumbers only:
// the low halves that the compensated variants read are not kept in the array.
static_assert(!kCompensatedConstants && !kCompensatedTwiddles,
              "the allocation-free entry point keeps no low-part tables");

constexpr long long kMaxCells = OSE_NOALLOC_MAX_CELLS;
constexpr int kMaxAxisLen = 1024;
// layout of the array, in float2 units: scratch field | twiddles x, y, z | k^2 x, y, z
constexpr long long kTwOff = kMaxCells;
constexpr long long kK2Off = kTwOff + 3LL * kMaxAxisLen;
constexpr long long kTotal = kK2Off + 3LL * kMaxAxisLen / 2;

static __device__ __align__(256) float2 g_scratch[kTotal];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
float2* g_addr[kMaxDevices] = {};

// W_n^t = exp(-2 pi i t / n) and (dk * wrapped index)^2 for the three axes.
__global__ void k_noalloc_tables(float2* tw, float* k2, int nx, int ny, int nz, double dkx, double dky,
                                 double dkz)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int ax = blockIdx.y;
    const int n = ax == 0 ? nx : (ax == 1 ? ny : nz);
    const double dk = ax == 0 ? dkx : (ax == 1 ? dky : dkz);
    if (t >= n) return;
    double s, c;
    sincospi(-2.0 * (double)t / (double)n, &s, &c);
    tw[ax * kMaxAxisLen + t] = make_float2((float)c, (float)s);
    const double k = dk * (double)(t > n / 2 ? n - t : t);
    k2[ax * kMaxAxisLen + t] = (float)(k * k);
}

}  // namespace
}  // namespace ose

extern "C" ose_status ose_apply_operator_noalloc(int nxb, int nyb, int nzb, float dx, float dy, float dz,
                                                 double R, const float* vel, const float* in, float* out,
                                                 void* stream)
{
    using namespace ose;
    if (!vel || !in || !out) return OSE_ERR_INVALID;
    if (nxb < 2 || nyb < 2 || nzb < 2 || (nxb & 1) || (nyb & 1) || (nzb & 1) || !(R > 0.0) ||
        !(dx > 0.f) || !(dy > 0.f) || !(dz > 0.f))
        return OSE_ERR_INVALID;
    if ((long long)nxb * nyb * nzb > kMaxCells || nxb > kMaxAxisLen || nyb > kMaxAxisLen || nzb > kMaxAxisLen)
        return OSE_ERR_UNSUPPORTED;
    AxisPlan px, py, pz;
    if (plan_axis(nxb, &px) || plan_axis(nyb, &py) || plan_axis(nzb, &pz)) return OSE_ERR_UNSUPPORTED;

    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return OSE_ERR_CUDA;
    float2* base;
    {
        std::lock_guard<std::mutex> lock(g_mutex);
        if (!g_addr[dev]) {
            void* p = nullptr;
            if (cudaGetSymbolAddress(&p, g_scratch) != cudaSuccess || !p) return OSE_ERR_CUDA;
            if (configure_kernels() != cudaSuccess || configure_plane_kernels() != cudaSuccess)
                return OSE_ERR_CUDA;
            g_addr[dev] = static_cast<float2*>(p);
        }
        base = g_addr[dev];
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    float2* tw = base + kTwOff;
    float* k2 = reinterpret_cast<float*>(base + kK2Off);
    const double pi2 = 2.0 * M_PI;
    k_noalloc_tables<<<dim3((kMaxAxisLen + 255) / 256, 3), 256, 0, s>>>(
        tw, k2, nxb, nyb, nzb, pi2 / dx / nxb, pi2 / dy / nyb, pi2 / dz / nzb);
    if (cudaGetLastError() != cudaSuccess) return OSE_ERR_CUDA;
    Geometry g{nxb, nyb, nzb, (long long)nxb * nyb * nzb};
    Tables t{};
    t.twx = tw;
    t.twy = tw + kMaxAxisLen;
    t.twz = tw + 2 * kMaxAxisLen;
    t.kx2 = k2;
    t.ky2 = k2 + kMaxAxisLen;
    t.kz2 = k2 + 2 * kMaxAxisLen;
    const double scale = 1.0 / (R * (double)g.ncell);
    cudaError_t e = launch_apply_operator_vel(s, g, px, py, pz, t, reinterpret_cast<const float2*>(in), base,
                                              reinterpret_cast<float2*>(out), vel, scale);
    return e == cudaSuccess ? OSE_OK : OSE_ERR_CUDA;
}
