/*
 * emu_runtime.cpp - host stand-ins for the CUDA runtime and cuFFT calls that
 * the reference makes, so its unmodified host code (ose_3d_lib.cu) and kernels
 * (ose_3d_kernel.cu, see emu_kernels.cpp) run on this machine without a GPU.
 * TEST INFRASTRUCTURE: part of oracle/_ref/ref_ose.
 *
 * Memory: one address space; "device" allocations are host allocations with
 * 4 KiB of slack, because hilbert_1d writes up to ceil(nt/16)*16 elements of
 * an nt-element buffer (ose_3d.cu:177, ose_3d_kernel.cu:154-172) and the
 * reference relies on the GPU allocator's granularity there.
 *
 * cuFFT: the published contract (unnormalised DFT, sign -1 forward) computed
 * in double by oracle/fft64.c and rounded to float.  The 2-GPU descriptor is
 * modelled as two halves: natural order = z-slabs [nzb/2][nyb][nxb] per GPU;
 * after a forward transform the data is "shuffled", GPU i holding
 * [nzb][nyb/2][nxb] for y in [i*nyb/2, (i+1)*nyb/2).  That is the layout
 * scale_kxkz_3D indexes (ose_3d_kernel.cu:101-126 with ny = nyb/2,
 * ose_3d.cu:143) and the one cuFFT documents for a multi-GPU 3-D transform.
 * C2R (1-D) drops the imaginary parts of the DC and Nyquist bins (the
 * Hermitian formula).
 */
#include <cuda_runtime_api.h>
#include <cufftXt.h>

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <map>
#include <vector>

#include "../fft64.h"

extern "C" int emu_launch(const char* device_name, dim3 grid, dim3 block, void** args);

namespace {
std::map<const void*, const char*>& functions()
{
    static std::map<const void*, const char*> m;
    return m;
}
struct LaunchCfg { dim3 grid, block; size_t smem; void* stream; };
std::vector<LaunchCfg>& cfgstack()
{
    static std::vector<LaunchCfg> s;
    return s;
}
cudaError_t g_last = cudaSuccess;
void* fatbin_handle[4];

struct Plan {
    int kind = 0;       /* 0 none, 1 = 3-D C2C multi-GPU, 2 = 1-D R2C, 3 = 1-D C2R */
    int n0 = 0, n1 = 0, n2 = 0;   /* 3-D: nx (slowest), ny, nz (fastest) in cuFFT terms */
    int ngpu = 1;
};
std::vector<Plan>& plans()
{
    static std::vector<Plan> p(1);
    return p;
}

void* emu_alloc(size_t bytes)
{
    void* p = calloc(1, bytes + 4096);
    return p;
}
}  // namespace

extern "C" {

/* ---- registration and launch (the stubs nvcc writes for <<<>>>) ---------- */
void** __cudaRegisterFatBinary(void*) { return fatbin_handle; }
void __cudaRegisterFatBinaryEnd(void**) {}
void __cudaUnregisterFatBinary(void**) {}
void __cudaRegisterFunction(void**, const char* hostFun, char*, const char* deviceName, int,
                            uint3*, uint3*, dim3*, dim3*, int*)
{
    functions()[(const void*)hostFun] = deviceName;
}
void __cudaRegisterVar(void**, char*, char*, const char*, int, size_t, int, int) {}
char __cudaInitModule(void**) { return 0; }
unsigned __cudaPushCallConfiguration(dim3 grid, dim3 block, size_t smem, struct CUstream_st* s)
{
    cfgstack().push_back({grid, block, smem, (void*)s});
    return 0;
}
cudaError_t __cudaPopCallConfiguration(dim3* grid, dim3* block, size_t* smem, void* stream)
{
    if (cfgstack().empty()) return cudaErrorInvalidConfiguration;
    LaunchCfg c = cfgstack().back();
    cfgstack().pop_back();
    *grid = c.grid;
    *block = c.block;
    *smem = c.smem;
    *(void**)stream = c.stream;
    return cudaSuccess;
}
cudaError_t __cudaGetKernel(cudaKernel_t* k, const void* func)
{
    *k = (cudaKernel_t)func;
    return cudaSuccess;
}
cudaError_t cudaLaunchKernel(const void* func, dim3 grid, dim3 block, void** args, size_t, cudaStream_t);
cudaError_t __cudaLaunchKernel(cudaKernel_t k, dim3 grid, dim3 block, void** args, size_t smem, cudaStream_t s)
{
    return cudaLaunchKernel((const void*)k, grid, block, args, smem, s);
}
cudaError_t cudaLaunchKernel(const void* func, dim3 grid, dim3 block, void** args, size_t, cudaStream_t)
{
    auto it = functions().find(func);
    if (it == functions().end()) { g_last = cudaErrorInvalidDeviceFunction; return g_last; }
    if (emu_launch(it->second, grid, block, args)) { g_last = cudaErrorInvalidDeviceFunction; return g_last; }
    return cudaSuccess;
}

/* ---- runtime ------------------------------------------------------------- */
cudaError_t cudaGetLastError(void) { cudaError_t e = g_last; g_last = cudaSuccess; return e; }
cudaError_t cudaPeekAtLastError(void) { return g_last; }
const char* cudaGetErrorString(cudaError_t e) { return e == cudaSuccess ? "no error" : "emulated error"; }
const char* cudaGetErrorName(cudaError_t e) { return e == cudaSuccess ? "cudaSuccess" : "cudaErrorEmulated"; }
cudaError_t cudaSetDevice(int) { return cudaSuccess; }
cudaError_t cudaGetDevice(int* d) { *d = 0; return cudaSuccess; }
cudaError_t cudaDeviceSynchronize(void) { return cudaSuccess; }
cudaError_t cudaMalloc(void** p, size_t bytes) { *p = emu_alloc(bytes); return *p ? cudaSuccess : cudaErrorMemoryAllocation; }
cudaError_t cudaMallocHost(void** p, size_t bytes) { *p = emu_alloc(bytes); return *p ? cudaSuccess : cudaErrorMemoryAllocation; }
cudaError_t cudaFree(void* p) { free(p); return cudaSuccess; }
cudaError_t cudaFreeHost(void* p) { free(p); return cudaSuccess; }
cudaError_t cudaMemset(void* p, int v, size_t n) { memset(p, v, n); return cudaSuccess; }
cudaError_t cudaMemcpy(void* d, const void* s, size_t n, enum cudaMemcpyKind) { memmove(d, s, n); return cudaSuccess; }
cudaError_t cudaEventCreate(cudaEvent_t* e) { *e = (cudaEvent_t)emu_alloc(8); return cudaSuccess; }
cudaError_t cudaEventRecord(cudaEvent_t, cudaStream_t) { return cudaSuccess; }
cudaError_t cudaEventSynchronize(cudaEvent_t) { return cudaSuccess; }
cudaError_t cudaEventElapsedTime(float* ms, cudaEvent_t, cudaEvent_t) { *ms = 0.f; return cudaSuccess; }

/* ---- cuFFT --------------------------------------------------------------- */
cufftResult cufftCreate(cufftHandle* h)
{
    plans().push_back(Plan());
    *h = (cufftHandle)(plans().size() - 1);
    return CUFFT_SUCCESS;
}
cufftResult cufftDestroy(cufftHandle) { return CUFFT_SUCCESS; }
cufftResult cufftXtSetGPUs(cufftHandle h, int n, int*)
{
    plans()[h].ngpu = n;
    return CUFFT_SUCCESS;
}
cufftResult cufftMakePlan3d(cufftHandle h, int nx, int ny, int nz, cufftType type, size_t*)
{
    if (type != CUFFT_C2C) return CUFFT_NOT_SUPPORTED;
    Plan& p = plans()[h];
    p.kind = 1; p.n0 = nx; p.n1 = ny; p.n2 = nz;
    return CUFFT_SUCCESS;
}
cufftResult cufftPlan1d(cufftHandle* h, int n, cufftType type, int batch)
{
    if (batch != 1 || (type != CUFFT_R2C && type != CUFFT_C2R)) return CUFFT_NOT_SUPPORTED;
    cufftCreate(h);
    Plan& p = plans()[*h];
    p.kind = type == CUFFT_R2C ? 2 : 3;
    p.n0 = n;
    return CUFFT_SUCCESS;
}
cufftResult cufftExecR2C(cufftHandle h, cufftReal* in, cufftComplex* out)
{
    const Plan& p = plans()[h];
    int n = p.n0;
    std::vector<double> b(2 * n);
    for (int i = 0; i < n; ++i) { b[2 * i] = in[i]; b[2 * i + 1] = 0.0; }
    fft64_plan fp;
    fft64_plan_init(&fp, n);
    std::vector<double> w(4 * n);
    fft64_exec(&fp, b.data(), -1, w.data());
    fft64_plan_free(&fp);
    for (int k = 0; k <= n / 2; ++k) { out[k].x = (float)b[2 * k]; out[k].y = (float)b[2 * k + 1]; }
    return CUFFT_SUCCESS;
}
cufftResult cufftExecC2R(cufftHandle h, cufftComplex* in, cufftReal* out)
{
    const Plan& p = plans()[h];
    int n = p.n0;
    int kmax = (n % 2 == 0) ? n / 2 - 1 : (n - 1) / 2;
    for (int t = 0; t < n; ++t) {
        double acc = in[0].x;
        if (n % 2 == 0) acc += (double)in[n / 2].x * ((t % 2) ? -1.0 : 1.0);
        for (int k = 1; k <= kmax; ++k) {
            long e = ((long)k * t) % n;
            double a = 2.0 * M_PI * (double)e / n;
            acc += 2.0 * ((double)in[k].x * cos(a) - (double)in[k].y * sin(a));
        }
        out[t] = (float)acc;
    }
    return CUFFT_SUCCESS;
}

cufftResult cufftXtMalloc(cufftHandle h, cudaLibXtDesc** desc, cufftXtSubFormat fmt)
{
    const Plan& p = plans()[h];
    cudaLibXtDesc* d = (cudaLibXtDesc*)calloc(1, sizeof(cudaLibXtDesc));
    d->descriptor = (cudaXtDesc*)calloc(1, sizeof(cudaXtDesc));
    d->library = LIB_FORMAT_CUFFT;
    d->subFormat = fmt;
    d->libDescriptor = (void*)(long)h;
    d->descriptor->nGPUs = p.ngpu;
    size_t total = (size_t)p.n0 * p.n1 * p.n2;
    for (int i = 0; i < p.ngpu; ++i) {
        d->descriptor->GPUs[i] = i;
        d->descriptor->size[i] = total / p.ngpu * sizeof(cufftComplex);
        d->descriptor->data[i] = emu_alloc(d->descriptor->size[i]);
    }
    *desc = d;
    return CUFFT_SUCCESS;
}
cufftResult cufftXtFree(cudaLibXtDesc* d)
{
    for (int i = 0; i < d->descriptor->nGPUs; ++i) free(d->descriptor->data[i]);
    free(d->descriptor);
    free(d);
    return CUFFT_SUCCESS;
}

namespace {
/* natural (z-slab) halves <-> full [n0][n1][n2] array */
void desc_to_full(const Plan& p, const cudaLibXtDesc* d, std::vector<double>& full)
{
    const int G = d->descriptor->nGPUs;
    const size_t n0 = p.n0, n1 = p.n1, n2 = p.n2;
    full.assign(2 * n0 * n1 * n2, 0.0);
    for (int g = 0; g < G; ++g) {
        const cufftComplex* s = (const cufftComplex*)d->descriptor->data[g];
        for (size_t a = 0; a < n0 / (d->subFormat == CUFFT_XT_FORMAT_INPLACE_SHUFFLED ? 1 : G); ++a)
            for (size_t b = 0; b < (d->subFormat == CUFFT_XT_FORMAT_INPLACE_SHUFFLED ? n1 / G : n1); ++b)
                for (size_t c = 0; c < n2; ++c) {
                    size_t ga, gb, li;
                    if (d->subFormat == CUFFT_XT_FORMAT_INPLACE_SHUFFLED) {
                        ga = a; gb = g * (n1 / G) + b; li = (a * (n1 / G) + b) * n2 + c;
                    } else {
                        ga = g * (n0 / G) + a; gb = b; li = (a * n1 + b) * n2 + c;
                    }
                    size_t gi = (ga * n1 + gb) * n2 + c;
                    full[2 * gi] = s[li].x;
                    full[2 * gi + 1] = s[li].y;
                }
    }
}
void full_to_desc(const Plan& p, const std::vector<double>& full, cudaLibXtDesc* d, int shuffled)
{
    const int G = d->descriptor->nGPUs;
    const size_t n0 = p.n0, n1 = p.n1, n2 = p.n2;
    d->subFormat = shuffled ? CUFFT_XT_FORMAT_INPLACE_SHUFFLED : CUFFT_XT_FORMAT_INPLACE;
    for (int g = 0; g < G; ++g) {
        cufftComplex* s = (cufftComplex*)d->descriptor->data[g];
        for (size_t a = 0; a < (shuffled ? n0 : n0 / G); ++a)
            for (size_t b = 0; b < (shuffled ? n1 / G : n1); ++b)
                for (size_t c = 0; c < n2; ++c) {
                    size_t ga, gb, li;
                    if (shuffled) { ga = a; gb = g * (n1 / G) + b; li = (a * (n1 / G) + b) * n2 + c; }
                    else { ga = g * (n0 / G) + a; gb = b; li = (a * n1 + b) * n2 + c; }
                    size_t gi = (ga * n1 + gb) * n2 + c;
                    s[li].x = (float)full[2 * gi];
                    s[li].y = (float)full[2 * gi + 1];
                }
    }
}
}  // namespace

cufftResult cufftXtMemcpy(cufftHandle h, void* dst, void* src, cufftXtCopyType type)
{
    const Plan& p = plans()[h];
    size_t total = (size_t)p.n0 * p.n1 * p.n2;
    std::vector<double> full;
    if (type == CUFFT_COPY_HOST_TO_DEVICE) {
        const cufftComplex* s = (const cufftComplex*)src;
        full.resize(2 * total);
        for (size_t i = 0; i < total; ++i) { full[2 * i] = s[i].x; full[2 * i + 1] = s[i].y; }
        full_to_desc(p, full, (cudaLibXtDesc*)dst, 0);
    } else if (type == CUFFT_COPY_DEVICE_TO_HOST) {
        desc_to_full(p, (const cudaLibXtDesc*)src, full);
        cufftComplex* d = (cufftComplex*)dst;
        for (size_t i = 0; i < total; ++i) { d[i].x = (float)full[2 * i]; d[i].y = (float)full[2 * i + 1]; }
    } else {
        desc_to_full(p, (const cudaLibXtDesc*)src, full);
        full_to_desc(p, full, (cudaLibXtDesc*)dst, ((cudaLibXtDesc*)src)->subFormat == CUFFT_XT_FORMAT_INPLACE_SHUFFLED);
    }
    return CUFFT_SUCCESS;
}

cufftResult cufftXtExecDescriptorC2C(cufftHandle h, cudaLibXtDesc* in, cudaLibXtDesc* out, int dir)
{
    const Plan& p = plans()[h];
    std::vector<double> full;
    desc_to_full(p, in, full);
    /* [n0][n1][n2] with n2 fastest */
    if (fft64_3d(full.data(), p.n2, p.n1, p.n0, dir == CUFFT_FORWARD ? -1 : +1)) return CUFFT_EXEC_FAILED;
    full_to_desc(p, full, out, dir == CUFFT_FORWARD ? 1 : 0);
    return CUFFT_SUCCESS;
}

}  // extern "C"
