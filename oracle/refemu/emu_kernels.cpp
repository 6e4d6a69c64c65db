/*
 * emu_kernels.cpp - the reference's device kernels (ose_3d_kernel.cu, included
 * unmodified from the reference tree at build time) compiled for the HOST, one
 * call per CUDA thread.  TEST INFRASTRUCTURE: builds oracle/_ref/ref_ose, the
 * reference run on this machine to pin the oracle.
 *
 * The reference kernels are plain SIMT code with no shared memory, barriers or
 * atomics (ose_3d_kernel.cu:1-436), so running the threads one after another
 * gives exactly what the GPU computes, up to the device math library
 * (expf, jnf, sqrt, pow come from the host libm here).
 */
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <cufft.h>          /* cufftComplex (float2) */
#include <vector_types.h>   /* dim3, uint3            */

#undef __global__
#undef __device__
#undef __host__
#define __global__
#define __device__
#define __host__

namespace emu {
uint3 threadIdx, blockIdx;
dim3 blockDim, gridDim;
#define pai 3.14159265359
#include "ose_3d_kernel.cu"
#undef pai
}  // namespace emu

namespace {

#define A(T, i) (*(T*)args[i])
typedef cufftComplex C;

struct Entry {
    const char* name;
    void (*call)(void** args);
};

void k_generate_wavelet_gpu(void** args) { emu::generate_wavelet_gpu(A(float*, 0), A(float, 1), A(int, 2), A(float, 3), A(float, 4)); }
void k_hilbert_1d(void** args) { emu::hilbert_1d(A(C*, 0), A(int, 1)); }
void k_scale_wavelet(void** args) { emu::scale_wavelet(A(float*, 0), A(int, 1)); }
void k_sg_init_device(void** args) { emu::sg_init_device(A(int*, 0), A(int, 1), A(int, 2), A(int, 3), A(int, 4), A(int, 5), A(int, 6), A(int, 7), A(int, 8), A(int, 9)); }
void k_Xtdata_devide_value(void** args) { emu::Xtdata_devide_value(A(C*, 0), A(int, 1), A(int, 2), A(int, 3), A(int, 4), A(float, 5)); }
void k_generate_att(void** args) { emu::generate_att(A(float*, 0), A(int, 1), A(int, 2), A(int, 3)); }
void k_apply_ABC_Xt(void** args) { emu::apply_ABC_Xt(A(C*, 0), A(float*, 1), A(float*, 2), A(float*, 3), A(int, 4), A(int, 5), A(int, 6), A(int, 7)); }
void k_add_wavelet_Xt(void** args) { emu::add_wavelet_Xt(A(C*, 0), A(float*, 1), A(int, 2), A(int, 3), A(int, 4), A(int, 5), A(int, 6), A(int, 7), A(int, 8), A(int, 9), A(int, 10), A(int, 11), A(int, 12)); }
void k_step1to4_3d(void** args) { emu::step1to4_3d(A(C*, 0), A(int, 1), A(int, 2), A(int, 3), A(float, 4), A(int, 5)); }
void k_memcpy_between_device_cr(void** args) { emu::memcpy_between_device_cr(A(C*, 0), A(C*, 1), A(int, 2), A(int, 3), A(int, 4)); }
void k_scale_kxkz_3D(void** args) { emu::scale_kxkz_3D(A(C*, 0), A(int, 1), A(int, 2), A(int, 3), A(int, 4), A(float, 5), A(float, 6), A(float, 7)); }
void k_scal_vr_3d(void** args) { emu::scal_vr_3d(A(C*, 0), A(C*, 1), A(C*, 2), A(float, 3), A(int, 4), A(int, 5), A(int, 6), A(float, 7), A(bool, 8)); }
void k_add_bessel_3d(void** args) { emu::add_bessel_3d(A(C*, 0), A(C*, 1), A(float, 2), A(int, 3), A(int, 4), A(int, 5), A(int, 6)); }
void k_replace_2array_3d(void** args) { emu::replace_2array_3d(A(C*, 0), A(C*, 1), A(int, 2), A(int, 3), A(int, 4)); }
void k_rec_shotdata_3d(void** args) { emu::rec_shotdata_3d(A(C*, 0), A(float*, 1), A(int*, 2), A(int, 3), A(int, 4), A(int, 5), A(int, 6), A(int, 7), A(int, 8), A(int, 9), A(int, 10), A(int, 11), A(int, 12)); }

const Entry kTable[] = {
    {"generate_wavelet_gpu", k_generate_wavelet_gpu},
    {"hilbert_1d", k_hilbert_1d},
    {"scale_wavelet", k_scale_wavelet},
    {"sg_init_device", k_sg_init_device},
    {"Xtdata_devide_value", k_Xtdata_devide_value},
    {"generate_att", k_generate_att},
    {"apply_ABC_Xt", k_apply_ABC_Xt},
    {"add_wavelet_Xt", k_add_wavelet_Xt},
    {"step1to4_3d", k_step1to4_3d},
    {"memcpy_between_device_cr", k_memcpy_between_device_cr},
    {"scale_kxkz_3D", k_scale_kxkz_3D},
    {"scal_vr_3d", k_scal_vr_3d},
    {"add_bessel_3d", k_add_bessel_3d},
    {"replace_2array_3d", k_replace_2array_3d},
    {"rec_shotdata_3d", k_rec_shotdata_3d},
};

}  // namespace

/* Find the emulated kernel whose Itanium-mangled name is in device_name
 * ("<len><name>") and run every thread of the grid. Returns 0 on success. */
extern "C" int emu_launch(const char* device_name, dim3 grid, dim3 block, void** args)
{
    for (const Entry& e : kTable) {
        char key[128];
        snprintf(key, sizeof key, "%zu%s", strlen(e.name), e.name);
        if (!strstr(device_name, key)) continue;
        emu::gridDim = grid;
        emu::blockDim = block;
        for (unsigned bz = 0; bz < grid.z; ++bz)
            for (unsigned by = 0; by < grid.y; ++by)
                for (unsigned bx = 0; bx < grid.x; ++bx)
                    for (unsigned tz = 0; tz < block.z; ++tz)
                        for (unsigned ty = 0; ty < block.y; ++ty)
                            for (unsigned tx = 0; tx < block.x; ++tx) {
                                emu::blockIdx.x = bx; emu::blockIdx.y = by; emu::blockIdx.z = bz;
                                emu::threadIdx.x = tx; emu::threadIdx.y = ty; emu::threadIdx.z = tz;
                                e.call(args);
                            }
        return 0;
    }
    fprintf(stderr, "refemu: no host version of kernel %s\n", device_name);
    return 1;
}
