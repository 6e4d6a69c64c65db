/*
 * ref_main.cu - drives the reference's own host library and kernels
 * (ose_3d_lib.cu and ose_3d_kernel.cu, #included unmodified from the reference
 * tree) through one shot with parameters read from a key=value file, on the
 * host emulation of emu_runtime.cpp / emu_kernels.cpp.
 * TEST INFRASTRUCTURE: the resulting binary oracle/_ref/ref_ose generates the
 * golden files of tests/golden/ and pins oracle/ose_oracle.c.
 *
 * The setup sequence is the one of main() (ose_3d.cu:79-276) with the
 * hard-coded values replaced by the file's; everything it calls is the
 * reference's code.  Outputs land in the working directory's output/, temp/
 * and wf/ folders, as in the reference.
 *
 * Usage: ref_ose params.txt     (keys: nx ny nz bu bd bl br bf bb nt nsteps fm
 *                                dt amp dx dy dz sxbeg sybeg szbeg model)
 */
#include <time.h>
#include <stdlib.h>
#include <stdio.h>
#include <string.h>
#include <math.h>
#define pai 3.14159265359
#include <cufftXt.h>
#include <cufft.h>
#include "su.h"
#include "segy.h"
#include "Complex.h"
#include <cuda_runtime.h>
#include <helper_functions.h>
#include <helper_cuda.h>
#include <timer.h>
#define BLOCK_SIZE_X 16
#define BLOCK_SIZE_Y 16

typedef float2 Complex;
#define batch 1

/* The global parameter block the reference library reads and writes
 * (names and types are its interface, ose_3d.cu:42-65). */
int nGPUs, M;
int nx, ny, nz, nt, bu, bd, bl, br, bf, bb, nxb, nyb, nzb, sxbeg, sybeg, szbeg, jsx, jsy, jsz,
    gxbeg, gybeg, gzbeg, jgx, jgy, jgz, csdgather, ng, nshot, is, it, sx, sy, sz, boundary;
float fm, dt, amp, dx, dy, dz, vmax, R, dtR, dkx, dky, dkz;
int *sxyz_h, *gxyz_h, *sxyz_d, *gxyz_d;
float *wavelet_h, *wavelet_d, *wavelethilbert_d;
cufftComplex* cwavelet_d;
float *wavelet_card, *wavelethilbert_card;
cufftComplex* cwavelet_card;
float *fdata_3dH, *fdata_3dD, *vb_3dH;
cufftComplex *cdata_3dH, *cvb_3dH;
cudaLibXtDesc *p1D, *p2D, *q1D, *q2D, *pcD, *vbD;
float *att_blr, *att_bfb, *att_bud;
float* att_host;
float *rec_slice_d, *rec_slice_h, *rec_data_h;
char parname[500];
char filename[500];

#include "ose_3d_kernel.cu"
#include "ose_3d_lib.cu"

static int get_key(const char* path, const char* key, char* out, size_t cap)
{
    FILE* f = fopen(path, "r");
    if (!f) return 0;
    char line[1024];
    int found = 0;
    while (fgets(line, sizeof line, f)) {
        char k[256], v[768];
        if (sscanf(line, " %255[^= ] = %767s", k, v) == 2 && strcmp(k, key) == 0) {
            snprintf(out, cap, "%s", v);
            found = 1;
        }
    }
    fclose(f);
    return found;
}
static int geti(const char* path, const char* key, int def)
{
    char v[768];
    return get_key(path, key, v, sizeof v) ? atoi(v) : def;
}
static float getf(const char* path, const char* key, float def)
{
    char v[768];
    return get_key(path, key, v, sizeof v) ? (float)atof(v) : def;
}

int main(int argc, char** argv)
{
    if (argc < 2) { fprintf(stderr, "usage: %s params.txt\n", argv[0]); return 2; }
    const char* pf = argv[1];
    char model[768];
    if (!get_key(pf, "model", model, sizeof model)) { fprintf(stderr, "no model= key\n"); return 2; }

    nx = geti(pf, "nx", 101); ny = geti(pf, "ny", 101); nz = geti(pf, "nz", 101);
    bu = geti(pf, "bu", 25); bd = geti(pf, "bd", 25); bl = geti(pf, "bl", 25);
    br = geti(pf, "br", 25); bf = geti(pf, "bf", 25); bb = geti(pf, "bb", 25);
    nxb = bl + nx + br; nyb = bf + ny + bb; nzb = bu + nz + bd;
    nxb = judge_odd(&br, &nxb);
    nyb = judge_odd(&bb, &nyb);
    nzb = judge_odd(&bd, &nzb);
    nt = geti(pf, "nt", 300);
    int nsteps = geti(pf, "nsteps", nt);
    fm = getf(pf, "fm", 40.0f);
    dt = getf(pf, "dt", 0.001f);
    amp = getf(pf, "amp", 100.0f);
    ng = nx * ny;
    nshot = 1;
    sxbeg = geti(pf, "sxbeg", nx / 2); sybeg = geti(pf, "sybeg", ny / 2); szbeg = geti(pf, "szbeg", 0);
    gxbeg = 0; gybeg = 0; gzbeg = 0;
    jsx = jsy = jsz = 1; jgx = jgy = jgz = 1;
    csdgather = 0;
    nGPUs = 2;
    dx = getf(pf, "dx", 10.0f); dy = getf(pf, "dy", 10.0f); dz = getf(pf, "dz", 10.0f);
    dkx = 2 * pai / dx / (float)nxb;
    dky = 2 * pai / dy / (float)nyb;
    dkz = 2 * pai / dz / (float)nzb;
    if (nxb > 300) { fprintf(stderr, "nxb > 300 overflows att_host in Alloc_mulGPU\n"); return 2; }
    sprintf(parname, "./output/partest.txt");

    dim3 dimBlock2D(BLOCK_SIZE_X, BLOCK_SIZE_Y);
    dim3 dimBlock_nt(BLOCK_SIZE_X, 1);
    dim3 dimGrid_nt((nt + dimBlock_nt.x - 1) / dimBlock_nt.x, 1);
    dim3 dimGrid3D_half_before_tran((nxb + 1 + dimBlock2D.x - 1) / dimBlock2D.x,
                                    (nyb + dimBlock2D.y - 1) / dimBlock2D.y, nzb / 2);

    Alloc();
    sg_init_host(sxyz_h, sxbeg, sybeg, szbeg, jsx, jsy, jsz, nshot, nx, ny);
    sg_init_host(gxyz_h, sxbeg, sybeg, szbeg, jsx, jsy, jsz, nshot, nx, ny);
    sg_init_device<<<1, 1>>>(gxyz_d, gxbeg, gybeg, gzbeg, jgx, jgy, jgz, ng, nx, ny);

    snprintf(filename, sizeof filename, "%s", model);
    input_file_xyz_boundary(filename, vb_3dH, nx, ny, nz, bl, bf, bu, nxb, nyb, nzb);
    add_pml_layers_v_h(vb_3dH, nx, ny, nz, bl, bf, bu, nxb, nyb, nzb);
    data_R2CR(vb_3dH, cvb_3dH, nxb, nyb, nzb);
    write_1dfile_from_1darray((char*)"./temp/vpad.bin", vb_3dH, nxb * nyb * nzb);

    Alloc_mulGPU();
    cudaMemcpy(att_host, att_bfb, nyb * sizeof(float), cudaMemcpyDefault);
    write_1dfile_from_1darray((char*)"./temp/att_y.bin", att_host, nyb);
    cudaMemcpy(att_host, att_bud, nzb * sizeof(float), cudaMemcpyDefault);
    write_1dfile_from_1darray((char*)"./temp/att_z.bin", att_host, nzb);

    generate_wavelet_gpu<<<1, 1>>>(wavelet_d, fm, nt, dt, amp);
    cudaMemcpy(wavelet_h, wavelet_d, nt * sizeof(float), cudaMemcpyDefault);
    write_1dfile_from_1darray((char*)"./temp/ricker.bin", wavelet_h, nt);

    cufftHandle plan_1d, plan_1d_r;
    checkCudaErrors(cufftPlan1d(&plan_1d, nt, CUFFT_R2C, 1));
    checkCudaErrors(cufftPlan1d(&plan_1d_r, nt, CUFFT_C2R, 1));
    checkCudaErrors(cufftExecR2C(plan_1d, wavelet_d, cwavelet_d));
    hilbert_1d<<<dimGrid_nt, dimBlock_nt>>>(cwavelet_d, nt);
    checkCudaErrors(cufftExecC2R(plan_1d_r, cwavelet_d, wavelethilbert_d));
    scale_wavelet<<<dimGrid_nt, dimBlock_nt>>>(wavelethilbert_d, nt);
    cudaMemcpy(wavelet_h, wavelethilbert_d, nt * sizeof(float), cudaMemcpyDefault);
    write_1dfile_from_1darray((char*)"./temp/ricker_hil.bin", wavelet_h, nt);

    vmax = find_max(vb_3dH, nxb * nyb * nzb);
    R = vmax * PI * sqrt(pow(1.0 / dx, 2.0) + pow(1.0 / dy, 2.0) + pow(1.0 / dz, 2.0));
    dtR = dt * R;
    M = (int)dtR + 6;
    R2C_3D_CPU(cdata_3dH, fdata_3dH, nxb, nyb, nzb, TRUE);

    cufftHandle plan_input;
    cufftResult result = cufftCreate(&plan_input);
    int whichGPUs[2] = {0, 1};
    result = cufftXtSetGPUs(plan_input, nGPUs, whichGPUs);
    size_t worksize[2];
    result = cufftMakePlan3d(plan_input, nzb, nyb, nxb, CUFFT_C2C, worksize);
    if (result != CUFFT_SUCCESS) { fprintf(stderr, "plan failed\n"); return 3; }
    Alloc_cufftXt(plan_input, result);
    result = cufftXtMemcpy(plan_input, p1D, cdata_3dH, CUFFT_COPY_HOST_TO_DEVICE);
    result = cufftXtMemcpy(plan_input, vbD, cvb_3dH, CUFFT_COPY_HOST_TO_DEVICE);

    for (is = 0; is < nshot; is++) {
        Xtdata_value(p1D, p2D, q1D, q2D, pcD, nxb, nyb, nzb, 0.0);
        Alloc_wavelet(is, plan_1d, plan_1d_r);
        for (it = 0; it < nsteps; it++) {
            Xt_add_wavelet_sxyz(p2D, wavelet_card, sxyz_h, is);
            Xt_add_wavelet_sxyz(q2D, wavelethilbert_card, sxyz_h, is);
            wavefield_extro_ori2(plan_input, result);
            rec_shotdata_3d<<<dimGrid3D_half_before_tran, dimBlock2D>>>(
                (cufftComplex*)q2D->descriptor->data[0], rec_slice_d, gxyz_d, nx, ny, nz, bl, bf, bu,
                nxb, nyb, nzb, ng);
            cudaMemcpy(rec_slice_h, rec_slice_d, ng * sizeof(float), cudaMemcpyDefault);
            rec_slice_to_data(rec_slice_h, rec_data_h, ng, it);
        }
        write_3dfile_from_1darray((char*)"./output/qshot2.bin", rec_data_h, ng, 1, nt);
        /* final state, in the ./wf dump layout [y][x][z] (ose_3d.cu:260-269) */
        result = cufftXtMemcpy(plan_input, cdata_3dH, q2D, CUFFT_COPY_DEVICE_TO_HOST);
        write_3dfile_from_1darray_ci((char*)"./wf/q-final.bin", cdata_3dH, nxb, nyb, nzb);
        result = cufftXtMemcpy(plan_input, cdata_3dH, p2D, CUFFT_COPY_DEVICE_TO_HOST);
        write_3dfile_from_1darray_ci((char*)"./wf/p-final.bin", cdata_3dH, nxb, nyb, nzb);
        Free_wavelet(is);
    }
    Output();
    printf("nxb=%d nyb=%d nzb=%d vmax=%f R=%f dtR=%f M=%d\n", nxb, nyb, nzb, vmax, R, dtR, M);
    Free_cufftXt(plan_input, result);
    Free();
    return 0;
}
