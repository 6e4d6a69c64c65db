/*
 * ose3d.h - C ABI of libose3d.so, a single-GPU (sm_103a) one-step-extrapolation
 * (OSE) acoustic modeler.
 *
 * The reference program (Littleke/3D-OSE) is one executable whose "interface"
 * is its global parameter block (ose_3d.cu:42-63) and the host functions that
 * main() calls around its time loop (ose_3d.cu:145-279).  Every entry point
 * below replaces one group of those calls; the citation on each says which.
 *
 * Conventions
 *   - Every function returns an ose_status (0 = OSE_OK).  Nothing throws across
 *     the ABI and nothing calls exit().  ose_last_error() gives the message of
 *     the last failure on a handle (or of ose_create when the handle is NULL).
 *   - The library owns all device memory of a handle.  The caller owns every
 *     host buffer; the library copies into and out of them.
 *   - One host thread per handle at a time.  Several handles may coexist; each
 *     runs on its own CUDA stream on the current device.
 *   - Grids: nx, ny, nz are INTERIOR sizes.  Padded sizes are
 *     nxb = bl + nx + br etc., with the trailing pad bumped by one when the
 *     sum is odd (judge_odd, ose_3d_lib.cu:36-44).  Device fields are stored
 *     [z][y][x] with x fastest (ose_3d.cu:226, plan dims (nzb, nyb, nxb)).
 */
#ifndef OSE3D_H
#define OSE3D_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum ose_status {
    OSE_OK = 0,
    OSE_ERR_INVALID = 1,      /* bad argument or parameter */
    OSE_ERR_CUDA = 2,         /* a CUDA runtime call failed */
    OSE_ERR_NOMEM = 3,        /* device or host allocation failed */
    OSE_ERR_IO = 4,           /* file could not be read or written */
    OSE_ERR_UNSUPPORTED = 5,  /* size or mode outside what the kernels handle */
    OSE_ERR_STATE = 6,        /* call out of order (e.g. ose_step before ose_reset_shot) */
    OSE_ERR_NUMERIC = 7,      /* non-finite value found in the wavefield */
    OSE_ERR_TIMEOUT = 8       /* a bounded wait inside a kernel ran out of time (2 s for the
                                 plane exchange and the batch's grid barrier, 1 s for an MMA
                                 completion); the results of that call are invalid, the
                                 device context stays usable */
} ose_status;

/* Sponge profile.  REFERENCE is generate_att (ose_3d_kernel.cu:242-261):
 * exp(-((b-1-i)/b)^2) on the leading side, exp(-((i+1)/a)^2) on the trailing
 * side, applied to the partial sum once per series term.  CERJAN is the
 * classical exp(-(alpha*d)^2) taper, d = distance into the sponge in cells. */
enum { OSE_SPONGE_REFERENCE = 0, OSE_SPONGE_CERJAN = 1 };

/* Which field ose_get_wavefield / ose_set_wavefield address. */
enum { OSE_FIELD_P = 0, OSE_FIELD_Q = 1, OSE_FIELD_V = 2 };

/* Host layouts of a padded field. */
enum {
    OSE_LAYOUT_ZYX = 0,  /* [z][y][x], x fastest: the device layout          */
    OSE_LAYOUT_YXZ = 1   /* [y][x][z], z fastest: write_3dfile_from_1darray_ci
                            (ose_3d_lib.cu:364-380), the per-step wf dump */
};

/* Parameter block: the reference's hard-coded globals (ose_3d.cu:42-44,
 * 75-118) plus a few switches whose zero value reproduces the reference. */
typedef struct ose_params {
    int nx, ny, nz;                 /* interior cells                        */
    int bu, bd, bl, br, bf, bb;     /* sponge widths: up/down (z), left/right (x), front/back (y) */
    int nt;                         /* time steps per shot                   */
    float fm;                       /* Ricker peak frequency (Hz)            */
    float dt;                       /* time step (s)                         */
    float amp;                      /* Ricker amplitude                      */
    float dx, dy, dz;               /* cell sizes (m)                        */
    int nshot;                      /* shots (the reference runs 1)          */
    int sxbeg, sybeg, szbeg;        /* first source, interior cell indices   */
    int jsx, jsy, jsz;              /* source step between shots             */
    int gxbeg, gybeg, gzbeg;        /* receiver origin; gzbeg = receiver depth */
    int jgx, jgy, jgz;              /* receiver steps (kept for partest.txt)  */
    int csdgather;                  /* kept for partest.txt                  */
    /* switches; 0 = reference behaviour */
    int sponge_mode;                /* OSE_SPONGE_*                          */
    float cerjan_factor;            /* alpha for OSE_SPONGE_CERJAN (e.g. 0.015) */
    int hilbert_div_nt;             /* 1: divide the Q source trace by nt.  The
                                       reference does not (ose_3d_lib.cu:578-581),
                                       so Q receives nt x the Hilbert transform. */
    int M_override;                 /* >0: series order M; 0: (int)(dt*R) + 6
                                       (ose_3d.cu:196-197)                   */
} ose_params;

/* Values derived from the parameters and the model (ose_3d.cu:85-90,120-122,
 * 191-199), as used by the kernels. */
typedef struct ose_derived {
    int nxb, nyb, nzb;              /* padded sizes                          */
    int br, bb, bd;                 /* trailing pads after the even-size fix */
    int ng;                         /* receivers per shot = nx*ny            */
    int M;                          /* series order: M+1 operator applications per step */
    float vmax;                     /* max velocity of the padded model      */
    double R;                       /* spectral radius bound vmax*pi*sqrt(1/dx^2+1/dy^2+1/dz^2) */
    double dtR;                     /* dt*R                                  */
    double dkx, dky, dkz;           /* 2*pi/(d*nb)                           */
    double bessel_tail;             /* |J_{M+2}(dtR)|: first dropped series coefficient */
    size_t device_bytes;            /* device memory held by the handle      */
    int path;                       /* kernel family in use (OSE_PATH_*)     */
} ose_derived;

/* Kernel families: GENERIC = five-pass FFT operator for any even size up to
 * 1024 per axis; PLANE = two-pass cluster path for 256^3 padded grids. */
enum { OSE_PATH_GENERIC = 0, OSE_PATH_PLANE = 1 };

typedef struct ose_handle ose_handle;

/* Fill *p with the reference main()'s hard-coded values (ose_3d.cu:75-118). */
ose_status ose_default_params(ose_params* p);

/* Padded sizes of a parameter block (judge_odd, ose_3d_lib.cu:36-44). */
ose_status ose_padded_dims(const ose_params* p, int* nxb, int* nyb, int* nzb);

/* Create a handle: pad the interior model, build sponge, series and |k|
 * tables, allocate and upload.  Replaces Alloc + input_file_xyz_boundary +
 * add_pml_layers_v_h + data_R2CR + Alloc_mulGPU + find_max + R/M + the
 * cufftXt plan/malloc/memcpy block (ose_3d.cu:145-237).
 * vel_xyz: nx*ny*nz floats in the reference model layout [x][y][z], z fastest
 * (input_file_xyz_boundary, ose_3d_lib.cu:887-909). */
ose_status ose_create(const ose_params* p, const float* vel_xyz, ose_handle** out);

/* Same, reading the raw float32 model file (ose_3d.cu:157-158). */
ose_status ose_create_from_file(const ose_params* p, const char* path, ose_handle** out);

/* Release every resource of the handle (Free_cufftXt + cufftDestroy + Free,
 * ose_3d.cu:286-298).  NULL is accepted. */
ose_status ose_destroy(ose_handle* h);

/* Message of the last failure on h (or of the last failed ose_create when h
 * is NULL).  The string stays valid until the next call on h. */
const char* ose_last_error(const ose_handle* h);

ose_status ose_get_derived(const ose_handle* h, ose_derived* d);

/* Self test of the bounded waits inside the kernels (no counterpart in the
 * reference, which has none): one single-CTA kernel per kind waits on
 * something that never completes — the plane kernels' DSMEM exchange
 * mbarrier, the persistent batch's grid barrier, the tensor-core MMA
 * completion barrier — with a limit of limit_ms (0 < limit_ms <= 100) instead
 * of the production 1-2 s.  *expired gets bit 0, 1, 2 set for each wait that
 * ran out and recorded it in its error word (7 = all three behave); the
 * device context stays usable.  Runs on its own stream; no handle needed
 * (ose_last_error(NULL) on failure). */
ose_status ose_self_test_waits(double limit_ms, int* expired);

/* Start shot `is`: zero P and Q, rebuild the shot's Ricker and Hilbert traces,
 * clear the device gather and set it = 0.  Replaces Xtdata_value +
 * Alloc_wavelet (ose_3d.cu:245-246, ose_3d_lib.cu:513-586). */
ose_status ose_reset_shot(ose_handle* h, int is);

/* One time step: inject the source sample of step it into P and Q,
 * advance (P, Q) by dt with the OSE series, record Q on the receiver plane
 * into the device gather row it, it += 1.  Replaces the body of the time loop
 * (ose_3d.cu:252-274): Xt_add_wavelet_sxyz x2, wavefield_extro_ori2,
 * rec_shotdata_3d and rec_slice_to_data. */
ose_status ose_step(ose_handle* h);

/* nsteps time steps as one replay of a captured CUDA graph (one step per
 * graph node group; the step index lives in device memory).  gather_out may
 * be NULL; otherwise it receives the WHOLE gather of the shot so far in the
 * reference file order [ig][it] (ng x nt floats, write_3dfile_from_1darray
 * with (ng,1,nt), ose_3d_lib.cu:327-343); rows of steps not run yet are 0. */
ose_status ose_run(ose_handle* h, int nsteps, float* gather_out);

/* nsteps steps, copying each step's receiver row to the host as the
 * reference's loop does (rec_shotdata_3d + cudaMemcpy of ng floats +
 * rec_slice_to_data, ose_3d.cu:271-274).  rows_out receives nsteps x ng
 * floats in step order [it][ig] (the rows of those steps only). */
ose_status ose_run_record(ose_handle* h, int nsteps, float* rows_out);

/* As ose_run, but times the device work with CUDA events on the handle's
 * stream and copies nothing back.  *ms receives the elapsed device time. */
ose_status ose_run_timed(ose_handle* h, int nsteps, float* ms);

/* Choose the kernel family: OSE_PATH_PLANE (256^3 padded grids only; the
 * default there) or OSE_PATH_GENERIC (any size).  Both compute the same
 * step; the choice exists for comparison and testing. */
ose_status ose_select_path(ose_handle* h, int path);

/* Arithmetic of the z-axis transforms (the precision form; no counterpart in
 * the reference, whose transforms are cuFFT FP32).  FP32 is the FFT kernels.
 * The others run the z pass (FFT_z, * |k|, IFFT_z) as four batched DFT-16
 * matmuls on the tensor cores with FP32 accumulation: TF32 one pass; TF32X3
 * and BF16X3 split each operand into hi + lo parts and add the three products
 * lo*hi + hi*lo + hi*hi.  Needs nzb = 256 and nxb a multiple of 16
 * (OSE_ERR_UNSUPPORTED otherwise); works with either path. */
enum {
    OSE_PRECISION_FP32 = 0,
    OSE_PRECISION_TF32 = 1,
    OSE_PRECISION_TF32X3 = 2,
    OSE_PRECISION_BF16X3 = 3
};
ose_status ose_set_precision(ose_handle* h, int mode);
ose_status ose_get_precision(const ose_handle* h, int* mode);

/* Receivers at an explicit list of interior cells (xyz: n triplets x, y, z,
 * 0-based interior coordinates) instead of the plane at depth gzbeg.  This is
 * the reference's gxyz geometry (sg_init_device, ose_3d_kernel.cu:202-212:
 * receiver i at (gxbeg + i jgx, gybeg + i jgy, gzbeg + i jgz)), which its
 * rec_shotdata_3d leaves unused in favour of the full surface plane
 * (ose_3d_kernel.cu:412-436); here it is honoured.  ng becomes n; the gather,
 * SU/SEG-Y headers and reverse-time migration follow the list.  n = 0 returns
 * to the plane.  Clears the gather. */
ose_status ose_set_receivers(ose_handle* h, int n, const int* xyz);

/* ---- learned boundary corrector (no counterpart in the reference) --------
 * A 3D convolutional network (4 layers of 3x3x3 convolutions, 8 -> 32 -> 32
 * -> 32 -> 2 channels, ReLU, ose_corrector_param_count() FP32 parameters)
 * that runs on the SHELL of the padded grid (cells within `shell` cells of a
 * face; the grid is periodic) and adds a correction to P and Q at the shell
 * cells outside the sponge, so that a thin sponge behaves like a wide one.
 * Inputs per cell: P/s, Q/s (s = RMS of P, Q over the shell), v/4500 and the
 * signed closeness to the nearest face of each axis.  Parameter layout: per
 * layer W[27][Cin][Cout] (tap = (dz+1)*9 + (dy+1)*3 + (dx+1)) then b[Cout];
 * layer 0 has Cin = 8 (channels 6, 7 are zero). */
#define OSE_CORRECTOR_SHELL 16
typedef struct ose_corrector ose_corrector;

/* Attach a trained corrector to a modeler (params: host, param_count floats;
 * NULL detaches).  Every time step then ends with the correction, inside the
 * captured graph.  The receiver row of a step is recorded before it. */
ose_status ose_set_corrector(ose_handle* h, const float* params, int shell);

/* Copy a box of the state (P + iQ as float pairs, [z][y][x]) to or from a
 * caller-owned DEVICE buffer: dir 0 state -> buffer, 1 buffer -> state.
 * box = {x0, y0, z0, nx, ny, nz} in the padded grid; buf = {bnx, bny, bx0,
 * by0, bz0}: the buffer's x and y sizes and the box's origin in it.  For
 * pipelines that pair two modelers on the device (training data). */
ose_status ose_state_box(ose_handle* h, int dir, const int* box, void* buf_dev, const int* buf);

/* Training objects: every call takes device pointers (state and target as
 * float pairs [z][y][x] on the corrector's grid, velocity as floats) and runs
 * on the legacy default stream, ordered with the caller's default-stream work. */
size_t ose_corrector_param_count(void);
ose_status ose_corrector_create(int nxb, int nyb, int nzb, int shell, const int* sponge6, ose_corrector** out);
ose_status ose_corrector_destroy(ose_corrector* c);
const char* ose_corrector_last_error(const ose_corrector* c);
ose_status ose_corrector_info(const ose_corrector* c, long long* shell_cells, long long* write_cells, int* tiles);
ose_status ose_corrector_set_params(ose_corrector* c, const float* params);
ose_status ose_corrector_get_params(ose_corrector* c, float* params);
ose_status ose_corrector_get_grads(ose_corrector* c, float* grads);
/* Network output (dP, dQ)/s per cell ([cell][2] floats, written at shell
 * cells) and the scale s. */
ose_status ose_corrector_forward(ose_corrector* c, const void* state_dev, const float* vel_dev, float* out_dev,
                                 float* scale_out);
/* state += s * output at the write cells (what a modeler's step does). */
ose_status ose_corrector_apply(ose_corrector* c, void* state_dev, const float* vel_dev);
/* Forward + backward of one sample: loss = mean over write cells of
 * |output - (target - state)/s|^2; gradients and loss accumulate. */
ose_status ose_corrector_train_sample(ose_corrector* c, const void* state_dev, const float* vel_dev,
                                      const void* target_dev);
/* Adam step (beta 0.9, 0.999) on the gradients accumulated over `batch`
 * samples, which it clears; *mean_loss = their mean loss. */
ose_status ose_corrector_adam(ose_corrector* c, float lr, int batch, float* mean_loss);
/* Accumulated loss; reset != 0 also clears it and the gradients. */
ose_status ose_corrector_loss(ose_corrector* c, float* loss, int reset);

/* Reverse-time migration of the current shot (ose_3d.cu:127 names an "rtm
 * result"; the reference has no migration code): forward-propagate the source
 * for nsteps steps keeping P on the device every `every` steps, then
 * propagate the observed receiver rows (host, nsteps x ng, [it][ig] as
 * ose_run_record returns them; the receivers record Q) backwards in time,
 * injected at the receivers as their analytic pair, and accumulate the
 * zero-lag cross-correlation image += P_source * P_receiver at the kept steps.
 * image: padded [z][y][x] floats; illum (may be NULL): the source
 * illumination sum P_source^2 at the same steps, the usual normaliser of the
 * image.  Device memory: nsteps/every + 3 padded fields.  Uses the handle's
 * model as the migration velocity; afterwards the state is the receiver
 * wavefield at time 0 and a new ose_reset_shot is needed to step again. */
ose_status ose_rtm(ose_handle* h, const float* rows, int nsteps, int every, float* image, float* illum);

/* Steps taken in the current shot. */
ose_status ose_get_it(const ose_handle* h, int* it);

/* Copy a padded field to host (OSE_FIELD_P, _Q or _V) in the given layout.
 * out holds nxb*nyb*nzb floats. */
ose_status ose_get_wavefield(ose_handle* h, int which, float* out, int layout);

/* Overwrite P or Q from a host buffer (padded, given layout). */
ose_status ose_set_wavefield(ose_handle* h, int which, const float* in, int layout);

/* Gather of the current shot in [ig][it] order (ng x nt floats). */
ose_status ose_get_gather(ose_handle* h, float* out);

/* The shot's source traces (nt floats each): the Ricker added to P and the
 * Hilbert trace added to Q (generate_wavelet_gpu + hilbert_1d + C2R,
 * ose_3d_lib.cu:575-583). */
ose_status ose_get_wavelets(const ose_handle* h, float* ricker, float* hilbert);

/* The 1-D sponge tables (nxb, nyb, nzb floats; generate_att). */
ose_status ose_get_sponge(const ose_handle* h, float* ax, float* ay, float* az);

/* Apply the normalised operator once to a packed complex field:
 *   out = v * IFFT3(|k| * FFT3(in)) / (R * nxb*nyb*nzb)
 * in/out are host arrays of nxb*nyb*nzb interleaved (re, im) float pairs,
 * [z][y][x].  Runs on the handle's kernel path.  This is one application of the operator that
 * wavefield_extro_ori2 applies 2(M+1) times per step (ose_3d_lib.cu:668-687:
 * cufftXtExecDescriptorC2C forward, scale_kxkz_3D, inverse, scal_vr_3d); the
 * real and imaginary parts carry two independent real fields. */
ose_status ose_apply_operator(ose_handle* h, const float* in, float* out);

/* Average device time per launch of each kernel class over `reps` steps,
 * measured with CUDA events bracketing each launch on the handle's stream
 * (not graph replay).  Advances the shot by `reps` steps.  names, ms, bytes
 * and launches are arrays of capacity cap; *count receives the number of
 * classes that launched in those steps (the source injection always listed).
 * bytes = algorithmic HBM bytes of one launch; launches = launches of the
 * class per step. */
ose_status ose_profile_step(ose_handle* h, int reps, int cap, int* count,
                            const char** names, float* ms, double* bytes,
                            int* launches);

/* Checkpoint of the current shot to a file: parameters, shot index, step
 * index, P and Q, and the receiver rows recorded so far - the whole state of
 * the time loop.  The reference has no checkpoint; its state is exactly these
 * (the p2D/q2D fields, it, rec_data_h: ose_3d.cu:242-276). */
ose_status ose_checkpoint_save(ose_handle* h, const char* path);

/* Restore a checkpoint on a handle created with identical parameters; the
 * shot then continues from the saved step (ose_run, ose_step...). */
ose_status ose_checkpoint_load(ose_handle* h, const char* path);

/* Called by ose_run_snapshots with the 0-based index of the last step done
 * and the padded P and Q (nxb*nyb*nzb floats each, in the requested layout).
 * The arrays are valid during the call only. */
typedef void (*ose_snapshot_fn)(int it, const float* P, const float* Q, void* user);

/* nsteps steps; after every `every` steps (and after the last) the state is
 * copied out and handed to fn.  Copies go device -> device -> pinned host on a
 * second stream while the next steps run, so the callback overlaps the GPU
 * work.  With OSE_LAYOUT_YXZ the arrays have the byte layout of the
 * reference's commented per-step dump ./wf/{p,q}-<it>-single.bin
 * (ose_3d.cu:260-269, write_3dfile_from_1darray_ci). */
ose_status ose_run_snapshots(ose_handle* h, int nsteps, int every, int layout,
                             ose_snapshot_fn fn, void* user);

/* The current shot's gather (ng traces x nt samples, trace ig = iy*nx + ix)
 * as an SU file (240-byte SEG-Y trace headers, native byte order, no file
 * header) or as a SEG-Y file (3200-byte text + 400-byte binary header,
 * big-endian IEEE float traces).  Coordinates in cm (scalco = -100), dt in
 * microseconds.  The reference names SU formats (ose_3d.cu:17-18) but writes
 * only raw floats. */
ose_status ose_write_su(ose_handle* h, const char* path);
ose_status ose_write_segy(ose_handle* h, const char* path);

/* ---- batched shots -------------------------------------------------------
 * The reference loops over shots one after another on the full model
 * (for(is...) in ose_3d.cu:242-279, nshot = 1 there).  A batch gives every
 * shot its own window of the model around its source and advances all
 * windows together: each pass of a time step is one launch over every shot,
 * and a step is one CUDA graph. */

/* One shot of a batch.  The window interior is model cells
 * [x0, x0+nx) x [y0, y0+ny) x [z0, z0+nz) (cells outside the model repeat its
 * edge); the shot pads it with the sponge widths of the batch parameters
 * (judge_odd applies).  (sx, sy, sz): source cell inside the window
 * interior.  Receivers: every interior (x, y) of the window at depth gzbeg. */
typedef struct ose_shot_window {
    int x0, y0, z0;
    int nx, ny, nz;
    int sx, sy, sz;
} ose_shot_window;

typedef struct ose_batch ose_batch;

/* p: shared parameters (sponge widths, nt, fm, dt, amp, dx..dz, gzbeg,
 * switches; its nx..nz and source fields are ignored).  model: mnx*mny*mnz
 * floats in the reference layout [x][y][z].  Each shot has its own velocity
 * window, vmax, R, series order M and tables (ose_batch_info). */
ose_status ose_batch_create(const ose_params* p, const float* model, int mnx, int mny, int mnz,
                            int nshots, const ose_shot_window* windows, ose_batch** out);
ose_status ose_batch_destroy(ose_batch* b);
const char* ose_batch_last_error(const ose_batch* b);
/* All shots back to rest at step 0. */
ose_status ose_batch_reset(ose_batch* b);
/* nsteps steps of every shot (graph replays). */
ose_status ose_batch_run(ose_batch* b, int nsteps);
/* As ose_batch_run, timed with CUDA events on the batch's stream. */
ose_status ose_batch_run_timed(ose_batch* b, int nsteps, float* ms);
/* Derived values and padded cell count of one shot. */
ose_status ose_batch_info(const ose_batch* b, int shot, ose_derived* d, long long* cells);
/* One shot's gather, [ig][it] (nx*ny x nt floats of its window). */
ose_status ose_batch_get_gather(ose_batch* b, int shot, float* out);
/* One shot's padded P or Q, [z][y][x]. */
ose_status ose_batch_get_wavefield(ose_batch* b, int shot, int which, float* out);
/* Pick the batching strategy (lanes = 0: one batched launch per pass and axis
 * length for all shots; lanes = k > 0: every shot's single-shot launches,
 * shots spread over k streams that run concurrently in the captured step;
 * lanes = -1: the source injection and then ONE persistent cooperative
 * launch per step that runs every batched pass, with grid barriers between
 * passes — available when every axis length is 16 C with C <= 16; a barrier
 * that waits longer than 2 s ends the step with OSE_ERR_TIMEOUT),
 * the shot grouping of batched launches (groups whose working set stays
 * within group_mb MB, so a group's fields can stay in L2 through its step;
 * 0 = all shots together) and, for axis lengths without register kernels, the rows
 * per x-pass block, the y/z column tile widths and the radix order, by timing
 * candidates over `steps` steps (coordinate search); reuse a cached choice for
 * the same window sizes from cache_path (a text file, one line per batch
 * shape; NULL = no cache).  Resets the batch. */
ose_status ose_batch_autotune(ose_batch* b, int steps, const char* cache_path, float* best_ms);
ose_status ose_batch_get_tuning(const ose_batch* b, int* rows_scale, int* txy, int* txz, int* radix_order,
                                int* group_mb, int* lanes);
/* Set the tuning by hand (the values ose_batch_get_tuning returns; -1 <= lanes
 * <= 8; OSE_ERR_UNSUPPORTED for lanes = -1 on a batch without the persistent
 * form).  Resets the batch. */
ose_status ose_batch_set_tuning(ose_batch* b, int rows_scale, int txy, int txz, int radix_order, int group_mb,
                                int lanes);

/* Largest padded grid (nxb*nyb*nzb) ose_apply_operator_noalloc accepts. */
#define OSE_NOALLOC_MAX_CELLS 262144

/* The operator of ose_apply_operator on caller-owned DEVICE buffers, with no
 * allocation of any kind.  This entry point has no counterpart in the
 * reference; it exists for callers that cannot call cudaMalloc: code running
 * inside a framework that owns the device allocator (a plugin or custom call
 * that must not allocate behind it), hosts that must not allocate after
 * start-up, and callers that already own every buffer.
 *   out = vel * IFFT3(|k| FFT3(in)) / (R * nxb*nyb*nzb)
 * vel: nxb*nyb*nzb floats (padded velocity, [z][y][x]); in, out: as many
 * interleaved (re, im) float pairs; all three in device memory, out may not
 * alias in.  |k| uses dk = 2 pi / (d * nb) per axis.  stream: a cudaStream_t
 * (NULL = the legacy default stream); the call only enqueues work.
 * Limits: nxb*nyb*nzb <= OSE_NOALLOC_MAX_CELLS, every axis even and at most
 * 1024; larger sizes return OSE_ERR_UNSUPPORTED.  The FFT scratch and the
 * twiddle/wavenumber tables live in one fixed device array of about 2 MiB
 * that every GPU loading the library keeps until the process exits; every
 * call shares it and leaves its contents behind, so calls that overlap on
 * the GPU (several streams or host threads) race: serialise them.  The first
 * call on a device looks up that array's address and sets kernel attributes;
 * make it before any stream capture. */
ose_status ose_apply_operator_noalloc(int nxb, int nyb, int nzb, float dx, float dy, float dz,
                                      double R, const float* vel, const float* in, float* out,
                                      void* stream);

/* Write ./output-style files of the current shot:
 * gather [ig][it] (ose_3d.cu:276) to gather_path and the parameter dump
 * (output_par, ose_3d_lib.cu:255-319) to par_path.  Either may be NULL. */
ose_status ose_write_outputs(ose_handle* h, const char* gather_path, const char* par_path);

/* Library version string. */
const char* ose_version(void);

#ifdef __cplusplus
}
#endif

#endif /* OSE3D_H */
