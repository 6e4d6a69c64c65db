/*
 * ose_oracle.h - FP64 CPU restatement of the reference's OSE time loop.
 *
 * TEST INFRASTRUCTURE.  Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg may load this library, and only as the checker (or as the
 * timed CPU baseline).  The product path (libose3d.so) never calls it.
 *
 * Every function cites the reference file:line it restates.  Parity pin: the
 * restatement is checked against the reference's own sources built and run on
 * this host (oracle/refemu, outputs in tests/golden/).
 */
#ifndef OSE_ORACLE_H
#define OSE_ORACLE_H

#include "../include/ose3d.h"

#ifdef __cplusplus
extern "C" {
#endif

/* judge_odd (ose_3d_lib.cu:36-44) applied to the three axes (ose_3d.cu:85-90).
 * d receives nxb..nzb, br/bb/bd after the fix, ng, and the dk values. */
int orc_derive_dims(const ose_params* p, ose_derived* d);

/* input_file_xyz_boundary + add_pml_layers_v_h (ose_3d_lib.cu:887-1032):
 * scatter the [x][y][z] interior into a [z][y][x] padded grid and replicate the
 * edges into the sponge. vb holds nxb*nyb*nzb floats. */
int orc_pad_model(const ose_params* p, const float* vel_xyz, float* vb);

/* R, dtR, M from vmax (ose_3d.cu:191-197).  M follows the reference's float
 * arithmetic exactly so the series order always matches. */
int orc_series(const ose_params* p, float vmax, double* R, double* dtR, int* M);

/* generate_att (ose_3d_kernel.cu:242-261) or the Cerjan taper. out: before+nn+after. */
int orc_sponge(int before, int nn, int after, int mode, float factor, float* out);

/* generate_wavelet_gpu (ose_3d_kernel.cu:3-13): Ricker with a 40-sample delay. */
int orc_ricker(int nt, float fm, float dt, float amp, float* out);

/* R2C + hilbert_1d + C2R (ose_3d_lib.cu:578-581, ose_3d_kernel.cu:154-172),
 * unnormalised (times nt) unless div_nt. */
int orc_hilbert(const float* ricker, int nt, int div_nt, float* out);

/* J_0..J_{M+1}(dtR) in double. */
int orc_bessel(int M, double dtR, double* J);

/* One application of the normalised operator (ose_3d_lib.cu:665-687):
 *   out = v * IFFT3(|k| FFT3(in)) / (R N), on interleaved complex doubles. */
int orc_apply_operator(const ose_params* p, const float* vb, double R,
                       const double* in, double* out);

/* Full time loop of one shot (ose_3d.cu:242-276):
 *   for it < nsteps: inject (Xt_add_wavelet_sxyz x2), step (wavefield_extro_ori2),
 *   record Q at receiver depth gzbeg (rec_shotdata_3d, rec_slice_to_data).
 * P, Q: in/out padded [z][y][x] doubles (zero them for a fresh shot; passing a
 * state continues it).  it0 = index of the first step (selects the wavelet
 * sample).  gather: nsteps*ng floats in memory order [it][ig] (may be NULL). */
int orc_run(const ose_params* p, const float* vel_xyz, int is, int it0, int nsteps,
            double* P, double* Q, float* gather);

/* Number of OpenMP threads the oracle uses (for reporting). */
int orc_threads(void);

#ifdef __cplusplus
}
#endif
#endif
