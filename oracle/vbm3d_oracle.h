/*
 * CPU restatement of the reference VBM3D hot path (tehret/vbm3d,
 * src/vbm3d.cpp:378-1956, src/lib_transforms.cpp, src/Utilities/).
 *
 * TEST INFRASTRUCTURE.  This library is the oracle the GPU kernels are
 * checked against and the CPU baseline bench.py times.  Nothing on the
 * product path links or calls it.
 *
 * Parity pins: tests/test_oracle_golden.py compares every entry point with
 * golden vectors produced by the reference's own code (oracle/_ref, built by
 * oracle/build_ref.sh from the reference sources with IEEE float arithmetic:
 * -O2 -ffp-contract=off), generated by tests/golden/make_golden.py.
 *
 * Arithmetic follows the reference's source order operation by operation
 * (float where it uses float, double where a double constant promotes),
 * so with -ffp-contract=off the results are bit-identical to that build.
 */
#ifndef VBM3D_ORACLE_H
#define VBM3D_ORACLE_H

#include <stddef.h>
#include "../include/vbm3d_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

int oracle_default_params(int step, float sigma, vbm3d_params *out);
int oracle_sigma_table(float sigma, unsigned chnls, int color_space, float *table);
/* Reference grid size: rows, columns (ind_initialize, Utilities.cpp:400-415). */
int oracle_grid(const vbm3d_params *p, vbm3d_dims d, unsigned *rows, unsigned *cols,
                unsigned *row_ind, unsigned *col_ind);
void oracle_kaiser(unsigned k, float *window);

/* computeSimilarPatches for a list of reference patch indices. */
int oracle_similar_batch(const vbm3d_params *p, const float *video, const float *fflow,
                         const float *bflow, vbm3d_dims d, const unsigned *pidx, size_t count,
                         float *dist, unsigned *idx, unsigned *nsimp, unsigned *nsx);

/* One step (1 = hard threshold, 2 = Wiener) into num / den.  `threads`
 * OpenMP threads compute groups in parallel; aggregation is done in the
 * reference's order, so the result does not depend on `threads`. */
int oracle_step(int step, const vbm3d_params *p, const float *noisy, const float *basic,
                const float *fflow, const float *bflow, vbm3d_dims d, float sigma,
                int color_space, float *num, float *den, int threads);

/* run_vbm3d single-thread semantics (src/vbm3d.cpp:87-211, :356-376).
 * noisy is modified in place as the reference does. */
int oracle_run(float sigma, float *noisy, const float *fflow, const float *bflow,
               float *basic, float *denoised, const vbm3d_params *p1,
               const vbm3d_params *p2, int color_space, vbm3d_dims d, int threads);

void oracle_color_transform(float *video, vbm3d_dims d, int forward);

/* The frozen linearisation of one step (groups, masks / Wiener gains and
 * weights from the forward pass on noisy / basic) applied to x, in double:
 * the FP64 reference of vbm3d_linear_apply.  kt == 1 only. */
int oracle_linear_apply(int step, const vbm3d_params *p, const float *noisy, const float *basic,
                        const float *fflow, const float *bflow, vbm3d_dims d, float sigma, int color_space,
                        const float *x, double *out, int threads);

/* Transform kernels exposed for unit tests on one k x k block. */
void oracle_dct2d_forward(const float *in, float *out, unsigned k);
void oracle_dct2d_inverse(const float *in, float *out, unsigned k);
void oracle_bior2d_forward(const float *in, float *out);
void oracle_bior2d_inverse(const float *in, float *out);
void oracle_haar_forward(float *v, unsigned n);
void oracle_haar_inverse(float *v, unsigned n);

#ifdef __cplusplus
}
#endif
#endif
