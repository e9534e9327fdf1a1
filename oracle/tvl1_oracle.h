/*
 * CPU restatement of the reference's TV-L1 optical flow (tvl1flow/):
 * TEST INFRASTRUCTURE, the oracle of the GPU flow kernels.  See
 * tvl1_oracle.c.
 */
#ifndef VBM3D_TVL1_ORACLE_H
#define VBM3D_TVL1_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct tv_params {
    float tau, lambda, theta;
    int nscales, fscale;
    float zfactor;
    int nwarps;
    float epsilon;
} tv_params;

void tv_default_params(tv_params *P);
int tv_scales(int nx, int ny, const tv_params *P, int *fscale);
/* flow: [2][ny][nx]; iters: nscales x nwarps iteration counts (or NULL) */
int tv_flow(const float *I0, const float *I1, int nx, int ny, const tv_params *P, float *flow, int *iters);
/* pieces, for unit tests */
float tv_bicubic_at(const float *in, float uu, float vv, int nx, int ny, int border_out);
void tv_gaussian(float *I, int xdim, int ydim, double sigma);
void tv_zoom_size(int nx, int ny, int *nxx, int *nyy, float factor);

#ifdef __cplusplus
}
#endif
#endif
