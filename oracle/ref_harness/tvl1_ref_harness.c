/*
 * Harness around the reference's own TV-L1 library (tvl1flow/tvl1flow_lib.c,
 * included from the reference tree at build time by oracle/build_ref.sh):
 * TEST INFRASTRUCTURE, used to pin the oracle restatement.  The scale
 * count is main.c's rule (tvl1flow/main.c:151-157), restated here because
 * main.c itself needs the image I/O library.
 */
#include <math.h>
#include <stdbool.h>

#include "tvl1flow_lib.c"

int ref_tvl1_flow(const float *I0, const float *I1, int nx, int ny, float tau, float lambda, float theta,
                  int nscales, int fscale, float zfactor, int nwarps, float epsilon, float *flow)
{
    const float N = 1 + log(hypot(nx, ny) / 16.0) / log(1 / zfactor);
    if (N < nscales) nscales = N;
    if (nscales < fscale) fscale = nscales;
    Dual_TVL1_optic_flow_multiscale((float *)I0, (float *)I1, flow, flow + nx * ny, nx, ny, tau, lambda, theta,
                                    nscales, fscale, zfactor, nwarps, epsilon, false);
    return nscales;
}
