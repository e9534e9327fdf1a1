/*
 * CPU restatement of the TV-L1 optical flow that produces VBM3D's flows
 * (tehret/vbm3d, tvl1flow/: Zach-Pock-Bischof dual TV-L1 with the
 * Chambolle projection, coarse-to-fine with bicubic warping).
 *
 * TEST INFRASTRUCTURE.  This is the oracle the GPU flow kernels are checked
 * against; nothing on the product path links or calls it.  It is pinned
 * bit-exactly against the reference's own tvl1flow_lib.c, compiled by
 * oracle/build_ref.sh (tests/test_oracle_golden.py, golden vectors made by
 * tests/golden/make_golden.py).
 *
 * Arithmetic follows the reference operation by operation: float where it
 * uses float, double where it uses double (the Gaussian convolution, the
 * bicubic cells, the promotions of double literals), sums in the
 * reference's order, so built with -ffp-contract=off the results equal the
 * reference's single-threaded build.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "tvl1_oracle.h"

#define TV_MAX_ITERATIONS 300          /* tvl1flow/tvl1flow_lib.c:22 */
#define TV_PRESMOOTHING_SIGMA 0.8      /* :23 */
#define TV_GRAD_IS_ZERO 1E-10          /* :24 */
#define TV_ZOOM_SIGMA_ZERO 0.6         /* tvl1flow/zoom.c:17 */
#define TV_GAUSSIAN_WINDOW 5           /* tvl1flow/mask.c: DEFAULT_GAUSSIAN_WINDOW_SIZE */

/* Neumann clamp with an out-of-range flag (bicubic_interpolation.c:24-40). */
static int tv_clamp(int x, int n, int *out)
{
    if (x < 0) {
        *out = 1;
        return 0;
    }
    if (x >= n) {
        *out = 1;
        return n - 1;
    }
    return x;
}

/* Keys cubic through v[0..3] at x in [0, 1] (bicubic_interpolation.c:118-127). */
static double tv_cubic(const double v[4], double x)
{
    return v[1] + 0.5 * x * (v[2] - v[0] + x * (2.0 * v[0] - 5.0 * v[1] + 4.0 * v[2] - v[3] +
                                                  x * (3.0 * (v[1] - v[2]) + v[3] - v[0])));
}

/* bicubic_interpolation_at (bicubic_interpolation.c:153-237), Neumann
 * boundary.  The row below is clamped with the x direction's sign, as in the
 * reference (its `my` uses sx). */
float tv_bicubic_at(const float *in, float uu, float vv, int nx, int ny, int border_out)
{
    const int sx = (uu < 0) ? -1 : 1;
    const int sy = (vv < 0) ? -1 : 1;
    int out = 0;
    const int x = tv_clamp((int)uu, nx, &out);
    const int y = tv_clamp((int)vv, ny, &out);
    const int mx = tv_clamp((int)uu - sx, nx, &out);
    const int my = tv_clamp((int)vv - sx, ny, &out);
    const int dx = tv_clamp((int)uu + sx, nx, &out);
    const int dy = tv_clamp((int)vv + sy, ny, &out);
    const int ddx = tv_clamp((int)uu + 2 * sx, nx, &out);
    const int ddy = tv_clamp((int)vv + 2 * sy, ny, &out);
    if (out && border_out) return 0.0f;
    const int cols[4] = {mx, x, dx, ddx}, rows[4] = {my, y, dy, ddy};
    double v[4];
    const double fy = (double)(vv - (float)y), fx = (double)(uu - (float)x);
    for (int c = 0; c < 4; c++) {
        double col[4];
        for (int r = 0; r < 4; r++) col[r] = (double)in[cols[c] + nx * rows[r]];
        v[c] = tv_cubic(col, fy);
    }
    return (float)tv_cubic(v, fx);
}

/* In-place separable Gaussian with reflecting boundaries and double
 * accumulation (mask.c: gaussian, rows then columns). */
void tv_gaussian(float *I, int xdim, int ydim, double sigma)
{
    const double den = 2 * sigma * sigma;
    const int size = (int)(TV_GAUSSIAN_WINDOW * sigma) + 1;
    const int bdx = xdim + size, bdy = ydim + size;
    double *B = malloc(size * sizeof *B);
    for (int i = 0; i < size; i++) B[i] = 1 / (sigma * sqrt(2.0 * 3.1415926)) * exp(-i * i / den);
    double norm = 0;
    for (int i = 0; i < size; i++) norm += B[i];
    norm *= 2;
    norm -= B[0];
    for (int i = 0; i < size; i++) B[i] /= norm;

    double *R = malloc((size + xdim + size) * sizeof *R);
    for (int k = 0; k < ydim; k++) {
        for (int i = size; i < bdx; i++) R[i] = I[k * xdim + i - size];
        for (int i = 0, j = bdx; i < size; i++, j++) {
            R[i] = I[k * xdim + size - i];
            R[j] = I[k * xdim + xdim - i - 1];
        }
        for (int i = size; i < bdx; i++) {
            double sum = B[0] * R[i];
            for (int j = 1; j < size; j++) sum += B[j] * (R[i - j] + R[i + j]);
            I[k * xdim + i - size] = (float)sum;
        }
    }
    double *T = malloc((size + ydim + size) * sizeof *T);
    for (int k = 0; k < xdim; k++) {
        for (int i = size; i < bdy; i++) T[i] = I[(i - size) * xdim + k];
        for (int i = 0, j = bdy; i < size; i++, j++) {
            T[i] = I[(size - i) * xdim + k];
            T[j] = I[(ydim - i - 1) * xdim + k];
        }
        for (int i = size; i < bdy; i++) {
            double sum = B[0] * T[i];
            for (int j = 1; j < size; j++) sum += B[j] * (T[i - j] + T[i + j]);
            I[(i - size) * xdim + k] = (float)sum;
        }
    }
    free(B);
    free(R);
    free(T);
}

/* zoom_size (zoom.c:24-36). */
void tv_zoom_size(int nx, int ny, int *nxx, int *nyy, float factor)
{
    *nxx = (int)((float)nx * factor + 0.5);
    *nyy = (int)((float)ny * factor + 0.5);
}

/* zoom_out (zoom.c:43-78): Gaussian pre-smoothing, bicubic resampling. */
static void tv_zoom_out(const float *I, float *out, int nx, int ny, float factor)
{
    float *Is = malloc((size_t)nx * ny * sizeof *Is);
    memcpy(Is, I, (size_t)nx * ny * sizeof *Is);
    int nxx, nyy;
    tv_zoom_size(nx, ny, &nxx, &nyy, factor);
    const float sigma = TV_ZOOM_SIGMA_ZERO * sqrt(1.0 / (factor * factor) - 1.0);
    tv_gaussian(Is, nx, ny, sigma);
    for (int i1 = 0; i1 < nyy; i1++)
        for (int j1 = 0; j1 < nxx; j1++)
            out[i1 * nxx + j1] = tv_bicubic_at(Is, (float)j1 / factor, (float)i1 / factor, nx, ny, 0);
    free(Is);
}

/* zoom_in (zoom.c:85-113): bicubic resampling to nxx x nyy. */
static void tv_zoom_in(const float *I, float *out, int nx, int ny, int nxx, int nyy)
{
    const float fx = ((float)nxx / nx), fy = ((float)nyy / ny);
    for (int i1 = 0; i1 < nyy; i1++)
        for (int j1 = 0; j1 < nxx; j1++)
            out[i1 * nxx + j1] = tv_bicubic_at(I, (float)j1 / fx, (float)i1 / fy, nx, ny, 0);
}

/* divergence, backward differences with the reference's border rules (mask.c). */
static void tv_divergence(const float *v1, const float *v2, float *div, int nx, int ny)
{
    for (int i = 1; i < ny - 1; i++)
        for (int j = 1; j < nx - 1; j++) {
            const int p = i * nx + j;
            div[p] = (v1[p] - v1[p - 1]) + (v2[p] - v2[p - nx]);
        }
    for (int j = 1; j < nx - 1; j++) {
        const int p = (ny - 1) * nx + j;
        div[j] = v1[j] - v1[j - 1] + v2[j];
        div[p] = v1[p] - v1[p - 1] - v2[p - nx];
    }
    for (int i = 1; i < ny - 1; i++) {
        const int p1 = i * nx, p2 = (i + 1) * nx - 1;
        div[p1] = v1[p1] + v2[p1] - v2[p1 - nx];
        div[p2] = -v1[p2 - 1] + v2[p2] - v2[p2 - nx];
    }
    div[0] = v1[0] + v2[0];
    div[nx - 1] = -v1[nx - 2] + v2[nx - 1];
    div[(ny - 1) * nx] = v1[(ny - 1) * nx] - v2[(ny - 2) * nx];
    div[ny * nx - 1] = -v1[ny * nx - 2] - v2[(ny - 1) * nx - 1];
}

/* forward_gradient (mask.c): zero on the last column / row. */
static void tv_forward_gradient(const float *f, float *fx, float *fy, int nx, int ny)
{
    for (int i = 0; i < ny - 1; i++)
        for (int j = 0; j < nx - 1; j++) {
            const int p = i * nx + j;
            fx[p] = f[p + 1] - f[p];
            fy[p] = f[p + nx] - f[p];
        }
    for (int j = 0; j < nx - 1; j++) {
        const int p = (ny - 1) * nx + j;
        fx[p] = f[p + 1] - f[p];
        fy[p] = 0;
    }
    for (int i = 1; i < ny; i++) {
        const int p = i * nx - 1;
        fx[p] = 0;
        fy[p] = f[p + nx] - f[p];
    }
    fx[ny * nx - 1] = 0;
    fy[ny * nx - 1] = 0;
}

/* centered_gradient (mask.c): one-sided at the borders, halved. */
static void tv_centered_gradient(const float *in, float *dx, float *dy, int nx, int ny)
{
    for (int i = 0; i < ny; i++)
        for (int j = 0; j < nx; j++) {
            const int k = i * nx + j;
            const float xr = in[j < nx - 1 ? k + 1 : k], xl = in[j > 0 ? k - 1 : k];
            const float yd = in[i < ny - 1 ? k + nx : k], yu = in[i > 0 ? k - nx : k];
            dx[k] = 0.5 * (xr - xl);
            dy[k] = 0.5 * (yd - yu);
        }
}

/* Dual_TVL1_optic_flow (tvl1flow_lib.c:96-283): one scale.  iters, when not
 * NULL, receives the iteration count of each warping. */
static void tv_one_scale(const float *I0, const float *I1, float *u1, float *u2, int nx, int ny,
                         const tv_params *P, int *iters)
{
    const int size = nx * ny;
    const float l_t = P->lambda * P->theta;
    float *buf = calloc((size_t)16 * size, sizeof(float));
    float *I1x = buf, *I1y = buf + size, *I1w = buf + 2 * size, *I1wx = buf + 3 * size, *I1wy = buf + 4 * size;
    float *rho_c = buf + 5 * size, *v1 = buf + 6 * size, *v2 = buf + 7 * size, *p11 = buf + 8 * size;
    float *p12 = buf + 9 * size, *p21 = buf + 10 * size, *p22 = buf + 11 * size, *grad = buf + 12 * size;
    float *div1 = buf + 13 * size, *div2 = buf + 14 * size, *gx = buf + 15 * size;
    float *gtmp = malloc((size_t)3 * size * sizeof(float));
    float *u1y = gtmp, *u2x = gtmp + size, *u2y = gtmp + 2 * size;

    tv_centered_gradient(I1, I1x, I1y, nx, ny);
    for (int w = 0; w < P->nwarps; w++) {
        for (int i = 0; i < size; i++) {
            const float uu = (float)(i % nx + u1[i]), vv = (float)(i / nx + u2[i]);
            I1w[i] = tv_bicubic_at(I1, uu, vv, nx, ny, 1);
            I1wx[i] = tv_bicubic_at(I1x, uu, vv, nx, ny, 1);
            I1wy[i] = tv_bicubic_at(I1y, uu, vv, nx, ny, 1);
        }
        for (int i = 0; i < size; i++) {
            const float Ix2 = I1wx[i] * I1wx[i], Iy2 = I1wy[i] * I1wy[i];
            grad[i] = Ix2 + Iy2;
            rho_c[i] = I1w[i] - I1wx[i] * u1[i] - I1wy[i] * u2[i] - I0[i];
        }
        int n = 0;
        float error = INFINITY;
        while (error > P->epsilon * P->epsilon && n < TV_MAX_ITERATIONS) {
            n++;
            /* thresholding step TH */
            for (int i = 0; i < size; i++) {
                const float rho = rho_c[i] + (I1wx[i] * u1[i] + I1wy[i] * u2[i]);
                float d1, d2;
                if (rho < -l_t * grad[i]) {
                    d1 = l_t * I1wx[i];
                    d2 = l_t * I1wy[i];
                } else if (rho > l_t * grad[i]) {
                    d1 = -l_t * I1wx[i];
                    d2 = -l_t * I1wy[i];
                } else if (grad[i] < TV_GRAD_IS_ZERO) {
                    d1 = d2 = 0;
                } else {
                    const float fi = -rho / grad[i];
                    d1 = fi * I1wx[i];
                    d2 = fi * I1wy[i];
                }
                v1[i] = u1[i] + d1;
                v2[i] = u2[i] + d2;
            }
            tv_divergence(p11, p12, div1, nx, ny);
            tv_divergence(p21, p22, div2, nx, ny);
            error = 0.0;
            for (int i = 0; i < size; i++) {
                const float u1k = u1[i], u2k = u2[i];
                u1[i] = v1[i] + P->theta * div1[i];
                u2[i] = v2[i] + P->theta * div2[i];
                error += (u1[i] - u1k) * (u1[i] - u1k) + (u2[i] - u2k) * (u2[i] - u2k);
            }
            error /= size;
            tv_forward_gradient(u1, gx, u1y, nx, ny);
            tv_forward_gradient(u2, u2x, u2y, nx, ny);
            /* projection of the dual variable */
            for (int i = 0; i < size; i++) {
                const float taut = P->tau / P->theta;
                const float g1 = hypot(gx[i], u1y[i]);
                const float g2 = hypot(u2x[i], u2y[i]);
                const float ng1 = 1.0 + taut * g1;
                const float ng2 = 1.0 + taut * g2;
                p11[i] = (p11[i] + taut * gx[i]) / ng1;
                p12[i] = (p12[i] + taut * u1y[i]) / ng1;
                p21[i] = (p21[i] + taut * u2x[i]) / ng2;
                p22[i] = (p22[i] + taut * u2y[i]) / ng2;
            }
        }
        if (iters) iters[w] = n;
    }
    free(buf);
    free(gtmp);
}

/* The number of scales main.c uses: min(nscales, 1 + log(hypot/16) / log(1/zfactor)). */
int tv_scales(int nx, int ny, const tv_params *P, int *fscale)
{
    int nscales = P->nscales;
    const float N = 1 + log(hypot(nx, ny) / 16.0) / log(1 / P->zfactor);
    if (N < nscales) nscales = N;
    *fscale = P->fscale;
    if (nscales < *fscale) *fscale = nscales;
    return nscales;
}

/* image_normalization then Dual_TVL1_optic_flow_multiscale
 * (tvl1flow_lib.c:290-488) with the scale count of main.c.  flow: [2][ny][nx]
 * (x then y component).  iters (optional): nscales x nwarps counts, -1 for
 * scales below fscale. */
int tv_flow(const float *I0, const float *I1, int nx, int ny, const tv_params *P, float *flow, int *iters)
{
    if (nx < 2 || ny < 2 || !P) return 1;
    int fscale;
    const int nscales = tv_scales(nx, ny, P, &fscale);
    if (nscales < 1) return 1;
    const int size = nx * ny;
    float **I0s = calloc(nscales, sizeof *I0s), **I1s = calloc(nscales, sizeof *I1s);
    float **u1s = calloc(nscales, sizeof *u1s), **u2s = calloc(nscales, sizeof *u2s);
    int *nxs = calloc(nscales, sizeof *nxs), *nys = calloc(nscales, sizeof *nys);
    I0s[0] = malloc(size * sizeof(float));
    I1s[0] = malloc(size * sizeof(float));
    u1s[0] = flow;
    u2s[0] = flow + size;
    nxs[0] = nx;
    nys[0] = ny;
    /* image_normalization (tvl1flow_lib.c:317-348) */
    float min0 = I0[0], max0 = I0[0], min1 = I1[0], max1 = I1[0];
    for (int i = 1; i < size; i++) {
        if (I0[i] < min0) min0 = I0[i];
        if (I0[i] > max0) max0 = I0[i];
        if (I1[i] < min1) min1 = I1[i];
        if (I1[i] > max1) max1 = I1[i];
    }
    const float mx = max0 > max1 ? max0 : max1, mn = min0 < min1 ? min0 : min1, den = mx - mn;
    for (int i = 0; i < size; i++) {
        I0s[0][i] = den > 0 ? 255.0 * (I0[i] - mn) / den : I0[i];
        I1s[0][i] = den > 0 ? 255.0 * (I1[i] - mn) / den : I1[i];
    }
    tv_gaussian(I0s[0], nx, ny, TV_PRESMOOTHING_SIGMA);
    tv_gaussian(I1s[0], nx, ny, TV_PRESMOOTHING_SIGMA);
    for (int s = 1; s < nscales; s++) {
        tv_zoom_size(nxs[s - 1], nys[s - 1], &nxs[s], &nys[s], P->zfactor);
        const int sz = nxs[s] * nys[s];
        I0s[s] = malloc(sz * sizeof(float));
        I1s[s] = malloc(sz * sizeof(float));
        u1s[s] = malloc(sz * sizeof(float));
        u2s[s] = malloc(sz * sizeof(float));
        tv_zoom_out(I0s[s - 1], I0s[s], nxs[s - 1], nys[s - 1], P->zfactor);
        tv_zoom_out(I1s[s - 1], I1s[s], nxs[s - 1], nys[s - 1], P->zfactor);
    }
    for (int i = 0; i < nxs[nscales - 1] * nys[nscales - 1]; i++) u1s[nscales - 1][i] = u2s[nscales - 1][i] = 0.0f;
    if (iters)
        for (int i = 0; i < nscales * P->nwarps; i++) iters[i] = -1;
    for (int s = nscales - 1; s >= 0; s--) {
        if (s >= fscale)
            tv_one_scale(I0s[s], I1s[s], u1s[s], u2s[s], nxs[s], nys[s], P, iters ? iters + s * P->nwarps : NULL);
        if (!s) break;
        tv_zoom_in(u1s[s], u1s[s - 1], nxs[s], nys[s], nxs[s - 1], nys[s - 1]);
        tv_zoom_in(u2s[s], u2s[s - 1], nxs[s], nys[s], nxs[s - 1], nys[s - 1]);
        for (int i = 0; i < nxs[s - 1] * nys[s - 1]; i++) {
            u1s[s - 1][i] *= (float)1.0 / P->zfactor;
            u2s[s - 1][i] *= (float)1.0 / P->zfactor;
        }
    }
    for (int s = 1; s < nscales; s++) {
        free(I0s[s]);
        free(I1s[s]);
        free(u1s[s]);
        free(u2s[s]);
    }
    free(I0s[0]);
    free(I1s[0]);
    free(I0s);
    free(I1s);
    free(u1s);
    free(u2s);
    free(nxs);
    free(nys);
    return 0;
}

void tv_default_params(tv_params *P)
{
    /* the values the reference's flow scripts pass (tvl1flow/tvl1flow_forward.sh,
     * tvl1flow_backward.sh): tau lambda theta nscales fscale zfactor nwarps epsilon */
    P->tau = 0.25f;
    P->lambda = 0.2f;
    P->theta = 0.3f;
    P->nscales = 100;
    P->fscale = 2;
    P->zfactor = 0.5f;
    P->nwarps = 5;
    P->epsilon = 0.01f;
}
