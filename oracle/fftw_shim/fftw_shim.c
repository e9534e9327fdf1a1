/*
 * REDFT10 / REDFT01 stand-in for libfftw3f (test infrastructure only).
 *
 * FFTW is an external dependency of the reference (CMakeLists.txt:32-34,
 * src/Makefile:38, unpinned version) that is not installed here.  This file
 * evaluates FFTW's documented unnormalised definitions directly, in double
 * precision, and rounds once to float:
 *   REDFT10 (DCT-II):  Y[k] = 2 * sum_j X[j] * cos(pi * (j + 1/2) * k / n)
 *   REDFT01 (DCT-III): Y[k] = X[0] + 2 * sum_{j>=1} X[j] * cos(pi * j * (k + 1/2) / n)
 * A rank-2 plan applies the 1D transform along both axes of each row-major
 * n[0] x n[1] block (rows first, then columns), which is FFTW's
 * multi-dimensional r2r definition.  Real FFTW computes the same values in
 * float with its own rounding; the difference is a few float ulps.
 * The oracle restatement (vbm3d_oracle.c) calls the same routines, so both
 * oracles see identical transform values.  The multiscaler's whole-frame
 * plans (multiscaler/multiscaler.cpp:21-100) run through fftwf_execute on
 * the plan's own buffers; sizes are unlimited (O(n^2) per line).
 */
#include "fftw3.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

struct oracle_fftwf_plan_s {
    int rank;
    int n[2];
    int howmany;
    int istride, idist, ostride, odist;
    float *in, *out;
    fftwf_r2r_kind kind[2];
    double *cosv[2]; /* cosv[axis][k*n + j] */
};

/* calloc: dct_2d_inv transforms its whole buffer, of which only the
 * prefix holding this row's groups is initialised (src/vbm3d.cpp:1689-1703). */
void *fftwf_malloc(size_t n) { return calloc(n ? n : 1, 1); }
void fftwf_free(void *p) { free(p); }
void fftwf_cleanup(void) {}

static void fill_cos(double *c, int n, fftwf_r2r_kind kind)
{
    const double pi = 3.14159265358979323846;
    for (int k = 0; k < n; k++)
        for (int j = 0; j < n; j++)
            c[k * n + j] = kind == FFTW_REDFT10 ? cos(pi * (j + 0.5) * k / n)
                                                : cos(pi * j * (k + 0.5) / n);
}

fftwf_plan fftwf_plan_many_r2r(int rank, const int *n, int howmany,
                               float *in, const int *inembed, int istride, int idist,
                               float *out, const int *onembed, int ostride, int odist,
                               const fftwf_r2r_kind *kind, unsigned flags)
{
    (void)inembed; (void)onembed; (void)flags;
    if (rank < 1 || rank > 2 || n[0] < 1 || (rank == 2 && n[1] < 1)) return NULL;
    struct oracle_fftwf_plan_s *p = (struct oracle_fftwf_plan_s *)calloc(1, sizeof(*p));
    p->rank = rank;
    p->n[0] = n[0];
    p->n[1] = rank == 2 ? n[1] : 1;
    p->howmany = howmany;
    p->istride = istride; p->idist = idist;
    p->ostride = ostride; p->odist = odist;
    p->in = in; p->out = out;
    p->kind[0] = kind[0];
    p->kind[1] = rank == 2 ? kind[1] : kind[0];
    p->cosv[0] = (double *)malloc(sizeof(double) * (size_t)p->n[0] * p->n[0]);
    fill_cos(p->cosv[0], p->n[0], p->kind[0]);
    if (rank == 2) {
        p->cosv[1] = (double *)malloc(sizeof(double) * (size_t)p->n[1] * p->n[1]);
        fill_cos(p->cosv[1], p->n[1], p->kind[1]);
    }
    return p;
}

void fftwf_destroy_plan(fftwf_plan p)
{
    if (!p) return;
    free(p->cosv[0]);
    free(p->cosv[1]);
    free(p);
}

/* One 1D transform of length n on a strided double vector, in place
 * (tmp: n doubles of scratch). */
static void r2r_1d(double *v, int n, int stride, fftwf_r2r_kind kind, const double *c, double *tmp)
{
    for (int k = 0; k < n; k++) {
        double s;
        if (kind == FFTW_REDFT10) {
            s = 0.0;
            for (int j = 0; j < n; j++) s += v[j * stride] * c[k * n + j];
            s *= 2.0;
        } else {
            s = v[0];
            for (int j = 1; j < n; j++) s += 2.0 * v[j * stride] * c[k * n + j];
        }
        tmp[k] = s;
    }
    for (int k = 0; k < n; k++) v[k * stride] = tmp[k];
}

void fftwf_execute_r2r(const fftwf_plan p, float *in, float *out)
{
    const int n0 = p->n[0], n1 = p->n[1];
    const size_t sz = (size_t)n0 * n1;
    double *blk = (double *)malloc(sizeof(double) * sz);
    double *tmp = (double *)malloc(sizeof(double) * (size_t)(n0 > n1 ? n0 : n1));
    for (int h = 0; h < p->howmany; h++) {
        const float *src = in + (size_t)h * p->idist;
        float *dst = out + (size_t)h * p->odist;
        for (size_t i = 0; i < sz; i++) blk[i] = (double)src[i * p->istride];
        if (p->rank == 1) {
            r2r_1d(blk, n0, 1, p->kind[0], p->cosv[0], tmp);
        } else {
            for (int r = 0; r < n0; r++) r2r_1d(blk + (size_t)r * n1, n1, 1, p->kind[1], p->cosv[1], tmp);
            for (int c = 0; c < n1; c++) r2r_1d(blk + c, n0, n1, p->kind[0], p->cosv[0], tmp);
        }
        for (size_t i = 0; i < sz; i++) dst[i * p->ostride] = (float)blk[i];
    }
    free(blk);
    free(tmp);
}

void fftwf_execute(const fftwf_plan p) { fftwf_execute_r2r(p, p->in, p->out); }
