/*
 * Declarations-only stand-in for the FFTW3 single-precision header.
 *
 * Test infrastructure: the oracle build links the reference's own sources
 * against this header and fftw_shim.c because libfftw3f is not installed.
 * Only the r2r surface the reference calls is declared
 * (src/Utilities/Utilities.cpp:346-398, src/vbm3d.cpp:1242-1303,
 * :1693-1712, :1882-1955, multiscaler/multiscaler.cpp:21-100).  The
 * enumerator values are this shim's own; the reference only passes them
 * back to the shim.
 */
#ifndef ORACLE_FFTW3_SHIM_H
#define ORACLE_FFTW3_SHIM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    FFTW_R2HC = 0, FFTW_HC2R = 1, FFTW_DHT = 2,
    FFTW_REDFT00 = 3, FFTW_REDFT01 = 4, FFTW_REDFT10 = 5, FFTW_REDFT11 = 6,
    FFTW_RODFT00 = 7, FFTW_RODFT01 = 8, FFTW_RODFT10 = 9, FFTW_RODFT11 = 10
} fftwf_r2r_kind;

#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)

typedef struct oracle_fftwf_plan_s *fftwf_plan;

void *fftwf_malloc(size_t n);
void fftwf_free(void *p);
fftwf_plan fftwf_plan_many_r2r(int rank, const int *n, int howmany,
                               float *in, const int *inembed, int istride, int idist,
                               float *out, const int *onembed, int ostride, int odist,
                               const fftwf_r2r_kind *kind, unsigned flags);
void fftwf_execute_r2r(const fftwf_plan p, float *in, float *out);
void fftwf_execute(const fftwf_plan p);
void fftwf_destroy_plan(fftwf_plan p);
void fftwf_cleanup(void);

#ifdef __cplusplus
}
#endif
#endif
