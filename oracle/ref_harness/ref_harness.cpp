/*
 * C entry points around the reference's own hot-path functions
 * (test infrastructure: built only into oracle/_ref/ from the reference's
 * sources by oracle/build_ref.sh; never shipped, never on the product path).
 *
 * Each function copies plain float buffers into the reference's
 * Video<float> container (src/Utilities/LibVideoT.hpp:133-190) and calls
 * the reference function named in its comment unchanged.
 */
#include <cstring>
#include <vector>
#include <omp.h>

#include "vbm3d.h"
#include "Utilities/Utilities.h"
#include "vbm3d_gb300.h"

#define REF_DCT 0

static Parameters to_ref(const vbm3d_params *p)
{
    Parameters r;
    r.k = p->k; r.kt = p->kt; r.p = p->p; r.N = p->N;
    r.tau = p->tau; r.d = p->d;
    r.Nf = p->Nf; r.Ns = p->Ns; r.Npr = p->Npr; r.Nb = p->Nb;
    r.T_2D = p->T_2D; r.T_3D = p->T_3D;
    r.lambda3D = p->lambda3D; r.mc = p->mc != 0; r.n = p->n;
    return r;
}

static void fill(Video<float> &v, const float *src, unsigned w, unsigned h, unsigned f, unsigned c)
{
    v.resize(w, h, f, c);
    if (src) std::memcpy(v.data.data(), src, sizeof(float) * (size_t)v.sz.whcf);
    else std::fill(v.data.begin(), v.data.end(), 0.f);
}

extern "C" {

/* vbm3d_1st_step / vbm3d_2nd_step (src/vbm3d.cpp:447-654, :676-928) with
 * crop == NULL and FFTW plans built as run_vbm3d builds them
 * (src/vbm3d.cpp:148-160, :176-190). */
int ref_step(int step, const vbm3d_params *prms, const float *noisy, const float *basic,
             const float *fflow, const float *bflow, vbm3d_dims d, float sigma,
             int color_space, float *num, float *den)
{
    Parameters p = to_ref(prms);
    Video<float> vn, vb, ff, bf, vnum, vden;
    fill(vn, noisy, d.width, d.height, d.frames, d.channels);
    if (step == 2) fill(vb, basic, d.width, d.height, d.frames, d.channels);
    fill(ff, fflow, d.width, d.height, d.frames, 2);
    fill(bf, bflow, d.width, d.height, d.frames, 2);
    const unsigned chnls = d.channels;
    const unsigned nb_cols = ind_size(0, d.width - p.k, p.p);
    fftwf_plan plan_2d = 0, plan_2d_inv = 0, plan_1d, plan_1d_inv;
    if (p.T_2D == REF_DCT) {
        allocate_plan_2d(&plan_2d, p.k, FFTW_REDFT10, p.N * chnls * p.kt);
        allocate_plan_2d(&plan_2d_inv, p.k, FFTW_REDFT01, p.N * nb_cols * chnls * p.kt);
    }
    allocate_plan_1d(&plan_1d, p.kt, FFTW_REDFT10, p.N * chnls * p.k * p.k);
    allocate_plan_1d(&plan_1d_inv, p.kt, FFTW_REDFT01, p.N * chnls * p.k * p.k);
    if (step == 1)
        vbm3d_1st_step(sigma, vn, ff, bf, p, &plan_2d, &plan_2d_inv, &plan_1d, &plan_1d_inv,
                       NULL, color_space != 0, vnum, vden);
    else
        vbm3d_2nd_step(sigma, vn, vb, ff, bf, p, &plan_2d, &plan_2d_inv, &plan_1d, &plan_1d_inv,
                       NULL, color_space != 0, vnum, vden);
    if (plan_2d) fftwf_destroy_plan(plan_2d);
    if (plan_2d_inv) fftwf_destroy_plan(plan_2d_inv);
    fftwf_destroy_plan(plan_1d);
    fftwf_destroy_plan(plan_1d_inv);
    if (vnum.sz.whcf != d.width * d.height * d.frames * d.channels) return 1;
    std::memcpy(num, vnum.data.data(), sizeof(float) * (size_t)vnum.sz.whcf);
    std::memcpy(den, vden.data.data(), sizeof(float) * (size_t)vden.sz.whcf);
    return 0;
}

/* computeSimilarPatches (src/vbm3d.cpp:1082-1197) for one reference patch.
 * Writes the nSimP sorted matches and returns the group size; *n_written
 * is the number of entries the reference wrote (nSimP). */
int ref_similar(const vbm3d_params *prms, const float *video, const float *fflow,
                const float *bflow, vbm3d_dims d, unsigned pidx,
                float *dist, unsigned *idx, unsigned *n_written)
{
    Parameters p = to_ref(prms);
    Video<float> v, ff, bf;
    fill(v, video, d.width, d.height, d.frames, d.channels);
    fill(ff, fflow, d.width, d.height, d.frames, 2);
    fill(bf, bflow, d.width, d.height, d.frames, 2);
    const unsigned sentinel = 0xFFFFFFFFu;
    std::vector<float> distances(p.N, 0.f);
    std::vector<unsigned> indexes(p.N, sentinel);
    int nsx = computeSimilarPatches(distances, indexes, pidx, v, ff, bf, p);
    unsigned nw = 0;
    while (nw < p.N && indexes[nw] != sentinel) nw++;
    for (unsigned i = 0; i < nw; i++) { dist[i] = distances[i]; idx[i] = indexes[i]; }
    *n_written = nw;
    return nsx;
}

/* Same as ref_similar for a batch of reference indices (one video copy). */
int ref_similar_batch(const vbm3d_params *prms, const float *video, const float *fflow,
                      const float *bflow, vbm3d_dims d, const unsigned *pidx, size_t count,
                      float *dist, unsigned *idx, unsigned *nsimp, unsigned *nsx)
{
    Parameters p = to_ref(prms);
    Video<float> v, ff, bf;
    fill(v, video, d.width, d.height, d.frames, d.channels);
    fill(ff, fflow, d.width, d.height, d.frames, 2);
    fill(bf, bflow, d.width, d.height, d.frames, 2);
    const unsigned sentinel = 0xFFFFFFFFu;
    std::vector<float> distances(p.N);
    std::vector<unsigned> indexes(p.N);
    for (size_t r = 0; r < count; r++) {
        std::fill(distances.begin(), distances.end(), 0.f);
        std::fill(indexes.begin(), indexes.end(), sentinel);
        nsx[r] = (unsigned)computeSimilarPatches(distances, indexes, pidx[r], v, ff, bf, p);
        unsigned nw = 0;
        while (nw < p.N && indexes[nw] != sentinel) nw++;
        nsimp[r] = nw;
        for (unsigned i = 0; i < p.N; i++) {
            dist[r * p.N + i] = i < nw ? distances[i] : 0.f;
            idx[r * p.N + i] = i < nw ? indexes[i] : sentinel;
        }
    }
    return 0;
}

/* run_vbm3d (src/vbm3d.cpp:87-376) with `threads` OpenMP threads; noisy is
 * modified in place as in the reference. */
int ref_run(float sigma, float *noisy, const float *fflow, const float *bflow,
            float *basic, float *denoised, const vbm3d_params *p1, const vbm3d_params *p2,
            int color_space, vbm3d_dims d, int threads)
{
    Parameters a = to_ref(p1), b = to_ref(p2);
    Video<float> vn, ff, bf, vb, vd;
    fill(vn, noisy, d.width, d.height, d.frames, d.channels);
    fill(ff, fflow, d.width, d.height, d.frames, 2);
    fill(bf, bflow, d.width, d.height, d.frames, 2);
    if (a.k == 0) fill(vb, basic, d.width, d.height, d.frames, d.channels);
    if (threads > 0) omp_set_num_threads(threads);
    int rc = run_vbm3d(sigma, vn, ff, bf, vb, vd, a, b, color_space != 0);
    const size_t n = (size_t)vn.sz.whcf;
    std::memcpy(noisy, vn.data.data(), sizeof(float) * n);
    std::memcpy(basic, vb.data.data(), sizeof(float) * n);
    std::memcpy(denoised, vd.data.data(), sizeof(float) * n);
    return rc;
}

}  // extern "C"
