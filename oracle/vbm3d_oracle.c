/*
 * CPU restatement of the reference VBM3D hot path — TEST INFRASTRUCTURE.
 *
 * This is the oracle the GPU path is checked against and the CPU baseline
 * that bench.py times ("port").  It is never linked into the product.
 * Every function cites the reference file:line it follows (paths relative
 * to the tehret/vbm3d project root).  Operations are written in the
 * reference's order and precision so that, compiled with
 * -ffp-contract=off, results are bit-identical to the reference built the
 * same way (pinned by tests/test_oracle_golden.py against golden vectors
 * from the reference's own code).
 *
 * Third-party arithmetic restated here:
 *  - FFTW3f REDFT10/REDFT01 (unpinned version; CMakeLists.txt:32-34):
 *    oracle/fftw_shim/fftw_shim.c evaluates FFTW's documented definitions;
 *  - libstdc++ std::partial_sort (GCC 13, bits/stl_algo.h __partial_sort,
 *    __heap_select; bits/stl_heap.h __make_heap, __adjust_heap,
 *    __push_heap, __pop_heap, __sort_heap): restated in oc_partial_sort so
 *    that the order among equal distances is the reference's.
 */
#include "vbm3d_oracle.h"
#include "fftw_shim/fftw3.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* src/vbm3d.cpp:32-37 */
#define OC_SQRT2 1.414213562373095
#define OC_SQRT2_INV 0.7071067811865475
#define OC_DCT 0u
#define OC_BIOR 1u
#define OC_HADAMARD 2u

/* ------------------------------------------------------------------ */
/* Parameters and small helpers                                        */
/* ------------------------------------------------------------------ */

/* initializeParameters_1 / _2 with every CLI option at its default
 * (src/main.cpp:35-125, :127-207).  HAAR is 3 in main.cpp (:30); any value
 * but 2 selects Haar in the steps (src/vbm3d.cpp:579). */
int oracle_default_params(int step, float sigma, vbm3d_params *o)
{
    memset(o, 0, sizeof(*o));
    if (step == 1) {
        o->k = 8;
        o->kt = 1;
        o->Nf = 4; o->Ns = 7; o->Npr = 5; o->Nb = 2;
        o->d = (float)((7. * 7. * 255.) / (o->k * o->k * o->kt));
        o->p = o->k / 4 * 3;
        o->N = 8;
        o->tau = (sigma > 30) ? 4500 : 3000;
        o->lambda3D = 2.7f;
        o->T_2D = o->k == 8 ? OC_BIOR : OC_DCT;
        o->T_3D = 3;
    } else if (step == 2) {
        o->k = (sigma > 30) ? 8 : 7;
        o->kt = 1;
        o->Nf = 4; o->Ns = 7; o->Npr = 5; o->Nb = 2;
        o->d = (float)((3. * 3. * 255.) / (o->k * o->k * o->kt));
        o->p = o->k / 2;
        o->N = 8;
        o->tau = (sigma > 30) ? 3000 : 1500;
        o->T_2D = OC_DCT;
        o->T_3D = 3;
    } else {
        return 1;
    }
    o->mc = 0;
    o->n = 16;
    return 0;
}

/* estimate_sigma (src/Utilities/Utilities.cpp:282-333); the caller passes
 * the bool color_space, so true selects the YCbCr row (1) and false YUV (0),
 * as src/vbm3d.cpp:467 does. */
int oracle_sigma_table(float sigma, unsigned chnls, int color_space, float *t)
{
    if (chnls == 1) {
        t[0] = sigma;
        return 0;
    }
    if (chnls != 3) return 1;
    if (!color_space) {
        t[0] = sqrtf(0.299f * 0.299f + 0.587f * 0.587f + 0.114f * 0.114f) * sigma;
        t[1] = sqrtf(0.14713f * 0.14713f + 0.28886f * 0.28886f + 0.436f * 0.436f) * sigma;
        t[2] = sqrtf(0.615f * 0.615f + 0.51498f * 0.51498f + 0.10001f * 0.10001f) * sigma;
    } else {
        t[0] = sqrtf(0.299f * 0.299f + 0.587f * 0.587f + 0.114f * 0.114f) * sigma;
        t[1] = sqrtf(0.169f * 0.169f + 0.331f * 0.331f + 0.500f * 0.500f) * sigma;
        t[2] = sqrtf(0.500f * 0.500f + 0.419f * 0.419f + 0.081f * 0.081f) * sigma;
    }
    return 0;
}

/* ind_initialize (src/Utilities/Utilities.cpp:400-415). */
static unsigned oc_ind(unsigned end, unsigned step, unsigned *out)
{
    unsigned n = 0, ind = 0, last = 0;
    while (ind <= end) {
        if (out) out[n] = ind;
        last = ind;
        n++;
        ind += step;
    }
    if (last < end) {
        if (out) out[n] = end;
        n++;
    }
    return n;
}

int oracle_grid(const vbm3d_params *p, vbm3d_dims d, unsigned *rows, unsigned *cols,
                unsigned *row_ind, unsigned *col_ind)
{
    if (p->k == 0 || p->p == 0 || d.height < p->k || d.width < p->k) return 1;
    *rows = oc_ind(d.height - p->k, p->p, row_ind);
    *cols = oc_ind(d.width - p->k, p->p, col_ind);
    return 0;
}

/* Modified Bessel function I0 by its power series (double). */
static double oc_bessel_i0(double x)
{
    double sum = 1.0, term = 1.0, q = x * x / 4.0;
    for (int m = 1; m < 60; m++) {
        term *= q / ((double)m * (double)m);
        sum += term;
        if (term < 1e-18 * sum) break;
    }
    return sum;
}

/* Kaiser window of preProcess (src/vbm3d.cpp:1754-1841).  The reference
 * lists literal 4-decimal tables for k in {4, 6, 7, 8, 12} and uses ones
 * otherwise.  Those tables are the outer product of the 1D Kaiser window
 * with beta = 2, rounded to 4 decimals; this generates the same values
 * (equality with the reference's tables is pinned by the golden tests). */
void oracle_kaiser(unsigned k, float *w)
{
    if (k != 4 && k != 6 && k != 7 && k != 8 && k != 12) {
        for (unsigned i = 0; i < k * k; i++) w[i] = 1.0f;
        return;
    }
    double w1[16];
    const double i0b = oc_bessel_i0(2.0);
    for (unsigned n = 0; n < k; n++) {
        double r = 2.0 * n / (k - 1) - 1.0;
        w1[n] = oc_bessel_i0(2.0 * sqrt(1.0 - r * r)) / i0b;
    }
    for (unsigned i = 0; i < k; i++)
        for (unsigned j = 0; j < k; j++) {
            /* round to 4 decimals */
            double v = floor(w1[i] * w1[j] * 1e4 + 0.5);
            w[i * k + j] = (float)(v / 1e4);
        }
}

/* DCT normalisation of preProcess (src/vbm3d.cpp:1843-1863). */
static void oc_coef_norm(unsigned k, float *cn, float *cni)
{
    const float coef = 0.5f / ((float)k);
    for (unsigned i = 0; i < k; i++)
        for (unsigned j = 0; j < k; j++) {
            if (i == 0 && j == 0) {
                cn[i * k + j] = 0.5f * coef;
                cni[i * k + j] = 2.0f;
            } else if (i * j == 0) {
                cn[i * k + j] = (float)(OC_SQRT2_INV * coef);
                cni[i * k + j] = (float)OC_SQRT2;
            } else {
                cn[i * k + j] = 1.0f * coef;
                cni[i * k + j] = 1.0f;
            }
        }
}

/* ------------------------------------------------------------------ */
/* libstdc++ std::partial_sort, restated (see file header)             */
/* ------------------------------------------------------------------ */

typedef struct { float d; unsigned i; } oc_pair;

static void oc_adjust_heap(oc_pair *a, long hole, long len, oc_pair value)
{
    const long top = hole;
    long child = hole;
    while (child < (len - 1) / 2) {
        child = 2 * (child + 1);
        if (a[child].d < a[child - 1].d) child--;
        a[hole] = a[child];
        hole = child;
    }
    if ((len & 1) == 0 && child == (len - 2) / 2) {
        child = 2 * (child + 1);
        a[hole] = a[child - 1];
        hole = child - 1;
    }
    long parent = (hole - 1) / 2;
    while (hole > top && a[parent].d < value.d) {
        a[hole] = a[parent];
        hole = parent;
        parent = (hole - 1) / 2;
    }
    a[hole] = value;
}

static void oc_pop_heap(oc_pair *a, long len, long result)
{
    oc_pair v = a[result];
    a[result] = a[0];
    oc_adjust_heap(a, 0, len, v);
}

static void oc_partial_sort(oc_pair *a, long middle, long last)
{
    if (middle <= 0) return; /* no element of the sorted prefix is used */
    if (middle >= 2) {
        long parent = (middle - 2) / 2;
        for (;;) {
            oc_pair v = a[parent];
            oc_adjust_heap(a, parent, middle, v);
            if (parent == 0) break;
            parent--;
        }
    }
    for (long i = middle; i < last; ++i)
        if (a[i].d < a[0].d) oc_pop_heap(a, middle, i);
    for (long l = middle; l > 1;) {
        --l;
        oc_pop_heap(a, l, l);
    }
}

/* ------------------------------------------------------------------ */
/* Block matching                                                      */
/* ------------------------------------------------------------------ */

typedef struct {
    const vbm3d_params *p;
    const float *vid, *fflow, *bflow;
    unsigned W, H, F, C;
    size_t wh, whc, fwhc; /* flow: 2*wh per frame */
} oc_ctx;

static inline size_t oc_index(const oc_ctx *c, unsigned x, unsigned y, unsigned t, unsigned ch)
{
    return (size_t)t * c->whc + (size_t)ch * c->wh + (size_t)y * c->W + x;
}

static inline void oc_coords(const oc_ctx *c, unsigned idx, unsigned *x, unsigned *y, unsigned *t)
{
    *t = (unsigned)(idx / c->whc);
    *y = (unsigned)((idx % c->wh) / c->W);
    *x = (unsigned)(idx % c->W);
}

static inline float oc_flow(const float *f, const oc_ctx *c, unsigned x, unsigned y, unsigned t,
                            unsigned ch)
{
    if (!f) return 0.f;
    return f[(size_t)t * 2 * c->wh + (size_t)ch * c->wh + (size_t)y * c->W + x];
}

/* patch_trajectory (src/vbm3d.cpp:378-425), FLOAT_TRAJECTORIES defined. */
static void oc_trajectory(const oc_ctx *c, int px, int py, int pt, int traj[][3])
{
    const int k = (int)c->p->k;
    float fpx = (float)px, fpy = (float)py;
    for (int ht = 0; ht < (int)c->p->kt; ht++) {
        traj[ht][0] = px;
        traj[ht][1] = py;
        traj[ht][2] = pt + ht;
        if (c->p->mc && ht < (int)c->p->kt - 1) {
            fpx += oc_flow(c->fflow, c, px + k / 2, py + k / 2, pt + ht, 0);
            fpy += oc_flow(c->fflow, c, px + k / 2, py + k / 2, pt + ht, 1);
            int rx = (int)roundf(fpx), ry = (int)roundf(fpy);
            px = (int)c->W - k < (rx > 0 ? rx : 0) ? (int)c->W - k : (rx > 0 ? rx : 0);
            py = (int)c->H - k < (ry > 0 ? ry : 0) ? (int)c->H - k : (ry > 0 ? ry : 0);
        }
    }
}

/* patchDistance (src/vbm3d.cpp:930-1011): sum over kt, channels, rows and
 * columns of the squared difference, in that order, divided by k*k*kt*C. */
static float oc_distance(const oc_ctx *c, unsigned p1, unsigned p2)
{
    unsigned px, py, pt, qx, qy, qt;
    oc_coords(c, p1, &px, &py, &pt);
    oc_coords(c, p2, &qx, &qy, &qt);
    const unsigned k = c->p->k, kt = c->p->kt;
    float dist = 0.f;
    if (kt == 1) {
        for (unsigned hc = 0; hc < c->C; ++hc)
            for (unsigned hy = 0; hy < k; hy++) {
                const float *a = c->vid + oc_index(c, px, py + hy, pt, hc);
                const float *b = c->vid + oc_index(c, qx, qy + hy, qt, hc);
                for (unsigned hx = 0; hx < k; hx++) {
                    float dif = a[hx] - b[hx];
                    dist += dif * dif;
                }
            }
    } else {
        int t1[16][3], t2[16][3];
        oc_trajectory(c, (int)px, (int)py, (int)pt, t1);
        oc_trajectory(c, (int)qx, (int)qy, (int)qt, t2);
        for (unsigned ht = 0; ht < kt; ht++) {
            unsigned ax = t1[ht][0], ay = t1[ht][1], bx = t2[ht][0], by = t2[ht][1];
            for (unsigned hc = 0; hc < c->C; ++hc)
                for (unsigned hy = 0; hy < k; hy++)
                    for (unsigned hx = 0; hx < k; hx++) {
                        float dif = c->vid[oc_index(c, ax + hx, ay + hy, pt + ht, hc)] -
                                    c->vid[oc_index(c, bx + hx, by + hy, qt + ht, hc)];
                        dist += dif * dif;
                    }
        }
    }
    return dist / (float)(k * k * kt * c->C);
}

/* A search window already scanned for the current reference: the
 * reference's alreadySeen map (src/vbm3d.cpp:1065) holds exactly the
 * positions of the windows scanned before, on the same frame. */
typedef struct { unsigned t, x0, x1, y0, y1; } oc_win;

#define OC_MAX_WINS 600
#define OC_MAX_CAND 1024
#define OC_MAX_BEST 1024

/* localSearch (src/vbm3d.cpp:1013-1080): scan the clamped window around
 * `center` row-major, skip positions already seen, bias the reference's
 * own (x, y) by -d, keep the Nb smallest (partial_sort) and append them. */
static void oc_local_search(const oc_ctx *c, unsigned center, unsigned rpidx, unsigned s,
                            oc_win *wins, int *nwins, oc_pair *out, int *nout)
{
    const int k = (int)c->p->k;
    unsigned rpx, rpy, rpt, px, py, pt;
    oc_coords(c, rpidx, &rpx, &rpy, &rpt);
    oc_coords(c, center, &px, &py, &pt);
    const int half = ((int)s - 1) / 2;
    unsigned x0 = (unsigned)((int)px - half > 0 ? (int)px - half : 0);
    unsigned y0 = (unsigned)((int)py - half > 0 ? (int)py - half : 0);
    unsigned x1 = (unsigned)((int)c->W - k < (int)px + half ? (int)c->W - k : (int)px + half);
    unsigned y1 = (unsigned)((int)c->H - k < (int)py + half ? (int)c->H - k : (int)py + half);

    oc_pair cand[OC_MAX_CAND];
    int n = 0;
    for (unsigned qy = y0; qy <= y1; qy++)
        for (unsigned qx = x0; qx <= x1; qx++) {
            int seen = 0;
            for (int w = 0; w < *nwins; w++)
                if (wins[w].t == pt && qx >= wins[w].x0 && qx <= wins[w].x1 &&
                    qy >= wins[w].y0 && qy <= wins[w].y1) {
                    seen = 1;
                    break;
                }
            if (seen) continue;
            unsigned cur = (unsigned)oc_index(c, qx, qy, pt, 0);
            float dist = oc_distance(c, rpidx, cur) - ((qx == rpx && qy == rpy) ? c->p->d : 0);
            cand[n].d = dist;
            cand[n].i = cur;
            n++;
        }
    wins[*nwins].t = pt;
    wins[*nwins].x0 = x0; wins[*nwins].x1 = x1;
    wins[*nwins].y0 = y0; wins[*nwins].y1 = y1;
    (*nwins)++;
    int nb = (int)c->p->Nb < n ? (int)c->p->Nb : n;
    oc_partial_sort(cand, nb, n);
    for (int i = 0; i < nb; i++) out[(*nout)++] = cand[i];
}

/* computeSimilarPatches (src/vbm3d.cpp:1082-1197), MTRICK off. */
static unsigned oc_similar(const oc_ctx *c, unsigned pidx, float *odist, unsigned *oidx,
                           unsigned *onsimp)
{
    const vbm3d_params *p = c->p;
    const int k = (int)p->k;
    oc_pair best[OC_MAX_BEST];
    int nbest = 0;
    oc_win wins[OC_MAX_WINS];
    int nwins = 0;
    unsigned pre[8], post[8];
    unsigned rpx, rpy, rpt;
    oc_coords(c, pidx, &rpx, &rpy, &rpt);

    oc_local_search(c, pidx, pidx, p->Ns, wins, &nwins, best, &nbest);
    for (unsigned i = 0; i < p->Nb; i++) {
        /* the reference reads bestPatches[i] for every i < Nb
         * (src/vbm3d.cpp:1115-1119); callers guarantee nbest >= Nb */
        pre[i] = best[i].i;
        post[i] = best[i].i;
    }

    unsigned fend = rpt + p->Nf < c->F - p->kt ? rpt + p->Nf : c->F - p->kt;
    unsigned final_f = fend - rpt;
    for (unsigned f = 0; f < final_f; ++f) {
        oc_pair fb[64];
        int nfb = 0;
        for (unsigned m = 0; m < p->Nb; ++m) {
            unsigned px, py, pt;
            oc_coords(c, post[m], &px, &py, &pt);
            int nx = (int)((float)px + roundf(oc_flow(c->fflow, c, px + k / 2, py + k / 2, pt, 0)));
            nx = nx > 0 ? nx : 0;
            px = (unsigned)(nx < (int)c->W - k ? nx : (int)c->W - k);
            int ny = (int)((float)py + roundf(oc_flow(c->fflow, c, px + k / 2, py + k / 2, pt, 1)));
            ny = ny > 0 ? ny : 0;
            py = (unsigned)(ny < (int)c->H - k ? ny : (int)c->H - k);
            unsigned cur = (unsigned)oc_index(c, px, py, pt + 1, 0);
            oc_local_search(c, cur, pidx, p->Npr, wins, &nwins, fb, &nfb);
        }
        int nb = (int)p->Nb < nfb ? (int)p->Nb : nfb;
        oc_partial_sort(fb, nb, nfb);
        for (int i = 0; i < nb; ++i) {
            post[i] = fb[i].i;
            best[nbest++] = fb[i];
        }
    }

    unsigned final_b = rpt - ((int)(rpt - p->Nf) > 0 ? (unsigned)(int)(rpt - p->Nf) : 0u);
    for (unsigned f = 0; f < final_b; ++f) {
        oc_pair fb[64];
        int nfb = 0;
        for (unsigned m = 0; m < p->Nb; ++m) {
            unsigned px, py, pt;
            oc_coords(c, pre[m], &px, &py, &pt);
            int nx = (int)((float)px + roundf(oc_flow(c->bflow, c, px + k / 2, py + k / 2, pt - 1, 0)));
            nx = nx > 0 ? nx : 0;
            px = (unsigned)(nx < (int)c->W - k ? nx : (int)c->W - k);
            int ny = (int)((float)py + roundf(oc_flow(c->bflow, c, px + k / 2, py + k / 2, pt - 1, 1)));
            ny = ny > 0 ? ny : 0;
            py = (unsigned)(ny < (int)c->H - k ? ny : (int)c->H - k);
            unsigned cur = (unsigned)oc_index(c, px, py, pt - 1, 0);
            oc_local_search(c, cur, pidx, p->Npr, wins, &nwins, fb, &nfb);
        }
        int nb = (int)p->Nb < nfb ? (int)p->Nb : nfb;
        oc_partial_sort(fb, nb, nfb);
        for (int i = 0; i < nb; ++i) {
            pre[i] = fb[i].i;
            best[nbest++] = fb[i];
        }
    }

    const unsigned nsimp = p->N < (unsigned)nbest ? p->N : (unsigned)nbest;
    oc_partial_sort(best, (long)nsimp, nbest);
    for (unsigned n = 0; n < nsimp; n++) {
        odist[n] = best[n].d;
        oidx[n] = best[n].i;
    }
    *onsimp = nsimp;
    unsigned thr = nsimp - 1;
    while (odist[thr] > p->tau && thr > 0) thr--;
    unsigned r = 1; /* closest_power_of_2, src/Utilities/Utilities.cpp:257-265 */
    while (r * 2 <= thr + 1) r *= 2;
    return r;
}

static int oc_check(const vbm3d_params *p, vbm3d_dims d)
{
    if (!p || p->k == 0 || p->kt == 0 || p->p == 0 || p->N == 0 || p->Nb == 0 || p->Nb > 8 ||
        p->N > 32 || p->k > 16 || p->kt > 16 || p->Ns > 31 || p->Npr > 31 || p->Nf > 32)
        return 1;
    if (d.width < p->k || d.height < p->k || d.frames < p->kt) return 1;
    if (d.channels != 1 && d.channels != 3) return 1;
    if (p->T_2D == OC_BIOR && p->k != 8) return 1;
    /* the reference reads Nb entries of the reference-frame window */
    unsigned h = (p->Ns - 1) / 2 + 1;
    unsigned wx = h < d.width - p->k + 1 ? h : d.width - p->k + 1;
    unsigned wy = h < d.height - p->k + 1 ? h : d.height - p->k + 1;
    if (wx * wy < p->Nb) return 1;
    return 0;
}

static void oc_ctx_init(oc_ctx *c, const vbm3d_params *p, const float *vid, const float *ff,
                        const float *bf, vbm3d_dims d)
{
    c->p = p;
    c->vid = vid; c->fflow = ff; c->bflow = bf;
    c->W = d.width; c->H = d.height; c->F = d.frames; c->C = d.channels;
    c->wh = (size_t)d.width * d.height;
    c->whc = c->wh * d.channels;
    c->fwhc = c->wh * 2;
}

int oracle_similar_batch(const vbm3d_params *p, const float *video, const float *fflow,
                         const float *bflow, vbm3d_dims d, const unsigned *pidx, size_t count,
                         float *dist, unsigned *idx, unsigned *nsimp, unsigned *nsx)
{
    if (oc_check(p, d)) return 1;
    oc_ctx c;
    oc_ctx_init(&c, p, video, fflow, bflow, d);
#pragma omp parallel for schedule(dynamic, 16)
    for (long r = 0; r < (long)count; r++) {
        float dd[32];
        unsigned ii[32], ns;
        nsx[r] = oc_similar(&c, pidx[r], dd, ii, &ns);
        nsimp[r] = ns;
        for (unsigned i = 0; i < p->N; i++) {
            dist[r * p->N + i] = i < ns ? dd[i] : 0.f;
            idx[r * p->N + i] = i < ns ? ii[i] : 0xFFFFFFFFu;
        }
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* Transforms                                                          */
/* ------------------------------------------------------------------ */

/* bior1.5 basis of the MATLAB path (src/lib_transforms.cpp:139-148 forward,
 * :279-288 inverse), restated as row-major tables: FWD[j][k] is basis row j.
 * Values are double literals stored as float, as the reference does. */
static const double OC_BIOR_FWD[8][8] = {
    {0.353553390593274, 0.353553390593274, 0.353553390593274, 0.353553390593274,
     0.353553390593274, 0.353553390593274, 0.353553390593274, 0.353553390593274},
    {0.219417649252501, 0.449283757993216, 0.449283757993216, 0.219417649252501,
     -0.219417649252501, -0.449283757993216, -0.449283757993216, -0.219417649252501},
    {0.569359398342846, 0.402347308162278, -0.402347308162278, -0.569359398342846,
     -0.083506045090284, 0.083506045090284, -0.083506045090284, 0.083506045090284},
    {-0.083506045090284, 0.083506045090284, -0.083506045090284, 0.083506045090284,
     0.569359398342846, 0.402347308162278, -0.402347308162278, -0.569359398342846},
    {0.707106781186547, -0.707106781186547, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0},
    {0.0, 0.0, 0.707106781186547, -0.707106781186547, 0.0, 0.0, 0.0, 0.0},
    {0.0, 0.0, 0.0, 0.0, 0.707106781186547, -0.707106781186547, 0.0, 0.0},
    {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.707106781186547, -0.707106781186547}};
static const double OC_BIOR_INV[8][8] = {
    {0.353553390593274, 0.353553390593274, 0.5, 0.0, 0.707106781186547, -0.121533978016438, 0.0, 0.121533978016438},
    {0.353553390593274, 0.353553390593274, 0.5, -0.0, -0.707106781186547, -0.121533978016438, 0.0, 0.121533978016438},
    {0.353553390593274, 0.353553390593274, -0.5, -0.0, 0.121533978016438, 0.707106781186548, -0.121533978016438, 0.0},
    {0.353553390593274, 0.353553390593274, -0.5, 0.0, 0.121533978016438, -0.707106781186548, -0.121533978016438, 0.0},
    {0.353553390593274, -0.353553390593274, 0.0, 0.5, 0.0, 0.121533978016438, 0.707106781186547, -0.121533978016438},
    {0.353553390593274, -0.353553390593274, 0.0, 0.5, 0.0, 0.121533978016438, -0.707106781186547, -0.121533978016438},
    {0.353553390593274, -0.353553390593274, 0.0, -0.5, -0.121533978016438, 0.0, 0.121533978016438, 0.707106781186547},
    {0.353553390593274, -0.353553390593274, 0.0, -0.5, -0.121533978016438, 0.0, 0.121533978016438, -0.707106781186547}};

/* Two passes of bior_2d_forward / bior_2d_inverse (src/lib_transforms.cpp
 * :158-176, :298-316): t2[i][j] = sum_k t[i][k] B[j][k]; then
 * out[i][j] = sum_k t2[k][i] B[j][k], each sum in k order from 0. */
static void oc_bior_passes(float *t, const double B[8][8])
{
    float b[8][8], t2[64];
    for (int j = 0; j < 8; j++)
        for (int k = 0; k < 8; k++) b[j][k] = (float)B[j][k];
    for (int i = 0; i < 8; i++)
        for (int j = 0; j < 8; j++) {
            float m = 0.f;
            for (int k = 0; k < 8; k++) m += t[i * 8 + k] * b[j][k];
            t2[i * 8 + j] = m;
        }
    for (int i = 0; i < 8; i++)
        for (int j = 0; j < 8; j++) {
            float m = 0.f;
            for (int k = 0; k < 8; k++) m += t2[k * 8 + i] * b[j][k];
            t[i * 8 + j] = m;
        }
}

/* bior_2d_forward: block row i = pixel row (src/lib_transforms.cpp:154-180). */
void oracle_bior2d_forward(const float *in, float *out)
{
    float t[64];
    memcpy(t, in, sizeof t);
    oc_bior_passes(t, OC_BIOR_FWD);
    memcpy(out, t, sizeof t);
}

/* bior_2d_inverse: transposed read and write (src/lib_transforms.cpp:294-320). */
void oracle_bior2d_inverse(const float *in, float *out)
{
    float t[64];
    for (int i = 0; i < 8; i++)
        for (int j = 0; j < 8; j++) t[i * 8 + j] = in[i + j * 8];
    oc_bior_passes(t, OC_BIOR_INV);
    for (int i = 0; i < 8; i++)
        for (int j = 0; j < 8; j++) out[j * 8 + i] = t[i * 8 + j];
}

/* FFTW REDFT10 / REDFT01 on one k x k block through the shim. */
static void oc_redft(const float *in, float *out, unsigned k, fftwf_r2r_kind kind)
{
    int n[2] = {(int)k, (int)k};
    fftwf_r2r_kind kinds[2] = {kind, kind};
    fftwf_plan pl = fftwf_plan_many_r2r(2, n, 1, (float *)in, n, 1, (int)(k * k), out, n, 1,
                                        (int)(k * k), kinds, FFTW_ESTIMATE);
    fftwf_execute_r2r(pl, (float *)in, out);
    fftwf_destroy_plan(pl);
}

/* dct_2d_process normalisation (src/vbm3d.cpp:1294-1302). */
void oracle_dct2d_forward(const float *in, float *out, unsigned k)
{
    float cn[256], cni[256], tmp[256];
    oc_coef_norm(k, cn, cni);
    oc_redft(in, tmp, k, FFTW_REDFT10);
    for (unsigned i = 0; i < k * k; i++) out[i] = tmp[i] * cn[i];
}

/* dct_2d_inv (src/vbm3d.cpp:1696-1709). */
void oracle_dct2d_inverse(const float *in, float *out, unsigned k)
{
    float cn[256], cni[256], tmp[256], tmp2[256];
    oc_coef_norm(k, cn, cni);
    for (unsigned i = 0; i < k * k; i++) tmp[i] = in[i] * cni[i];
    oc_redft(tmp, tmp2, k, FFTW_REDFT01);
    const float coef = 1.0f / (float)(k * 2);
    for (unsigned i = 0; i < k * k; i++) out[i] = coef * tmp2[i];
}

/* haar_forward (src/lib_transforms.cpp:453-476): the double constant
 * promotes each product to double before the float store. */
void oracle_haar_forward(float *v, unsigned n)
{
    float tmp[64];
    int k = (int)n;
    while (1 < k) {
        k = k / 2;
        for (int i = 0; i < k; i++) {
            tmp[i] = (float)((double)(v[2 * i] + v[2 * i + 1]) * OC_SQRT2_INV);
            tmp[i + k] = (float)((double)(v[2 * i] - v[2 * i + 1]) * OC_SQRT2_INV);
        }
        for (int i = 0; i < k * 2; i++) v[i] = tmp[i];
    }
}

/* haar_inverse (src/lib_transforms.cpp:489-512). */
void oracle_haar_inverse(float *v, unsigned n)
{
    float tmp[64];
    int k = 1;
    while (k * 2 <= (int)n) {
        for (int i = 0; i < k; ++i) {
            tmp[2 * i] = (float)((double)(v[i] + v[i + k]) * OC_SQRT2_INV);
            tmp[2 * i + 1] = (float)((double)(v[i] - v[i + k]) * OC_SQRT2_INV);
        }
        for (int i = 0; i < k * 2; i++) v[i] = tmp[i];
        k = k * 2;
    }
}

/* hadamard_transform (src/lib_transforms.cpp:410-440), unnormalised. */
static void oc_hadamard(float *v, unsigned n)
{
    if (n == 1) return;
    if (n == 2) {
        const float a = v[0], b = v[1];
        v[0] = a + b;
        v[1] = a - b;
        return;
    }
    float tmp[64];
    const unsigned h = n / 2;
    for (unsigned k = 0; k < h; k++) {
        const float a = v[2 * k], b = v[2 * k + 1];
        v[k] = a + b;
        tmp[k] = a - b;
    }
    for (unsigned k = 0; k < h; k++) v[h + k] = tmp[k];
    oc_hadamard(v, h);
    oc_hadamard(v + h, h);
}

/* temporal_transform / temporal_inv_transform (src/vbm3d.cpp:1866-1956)
 * on a group laid out [c][k2t][n]; kt > 1 and T_2D != BIOR only. */
static void oc_temporal(float *g, unsigned k, unsigned kt, unsigned chnls, unsigned nsx, int inverse)
{
    const unsigned k2 = k * k, k2t = k2 * kt;
    const float norm = (float)(1. / sqrt(2 * kt));
    int n1[1] = {(int)kt};
    fftwf_r2r_kind kind = inverse ? FFTW_REDFT01 : FFTW_REDFT10;
    fftwf_plan pl = fftwf_plan_many_r2r(1, n1, 1, NULL, n1, 1, (int)kt, NULL, n1, 1, (int)kt,
                                        &kind, FFTW_ESTIMATE);
    float in[16], out[16];
    for (unsigned c = 0; c < chnls; c++)
        for (unsigned n = 0; n < nsx; n++)
            for (unsigned q = 0; q < k2; q++) {
                for (unsigned t = 0; t < kt; t++) {
                    float v = g[n + (q + t * k2) * nsx + c * k2t * nsx];
                    in[t] = inverse ? (float)(v * (t == 0 ? OC_SQRT2 : 1.)) : v;
                }
                fftwf_execute_r2r(pl, in, out);
                for (unsigned t = 0; t < kt; t++)
                    g[n + (q + t * k2) * nsx + c * k2t * nsx] =
                        inverse ? out[t] * norm
                                : (float)(out[t] * norm * (t == 0 ? OC_SQRT2_INV : 1.));
            }
    fftwf_destroy_plan(pl);
}

/* ------------------------------------------------------------------ */
/* Steps                                                               */
/* ------------------------------------------------------------------ */

typedef struct {
    unsigned nsx;
    unsigned idx[32];
    float w[3];
} oc_ref_out;

/* Gather the 2D-transformed table of one video for the group
 * (dct_2d_process / bior_2d_process, src/vbm3d.cpp:1218-1386), laid out
 * as the reference's group_3D: [c][k2t][n] (src/vbm3d.cpp:565-570). */
static void oc_build_group(const oc_ctx *c, const float *vid, const unsigned *idx, unsigned nsx,
                           const float *cn, float *g)
{
    const vbm3d_params *p = c->p;
    const unsigned k = p->k, k2 = k * k, k2t = k2 * p->kt;
    float blk[256], tr[256];
    for (unsigned ch = 0; ch < c->C; ch++)
        for (unsigned n = 0; n < nsx; n++) {
            unsigned x, y, t;
            oc_coords(c, idx[n], &x, &y, &t);
            int traj[16][3];
            oc_trajectory(c, (int)x, (int)y, (int)t, traj);
            for (unsigned ht = 0; ht < p->kt; ht++) {
                unsigned tx = traj[ht][0], ty = traj[ht][1];
                for (unsigned pp = 0; pp < k; pp++)
                    for (unsigned q = 0; q < k; q++)
                        blk[pp * k + q] = vid[oc_index(c, tx + q, ty + pp, t + ht, ch)];
                if (p->T_2D == OC_BIOR) {
                    oracle_bior2d_forward(blk, tr);
                } else {
                    oc_redft(blk, tr, k, FFTW_REDFT10);
                    for (unsigned i = 0; i < k2; i++) tr[i] = tr[i] * cn[i];
                }
                for (unsigned q = 0; q < k2; q++)
                    g[n + (q + ht * k2) * nsx + ch * k2t * nsx] = tr[q];
            }
        }
}

/* One reference patch: block matching, 2D transforms, 1D transform along
 * the group, shrinkage, inverse transforms.  Writes the group estimate
 * laid out [c][n][k2t] (the push order of src/vbm3d.cpp:592-595) after the
 * 2D inverse of dct_2d_inv / bior_2d_inv (src/vbm3d.cpp:1678-1731). */
static void oc_process_ref(int step, const oc_ctx *c, const float *noisy, const float *basic,
                           unsigned pidx, const float *sig, const float *cn, const float *cni,
                           float *est, oc_ref_out *ro)
{
    const vbm3d_params *p = c->p;
    const unsigned k = p->k, k2 = k * k, kt = p->kt, k2t = k2 * kt, C = c->C;
    float dd[32];
    unsigned ns;
    const unsigned nsx = oc_similar(c, pidx, dd, ro->idx, &ns);
    ro->nsx = nsx;
    const size_t gsz = (size_t)C * k2t * nsx;
    float *g = (float *)malloc(sizeof(float) * gsz);
    float *gb = step == 2 ? (float *)malloc(sizeof(float) * gsz) : NULL;
    const int temporal = kt > 1 && p->T_2D != OC_BIOR;

    if (step == 1) {
        oc_build_group(c, noisy, ro->idx, nsx, cn, g);
        if (temporal) oc_temporal(g, k, kt, C, nsx, 0);
        float wt[3] = {0.f, 0.f, 0.f};
        if (p->T_3D == OC_HADAMARD) {
            /* ht_filtering_hadamard, src/vbm3d.cpp:1405-1456 */
            const float coef_norm = sqrtf((float)nsx);
            const float coef = 1.0f / (float)nsx;
            for (unsigned v = 0; v < k2t * C; v++) oc_hadamard(g + v * nsx, nsx);
            for (unsigned ch = 0; ch < C; ch++) {
                const unsigned dc = ch * nsx * k2t;
                const float T = p->lambda3D * sig[ch] * coef_norm;
                for (unsigned q = 0; q < k2t * nsx; q++) {
                    if (q == 0 || fabsf(g[q + dc]) > T) wt[ch]++;
                    else g[q + dc] = 0.0f;
                }
            }
            for (unsigned v = 0; v < k2t * C; v++) oc_hadamard(g + v * nsx, nsx);
            for (size_t q = 0; q < gsz; q++) g[q] *= coef;
        } else {
            /* ht_filtering_haar, src/vbm3d.cpp:1475-1521 */
            for (unsigned v = 0; v < k2t * C; v++) oracle_haar_forward(g + v * nsx, nsx);
            for (unsigned ch = 0; ch < C; ch++) {
                const unsigned dc = ch * nsx * k2t;
                const float T = p->lambda3D * sig[ch];
                for (unsigned q = 0; q < k2t * nsx; q++) {
                    if (q == 0 || fabsf(g[q + dc]) > T) wt[ch]++;
                    else g[q + dc] = 0.0f;
                }
            }
            for (unsigned v = 0; v < k2t * C; v++) oracle_haar_inverse(g + v * nsx, nsx);
        }
        for (unsigned ch = 0; ch < C; ch++)
            ro->w[ch] = 1.f / (float)(sig[ch] * sig[ch] * wt[ch]);
        if (temporal) oc_temporal(g, k, kt, C, nsx, 1);
    } else {
        oc_build_group(c, noisy, ro->idx, nsx, cn, g);   /* group_3D_vid */
        oc_build_group(c, basic, ro->idx, nsx, cn, gb);  /* group_3D_est */
        if (temporal) {
            oc_temporal(gb, k, kt, C, nsx, 0);
            oc_temporal(g, k, kt, C, nsx, 0);
        }
        float wt[3] = {0.f, 0.f, 0.f};
        if (p->T_3D == OC_HADAMARD) {
            /* wiener_filtering_hadamard, src/vbm3d.cpp:1539-1594 (DCWIENER) */
            const float coef = 1.0f / (float)nsx;
            for (unsigned v = 0; v < k2t * C; v++) {
                oc_hadamard(g + v * nsx, nsx);
                oc_hadamard(gb + v * nsx, nsx);
            }
            for (unsigned ch = 0; ch < C; ch++) {
                const unsigned dc = ch * nsx * k2t;
                for (unsigned q = 0; q < k2t * nsx; q++) {
                    float value = gb[dc + q] * gb[dc + q] * coef;
                    value /= (value + sig[ch] * sig[ch]);
                    gb[q + dc] = g[q + dc] * value * coef;
                    wt[ch] += (value * value);
                }
            }
            for (unsigned v = 0; v < k2t * C; v++) oc_hadamard(gb + v * nsx, nsx);
            for (unsigned ch = 0; ch < C; ch++)
                ro->w[ch] = (wt[ch] > 0.0f ? 1.0f / (float)(sig[ch] * sig[ch] * wt[ch]) : 1.0f);
        } else {
            /* wiener_filtering_haar, src/vbm3d.cpp:1613-1666 (DCWIENER) */
            for (unsigned v = 0; v < k2t * C; v++) {
                oracle_haar_forward(g + v * nsx, nsx);
                oracle_haar_forward(gb + v * nsx, nsx);
            }
            for (unsigned ch = 0; ch < C; ch++) {
                const unsigned dc = ch * nsx * k2t;
                for (unsigned q = 0; q < k2t * nsx; q++) {
                    float value = gb[dc + q] * gb[dc + q];
                    value /= (value + sig[ch] * sig[ch]);
                    gb[q + dc] = g[q + dc] * value;
                    wt[ch] += (value * value);
                }
            }
            for (unsigned v = 0; v < k2t * C; v++) oracle_haar_inverse(gb + v * nsx, nsx);
            for (unsigned ch = 0; ch < C; ch++)
                ro->w[ch] = 1.f / (float)(sig[ch] * sig[ch] * wt[ch]);
        }
        if (temporal) oc_temporal(gb, k, kt, C, nsx, 1);
        float *sw = g; g = gb; gb = sw; /* the estimate is group_3D_est */
    }

    /* regroup [c][k2t][n] -> [c][n][k2t] and apply the 2D inverse */
    float blk[256], out[256];
    for (unsigned ch = 0; ch < C; ch++)
        for (unsigned n = 0; n < nsx; n++)
            for (unsigned ht = 0; ht < kt; ht++) {
                for (unsigned q = 0; q < k2; q++)
                    blk[q] = g[n + (q + ht * k2) * nsx + ch * k2t * nsx];
                if (p->T_2D == OC_BIOR) {
                    oracle_bior2d_inverse(blk, out);
                } else {
                    float tmp[256];
                    for (unsigned q = 0; q < k2; q++) tmp[q] = blk[q] * cni[q];
                    oc_redft(tmp, out, k, FFTW_REDFT01);
                    const float coef = 1.0f / (float)(k * 2);
                    for (unsigned q = 0; q < k2; q++) out[q] = coef * out[q];
                }
                memcpy(est + (size_t)ch * nsx * k2t + (size_t)n * k2t + ht * k2, out,
                       sizeof(float) * k2);
            }
    free(g);
    if (gb) free(gb);
}

/* vbm3d_1st_step / vbm3d_2nd_step with crop == NULL
 * (src/vbm3d.cpp:447-654, :676-928). */
int oracle_step(int step, const vbm3d_params *p, const float *noisy, const float *basic,
                const float *fflow, const float *bflow, vbm3d_dims d, float sigma,
                int color_space, float *num, float *den, int threads)
{
    if ((step != 1 && step != 2) || oc_check(p, d)) return 1;
    float sig[3];
    if (oracle_sigma_table(sigma, d.channels, color_space, sig)) return 5;
    oc_ctx c;
    oc_ctx_init(&c, p, step == 1 ? noisy : basic, fflow, bflow, d);
    const unsigned k = p->k, k2 = k * k, kt = p->kt, k2t = k2 * kt, C = d.channels;
    unsigned *rows = (unsigned *)malloc(sizeof(unsigned) * (d.height + 2));
    unsigned *cols = (unsigned *)malloc(sizeof(unsigned) * (d.width + 2));
    unsigned nr, nc;
    oracle_grid(p, d, &nr, &nc, rows, cols);
    float kai[256], cn[256], cni[256];
    oracle_kaiser(k, kai);
    oc_coef_norm(k, cn, cni);
    const size_t total = (size_t)c.whc * d.frames;
    memset(num, 0, sizeof(float) * total);
    memset(den, 0, sizeof(float) * total);

    const size_t per_ref = (size_t)C * p->N * k2t;
    const size_t chunk = nc;  /* one row of references, as the reference aggregates per row */
    float *est = (float *)malloc(sizeof(float) * per_ref * chunk);
    oc_ref_out *ro = (oc_ref_out *)malloc(sizeof(oc_ref_out) * chunk);
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#else
    (void)threads;
#endif
    for (unsigned tr = 0; tr < d.frames - kt + 1; ++tr)
        for (unsigned ir = 0; ir < nr; ir++) {
#pragma omp parallel for schedule(dynamic, 4)
            for (long jr = 0; jr < (long)nc; jr++) {
                unsigned pidx = (unsigned)oc_index(&c, cols[jr], rows[ir], tr, 0);
                oc_process_ref(step, &c, noisy, basic, pidx, sig, cn, cni,
                               est + (size_t)jr * per_ref, &ro[jr]);
            }
            /* aggregation in the reference's order (src/vbm3d.cpp:612-650) */
            for (unsigned jr = 0; jr < nc; jr++) {
                const unsigned nsx = ro[jr].nsx;
                const float *e = est + (size_t)jr * per_ref;
                for (unsigned ch = 0; ch < C; ch++)
                    for (unsigned n = 0; n < nsx; n++) {
                        unsigned x, y, t;
                        oc_coords(&c, ro[jr].idx[n], &x, &y, &t);
                        int traj[16][3];
                        oc_trajectory(&c, (int)x, (int)y, (int)t, traj);
                        for (unsigned ht = 0; ht < kt; ht++) {
                            unsigned tx = traj[ht][0], ty = traj[ht][1];
                            for (unsigned pp = 0; pp < k; pp++)
                                for (unsigned q = 0; q < k; q++) {
                                    size_t o = oc_index(&c, tx + q, ty + pp, t + ht, ch);
                                    num[o] += kai[pp * k + q] * ro[jr].w[ch] *
                                              e[pp * k + q + ht * k2 + n * k2t + ch * k2t * nsx];
                                    den[o] += kai[pp * k + q] * ro[jr].w[ch];
                                }
                        }
                    }
            }
        }
    free(est);
    free(ro);
    free(rows);
    free(cols);
    return 0;
}

/* transformColorSpace, 3 channels (src/Utilities/LibVideoT.hpp:763-888). */
void oracle_color_transform(float *v, vbm3d_dims d, int forward)
{
    if (d.channels != 3) return;
    const size_t wh = (size_t)d.width * d.height;
    for (unsigned f = 0; f < d.frames; f++) {
        float *r = v + (size_t)f * wh * 3, *g = r + wh, *b = g + wh;
        for (size_t k = 0; k < wh; k++) {
            float o0, o1, o2;
            if (forward) {
                o0 = 0.299f * r[k] + 0.587f * g[k] + 0.114f * b[k];
                o1 = -0.14713f * r[k] - 0.28886f * g[k] + 0.436f * b[k];
                o2 = 0.615f * r[k] - 0.51498f * g[k] - 0.10001f * b[k];
            } else {
                o0 = r[k] + 1.13983f * b[k];
                o1 = r[k] - 0.39465f * g[k] - 0.5806f * b[k];
                o2 = r[k] + 2.03211f * g[k];
            }
            r[k] = o0; g[k] = o1; b[k] = o2;
        }
    }
}

int oracle_run(float sigma, float *noisy, const float *fflow, const float *bflow,
               float *basic, float *denoised, const vbm3d_params *p1,
               const vbm3d_params *p2, int color_space, vbm3d_dims d, int threads)
{
    const size_t n = (size_t)d.width * d.height * d.frames * d.channels;
    if (color_space) {
        if (p1->k > 0) oracle_color_transform(noisy, d, 1);
        else oracle_color_transform(basic, d, 1);
    }
    float *num = (float *)malloc(sizeof(float) * n), *den = (float *)malloc(sizeof(float) * n);
    int rc = 0;
    if (p1->k > 0) {
        rc = oracle_step(1, p1, noisy, NULL, fflow, bflow, d, sigma, color_space, num, den, threads);
        if (rc) goto out;
        for (size_t i = 0; i < n; i++) basic[i] = den[i] == 0 ? noisy[i] : num[i] / den[i];
    }
    if (p2->k > 0) {
        rc = oracle_step(2, p2, noisy, basic, fflow, bflow, d, sigma, color_space, num, den, threads);
        if (rc) goto out;
        for (size_t i = 0; i < n; i++) denoised[i] = den[i] == 0 ? basic[i] : num[i] / den[i];
    } else {
        memcpy(denoised, basic, sizeof(float) * n);
    }
    if (color_space) {
        oracle_color_transform(denoised, d, 0);
        oracle_color_transform(noisy, d, 0);
        oracle_color_transform(basic, d, 0);
    }
out:
    free(num);
    free(den);
    return rc;
}

/* ------------------------------------------------------------------ */
/* Frozen linearisation of one step, in double precision              */
/* ------------------------------------------------------------------ */

/* 1D transforms in double: haar_forward / haar_inverse and the reference's
 * Walsh-Hadamard (src/lib_transforms.cpp:410-512). */
static void od_haar(double *v, unsigned n, int inverse)
{
    double tmp[64];
    const double s = 0.7071067811865475;
    if (!inverse) {
        for (int k = (int)n / 2; k >= 1; k /= 2) {
            for (int i = 0; i < k; i++) {
                tmp[i] = (v[2 * i] + v[2 * i + 1]) * s;
                tmp[i + k] = (v[2 * i] - v[2 * i + 1]) * s;
            }
            for (int i = 0; i < 2 * k; i++) v[i] = tmp[i];
        }
    } else {
        for (int k = 1; k * 2 <= (int)n; k *= 2) {
            for (int i = 0; i < k; i++) {
                tmp[2 * i] = (v[i] + v[i + k]) * s;
                tmp[2 * i + 1] = (v[i] - v[i + k]) * s;
            }
            for (int i = 0; i < 2 * k; i++) v[i] = tmp[i];
        }
    }
}

static void od_hadamard(double *v, unsigned n)
{
    if (n == 1) return;
    double tmp[64];
    const unsigned h = n / 2;
    for (unsigned k = 0; k < h; k++) {
        tmp[k] = v[2 * k] + v[2 * k + 1];
        tmp[h + k] = v[2 * k] - v[2 * k + 1];
    }
    od_hadamard(tmp, h);
    od_hadamard(tmp + h, h);
    for (unsigned k = 0; k < n; k++) v[k] = tmp[k];
}

/* 2D transforms of one k x k block in double with the float-valued
 * coefficients of the forward pass (bior1.5 bases, DCT normalisations). */
static void od_2d(const double *in, double *out, unsigned k, unsigned t2d, int inverse)
{
    float cn[256], cni[256];
    oc_coef_norm(k, cn, cni);
    if (t2d == OC_BIOR) {
        double b[8][8], t[64], t2[64];
        for (int j = 0; j < 8; j++)
            for (int q = 0; q < 8; q++) b[j][q] = (double)(float)(inverse ? OC_BIOR_INV[j][q] : OC_BIOR_FWD[j][q]);
        for (int i = 0; i < 8; i++)
            for (int j = 0; j < 8; j++) t[i * 8 + j] = inverse ? in[i + j * 8] : in[i * 8 + j];
        for (int i = 0; i < 8; i++)
            for (int j = 0; j < 8; j++) {
                double m = 0;
                for (int q = 0; q < 8; q++) m += t[i * 8 + q] * b[j][q];
                t2[i * 8 + j] = m;
            }
        for (int i = 0; i < 8; i++)
            for (int j = 0; j < 8; j++) {
                double m = 0;
                for (int q = 0; q < 8; q++) m += t2[q * 8 + i] * b[j][q];
                if (inverse) out[j * 8 + i] = m;
                else out[i * 8 + j] = m;
            }
        return;
    }
    const double pi = 3.14159265358979323846;
    double m[16][16], t[256];
    for (unsigned u = 0; u < k; u++)
        for (unsigned j = 0; j < k; j++)
            m[u][j] = inverse ? (u == 0 ? 1.0 : 2.0 * cos(pi * u * (j + 0.5) / k)) : 2.0 * cos(pi * (j + 0.5) * u / k);
    double z[256];
    for (unsigned e = 0; e < k * k; e++) z[e] = inverse ? in[e] * (double)cni[e] : in[e];
    /* rows then columns: Y = M Z M^T, with M[u][j] the 1D transform matrix
     * (REDFT10: Y[u] = sum_j X[j] m[u][j]; REDFT01: X[j] = sum_u Z[u] m[u][j]) */
    for (unsigned i = 0; i < k; i++)
        for (unsigned v = 0; v < k; v++) {
            double a = 0;
            for (unsigned j = 0; j < k; j++) a += z[i * k + j] * (inverse ? m[j][v] : m[v][j]);
            t[i * k + v] = a;
        }
    for (unsigned u = 0; u < k; u++)
        for (unsigned v = 0; v < k; v++) {
            double a = 0;
            for (unsigned i = 0; i < k; i++) a += (inverse ? m[i][u] : m[u][i]) * t[i * k + v];
            out[u * k + v] = inverse ? a * (double)(1.0f / (float)(k * 2)) : a * (double)cn[u * k + v];
        }
}

int oracle_linear_apply(int step, const vbm3d_params *p, const float *noisy, const float *basic,
                        const float *fflow, const float *bflow, vbm3d_dims d, float sigma, int color_space,
                        const float *x, double *out, int threads)
{
    if ((step != 1 && step != 2) || oc_check(p, d) || p->kt != 1) return 1;
    float sig[3];
    if (oracle_sigma_table(sigma, d.channels, color_space, sig)) return 5;
    const float *src = step == 1 ? noisy : basic;
    oc_ctx c;
    oc_ctx_init(&c, p, src, fflow, bflow, d);
    const unsigned k = p->k, k2 = k * k, C = d.channels;
    unsigned *rows = (unsigned *)malloc(sizeof(unsigned) * (d.height + 2));
    unsigned *cols = (unsigned *)malloc(sizeof(unsigned) * (d.width + 2));
    unsigned nr, nc;
    oracle_grid(p, d, &nr, &nc, rows, cols);
    float kai[256], cn[256], cni[256];
    oracle_kaiser(k, kai);
    oc_coef_norm(k, cn, cni);
    const size_t total = (size_t)c.whc * d.frames;
    double *num = (double *)calloc(total, sizeof(double)), *den = (double *)calloc(total, sizeof(double));
    const size_t per_ref = (size_t)C * p->N * k2;
    double *est = (double *)malloc(sizeof(double) * per_ref * nc);
    oc_ref_out *ro = (oc_ref_out *)malloc(sizeof(oc_ref_out) * nc);
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#else
    (void)threads;
#endif
    for (unsigned tr = 0; tr < d.frames; ++tr)
        for (unsigned ir = 0; ir < nr; ir++) {
#pragma omp parallel for schedule(dynamic, 4)
            for (long jr = 0; jr < (long)nc; jr++) {
                unsigned pidx = (unsigned)oc_index(&c, cols[jr], rows[ir], tr, 0);
                float dd[32];
                unsigned ns;
                const unsigned nsx = oc_similar(&c, pidx, dd, ro[jr].idx, &ns);
                ro[jr].nsx = nsx;
                /* frozen gains from the source group, float as the forward */
                float *g = (float *)malloc(sizeof(float) * C * k2 * nsx);
                oc_build_group(&c, src, ro[jr].idx, nsx, cn, g);
                double *lam = (double *)malloc(sizeof(double) * C * k2 * nsx);
                float wt[3] = {0.f, 0.f, 0.f};
                const float coefn = 1.0f / (float)nsx;
                for (unsigned ch = 0; ch < C; ch++)
                    for (unsigned q = 0; q < k2; q++) {
                        float *v = g + (ch * k2 + q) * nsx;
                        if (p->T_3D == OC_HADAMARD) oc_hadamard(v, nsx);
                        else oracle_haar_forward(v, nsx);
                        for (unsigned n = 0; n < nsx; n++) {
                            double l;
                            if (step == 1) {
                                const float T = p->lambda3D * sig[ch] * (p->T_3D == OC_HADAMARD ? sqrtf((float)nsx) : 1.0f);
                                l = ((q == 0 && n == 0) || fabsf(v[n]) > T) ? 1.0 : 0.0;
                                wt[ch] += (float)l;
                            } else if (p->T_3D == OC_HADAMARD) {
                                float value = v[n] * v[n] * coefn;
                                value /= (value + sig[ch] * sig[ch]);
                                l = (double)value * (double)coefn;
                                wt[ch] += value * value;
                            } else {
                                float value = v[n] * v[n];
                                value /= (value + sig[ch] * sig[ch]);
                                l = value;
                                wt[ch] += value * value;
                            }
                            lam[(ch * k2 + q) * nsx + n] = l;
                        }
                    }
                for (unsigned ch = 0; ch < C; ch++) {
                    if (step == 2 && p->T_3D == OC_HADAMARD)
                        ro[jr].w[ch] = wt[ch] > 0.0f ? 1.0f / (float)(sig[ch] * sig[ch] * wt[ch]) : 1.0f;
                    else
                        ro[jr].w[ch] = 1.f / (float)(sig[ch] * sig[ch] * wt[ch]);
                }
                /* the linear map on x, in double */
                double *gx = (double *)malloc(sizeof(double) * C * k2 * nsx);
                double blk[256], tr2[256];
                for (unsigned ch = 0; ch < C; ch++)
                    for (unsigned n = 0; n < nsx; n++) {
                        unsigned px, py, pt;
                        oc_coords(&c, ro[jr].idx[n], &px, &py, &pt);
                        for (unsigned pp = 0; pp < k; pp++)
                            for (unsigned q = 0; q < k; q++) blk[pp * k + q] = x[oc_index(&c, px + q, py + pp, pt, ch)];
                        od_2d(blk, tr2, k, p->T_2D, 0);
                        for (unsigned q = 0; q < k2; q++) gx[(ch * k2 + q) * nsx + n] = tr2[q];
                    }
                for (unsigned v = 0; v < C * k2; v++) {
                    double *xv = gx + v * nsx;
                    const double *lv = lam + v * nsx;
                    if (p->T_3D == OC_HADAMARD) {
                        od_hadamard(xv, nsx);
                        for (unsigned n = 0; n < nsx; n++) xv[n] *= lv[n];
                        od_hadamard(xv, nsx);
                        if (step == 1)
                            for (unsigned n = 0; n < nsx; n++) xv[n] *= (double)coefn;
                    } else {
                        od_haar(xv, nsx, 0);
                        for (unsigned n = 0; n < nsx; n++) xv[n] *= lv[n];
                        od_haar(xv, nsx, 1);
                    }
                }
                double *e = est + (size_t)jr * per_ref;
                for (unsigned ch = 0; ch < C; ch++)
                    for (unsigned n = 0; n < nsx; n++) {
                        for (unsigned q = 0; q < k2; q++) blk[q] = gx[(ch * k2 + q) * nsx + n];
                        od_2d(blk, tr2, k, p->T_2D, 1);
                        for (unsigned q = 0; q < k2; q++) e[(size_t)ch * nsx * k2 + (size_t)n * k2 + q] = tr2[q];
                    }
                free(g);
                free(lam);
                free(gx);
            }
            for (unsigned jr = 0; jr < nc; jr++) {
                const unsigned nsx = ro[jr].nsx;
                const double *e = est + (size_t)jr * per_ref;
                for (unsigned ch = 0; ch < C; ch++)
                    for (unsigned n = 0; n < nsx; n++) {
                        unsigned px, py, pt;
                        oc_coords(&c, ro[jr].idx[n], &px, &py, &pt);
                        for (unsigned pp = 0; pp < k; pp++)
                            for (unsigned q = 0; q < k; q++) {
                                const size_t o = oc_index(&c, px + q, py + pp, pt, ch);
                                const double kw = (double)(kai[pp * k + q] * ro[jr].w[ch]);
                                num[o] += kw * e[(size_t)ch * nsx * k2 + (size_t)n * k2 + pp * k + q];
                                den[o] += kw;
                            }
                    }
            }
        }
    for (size_t i = 0; i < total; i++) out[i] = den[i] == 0 ? (step == 1 ? (double)x[i] : 0.0) : num[i] / den[i];
    free(num);
    free(den);
    free(est);
    free(ro);
    free(rows);
    free(cols);
    return 0;
}

