/*
 * vbm3d_gb300 — C ABI of the GB300 (sm_103a) VBM3D denoiser.
 *
 * This is the drop-in boundary for the two denoising passes of tehret/vbm3d.
 * Every entry point replaces one reference function; the replaced interface
 * is cited beside each declaration (paths are relative to the reference
 * project root).  Plain pointers and sizes only; no C++ or torch types.
 *
 * Video layout (identical to the reference's VideoSize::index,
 * src/Utilities/LibVideoT.hpp:88-92): float32, planar per frame,
 *     index(x, y, t, c) = t*W*H*C + c*W*H + y*W + x.
 * Flows use the same layout with C = 2 (x displacement, then y):
 *     fflow frame t holds the motion t -> t+1, bflow frame t-1 holds the
 *     motion t -> t-1 (src/main.cpp:353-369, src/vbm3d.cpp:1129-1130,1153-1154).
 * A NULL flow pointer means an all-zero flow, which is what the reference's
 * CLI builds when no flow file is given (src/main.cpp:353-369).
 *
 * Pointer arguments of the vbm3d_gpu_* functions are DEVICE pointers on the
 * current CUDA device; `stream` is a cudaStream_t (NULL = legacy default
 * stream).  All calls are stream-ordered and return before the GPU work ends,
 * except where noted.  vbm3d_run_host takes HOST pointers and synchronises.
 *
 * Return value: VBM3D_OK (0) or a vbm3d_status code; vbm3d_last_error()
 * gives a message for the calling thread's last failure.  The reference's
 * steps return void and silently return on a bad colour space
 * (src/vbm3d.cpp:467-468); here that case is VBM3D_ERR_COLOR_SPACE.
 */
#ifndef VBM3D_GB300_H
#define VBM3D_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* 2D transform codes, src/vbm3d.cpp:34-35. */
#define VBM3D_DCT 0u
#define VBM3D_BIOR 1u
/* 1D transform codes, src/vbm3d.cpp:36-37.  Only T_3D == VBM3D_HADAMARD
 * selects the Walsh-Hadamard path; every other value selects Haar
 * (src/vbm3d.cpp:579-584, :828-833). */
#define VBM3D_HADAMARD 2u
#define VBM3D_HAAR 4u

typedef enum vbm3d_status {
    VBM3D_OK = 0,
    VBM3D_ERR_INVALID_ARGUMENT = 1, /* NULL pointer, zero size, bad parameter */
    VBM3D_ERR_UNSUPPORTED = 2,      /* valid for the reference, outside this build's limits */
    VBM3D_ERR_CUDA = 3,             /* a CUDA runtime call failed */
    VBM3D_ERR_OUT_OF_MEMORY = 4,
    VBM3D_ERR_COLOR_SPACE = 5,      /* estimate_sigma rejected the channel count */
    VBM3D_ERR_SIZE_MISMATCH = 6     /* flows / videos of different sizes, src/main.cpp:372-376 */
} vbm3d_status;

/* Mirror of `struct Parameters`, src/parameters.h:21-58, field for field.
 * `mc` is the reference's bool; `n` is the tile border it uses only for
 * OpenMP tiling (src/vbm3d.cpp:474-489), ignored on the GPU. */
typedef struct vbm3d_params {
    unsigned k;       /* spatial patch size */
    unsigned kt;      /* temporal patch size */
    unsigned p;       /* step between reference patches */
    unsigned N;       /* maximum number of similar patches */
    float tau;        /* distance threshold */
    float d;          /* bias toward the reference position */
    unsigned Nf;      /* frames searched forward and backward */
    unsigned Ns;      /* search window in the reference frame */
    unsigned Npr;     /* search window in the other frames */
    unsigned Nb;      /* matches kept per frame */
    unsigned T_2D;    /* VBM3D_DCT or VBM3D_BIOR */
    unsigned T_3D;    /* VBM3D_HADAMARD or anything else (Haar) */
    float lambda3D;   /* hard threshold factor (step 1) */
    int mc;           /* motion-compensated 3D patches */
    int n;            /* tiling border (CPU-only) */
} vbm3d_params;

typedef struct vbm3d_dims {
    unsigned width, height, frames, channels;
} vbm3d_dims;

/* Limits of this build (a call outside them returns VBM3D_ERR_UNSUPPORTED):
 * channels in {1, 3}; k <= 16; kt <= 4; N <= 32; Nb <= 8; Ns, Npr <= 15;
 * Nf <= 16; W * H * F * C < 2^32 (32-bit patch indices, as the reference). */

/* Default parameters of the reference CLI for step 1 (hard threshold) or
 * step 2 (Wiener) at noise level sigma, i.e. initializeParameters_1 /
 * initializeParameters_2 with every option left at its default
 * (src/main.cpp:35-125, :127-207).  `step` is 1 or 2. */
int vbm3d_default_params(int step, float sigma, vbm3d_params *out);

/* Per-channel noise levels used by both steps: estimate_sigma
 * (src/Utilities/Utilities.cpp:282-333) called with the bool color_space
 * read as an integer, exactly as src/vbm3d.cpp:467 and :697 do. */
int vbm3d_sigma_table(float sigma, unsigned channels, int color_space, float *sigma_table);

/* Step 1 (hard thresholding) into numerator / denominator.
 * Replaces vbm3d_1st_step (src/vbm3d.h:38-52, src/vbm3d.cpp:447-654) with
 * crop == NULL; the FFTW plans have no counterpart.  numerator and
 * denominator (W*H*F*C floats each) are overwritten, as the reference
 * resizes and zeroes them (src/vbm3d.cpp:509-515). */
int vbm3d_gpu_step1(const vbm3d_params *prms, const float *noisy,
                    const float *fflow, const float *bflow, vbm3d_dims dims,
                    float sigma, int color_space,
                    float *numerator, float *denominator, void *stream);

/* Step 2 (Wiener) into numerator / denominator.
 * Replaces vbm3d_2nd_step (src/vbm3d.h:54-70, src/vbm3d.cpp:676-928) with
 * crop == NULL.  Block matching runs on `basic`. */
int vbm3d_gpu_step2(const vbm3d_params *prms, const float *noisy, const float *basic,
                    const float *fflow, const float *bflow, vbm3d_dims dims,
                    float sigma, int color_space,
                    float *numerator, float *denominator, void *stream);

/* Step 1 without any device allocation.  No counterpart in the reference:
 * it is vbm3d_gpu_step1 for callers that cannot let a library allocate
 * device memory (plug-in hosts that own all device memory through their own
 * allocator, real-time pipelines that forbid allocation once running,
 * processes under a fixed memory budget).  The block-matching table that
 * vbm3d_gpu_step1 allocates lives instead in a fixed 32 MiB device array
 * that every GPU using this library holds until the process exits; a call
 * needs (reference patches) * (N + 1) 4-byte words of it and returns
 * VBM3D_ERR_UNSUPPORTED when that exceeds 8 Mi words (for 1080p RGB with
 * the default step-1 parameters: at most 16 frames per call).  The driver
 * reserves the 32 MiB when it loads the library's module: at context
 * creation under CUDA_MODULE_LOADING=EAGER, at the first call of this
 * entry point under lazy loading (the default); a caller with a strict
 * memory budget makes one call at start-up.  The first call in a device
 * context looks up the array's device address (again after a device reset,
 * which reloads the module); make that first call before any stream
 * capture.  All calls share the one array, so calls whose GPU work
 * overlaps (different streams, or different host threads on one device)
 * race: serialise them.  Same arguments and results as vbm3d_gpu_step1. */
int vbm3d_gpu_step1_noalloc(const vbm3d_params *prms, const float *noisy,
                            const float *fflow, const float *bflow, vbm3d_dims dims,
                            float sigma, int color_space,
                            float *numerator, float *denominator, void *stream);

/* Aggregation mode of the plain path, process-wide (no counterpart in the
 * reference, whose single-thread run_vbm3d is deterministic by
 * construction).  Off (0, the default): groups add into numerator /
 * denominator with float atomics, so the order of the additions, and the
 * last bits of the sums, vary from run to run.  On (1): the filter keeps
 * every group's weighted estimates and one ordered pass sums them, at
 * every pixel, in the reference's order (reference patches in grid order,
 * then group members, src/vbm3d.cpp:612-650, :860-924): runs are
 * bit-reproducible and, where the per-group estimates are the reference's
 * own bits (the bior1.5 / Haar hard-threshold step), the step's numerator
 * and denominator are the reference's to the bit.  Applies to
 * vbm3d_gpu_step1 / _step2 / _run / _run_host / vbm3d_step_host (k in
 * {7, 8}, kt == 1, N <= 8, else VBM3D_ERR_UNSUPPORTED while it is on);
 * not to vbm3d_gpu_step1_noalloc, the batched form or the linearised form,
 * which always add with atomics.  Costs device memory for the estimates:
 * (reference patches) * C * N * k^2 floats per step (32 GB for step 2 of a
 * 1920x1080x30 RGB clip), and about 1.15x the time of the atomic path. */
int vbm3d_set_deterministic(int on);
int vbm3d_get_deterministic(void);

/* out[i] = denominator[i] == 0 ? fallback[i] : numerator[i] / denominator[i]
 * over `count` floats: the division in run_vbm3d (src/vbm3d.cpp:168-170,
 * :198-202).  `out` may alias `numerator`. */
int vbm3d_gpu_normalize(const float *numerator, const float *denominator,
                        const float *fallback, float *out, size_t count, void *stream);

/* In-place RGB -> YUV (forward != 0) or YUV -> RGB colour transform of a
 * 3-channel video: VideoUtils::transformColorSpace
 * (src/Utilities/LibVideoT.hpp:763-888).  One-channel videos are left as
 * they are, as in the reference. */
int vbm3d_gpu_color_transform(float *video, vbm3d_dims dims, int forward, void *stream);

/* Both passes with run_vbm3d's single-thread semantics
 * (src/vbm3d.h:25-35, src/vbm3d.cpp:87-211, :356-376): optional colour
 * transform of `noisy` (in place, and back at the end), step 1, division
 * with fallback to noisy, step 2, division with fallback to basic.  A step
 * whose k is 0 is skipped as in the reference; with prms_1->k == 0 `basic`
 * is an input.  Device pointers; `noisy`, `basic` and `denoised` hold
 * W*H*F*C floats. */
int vbm3d_gpu_run(float sigma, float *noisy, const float *fflow, const float *bflow,
                  float *basic, float *denoised,
                  const vbm3d_params *prms_1, const vbm3d_params *prms_2,
                  int color_space, vbm3d_dims dims, void *stream);

/* vbm3d_gpu_run on HOST buffers: copies noisy (and flows, when not NULL) to
 * the device, runs both passes, copies basic and denoised back, and waits.
 * `noisy` is not modified (the reference converts its copy back to RGB).
 * This is the call a CPU program that used run_vbm3d makes.  Host flows
 * need only F - 1 frames (the frames the reference's flow files hold,
 * src/main.cpp:360, :369): the steps never read the last one, and only the
 * first F - 1 are copied. */
int vbm3d_run_host(float sigma, const float *noisy, const float *fflow, const float *bflow,
                   float *basic, float *denoised,
                   const vbm3d_params *prms_1, const vbm3d_params *prms_2,
                   int color_space, vbm3d_dims dims);

/* One step on HOST buffers (copies in, runs vbm3d_gpu_step1 or _step2,
 * copies numerator and denominator out, waits): the call a CPU caller of
 * vbm3d_1st_step / vbm3d_2nd_step (src/vbm3d.h:38-70) makes.  `step` is 1
 * or 2; `basic` is read for step 2 only.  Host flows need only F - 1
 * frames, as for vbm3d_run_host. */
int vbm3d_step_host(int step, const vbm3d_params *prms, const float *noisy, const float *basic,
                    const float *fflow, const float *bflow, vbm3d_dims dims,
                    float sigma, int color_space, float *numerator, float *denominator);

/* Block matching alone, for every reference patch of the step's grid:
 * computeSimilarPatches (src/vbm3d.cpp:1082-1197) on `video`, with the
 * reference grid of ind_initialize (src/Utilities/Utilities.cpp:400-415,
 * src/vbm3d.cpp:471-489).  For reference r (frames outer, rows, then
 * columns, as the loops at src/vbm3d.cpp:527-538 visit them):
 *   indexes[r*N + i], distances[r*N + i] for i < nsimp[r]: the sorted
 *   matches (patch index = index(x, y, t, 0)); nsx[r]: the returned group
 *   size (largest power of 2 <= matches under tau).
 * Any of the three outputs may be NULL.  Returns the number of references
 * in *n_refs when n_refs is not NULL (call with all outputs NULL to size). */
int vbm3d_gpu_similar_patches(const vbm3d_params *prms, const float *video,
                              const float *fflow, const float *bflow, vbm3d_dims dims,
                              unsigned *indexes, float *distances,
                              unsigned *nsimp, unsigned *nsx,
                              size_t *n_refs, void *stream);

/* Frozen linearisation of one step and its adjoint (no reference
 * counterpart; the differentiation form of the filter).  With the
 * block-matching groups, the hard-threshold masks (step 1) or Wiener gains
 * (step 2) and the aggregation weights frozen at their forward-pass values,
 * a step's output is a linear map L of its noisy input; applied to the
 * noisy input itself it is the forward step.
 *   vbm3d_linear_create: runs the step's block matching and forward filter
 *     on (noisy, basic) and keeps the groups and the denominator; `noisy`
 *     (and `basic` for step 2) must stay valid until vbm3d_linear_destroy.
 *   vbm3d_linear_apply: out = L x (adjoint == 0) or out = L^T x.
 * Limits: k in {7, 8}, kt == 1, N <= 8.  Device pointers, stream-ordered;
 * create allocates the state with cudaMalloc. */
typedef struct vbm3d_linear vbm3d_linear;
int vbm3d_linear_create(int step, const vbm3d_params *prms, const float *noisy, const float *basic,
                        const float *fflow, const float *bflow, vbm3d_dims dims, float sigma,
                        int color_space, vbm3d_linear **state, void *stream);
int vbm3d_linear_apply(vbm3d_linear *state, const float *x, float *out, int adjoint, void *stream);
int vbm3d_linear_den(vbm3d_linear *state, const float **denominator);
void vbm3d_linear_destroy(vbm3d_linear *state);

/* Batched form, no reference counterpart (the reference denoises one clip
 * per process run, src/main.cpp): many clips of uneven size, channel count
 * and noise level denoised by one CUDA graph launch, each with
 * vbm3d_gpu_run's semantics.  Unlike vbm3d_gpu_run, `noisy` is not
 * modified; the outputs are written in RGB when colour_space is set.
 *   vbm3d_batch_create: validates every clip, allocates the working buffers
 *     (one cudaMalloc arena), builds the work queues, autotunes the phases
 *     whose configuration is not given (one eager pass over the batch, on
 *     the clips' current inputs), and captures the CUDA graph.  Synchronises
 *     `stream` first, and the device before it returns.  The clips' device
 *     pointers are baked into the graph: they must stay valid, and hold the
 *     new inputs, for every vbm3d_batch_run.
 *   vbm3d_batch_run: one graph launch on `stream` (stream-ordered).  Runs of
 *     one batch share its working buffers: serialise them.
 * Limits: both steps run (k > 0), k in {7, 8}, kt == 1, N <= 8, and the
 * staged block-matching layout of the search windows fits 24 KB (true of
 * the reference defaults for every sigma); other clips are rejected with
 * VBM3D_ERR_UNSUPPORTED and run through vbm3d_gpu_run. */
typedef struct vbm3d_clip {
    vbm3d_dims dims;
    float sigma;
    const vbm3d_params *prms_1;  /* NULL: the reference defaults for sigma */
    const vbm3d_params *prms_2;
    const float *noisy;          /* device, W*H*F*C floats, read only */
    const float *fflow;          /* device or NULL (zero flow) */
    const float *bflow;
    float *basic;                /* device output or NULL */
    float *denoised;             /* device output */
} vbm3d_clip;

/* Per phase (block matching / filtering of each step): reference patches
 * per work item and warps per block; 0 and 0 = autotune, which picks per
 * work launch (class of clips) and reports, from vbm3d_batch_get_config,
 * the choice of each phase's largest launch.  Block matching of
 * one-channel clips runs two reference patches per warp, and its items hold
 * twice the tile, so every warp has the same work.  no_graph = 1
 * enqueues the kernels at each run instead of launching the graph.  The
 * last three fields are outputs of vbm3d_batch_get_config. */
typedef struct vbm3d_batch_config {
    int bm1_tile, bm1_warps;
    int filter1_tile, filter1_warps;
    int bm2_tile, bm2_warps;
    int filter2_tile, filter2_warps;
    int no_graph;
    float tune_ms;               /* time spent in vbm3d_batch_create's tuning pass */
    unsigned work_items;         /* items of the four work phases */
    size_t device_bytes;         /* working arena */
} vbm3d_batch_config;

/* One work launch of a batch, as measured by vbm3d_batch_profile. */
typedef struct vbm3d_batch_launch {
    int phase;                   /* 0 / 2: block matching of step 1 / 2; 1 / 3: filtering */
    int k, channels;             /* the launch's class (channels 0: any, for filtering) */
    int clips;                   /* clips in the launch */
    unsigned items;              /* work items */
    unsigned long long refs;     /* reference patches */
    int tile, warps, grid;       /* refs per item, warps per block, blocks */
    float ms;                    /* CUDA-event duration */
} vbm3d_batch_launch;

typedef struct vbm3d_batch vbm3d_batch;
int vbm3d_batch_create(const vbm3d_clip *clips, int nclips, int color_space,
                       const vbm3d_batch_config *config, vbm3d_batch **batch, void *stream);
int vbm3d_batch_run(vbm3d_batch *batch, void *stream);
int vbm3d_batch_get_config(const vbm3d_batch *batch, vbm3d_batch_config *config);
/* One run of the batch with its kernels enqueued one by one and a CUDA
 * event around every work launch (same results as vbm3d_batch_run); fills
 * out[0 .. *count) in launch order and synchronises `stream`.  Fails with
 * VBM3D_ERR_INVALID_ARGUMENT, *count set, when cap < *count. */
int vbm3d_batch_profile(vbm3d_batch *batch, void *stream, vbm3d_batch_launch *out, int cap, int *count);
void vbm3d_batch_destroy(vbm3d_batch *batch);

/* TV-L1 optical flow: the flows the block matching's predictive search
 * reads, which the reference computes on the CPU with tvl1flow
 * (Dual_TVL1_optic_flow_multiscale, tvl1flow/tvl1flow_lib.c:356-488, after
 * image_normalization, with the scale count of tvl1flow/main.c:151-157).
 * Options mirror tvl1flow's command line (tvl1flow/main.c:84-96). */
typedef struct vbm3d_tvl1_params {
    float tau;       /* time step, (0, 0.25] */
    float lambda;    /* data-term weight */
    float theta;     /* tightness */
    int nscales;     /* maximum number of scales */
    int fscale;      /* finest scale computed (finer ones are upsampled) */
    float zfactor;   /* pyramid factor, (0, 1) */
    int nwarps;      /* warpings per scale */
    float epsilon;   /* stopping threshold */
} vbm3d_tvl1_params;

/* The options the reference's flow scripts pass (tvl1flow/tvl1flow_forward.sh,
 * tvl1flow_backward.sh: 0.25 0.2 0.3 100 2 0.5 5 0.01). */
int vbm3d_tvl1_default_params(vbm3d_tvl1_params *params);

/* Scales used for a width x height image (tvl1flow/main.c:151-157). */
int vbm3d_tvl1_scales(unsigned width, unsigned height, const vbm3d_tvl1_params *params,
                      int *nscales, int *fscale);

/* Flows of `npairs` frame pairs: I0 and I1 hold npairs one-channel frames
 * each ([npairs][H][W], device), flow receives [npairs][2][H][W] (x then y
 * component, the motion from I0 to I1).  iterations: NULL, or HOST
 * int[npairs][nscales][nwarps] for the iteration count of every warping (-1
 * for scales below fscale).  Synchronises `stream`. */
int vbm3d_gpu_tvl1_pairs(const float *I0, const float *I1, unsigned npairs, unsigned width,
                         unsigned height, const vbm3d_tvl1_params *params, float *flow,
                         int *iterations, void *stream);

/* Forward and backward flows of a one-channel video ([F][H][W], device) in
 * the layout the steps read (see the top of this file): fflow[t] = flow of
 * frame t -> t+1, bflow[t] = flow of frame t+1 -> t, the last frame's
 * entries zero; what tvl1flow_forward.sh / tvl1flow_backward.sh compute frame
 * pair by frame pair.  All 2 (F - 1) pairs run together.  Synchronises
 * `stream`. */
int vbm3d_gpu_tvl1_video(const float *video, unsigned width, unsigned height, unsigned frames,
                         const vbm3d_tvl1_params *params, float *fflow, float *bflow, void *stream);

/* Multiscaler DCT pyramid: the pre- and post-processing of the reference's
 * multiscale denoising (src/utils/VBM3Ddenoising_multiscale.sh), which
 * decomposes every frame into DCT levels, denoises each level with VBM3D at
 * sigma / 2^level and recomposes the frame.  Replace the `decompose`,
 * `recompose` and `merge_coarse` programs with the DCT type (-t 0;
 * multiscaler/decompose.cpp, recompose.cpp, merge_coarse.cpp over
 * dct_inplace / idct_inplace, multiscaler/multiscaler.cpp:21-100).  Images
 * are `planes` planar float planes (frames x channels) of height x width
 * rows, device memory; level i is the previous level halved by integer
 * division (level 0 is the full size).  The transforms are FFTW's REDFT10 /
 * REDFT01 in float, so results match the reference to float rounding.
 * Asynchronous on `stream`.
 *
 * decompose: out[0 .. levels) receive the levels ([planes][h_i][w_i]). */
int vbm3d_gpu_ms_decompose(const float *in, unsigned width, unsigned height, unsigned planes,
                           unsigned levels, float *const *out, void *stream);

/* recompose: level_in[0 .. levels) hold the (denoised) levels, out the
 * full-size image: level 0's DCT with the block of rows < h_i * factor and
 * columns < w_i * factor (float product, as the reference's loop bound) of
 * every coarser level's DCT written over it, then the inverse DCT.
 * VBM3D_ERR_INVALID_ARGUMENT for factor > 1 (the reference would read past
 * the level). */
int vbm3d_gpu_ms_recompose(const float *const *level_in, unsigned width, unsigned height,
                           unsigned planes, unsigned levels, float factor, float *out, void *stream);

/* merge_coarse: the fine image's DCT with the coarse image's low-frequency
 * block (rows < cheight * factor, columns < cwidth * factor) written over
 * it, then the inverse DCT, into out (width x height planes). */
int vbm3d_gpu_ms_merge_coarse(const float *fine, const float *coarse, unsigned width,
                              unsigned height, unsigned cwidth, unsigned cheight, unsigned planes,
                              float factor, float *out, void *stream);

/* Measurement helper with no reference counterpart: runs the block
 * matching of vbm3d_gpu_similar_patches and returns in *count the total
 * number of patch distances it evaluated (calls of the reference's
 * patchDistance, src/vbm3d.cpp:1068).  Synchronises `stream`. */
int vbm3d_gpu_bm_distance_count(const vbm3d_params *prms, const float *video,
                                const float *fflow, const float *bflow, vbm3d_dims dims,
                                unsigned long long *count, void *stream);

/* Number of reference patches of one step's grid (rows x columns x frames). */
int vbm3d_ref_count(const vbm3d_params *prms, vbm3d_dims dims, size_t *n_refs);

const char *vbm3d_status_string(int status);
const char *vbm3d_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* VBM3D_GB300_H */
