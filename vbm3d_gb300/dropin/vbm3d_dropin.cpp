// Drop-in replacement of the reference's step entry points (tehret/vbm3d,
// src/vbm3d.h:25-70) that forwards to the GB300 library's C ABI.
//
// Build it inside the reference tree instead of src/vbm3d.cpp:
//     g++ -std=c++11 -O2 -I<vbm3d>/src -I<vbm3d>/src/Utilities
//         -I<this repo>/include -c vbm3d_dropin.cpp
// and link libvbm3d_gb300.so.  main.cpp, run_vbm3d's callers and the
// Video<float> / Parameters types stay unchanged.  FFTW plans are accepted
// and ignored (the GPU needs none).  Differences from the reference:
//  * crop must be NULL (the GPU processes the whole video; the OpenMP crop
//    tiling of run_vbm3d has no counterpart);
//  * errors (which the reference cannot report) are printed to stderr and
//    leave numerator / denominator zero, so run_vbm3d's division falls back
//    to its fallback video, like the reference's silent early return
//    (src/vbm3d.cpp:467-468);
//  * run_vbm3d leaves vid_noisy in RGB without the YUV round trip the
//    reference applies to it in place.
// Flows: an empty Video means zero flow.  A flow of the video's width and
// height holds either F frames (the zero flows main.cpp builds when no flow
// file is given, src/main.cpp:353-369) or F - 1 frames (what main.cpp loads
// from flow files: fflow of frames first..last-1, bflow of first+1..last,
// src/main.cpp:360, :369).  The steps never read a flow's frame F - 1
// (forward chains stop at the last frame, backward chains read bflow[t - 1]),
// and the host entry points copy only the first F - 1 frames, so both are
// passed as they are.  Any other size is the mismatch main.cpp rejects
// (src/main.cpp:372-376): VBM3D_ERR_SIZE_MISMATCH.
#include <cassert>
#include <cstdio>
#include <cstdlib>
#include <ctime>  // the reference headers use time() and assert() without including them

#include "vbm3d.h"
#include "vbm3d_gb300.h"

namespace {

vbm3d_params to_c(const Parameters& p)
{
    vbm3d_params o;
    o.k = p.k; o.kt = p.kt; o.p = p.p; o.N = p.N;
    o.tau = p.tau; o.d = p.d;
    o.Nf = p.Nf; o.Ns = p.Ns; o.Npr = p.Npr; o.Nb = p.Nb;
    o.T_2D = p.T_2D; o.T_3D = p.T_3D;
    o.lambda3D = p.lambda3D; o.mc = p.mc ? 1 : 0; o.n = p.n;
    return o;
}

vbm3d_dims dims_of(const Video<float>& v)
{
    vbm3d_dims d;
    d.width = v.sz.width; d.height = v.sz.height; d.frames = v.sz.frames; d.channels = v.sz.channels;
    return d;
}

// The flow the C ABI reads (its first F - 1 frames; NULL for zero flow) for
// flow f of video vid.  Returns VBM3D_OK or VBM3D_ERR_SIZE_MISMATCH.
int flow_arg(const Video<float>& f, const Video<float>& vid, const float** out)
{
    *out = NULL;
    if (f.sz.whcf == 0) return VBM3D_OK;
    if (f.sz.width != vid.sz.width || f.sz.height != vid.sz.height || f.sz.channels != 2)
        return VBM3D_ERR_SIZE_MISMATCH;
    if (f.sz.frames != vid.sz.frames && f.sz.frames + 1 != vid.sz.frames) return VBM3D_ERR_SIZE_MISMATCH;
    *out = f.data.data();
    return VBM3D_OK;
}

// Both flows of a call; prints the reason and returns the status on a
// mismatch.
int flow_args(const Video<float>& ff, const Video<float>& bf, const Video<float>& vid, const float** fp,
              const float** bp)
{
    int rc = flow_arg(ff, vid, fp);
    if (rc == VBM3D_OK) rc = flow_arg(bf, vid, bp);
    if (rc != VBM3D_OK)
        std::fprintf(stderr, "vbm3d_gb300: %s: flows of %ux%ux%u(x%u) / %ux%ux%u(x%u) for a %ux%ux%u video\n",
                     vbm3d_status_string(rc), ff.sz.width, ff.sz.height, ff.sz.frames, ff.sz.channels, bf.sz.width,
                     bf.sz.height, bf.sz.frames, bf.sz.channels, vid.sz.width, vid.sz.height, vid.sz.frames);
    return rc;
}

void step(int which, const float sigma, const Video<float>& noisy, const Video<float>* basic,
          const Video<float>& fflow, const Video<float>& bflow, const Parameters& prms,
          VideoUtils::CropPosition* crop, bool color_space, Video<float>& num, Video<float>& den)
{
    num.resize(noisy.sz);
    den.resize(noisy.sz);
    if (crop) {
        std::fprintf(stderr, "vbm3d_gb300: crop != NULL is not supported\n");
        return;
    }
    vbm3d_params p = to_c(prms);
    const float *fp = NULL, *bp = NULL;
    int rc = flow_args(fflow, bflow, noisy, &fp, &bp);
    if (rc == VBM3D_OK) {
        rc = vbm3d_step_host(which, &p, noisy.data.data(), basic ? basic->data.data() : NULL, fp, bp,
                             dims_of(noisy), sigma, color_space ? 1 : 0, num.data.data(), den.data.data());
        if (rc != VBM3D_OK) std::fprintf(stderr, "vbm3d_gb300: %s: %s\n", vbm3d_status_string(rc), vbm3d_last_error());
    }
    if (rc != VBM3D_OK)
        for (unsigned k = 0; k < num.sz.whcf; k++) num(k) = den(k) = 0.f;
}

}  // namespace

void vbm3d_1st_step(const float sigma, Video<float> const& vid_noisy, Video<float>& fflow, Video<float>& bflow,
                    const Parameters& prms, fftwf_plan*, fftwf_plan*, fftwf_plan*, fftwf_plan*,
                    VideoUtils::CropPosition* crop, const bool color_space, Video<float>& numerator,
                    Video<float>& denominator)
{
    step(1, sigma, vid_noisy, NULL, fflow, bflow, prms, crop, color_space, numerator, denominator);
}

void vbm3d_2nd_step(const float sigma, Video<float> const& vid_noisy, Video<float> const& vid_basic,
                    Video<float>& fflow, Video<float>& bflow, const Parameters& prms, fftwf_plan*, fftwf_plan*,
                    fftwf_plan*, fftwf_plan*, VideoUtils::CropPosition* crop, const bool color_space,
                    Video<float>& numerator, Video<float>& denominator)
{
    step(2, sigma, vid_noisy, &vid_basic, fflow, bflow, prms, crop, color_space, numerator, denominator);
}

int run_vbm3d(const float sigma, Video<float>& vid_noisy, Video<float>& fflow, Video<float>& bflow,
              Video<float>& vid_basic, Video<float>& vid_denoised, const Parameters& prms_1,
              const Parameters& prms_2, const bool color_space)
{
    if (vid_basic.sz != vid_noisy.sz) vid_basic.resize(vid_noisy.sz);
    if (vid_denoised.sz != vid_noisy.sz) vid_denoised.resize(vid_noisy.sz);
    vbm3d_params p1 = to_c(prms_1), p2 = to_c(prms_2);
    const float *fp = NULL, *bp = NULL;
    if (flow_args(fflow, bflow, vid_noisy, &fp, &bp) != VBM3D_OK) return EXIT_FAILURE;
    int rc = vbm3d_run_host(sigma, vid_noisy.data.data(), fp, bp, vid_basic.data.data(), vid_denoised.data.data(),
                            &p1, &p2, color_space ? 1 : 0, dims_of(vid_noisy));
    if (rc != VBM3D_OK) {
        std::fprintf(stderr, "vbm3d_gb300: %s: %s\n", vbm3d_status_string(rc), vbm3d_last_error());
        return EXIT_FAILURE;
    }
    return EXIT_SUCCESS;
}
