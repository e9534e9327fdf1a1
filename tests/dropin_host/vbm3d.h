// Test stand-in for the reference's src/vbm3d.h interface (tehret/vbm3d),
// so that the drop-in shim vbm3d_gb300/dropin/vbm3d_dropin.cpp builds and
// runs where the reference sources are absent.  TEST INFRASTRUCTURE.
//
// It declares only what the shim and its callers touch, with the
// reference's names and meanings:
//  * VideoSize / Video<float>: width, height, frames, channels, the derived
//    products and the planar index t*whc + c*wh + y*width + x
//    (src/Utilities/LibVideoT.hpp:40-121), a std::vector<float> `data`,
//    resize() and element access by linear index;
//  * Parameters: the fields of src/parameters.h:21-58;
//  * fftwf_plan and VideoUtils::CropPosition as opaque types (the shim
//    accepts plans and ignores them, and requires crop == NULL);
//  * the three entry points of src/vbm3d.h:25-70.
#ifndef VBM3D_DROPIN_HOST_H
#define VBM3D_DROPIN_HOST_H

#include <vector>

struct VideoSize {
    unsigned width, height, frames, channels;
    unsigned wh, whc, whcf, whf;
    VideoSize() : width(0), height(0), frames(0), channels(0) { update_fields(); }
    VideoSize(unsigned w, unsigned h, unsigned f, unsigned c) : width(w), height(h), frames(f), channels(c)
    {
        update_fields();
    }
    void update_fields()
    {
        wh = width * height;
        whc = wh * channels;
        whcf = whc * frames;
        whf = wh * frames;
    }
    bool operator==(const VideoSize& o) const
    {
        return width == o.width && height == o.height && frames == o.frames && channels == o.channels;
    }
    bool operator!=(const VideoSize& o) const { return !(*this == o); }
};

template <class T>
class Video {
   public:
    VideoSize sz;
    std::vector<T> data;
    void resize(const VideoSize& s)
    {
        sz = s;
        sz.update_fields();
        data.assign(sz.whcf, T(0));
    }
    void resize(unsigned w, unsigned h, unsigned f, unsigned c = 1) { resize(VideoSize(w, h, f, c)); }
    T& operator()(unsigned i) { return data[i]; }
    const T& operator()(unsigned i) const { return data[i]; }
};

struct Parameters {
    unsigned k, kt, p, N;
    float tau, d;
    unsigned Nf, Ns, Npr, Nb, T_2D, T_3D;
    float lambda3D = 0.;
    bool mc = false;
    int n = 16;
};

typedef struct fftwf_plan_opaque* fftwf_plan;

namespace VideoUtils {
struct CropPosition;
}

int run_vbm3d(const float sigma, Video<float>& vid_noisy, Video<float>& fflow, Video<float>& bflow,
              Video<float>& vid_basic, Video<float>& vid_denoised, const Parameters& prms_1,
              const Parameters& prms_2, const bool color_space);
void vbm3d_1st_step(const float sigma, Video<float> const& vid_noisy, Video<float>& fflow, Video<float>& bflow,
                    const Parameters& prms, fftwf_plan* plan_2d, fftwf_plan* plan_2d_inv, fftwf_plan* plan_1d,
                    fftwf_plan* plan_1d_inv, VideoUtils::CropPosition* crop, const bool color_space,
                    Video<float>& numerator, Video<float>& denominator);
void vbm3d_2nd_step(const float sigma, Video<float> const& vid_noisy, Video<float> const& vid_basic,
                    Video<float>& fflow, Video<float>& bflow, const Parameters& prms, fftwf_plan* plan_2d,
                    fftwf_plan* plan_2d_inv, fftwf_plan* plan_1d, fftwf_plan* plan_1d_inv,
                    VideoUtils::CropPosition* crop, const bool color_space, Video<float>& numerator,
                    Video<float>& denominator);

#endif
