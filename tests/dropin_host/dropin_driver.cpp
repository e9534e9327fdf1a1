// Test driver of the drop-in shim: a C++ caller of the reference's API
// (run_vbm3d, vbm3d_1st_step, vbm3d_2nd_step of src/vbm3d.h) linked against
// vbm3d_gb300/dropin/vbm3d_dropin.cpp and the GPU library, as a reference
// program would be.  TEST INFRASTRUCTURE.
//
//   dropin_driver run|step1|step2 <input> <output>
//
// <input>: int32 W, H, F, C, fflow's width, height, frames, channels,
// bflow's likewise, color_space; float32 sigma; the noisy video (W*H*F*C),
// for step2 the basic estimate (W*H*F*C), then fflow and bflow (0 frames =
// an empty Video, i.e. zero flow).  Parameters: the reference defaults for sigma.
// <output>: run: basic then denoised; step1 / step2: numerator then
// denominator.  The exit status is run_vbm3d's (EXIT_FAILURE on a size
// mismatch); the steps exit 0.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "vbm3d.h"
#include "vbm3d_gb300.h"

static Parameters defaults(int step, float sigma)
{
    vbm3d_params c;
    if (vbm3d_default_params(step, sigma, &c) != VBM3D_OK) std::exit(3);
    Parameters p;
    p.k = c.k; p.kt = c.kt; p.p = c.p; p.N = c.N; p.tau = c.tau; p.d = c.d;
    p.Nf = c.Nf; p.Ns = c.Ns; p.Npr = c.Npr; p.Nb = c.Nb; p.T_2D = c.T_2D; p.T_3D = c.T_3D;
    p.lambda3D = c.lambda3D; p.mc = c.mc != 0; p.n = c.n;
    return p;
}

static void read_video(FILE* f, Video<float>& v, unsigned w, unsigned h, unsigned fr, unsigned c)
{
    if (fr == 0) return;  // an empty Video
    v.resize(w, h, fr, c);
    if (std::fread(v.data.data(), sizeof(float), v.sz.whcf, f) != v.sz.whcf) std::exit(4);
}

int main(int argc, char** argv)
{
    if (argc != 4) return 2;
    FILE* f = std::fopen(argv[2], "rb");
    if (!f) return 2;
    int hdr[13];
    float sigma;
    if (std::fread(hdr, sizeof(int), 13, f) != 13 || std::fread(&sigma, sizeof(float), 1, f) != 1) return 4;
    const unsigned W = hdr[0], H = hdr[1], F = hdr[2], C = hdr[3];
    const bool color_space = hdr[12] != 0;
    Video<float> noisy, basic, fflow, bflow, out1, out2;
    read_video(f, noisy, W, H, F, C);
    if (!std::strcmp(argv[1], "step2")) read_video(f, basic, W, H, F, C);
    read_video(f, fflow, hdr[4], hdr[5], hdr[6], hdr[7]);
    read_video(f, bflow, hdr[8], hdr[9], hdr[10], hdr[11]);
    std::fclose(f);
    int rc = EXIT_SUCCESS;
    if (!std::strcmp(argv[1], "run")) {
        rc = run_vbm3d(sigma, noisy, fflow, bflow, out1, out2, defaults(1, sigma), defaults(2, sigma), color_space);
    } else if (!std::strcmp(argv[1], "step1")) {
        vbm3d_1st_step(sigma, noisy, fflow, bflow, defaults(1, sigma), NULL, NULL, NULL, NULL, NULL, color_space,
                       out1, out2);
    } else if (!std::strcmp(argv[1], "step2")) {
        vbm3d_2nd_step(sigma, noisy, basic, fflow, bflow, defaults(2, sigma), NULL, NULL, NULL, NULL, NULL,
                       color_space, out1, out2);
    } else {
        return 2;
    }
    FILE* o = std::fopen(argv[3], "wb");
    if (!o) return 2;
    std::fwrite(out1.data.data(), sizeof(float), out1.data.size(), o);
    std::fwrite(out2.data.data(), sizeof(float), out2.data.size(), o);
    std::fclose(o);
    return rc;
}
