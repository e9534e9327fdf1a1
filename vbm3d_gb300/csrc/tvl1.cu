// TV-L1 optical flow on the GPU: the flows VBM3D's predictive search reads
// (the reference computes them on the CPU with tvl1flow/, Zach-Pock-Bischof
// dual TV-L1, tvl1flow/tvl1flow_lib.c:96-488, called with the options of
// tvl1flow/tvl1flow_forward.sh and tvl1flow_backward.sh).
//
// Every launch covers all frame pairs of a call (the pair is the grid's z
// index), so one pyramid level of a whole clip is one kernel.  Per pixel the
// arithmetic is the reference's, operation by operation (float where it
// uses float, double in the Gaussian convolution and the bicubic cells;
// this file is compiled with --fmad=false).  The only difference is the
// order of the per-iteration error sum that decides when a warping stops
// (the reference's OpenMP reduction has no fixed order either): when it
// falls within rounding of epsilon^2, a pair may stop one iteration earlier
// or later than the reference.
//
// Iteration loop (one warping): kernel A = thresholding step, divergence
// of the dual field, primal update and the error sum; kernel B = forward
// gradient of the new flow and the dual projection.  Each pair decides
// whether it still iterates from its own error sum of the previous
// iteration (double-buffered on the device), so converged pairs stop while
// the others go on; the host reads the pairs' activity every 16 iterations
// and ends the warping when none is left or after 300 iterations.  Nothing
// waits on anything inside a kernel.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "../../include/vbm3d_gb300.h"

namespace vbm3d {
void set_last_error(int status, const char* msg);

namespace tvl1 {

constexpr int kMaxIterations = 300;    // tvl1flow/tvl1flow_lib.c:22
constexpr double kPresmoothSigma = 0.8; // :23
constexpr double kZoomSigma0 = 0.6;    // tvl1flow/zoom.c:17
constexpr int kMaxTaps = 32;           // Gaussian half-window (size) limit
constexpr int kCheckEvery = 16;        // iterations between activity reads

struct Taps {
    double b[kMaxTaps];
    int size;
};

// ------------------------------------------------------------ device ---

__device__ __forceinline__ int clamp_flag(int x, int n, bool& out)
{
    if (x < 0) {
        out = true;
        return 0;
    }
    if (x >= n) {
        out = true;
        return n - 1;
    }
    return x;
}

// Keys cubic (tvl1flow/bicubic_interpolation.c:118-127), double.
__device__ __forceinline__ double cubic(double v0, double v1, double v2, double v3, double x)
{
    return v1 + 0.5 * x * (v2 - v0 + x * (2.0 * v0 - 5.0 * v1 + 4.0 * v2 - v3 + x * (3.0 * (v1 - v2) + v3 - v0)));
}

// The 4x4 sample positions of bicubic_interpolation_at
// (bicubic_interpolation.c:153-237, Neumann boundary; the row above uses
// the x direction's sign, as the reference does).
struct Cell {
    int cols[4], rows[4];
    double fx, fy;
    bool out;
};

__device__ __forceinline__ Cell cell_at(float uu, float vv, int nx, int ny)
{
    Cell c;
    const int sx = (uu < 0) ? -1 : 1, sy = (vv < 0) ? -1 : 1;
    bool out = false;
    const int iu = (int)uu, iv = (int)vv;
    const int x = clamp_flag(iu, nx, out);
    const int y = clamp_flag(iv, ny, out);
    c.cols[0] = clamp_flag(iu - sx, nx, out);
    c.rows[0] = clamp_flag(iv - sx, ny, out);
    c.cols[2] = clamp_flag(iu + sx, nx, out);
    c.rows[2] = clamp_flag(iv + sy, ny, out);
    c.cols[3] = clamp_flag(iu + 2 * sx, nx, out);
    c.rows[3] = clamp_flag(iv + 2 * sy, ny, out);
    c.cols[1] = x;
    c.rows[1] = y;
    c.fx = (double)(uu - (float)x);
    c.fy = (double)(vv - (float)y);
    c.out = out;
    return c;
}

__device__ __forceinline__ float interp(const float* __restrict__ in, int nx, const Cell& c)
{
    double v[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const float* col = in + c.cols[k];
        v[k] = cubic((double)col[nx * c.rows[0]], (double)col[nx * c.rows[1]], (double)col[nx * c.rows[2]],
                     (double)col[nx * c.rows[3]], c.fy);
    }
    return (float)cubic(v[0], v[1], v[2], v[3], c.fx);
}

// Per-pair min and max of both frames (getminmax, tvl1flow_lib.c:296-312):
// block partials, then one block per pair.
__global__ void minmax_partial(const float* const* __restrict__ I0, const float* const* __restrict__ I1, int size,
                               float2* __restrict__ part)
{
    const int p = blockIdx.y;
    float mn = __int_as_float(0x7f800000), mx = -mn;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < size; i += gridDim.x * blockDim.x) {
        const float a = I0[p][i], b = I1[p][i];
        mn = fminf(mn, fminf(a, b));
        mx = fmaxf(mx, fmaxf(a, b));
    }
    __shared__ float smn[256], smx[256];
    smn[threadIdx.x] = mn;
    smx[threadIdx.x] = mx;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            smn[threadIdx.x] = fminf(smn[threadIdx.x], smn[threadIdx.x + o]);
            smx[threadIdx.x] = fmaxf(smx[threadIdx.x], smx[threadIdx.x + o]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) part[(size_t)p * gridDim.x + blockIdx.x] = make_float2(smn[0], smx[0]);
}

// image_normalization (tvl1flow_lib.c:317-348) of both frames of each pair.
__global__ void normalize(const float* const* __restrict__ I0, const float* const* __restrict__ I1,
                          const float2* __restrict__ part, int nparts, int size, float* __restrict__ o0,
                          float* __restrict__ o1)
{
    const int p = blockIdx.y;
    float mn = part[(size_t)p * nparts].x, mx = part[(size_t)p * nparts].y;
    for (int k = 1; k < nparts; k++) {
        mn = fminf(mn, part[(size_t)p * nparts + k].x);
        mx = fmaxf(mx, part[(size_t)p * nparts + k].y);
    }
    const float den = mx - mn;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < size; i += gridDim.x * blockDim.x) {
        const float a = I0[p][i], b = I1[p][i];
        o0[(size_t)p * size + i] = den > 0 ? (float)(255.0 * (double)(a - mn) / (double)den) : a;
        o1[(size_t)p * size + i] = den > 0 ? (float)(255.0 * (double)(b - mn) / (double)den) : b;
    }
}

// One pass of the separable Gaussian of mask.c (reflecting boundary, double
// sums): rows (dir 0) or columns (dir 1), out of place.  The reflection is
// the reference's: before the start index -x, past the end 2n - 1 - x.
__global__ void gauss_pass(const float* __restrict__ in, float* __restrict__ out, int nx, int ny, int dir,
                           const Taps T)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= nx || y >= ny) return;
    const size_t base = (size_t)blockIdx.z * nx * ny;
    const int n = dir ? ny : nx, pos = dir ? y : x;
    const int stride = dir ? nx : 1;
    const float* line = in + base + (dir ? (size_t)x : (size_t)y * nx);
    auto R = [&](int q) -> double {
        const int r = q < 0 ? -q : (q >= n ? 2 * n - 1 - q : q);
        return (double)line[(size_t)r * stride];
    };
    double sum = T.b[0] * R(pos);
    for (int j = 1; j < T.size; j++) sum += T.b[j] * (R(pos - j) + R(pos + j));
    out[base + (size_t)y * nx + x] = (float)sum;
}

// Bicubic resampling out(i1, j1) = in((float)j1 / fx, (float)i1 / fy), no
// border zeroing (zoom_out / zoom_in, zoom.c:43-113); `scale` multiplies the
// result when not 1 (the flow rescaling of tvl1flow_lib.c:447-451).
__global__ void resample(const float* __restrict__ in, int nx, int ny, float* __restrict__ out, int nxx, int nyy,
                         float fx, float fy, float scale)
{
    const int j1 = blockIdx.x * blockDim.x + threadIdx.x, i1 = blockIdx.y * blockDim.y + threadIdx.y;
    if (j1 >= nxx || i1 >= nyy) return;
    const Cell c = cell_at((float)j1 / fx, (float)i1 / fy, nx, ny);
    float g = interp(in + (size_t)blockIdx.z * nx * ny, nx, c);
    if (scale != 1.0f) g *= scale;
    out[(size_t)blockIdx.z * nxx * nyy + (size_t)i1 * nxx + j1] = g;
}

// centered_gradient (mask.c): one-sided at the borders, halved.
__global__ void centered_gradient(const float* __restrict__ in, float* __restrict__ dx, float* __restrict__ dy,
                                  int nx, int ny)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y;
    if (j >= nx || i >= ny) return;
    const size_t base = (size_t)blockIdx.z * nx * ny;
    const float* f = in + base;
    const int k = i * nx + j;
    const float xr = f[j < nx - 1 ? k + 1 : k], xl = f[j > 0 ? k - 1 : k];
    const float yd = f[i < ny - 1 ? k + nx : k], yu = f[i > 0 ? k - nx : k];
    dx[base + k] = (float)(0.5 * (double)(xr - xl));
    dy[base + k] = (float)(0.5 * (double)(yd - yu));
}

// The warping step (tvl1flow_lib.c:144-163): I1, I1x, I1y warped by the
// current flow (zero outside the image), and the constant part of rho.
__global__ void warp_step(const float* __restrict__ I0, const float* __restrict__ I1, const float* __restrict__ I1x,
                          const float* __restrict__ I1y, const float* __restrict__ u1, const float* __restrict__ u2,
                          float* __restrict__ wx, float* __restrict__ wy, float* __restrict__ rho_c, int nx, int ny)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y;
    if (j >= nx || i >= ny) return;
    const size_t base = (size_t)blockIdx.z * nx * ny, k = base + (size_t)i * nx + j;
    const float a = u1[k], b = u2[k];
    const Cell c = cell_at((float)(j + a), (float)(i + b), nx, ny);
    float w = 0.f, gx = 0.f, gy = 0.f;
    if (!c.out) {
        w = interp(I1 + base, nx, c);
        gx = interp(I1x + base, nx, c);
        gy = interp(I1y + base, nx, c);
    }
    wx[k] = gx;
    wy[k] = gy;
    rho_c[k] = w - gx * a - gy * b - I0[k];
}

// divergence of (v1, v2) at (i, j) with mask.c's border rules.
__device__ __forceinline__ float div_at(const float* __restrict__ v1, const float* __restrict__ v2, int i, int j,
                                        int nx, int ny)
{
    const int p = i * nx + j;
    const bool top = i == 0, bottom = i == ny - 1, left = j == 0, right = j == nx - 1;
    if (!top && !bottom && !left && !right) return (v1[p] - v1[p - 1]) + (v2[p] - v2[p - nx]);
    if (top && !left && !right) return v1[p] - v1[p - 1] + v2[p];
    if (bottom && !left && !right) return v1[p] - v1[p - 1] - v2[p - nx];
    if (left && !top && !bottom) return v1[p] + v2[p] - v2[p - nx];
    if (right && !top && !bottom) return -v1[p - 1] + v2[p] - v2[p - nx];
    if (top && left) return v1[p] + v2[p];
    if (top && right) return -v1[p - 1] + v2[p];
    if (bottom && left) return v1[p] - v2[p - nx];
    return -v1[p - 1] - v2[p - nx];  // bottom right
}

struct IterArgs {
    const float* wx;
    const float* wy;
    const float* rho_c;
    float* u1;
    float* u2;
    float* p11;
    float* p12;
    float* p21;
    float* p22;
    float* errsum;  // [pairs][2]
    int* active;    // [pairs]
    int* iters;     // [pairs]: iterations of the current warping
    int nx, ny;
    float l_t, theta, taut, eps2;
};

// Iteration n, first half: thresholding step TH, divergence of the dual
// field, primal update, error sum (tvl1flow_lib.c:166-241).
__global__ void __launch_bounds__(256) iter_primal(const IterArgs A, int n)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y;
    const int p = blockIdx.z, nx = A.nx, ny = A.ny;
    const int size = nx * ny;
    bool act = n == 1;
    if (!act) act = A.errsum[2 * p + ((n - 1) & 1)] / (float)size > A.eps2;
    const bool lead = blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0 && threadIdx.y == 0;
    if (lead) {
        A.active[p] = act ? 1 : 0;
        if (act) A.iters[p] = n;
    }
    if (!act) return;  // uniform over the block
    float e = 0.f;
    if (j < nx && i < ny) {
        const size_t base = (size_t)p * size, k = base + (size_t)i * nx + j;
        const float gx = A.wx[k], gy = A.wy[k];
        const float u1k = A.u1[k], u2k = A.u2[k];
        const float grad = gx * gx + gy * gy;
        const float rho = A.rho_c[k] + (gx * u1k + gy * u2k);
        float d1, d2;
        if (rho < -A.l_t * grad) {
            d1 = A.l_t * gx;
            d2 = A.l_t * gy;
        } else if (rho > A.l_t * grad) {
            d1 = -A.l_t * gx;
            d2 = -A.l_t * gy;
        } else if ((double)grad < 1E-10) {
            d1 = d2 = 0;
        } else {
            const float fi = -rho / grad;
            d1 = fi * gx;
            d2 = fi * gy;
        }
        const float v1 = u1k + d1, v2 = u2k + d2;
        const float dv1 = div_at(A.p11 + base, A.p12 + base, i, j, nx, ny);
        const float dv2 = div_at(A.p21 + base, A.p22 + base, i, j, nx, ny);
        const float a = v1 + A.theta * dv1, b = v2 + A.theta * dv2;
        A.u1[k] = a;
        A.u2[k] = b;
        e = (a - u1k) * (a - u1k) + (b - u2k) * (b - u2k);
    }
    // block sum, one atomic per block
    __shared__ float red[8];
    for (int o = 16; o > 0; o >>= 1) e += __shfl_xor_sync(kFull, e, o);
    const int t = threadIdx.y * blockDim.x + threadIdx.x;
    if ((t & 31) == 0) red[t >> 5] = e;
    __syncthreads();
    if (t == 0) {
        float s = 0.f;
        for (int w = 0; w < (int)(blockDim.x * blockDim.y) / 32; w++) s += red[w];
        atomicAdd(&A.errsum[2 * p + (n & 1)], s);
    }
}

// Iteration n, second half: forward gradient of the new flow and the dual
// projection (tvl1flow_lib.c:243-263); clears the error sum iteration n + 1
// adds into.
__global__ void __launch_bounds__(256) iter_dual(const IterArgs A, int n)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y;
    const int p = blockIdx.z, nx = A.nx, ny = A.ny;
    if (!A.active[p]) return;
    if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0 && threadIdx.y == 0)
        A.errsum[2 * p + ((n + 1) & 1)] = 0.f;
    if (j >= nx || i >= ny) return;
    const size_t base = (size_t)p * nx * ny, k = base + (size_t)i * nx + j;
    const float* u1 = A.u1 + base;
    const float* u2 = A.u2 + base;
    const int q = i * nx + j;
    float u1x = 0.f, u1y = 0.f, u2x = 0.f, u2y = 0.f;
    if (j < nx - 1) {
        u1x = u1[q + 1] - u1[q];
        u2x = u2[q + 1] - u2[q];
    }
    if (i < ny - 1) {
        u1y = u1[q + nx] - u1[q];
        u2y = u2[q + nx] - u2[q];
    }
    // hypot of floats in double: the squares and their sum are exact or
    // rounded once, the square root correctly rounded
    const float g1 = (float)sqrt((double)u1x * (double)u1x + (double)u1y * (double)u1y);
    const float g2 = (float)sqrt((double)u2x * (double)u2x + (double)u2y * (double)u2y);
    const float ng1 = (float)(1.0 + (double)(A.taut * g1));
    const float ng2 = (float)(1.0 + (double)(A.taut * g2));
    A.p11[k] = (A.p11[k] + A.taut * u1x) / ng1;
    A.p12[k] = (A.p12[k] + A.taut * u1y) / ng1;
    A.p21[k] = (A.p21[k] + A.taut * u2x) / ng2;
    A.p22[k] = (A.p22[k] + A.taut * u2y) / ng2;
}

// Scale-0 flows into the caller's [2][H][W] buffers (u, then v).
__global__ void write_flow(const float* __restrict__ u1, const float* __restrict__ u2, float* const* __restrict__ dst,
                           int size)
{
    const int p = blockIdx.y;
    float* d = dst[p];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < size; i += gridDim.x * blockDim.x) {
        d[i] = u1[(size_t)p * size + i];
        d[size + i] = u2[(size_t)p * size + i];
    }
}

// ------------------------------------------------------------- host ---

int fail(int status, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
int fail(int status, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    set_last_error(status, buf);
    return status;
}

#define TCK(call)                                                                                              \
    do {                                                                                                       \
        cudaError_t e_ = (call);                                                                               \
        if (e_ != cudaSuccess)                                                                                 \
            return fail(e_ == cudaErrorMemoryAllocation ? VBM3D_ERR_OUT_OF_MEMORY : VBM3D_ERR_CUDA, "%s: %s", \
                        #call, cudaGetErrorString(e_));                                                        \
    } while (0)

// Gaussian taps of mask.c (window 5 sigma, normalised), in double.
int gaussian_taps(double sigma, Taps& T)
{
    const double den = 2 * sigma * sigma;
    const int size = (int)(5 * sigma) + 1;
    if (size > kMaxTaps) return fail(VBM3D_ERR_UNSUPPORTED, "Gaussian sigma %g too large", sigma);
    T.size = size;
    for (int i = 0; i < size; i++) T.b[i] = 1 / (sigma * sqrt(2.0 * 3.1415926)) * exp(-i * i / den);
    double norm = 0;
    for (int i = 0; i < size; i++) norm += T.b[i];
    norm *= 2;
    norm -= T.b[0];
    for (int i = 0; i < size; i++) T.b[i] /= norm;
    return VBM3D_OK;
}

void zoom_size(int nx, int ny, int* nxx, int* nyy, float factor)
{
    *nxx = (int)((float)nx * factor + 0.5);
    *nyy = (int)((float)ny * factor + 0.5);
}

int check_params(const vbm3d_tvl1_params* p)
{
    if (!p) return fail(VBM3D_ERR_INVALID_ARGUMENT, "NULL TV-L1 parameters");
    // the reference CLI's checks (tvl1flow/main.c:95-136) reject, here
    if (!(p->tau > 0 && p->tau <= 0.25f) || !(p->lambda > 0) || !(p->theta > 0) || p->nscales <= 0 ||
        p->fscale < 0 || !(p->zfactor > 0 && p->zfactor < 1) || p->nwarps <= 0 || !(p->epsilon > 0))
        return fail(VBM3D_ERR_INVALID_ARGUMENT, "TV-L1 parameters out of range (tau in (0, 0.25], lambda, theta, "
                                                "epsilon > 0, nscales, nwarps > 0, fscale >= 0, zfactor in (0, 1))");
    return VBM3D_OK;
}

dim3 grid2(int nx, int ny, int pairs) { return dim3((nx + 31) / 32, (ny + 7) / 8, pairs); }

// The whole multiscale flow of `pairs` frame pairs (pointer tables on the
// device), into the flow pointer table.  iters (host, optional):
// [pairs][nscales][nwarps].
int run(const float* const* d_I0, const float* const* d_I1, float* const* d_flow, int pairs, int nx, int ny,
        const vbm3d_tvl1_params& prm, int* iters, cudaStream_t s)
{
    int fscale = 0;
    const int nscales = [&] {
        int ns = prm.nscales;
        const float N = 1 + log(hypot(nx, ny) / 16.0) / log(1 / prm.zfactor);
        if (N < ns) ns = N;
        fscale = prm.fscale;
        if (ns < fscale) fscale = ns;
        return ns;
    }();
    if (nscales < 1) return fail(VBM3D_ERR_UNSUPPORTED, "image %dx%d too small for TV-L1", nx, ny);
    std::vector<int> nxs(nscales), nys(nscales);
    nxs[0] = nx;
    nys[0] = ny;
    for (int k = 1; k < nscales; k++) zoom_size(nxs[k - 1], nys[k - 1], &nxs[k], &nys[k], prm.zfactor);
    Taps pre, zoom;
    int rc = gaussian_taps(kPresmoothSigma, pre);
    if (rc) return rc;
    const float zsig = kZoomSigma0 * sqrt(1.0 / (prm.zfactor * prm.zfactor) - 1.0);
    if ((rc = gaussian_taps(zsig, zoom))) return rc;
    // the reflecting Gaussian reads up to `size` pixels past each border
    if (pre.size >= nx || pre.size >= ny)
        return fail(VBM3D_ERR_UNSUPPORTED, "image %dx%d smaller than the pre-smoothing window", nx, ny);
    for (int k = 0; k + 1 < nscales; k++)
        if (zoom.size >= nxs[k] || zoom.size >= nys[k])
            return fail(VBM3D_ERR_UNSUPPORTED, "pyramid level %dx%d smaller than the zoom window", nxs[k], nys[k]);
    for (int k = 0; k < nscales; k++)
        if (nxs[k] < 2 || nys[k] < 2) return fail(VBM3D_ERR_UNSUPPORTED, "pyramid level below 2x2");

    // buffers: per level I0, I1, u1, u2; work buffers sized for the finest computed level
    const size_t P = pairs;
    std::vector<size_t> off(4 * nscales);
    size_t total = 0;
    auto take = [&](size_t n) {
        const size_t o = total;
        total += (n + 63) & ~size_t(63);
        return o;
    };
    for (int k = 0; k < nscales; k++)
        for (int b = 0; b < 4; b++) off[4 * k + b] = take(P * nxs[k] * nys[k]);
    const size_t wsz = P * nxs[fscale] * nys[fscale];
    const size_t o_tmp = take(2 * P * nx * ny);  // two full-size images: the smoothing passes of zoom_out
    size_t o_work[9];
    for (int b = 0; b < 9; b++) o_work[b] = take(wsz);
    const size_t o_err = take(2 * P), o_act = take(P), o_it = take(P);
    const int nparts = 64;
    const size_t o_part = take(2 * P * nparts);
    float* buf = nullptr;
    TCK(cudaMallocAsync(&buf, total * sizeof(float), s));
    auto L = [&](int k, int b) { return buf + off[4 * k + b]; };  // b: 0 I0, 1 I1, 2 u1, 3 u2
    float* tmp = buf + o_tmp;
    float *I1x = buf + o_work[0], *I1y = buf + o_work[1], *wx = buf + o_work[2], *wy = buf + o_work[3];
    float *rho = buf + o_work[4], *p11 = buf + o_work[5], *p12 = buf + o_work[6], *p21 = buf + o_work[7];
    float* p22 = buf + o_work[8];
    float* errsum = buf + o_err;
    int* active = reinterpret_cast<int*>(buf + o_act);
    int* itdev = reinterpret_cast<int*>(buf + o_it);
    float2* part = reinterpret_cast<float2*>(buf + o_part);
    int* h_act = nullptr;
    int result = VBM3D_OK;
    cudaError_t e = cudaMallocHost(&h_act, 2 * P * sizeof(int));
    if (e != cudaSuccess) {
        cudaFreeAsync(buf, s);
        return fail(VBM3D_ERR_OUT_OF_MEMORY, "cudaMallocHost: %s", cudaGetErrorString(e));
    }
    const dim3 blk(32, 8);
#define TRY(call)                                                                                            \
    do {                                                                                                     \
        e = (call);                                                                                          \
        if (e != cudaSuccess) {                                                                              \
            result = fail(e == cudaErrorMemoryAllocation ? VBM3D_ERR_OUT_OF_MEMORY : VBM3D_ERR_CUDA, "%s: %s", \
                          #call, cudaGetErrorString(e));                                                     \
            goto done;                                                                                       \
        }                                                                                                    \
    } while (0)
    {
        // level 0: normalisation and pre-smoothing of both frames
        minmax_partial<<<dim3(nparts, pairs), 256, 0, s>>>(d_I0, d_I1, nx * ny, part);
        normalize<<<dim3(64, pairs), 256, 0, s>>>(d_I0, d_I1, part, nparts, nx * ny, L(0, 0), L(0, 1));
        TRY(cudaGetLastError());
        for (int b = 0; b < 2; b++) {
            gauss_pass<<<grid2(nx, ny, pairs), blk, 0, s>>>(L(0, b), tmp, nx, ny, 0, pre);
            gauss_pass<<<grid2(nx, ny, pairs), blk, 0, s>>>(tmp, L(0, b), nx, ny, 1, pre);
        }
        TRY(cudaGetLastError());
        // pyramid (zoom_out: smoothing of a copy, bicubic resampling)
        for (int k = 1; k < nscales; k++)
            for (int b = 0; b < 2; b++) {
                const int px = nxs[k - 1], py = nys[k - 1];
                float* tmp2 = tmp + P * px * py;  // within the 2 P nx ny of tmp
                gauss_pass<<<grid2(px, py, pairs), blk, 0, s>>>(L(k - 1, b), tmp2, px, py, 0, zoom);
                gauss_pass<<<grid2(px, py, pairs), blk, 0, s>>>(tmp2, tmp, px, py, 1, zoom);
                resample<<<grid2(nxs[k], nys[k], pairs), blk, 0, s>>>(tmp, px, py, L(k, b), nxs[k], nys[k],
                                                                      prm.zfactor, prm.zfactor, 1.0f);
            }
        TRY(cudaGetLastError());
        TRY(cudaMemsetAsync(L(nscales - 1, 2), 0, P * nxs[nscales - 1] * nys[nscales - 1] * sizeof(float), s));
        TRY(cudaMemsetAsync(L(nscales - 1, 3), 0, P * nxs[nscales - 1] * nys[nscales - 1] * sizeof(float), s));
        if (iters)
            for (size_t q = 0; q < P * nscales * prm.nwarps; q++) iters[q] = -1;
        const float inv_z = (float)1.0 / prm.zfactor;
        for (int k = nscales - 1; k >= 0; k--) {
            const int cx = nxs[k], cy = nys[k];
            if (k >= fscale) {
                const size_t sz = P * cx * cy;
                centered_gradient<<<grid2(cx, cy, pairs), blk, 0, s>>>(L(k, 1), I1x, I1y, cx, cy);
                TRY(cudaMemsetAsync(p11, 0, sz * sizeof(float), s));
                TRY(cudaMemsetAsync(p12, 0, sz * sizeof(float), s));
                TRY(cudaMemsetAsync(p21, 0, sz * sizeof(float), s));
                TRY(cudaMemsetAsync(p22, 0, sz * sizeof(float), s));
                IterArgs A;
                A.wx = wx;
                A.wy = wy;
                A.rho_c = rho;
                A.u1 = L(k, 2);
                A.u2 = L(k, 3);
                A.p11 = p11;
                A.p12 = p12;
                A.p21 = p21;
                A.p22 = p22;
                A.errsum = errsum;
                A.active = active;
                A.iters = itdev;
                A.nx = cx;
                A.ny = cy;
                A.l_t = prm.lambda * prm.theta;
                A.theta = prm.theta;
                A.taut = prm.tau / prm.theta;
                A.eps2 = prm.epsilon * prm.epsilon;
                for (int w = 0; w < prm.nwarps; w++) {
                    warp_step<<<grid2(cx, cy, pairs), blk, 0, s>>>(L(k, 0), L(k, 1), I1x, I1y, L(k, 2), L(k, 3), wx,
                                                                  wy, rho, cx, cy);
                    TRY(cudaMemsetAsync(errsum, 0, 2 * P * sizeof(float), s));
                    TRY(cudaMemsetAsync(itdev, 0, P * sizeof(int), s));
                    for (int n = 1; n <= kMaxIterations; n++) {
                        iter_primal<<<grid2(cx, cy, pairs), blk, 0, s>>>(A, n);
                        iter_dual<<<grid2(cx, cy, pairs), blk, 0, s>>>(A, n);
                        if (n % kCheckEvery == 0 && n < kMaxIterations) {
                            TRY(cudaMemcpyAsync(h_act, active, P * sizeof(int), cudaMemcpyDeviceToHost, s));
                            TRY(cudaStreamSynchronize(s));
                            bool any = false;
                            for (size_t q = 0; q < P; q++) any = any || h_act[q];
                            if (!any) break;
                        }
                    }
                    TRY(cudaGetLastError());
                    if (iters) {
                        TRY(cudaMemcpyAsync(h_act + P, itdev, P * sizeof(int), cudaMemcpyDeviceToHost, s));
                        TRY(cudaStreamSynchronize(s));
                        for (size_t q = 0; q < P; q++) iters[(q * nscales + k) * prm.nwarps + w] = h_act[P + q];
                    }
                }
            }
            if (!k) break;
            for (int b = 2; b < 4; b++)
                resample<<<grid2(nxs[k - 1], nys[k - 1], pairs), blk, 0, s>>>(
                    L(k, b), cx, cy, L(k - 1, b), nxs[k - 1], nys[k - 1], (float)nxs[k - 1] / cx,
                    (float)nys[k - 1] / cy, inv_z);
            TRY(cudaGetLastError());
        }
        write_flow<<<dim3(64, pairs), 256, 0, s>>>(L(0, 2), L(0, 3), d_flow, nx * ny);
        TRY(cudaGetLastError());
        TRY(cudaStreamSynchronize(s));
    }
done:
#undef TRY
    cudaFreeAsync(buf, s);
    cudaStreamSynchronize(s);
    cudaFreeHost(h_act);
    return result;
}

// Device pointer tables of a call.
int tables(const std::vector<const float*>& i0, const std::vector<const float*>& i1, const std::vector<float*>& fl,
           void** mem, cudaStream_t s)
{
    const size_t n = i0.size();
    std::vector<const void*> h(3 * n);
    for (size_t q = 0; q < n; q++) {
        h[q] = i0[q];
        h[n + q] = i1[q];
        h[2 * n + q] = fl[q];
    }
    TCK(cudaMallocAsync(mem, 3 * n * sizeof(void*), s));
    TCK(cudaMemcpyAsync(*mem, h.data(), 3 * n * sizeof(void*), cudaMemcpyHostToDevice, s));
    TCK(cudaStreamSynchronize(s));  // h is a temporary
    return VBM3D_OK;
}

int run_tables(const std::vector<const float*>& i0, const std::vector<const float*>& i1, const std::vector<float*>& fl,
               int nx, int ny, const vbm3d_tvl1_params& p, int* iters, cudaStream_t s)
{
    void* mem = nullptr;
    int rc = tables(i0, i1, fl, &mem, s);
    if (rc) return rc;
    const size_t n = i0.size();
    const float* const* t = reinterpret_cast<const float* const*>(mem);
    float* const* f = reinterpret_cast<float* const*>(reinterpret_cast<void**>(mem) + 2 * n);
    rc = run(t, t + n, f, (int)n, nx, ny, p, iters, s);
    cudaFreeAsync(mem, s);
    return rc;
}

}  // namespace tvl1
}  // namespace vbm3d

using namespace vbm3d::tvl1;

extern "C" {

int vbm3d_tvl1_default_params(vbm3d_tvl1_params* p)
{
    if (!p) return fail(VBM3D_ERR_INVALID_ARGUMENT, "NULL output");
    // the options of tvl1flow/tvl1flow_forward.sh and tvl1flow_backward.sh
    p->tau = 0.25f;
    p->lambda = 0.2f;
    p->theta = 0.3f;
    p->nscales = 100;
    p->fscale = 2;
    p->zfactor = 0.5f;
    p->nwarps = 5;
    p->epsilon = 0.01f;
    return VBM3D_OK;
}

int vbm3d_tvl1_scales(unsigned width, unsigned height, const vbm3d_tvl1_params* p, int* nscales, int* fscale)
{
    int rc = check_params(p);
    if (rc) return rc;
    if (!nscales || !fscale) return fail(VBM3D_ERR_INVALID_ARGUMENT, "NULL output");
    int ns = p->nscales;
    const float N = 1 + log(hypot((double)width, (double)height) / 16.0) / log(1 / p->zfactor);
    if (N < ns) ns = N;
    *nscales = ns;
    *fscale = p->fscale < ns ? p->fscale : ns;
    return VBM3D_OK;
}

int vbm3d_gpu_tvl1_pairs(const float* I0, const float* I1, unsigned npairs, unsigned width, unsigned height,
                         const vbm3d_tvl1_params* p, float* flow, int* iterations, void* stream)
{
    int rc = check_params(p);
    if (rc) return rc;
    if (!I0 || !I1 || !flow) return fail(VBM3D_ERR_INVALID_ARGUMENT, "NULL pointer");
    if (!npairs || width < 2 || height < 2) return fail(VBM3D_ERR_INVALID_ARGUMENT, "empty or 1-pixel-wide input");
    if ((unsigned long long)width * height * npairs >= (1ull << 31))
        return fail(VBM3D_ERR_UNSUPPORTED, "more than 2^31 pixels in one call");
    const size_t wh = (size_t)width * height;
    std::vector<const float*> a(npairs), b(npairs);
    std::vector<float*> f(npairs);
    for (unsigned q = 0; q < npairs; q++) {
        a[q] = I0 + q * wh;
        b[q] = I1 + q * wh;
        f[q] = flow + q * 2 * wh;
    }
    return run_tables(a, b, f, (int)width, (int)height, *p, iterations, (cudaStream_t)stream);
}

int vbm3d_gpu_tvl1_video(const float* video, unsigned width, unsigned height, unsigned frames,
                         const vbm3d_tvl1_params* p, float* fflow, float* bflow, void* stream)
{
    int rc = check_params(p);
    if (rc) return rc;
    if (!video || !fflow || !bflow) return fail(VBM3D_ERR_INVALID_ARGUMENT, "NULL pointer");
    if (frames < 2 || width < 2 || height < 2) return fail(VBM3D_ERR_INVALID_ARGUMENT, "fewer than 2 frames");
    if ((unsigned long long)width * height * 2 * (frames - 1) >= (1ull << 31))
        return fail(VBM3D_ERR_UNSUPPORTED, "more than 2^31 pixels in one call");
    const size_t wh = (size_t)width * height;
    cudaStream_t s = (cudaStream_t)stream;
    // the last frame has no forward flow and bflow[F-1] no pair: zero, as
    // the reference's loader leaves missing flows
    TCK(cudaMemsetAsync(fflow + (size_t)(frames - 1) * 2 * wh, 0, 2 * wh * sizeof(float), s));
    TCK(cudaMemsetAsync(bflow + (size_t)(frames - 1) * 2 * wh, 0, 2 * wh * sizeof(float), s));
    std::vector<const float*> a, b;
    std::vector<float*> f;
    for (unsigned t = 0; t + 1 < frames; t++) {  // forward: frame t -> t + 1 into fflow[t]
        a.push_back(video + t * wh);
        b.push_back(video + (t + 1) * wh);
        f.push_back(fflow + (size_t)t * 2 * wh);
    }
    for (unsigned t = 0; t + 1 < frames; t++) {  // backward: frame t + 1 -> t into bflow[t]
        a.push_back(video + (t + 1) * wh);
        b.push_back(video + t * wh);
        f.push_back(bflow + (size_t)t * 2 * wh);
    }
    return run_tables(a, b, f, (int)width, (int)height, *p, nullptr, s);
}

}  // extern "C"
