// Host side of the C ABI declared in include/vbm3d_gb300.h.
//
// Validates arguments the way the reference's code paths require them,
// builds the per-step parameter block (tables of preProcess, the bior1.5
// bases, the DCT matrices, the noise table of estimate_sigma), owns the
// scratch memory of a step (block-matching table) in a stream-ordered pool,
// and launches the kernels on the caller's stream.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <atomic>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"
#include "../../include/vbm3d_gb300.h"

namespace vbm3d {
int bm_warp_bytes(const StepParams& P, int& list_cap, int& best_cap, int& win_cap);
cudaError_t launch_bm(const StepParams& P, const float* vid, const float* fflow, const float* bflow,
                      unsigned* out_idx, float* out_dist, unsigned* out_nsimp, unsigned* out_nsx,
                      long long count, cudaStream_t stream, unsigned long long* out_count = nullptr);
cudaError_t launch_filter(int step, const StepParams& P, const float* noisy, const float* basic,
                          const float* fflow, const unsigned* tab_idx, const unsigned* tab_nsx, float* num,
                          float* den, float* pair, long long count, cudaStream_t stream);
cudaError_t launch_split_pair(const float* pair, float* num, float* den, size_t n, cudaStream_t s);
cudaError_t launch_normalize_pair(const float* pair, const float* fb, float* out, size_t n, cudaStream_t s);
cudaError_t launch_normalize(const float* num, const float* den, const float* fb, float* out, size_t n,
                             cudaStream_t s);
cudaError_t launch_color(float* v, unsigned wh, unsigned frames, int forward, cudaStream_t s);
cudaError_t launch_filter_store(int step, const StepParams& P, const float* noisy, const float* basic,
                                const unsigned* tab_idx, const unsigned* tab_nsx, float* est, float* wts,
                                long long count, cudaStream_t stream);
size_t det_scratch_words(const StepHead& P);
cudaError_t launch_det_aggregate(const StepParams& P, const unsigned* tab_idx, const unsigned* tab_nsx,
                                 const float* est, const float* wts, unsigned* scratch, float* pair,
                                 cudaStream_t s);
}  // namespace vbm3d

using namespace vbm3d;

namespace {

thread_local std::string g_err;

int fail(int status, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return status;
}

int cuda_fail(cudaError_t e, const char* what)
{
    if (e == cudaErrorMemoryAllocation)
        return fail(VBM3D_ERR_OUT_OF_MEMORY, "%s: %s", what, cudaGetErrorString(e));
    return fail(VBM3D_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define CK(call)                                              \
    do {                                                      \
        cudaError_t e_ = (call);                              \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call);   \
    } while (0)

// One stream-ordered memory pool per device, created on first use; memory
// freed into it is kept for the next call (release threshold = max).
cudaMemPool_t pool_for_current_device()
{
    static std::mutex mu;
    static std::vector<cudaMemPool_t> pools;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lock(mu);
    if ((int)pools.size() <= dev) pools.resize(dev + 1, nullptr);
    if (!pools[dev]) {
        cudaMemPoolProps props;
        memset(&props, 0, sizeof props);
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        cudaMemPool_t p = nullptr;
        if (cudaMemPoolCreate(&p, &props) != cudaSuccess) return nullptr;
        uint64_t thr = ~0ull;
        cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &thr);
        pools[dev] = p;
    }
    return pools[dev];
}

template <class T>
cudaError_t pool_alloc(T** p, size_t count, cudaStream_t s)
{
    cudaMemPool_t pool = pool_for_current_device();
    if (!pool) return cudaErrorMemoryAllocation;
    return cudaMallocFromPoolAsync(reinterpret_cast<void**>(p), count * sizeof(T) + 16, pool, s);
}

// A pool allocation freed (stream-ordered) when it goes out of scope, so
// that an early error return (CK) releases it too.
template <class T>
struct PoolBuf {
    T* p = nullptr;
    cudaStream_t s;
    explicit PoolBuf(cudaStream_t st) : s(st) {}
    PoolBuf(const PoolBuf&) = delete;
    PoolBuf& operator=(const PoolBuf&) = delete;
    cudaError_t alloc(size_t count) { return pool_alloc(&p, count, s); }
    ~PoolBuf()
    {
        if (p) cudaFreeAsync(p, s);
    }
};

// ind_size (src/Utilities/Utilities.cpp:441-458) for beginning = 0.
unsigned grid_size(unsigned end, unsigned step)
{
    unsigned ind = 0, k = 0, last = 0;
    while (ind <= end) {
        last = ind;
        k++;
        ind += step;
    }
    if (last < end) k++;
    return k;
}

double bessel_i0(double x)
{
    double sum = 1.0, term = 1.0, q = x * x / 4.0;
    for (int m = 1; m < 60; m++) {
        term *= q / ((double)m * (double)m);
        sum += term;
        if (term < 1e-18 * sum) break;
    }
    return sum;
}

// The Kaiser window of preProcess (src/vbm3d.cpp:1754-1841): for k in
// {4, 6, 7, 8, 12} the reference lists 4-decimal tables, which are the
// outer product of the beta = 2 Kaiser window rounded to 4 decimals; other
// k use ones.
void kaiser_window(unsigned k, float* w)
{
    if (k != 4 && k != 6 && k != 7 && k != 8 && k != 12) {
        for (unsigned i = 0; i < k * k; i++) w[i] = 1.0f;
        return;
    }
    double w1[kMaxK];
    const double i0b = bessel_i0(2.0);
    for (unsigned n = 0; n < k; n++) {
        const double r = 2.0 * n / (k - 1) - 1.0;
        w1[n] = bessel_i0(2.0 * std::sqrt(1.0 - r * r)) / i0b;
    }
    for (unsigned i = 0; i < k; i++)
        for (unsigned j = 0; j < k; j++) w[i * k + j] = (float)(std::floor(w1[i] * w1[j] * 1e4 + 0.5) / 1e4);
}

// bior1.5 basis rows of the reference's MATLAB path
// (src/lib_transforms.cpp:139-148 forward, :279-288 inverse).
const double kBiorFwd[8][8] = {
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
const double kBiorInv[8][8] = {
    {0.353553390593274, 0.353553390593274, 0.5, 0.0, 0.707106781186547, -0.121533978016438, 0.0, 0.121533978016438},
    {0.353553390593274, 0.353553390593274, 0.5, -0.0, -0.707106781186547, -0.121533978016438, 0.0, 0.121533978016438},
    {0.353553390593274, 0.353553390593274, -0.5, -0.0, 0.121533978016438, 0.707106781186548, -0.121533978016438, 0.0},
    {0.353553390593274, 0.353553390593274, -0.5, 0.0, 0.121533978016438, -0.707106781186548, -0.121533978016438, 0.0},
    {0.353553390593274, -0.353553390593274, 0.0, 0.5, 0.0, 0.121533978016438, 0.707106781186547, -0.121533978016438},
    {0.353553390593274, -0.353553390593274, 0.0, 0.5, 0.0, 0.121533978016438, -0.707106781186547, -0.121533978016438},
    {0.353553390593274, -0.353553390593274, 0.0, -0.5, -0.121533978016438, 0.0, 0.121533978016438, 0.707106781186547},
    {0.353553390593274, -0.353553390593274, 0.0, -0.5, -0.121533978016438, 0.0, 0.121533978016438, -0.707106781186547}};

int sigma_table(float sigma, unsigned chnls, int color_space, float* t)
{
    // estimate_sigma (src/Utilities/Utilities.cpp:282-333) with the bool
    // color_space read as an int: true -> YCbCr norms, false -> YUV norms.
    if (chnls == 1) {
        t[0] = sigma;
        return VBM3D_OK;
    }
    if (chnls != 3) return fail(VBM3D_ERR_COLOR_SPACE, "estimate_sigma supports 1 or 3 channels, got %u", chnls);
    if (!color_space) {
        t[0] = sqrtf(0.299f * 0.299f + 0.587f * 0.587f + 0.114f * 0.114f) * sigma;
        t[1] = sqrtf(0.14713f * 0.14713f + 0.28886f * 0.28886f + 0.436f * 0.436f) * sigma;
        t[2] = sqrtf(0.615f * 0.615f + 0.51498f * 0.51498f + 0.10001f * 0.10001f) * sigma;
    } else {
        t[0] = sqrtf(0.299f * 0.299f + 0.587f * 0.587f + 0.114f * 0.114f) * sigma;
        t[1] = sqrtf(0.169f * 0.169f + 0.331f * 0.331f + 0.500f * 0.500f) * sigma;
        t[2] = sqrtf(0.500f * 0.500f + 0.419f * 0.419f + 0.081f * 0.081f) * sigma;
    }
    return VBM3D_OK;
}

int check_dims(vbm3d_dims d)
{
    if (d.width == 0 || d.height == 0 || d.frames == 0 || d.channels == 0)
        return fail(VBM3D_ERR_INVALID_ARGUMENT, "zero-sized video %ux%ux%ux%u", d.width, d.height, d.frames,
                    d.channels);
    if (d.channels != 1 && d.channels != 3)
        return fail(VBM3D_ERR_UNSUPPORTED, "channels must be 1 or 3, got %u", d.channels);
    const unsigned long long n = (unsigned long long)d.width * d.height * d.frames * d.channels;
    if (n >= (1ull << 32))
        return fail(VBM3D_ERR_UNSUPPORTED, "video of %llu values: patch indices are 32-bit as in the reference", n);
    return VBM3D_OK;
}

int check_params(const vbm3d_params* p, vbm3d_dims d)
{
    if (!p) return fail(VBM3D_ERR_INVALID_ARGUMENT, "NULL parameters");
    if (p->k == 0) return fail(VBM3D_ERR_INVALID_ARGUMENT, "k == 0 (a skipped step cannot be run)");
    if (p->p == 0) return fail(VBM3D_ERR_INVALID_ARGUMENT, "step p == 0");
    if (p->N == 0 || p->Nb == 0) return fail(VBM3D_ERR_INVALID_ARGUMENT, "N and Nb must be positive");
    if (p->T_2D != VBM3D_DCT && p->T_2D != VBM3D_BIOR)
        return fail(VBM3D_ERR_INVALID_ARGUMENT, "T_2D must be DCT (0) or BIOR (1), got %u", p->T_2D);
    if (p->T_2D == VBM3D_BIOR && p->k != 8)
        return fail(VBM3D_ERR_INVALID_ARGUMENT, "bior1.5 needs k == 8 (src/lib_transforms.cpp:137)");
    if (p->k > (unsigned)kMaxK) return fail(VBM3D_ERR_UNSUPPORTED, "k > %d", kMaxK);
    if (p->kt > (unsigned)kMaxKt) return fail(VBM3D_ERR_UNSUPPORTED, "kt > %d", kMaxKt);
    if (p->N > (unsigned)kMaxN) return fail(VBM3D_ERR_UNSUPPORTED, "N > %d", kMaxN);
    if (p->Nb > (unsigned)kMaxNb) return fail(VBM3D_ERR_UNSUPPORTED, "Nb > %d", kMaxNb);
    if (p->Ns > (unsigned)kMaxWin || p->Npr > (unsigned)kMaxWin)
        return fail(VBM3D_ERR_UNSUPPORTED, "search windows above %d", kMaxWin);
    if (p->Nf > (unsigned)kMaxNf) return fail(VBM3D_ERR_UNSUPPORTED, "Nf > %d", kMaxNf);
    if (d.width < p->k || d.height < p->k || d.frames < p->kt)
        return fail(VBM3D_ERR_INVALID_ARGUMENT, "video %ux%ux%u smaller than a %ux%ux%u patch", d.width, d.height,
                    d.frames, p->k, p->k, p->kt);
    // The reference reads Nb matches of the reference-frame window
    // (src/vbm3d.cpp:1115-1119) even when the window holds fewer.
    const int s = (int)p->Ns, half = (s - 1) / 2;
    const unsigned wx = std::min<unsigned>((unsigned)half + 1, d.width - p->k + 1);
    const unsigned wy = std::min<unsigned>((unsigned)half + 1, d.height - p->k + 1);
    if (wx * wy < p->Nb)
        return fail(VBM3D_ERR_INVALID_ARGUMENT,
                    "a corner search window holds %u positions < Nb = %u (the reference reads past its end)",
                    wx * wy, p->Nb);
    return VBM3D_OK;
}

int build_params(const vbm3d_params* p, vbm3d_dims d, float sigma, int color_space, StepParams& P)
{
    int rc = check_dims(d);
    if (rc) return rc;
    rc = check_params(p, d);
    if (rc) return rc;
    memset(&P, 0, sizeof P);
    P.W = (int)d.width;
    P.H = (int)d.height;
    P.F = (int)d.frames;
    P.C = (int)d.channels;
    P.wh = d.width * d.height;
    P.whc = P.wh * d.channels;
    P.k = (int)p->k;
    P.kt = (int)p->kt;
    P.p = (int)p->p;
    P.N = (int)p->N;
    P.Nf = (int)p->Nf;
    P.Ns = (int)p->Ns;
    P.Npr = (int)p->Npr;
    P.Nb = (int)p->Nb;
    P.T2D = (int)p->T_2D;
    P.T3D = p->T_3D == VBM3D_HADAMARD ? kHADAMARD : 4;
    P.mc = p->mc;
    P.tau = p->tau;
    P.dbias = p->d;
    P.lambda3D = p->lambda3D;
    P.nrows = (int)grid_size(d.height - p->k, p->p);
    P.ncols = (int)grid_size(d.width - p->k, p->p);
    P.nframes = (int)(d.frames - p->kt + 1);
    P.nrefs = (long long)P.nrows * P.ncols * P.nframes;
    rc = sigma_table(sigma, d.channels, color_space, P.sigma);
    if (rc) return rc;
    const unsigned k = p->k;
    kaiser_window(k, P.kaiser);
    // preProcess normalisation (src/vbm3d.cpp:1843-1863)
    const float coef = 0.5f / ((float)k);
    for (unsigned i = 0; i < k; i++)
        for (unsigned j = 0; j < k; j++) {
            if (i == 0 && j == 0) {
                P.cn[i * k + j] = 0.5f * coef;
                P.cni[i * k + j] = 2.0f;
            } else if (i * j == 0) {
                P.cn[i * k + j] = (float)(0.7071067811865475 * coef);
                P.cni[i * k + j] = (float)1.414213562373095;
            } else {
                P.cn[i * k + j] = 1.0f * coef;
                P.cni[i * k + j] = 1.0f;
            }
        }
    if (p->T_2D == VBM3D_BIOR) {
        for (int j = 0; j < 8; j++)
            for (int q = 0; q < 8; q++) {
                P.fwd[j * 8 + q] = (float)kBiorFwd[j][q];
                P.inv[j * 8 + q] = (float)kBiorInv[j][q];
            }
    } else {
        const double pi = 3.14159265358979323846;
        for (unsigned u = 0; u < k; u++)
            for (unsigned j = 0; j < k; j++) {
                P.fwd[u * k + j] = (float)(2.0 * std::cos(pi * (j + 0.5) * u / k));  // REDFT10
                P.inv[j * k + u] = u == 0 ? 1.0f : (float)(2.0 * std::cos(pi * u * (j + 0.5) / k));  // REDFT01
            }
    }
    for (unsigned i = 0; i < k; i++)
        for (unsigned j = 0; j < k; j++) {
            P.fwdT[i * k + j] = P.fwd[j * k + i];
            P.invT[i * k + j] = P.inv[j * k + i];
        }
    P.bm_warp_bytes = bm_warp_bytes(P, P.bm_list_cap, P.bm_best_cap, P.bm_win_cap);
    P.neg_zero = -0.0f;
    // Aggregation bands: a band's groups add into the 2 Nf + 1 frames around
    // each frame of it, over its rows plus the search reach; size the band so
    // that these (num, den) rows (8 bytes per value) take about 32 MB of L2.
    {
        const double frames = 2.0 * p->Nf + p->kt;
        const double reach = (double)p->Ns / 2 + (double)p->Nf * p->Npr / 2 + p->k;
        const double rows_px = 32e6 / (8.0 * d.width * d.channels * frames) - 2.0 * reach;
        P.band_rows = std::max(4, (int)(rows_px / p->p));
        if (P.band_rows >= P.nrows) P.band_rows = 0;
    }
    return VBM3D_OK;
}

// Aggregation mode of the plain path (vbm3d_set_deterministic).
std::atomic<int> g_deterministic{0};

// One step with the deterministic aggregation (det_agg.cu): the filter
// keeps every group's weighted estimates, then one ordered pass sums them
// into `pair`, in the reference's order.
int run_step_pair_det(int step, const StepParams& P, const float* noisy, const float* basic, const float* fflow,
                      const float* bflow, const unsigned* tab_idx, const unsigned* tab_nsx, float* pair,
                      cudaStream_t s)
{
    (void)fflow;
    (void)bflow;
    if (!((P.k == 7 || P.k == 8) && P.kt == 1 && P.N <= 8))
        return fail(VBM3D_ERR_UNSUPPORTED, "deterministic aggregation: k in {7, 8}, kt == 1 and N <= 8 only");
    if (P.nrefs >= (1ll << 29) || P.W >= 65536 || P.H >= 65536)
        return fail(VBM3D_ERR_UNSUPPORTED, "deterministic aggregation: video too large for its 32-bit keys");
    PoolBuf<float> est(s), wts(s);
    PoolBuf<unsigned> scr(s);
    CK(est.alloc((size_t)P.nrefs * P.C * P.N * P.k * P.k));
    CK(wts.alloc((size_t)P.nrefs * P.C));
    CK(scr.alloc(det_scratch_words(P)));
    CK(launch_filter_store(step, P, noisy, basic, tab_idx, tab_nsx, est.p, wts.p, P.nrefs, s));
    CK(launch_det_aggregate(P, tab_idx, tab_nsx, est.p, wts.p, scr.p, pair, s));
    return VBM3D_OK;
}

// One step into the interleaved (numerator, denominator) accumulator
// `pair` (2 floats per video value), which it overwrites.  P is validated.
int run_step_pair(int step, const StepParams& P, const float* noisy, const float* basic, const float* fflow,
                  const float* bflow, float* pair, cudaStream_t s)
{
    const size_t n = (size_t)P.whc * P.F;
    PoolBuf<unsigned> tab_idx(s), tab_nsx(s);
    CK(tab_idx.alloc((size_t)P.nrefs * P.N));
    CK(tab_nsx.alloc((size_t)P.nrefs));
    CK(launch_bm(P, step == 1 ? noisy : basic, fflow, bflow, tab_idx.p, nullptr, nullptr, tab_nsx.p, P.nrefs, s));
    if (g_deterministic.load())
        return run_step_pair_det(step, P, noisy, basic, fflow, bflow, tab_idx.p, tab_nsx.p, pair, s);
    CK(cudaMemsetAsync(pair, 0, 2 * n * sizeof(float), s));
    CK(launch_filter(step, P, noisy, basic, fflow, tab_idx.p, tab_nsx.p, nullptr, nullptr, pair, P.nrefs, s));
    return VBM3D_OK;
}

int run_step(int step, const vbm3d_params* prms, const float* noisy, const float* basic, const float* fflow,
             const float* bflow, vbm3d_dims dims, float sigma, int color_space, float* num, float* den,
             void* stream)
{
    if (!noisy || !num || !den || (step == 2 && !basic))
        return fail(VBM3D_ERR_INVALID_ARGUMENT, "NULL video pointer");
    StepParams P;
    int rc = build_params(prms, dims, sigma, color_space, P);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    const size_t n = (size_t)P.whc * P.F;
    float* pair = nullptr;
    CK(pool_alloc(&pair, 2 * n, s));
    rc = run_step_pair(step, P, noisy, basic, fflow, bflow, pair, s);
    if (rc == VBM3D_OK) {
        cudaError_t e = launch_split_pair(pair, num, den, n, s);
        if (e != cudaSuccess) rc = cuda_fail(e, "split");
    }
    cudaFreeAsync(pair, s);
    return rc;
}

// A host flow onto the device: the steps never read a flow's last frame
// (forward chains stop at the last frame, backward chains and trajectories
// read frames up to F - 2), so only the first F - 1 frames are copied, and
// a caller may pass the F - 1 frames its flow files hold; the device copy's
// last frame is zeroed.
cudaError_t upload_flow(float* d, const float* h, vbm3d_dims dims, cudaStream_t s)
{
    const size_t frame = (size_t)dims.width * dims.height * 2;
    const size_t used = frame * (dims.frames - 1);
    cudaError_t e = cudaSuccess;
    if (used) e = cudaMemcpyAsync(d, h, used * sizeof(float), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(d + used, 0, frame * sizeof(float), s);
    return e;
}

}  // namespace

namespace vbm3d {
// For entry points defined in other translation units.
int build_step_params(const vbm3d_params* p, vbm3d_dims d, float sigma, int color_space, StepParams& P)
{
    return build_params(p, d, sigma, color_space, P);
}
void set_last_error(int status, const char* msg) { fail(status, "%s", msg); }
}  // namespace vbm3d

extern "C" {

const char* vbm3d_last_error(void) { return g_err.c_str(); }

const char* vbm3d_status_string(int status)
{
    switch (status) {
        case VBM3D_OK: return "VBM3D_OK";
        case VBM3D_ERR_INVALID_ARGUMENT: return "VBM3D_ERR_INVALID_ARGUMENT";
        case VBM3D_ERR_UNSUPPORTED: return "VBM3D_ERR_UNSUPPORTED";
        case VBM3D_ERR_CUDA: return "VBM3D_ERR_CUDA";
        case VBM3D_ERR_OUT_OF_MEMORY: return "VBM3D_ERR_OUT_OF_MEMORY";
        case VBM3D_ERR_COLOR_SPACE: return "VBM3D_ERR_COLOR_SPACE";
        case VBM3D_ERR_SIZE_MISMATCH: return "VBM3D_ERR_SIZE_MISMATCH";
        default: return "unknown vbm3d status";
    }
}

int vbm3d_default_params(int step, float sigma, vbm3d_params* o)
{
    if (!o) return fail(VBM3D_ERR_INVALID_ARGUMENT, "NULL output");
    memset(o, 0, sizeof *o);
    if (step == 1) {  // initializeParameters_1 (src/main.cpp:35-125)
        o->k = 8;
        o->kt = 1;
        o->Nf = 4;
        o->Ns = 7;
        o->Npr = 5;
        o->Nb = 2;
        o->d = (float)((7. * 7. * 255.) / (o->k * o->k * o->kt));
        o->p = o->k / 4 * 3;
        o->N = 8;
        o->tau = (sigma > 30) ? 4500 : 3000;
        o->lambda3D = 2.7f;
        o->T_2D = o->k == 8 ? VBM3D_BIOR : VBM3D_DCT;
        o->T_3D = 3;  // HAAR in src/main.cpp:30
    } else if (step == 2) {  // initializeParameters_2 (src/main.cpp:127-207)
        o->k = (sigma > 30) ? 8 : 7;
        o->kt = 1;
        o->Nf = 4;
        o->Ns = 7;
        o->Npr = 5;
        o->Nb = 2;
        o->d = (float)((3. * 3. * 255.) / (o->k * o->k * o->kt));
        o->p = o->k / 2;
        o->N = 8;
        o->tau = (sigma > 30) ? 3000 : 1500;
        o->T_2D = VBM3D_DCT;
        o->T_3D = 3;
    } else {
        return fail(VBM3D_ERR_INVALID_ARGUMENT, "step must be 1 or 2, got %d", step);
    }
    o->mc = 0;
    o->n = 16;
    return VBM3D_OK;
}

int vbm3d_set_deterministic(int on)
{
    g_deterministic.store(on ? 1 : 0);
    return VBM3D_OK;
}

int vbm3d_get_deterministic(void) { return g_deterministic.load(); }

int vbm3d_sigma_table(float sigma, unsigned channels, int color_space, float* t)
{
    if (!t) return fail(VBM3D_ERR_INVALID_ARGUMENT, "NULL output");
    return sigma_table(sigma, channels, color_space, t);
}

int vbm3d_ref_count(const vbm3d_params* prms, vbm3d_dims dims, size_t* n_refs)
{
    if (!n_refs) return fail(VBM3D_ERR_INVALID_ARGUMENT, "NULL output");
    int rc = check_dims(dims);
    if (rc) return rc;
    rc = check_params(prms, dims);
    if (rc) return rc;
    *n_refs = (size_t)grid_size(dims.height - prms->k, prms->p) * grid_size(dims.width - prms->k, prms->p) *
              (dims.frames - prms->kt + 1);
    return VBM3D_OK;
}

int vbm3d_gpu_step1(const vbm3d_params* prms, const float* noisy, const float* fflow, const float* bflow,
                    vbm3d_dims dims, float sigma, int color_space, float* numerator, float* denominator,
                    void* stream)
{
    return run_step(1, prms, noisy, nullptr, fflow, bflow, dims, sigma, color_space, numerator, denominator,
                    stream);
}

int vbm3d_gpu_step2(const vbm3d_params* prms, const float* noisy, const float* basic, const float* fflow,
                    const float* bflow, vbm3d_dims dims, float sigma, int color_space, float* numerator,
                    float* denominator, void* stream)
{
    return run_step(2, prms, noisy, basic, fflow, bflow, dims, sigma, color_space, numerator, denominator,
                    stream);
}

int vbm3d_gpu_normalize(const float* numerator, const float* denominator, const float* fallback, float* out,
                        size_t count, void* stream)
{
    if (!numerator || !denominator || !fallback || !out) return fail(VBM3D_ERR_INVALID_ARGUMENT, "NULL pointer");
    if (count == 0) return VBM3D_OK;
    CK(launch_normalize(numerator, denominator, fallback, out, count, (cudaStream_t)stream));
    return VBM3D_OK;
}

int vbm3d_gpu_color_transform(float* video, vbm3d_dims dims, int forward, void* stream)
{
    if (!video) return fail(VBM3D_ERR_INVALID_ARGUMENT, "NULL pointer");
    int rc = check_dims(dims);
    if (rc) return rc;
    if (dims.channels != 3) return VBM3D_OK;  // src/Utilities/LibVideoT.hpp:770
    CK(launch_color(video, dims.width * dims.height, dims.frames, forward, (cudaStream_t)stream));
    return VBM3D_OK;
}

int vbm3d_gpu_similar_patches(const vbm3d_params* prms, const float* video, const float* fflow,
                              const float* bflow, vbm3d_dims dims, unsigned* indexes, float* distances,
                              unsigned* nsimp, unsigned* nsx, size_t* n_refs, void* stream)
{
    StepParams P;
    int rc = build_params(prms, dims, 0.f, 0, P);
    if (rc) return rc;
    if (n_refs) *n_refs = (size_t)P.nrefs;
    if (!indexes && !distances && !nsimp && !nsx) return VBM3D_OK;
    if (!video) return fail(VBM3D_ERR_INVALID_ARGUMENT, "NULL video pointer");
    cudaStream_t s = (cudaStream_t)stream;
    PoolBuf<unsigned> own_idx(s), own_ns(s);  // the tables the caller does not take
    unsigned *idx = indexes, *ns = nsx;
    if (!idx) {
        CK(own_idx.alloc((size_t)P.nrefs * P.N));
        idx = own_idx.p;
    }
    if (!ns) {
        CK(own_ns.alloc((size_t)P.nrefs));
        ns = own_ns.p;
    }
    CK(launch_bm(P, video, fflow, bflow, idx, distances, nsimp, ns, P.nrefs, s));
    return VBM3D_OK;
}

int vbm3d_gpu_bm_distance_count(const vbm3d_params* prms, const float* video, const float* fflow,
                                 const float* bflow, vbm3d_dims dims, unsigned long long* count, void* stream)
{
    if (!video || !count) return fail(VBM3D_ERR_INVALID_ARGUMENT, "NULL pointer");
    StepParams P;
    int rc = build_params(prms, dims, 0.f, 0, P);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    PoolBuf<unsigned> idx(s), ns(s);
    PoolBuf<unsigned long long> d_count(s);
    CK(idx.alloc((size_t)P.nrefs * P.N));
    CK(ns.alloc((size_t)P.nrefs));
    CK(d_count.alloc(1));
    CK(cudaMemsetAsync(d_count.p, 0, sizeof(unsigned long long), s));
    CK(launch_bm(P, video, fflow, bflow, idx.p, nullptr, nullptr, ns.p, P.nrefs, s, d_count.p));
    CK(cudaMemcpyAsync(count, d_count.p, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return VBM3D_OK;
}

int vbm3d_gpu_run(float sigma, float* noisy, const float* fflow, const float* bflow, float* basic,
                  float* denoised, const vbm3d_params* prms_1, const vbm3d_params* prms_2, int color_space,
                  vbm3d_dims dims, void* stream)
{
    if (!noisy || !basic || !denoised || !prms_1 || !prms_2)
        return fail(VBM3D_ERR_INVALID_ARGUMENT, "NULL pointer");
    int rc = check_dims(dims);
    if (rc) return rc;
    if (prms_1->k > 0 && (rc = check_params(prms_1, dims))) return rc;
    if (prms_2->k > 0 && (rc = check_params(prms_2, dims))) return rc;
    float tab[3];
    if ((rc = sigma_table(sigma, dims.channels, color_space, tab))) return rc;
    StepParams P1, P2;
    if (prms_1->k > 0 && (rc = build_params(prms_1, dims, sigma, color_space, P1))) return rc;
    if (prms_2->k > 0 && (rc = build_params(prms_2, dims, sigma, color_space, P2))) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    const size_t n = (size_t)dims.width * dims.height * dims.frames * dims.channels;
    const unsigned wh = dims.width * dims.height;
    if (color_space) {
        if (prms_1->k > 0) rc = vbm3d_gpu_color_transform(noisy, dims, 1, stream);
        else rc = vbm3d_gpu_color_transform(basic, dims, 1, stream);
        if (rc) return rc;
    }
    float* pair = nullptr;
    CK(pool_alloc(&pair, 2 * n, s));
    if (prms_1->k > 0) {
        if ((rc = run_step_pair(1, P1, noisy, nullptr, fflow, bflow, pair, s))) goto out;
        cudaError_t e = launch_normalize_pair(pair, noisy, basic, n, s);
        if (e != cudaSuccess) {
            rc = cuda_fail(e, "normalize");
            goto out;
        }
    }
    if (prms_2->k > 0) {
        if ((rc = run_step_pair(2, P2, noisy, basic, fflow, bflow, pair, s))) goto out;
        cudaError_t e = launch_normalize_pair(pair, basic, denoised, n, s);
        if (e != cudaSuccess) {
            rc = cuda_fail(e, "normalize");
            goto out;
        }
    } else {
        cudaError_t e = cudaMemcpyAsync(denoised, basic, n * sizeof(float), cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess) {
            rc = cuda_fail(e, "cudaMemcpyAsync");
            goto out;
        }
    }
    if (color_space && dims.channels == 3) {  // one-channel videos are left as they are
        launch_color(denoised, wh, dims.frames, 0, s);
        launch_color(noisy, wh, dims.frames, 0, s);
        cudaError_t e = launch_color(basic, wh, dims.frames, 0, s);
        if (e != cudaSuccess) rc = cuda_fail(e, "color transform");
    }
out:
    cudaFreeAsync(pair, s);
    return rc;
}

int vbm3d_step_host(int step, const vbm3d_params* prms, const float* noisy, const float* basic,
                    const float* fflow, const float* bflow, vbm3d_dims dims, float sigma, int color_space,
                    float* numerator, float* denominator)
{
    if (step != 1 && step != 2) return fail(VBM3D_ERR_INVALID_ARGUMENT, "step must be 1 or 2, got %d", step);
    if (!noisy || !numerator || !denominator || (step == 2 && !basic))
        return fail(VBM3D_ERR_INVALID_ARGUMENT, "NULL pointer");
    StepParams P;
    int rc = build_params(prms, dims, sigma, color_space, P);
    if (rc) return rc;
    const size_t n = (size_t)dims.width * dims.height * dims.frames * dims.channels;
    const size_t nf = (size_t)dims.width * dims.height * dims.frames * 2;
    cudaStream_t s = nullptr;
    CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    float *d_noisy = nullptr, *d_basic = nullptr, *d_num = nullptr, *d_den = nullptr, *d_ff = nullptr,
          *d_bf = nullptr;
    cudaError_t e = pool_alloc(&d_noisy, n, s);
    if (e == cudaSuccess && step == 2) e = pool_alloc(&d_basic, n, s);
    if (e == cudaSuccess) e = pool_alloc(&d_num, n, s);
    if (e == cudaSuccess) e = pool_alloc(&d_den, n, s);
    if (e == cudaSuccess && fflow) e = pool_alloc(&d_ff, nf, s);
    if (e == cudaSuccess && bflow) e = pool_alloc(&d_bf, nf, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_noisy, noisy, n * sizeof(float), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && step == 2) e = cudaMemcpyAsync(d_basic, basic, n * sizeof(float), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && fflow) e = upload_flow(d_ff, fflow, dims, s);
    if (e == cudaSuccess && bflow) e = upload_flow(d_bf, bflow, dims, s);
    if (e != cudaSuccess) {
        rc = cuda_fail(e, "device buffers");
    } else {
        rc = run_step(step, prms, d_noisy, d_basic, d_ff, d_bf, dims, sigma, color_space, d_num, d_den, s);
        if (rc == VBM3D_OK) {
            e = cudaMemcpyAsync(numerator, d_num, n * sizeof(float), cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaMemcpyAsync(denominator, d_den, n * sizeof(float), cudaMemcpyDeviceToHost, s);
            if (e != cudaSuccess) rc = cuda_fail(e, "cudaMemcpyAsync D2H");
        }
    }
    for (float* ptr : {d_noisy, d_basic, d_num, d_den, d_ff, d_bf})
        if (ptr) cudaFreeAsync(ptr, s);
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess && rc == VBM3D_OK) rc = cuda_fail(e, "cudaStreamSynchronize");
    cudaStreamDestroy(s);
    return rc;
}

int vbm3d_run_host(float sigma, const float* noisy, const float* fflow, const float* bflow, float* basic,
                   float* denoised, const vbm3d_params* prms_1, const vbm3d_params* prms_2, int color_space,
                   vbm3d_dims dims)
{
    if (!noisy || !basic || !denoised) return fail(VBM3D_ERR_INVALID_ARGUMENT, "NULL pointer");
    int rc = check_dims(dims);
    if (rc) return rc;
    const size_t n = (size_t)dims.width * dims.height * dims.frames * dims.channels;
    const size_t nf = (size_t)dims.width * dims.height * dims.frames * 2;
    cudaStream_t s = nullptr;
    CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    float *d_noisy = nullptr, *d_basic = nullptr, *d_den = nullptr, *d_ff = nullptr, *d_bf = nullptr;
    cudaError_t e = pool_alloc(&d_noisy, n, s);
    if (e == cudaSuccess) e = pool_alloc(&d_basic, n, s);
    if (e == cudaSuccess) e = pool_alloc(&d_den, n, s);
    if (e == cudaSuccess && fflow) e = pool_alloc(&d_ff, nf, s);
    if (e == cudaSuccess && bflow) e = pool_alloc(&d_bf, nf, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_noisy, noisy, n * sizeof(float), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && fflow) e = upload_flow(d_ff, fflow, dims, s);
    if (e == cudaSuccess && bflow) e = upload_flow(d_bf, bflow, dims, s);
    if (e == cudaSuccess && prms_1 && prms_1->k == 0)
        e = cudaMemcpyAsync(d_basic, basic, n * sizeof(float), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) {
        rc = cuda_fail(e, "device buffers");
    } else {
        rc = vbm3d_gpu_run(sigma, d_noisy, d_ff, d_bf, d_basic, d_den, prms_1, prms_2, color_space, dims, s);
        if (rc == VBM3D_OK) {
            e = cudaMemcpyAsync(basic, d_basic, n * sizeof(float), cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaMemcpyAsync(denoised, d_den, n * sizeof(float), cudaMemcpyDeviceToHost, s);
            if (e != cudaSuccess) rc = cuda_fail(e, "cudaMemcpyAsync D2H");
        }
    }
    cudaFreeAsync(d_noisy, s);
    cudaFreeAsync(d_basic, s);
    cudaFreeAsync(d_den, s);
    if (d_ff) cudaFreeAsync(d_ff, s);
    if (d_bf) cudaFreeAsync(d_bf, s);
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess && rc == VBM3D_OK) rc = cuda_fail(e, "cudaStreamSynchronize");
    cudaStreamDestroy(s);
    return rc;
}

}  // extern "C"
