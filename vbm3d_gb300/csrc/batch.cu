// Batched form: many clips of uneven size, channel count and noise level
// denoised by one CUDA graph launch.  (No reference counterpart: the
// reference denoises one clip per process, src/main.cpp.)
//
// Each clip is run with run_vbm3d's semantics (src/vbm3d.cpp:87-211):
// optional colour transform, step 1, division with fallback to the noisy
// clip, step 2, division with fallback to the basic estimate, inverse colour
// transform.  The graph holds, for the whole batch:
//
//   reset of the work-queue heads
//   prep      noisy -> working colour space; zero the (num, den) accumulator
//   bm<1>     persistent block matching of every clip's step-1 grid
//   filter<1> persistent hard-threshold filtering + aggregation
//   mid       basic = num / den (fallback noisy); zero the accumulator
//   bm<2>     persistent block matching on the basic estimates
//   filter<2> persistent Wiener filtering + aggregation
//   final     denoised = num / den (fallback basic); inverse colour transform
//
// Each work phase is one persistent kernel per class of clip present in
// the batch (block matching: (k, C); filtering: the transform table set),
// sized to the GPU's occupancy and launched back to back.  A kernel's
// blocks pull work items (clip, reference-patch tile inside one frame) from
// its class's device queue with one atomicAdd per item and run the
// per-reference bodies of the plain kernels (bm2_impl.cuh,
// filter_common.cuh) over the tile (batch_kernels.cuh).  Nothing waits on
// anything: a block leaves when its queue is empty, and kernel boundaries
// are the only barriers.  Items are ordered by clip cost, most expensive
// first, so a phase ends on cheap items.
//
// The autotuner picks refs per item and warps per block for each phase by
// timing candidates on a strided sample of the phase's items during one
// eager pass over the batch (whose results the graph's runs overwrite).
// Choices are cached per batch signature for the life of the process.
#include <algorithm>
#include <chrono>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "batch.cuh"
#include "../../include/vbm3d_gb300.h"

namespace vbm3d {
int build_step_params(const vbm3d_params* p, vbm3d_dims d, float sigma, int color_space, StepParams& P);
void set_last_error(int status, const char* msg);

// A named namespace: bm2_impl.cuh's helpers live in an anonymous namespace
// inside vbm3d, and a second anonymous one here would make the kernels'
// host stubs ambiguous.
namespace batched {

// ------------------------------------------------ elementwise phases ---
// One block per chunk (clip, first pixel position, count); a position is a
// (frame, pixel) pair and covers the clip's C channels.

__global__ void __launch_bounds__(256) batch_prep_kernel(const BatchClip* __restrict__ clips,
                                                        const uint4* __restrict__ chunks)
{
    const uint4 K = chunks[blockIdx.x];
    const BatchClip& B = clips[K.x];
    const unsigned wh = B.wh, C = B.C;
    const float* __restrict__ in = B.in;
    float* __restrict__ y = B.y;
    float2* __restrict__ pr = reinterpret_cast<float2*>(B.pair);
    for (unsigned i = threadIdx.x; i < K.z; i += blockDim.x) {
        const size_t pos = (size_t)K.y + i, t = pos / wh, k = pos - t * wh;
        const size_t o = t * C * wh + k;
        if (C == 3) {
            float a = in[o], b = in[o + wh], c = in[o + 2 * (size_t)wh];
            if (B.color) color3(a, b, c, true);
            y[o] = a;
            y[o + wh] = b;
            y[o + 2 * (size_t)wh] = c;
            pr[o] = make_float2(0.f, 0.f);
            pr[o + wh] = make_float2(0.f, 0.f);
            pr[o + 2 * (size_t)wh] = make_float2(0.f, 0.f);
        } else {
            y[o] = in[o];
            pr[o] = make_float2(0.f, 0.f);
        }
    }
}

// run_vbm3d's first division (src/vbm3d.cpp:168-170) and the reset of the
// accumulator for step 2.
__global__ void __launch_bounds__(256) batch_mid_kernel(const BatchClip* __restrict__ clips,
                                                       const uint4* __restrict__ chunks)
{
    const uint4 K = chunks[blockIdx.x];
    const BatchClip& B = clips[K.x];
    const unsigned wh = B.wh, C = B.C;
    const float* __restrict__ y = B.y;
    float* __restrict__ bs = B.basic;
    float2* __restrict__ pr = reinterpret_cast<float2*>(B.pair);
    for (unsigned i = threadIdx.x; i < K.z; i += blockDim.x) {
        const size_t pos = (size_t)K.y + i, t = pos / wh, k = pos - t * wh;
        for (unsigned c = 0; c < C; c++) {
            const size_t o = t * C * wh + (size_t)c * wh + k;
            const float2 v = pr[o];
            bs[o] = v.y == 0 ? y[o] : v.x / v.y;
            pr[o] = make_float2(0.f, 0.f);
        }
    }
}

// The second division (src/vbm3d.cpp:198-202) and the inverse colour
// transform of both estimates (src/vbm3d.cpp:356-376).
__global__ void __launch_bounds__(256) batch_final_kernel(const BatchClip* __restrict__ clips,
                                                         const uint4* __restrict__ chunks)
{
    const uint4 K = chunks[blockIdx.x];
    const BatchClip& B = clips[K.x];
    const unsigned wh = B.wh, C = B.C;
    const float* __restrict__ bs = B.basic;
    const float2* __restrict__ pr = reinterpret_cast<const float2*>(B.pair);
    float* __restrict__ ob = B.out_basic;
    float* __restrict__ od = B.out_den;
    for (unsigned i = threadIdx.x; i < K.z; i += blockDim.x) {
        const size_t pos = (size_t)K.y + i, t = pos / wh, k = pos - t * wh;
        const size_t o = t * C * wh + k;
        float d[3], b[3];
        for (unsigned c = 0; c < C; c++) {
            const float2 v = pr[o + (size_t)c * wh];
            b[c] = bs[o + (size_t)c * wh];
            d[c] = v.y == 0 ? b[c] : v.x / v.y;
        }
        if (C == 3 && B.color) {
            color3(d[0], d[1], d[2], false);
            color3(b[0], b[1], b[2], false);
        }
        for (unsigned c = 0; c < C; c++) {
            od[o + (size_t)c * wh] = d[c];
            if (ob) ob[o + (size_t)c * wh] = b[c];
        }
    }
}

// ------------------------------------------------------------- host ---

constexpr int kChunk = 8192;  // pixel positions per elementwise block
constexpr int kSample = 8;    // the autotuner times every 8th item

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

int cuda_fail(cudaError_t e, const char* what)
{
    if (e == cudaErrorMemoryAllocation)
        return fail(VBM3D_ERR_OUT_OF_MEMORY, "%s: %s", what, cudaGetErrorString(e));
    return fail(VBM3D_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define BCK(call)                                              \
    do {                                                       \
        cudaError_t e_ = (call);                               \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call);    \
    } while (0)

struct PhaseCfg {
    int tile;   // refs per work item
    int warps;  // warps per block
};

// Host record of one clip's steps.
struct ClipHost {
    StepHead h[2];
    Layout L[2];
    CompactTables t[2];
    long long nrefs[2];
};

// One kernel launch of a work phase: the clips of one class.
struct WorkLaunch {
    int phase = 0, cls = 0;
    std::vector<int> clips;  // batch indices, in cost order; slot = position
    std::vector<unsigned char> table;  // passed by value: block matching its BmTable, filtering its tables
    int ws = 0;              // per-warp workspace (bm: bytes, filter: floats)
    uint4* d_items = nullptr;
    unsigned nitems = 0;
    size_t cap = 0;
    int grid = 0;
    PhaseCfg cfg{0, 0};      // refs per item and warps per block of this launch
};

// Tuned configurations per batch signature: one per work launch, in phase
// order (the signature fixes the launches).
std::mutex g_tune_mu;
std::map<std::string, std::vector<PhaseCfg>> g_tune_cache;

size_t up256(size_t x) { return (x + 255) & ~size_t(255); }

const void* work_kernel(int phase, int cls)
{
    return phase < 2 ? work_kernel_step1(phase, cls) : work_kernel_step2(phase, cls);
}

}  // namespace batched
}  // namespace vbm3d

struct vbm3d_batch {
    using BatchClip = vbm3d::batched::BatchClip;
    using ClipHost = vbm3d::batched::ClipHost;
    using PhaseCfg = vbm3d::batched::PhaseCfg;
    using WorkLaunch = vbm3d::batched::WorkLaunch;
    static constexpr int kPhases = vbm3d::batched::kPhases;
    int device = 0;
    int sms = 0;
    int nclips = 0;
    std::vector<BatchClip> hc;
    std::vector<ClipHost> ch;
    std::vector<int> order;        // clips by cost, most expensive first
    BatchClip* d_clips = nullptr;
    unsigned char* arena = nullptr;
    size_t arena_bytes = 0;
    size_t pair_bytes = 0;         // the accumulators, at the start of the arena
    std::vector<WorkLaunch> work[kPhases];
    uint4* d_chunks = nullptr;
    unsigned nchunks = 0;
    unsigned* d_heads = nullptr;   // a queue head and a sample head per work launch
    int nheads = 0;
    PhaseCfg cfg[kPhases] = {};
    bool graph = true;
    float tune_ms = 0.f;
    cudaStream_t cs = nullptr;
    cudaGraphExec_t exec = nullptr;
};

namespace vbm3d {
namespace batched {

// Work estimate of one reference of a clip's step, for ordering only.
double ref_cost(const StepHead& P)
{
    const double kk = (double)P.k * P.k * P.C;
    return kk * (P.Ns * P.Ns + 2.0 * P.Nf * P.Nb * P.Npr * P.Npr);
}

int bm_groups_per_warp(int cls);

// Items of one launch: tiles of `tile` consecutive references inside one
// frame (times the groups per warp for block matching: a block's groups
// all take part in an item), clips in cost order.  With stride > 1 only
// every stride-th item is kept (the autotuner's sample).
std::vector<uint4> make_items(const vbm3d_batch& b, const WorkLaunch& w, int tile, int stride)
{
    std::vector<uint4> v;
    const int s = w.phase / 2;
    if (!(w.phase & 1)) tile *= bm_groups_per_warp(w.cls);
    long long n = 0;
    for (size_t slot = 0; slot < w.clips.size(); slot++) {
        const int c = w.clips[slot];
        const StepHead& P = b.ch[c].h[s];
        const long long per_frame = (long long)P.nrows * P.ncols;
        // filtering: rows in bands of band_rows, each band frame by frame
        // (the aggregation order of band_order_ref); block matching: frames
        const int band = (w.phase & 1) && P.band_rows > 0 ? P.band_rows : P.nrows;
        for (int row0 = 0; row0 < P.nrows; row0 += band) {
            const long long r0 = (long long)row0 * P.ncols;
            const long long r1 = (long long)std::min(row0 + band, P.nrows) * P.ncols;
            for (int t = 0; t < P.nframes; t++)
                for (long long r = r0; r < r1; r += tile, n++)
                    if (n % stride == 0)
                        v.push_back(make_uint4((unsigned)c, (unsigned)(t * per_frame + r),
                                               (unsigned)std::min<long long>(tile, r1 - r), (unsigned)slot));
        }
    }
    return v;
}

int upload_items(WorkLaunch& w, const std::vector<uint4>& v, cudaStream_t s)
{
    if (v.size() > w.cap) {
        if (w.d_items) BCK(cudaFree(w.d_items));
        w.d_items = nullptr;
        BCK(cudaMalloc(&w.d_items, v.size() * sizeof(uint4)));
        w.cap = v.size();
    }
    if (!v.empty()) BCK(cudaMemcpyAsync(w.d_items, v.data(), v.size() * sizeof(uint4), cudaMemcpyHostToDevice, s));
    BCK(cudaStreamSynchronize(s));  // v is a temporary
    w.nitems = (unsigned)v.size();
    return VBM3D_OK;
}

int upload_phase(vbm3d_batch& b, int phase, int stride, cudaStream_t s)
{
    for (WorkLaunch& w : b.work[phase]) {
        int rc = upload_items(w, make_items(b, w, w.cfg.tile, stride), s);
        if (rc) return rc;
    }
    return VBM3D_OK;
}

// Block matching: a reference per half warp for one-channel classes (even
// class numbers), per warp otherwise (batch_bm_kernel's G).
int bm_groups_per_warp(int cls) { return (cls & 1) ? 1 : 2; }

size_t launch_smem(const WorkLaunch& w, int warps)
{
    return (w.phase & 1) ? (size_t)warps * w.ws * sizeof(float)
                         : (size_t)warps * bm_groups_per_warp(w.cls) * w.ws;
}

// Grid of a launch: resident blocks per SM x SMs.
int launch_grid(const vbm3d_batch& b, const WorkLaunch& w, int& grid)
{
    const int warps = w.cfg.warps;
    const void* k = work_kernel(w.phase, w.cls);
    const size_t smem = launch_smem(w, warps);
    BCK(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    BCK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, warps * 32, smem));
    if (per_sm <= 0)
        return fail(VBM3D_ERR_UNSUPPORTED, "batched kernel of phase %d does not fit on an SM (%zu B)", w.phase, smem);
    grid = per_sm * b.sms;
    return VBM3D_OK;
}

int phase_grids(vbm3d_batch& b, int phase)
{
    for (WorkLaunch& w : b.work[phase]) {
        int rc = launch_grid(b, w, w.grid);
        if (rc) return rc;
    }
    return VBM3D_OK;
}

// One work launch, pulling from queue head h.
cudaError_t launch_work(const vbm3d_batch& b, const WorkLaunch& w, unsigned* h, cudaStream_t s)
{
    const int warps = w.cfg.warps;
    if (!w.nitems) return cudaSuccess;
    const BatchClip* clips = b.d_clips;
    const uint4* items = w.d_items;
    unsigned n = w.nitems;
    int ws = w.ws;
    void* args[] = {&clips, &items, &n, &h, &ws, const_cast<unsigned char*>(w.table.data())};
    return cudaLaunchKernel(work_kernel(w.phase, w.cls), dim3(w.grid), dim3(warps * 32), args, launch_smem(w, warps),
                            s);
}

// The launches of one phase, launch i pulling from heads[i].
cudaError_t launch_phase(const vbm3d_batch& b, int phase, unsigned* heads, cudaStream_t s)
{
    for (size_t i = 0; i < b.work[phase].size(); i++) {
        cudaError_t e = launch_work(b, b.work[phase][i], heads + i, s);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// First head of a phase's launches: queue heads in [0, n), sample heads in
// [n, 2n), n = b.nheads / 2.
unsigned* phase_heads(const vbm3d_batch& b, int phase, bool sample)
{
    int off = 0;
    for (int p = 0; p < phase; p++) off += (int)b.work[p].size();
    return b.d_heads + off + (sample ? b.nheads / 2 : 0);
}

cudaError_t launch_elementwise(const vbm3d_batch& b, int which, cudaStream_t s)
{
    if (!b.nchunks) return cudaSuccess;
    if (which == 0) batch_prep_kernel<<<b.nchunks, 256, 0, s>>>(b.d_clips, b.d_chunks);
    else if (which == 1) batch_mid_kernel<<<b.nchunks, 256, 0, s>>>(b.d_clips, b.d_chunks);
    else batch_final_kernel<<<b.nchunks, 256, 0, s>>>(b.d_clips, b.d_chunks);
    return cudaGetLastError();
}

// The whole batch on stream s with the chosen configuration.
int enqueue_all(const vbm3d_batch& b, cudaStream_t s)
{
    BCK(cudaMemsetAsync(b.d_heads, 0, (b.nheads / 2) * sizeof(unsigned), s));
    BCK(launch_elementwise(b, 0, s));
    for (int ph = 0; ph < kPhases; ph++) {
        BCK(launch_phase(b, ph, phase_heads(b, ph, false), s));
        if (ph == 1) BCK(launch_elementwise(b, 1, s));
    }
    BCK(launch_elementwise(b, 2, s));
    return VBM3D_OK;
}

std::string signature(const vbm3d_batch& b)
{
    std::string sig = std::to_string(b.device) + ":";
    char buf[160];
    for (int c : b.order) {
        const StepHead& P1 = b.ch[c].h[0];
        const StepHead& P2 = b.ch[c].h[1];
        snprintf(buf, sizeof buf, "%dx%dx%dx%d/%d,%d,%d,%d,%d,%d,%d/%d,%d,%d,%d,%d,%d,%d;", P1.W, P1.H, P1.F, P1.C,
                 P1.k, P1.p, P1.N, P1.Ns, P1.Npr, P1.Nb, P1.Nf, P2.k, P2.p, P2.N, P2.Ns, P2.Npr, P2.Nb, P2.Nf);
        sig += buf;
    }
    return sig;
}

// Times one candidate configuration (set in every launch of the phase) on
// the sampled items uploaded for it: ms[i] for launch i, in ms.
int time_candidate(vbm3d_batch& b, int phase, std::vector<float>& ms)
{
    int rc = phase_grids(b, phase);
    if (rc) return rc;
    const size_t n = b.work[phase].size();
    std::vector<cudaEvent_t> ev(n + 1);
    for (auto& e : ev) BCK(cudaEventCreate(&e));
    unsigned* h = phase_heads(b, phase, true);
    BCK(cudaMemsetAsync(h, 0, n * sizeof(unsigned), b.cs));
    for (size_t i = 0; i < n; i++) {
        BCK(cudaEventRecord(ev[i], b.cs));
        BCK(launch_work(b, b.work[phase][i], h + i, b.cs));
    }
    BCK(cudaEventRecord(ev[n], b.cs));
    BCK(cudaEventSynchronize(ev[n]));
    ms.assign(n, 0.f);
    for (size_t i = 0; i < n; i++) BCK(cudaEventElapsedTime(&ms[i], ev[i], ev[i + 1]));
    for (auto& e : ev) cudaEventDestroy(e);
    return VBM3D_OK;
}

// The configuration reported for a phase: that of its launch with the most
// reference patches.
PhaseCfg phase_cfg(const vbm3d_batch& b, int phase)
{
    PhaseCfg c{0, 0};
    long long most = -1;
    for (const WorkLaunch& w : b.work[phase]) {
        long long n = 0;
        for (int i : w.clips) n += b.ch[i].nrefs[phase / 2];
        if (n > most) {
            most = n;
            c = w.cfg;
        }
    }
    return c;
}

// Uploads every phase's work items and sizes its grids.  Phases whose
// configuration is not fixed (by the caller or the cache) are first tuned
// during one eager pass over the batch, each on a sample of its items with
// the inputs of the previous phases in place; every launch (class) of the
// phase keeps the candidate that was fastest for it.
int tune_and_prepare(vbm3d_batch& b, const bool fixed[kPhases])
{
    // candidates (refs per item, warps per block): one or two references
    // per warp and item for block matching, two to eight for filtering
    static const PhaseCfg cand_bm[] = {{4, 4}, {8, 4}, {8, 8}, {16, 8}};
    static const PhaseCfg cand_f[] = {{16, 8}, {32, 8}, {16, 4}, {8, 4}};
    constexpr int kCandBm = 4, kCandF = 4;
    bool any = false;
    for (int ph = 0; ph < kPhases; ph++) any = any || !fixed[ph];
    cudaStream_t s = b.cs;
    if (any) {
        BCK(cudaMemsetAsync(b.d_heads, 0, b.nheads * sizeof(unsigned), s));
        BCK(launch_elementwise(b, 0, s));
    }
    for (int ph = 0; ph < kPhases; ph++) {
        int rc;
        std::vector<WorkLaunch>& ws = b.work[ph];
        if (!fixed[ph]) {
            std::vector<float> best(ws.size(), 3.0e38f), ms;
            std::vector<PhaseCfg> pick(ws.size(), PhaseCfg{0, 0});
            const PhaseCfg* cand = (ph & 1) ? cand_f : cand_bm;
            int uploaded = 0;
            for (int ci = 0; ci < ((ph & 1) ? kCandF : kCandBm); ci++) {
                const PhaseCfg c = cand[ci];
                for (WorkLaunch& w : ws) w.cfg = c;
                if (c.tile != uploaded) {
                    if ((rc = upload_phase(b, ph, kSample, s))) return rc;
                    uploaded = c.tile;
                    if ((rc = time_candidate(b, ph, ms))) return rc;  // warm-up on the same sample
                }
                if ((rc = time_candidate(b, ph, ms))) return rc;
                for (size_t i = 0; i < ws.size(); i++)
                    if (ms[i] < best[i]) {
                        best[i] = ms[i];
                        pick[i] = c;
                    }
            }
            for (size_t i = 0; i < ws.size(); i++) ws[i].cfg = pick[i];
            // the sampled filter runs added into the accumulators
            if (ph & 1) BCK(cudaMemsetAsync(b.arena, 0, b.pair_bytes, s));
        }
        b.cfg[ph] = phase_cfg(b, ph);
        if ((rc = upload_phase(b, ph, 1, s))) return rc;
        if ((rc = phase_grids(b, ph))) return rc;
        if (any) {
            BCK(launch_phase(b, ph, phase_heads(b, ph, false), s));
            if (ph == 1) BCK(launch_elementwise(b, 1, s));
        }
    }
    if (any) BCK(launch_elementwise(b, 2, s));
    BCK(cudaStreamSynchronize(s));
    return VBM3D_OK;
}

void release(vbm3d_batch* b)
{
    if (!b) return;
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(b->device);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->cs) cudaStreamDestroy(b->cs);
    for (auto& ph : b->work)
        for (auto& w : ph)
            if (w.d_items) cudaFree(w.d_items);
    if (b->d_chunks) cudaFree(b->d_chunks);
    if (b->d_heads) cudaFree(b->d_heads);
    if (b->d_clips) cudaFree(b->d_clips);
    if (b->arena) cudaFree(b->arena);
    cudaSetDevice(cur);
    delete b;
}

// The work launches of every phase: one per class present, its clips in
// cost order.
void plan_launches(vbm3d_batch& b)
{
    for (int ph = 0; ph < kPhases; ph++) {
        const int s = ph / 2;
        for (int cls = 0; cls < kClasses; cls++) {
            WorkLaunch w;
            w.phase = ph;
            w.cls = cls;
            for (int c : b.order) {
                const StepHead& P = b.ch[c].h[s];
                if (class_of(ph, P) != cls) continue;
                // a full table, or (filtering) transform tables other than the
                // launch's: next launch
                const bool next = (int)w.clips.size() == kTableClips ||
                                  ((ph & 1) && !w.clips.empty() &&
                                   memcmp(&b.ch[w.clips[0]].t[s], &b.ch[c].t[s], sizeof(CompactTables)) != 0);
                if (next) {
                    b.work[ph].push_back(w);
                    w.clips.clear();
                    w.ws = 0;
                }
                w.clips.push_back(c);
                if (ph & 1) {
                    // slices at the stride of the class's lanes per slice
                    const int sl = std::max(P.k * P.k + 1, slice_stride(P.k, P.C == 1 ? 4 : 1));
                    w.ws = std::max(w.ws, (kMaxN + (s == 0 ? 1 : 2) * P.C * P.N * sl + 3) & ~3);
                }
                else w.ws = std::max(w.ws, (b.ch[c].L[s].warp_bytes + 15) & ~15);
            }
            if (!w.clips.empty()) b.work[ph].push_back(std::move(w));
        }
    }
    int n = 0;
    for (auto& ph : b.work) n += (int)ph.size();
    b.nheads = 2 * n;
}

// Validation and host-side set-up of the clip descriptors; no CUDA call.
int describe(const vbm3d_clip* clips, int nclips, int color_space, vbm3d_batch& b)
{
    if (!clips || nclips <= 0) return fail(VBM3D_ERR_INVALID_ARGUMENT, "empty batch");
    b.nclips = nclips;
    b.hc.assign(nclips, BatchClip{});
    b.ch.assign(nclips, ClipHost{});
    for (int i = 0; i < nclips; i++) {
        const vbm3d_clip& c = clips[i];
        if (!c.noisy || !c.denoised) return fail(VBM3D_ERR_INVALID_ARGUMENT, "clip %d: NULL video pointer", i);
        vbm3d_params dp[2];
        const vbm3d_params* pp[2] = {c.prms_1, c.prms_2};
        for (int s = 0; s < 2; s++) {
            if (!pp[s]) {
                vbm3d_default_params(s + 1, c.sigma, &dp[s]);
                pp[s] = &dp[s];
            }
            StepParams P;
            int rc = build_step_params(pp[s], c.dims, c.sigma, color_space, P);
            if (rc) return rc;
            const Layout L = bm2_layout(P);
            if (!((P.k == 7 || P.k == 8) && P.kt == 1 && P.N <= 8 && L.warp_bytes > 0))
                return fail(VBM3D_ERR_UNSUPPORTED,
                            "clip %d step %d: the batched kernels take k in {7, 8}, kt == 1, N <= 8 and search "
                            "windows whose staged layout fits 24 KB (use vbm3d_gpu_run for this clip)",
                            i, s + 1);
            ClipHost& h = b.ch[i];
            h.h[s] = static_cast<const StepHead&>(P);
            h.L[s] = L;
            const int kk = P.k * P.k;
            for (int e = 0; e < kTab; e++) {
                h.t[s].kaiser[e] = e < kk ? P.kaiser[e] : 0.f;
                h.t[s].fwd[e] = e < kk ? P.fwd[e] : 0.f;
                h.t[s].inv[e] = e < kk ? P.inv[e] : 0.f;
                h.t[s].cn[e] = e < kk ? P.cn[e] : 0.f;
                h.t[s].cni[e] = e < kk ? P.cni[e] : 0.f;
            }
            h.nrefs[s] = P.nrefs;
        }
        BatchClip& h = b.hc[i];
        h.in = c.noisy;
        h.fflow = c.fflow;
        h.bflow = c.bflow;
        h.out_basic = c.basic;
        h.out_den = c.denoised;
        h.wh = c.dims.width * c.dims.height;
        h.C = c.dims.channels;
        h.color = (color_space && c.dims.channels == 3) ? 1u : 0u;
    }
    b.order.resize(nclips);
    for (int i = 0; i < nclips; i++) b.order[i] = i;
    std::stable_sort(b.order.begin(), b.order.end(),
                     [&](int a, int c) { return ref_cost(b.ch[a].h[1]) > ref_cost(b.ch[c].h[1]); });
    plan_launches(b);
    return VBM3D_OK;
}

// Device buffers: one arena for every clip's working videos and tables,
// the accumulators first so that one memset clears them all.
int allocate(vbm3d_batch& b, cudaStream_t s)
{
    std::vector<size_t> off(b.nclips * 5);
    size_t total = 0;
    for (int i = 0; i < b.nclips; i++) {
        const StepHead& P1 = b.ch[i].h[0];
        off[5 * i + 0] = total;
        total += up256(2 * (size_t)P1.whc * P1.F * sizeof(float));
    }
    b.pair_bytes = total;
    for (int i = 0; i < b.nclips; i++) {
        const ClipHost& h = b.ch[i];
        const size_t n = (size_t)h.h[0].whc * h.h[0].F;
        const size_t nidx = std::max((size_t)h.nrefs[0] * h.h[0].N, (size_t)h.nrefs[1] * h.h[1].N);
        const size_t nref = std::max((size_t)h.nrefs[0], (size_t)h.nrefs[1]);
        off[5 * i + 1] = total;
        total += up256(n * sizeof(float));
        off[5 * i + 2] = total;
        total += up256(n * sizeof(float));
        off[5 * i + 3] = total;
        total += up256(nidx * sizeof(unsigned));
        off[5 * i + 4] = total;
        total += up256(nref * sizeof(unsigned));
    }
    BCK(cudaMalloc(&b.arena, total));
    b.arena_bytes = total;
    for (int i = 0; i < b.nclips; i++) {
        BatchClip& h = b.hc[i];
        h.pair = reinterpret_cast<float*>(b.arena + off[5 * i + 0]);
        h.y = reinterpret_cast<float*>(b.arena + off[5 * i + 1]);
        h.basic = reinterpret_cast<float*>(b.arena + off[5 * i + 2]);
        h.tab_idx = reinterpret_cast<unsigned*>(b.arena + off[5 * i + 3]);
        h.tab_nsx = reinterpret_cast<unsigned*>(b.arena + off[5 * i + 4]);
    }
    // filtering tables: the transform tables every clip of the launch
    // shares, the parameters and buffers of each of its clips
    for (int ph = 1; ph < kPhases; ph += 2)
        for (WorkLaunch& w : b.work[ph]) {
            w.table.assign(sizeof(FilterTable), 0);
            FilterTable* t = reinterpret_cast<FilterTable*>(w.table.data());
            t->t = b.ch[w.clips[0]].t[ph / 2];
            for (size_t i = 0; i < w.clips.size(); i++) {
                const int c = w.clips[i];
                t->h[i] = b.ch[c].h[ph / 2];
                t->pair[i] = b.hc[c].pair;
                t->noisy[i] = b.hc[c].y;
                t->basic[i] = b.hc[c].basic;
                t->tab_idx[i] = b.hc[c].tab_idx;
                t->tab_nsx[i] = b.hc[c].tab_nsx;
            }
        }
    // block-matching tables: parameters and buffers of each launch's clips
    for (int ph = 0; ph < kPhases; ph += 2)
        for (WorkLaunch& w : b.work[ph]) {
            w.table.assign(sizeof(BmTable), 0);
            BmTable* t = reinterpret_cast<BmTable*>(w.table.data());
            for (size_t i = 0; i < w.clips.size(); i++) {
                const int c = w.clips[i];
                t->h[i] = b.ch[c].h[ph / 2];
                t->L[i] = b.ch[c].L[ph / 2];
                t->vid[i] = ph == 0 ? b.hc[c].y : b.hc[c].basic;
                t->fflow[i] = b.hc[c].fflow;
                t->bflow[i] = b.hc[c].bflow;
                t->tab_idx[i] = b.hc[c].tab_idx;
                t->tab_nsx[i] = b.hc[c].tab_nsx;
            }
        }
    BCK(cudaMalloc(&b.d_clips, b.hc.size() * sizeof(BatchClip)));
    BCK(cudaMemcpyAsync(b.d_clips, b.hc.data(), b.hc.size() * sizeof(BatchClip), cudaMemcpyHostToDevice, s));
    std::vector<uint4> ch;
    for (int c : b.order) {
        const StepHead& P = b.ch[c].h[0];
        const size_t npos = (size_t)P.wh * P.F;
        for (size_t p = 0; p < npos; p += kChunk)
            ch.push_back(make_uint4((unsigned)c, (unsigned)p, (unsigned)std::min<size_t>(kChunk, npos - p), 0u));
    }
    b.nchunks = (unsigned)ch.size();
    BCK(cudaMalloc(&b.d_chunks, std::max<size_t>(ch.size(), 1) * sizeof(uint4)));
    if (!ch.empty())
        BCK(cudaMemcpyAsync(b.d_chunks, ch.data(), ch.size() * sizeof(uint4), cudaMemcpyHostToDevice, s));
    BCK(cudaMalloc(&b.d_heads, std::max(b.nheads, 1) * sizeof(unsigned)));
    BCK(cudaStreamSynchronize(s));
    return VBM3D_OK;
}

void config_of(const vbm3d_batch& b, vbm3d_batch_config* c)
{
    memset(c, 0, sizeof *c);
    c->bm1_tile = b.cfg[0].tile;
    c->bm1_warps = b.cfg[0].warps;
    c->filter1_tile = b.cfg[1].tile;
    c->filter1_warps = b.cfg[1].warps;
    c->bm2_tile = b.cfg[2].tile;
    c->bm2_warps = b.cfg[2].warps;
    c->filter2_tile = b.cfg[3].tile;
    c->filter2_warps = b.cfg[3].warps;
    c->no_graph = b.graph ? 0 : 1;
    c->tune_ms = b.tune_ms;
    for (auto& ph : b.work)
        for (auto& w : ph) c->work_items += w.nitems;
    c->device_bytes = b.arena_bytes;
}

}  // namespace batched
}  // namespace vbm3d

using namespace vbm3d::batched;

extern "C" {

int vbm3d_batch_create(const vbm3d_clip* clips, int nclips, int color_space, const vbm3d_batch_config* config,
                       vbm3d_batch** out, void* stream)
{
    if (!out) return fail(VBM3D_ERR_INVALID_ARGUMENT, "NULL output handle");
    *out = nullptr;
    vbm3d_batch* b = new vbm3d_batch;
    int rc = describe(clips, nclips, color_space, *b);
    if (rc) {
        delete b;
        return rc;
    }
    if (config) {
        const int v[kPhases][2] = {{config->bm1_tile, config->bm1_warps},
                                   {config->filter1_tile, config->filter1_warps},
                                   {config->bm2_tile, config->bm2_warps},
                                   {config->filter2_tile, config->filter2_warps}};
        for (int ph = 0; ph < kPhases; ph++) {
            const int t = v[ph][0], w = v[ph][1];
            if ((t != 0) != (w != 0) || t < 0 || t > 4096 || !(w == 0 || w == 1 || w == 2 || w == 4 || w == 8)) {
                delete b;
                return fail(VBM3D_ERR_INVALID_ARGUMENT,
                            "phase %d: tile and warps must both be 0 (autotune) or both set, tile <= 4096, warps in "
                            "{1, 2, 4, 8}",
                            ph);
            }
            b->cfg[ph] = PhaseCfg{t, w};
        }
        b->graph = config->no_graph == 0;
    }
    cudaError_t e = cudaGetDevice(&b->device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, b->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->cs, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        release(b);
        return cuda_fail(e, "batch set-up");
    }
    if ((rc = allocate(*b, b->cs))) {
        release(b);
        return rc;
    }
    // the clips' inputs may still be written on the caller's stream
    if ((e = cudaStreamSynchronize((cudaStream_t)stream)) != cudaSuccess) {
        release(b);
        return cuda_fail(e, "cudaStreamSynchronize");
    }
    // per phase: the caller's configuration for all its launches, else the
    // cached per-launch choices of an earlier batch of the same signature,
    // else tuning
    bool fixed[kPhases];
    const std::string sig = signature(*b);
    {
        std::lock_guard<std::mutex> g(g_tune_mu);
        auto it = g_tune_cache.find(sig);
        size_t k = 0;
        for (int ph = 0; ph < kPhases; ph++) {
            fixed[ph] = b->cfg[ph].tile != 0 || it != g_tune_cache.end();
            for (WorkLaunch& w : b->work[ph]) {
                w.cfg = b->cfg[ph].tile != 0 ? b->cfg[ph] : it != g_tune_cache.end() ? it->second[k] : PhaseCfg{0, 0};
                k++;
            }
        }
    }
    const auto t0 = std::chrono::steady_clock::now();
    if ((rc = tune_and_prepare(*b, fixed))) {
        release(b);
        return rc;
    }
    b->tune_ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
    {
        std::lock_guard<std::mutex> g(g_tune_mu);
        std::vector<PhaseCfg> v;
        for (int ph = 0; ph < kPhases; ph++)
            for (const WorkLaunch& w : b->work[ph]) v.push_back(w.cfg);
        g_tune_cache[sig] = v;
    }
    if (b->graph) {
        cudaGraph_t g = nullptr;
        e = cudaStreamBeginCapture(b->cs, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            rc = enqueue_all(*b, b->cs);
            e = cudaStreamEndCapture(b->cs, &g);
            if (rc == VBM3D_OK && e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, g, 0);
            if (g) cudaGraphDestroy(g);
        }
        if (rc || e != cudaSuccess) {
            release(b);
            return rc ? rc : cuda_fail(e, "graph capture");
        }
    }
    *out = b;
    return VBM3D_OK;
}

int vbm3d_batch_run(vbm3d_batch* b, void* stream)
{
    if (!b) return fail(VBM3D_ERR_INVALID_ARGUMENT, "NULL batch");
    int cur = -1;
    BCK(cudaGetDevice(&cur));
    if (cur != b->device) return fail(VBM3D_ERR_INVALID_ARGUMENT, "batch was created on device %d", b->device);
    cudaStream_t s = (cudaStream_t)stream;
    if (b->exec) {
        BCK(cudaGraphLaunch(b->exec, s));
        return VBM3D_OK;
    }
    return enqueue_all(*b, s);
}

int vbm3d_batch_get_config(const vbm3d_batch* b, vbm3d_batch_config* c)
{
    if (!b || !c) return fail(VBM3D_ERR_INVALID_ARGUMENT, "NULL argument");
    config_of(*b, c);
    return VBM3D_OK;
}

int vbm3d_batch_profile(vbm3d_batch* b, void* stream, vbm3d_batch_launch* out, int cap, int* count)
{
    if (!b || !count || (cap > 0 && !out)) return fail(VBM3D_ERR_INVALID_ARGUMENT, "NULL argument");
    int n = 0;
    for (auto& ph : b->work) n += (int)ph.size();
    *count = n;
    if (cap < n) return fail(VBM3D_ERR_INVALID_ARGUMENT, "%d work launches, room for %d", n, cap);
    cudaStream_t s = (cudaStream_t)stream;
    std::vector<cudaEvent_t> ev(n + 1);
    for (auto& e : ev) BCK(cudaEventCreate(&e));
    BCK(cudaMemsetAsync(b->d_heads, 0, (b->nheads / 2) * sizeof(unsigned), s));
    BCK(launch_elementwise(*b, 0, s));
    int i = 0;
    for (int ph = 0; ph < kPhases; ph++) {
        unsigned* heads = phase_heads(*b, ph, false);
        for (size_t j = 0; j < b->work[ph].size(); j++, i++) {
            const WorkLaunch& w = b->work[ph][j];
            BCK(cudaEventRecord(ev[i], s));
            BCK(launch_work(*b, w, heads + j, s));
            BCK(cudaEventRecord(ev[i + 1], s));
            vbm3d_batch_launch& o = out[i];
            memset(&o, 0, sizeof o);
            o.phase = ph;
            const vbm3d::StepHead& P = b->ch[w.clips[0]].h[ph / 2];
            o.k = P.k;
            o.channels = (ph & 1) ? 0 : P.C;
            o.clips = (int)w.clips.size();
            o.items = w.nitems;
            for (int c : w.clips) o.refs += (unsigned long long)b->ch[c].nrefs[ph / 2];
            o.tile = w.cfg.tile;
            o.warps = w.cfg.warps;
            o.grid = w.grid;
        }
        if (ph == 1) BCK(launch_elementwise(*b, 1, s));
    }
    BCK(launch_elementwise(*b, 2, s));
    BCK(cudaEventSynchronize(ev[n]));
    for (int j = 0; j < n; j++) BCK(cudaEventElapsedTime(&out[j].ms, ev[j], ev[j + 1]));
    for (auto& e : ev) cudaEventDestroy(e);
    return VBM3D_OK;
}

void vbm3d_batch_destroy(vbm3d_batch* b) { release(b); }

}  // extern "C"
