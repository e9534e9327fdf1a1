// Allocation-free variant of step 1 (hard thresholding).
//
// vbm3d_gpu_step1 keeps its block-matching table (the matches of every
// reference patch, handed from the matching kernel to the filtering kernel)
// in memory it allocates from a stream-ordered pool.  Some callers cannot
// let a library allocate device memory: plug-in hosts (video editors,
// broadcast and capture pipelines) that own every device byte through their
// own allocator, real-time pipelines that forbid any allocation once they
// are running, and processes under a strict per-tenant memory budget.  For
// them vbm3d_gpu_step1_noalloc runs the same two kernels with the table in
// the fixed device array below and calls no cudaMalloc, cudaFree or other
// allocating routine.
//
// The array is a file-scope __device__ object: every GPU on which this
// library's module is loaded holds it (32 MiB) until the process exits.
// The driver reserves it when it loads the module: at context creation
// when module loading is eager (CUDA_MODULE_LOADING=EAGER), at the first
// use of the module (the first call of this entry point, whose address
// lookup loads it) under lazy loading, the default.  A caller with a strict
// memory budget makes one call at start-up.  Host code cannot use the
// array's name as a device address (in host code it names a host-side
// shadow); its device address is looked up with cudaGetSymbolAddress once
// per device context, with that device current, and passed to the kernels.
// The lookup is cached per context (the driver's unique context id), so a
// device reset or a re-created primary context, which reloads the module
// at a new address, triggers a new lookup.
#include <cstring>
#include <mutex>
#include <string>

#include "common.cuh"
#include "../../include/vbm3d_gb300.h"

namespace vbm3d {
cudaError_t launch_bm(const StepParams& P, const float* vid, const float* fflow, const float* bflow,
                      unsigned* out_idx, float* out_dist, unsigned* out_nsimp, unsigned* out_nsx,
                      long long count, cudaStream_t stream, unsigned long long* out_count);
cudaError_t launch_filter(int step, const StepParams& P, const float* noisy, const float* basic,
                          const float* fflow, const unsigned* tab_idx, const unsigned* tab_nsx, float* num,
                          float* den, float* pair, long long count, cudaStream_t stream);
int build_step_params(const vbm3d_params* p, vbm3d_dims d, float sigma, int color_space, StepParams& P);
void set_last_error(int status, const char* msg);
}  // namespace vbm3d

namespace {

// 32 MiB: 8 Mi table words.  A step needs nrefs * (N + 1) words (N match
// indices and one group size per reference patch).
constexpr size_t kNoAllocTableWords = (size_t)8 << 20;
__device__ __align__(256) unsigned g_noalloc_table[kNoAllocTableWords];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned* g_table_ptr[kMaxDevices] = {};
unsigned long long g_table_ctx[kMaxDevices] = {};  // context id of each cached address

// The driver's id of the calling thread's current context (cuCtxGetCurrent,
// cuCtxGetId through the runtime's driver entry points, so that the
// library needs no link against the driver library).
cudaError_t current_context_id(unsigned long long* id)
{
    typedef int (*GetCurrentFn)(void**);
    typedef int (*GetIdFn)(void*, unsigned long long*);
    static GetCurrentFn get_current = nullptr;
    static GetIdFn get_id = nullptr;
    if (!get_current || !get_id) {
        void* f1 = nullptr;
        void* f2 = nullptr;
        cudaDriverEntryPointQueryResult q1, q2;
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1);
        if (e == cudaSuccess) e = cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2);
        if (e != cudaSuccess) return e;
        if (q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
            return cudaErrorNotSupported;
        get_current = reinterpret_cast<GetCurrentFn>(f1);
        get_id = reinterpret_cast<GetIdFn>(f2);
    }
    void* ctx = nullptr;
    if (get_current(&ctx) != 0) return cudaErrorDeviceUninitialized;
    if (!ctx) {
        // no context yet on this thread: the runtime's first call would make
        // the device's primary context current; cudaSetDevice does that now
        int dev = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaSetDevice(dev);
        if (e != cudaSuccess) return e;
        if (get_current(&ctx) != 0 || !ctx) return cudaErrorDeviceUninitialized;
    }
    return get_id(ctx, id) == 0 ? cudaSuccess : cudaErrorDeviceUninitialized;
}

// Looks up the device address of g_noalloc_table on the current device,
// once per device context (the first call in a context performs it).
int table_for_current_device(unsigned** out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    unsigned long long ctx = 0;
    if (e == cudaSuccess) e = current_context_id(&ctx);
    if (e != cudaSuccess) {
        vbm3d::set_last_error(VBM3D_ERR_CUDA, cudaGetErrorString(e));
        return VBM3D_ERR_CUDA;
    }
    if (dev < 0 || dev >= kMaxDevices) {
        vbm3d::set_last_error(VBM3D_ERR_UNSUPPORTED, "device ordinal above 63");
        return VBM3D_ERR_UNSUPPORTED;
    }
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_table_ptr[dev] || g_table_ctx[dev] != ctx) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_table);
        if (e != cudaSuccess || !p) {
            vbm3d::set_last_error(VBM3D_ERR_CUDA, e != cudaSuccess ? cudaGetErrorString(e)
                                                                  : "cudaGetSymbolAddress returned NULL");
            return VBM3D_ERR_CUDA;
        }
        g_table_ptr[dev] = static_cast<unsigned*>(p);
        g_table_ctx[dev] = ctx;
    }
    *out = g_table_ptr[dev];
    return VBM3D_OK;
}

}  // namespace

extern "C" int vbm3d_gpu_step1_noalloc(const vbm3d_params* prms, const float* noisy, const float* fflow,
                                       const float* bflow, vbm3d_dims dims, float sigma, int color_space,
                                       float* numerator, float* denominator, void* stream)
{
    if (!noisy || !numerator || !denominator) {
        vbm3d::set_last_error(VBM3D_ERR_INVALID_ARGUMENT, "NULL video pointer");
        return VBM3D_ERR_INVALID_ARGUMENT;
    }
    vbm3d::StepParams P;
    int rc = vbm3d::build_step_params(prms, dims, sigma, color_space, P);
    if (rc) return rc;
    const unsigned long long words = (unsigned long long)P.nrefs * (P.N + 1);
    if (words > kNoAllocTableWords) {
        char msg[256];
        snprintf(msg, sizeof msg,
                 "vbm3d_gpu_step1_noalloc: %lld reference patches x (N + 1) = %llu table words exceed the "
                 "fixed table of %zu words (32 MiB); use vbm3d_gpu_step1 or fewer frames per call",
                 P.nrefs, words, kNoAllocTableWords);
        vbm3d::set_last_error(VBM3D_ERR_UNSUPPORTED, msg);
        return VBM3D_ERR_UNSUPPORTED;
    }
    unsigned* table = nullptr;
    if ((rc = table_for_current_device(&table))) return rc;
    // Every table word a kernel reads is written first by the matching
    // kernel of the same call, so nothing needs clearing here.
    unsigned* tab_idx = table;
    unsigned* tab_nsx = table + (size_t)P.nrefs * P.N;
    cudaStream_t s = (cudaStream_t)stream;
    const size_t n = (size_t)P.whc * P.F;
    cudaError_t e = cudaMemsetAsync(numerator, 0, n * sizeof(float), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(denominator, 0, n * sizeof(float), s);
    if (e == cudaSuccess) e = vbm3d::launch_bm(P, noisy, fflow, bflow, tab_idx, nullptr, nullptr, tab_nsx, P.nrefs, s,
                                               nullptr);
    if (e == cudaSuccess)
        e = vbm3d::launch_filter(1, P, noisy, nullptr, fflow, tab_idx, tab_nsx, numerator, denominator, nullptr,
                                 P.nrefs, s);
    if (e != cudaSuccess) {
        vbm3d::set_last_error(VBM3D_ERR_CUDA, cudaGetErrorString(e));
        return VBM3D_ERR_CUDA;
    }
    return VBM3D_OK;
}
