// Shared definitions of the GB300 VBM3D kernels.
//
// Video layout (the reference's VideoSize::index, src/Utilities/LibVideoT.hpp:88-92):
//   index(x, y, t, c) = t*W*H*C + c*W*H + y*W + x, float32.
// A patch is named by the index of its top-left pixel in channel 0, exactly
// as the reference names it (src/vbm3d.cpp:546, :1062).
//
// This file is compiled with --fmad=false: every a*b+c written in the
// kernels rounds the product and the sum separately, as the reference's C++
// does when built without fast-math, so block-matching distances, the
// bior1.5 passes and the shrinkage decisions reproduce the reference's float
// arithmetic operation by operation.  FMAs are written explicitly
// (__fmaf_rn) only where the reference's value is not reproducible anyway
// (the DCT, whose reference value comes from FFTW's own float codelets).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace vbm3d {

constexpr int kMaxK = 16;        // patch side
constexpr int kMaxN = 32;        // similar patches per group
constexpr int kMaxNb = 8;        // matches kept per frame
constexpr int kMaxWin = 15;      // search window side (Ns, Npr)
constexpr int kMaxNf = 16;       // frames searched each way
constexpr int kMaxC = 3;         // channels
constexpr int kMaxKt = 4;        // temporal patch size
constexpr int kSlots = 8;        // window candidates per lane: 32*8 >= 15*15
constexpr unsigned kFull = 0xffffffffu;

// bior1.5 / DCT codes of the reference (src/vbm3d.cpp:34-37).
constexpr int kDCT = 0;
constexpr int kBIOR = 1;
constexpr int kHADAMARD = 2;

// sqrt(1/2) as the reference's double literal SQRT2_INV
// (src/vbm3d.cpp:33), split into a float head and a float tail so that
// fmaf(s, kS2iHi, s * kS2iLo) rounds s * SQRT2_INV to float the way the
// reference's (float)((double)s * SQRT2_INV) does.
constexpr float kS2iHi = 0.70710676908493042f;          // float(0.7071067811865475)
constexpr float kS2iLo = 1.2101617485882343e-08f;       // float(0.7071067811865475 - kS2iHi)

// The scalar part of a step's parameters: everything block matching
// needs, and all but the transform tables of the filter.
struct StepHead {
    // video
    int W, H, F, C;
    unsigned wh, whc;
    // algorithm parameters (struct Parameters, src/parameters.h:21-58)
    int k, kt, p, N, Nf, Ns, Npr, Nb, T2D, T3D, mc;
    float tau, dbias, lambda3D;
    // reference grid (ind_initialize, src/Utilities/Utilities.cpp:400-415)
    int nrows, ncols, nframes;
    long long nrefs;
    long long ref_base;         // first reference of this launch (chunking)
    // noise per channel (estimate_sigma)
    float sigma[kMaxC];
    // block-matching shared-memory layout (floats / pairs per warp)
    int bm_list_cap, bm_best_cap, bm_win_cap, bm_warp_bytes;
    // -0.0f, read by the kernels at run time (the addend of the exact
    // squaring FMA of block matching, which must not be a constant)
    float neg_zero;
    // aggregation order: reference patches in bands of band_rows grid rows,
    // each band through all frames (0: frames outer, the grid's order)
    int band_rows;
};

// Transform tables of a step (k*k each, row-major, row stride k).
struct StepTables {
    float kaiser[kMaxK * kMaxK];
    float fwd[kMaxK * kMaxK];   // DCT: 2cos(pi (j+1/2) u / k) [u][j]; bior: basis rows
    float inv[kMaxK * kMaxK];   // DCT: REDFT01 matrix [i][u]; bior: inverse basis rows
    float cn[kMaxK * kMaxK];    // DCT normalisation (preProcess, src/vbm3d.cpp:1843-1863)
    float cni[kMaxK * kMaxK];
    float fwdT[kMaxK * kMaxK];  // transposes of fwd / inv (adjoint of the linearised filter)
    float invT[kMaxK * kMaxK];
};

// Everything a step kernel needs, passed by value (a few KB of kernel
// parameter space).
struct StepParams : StepHead, StepTables {};

// Slice stride (floats) of a group held in shared memory: k*k | 1 when a
// lane owns a slice (the lanes' reads of one element fall on distinct
// banks); with four lanes per slice (one-channel groups: 8 slices x 4
// lanes) a stride that spreads the row and column passes over the banks
// (k = 7: 52, no conflict; k = 8: 67, at most 2-way; k*k | 1 gave 2-way and
// 4-way conflicts).
__host__ __device__ constexpr int slice_stride(int k, int lps)
{
    return lps == 4 ? (k == 7 ? 52 : k == 8 ? 67 : ((k * k) | 1)) : ((k * k) | 1);
}

// Reference r of the grid, frames outer, then rows, then columns
// (the loop order of src/vbm3d.cpp:527-538).
__device__ __forceinline__ void ref_coords(const StepHead& P, long long r, int& x, int& y, int& t)
{
    const long long per_frame = (long long)P.nrows * P.ncols;
    t = (int)(r / per_frame);
    const int rem = (int)(r - (long long)t * per_frame);
    const int ir = rem / P.ncols, jr = rem - ir * P.ncols;
    y = min(ir * P.p, P.H - P.k);
    x = min(jr * P.p, P.W - P.k);
}

// The i-th reference patch of the filtering order: bands of band_rows
// grid rows, each band frame by frame, row by row.  A group adds into
// frames t - Nf .. t + Nf near its reference patch, so the numerator /
// denominator rows a band touches in all its frames stay in L2 while the
// band is filtered, instead of being read back from DRAM once per frame
// that reaches them.  A bijection of [0, nrefs).
__device__ __forceinline__ long long band_order_ref(const StepHead& P, long long i)
{
    if (P.band_rows <= 0 || P.band_rows >= P.nrows) return i;
    const long long per_band = (long long)P.band_rows * P.ncols * P.nframes;
    const int band = (int)(i / per_band);
    const long long rem = i - band * per_band;
    const int row0 = band * P.band_rows;
    const int rows = min(P.band_rows, P.nrows - row0);
    const long long per_frame = (long long)rows * P.ncols;
    const int t = (int)(rem / per_frame);
    const long long in_frame = rem - t * per_frame;
    return (long long)t * P.nrows * P.ncols + (long long)row0 * P.ncols + in_frame;
}

__device__ __forceinline__ unsigned patch_index(const StepHead& P, int x, int y, int t)
{
    return (unsigned)t * P.whc + (unsigned)y * (unsigned)P.W + (unsigned)x;
}

__device__ __forceinline__ void patch_coords(const StepHead& P, unsigned idx, int& x, int& y, int& t)
{
    t = (int)(idx / P.whc);
    const unsigned r = idx - (unsigned)t * P.whc;   // channel 0: r < wh
    y = (int)(r / (unsigned)P.W);
    x = (int)(r - (unsigned)y * (unsigned)P.W);
}

// patch_trajectory (src/vbm3d.cpp:378-425, FLOAT_TRAJECTORIES): the
// top-left corner of the patch's slice ht, for ht < kt.  Static unless mc;
// with mc the corner follows the forward flow read at the previous corner,
// accumulated in float and rounded (half away from zero) and clamped.
__device__ __forceinline__ void trajectory(const StepHead& P, const float* __restrict__ fflow, int px, int py,
                                           int pt, int* tx, int* ty)
{
    float fpx = (float)px, fpy = (float)py;
    for (int ht = 0; ht < P.kt; ht++) {
        tx[ht] = px;
        ty[ht] = py;
        if (P.mc && ht < P.kt - 1) {
            float fx = 0.f, fy = 0.f;
            if (fflow) {
                const float* fl = fflow + (size_t)(pt + ht) * 2 * P.wh + (size_t)(py + P.k / 2) * P.W + px + P.k / 2;
                fx = __ldg(fl);
                fy = __ldg(fl + P.wh);
            }
            fpx = fpx + fx;
            fpy = fpy + fy;
            px = min(P.W - P.k, max(0, (int)roundf(fpx)));
            py = min(P.H - P.k, max(0, (int)roundf(fpy)));
        }
    }
}

// (float)((double)s * SQRT2_INV) with float arithmetic (see kS2iHi).
__device__ __forceinline__ float mul_sqrt2_inv(float s)
{
    return __fmaf_rn(s, kS2iHi, __fmul_rn(s, kS2iLo));
}

// (float)((double)s * SQRT2) likewise, SQRT2 being the reference's double
// literal 1.414213562373095 (src/vbm3d.cpp:32).
constexpr float kS2Hi = 1.41421353816986084f;       // float(1.414213562373095)
constexpr float kS2Lo = 2.4203234972131361e-08f;    // float(1.414213562373095 - kS2Hi)
__device__ __forceinline__ float mul_sqrt2(float s)
{
    return __fmaf_rn(s, kS2Hi, __fmul_rn(s, kS2Lo));
}

// transformColorSpace of one RGB / YUV pixel (src/Utilities/LibVideoT.hpp:763-888),
// float operations in the reference's order.
__device__ __forceinline__ void color3(float& a, float& b, float& c, bool forward)
{
    const float R = a, G = b, B = c;
    if (forward) {
        a = 0.299f * R + 0.587f * G + 0.114f * B;
        b = -0.14713f * R - 0.28886f * G + 0.436f * B;
        c = 0.615f * R - 0.51498f * G - 0.10001f * B;
    } else {
        a = R + 1.13983f * B;
        b = R - 0.39465f * G - 0.5806f * B;
        c = R + 2.03211f * G;
    }
}

// 4-byte asynchronous global -> shared copy (no register round trip) to a
// shared-window address (smem_addr), and the wait for all of the calling
// thread's copies; after the wait, a __syncwarp makes every lane's copies
// visible to the warp.  The "memory" clobber of every copy makes the
// compiler reload values that live in memory (kernel parameters included)
// after it, so callers keep what a copy loop needs in registers.
__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void cp_async4s(unsigned dst, const float* src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(dst), "l"(src) : "memory");
}
// The same copy without a compiler memory barrier, for loops that issue
// only copies: the wait that follows them (cp_async_wait_all) is the
// barrier that orders the tiles' reads after the copies.
__device__ __forceinline__ void cp_async4s_nc(unsigned dst, const float* src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(dst), "l"(src));
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

struct Pair {
    float d;
    unsigned i;
};

// libstdc++ std::partial_sort (GCC 13: bits/stl_algo.h __partial_sort /
// __heap_select, bits/stl_heap.h __make_heap / __adjust_heap / __push_heap /
// __pop_heap / __sort_heap) with the reference's comparator
// (a.first < b.first, src/Utilities/Utilities.cpp:40-45).  One thread.
// Reproducing it keeps the reference's order among equal distances.
__device__ __forceinline__ void heap_adjust(Pair* a, int hole, int len, Pair value)
{
    const int top = hole;
    int child = hole;
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
    int parent = (hole - 1) / 2;
    while (hole > top && a[parent].d < value.d) {
        a[hole] = a[parent];
        hole = parent;
        parent = (hole - 1) / 2;
    }
    a[hole] = value;
}

__device__ __forceinline__ void heap_pop(Pair* a, int len, int result)
{
    Pair v = a[result];
    a[result] = a[0];
    heap_adjust(a, 0, len, v);
}

__device__ inline void partial_sort(Pair* a, int middle, int last)
{
    if (middle <= 0) return;
    if (middle >= 2) {
        for (int parent = (middle - 2) / 2;; parent--) {
            heap_adjust(a, parent, middle, a[parent]);
            if (parent == 0) break;
        }
    }
    for (int i = middle; i < last; ++i)
        if (a[i].d < a[0].d) heap_pop(a, middle, i);
    for (int l = middle; l > 1;) {
        --l;
        heap_pop(a, l, l);
    }
}

}  // namespace vbm3d
