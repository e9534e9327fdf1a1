// Types of the batched form shared by its host code (batch.cu) and its
// work kernels (batch_kernels.cuh, instantiated in batch_step1.cu and
// batch_step2.cu).
#pragma once

#include "bm2_impl.cuh"

namespace vbm3d {
namespace batched {

constexpr int kTab = 64;  // k*k entries of a compact table (k <= 8)

// The filter's view of a clip's step: scalar head and compact transform
// tables.
struct CompactTables {
    float kaiser[kTab];
    float fwd[kTab];
    float inv[kTab];
    float cn[kTab];
    float cni[kTab];
};

// One clip of the batch, in device memory.
struct BatchClip {
    const float* in;     // the caller's noisy clip
    const float* fflow;  // NULL: zero flow
    const float* bflow;
    float* y;            // noisy clip in the working colour space
    float* basic;        // basic estimate, working colour space
    float* pair;         // interleaved (numerator, denominator)
    unsigned* tab_idx;   // block-matching table: nrefs * N indices
    unsigned* tab_nsx;   // group size per reference
    float* out_basic;    // the caller's outputs (NULL: no basic output)
    float* out_den;
    unsigned wh, C, color, pad;
};

// Block matching reads its clips' parameters and buffers from a table
// passed by value as a __grid_constant__ kernel argument (under the 32 KB
// parameter limit), indexed by the work item's slot.  In parameter space
// they are read through the constant cache and need no registers, as in
// the plain kernel, whose parameters are kernel arguments too; copies in
// shared memory or registers measured 10-40 % slower, the registers they
// take being the ones the distance loop runs short of.
constexpr int kTableClips = 150;
struct BmTable {
    StepHead h[kTableClips];
    Layout L[kTableClips];
    const float* vid[kTableClips];  // the video block matching reads
    const float* fflow[kTableClips];
    const float* bflow[kTableClips];
    unsigned* tab_idx[kTableClips];
    unsigned* tab_nsx[kTableClips];
};
static_assert(sizeof(BmTable) <= 31 * 1024, "kernel parameter limit");

// Filtering reads the transform tables its launch's clips share and each
// clip's parameters and buffers from a table of the same kind.
struct FilterTable {
    CompactTables t;
    StepHead h[kTableClips];
    float* pair[kTableClips];          // interleaved (numerator, denominator)
    const float* noisy[kTableClips];   // the clip in the working colour space
    const float* basic[kTableClips];
    const unsigned* tab_idx[kTableClips];
    const unsigned* tab_nsx[kTableClips];
};
static_assert(sizeof(FilterTable) <= 31 * 1024, "kernel parameter limit");

// A work item is a uint4 (clip, first reference, references, slot): the
// references lie in one frame of the clip's grid; the work kernels read
// the clip's entries at `slot` of their launch's table.

// Work phases and kernel classes: block matching has one class per
// (k, C) in {7, 8} x {1, 3}; filtering one per transform table set,
// (k, T_2D) in {(7, DCT), (8, DCT), (8, bior1.5)}, and channel count (one
// channel: the shared-slice transforms, four lanes per slice; classes 3-5).
constexpr int kPhases = 4;   // bm1, filter1, bm2, filter2
constexpr int kClasses = 6;

inline int class_of(int phase, const StepHead& P)
{
    if (phase & 1) return (P.k == 8 ? (P.T2D == kBIOR ? 2 : 1) : 0) + (P.C == 1 ? 3 : 0);
    return (P.k == 8 ? 2 : 0) + (P.C == 3 ? 1 : 0);
}

// The work kernel of (phase, class): a host function pointer for
// cudaFuncSetAttribute, the occupancy query and cudaLaunchKernel; NULL for
// a class the phase does not have.
const void* work_kernel_step1(int phase, int cls);
const void* work_kernel_step2(int phase, int cls);

}  // namespace batched
}  // namespace vbm3d
