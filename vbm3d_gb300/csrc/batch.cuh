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
struct FilterView {
    StepHead h;
    CompactTables t;
};

struct ClipStep {
    FilterView v;
    Layout L;
    int pad[4];
};

// One clip of the batch, in device memory.
struct BatchClip {
    ClipStep s[2];
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

// Shared-memory copies of a clip's parameters at the start of a block's
// dynamic shared memory (block matching: StepHead and Layout; filtering:
// FilterView), 16-byte multiples.
constexpr int kHeadBytes = (int)((sizeof(StepHead) + 15) & ~size_t(15));
constexpr int kLayoutBytes = (int)((sizeof(Layout) + 15) & ~size_t(15));
constexpr int kViewFloats = (int)(((sizeof(FilterView) + 15) & ~size_t(15)) / 4);
static_assert(sizeof(StepHead) % 4 == 0 && sizeof(Layout) % 4 == 0 && sizeof(FilterView) % 4 == 0, "word copies");

// A work item is a uint4 (clip, first reference, references, 0); the
// references lie in one frame of the clip's grid.

// Work phases and kernel classes: block matching has one class per
// (k, C) in {7, 8} x {1, 3}; filtering one per transform table set,
// (k, T_2D) in {(7, DCT), (8, DCT), (8, bior1.5)}.
constexpr int kPhases = 4;   // bm1, filter1, bm2, filter2
constexpr int kClasses = 4;

inline int class_of(int phase, const StepHead& P)
{
    if (phase & 1) return P.k == 8 ? (P.T2D == kBIOR ? 2 : 1) : 0;
    return (P.k == 8 ? 2 : 0) + (P.C == 3 ? 1 : 0);
}

// The work kernel of (phase, class): a host function pointer for
// cudaFuncSetAttribute, the occupancy query and cudaLaunchKernel; NULL for
// a class the phase does not have.
const void* work_kernel_step1(int phase, int cls);
const void* work_kernel_step2(int phase, int cls);

}  // namespace batched
}  // namespace vbm3d
