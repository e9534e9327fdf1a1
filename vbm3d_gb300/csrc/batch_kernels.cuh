// Work kernels of the batched form (persistent, queue-driven); included by
// batch_step1.cu and batch_step2.cu, which instantiate them.
#pragma once

#include "batch.cuh"
#include "filter_common.cuh"

namespace vbm3d {
namespace batched {

constexpr unsigned kNoItem = 0xffffffffu;

// Work items are taken one ahead: thread 0 claims the block's next item
// (one atomicAdd on the queue head) while the block works on the current
// one, and the barrier that ends the current item publishes it, so a block
// waits at one barrier per item and never for the queue.
__device__ __forceinline__ void claim_item(const uint4* __restrict__ items, unsigned nitems, unsigned* head,
                                           uint4* slot)
{
    if (threadIdx.x == 0) {
        const unsigned it = atomicAdd(head, 1u);
        *slot = it < nitems ? items[it] : make_uint4(kNoItem, 0u, 0u, 0u);
    }
}

// ------------------------------------------------------- work phases ---
// One kernel per class (K, C) of block matching and per table set of
// filtering, as the plain path has, so each holds one copy of the
// per-reference body.  A work item is taken by a whole block; its warps
// handle interleaved references of the tile (warp w: references w,
// w + warps, ...), so at any time a block works on neighbouring reference
// patches whose search windows and groups overlap in L1, as a block of the
// plain kernel does.  Block matching reads its clips' parameters from the
// launch's kernel-argument table (batch.cuh), and so does filtering, whose
// table also holds the transform tables of its class (the same for every
// clip of the launch): each table entry is a constant-bank operand of the
// transforms' FMAs (k = 8: -7 % to -16 % per launch against tables in
// shared memory; k = 7, with the DCT passes through their even and odd
// halves: 96 registers instead of 128, step-2 RGB launches -3.5 % to
// -7 %), and the clip's parameters are constant-cache reads instead of
// shared-memory loads.

// A reference patch takes a group of G lanes, as in bm2_kernel: a warp for
// three channels, a half warp for one.
template <int STEP, int K, int C, int G>
__global__ void __maxnreg__(C == 3 ? 96 : 80)  // as bm2_kernel
batch_bm_kernel(const BatchClip* __restrict__ clips, const uint4* __restrict__ items, unsigned nitems,
                unsigned* __restrict__ head, int warp_bytes, const __grid_constant__ BmTable T)
{
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ uint4 s_item[2];
    const int lane = threadIdx.x & 31, gid = threadIdx.x / G, ngroups = blockDim.x / G;
    unsigned char* ws = smem + (size_t)gid * warp_bytes;
    const Grp<G> g(lane);
    claim_item(items, nitems, head, &s_item[0]);
    __syncthreads();
    for (int buf = 0;; buf ^= 1) {
        const uint4 I = s_item[buf];
        if (I.x == kNoItem) break;
        claim_item(items, nitems, head, &s_item[buf ^ 1]);
        const int t = (int)I.w;
        for (unsigned j = gid; j < I.z; j += ngroups) {
            bm2_ref<K, C, G>(T.h[t], T.L[t], (long long)I.y + j, ws, g, T.vid[t], T.fflow[t], T.bflow[t],
                             T.tab_idx[t], nullptr, nullptr, T.tab_nsx[t]);
            g.sync();
        }
        __syncthreads();  // publishes the next item
    }
}

// Registers: the four-lanes-per-slice kernels (one-channel groups) at 96,
// which holds 5 blocks of 4 warps per SM (their step-2 k = 7 launch -4.7 %
// against the 116 registers the compiler takes with room for 128); the
// one-slice-per-lane kernels need up to 128.
template <int STEP, int K, int LPS>
__global__ void __maxnreg__(LPS == 4 ? 96 : 128)
batch_filter_kernel(const BatchClip* __restrict__ clips, const uint4* __restrict__ items, unsigned nitems,
                    unsigned* __restrict__ head, int warp_floats, const __grid_constant__ FilterTable T)
{
    extern __shared__ __align__(16) float fsm[];
    __shared__ uint4 s_item[2];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    float* base = fsm + (size_t)wid * warp_floats;
    claim_item(items, nitems, head, &s_item[0]);
    __syncthreads();
    for (int buf = 0;; buf ^= 1) {
        const uint4 I = s_item[buf];
        if (I.x == kNoItem) break;
        claim_item(items, nitems, head, &s_item[buf ^ 1]);
        const int t = (int)I.w;
        const AggTarget A{nullptr, nullptr, T.pair[t]};
        for (unsigned j = wid; j < I.z; j += nwarps) {
            filter_ref<STEP, K, true, LPS>(T.h[t], T.t, (long long)I.y + j, base, lane, T.noisy[t], T.basic[t],
                                           T.tab_idx[t], T.tab_nsx[t], A);
            __syncwarp();
        }
        __syncthreads();
    }
}

}  // namespace batched
}  // namespace vbm3d
