// K-BM, staged form: predictive block matching with shared-memory windows
// and packed f32x2 arithmetic, for k in {7, 8} and 1 or 3 channels (other
// shapes use bm.cu).  Same results as bm.cu, bit for bit.
//
// One warp handles one reference patch, in phases:
//   phase 0: the Ns x Ns window of the reference frame;
//   phase f (1..Nf): forward step f and backward step f together (the two
//     chains are independent until the final sort, and never share a
//     frame), i.e. up to 2*Nb windows of Npr x Npr.
// Each phase stages its windows' pixels (window + k - 1 per side, all
// channels) in shared memory, then evaluates every window position.  Two
// candidates share one lane through packed f32x2 sub / mul / add, which
// round each half exactly like the scalar operations, so every distance is
// the reference's sequential float sum (src/vbm3d.cpp:965-1010).  The
// reference patch is held as duplicated (r, r) pairs for the packed
// operand.  Positions seen in an earlier window of the same frame are
// evaluated but not used (the reference's alreadySeen, src/vbm3d.cpp:1065).
// Selections use exact-rank fast paths and fall back to the reference's
// std::partial_sort order (common.cuh) whenever two distances tie.
#include "bm2_impl.cuh"

namespace vbm3d {

namespace {

// Register budget: 96 for three channels (shared memory limits residency
// to 5 blocks of 4 warps, so 96 registers cost no occupancy and remove
// spills; 88, also spill-free, measured 2 % slower on the RGB batch
// launches, and 7 blocks of 3 warps at 88 registers 17 % slower), 80 for
// one channel (more resident blocks pay more).  A reference patch takes a
// group of G lanes: a warp for three channels, a half warp for one (whose
// distance sums are short, so the per-reference bookkeeping a group runs
// once is shared by two references per warp).
template <int K, int C>
__host__ __device__ constexpr int bm2_group() { return C == 1 ? 16 : 32; }

template <int K, int C>
__global__ void __maxnreg__(C == 3 ? 96 : 80)
bm2_kernel(const StepParams P, const float* __restrict__ vid, const float* __restrict__ fflow,
           const float* __restrict__ bflow, unsigned* __restrict__ out_idx, float* __restrict__ out_dist,
           unsigned* __restrict__ out_nsimp, unsigned* __restrict__ out_nsx, const Layout L)
{
    constexpr int G = bm2_group<K, C>();
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31, gid = threadIdx.x / G;
    const long long r = P.ref_base + (long long)blockIdx.x * (blockDim.x / G) + gid;
    if (r >= P.nrefs) return;  // the group's lanes only: the other half of the warp may go on
    const Grp<G> g(lane);
    bm2_ref<K, C, G>(P, L, r, smem + (size_t)gid * L.warp_bytes, g, vid, fflow, bflow, out_idx, out_dist,
                     out_nsimp, out_nsx);
}

}  // namespace

bool bm2_supported(const StepParams& P) { return bm2_layout(P).warp_bytes > 0; }

cudaError_t launch_bm2(const StepParams& P, const float* vid, const float* fflow, const float* bflow,
                       unsigned* out_idx, float* out_dist, unsigned* out_nsimp, unsigned* out_nsx, long long count,
                       cudaStream_t stream)
{
    const Layout L = bm2_layout(P);
    if (!L.warp_bytes) return cudaErrorInvalidValue;
    // one-channel k = 7 patches: 16 per block (eight warps of two), whose
    // staged windows overlap in L1; otherwise 4 warps
    const int warps = (P.C == 1 && P.k == 7) ? 8 : 4;
    cudaError_t e = cudaSuccess;
#define VBM3D_BM2(KV, CV)                                                                                  \
    if (P.k == KV && P.C == CV) {                                                                          \
        const int groups = warps * 32 / bm2_group<KV, CV>();                                               \
        const size_t smem = (size_t)groups * L.warp_bytes;                                                 \
        const long long blocks = (count + groups - 1) / groups;                                            \
        e = cudaFuncSetAttribute(bm2_kernel<KV, CV>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
        if (e != cudaSuccess) return e;                                                                    \
        bm2_kernel<KV, CV><<<(unsigned)blocks, warps * 32, smem, stream>>>(P, vid, fflow, bflow, out_idx,   \
                                                                          out_dist, out_nsimp, out_nsx, L);  \
        return cudaGetLastError();                                                                         \
    }
    VBM3D_BM2(7, 1)
    VBM3D_BM2(7, 3)
    VBM3D_BM2(8, 1)
    VBM3D_BM2(8, 3)
#undef VBM3D_BM2
    return cudaErrorInvalidValue;
}

}  // namespace vbm3d
