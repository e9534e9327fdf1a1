// Deterministic aggregation (opt-in, vbm3d_set_deterministic): the sums of
// the aggregation in the reference's own order, without atomics.
//
// The reference adds, reference patch by reference patch in grid order
// (frames, rows, columns) and within a group patch by patch, the weighted
// estimates into num / den (src/vbm3d.cpp:612-650, :860-924).  So the
// value at a pixel is a float sum over the (reference r, group member n)
// pairs whose patch covers it, in increasing (r, n).  The atomic
// aggregation of the fast path adds the same terms in whatever order the
// GPU runs them, so its last bits vary from run to run.  Here:
//
//  1. the filter stores each group's products kaiser * w * est (and w) in
//     est / wts instead of adding them (filter_common.cuh, STORE);
//  2. det_count / scan / det_fill bucket every (r, n) by its patch's
//     position (a counting sort; the order inside a bucket is arbitrary);
//  3. det_gather: one warp per row segment of 32 pixels (lane = pixel)
//     collects the entries of every patch position that covers the
//     segment (k rows of contiguous bucket ranges), sorts them by the key
//     r * 8 + n in shared memory (bitonic) and walks them in that order,
//     32 at a time: each entry's mask of covered pixels, bit-transposed,
//     gives every lane the entries that cover its pixel, and the lane adds
//     their terms in key order, for every channel.  Segments with more entries than a warp holds go to
//     det_gather_big (a block sorts up to 16384; beyond that each lane
//     selects its entries in key order by repeated minimum search).
//
// Every sum is the reference's sequence of float additions, so with the
// same products the result is the reference's to the bit, and it does not
// depend on the schedule: two runs give identical outputs.
#include <cstdint>

#include "common.cuh"

namespace vbm3d {

namespace {

constexpr int kSegW = 32;          // pixels per segment: a warp, lane = pixel
constexpr int kGatherWarps = 4;
constexpr int kWarpCap = 512;      // entries a warp sorts in shared memory
constexpr int kBlockCap = 16384;   // entries an overflow block sorts
constexpr int kBigThreads = 512;
constexpr int kScanItems = 4;      // per thread
constexpr int kScanThreads = 1024;
constexpr int kScanBlock = kScanItems * kScanThreads;
constexpr unsigned kNoKey = 0xffffffffu;

struct KaiserTable {
    float w[kMaxK * kMaxK];
};

// Position of patch index idx (channel 0, the reference's linear index) in
// the frames' channel-0 planes: t * wh + y * W + x.
__device__ __forceinline__ unsigned det_pos(const StepHead& P, unsigned idx, int& x, int& y, int& t)
{
    patch_coords(P, idx, x, y, t);
    return (unsigned)t * P.wh + (unsigned)y * (unsigned)P.W + (unsigned)x;
}

__global__ void det_count(const StepHead P, const unsigned* __restrict__ tab_idx,
                          const unsigned* __restrict__ tab_nsx, unsigned* __restrict__ cnt)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;  // r * N + n
    if (i >= P.nrefs * P.N) return;
    const long long r = i / P.N;
    const int n = (int)(i - r * P.N);
    if (n >= (int)tab_nsx[r]) return;
    int x, y, t;
    atomicAdd(cnt + det_pos(P, tab_idx[i], x, y, t), 1u);
}

// Exclusive scan of one block's values (v per thread); the block total in
// *total.  ws: 32 words of shared memory.
__device__ __forceinline__ unsigned block_exclusive(unsigned v, unsigned* ws, unsigned* total)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    unsigned incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned u = __shfl_up_sync(kFull, incl, o);
        if (lane >= o) incl += u;
    }
    if (lane == 31) ws[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        unsigned w = lane < nw ? ws[lane] : 0u, wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned u = __shfl_up_sync(kFull, wi, o);
            if (lane >= o) wi += u;
        }
        if (lane < nw) ws[lane] = wi - w;
        if (lane == 31) ws[32] = wi;
    }
    __syncthreads();
    const unsigned res = incl - v + ws[wid];
    *total = ws[32];
    __syncthreads();
    return res;
}

// off[i] = sum of cnt[0 .. i) within the block's kScanBlock values; the
// block's total in bsum[block].
__global__ void __launch_bounds__(kScanThreads) det_scan_blocks(const unsigned* __restrict__ cnt, size_t n,
                                                                unsigned* __restrict__ off,
                                                                unsigned* __restrict__ bsum)
{
    __shared__ unsigned ws[33];
    const size_t base = (size_t)blockIdx.x * kScanBlock + (size_t)threadIdx.x * kScanItems;
    unsigned v[kScanItems], s = 0;
#pragma unroll
    for (int j = 0; j < kScanItems; j++) {
        v[j] = base + j < n ? cnt[base + j] : 0u;
        s += v[j];
    }
    unsigned total;
    unsigned run = block_exclusive(s, ws, &total);
#pragma unroll
    for (int j = 0; j < kScanItems; j++) {
        if (base + j < n) off[base + j] = run;
        run += v[j];
    }
    if (threadIdx.x == 0) bsum[blockIdx.x] = total;
}

// Exclusive scan of the nb block totals in place (one block, a carry over
// chunks); the grand total in bsum[nb].
__global__ void __launch_bounds__(kScanThreads) det_scan_sums(unsigned* __restrict__ bsum, size_t nb)
{
    __shared__ unsigned ws[33];
    unsigned carry = 0;
    for (size_t c0 = 0; c0 < nb; c0 += kScanThreads) {
        const size_t i = c0 + threadIdx.x;
        const unsigned v = i < nb ? bsum[i] : 0u;
        unsigned total;
        const unsigned e = block_exclusive(v, ws, &total);
        if (i < nb) bsum[i] = carry + e;
        carry += total;
    }
    if (threadIdx.x == 0) bsum[nb] = carry;
}

__global__ void __launch_bounds__(kScanThreads) det_scan_add(unsigned* __restrict__ off, size_t n,
                                                             const unsigned* __restrict__ bsum, size_t nb)
{
    const size_t base = (size_t)blockIdx.x * kScanBlock + (size_t)threadIdx.x * kScanItems;
    const unsigned add = bsum[blockIdx.x];
#pragma unroll
    for (int j = 0; j < kScanItems; j++)
        if (base + j < n) off[base + j] += add;
    if (blockIdx.x == 0 && threadIdx.x == 0) off[n] = bsum[nb];
}

// Entry of (r, n): key r * 8 + n (N <= 8), and the patch position packed
// as (y << 16) | x.  cnt is consumed (counted down to the bucket starts).
__global__ void det_fill(const StepHead P, const unsigned* __restrict__ tab_idx,
                         const unsigned* __restrict__ tab_nsx, const unsigned* __restrict__ off,
                         unsigned* __restrict__ cnt, uint2* __restrict__ ent)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.nrefs * P.N) return;
    const long long r = i / P.N;
    const int n = (int)(i - r * P.N);
    if (n >= (int)tab_nsx[r]) return;
    int x, y, t;
    const unsigned pos = det_pos(P, tab_idx[i], x, y, t);
    const unsigned slot = off[pos] + atomicSub(cnt + pos, 1u) - 1u;
    ent[slot] = make_uint2((unsigned)(r << 3) | (unsigned)n, ((unsigned)y << 16) | (unsigned)x);
}

// Geometry of segment seg: frame t, row y, first column x0, and the
// entries of every patch position covering it: bucket rows py0 .. py1,
// columns px0 .. px1 (empty when px0 > px1 or py0 > py1).
struct Seg {
    int t, y, x0, py0, py1, px0, px1;
};

__device__ __forceinline__ Seg seg_of(const StepHead& P, long long seg)
{
    const int spr = (P.W + kSegW - 1) / kSegW;
    Seg s;
    s.t = (int)(seg / ((long long)P.H * spr));
    const int rem = (int)(seg - (long long)s.t * P.H * spr);
    s.y = rem / spr;
    s.x0 = (rem - s.y * spr) * kSegW;
    s.py0 = max(0, s.y - P.k + 1);
    s.py1 = min(s.y, P.H - P.k);
    s.px0 = max(0, s.x0 - P.k + 1);
    s.px1 = min(s.x0 + kSegW - 1, P.W - P.k);
    return s;
}

// The bucket range of row py of the segment.
__device__ __forceinline__ void seg_range(const StepHead& P, const Seg& s, int py, const unsigned* __restrict__ off,
                                          unsigned& a, unsigned& b)
{
    const size_t row = (size_t)s.t * P.wh + (size_t)py * P.W;
    a = off[row + s.px0];
    b = off[row + s.px1 + 1];
}

__device__ __forceinline__ unsigned seg_total(const StepHead& P, const Seg& s, const unsigned* __restrict__ off)
{
    if (s.px0 > s.px1 || s.py0 > s.py1) return 0u;
    unsigned T = 0;
    for (int py = s.py0; py <= s.py1; py++) {
        unsigned a, b;
        seg_range(P, s, py, off, a, b);
        T += b - a;
    }
    return T;
}

// Index of list element e: PAD inserts one element after every 16, so that
// the sorting network's accesses of a warp (stride-s pairs of 8-byte
// elements) spread over the 32 banks.
template <bool PAD>
__device__ __forceinline__ int lix(int e)
{
    return PAD ? e + (e >> 4) : e;
}

// Copies the segment's entries into list[0 .. T) with the `nthreads`
// threads of index `tid`.
template <bool PAD>
__device__ __forceinline__ void seg_collect(const StepHead& P, const Seg& s, const unsigned* __restrict__ off,
                                            const uint2* __restrict__ ent, uint2* list, int tid, int nthreads)
{
    unsigned o = 0;
    for (int py = s.py0; py <= s.py1; py++) {
        unsigned a, b;
        seg_range(P, s, py, off, a, b);
        for (unsigned j = (unsigned)tid; j < b - a; j += (unsigned)nthreads) list[lix<PAD>((int)(o + j))] = ent[a + j];
        o += b - a;
    }
}

template <bool PAD>
__device__ __forceinline__ void cmp_swap(uint2* list, int i, int size, int stride)
{
    const int lo0 = ((i & ~(stride - 1)) << 1) | (i & (stride - 1));
    const bool up = (lo0 & size) == 0;
    const int lo = lix<PAD>(lo0), hi = lix<PAD>(lo0 + stride);
    const uint2 a = list[lo], b = list[hi];
    if ((a.x > b.x) == up) {
        list[lo] = b;
        list[hi] = a;
    }
}

// The entries' terms at pixel x of row y, in key order, into num / den.
template <int K>
__device__ __forceinline__ void add_entry(const StepHead& P, const KaiserTable& kt, uint2 e, int x, int y,
                                          const float* __restrict__ est, const float* __restrict__ wts,
                                          float (&num)[kMaxC], float (&den)[kMaxC])
{
    const int px = (int)(e.y & 0xffffu), py = (int)(e.y >> 16), dx = x - px;
    if (dx < 0 || dx >= K) return;
    const int pq = (y - py) * K + dx;
    const size_t r = e.x >> 3, n = e.x & 7u;
    const float kai = kt.w[pq];
#pragma unroll
    for (int c = 0; c < kMaxC; c++) {
        if (c < P.C) {
            num[c] = num[c] + est[((r * P.C + c) * P.N + n) * (K * K) + pq];
            den[c] = den[c] + kai * wts[r * P.C + c];
        }
    }
}

// Column `lane` of the 32 x 32 bit matrix whose row r lane r holds in x:
// bit r of the result is bit `lane` of lane r's x (five exchange rounds of
// the off-diagonal blocks).
__device__ __forceinline__ unsigned transpose_round(unsigned x, int lane, int j, unsigned hi)
{
    const unsigned y = __shfl_xor_sync(kFull, x, j);
    return (lane & j) ? ((x & hi) | ((y & hi) >> j)) : ((x & ~hi) | ((y & ~hi) << j));
}
__device__ __forceinline__ unsigned transpose32(unsigned x, int lane)
{
    x = transpose_round(x, lane, 16, 0xFFFF0000u);
    x = transpose_round(x, lane, 8, 0xFF00FF00u);
    x = transpose_round(x, lane, 4, 0xF0F0F0F0u);
    x = transpose_round(x, lane, 2, 0xCCCCCCCCu);
    return transpose_round(x, lane, 1, 0xAAAAAAAAu);
}

// The sorted entries list[0 .. T) of segment s, added at the pixels they
// cover: a warp takes them 32 at a time; each lane's entry gives a mask of
// the lanes (pixels) its patch covers, the transposed masks give each lane
// the entries of the chunk that cover its pixel, which it adds in key
// order.  A lane loads the terms of up to kBatch of its entries before it
// adds them (the same products, added in the same order), so their loads
// are in flight together.  Every lane of the warp calls it.
template <int K, bool PAD>
__device__ __forceinline__ void walk_sorted(const StepHead& P, const KaiserTable& kt, const uint2* list, unsigned T,
                                            const Seg& s, int lane, const float* __restrict__ est,
                                            const float* __restrict__ wts, float (&num)[kMaxC], float (&den)[kMaxC])
{
    constexpr int kBatch = 4;
    const int x = s.x0 + lane;
    for (unsigned c0 = 0; c0 < T; c0 += 32) {
        unsigned m = 0;
        if (c0 + lane < T) {
            const int lo = (int)(list[lix<PAD>((int)c0 + lane)].y & 0xffffu) - s.x0;  // first covered lane (may be < 0)
            const int a = max(lo, 0), b = min(lo + K, 32);
            if (b > a) m = (b - a == 32 ? 0xffffffffu : ((1u << (b - a)) - 1u)) << a;
        }
        for (unsigned mine = transpose32(m, lane); mine;) {
            float e[kBatch][kMaxC], w[kBatch][kMaxC];
#pragma unroll
            for (int q = 0; q < kBatch; q++) {
#pragma unroll
                for (int c = 0; c < kMaxC; c++) e[q][c] = w[q][c] = 0.f;
                if (mine) {
                    const uint2 en = list[lix<PAD>((int)c0 + __ffs(mine) - 1)];
                    mine &= mine - 1;
                    // the pixel is covered: column x - px in [0, K)
                    const int px = (int)(en.y & 0xffffu), py = (int)(en.y >> 16);
                    const int pq = (s.y - py) * K + (x - px);
                    const size_t r = en.x >> 3, n = en.x & 7u;
                    const float kai = kt.w[pq];
#pragma unroll
                    for (int c = 0; c < kMaxC; c++) {
                        if (c < P.C) {
                            e[q][c] = __ldg(est + ((r * P.C + c) * P.N + n) * (K * K) + pq);
                            w[q][c] = kai * __ldg(wts + r * P.C + c);
                        }
                    }
                }
            }
            // adding 0 to a sum leaves it unchanged (the sums are never -0)
#pragma unroll
            for (int q = 0; q < kBatch; q++)
#pragma unroll
                for (int c = 0; c < kMaxC; c++) {
                    num[c] = num[c] + e[q][c];
                    den[c] = den[c] + w[q][c];
                }
        }
    }
}

template <int K>
__device__ __forceinline__ void seg_write(const StepHead& P, const Seg& s, int x, const float (&num)[kMaxC],
                                          const float (&den)[kMaxC], float* __restrict__ pair)
{
    if (x >= P.W) return;
#pragma unroll
    for (int c = 0; c < kMaxC; c++) {
        if (c < P.C) {
            const size_t o = (size_t)s.t * P.whc + (size_t)c * P.wh + (size_t)s.y * P.W + x;
            reinterpret_cast<float2*>(pair)[o] = make_float2(num[c], den[c]);
        }
    }
}

template <int K>
__global__ void __launch_bounds__(kGatherWarps * 32)
det_gather(const StepHead P, const KaiserTable kt, const float* __restrict__ est, const float* __restrict__ wts,
           const unsigned* __restrict__ off, const uint2* __restrict__ ent, float* __restrict__ pair,
           unsigned* __restrict__ ovf, long long nseg)
{
    __shared__ uint2 lists[kGatherWarps][kWarpCap + kWarpCap / 16];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const long long seg = (long long)blockIdx.x * kGatherWarps + wid;
    if (seg >= nseg) return;
    const Seg s = seg_of(P, seg);
    const unsigned T = seg_total(P, s, off);
    if (T > (unsigned)kWarpCap) {  // to det_gather_big: ovf[0] counts, ovf[1 ..] lists
        if (lane == 0) ovf[1 + atomicAdd(ovf, 1u)] = (unsigned)seg;
        return;
    }
    uint2* list = lists[wid];
    seg_collect<true>(P, s, off, ent, list, lane, 32);
    int M = 32;
    while (M < (int)T) M <<= 1;
    for (int j = (int)T + lane; j < M; j += 32) list[lix<true>(j)] = make_uint2(kNoKey, 0u);
    __syncwarp();
    for (int size = 2; size <= M; size <<= 1)
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int i = lane; i < M / 2; i += 32) cmp_swap<true>(list, i, size, stride);
            __syncwarp();
        }
    float num[kMaxC] = {0.f, 0.f, 0.f}, den[kMaxC] = {0.f, 0.f, 0.f};
    const int x = s.x0 + lane;
    walk_sorted<K, true>(P, kt, list, T, s, lane, est, wts, num, den);
    seg_write<K>(P, s, x, num, den, pair);
}

// Segments with more than kWarpCap entries: a block sorts up to kBlockCap
// of them in shared memory; beyond that, each lane of warp 0 takes its
// pixel's entries in key order by repeated minimum search in global memory.
template <int K>
__global__ void __launch_bounds__(kBigThreads)
det_gather_big(const StepHead P, const KaiserTable kt, const float* __restrict__ est,
               const float* __restrict__ wts, const unsigned* __restrict__ off, const uint2* __restrict__ ent,
               float* __restrict__ pair, const unsigned* __restrict__ ovf)
{
    extern __shared__ uint2 blist[];
    const int lane = threadIdx.x & 31;
    const unsigned nov = ovf[0];
    for (unsigned b = blockIdx.x; b < nov; b += gridDim.x) {
        const Seg s = seg_of(P, (long long)ovf[1 + b]);
        const unsigned T = seg_total(P, s, off);
        const int x = s.x0 + lane;
        float num[kMaxC] = {0.f, 0.f, 0.f}, den[kMaxC] = {0.f, 0.f, 0.f};
        if (T <= (unsigned)kBlockCap) {
            seg_collect<false>(P, s, off, ent, blist, threadIdx.x, blockDim.x);
            int M = 32;
            while (M < (int)T) M <<= 1;
            for (int j = (int)T + threadIdx.x; j < M; j += blockDim.x) blist[j] = make_uint2(kNoKey, 0u);
            __syncthreads();
            for (int size = 2; size <= M; size <<= 1)
                for (int stride = size >> 1; stride > 0; stride >>= 1) {
                    for (int i = threadIdx.x; i < M / 2; i += blockDim.x) cmp_swap<false>(blist, i, size, stride);
                    __syncthreads();
                }
            if (threadIdx.x < 32) {
                walk_sorted<K, false>(P, kt, blist, T, s, lane, est, wts, num, den);
                seg_write<K>(P, s, x, num, den, pair);
            }
            __syncthreads();
        } else if (threadIdx.x < 32) {
            // keys are distinct: each pass takes the smallest key above the
            // last one among the entries that cover this lane's pixel
            unsigned long long last = 0;  // last key + 1
            for (;;) {
                unsigned best = kNoKey;
                uint2 be = make_uint2(kNoKey, 0u);
                for (int py = s.py0; py <= s.py1; py++) {
                    unsigned a, bnd;
                    seg_range(P, s, py, off, a, bnd);
                    for (unsigned j = a; j < bnd; j++) {
                        const uint2 e = ent[j];
                        const int dx = x - (int)(e.y & 0xffffu);
                        if (dx >= 0 && dx < K && (unsigned long long)e.x >= last && e.x < best) {
                            best = e.x;
                            be = e;
                        }
                    }
                }
                if (best == kNoKey) break;
                add_entry<K>(P, kt, be, x, s.y, est, wts, num, den);
                last = (unsigned long long)best + 1;
            }
            seg_write<K>(P, s, x, num, den, pair);
        }
    }
}

template <int K>
cudaError_t launch_gather(const StepHead& P, const KaiserTable& kt, const float* est, const float* wts,
                          const unsigned* off, const uint2* ent, float* pair, unsigned* ovf, cudaStream_t s)
{
    const long long nseg = (long long)P.F * P.H * ((P.W + kSegW - 1) / kSegW);
    const long long blocks = (nseg + kGatherWarps - 1) / kGatherWarps;
    det_gather<K><<<(unsigned)blocks, kGatherWarps * 32, 0, s>>>(P, kt, est, wts, off, ent, pair, ovf, nseg);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const size_t smem = (size_t)kBlockCap * sizeof(uint2);
    e = cudaFuncSetAttribute(det_gather_big<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    det_gather_big<K><<<152, kBigThreads, smem, s>>>(P, kt, est, wts, off, ent, pair, ovf);
    return cudaGetLastError();
}

}  // namespace

// Scratch of the deterministic aggregation of one step, in 4-byte words:
// bucket counts and starts (2 (npos + 1) with npos = W * H * F), block sums,
// entries (2 nrefs N) and the overflow list (segments + 1).
size_t det_scratch_words(const StepHead& P)
{
    const size_t npos = (size_t)P.wh * P.F;
    const size_t nb = (npos + 1 + kScanBlock - 1) / kScanBlock;
    const size_t nseg = (size_t)P.F * P.H * ((P.W + kSegW - 1) / kSegW);
    return 2 * (npos + 1) + (nb + 1) + 2 * (size_t)P.nrefs * P.N + (nseg + 1) + 8;
}

// The ordered sums of one step into `pair` (interleaved num, den, every
// value written), from the stored products est / wts of the filter's STORE
// mode.  scratch: det_scratch_words(P) words.
cudaError_t launch_det_aggregate(const StepParams& P, const unsigned* tab_idx, const unsigned* tab_nsx,
                                 const float* est, const float* wts, unsigned* scratch, float* pair,
                                 cudaStream_t s)
{
    const size_t npos = (size_t)P.wh * P.F;
    const size_t nb = (npos + 1 + kScanBlock - 1) / kScanBlock;
    const size_t nseg = (size_t)P.F * P.H * ((P.W + kSegW - 1) / kSegW);
    unsigned* cnt = scratch;
    unsigned* off = cnt + (npos + 1);
    unsigned* bsum = off + (npos + 1);
    uint2* ent = reinterpret_cast<uint2*>(bsum + ((nb + 2) & ~(size_t)1));  // 8-byte aligned
    unsigned* ovf = reinterpret_cast<unsigned*>(ent + (size_t)P.nrefs * P.N);
    cudaError_t e = cudaMemsetAsync(cnt, 0, (npos + 1) * sizeof(unsigned), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(ovf, 0, sizeof(unsigned), s);
    if (e != cudaSuccess) return e;
    const StepHead& H = P;
    const long long pairs = P.nrefs * P.N;
    const unsigned tb = 256;
    det_count<<<(unsigned)((pairs + tb - 1) / tb), tb, 0, s>>>(H, tab_idx, tab_nsx, cnt);
    det_scan_blocks<<<(unsigned)nb, kScanThreads, 0, s>>>(cnt, npos + 1, off, bsum);
    det_scan_sums<<<1, kScanThreads, 0, s>>>(bsum, nb);
    det_scan_add<<<(unsigned)nb, kScanThreads, 0, s>>>(off, npos, bsum, nb);
    det_fill<<<(unsigned)((pairs + tb - 1) / tb), tb, 0, s>>>(H, tab_idx, tab_nsx, off, cnt, ent);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    (void)nseg;
    KaiserTable kt;
    for (int i = 0; i < kMaxK * kMaxK; i++) kt.w[i] = i < P.k * P.k ? P.kaiser[i] : 0.f;
    if (P.k == 7) return launch_gather<7>(H, kt, est, wts, off, ent, pair, ovf, s);
    if (P.k == 8) return launch_gather<8>(H, kt, est, wts, off, ent, pair, ovf, s);
    return cudaErrorInvalidValue;
}

}  // namespace vbm3d
