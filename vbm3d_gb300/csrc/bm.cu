// K-BM: predictive spatio-temporal block matching.
//
// Replaces computeSimilarPatches / localSearch / patchDistance of the
// reference (src/vbm3d.cpp:930-1197).  One warp handles one reference patch:
//
//  * the reference patch is staged in shared memory once;
//  * each search window (Ns x Ns in the reference frame, Npr x Npr around the
//    Nb predicted positions in the other frames) is scanned in the
//    reference's row-major order, one candidate per lane and slot; every
//    candidate's distance is a sequential float sum over (channel, row,
//    column) in the reference's order (compiled with --fmad=false), divided
//    by k*k*C, so distances are bit-identical to the reference's;
//  * the Nb smallest distances of a window are picked by warp shuffles; when
//    two candidates tie exactly, the window falls back to the reference's
//    own selection order (std::partial_sort restated in common.cuh) on one
//    lane, so ties resolve as the reference resolves them;
//  * positions already scanned for this reference are skipped (the
//    reference's alreadySeen map, src/vbm3d.cpp:1065): a position is seen
//    iff it lies in an earlier window on the same frame;
//  * the forward / backward chains follow the flows exactly as
//    src/vbm3d.cpp:1122-1167 (the y update reads the flow at the already
//    updated x; stale entries are kept when a frame yields fewer than Nb).
#include "common.cuh"

namespace vbm3d {

struct Win {
    int t, x0, x1, y0, y1;
};

struct WarpBM {
    float* ref;      // C*k*k reference pixels, [c][y][x]
    Pair* list;      // tie fallback list (window candidates in scan order)
    Pair* best;      // bestPatches (src/vbm3d.cpp:1091)
    Pair* fc;        // frameBestPatches (src/vbm3d.cpp:1095)
    Win* wins;       // windows scanned so far
    unsigned* pre;   // tempMatchesPre
    unsigned* post;  // tempMatchesPost
    int nwins;
    int nevals;      // patchDistance evaluations so far (measurement)
};

// patchDistance (src/vbm3d.cpp:930-1011): the reference patch is staged as
// [ht][c][y][x] along its own trajectory; the candidate follows its own.
__device__ __forceinline__ float cand_distance(const StepParams& P, const float* __restrict__ ref,
                                               const float* __restrict__ vid, const float* __restrict__ fflow,
                                               int qx, int qy, int t)
{
    const int k = P.k;
    float s = 0.f;
    if (P.kt > 1) {
        int tx[kMaxKt], ty[kMaxKt];
        trajectory(P, fflow, qx, qy, t, tx, ty);
        for (int ht = 0; ht < P.kt; ht++)
            for (int c = 0; c < P.C; c++) {
                const float* pc = vid + (size_t)(t + ht) * P.whc + (size_t)c * P.wh + (size_t)ty[ht] * P.W + tx[ht];
                const float* rc = ref + (ht * P.C + c) * k * k;
                for (int hy = 0; hy < k; hy++)
                    for (int hx = 0; hx < k; hx++) {
                        const float d = rc[hy * k + hx] - __ldg(pc + (size_t)hy * P.W + hx);
                        s = s + d * d;
                    }
            }
        return s / (float)(k * k * P.kt * P.C);
    }
    const float* base = vid + (size_t)t * P.whc + (size_t)qy * P.W + qx;
    for (int c = 0; c < P.C; c++) {
        const float* pc = base + (size_t)c * P.wh;
        const float* rc = ref + c * k * k;
        for (int hy = 0; hy < k; hy++) {
            const float* row = pc + (size_t)hy * P.W;
            const float* rr = rc + hy * k;
#pragma unroll 4
            for (int hx = 0; hx < k; hx++) {
                const float d = rr[hx] - __ldg(row + hx);
                s = s + d * d;
            }
        }
    }
    return s / (float)(k * k * P.C);
}

// localSearch (src/vbm3d.cpp:1013-1080): scans the window of side `s`
// centred on (cx, cy) in frame t and appends its min(Nb, #unseen) best
// candidates, sorted, to out[nout...].
__device__ void search_window(const StepParams& P, WarpBM& w, const float* __restrict__ vid,
                              const float* __restrict__ fflow, int lane, int t, int cx, int cy, int s, int rx, int ry,
                              Pair* out, int& nout)
{
    const int half = (s - 1) / 2;
    const int x0 = max(0, cx - half), y0 = max(0, cy - half);
    const int x1 = min(P.W - P.k, cx + half), y1 = min(P.H - P.k, cy + half);
    const int ww = x1 - x0 + 1;
    const int n = ww * (y1 - y0 + 1);
    const int nwins = w.nwins;

    float cd[kSlots];
    bool cv[kSlots];
#pragma unroll
    for (int j = 0; j < kSlots; j++) {
        const int pos = j * 32 + lane;
        cv[j] = false;
        cd[j] = 0.f;
        if (pos < n) {
            const int qy = y0 + pos / ww, qx = x0 + pos % ww;
            bool seen = false;
            for (int wi = 0; wi < nwins; wi++) {
                const Win v = w.wins[wi];
                if (v.t == t && qx >= v.x0 && qx <= v.x1 && qy >= v.y0 && qy <= v.y1) {
                    seen = true;
                    break;
                }
            }
            if (!seen) {
                float d = cand_distance(P, w.ref, vid, fflow, qx, qy, t);
                if (qx == rx && qy == ry) d = d - P.dbias;
                cd[j] = d;
                cv[j] = true;
            }
        }
    }
    __syncwarp();
    if (lane == 0) w.wins[nwins] = Win{t, x0, x1, y0, y1};
    w.nwins = nwins + 1;

    int nvalid = 0;
#pragma unroll
    for (int j = 0; j < kSlots; j++) nvalid += __popc(__ballot_sync(kFull, cv[j]));
    const int m = min(P.Nb, nvalid);
    w.nevals += nvalid;

    // Fast path: m rounds of warp argmin; an exact tie anywhere in the
    // selection (including at the m-th place) sends the window to the
    // reference's own selection routine.
    bool tie = false;
    unsigned taken = 0;
    for (int r = 0; r < m; r++) {
        float lmin = 0.f;
        int lj = -1, lcnt = 0;
#pragma unroll
        for (int j = 0; j < kSlots; j++) {
            if (cv[j] && !((taken >> j) & 1u)) {
                if (lj < 0 || cd[j] < lmin) {
                    lmin = cd[j];
                    lj = j;
                    lcnt = 1;
                } else if (cd[j] == lmin) {
                    lcnt++;
                }
            }
        }
        float wmin = lj >= 0 ? lmin : __int_as_float(0x7f800000);
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) wmin = fminf(wmin, __shfl_xor_sync(kFull, wmin, off));
        const int cnt = (lj >= 0 && lmin == wmin) ? lcnt : 0;
        const int tot = __reduce_add_sync(kFull, cnt);
        if (tot != 1) {
            tie = true;
            break;
        }
        const unsigned bal = __ballot_sync(kFull, cnt == 1);
        const int wl = __ffs(bal) - 1;
        const int wj = __shfl_sync(kFull, lj, wl);
        if (lane == wl) taken |= 1u << lj;
        const int pos = wj * 32 + wl;
        const int qy = y0 + pos / ww, qx = x0 + pos % ww;
        if (lane == 0) out[nout + r] = Pair{wmin, patch_index(P, qx, qy, t)};
    }
    if (tie) {
        int base = 0;
        const unsigned lt = (1u << lane) - 1u;
#pragma unroll
        for (int j = 0; j < kSlots; j++) {
            const unsigned bal = __ballot_sync(kFull, cv[j]);
            if (cv[j]) {
                const int pos = j * 32 + lane;
                const int qy = y0 + pos / ww, qx = x0 + pos % ww;
                w.list[base + __popc(bal & lt)] = Pair{cd[j], patch_index(P, qx, qy, t)};
            }
            base += __popc(bal);
        }
        __syncwarp();
        if (lane == 0) {
            partial_sort(w.list, m, base);
            for (int r = 0; r < m; r++) out[nout + r] = w.list[r];
        }
    }
    nout += m;
    __syncwarp();
}

// One prediction step of the forward (dir = +1) or backward (dir = -1)
// chain (src/vbm3d.cpp:1123-1143, :1147-1167).
__device__ void chain_step(const StepParams& P, WarpBM& w, const float* __restrict__ vid,
                           const float* __restrict__ flow, const float* __restrict__ fflow, unsigned* centres, int dir,
                           int lane, int rx, int ry, int& nbest)
{
    const int k = P.k;
    int nfc = 0;
    for (int m = 0; m < P.Nb; m++) {
        int px, py, pt;
        patch_coords(P, centres[m], px, py, pt);
        const int ft = dir > 0 ? pt : pt - 1;  // fflow(.., pt) / bflow(.., pt - 1)
        const float* fl = flow ? flow + (size_t)ft * 2 * P.wh : nullptr;
        const float fx = fl ? __ldg(fl + (size_t)(py + k / 2) * P.W + px + k / 2) : 0.f;
        int nx = (int)((float)px + roundf(fx));
        px = min(max(nx, 0), P.W - k);
        const float fy = fl ? __ldg(fl + P.wh + (size_t)(py + k / 2) * P.W + px + k / 2) : 0.f;
        int ny = (int)((float)py + roundf(fy));
        py = min(max(ny, 0), P.H - k);
        search_window(P, w, vid, fflow, lane, pt + dir, px, py, P.Npr, rx, ry, w.fc, nfc);
    }
    const int m2 = min(P.Nb, nfc);
    if (lane == 0) {
        partial_sort(w.fc, m2, nfc);
        for (int i = 0; i < m2; i++) {
            centres[i] = w.fc[i].i;
            w.best[nbest + i] = w.fc[i];
        }
    }
    nbest += m2;
    __syncwarp();
}

__global__ void __launch_bounds__(128)
bm_kernel(const StepParams P, const float* __restrict__ vid, const float* __restrict__ fflow,
          const float* __restrict__ bflow, unsigned* __restrict__ out_idx,
          float* __restrict__ out_dist, unsigned* __restrict__ out_nsimp,
          unsigned* __restrict__ out_nsx, unsigned long long* __restrict__ out_count)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const long long r = P.ref_base + (long long)blockIdx.x * (blockDim.x >> 5) + wid;
    if (r >= P.nrefs) return;

    unsigned char* ws = smem + (size_t)wid * P.bm_warp_bytes;
    const int k = P.k, k2 = k * k;
    WarpBM w;
    w.ref = reinterpret_cast<float*>(ws);
    size_t off = ((size_t)P.C * P.kt * k2 * sizeof(float) + 15) & ~size_t(15);
    w.list = reinterpret_cast<Pair*>(ws + off);
    off += (size_t)P.bm_list_cap * sizeof(Pair);
    w.best = reinterpret_cast<Pair*>(ws + off);
    off += (size_t)P.bm_best_cap * sizeof(Pair);
    w.fc = reinterpret_cast<Pair*>(ws + off);
    off += (size_t)kMaxNb * kMaxNb * sizeof(Pair);
    w.pre = reinterpret_cast<unsigned*>(ws + off);
    w.post = w.pre + kMaxNb;
    off += 2 * kMaxNb * sizeof(unsigned);
    w.wins = reinterpret_cast<Win*>(ws + off);
    w.nwins = 0;
    w.nevals = 0;

    int rx, ry, rt;
    ref_coords(P, r, rx, ry, rt);
    {
        int tx[kMaxKt], ty[kMaxKt];
        trajectory(P, fflow, rx, ry, rt, tx, ty);
        for (int e = lane; e < P.kt * P.C * k2; e += 32) {
            const int sl = e / k2, pq = e - sl * k2, ht = sl / P.C, c = sl - ht * P.C;
            const int py = pq / k, px = pq - py * k;
            w.ref[e] = __ldg(vid + (size_t)(rt + ht) * P.whc + (size_t)c * P.wh + (size_t)(ty[ht] + py) * P.W +
                             tx[ht] + px);
        }
    }
    __syncwarp();

    int nbest = 0;
    search_window(P, w, vid, fflow, lane, rt, rx, ry, P.Ns, rx, ry, w.best, nbest);
    if (lane < P.Nb) {
        // the reference reads bestPatches[i] for every i < Nb
        // (src/vbm3d.cpp:1115-1119); the host rejects grids where the
        // reference-frame window holds fewer than Nb positions
        w.pre[lane] = w.best[lane].i;
        w.post[lane] = w.best[lane].i;
    }
    __syncwarp();

    const int fend = min(rt + P.Nf, P.F - P.kt) - rt;
    for (int f = 0; f < fend; f++) chain_step(P, w, vid, fflow, fflow, w.post, +1, lane, rx, ry, nbest);
    const int bend = min(rt, P.Nf);
    for (int f = 0; f < bend; f++) chain_step(P, w, vid, bflow, fflow, w.pre, -1, lane, rx, ry, nbest);

    if (lane == 0) {
        const int nsimp = min(P.N, nbest);
        partial_sort(w.best, nsimp, nbest);
        unsigned* oi = out_idx + (size_t)r * P.N;
        for (int i = 0; i < nsimp; i++) oi[i] = w.best[i].i;
        if (out_dist) {
            float* od = out_dist + (size_t)r * P.N;
            for (int i = 0; i < P.N; i++) od[i] = i < nsimp ? w.best[i].d : 0.f;
        }
        for (int i = nsimp; i < P.N; i++) oi[i] = 0xffffffffu;
        int thr = nsimp - 1;
        while (w.best[thr].d > P.tau && thr > 0) thr--;
        unsigned pw = 1;  // closest_power_of_2 (src/Utilities/Utilities.cpp:257-265)
        while (pw * 2 <= (unsigned)(thr + 1)) pw *= 2;
        if (out_nsimp) out_nsimp[r] = (unsigned)nsimp;
        out_nsx[r] = pw;
        if (out_count) atomicAdd(out_count, (unsigned long long)w.nevals);
    }
}

int bm_warp_bytes(const StepParams& P, int& list_cap, int& best_cap, int& win_cap)
{
    const int win = P.Ns > P.Npr ? P.Ns : P.Npr;
    list_cap = win * win;
    best_cap = P.Nb * (1 + 2 * P.Nf);
    win_cap = 1 + 2 * P.Nf * P.Nb;
    size_t off = ((size_t)P.C * P.kt * P.k * P.k * sizeof(float) + 15) & ~size_t(15);
    off += (size_t)list_cap * sizeof(Pair) + (size_t)best_cap * sizeof(Pair);
    off += (size_t)kMaxNb * kMaxNb * sizeof(Pair) + 2 * kMaxNb * sizeof(unsigned);
    off += (size_t)win_cap * sizeof(Win);
    return (int)((off + 15) & ~size_t(15));
}

bool bm2_supported(const StepParams& P);
cudaError_t launch_bm2(const StepParams& P, const float* vid, const float* fflow, const float* bflow,
                       unsigned* out_idx, float* out_dist, unsigned* out_nsimp, unsigned* out_nsx, long long count,
                       cudaStream_t stream);

// The staged kernel (bm2.cu) for the shapes it handles, this one otherwise
// and whenever the distance count is requested.
cudaError_t launch_bm(const StepParams& P, const float* vid, const float* fflow, const float* bflow,
                      unsigned* out_idx, float* out_dist, unsigned* out_nsimp, unsigned* out_nsx,
                      long long count, cudaStream_t stream, unsigned long long* out_count)
{
    if (!out_count && bm2_supported(P))
        return launch_bm2(P, vid, fflow, bflow, out_idx, out_dist, out_nsimp, out_nsx, count, stream);
    const int warps = 4;
    const size_t smem = (size_t)warps * P.bm_warp_bytes;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(bm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    const long long blocks = (count + warps - 1) / warps;
    bm_kernel<<<(unsigned)blocks, warps * 32, smem, stream>>>(P, vid, fflow, bflow, out_idx, out_dist,
                                                            out_nsimp, out_nsx, out_count);
    return cudaGetLastError();
}

}  // namespace vbm3d
