// Staged block matching (see bm2.cu): device code shared by the
// single-video kernel (bm2.cu) and the batched persistent kernels
// (batch_kernels.cuh).
#pragma once

#include "common.cuh"

namespace vbm3d {

// Shared-memory layout of one warp of the staged kernel (bm2_layout).
struct Layout {
    int warp_bytes;   // shared memory per warp
    int tile_floats;  // staged windows
    int res_cap;      // distances of a phase / the final list
    int scr_cap;      // tie fallback scratch (one window), inside the tile area
};

namespace {


struct Win {
    int t, x0, x1, y0, y1;
};

// A window of the current phase.
struct PWin {
    int t, x0, y0, ww, wh;  // clamped window: positions x0..x0+ww-1, y0..y0+wh-1
    int tile;               // float offset of its staged tile
    int res;                // offset of its results in the phase result array
    int chain;              // 0: reference frame, 1: forward, 2: backward
    unsigned base;          // video offset of its top-left pixel in channel 0 (t*whc + y0*W + x0)
    unsigned long long seen;  // earlier windows on the same frame (bit i: scanned window i)
};

static_assert(sizeof(PWin) % 16 == 0, "phase windows stay 8-byte aligned in shared memory");

// Inside the kernel a patch is named by packed coordinates
// ((t - rt + 32) << 26) | (y << 13) | x (x, y < 8192, |t - rt| <= 16),
// which decode without divisions; the output converts them to the
// reference's linear indices.
__device__ __forceinline__ unsigned pack_xyt(int x, int y, int t, int rt)
{
    return ((unsigned)(t - rt + 32) << 26) | ((unsigned)y << 13) | (unsigned)x;
}
__device__ __forceinline__ void unpack_xyt(unsigned v, int rt, int& x, int& y, int& t)
{
    x = (int)(v & 8191u);
    y = (int)((v >> 13) & 8191u);
    t = (int)(v >> 26) - 32 + rt;
}

constexpr unsigned kNone = 0xffffffffu;

// Row pitch (and height) of a staged window tile of side s + k - 1: at
// least 13 and odd, which keeps the rows of a 5-wide window on distinct
// shared-memory banks.
__host__ __device__ __forceinline__ int bm2_pitch(int s, int k)
{
    const int p = s + k - 1;
    return p <= 13 ? 13 : (p | 1);
}

// (a, b) += ((r, r) - (xa, xb))^2 with the rounding of the scalar
// sequence d = r - x; p = d * d; s = s + p.  Three packed f32x2
// operations: subtract, square, add.  The square is fma(d, d, -0.0), which
// rounds d * d once and adds an exact -0.0, so it equals the scalar
// product in every case (including signed zeros).  A packed multiply
// followed by a packed add is contracted into a fused multiply-add below
// the PTX level (a GB300 probe found that pairing changes about half of all
// 192-term sums), so the square must not be a plain multiply; `nz` is -0.0
// read at run time, so that the compiler cannot turn the FMA into one.  A
// GB300 probe found this form equal to the scalar sums in all of 65536
// 192-term sums.
__device__ __forceinline__ void sq_acc2(float& ax, float& ay, float rx, float ry, float xa, float xb, float nz)
{
    asm("{\n\t.reg .b64 r, x, d, p, a, z;\n\t"
        "mov.b64 r, {%2, %3};\n\t"
        "mov.b64 x, {%4, %5};\n\t"
        "mov.b64 z, {%6, %6};\n\t"
        "sub.rn.f32x2 d, r, x;\n\t"
        "fma.rn.f32x2 p, d, d, z;\n\t"
        "mov.b64 a, {%0, %1};\n\t"
        "add.rn.f32x2 a, a, p;\n\t"
        "mov.b64 {%0, %1}, a;\n\t}"
        : "+f"(ax), "+f"(ay)
        : "f"(rx), "f"(ry), "f"(xa), "f"(xb), "f"(nz));
}

struct Smem {
    Pair* scr;     // tie fallback scratch
    float2* refp;  // duplicated reference pixels, rows of bm2_ref_row(k) (padded to even)
    float* tiles;  // staged windows of the phase
    Win* wins;     // every window scanned so far
    PWin* pw;      // windows of the current phase
    Pair* res;     // distances of the phase, per window in scan order (i == kNone: not a candidate)
    Pair* fc;      // [2][Nb*Nb] frame candidates of the forward / backward step
    Pair* best;    // [Nb | Nb*Nf forward | Nb*Nf backward]
    unsigned* cen; // [2][Nb] forward / backward centres (tempMatchesPost / Pre)
    int* cnt;      // per-chain counters
};

__host__ __device__ __forceinline__ size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

// Row length (float2 entries) of the staged reference patch: k rounded up
// to even, so that each 16-byte load brings two duplicated pixels.
__host__ __device__ __forceinline__ int bm2_ref_row(int k) { return (k + 1) & ~1; }

// Number of positions of a window.
__device__ __forceinline__ int npos(const PWin& w) { return w.ww * w.wh; }

// The lanes one reference's block matching runs on: the whole warp
// (G == 32) or one half of it (G == 16, two references per warp).  Every
// collective goes through these members, over the group's lanes only, so
// the two halves of a warp may take different branches (a tie, a shorter
// pass) without waiting for each other.
template <int G>
struct Grp {
    static_assert(G == 16 || G == 32, "a warp or a half warp");
    int gl;         // lane within the group
    unsigned mask;  // the group's lanes
    int base;       // its first lane in the warp
    __device__ __forceinline__ explicit Grp(int lane)
        : gl(lane & (G - 1)), mask(G == 32 ? kFull : 0xffffu << (lane & 16)), base(G == 32 ? 0 : (lane & 16))
    {
    }
    __device__ __forceinline__ void sync() const { __syncwarp(mask); }
    __device__ __forceinline__ unsigned ballot(bool p) const
    {
        return G == 32 ? __ballot_sync(kFull, p) : (__ballot_sync(mask, p) >> base) & 0xffffu;
    }
    __device__ __forceinline__ bool all(bool p) const { return __all_sync(mask, p); }
    __device__ __forceinline__ unsigned sum(unsigned v) const { return __reduce_add_sync(mask, v); }
    __device__ __forceinline__ int sum(int v) const { return __reduce_add_sync(mask, v); }
    __device__ __forceinline__ unsigned minu(unsigned v) const { return __reduce_min_sync(mask, v); }
    template <class T>
    __device__ __forceinline__ T shfl(T v, int src) const
    {
        return __shfl_sync(mask, v, src, G);
    }
    template <class T>
    __device__ __forceinline__ T shfl_xor(T v, int m) const
    {
        return __shfl_xor_sync(mask, v, m, G);
    }
    template <class T>
    __device__ __forceinline__ T shfl_up(T v, int d) const
    {
        return __shfl_up_sync(mask, v, d, G);
    }
};

// The m smallest valid entries of res[0..n) (scan order), sorted into
// out[0..m) by the restatement of the reference's partial_sort on one
// thread: the order among equal distances that std::partial_sort leaves.
__device__ void tie_sort(const Pair* res, int n, int m, Pair* out, Pair* scratch)
{
    int k = 0;
    for (int j = 0; j < n; j++)
        if (res[j].i != kNone) scratch[k++] = res[j];
    partial_sort(scratch, m, k);
    for (int r = 0; r < m; r++) out[r] = scratch[r];
}
template <int G>
__device__ void tie_fallback(const Pair* res, int n, int m, const Grp<G>& g, Pair* out, Pair* scratch)
{
    g.sync();
    if (g.gl == 0) tie_sort(res, n, m, out, scratch);
}

constexpr unsigned kNoKey = 0xffffffffu;   // no entry: above every key
constexpr unsigned kNanKey = 0xfffffffeu;  // a NaN distance (from NaN or Inf pixels): above every number

// An unsigned key with the order of the distance d under float
// comparison (-0 ranks with +0; every NaN is kNanKey), and back (-0 comes
// back as +0, which no distance here is: sums of squares from +0, less a
// bias).
__device__ __forceinline__ unsigned dist_key(float d)
{
    unsigned u = __float_as_uint(d);
    if ((u & 0x7fffffffu) > 0x7f800000u) return kNanKey;
    if (u == 0x80000000u) u = 0u;
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float key_dist(unsigned k)
{
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

// Top-min(Nb, #valid) of window w (distances in S.res[w.res ...], scan
// order), appended sorted to out[*nout]: localSearch's partial_sort
// (src/vbm3d.cpp:1075-1079).
template <int G>
__device__ void select_window(const StepHead& P, const Smem& S, const PWin& w, const Grp<G>& g, Pair* out,
                              int& nout, Pair* scratch)
{
    const int n = npos(w);
    const Pair* res = S.res + w.res;
    if (n <= 64) {
        // up to 64 / G entries per lane, as keys: each rank is one group
        // minimum, and a rank held by two entries is a tie.  Every valid
        // entry counts towards m and has a key below kNoKey, so each of
        // the m ranks finds one; a NaN at a rank goes to the restatement
        // of partial_sort, as a tie does
        constexpr int E = 64 / G;
        unsigned k[E], ix[E];
        unsigned mine = 0;
#pragma unroll
        for (int e = 0; e < E; e++) {
            const int j = g.gl + G * e;
            k[e] = kNoKey;
            ix[e] = 0;
            if (j < n) {
                const Pair q = res[j];
                if (q.i != kNone) {
                    k[e] = dist_key(q.d);
                    ix[e] = q.i;
                    mine++;
                }
            }
        }
        const int m = min(P.Nb, (int)g.sum(mine));
        bool tie = false;
        for (int r = 0; r < m; r++) {
            unsigned lm = k[0];
#pragma unroll
            for (int e = 1; e < E; e++) lm = min(lm, k[e]);
            const unsigned wmin = g.minu(lm);
            unsigned c = 0;
#pragma unroll
            for (int e = 0; e < E; e++) c += k[e] == wmin ? 1u : 0u;
            if (wmin == kNanKey || g.sum(c) != 1u) {
                tie = true;
                break;
            }
#pragma unroll
            for (int e = 0; e < E; e++)
                if (k[e] == wmin) {
                    out[nout + r] = Pair{key_dist(wmin), ix[e]};
                    k[e] = kNoKey;
                }
        }
        if (tie) tie_fallback(res, n, m, g, out + nout, scratch);
        nout += m;
        g.sync();
        return;
    }
    int nvalid = 0;
    for (int j0 = 0; j0 < n; j0 += G) {
        const int j = j0 + g.gl;
        nvalid += __popc(g.ballot(j < n && res[j].i != kNone));
    }
    const int m = min(P.Nb, nvalid);
    bool tie = false;
    // fast path: exact ranks of the m smallest
    float last = -__int_as_float(0x7f800000);
    for (int r = 0; r < m; r++) {
        // smallest distance strictly above `last`
        float lmin = __int_as_float(0x7f800000);
        int lj = -1, lcnt = 0;
        for (int j = g.gl; j < n; j += G) {
            const Pair e = res[j];
            if (e.i == kNone || !(e.d > last)) continue;
            if (lj < 0 || e.d < lmin) {
                lmin = e.d;
                lj = j;
                lcnt = 1;
            } else if (e.d == lmin) {
                lcnt++;
            }
        }
        float wmin = lmin;
#pragma unroll
        for (int off = G / 2; off > 0; off >>= 1) wmin = fminf(wmin, g.shfl_xor(wmin, off));
        const int c = (lj >= 0 && lmin == wmin) ? lcnt : 0;
        const int tot = g.sum(c);
        if (tot != 1) {
            tie = true;
            break;
        }
        const unsigned bal = g.ballot(c == 1);
        const int wl = __ffs(bal) - 1;
        const int wj = g.shfl(lj, wl);
        if (g.gl == 0) out[nout + r] = res[wj];
        last = wmin;
    }
    if (tie) tie_fallback(res, n, m, g, out + nout, scratch);
    nout += m;
    g.sync();
}

// Sorted smallest `m` of a[0..n) written to out (std::partial_sort order):
// exact ranks (EP entries per lane, EP = 1 for a warp, 2 for a half warp)
// when all keys of the prefix are distinct, else the restatement of the
// reference's routine on one lane.
template <int G>
__device__ void small_partial_sort(Pair* a, int m, int n, const Grp<G>& g)
{
    constexpr int EP = G == 32 ? 1 : 2;
    if (n > EP * G) {
        if (g.gl == 0) partial_sort(a, m, n);
        g.sync();
        return;
    }
    bool ok = true;
    int rank[EP];
    Pair mine[EP];
#pragma unroll
    for (int e = 0; e < EP; e++) {
        const int j = g.gl + G * e;
        rank[e] = 0;
        mine[e] = Pair{0.f, 0};
        if (j < n) {
            mine[e] = a[j];
            for (int i = 0; i < n; i++) {
                const float d = a[i].d;
                if (d < mine[e].d) rank[e]++;
                else if (d == mine[e].d && i != j) ok = false;
            }
        }
    }
    // ties among entries that cannot reach the prefix do not matter, but
    // keep it simple: any tie sends the list to the exact routine
    ok = g.all(ok);
    g.sync();
    if (ok) {
#pragma unroll
        for (int e = 0; e < EP; e++)
            if (g.gl + G * e < n && rank[e] < m) a[rank[e]] = mine[e];  // distinct ranks: a permutation of the prefix
    } else if (g.gl == 0) {
        partial_sort(a, m, n);
    }
    g.sync();
}

// select_window for every window of a phase at once (nw <= G / GS, each
// window at most 32 positions): window w on the GS lanes of subgroup w of
// the group, up to 32 / GS entries per lane, each rank one subgroup minimum
// of the keys and one subgroup count of the entries holding it.  The picks
// of the windows of a chain are appended in window order to the chain's
// frame candidates (S.fc: forward chain first), as the per-window calls
// append them; nfc_f and nfc_b count them.  Windows with a tie (or a NaN)
// at a rank go, one at a time, to the partial_sort restatement on their
// subgroup's first lane.
template <int GS, int G>
__device__ void select_phase(const StepHead& P, const Smem& S, int nw, bool fa, const Grp<G>& g, int& nfc_f,
                             int& nfc_b)
{
    constexpr int E = 32 / GS, NS = G / GS;
    const int Nb = P.Nb;
    const int w = g.gl / GS, sl = g.gl & (GS - 1);
    int n = 0, res = 0;
    if (w < nw) {
        const PWin& W = S.pw[w];
        n = W.ww * W.wh;
        res = W.res;
    }
    unsigned key[E], idx[E];
    unsigned nv = 0;
#pragma unroll
    for (int i = 0; i < E; i++) {
        const int j = sl + GS * i;
        key[i] = kNoKey;
        idx[i] = 0;
        if (j < n) {
            const Pair e = S.res[res + j];
            if (e.i != kNone) {
                key[i] = dist_key(e.d);
                idx[i] = e.i;
                nv++;
            }
        }
    }
#pragma unroll
    for (int o = GS / 2; o > 0; o >>= 1) nv += g.shfl_xor(nv, o);
    const int m = min(Nb, (int)nv);  // 0 for the subgroups past nw
    // the window's chain (forward: windows 0 .. Nb-1 when the forward
    // chain is active) and its offset among the chain's candidates
    const bool fwd = fa && w < Nb;
    const int c0 = fwd ? 0 : (fa ? Nb : 0);
    int off = 0, nf = 0, nb = 0;
#pragma unroll
    for (int v = 0; v < NS; v++) {
        const int mv = g.shfl(m, v * GS);
        if (fa && v < Nb) nf += mv;
        else nb += mv;
        if (v >= c0 && v < w) off += mv;
    }
    Pair* out = S.fc + (fwd ? 0 : Nb * Nb) + off;
    bool tie = false;
    for (int r = 0; r < Nb; r++) {
        unsigned gmin = key[0];
#pragma unroll
        for (int i = 1; i < E; i++) gmin = min(gmin, key[i]);
#pragma unroll
        for (int o = GS / 2; o > 0; o >>= 1) gmin = min(gmin, (unsigned)g.shfl_xor(gmin, o));
        unsigned c = 0;
#pragma unroll
        for (int i = 0; i < E; i++) c += key[i] == gmin ? 1u : 0u;
        unsigned cs = c;
#pragma unroll
        for (int o = GS / 2; o > 0; o >>= 1) cs += g.shfl_xor(cs, o);
        if (tie || r >= m) continue;  // uniform over the subgroup
        if (gmin == kNanKey || cs != 1u) {
            tie = true;
            continue;
        }
#pragma unroll
        for (int i = 0; i < E; i++)
            if (key[i] == gmin) {
                out[r] = Pair{key_dist(gmin), idx[i]};
                key[i] = kNoKey;
            }
    }
    g.sync();
    for (unsigned tb = g.ballot(sl == 0 && tie); tb; tb &= tb - 1) {
        if (g.gl == __ffs(tb) - 1) tie_sort(S.res + res, n, m, out, S.scr);
        g.sync();
    }
    nfc_f = nf;
    nfc_b = nb;
}

// Float offset of the staged tile of window w of a phase whose tiles hold
// tile_sz floats: windows are paired (0, 1), (2, 3), ..., and each pair
// starts one float past a 32-float boundary after the previous one, so the
// two pairs read by one pass fall on disjoint banks.
__host__ __device__ __forceinline__ int bm2_pair_stride(int tile_sz) { return ((2 * tile_sz + 31) & ~31) + 1; }
__host__ __device__ __forceinline__ int bm2_tile_offset(int w, int tile_sz)
{
    return (w >> 1) * bm2_pair_stride(tile_sz) + (w & 1) * tile_sz;
}

// acc / norm rounded once, for this kernel's distance normalisations
// (norm = k^2 C, one of 49, 64, 147, 192): q = acc * rcp with rcp the
// rounded reciprocal, then Markstein's correction step with the exact
// remainder acc - q norm (one FMA), q + (acc - q norm) rcp.  For these four
// divisors the result equals the IEEE quotient acc / norm for every float
// acc >= 2^-100 (tests/test_div_norm.py checks all of them); smaller,
// infinite and NaN sums take the division itself.
__device__ __forceinline__ float div_norm(float acc, float norm, float rcp)
{
    if (!(acc >= 0x1p-100f && acc <= 3.40282347e38f)) return __fdiv_rn(acc, norm);
    const float q = __fmul_rn(acc, rcp);
    const float r = __fmaf_rn(-q, norm, acc);
    return __fmaf_rn(r, rcp, q);
}

// One phase entry: position (dy, cx) of window W with squared-difference
// sum acc, unless it lies outside the window; an entry seen in an earlier
// window of the same frame is stored as not a candidate (i == kNone).
__device__ __forceinline__ void store_entry(const StepHead& P, const Smem& S, const PWin& W, int dy, int cx,
                                            float acc, float norm, float rcp, int rx, int ry, int rt)
{
    if (dy >= W.wh || cx >= W.ww) return;
    const int qx = W.x0 + cx, qy = W.y0 + dy;
    bool seen = false;
    for (unsigned long long m = W.seen; m; m &= m - 1) {
        const Win v = S.wins[__ffsll((long long)m) - 1];
        if (qx >= v.x0 && qx <= v.x1 && qy >= v.y0 && qy <= v.y1) {
            seen = true;
            break;
        }
    }
    Pair e{0.f, kNone};
    if (!seen) {
        float d = div_norm(acc, norm, rcp);
        if (qx == rx && qy == ry) d = d - P.dbias;
        e = Pair{d, pack_xyt(qx, qy, W.t, rt)};
    }
    S.res[W.res + dy * W.ww + cx] = e;
}

// Distances of every position of the phase's nw windows.  Windows are
// taken in pairs (0, 1), (2, 3), ...; a lane owns one slot (dy, 2cx) of a
// pair and evaluates positions (dy, 2cx) and (dy, 2cx + 1) of both windows
// (4 candidates): per row of the patch it loads K + 1 staged pixels of
// each window and the K reference pixels once, and the two windows share
// each packed f32x2 operation.  An odd last window runs in passes of its
// own, a lane evaluating positions (dy, 2cx) and (dy, 2cx + 1) of it as the
// packed pair.  A pass covers G slots.  Every distance is the reference's
// sequential sum over (c, hy, hx).  Only the slot (window, dy, dx) is live
// across the sums; the windows' fields are read again for the results.
template <int K, int C, int G>
__device__ void phase_distances(const StepHead& P, const Smem& S, int nw, const Grp<G>& g, int rx, int ry, int rt,
                                int pitch, int plane)
{
    constexpr int KK = K * K, KR = (K + 1) & ~1;  // KR: bm2_ref_row(K)
    const int npairs = nw >> 1;
    // pair `gl` (lanes < npairs): `cols` slot columns (ceil(max ww / 2)),
    // max wh rows; pend = one past its last slot (inclusive scan)
    int cols = 1, slots = 0;
    if (g.gl < npairs) {
        const PWin& A = S.pw[2 * g.gl];
        const PWin& B = S.pw[2 * g.gl + 1];
        cols = (max(A.ww, B.ww) + 1) >> 1;
        slots = max(A.wh, B.wh) * cols;
    }
    int pend = slots;
#pragma unroll
    for (int o = 1; o < kMaxNb; o <<= 1) {
        const int v = g.shfl_up(pend, o);
        if (g.gl >= o) pend += v;
    }
    const int total = npairs > 0 ? g.shfl(pend, npairs - 1) : 0;
    const int pair_passes = (total + G - 1) / G;
    int lone_cols = 1, lone_slots = 0;
    if (nw & 1) {
        const PWin& L = S.pw[nw - 1];
        lone_cols = (L.ww + 1) >> 1;
        lone_slots = L.wh * lone_cols;
    }
    const int passes = pair_passes + (lone_slots + G - 1) / G;
    const float nz = P.neg_zero;
    const float norm = (float)(KK * C);
    const float rcp = __frcp_rn(norm);

    for (int pass = 0; pass < passes; pass++) {
        const bool pm = pass < pair_passes;  // uniform over the group
        const int sl = (pm ? pass : pass - pair_passes) * G + g.gl;
        // the lane's slot: window wa (pairs: and wa + 1), row dy, column dx
        int wa = nw - 1, j = sl, limit = lone_slots, cp = lone_cols;
        if (pm) {
            int p = 0;
            for (int q = 0; q + 1 < npairs; q++) p += sl >= g.shfl(pend, q) ? 1 : 0;
            const int e = g.shfl(pend, p), n = g.shfl(slots, p);
            cp = g.shfl(cols, p);
            wa = 2 * p;
            j = sl - (e - n);
            limit = n;
        }
        const bool act = j < limit;
        // row of slot j: (j + 0.5) / cp lies at least 0.5 / cp from an
        // integer, and the approximate reciprocal (2 ulp) moves it by less
        // for every j < 2^20, so the truncation is exact
        const int dy = act ? (int)(((float)j + 0.5f) * __fdividef(1.0f, (float)cp)) : 0;
        const int dx = act ? 2 * (j - dy * cp) : 0;
        const int roff = dy * pitch + dx;
        const float* tA = S.tiles + (act ? S.pw[wa].tile + roff : 0);
        const float* tB = S.tiles + (act && pm ? S.pw[wa + 1].tile + roff : 0);
        float a0x = 0.f, a0y = 0.f, a1x = 0.f, a1y = 0.f;
        if (pm) {
#pragma unroll 1
            for (int c = 0; c < C; c++) {
                const float* pa = tA + c * plane;
                const float* pb = tB + c * plane;
                const float4* rr = reinterpret_cast<const float4*>(S.refp + c * K * KR);
#pragma unroll 1
                for (int hy = 0; hy < K; hy++) {
                    float va[K + 1], vb[K + 1];
#pragma unroll
                    for (int x = 0; x <= K; x++) {
                        va[x] = pa[hy * pitch + x];
                        vb[x] = pb[hy * pitch + x];
                    }
                    // terms hx, hx + 1 of both accumulators, in order
#pragma unroll
                    for (int hx = 0; hx < K; hx += 2) {
                        const float4 r4 = rr[(hy * KR + hx) >> 1];
                        sq_acc2(a0x, a0y, r4.x, r4.y, va[hx], vb[hx], nz);
                        sq_acc2(a1x, a1y, r4.x, r4.y, va[hx + 1], vb[hx + 1], nz);
                        if (hx + 1 < K) {
                            sq_acc2(a0x, a0y, r4.z, r4.w, va[hx + 1], vb[hx + 1], nz);
                            sq_acc2(a1x, a1y, r4.z, r4.w, va[hx + 2], vb[hx + 2], nz);
                        }
                    }
                }
            }
        } else {
#pragma unroll 1
            for (int c = 0; c < C; c++) {
                const float* pa = tA + c * plane;
                const float4* rr = reinterpret_cast<const float4*>(S.refp + c * K * KR);
#pragma unroll 1
                for (int hy = 0; hy < K; hy++) {
                    float va[K + 1];
#pragma unroll
                    for (int x = 0; x <= K; x++) va[x] = pa[hy * pitch + x];
#pragma unroll
                    for (int hx = 0; hx < K; hx += 2) {
                        const float4 r4 = rr[(hy * KR + hx) >> 1];
                        sq_acc2(a0x, a0y, r4.x, r4.y, va[hx], va[hx + 1], nz);
                        if (hx + 1 < K) sq_acc2(a0x, a0y, r4.z, r4.w, va[hx + 1], va[hx + 2], nz);
                    }
                }
            }
        }
        if (act) {
            // pairs: (A dx, B dx, A dx+1, B dx+1) -> (a0x, a0y, a1x, a1y);
            // lone: (A dx, A dx+1) -> (a0x, a0y)
            const PWin A = S.pw[wa];
            store_entry(P, S, A, dy, dx, a0x, norm, rcp, rx, ry, rt);
            if (pm) {
                const PWin B = S.pw[wa + 1];
                store_entry(P, S, B, dy, dx, a0y, norm, rcp, rx, ry, rt);
                store_entry(P, S, A, dy, dx + 1, a1x, norm, rcp, rx, ry, rt);
                store_entry(P, S, B, dy, dx + 1, a1y, norm, rcp, rx, ry, rt);
            } else {
                store_entry(P, S, A, dy, dx + 1, a0y, norm, rcp, rx, ry, rt);
            }
        }
    }
    g.sync();
}

// Stages window tiles: rows y0 .. y0+wh+K-2, columns x0 .. x0+ww+K-2, all
// channels, at tile pitch `pitch`.  A warp copies two rows of a tile up to
// 16 wide per step, a half warp one row (16 columns) per step.  (Staging
// channel by channel, one cp.async group each, with every channel's sums
// starting when its copies land, measured 4-5 % slower on the RGB batch
// launches: the per-window set-up then runs once per channel.)
template <int K, int C, int G>
__device__ void stage_tiles(const StepHead& P, const Smem& S, const float* __restrict__ vid, int nw, const Grp<G>& g,
                            int pitch, int plane)
{
    // every tile row of every window is copied asynchronously, then waited
    // for once: the loads of the whole phase are in flight together.  The
    // clip's geometry is read into registers before the first copy; video
    // offsets fit 32 bits (W * H * F * C < 2^32).
    const unsigned W = (unsigned)P.W, wh = P.wh;
    const unsigned tiles = smem_addr(S.tiles);
    // a warp's tiles of at most 16 x 14 (the default windows): lane (column
    // gl & 15, first row gl >> 4) copies rows y0, y0 + 2, ... of every
    // channel in one unrolled, predicated sequence (RGB launches -1 %; for
    // half warps the loop below measured faster)
    constexpr int kRows = 7;
    for (int w = 0; w < nw; w++) {
        const PWin pwn = S.pw[w];
        const int tw = pwn.ww + K - 1, th = pwn.wh + K - 1;
        if (G == 32 && tw <= 16 && th <= 2 * kRows) {
            const int x = g.gl & 15, y0 = g.gl >> 4;
            if (x < tw) {
                const float* src = vid + (pwn.base + (unsigned)y0 * W + (unsigned)x);
                const unsigned dst = tiles + 4u * (unsigned)(pwn.tile + y0 * pitch + x);
#pragma unroll
                for (int c = 0; c < C; c++)
#pragma unroll
                    for (int i = 0; i < kRows; i++)
                        if (y0 + 2 * i < th)
                            cp_async4s_nc(dst + 4u * (unsigned)(c * plane + 2 * i * pitch),
                                          src + ((unsigned)c * wh + 2u * (unsigned)i * W));
            }
            continue;
        }
        int x0 = g.gl, ystep = 1, y0 = 0, xstep = G;
        if (G == 32 && tw <= 16) {
            x0 = g.gl & 15;
            ystep = 2;
            y0 = g.gl >> 4;
        }
        for (int x = x0; x < tw; x += xstep) {
            const unsigned src = pwn.base + (unsigned)y0 * W + (unsigned)x;
            const unsigned dst = tiles + 4u * (unsigned)(pwn.tile + y0 * pitch + x);
            const unsigned sstep = (unsigned)ystep * W;
            const unsigned dstep = 4u * (unsigned)(ystep * pitch);
#pragma unroll 1
            for (int c = 0; c < C; c++) {
                const float* s = vid + (src + (unsigned)c * wh);
                unsigned d = dst + 4u * (unsigned)(c * plane);
#pragma unroll 4
                for (int y = y0; y < th; y += ystep, s += sstep, d += dstep) cp_async4s(d, s);
            }
            if (G == 32 && tw <= 16) break;  // the two half warps cover the 16 columns
        }
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
    g.sync();
}

// Registers the phase's windows in the list of scanned windows (after the
// phase's seen masks were computed against the earlier ones).
template <int G>
__device__ void register_windows(const Smem& S, int nw, const Grp<G>& g)
{
    const int n0 = S.cnt[2];
    if (g.gl < nw) {
        const PWin pwn = S.pw[g.gl];
        S.wins[n0 + g.gl] = Win{pwn.t, pwn.x0, pwn.x0 + pwn.ww - 1, pwn.y0, pwn.y0 + pwn.wh - 1};
    }
    g.sync();
    if (g.gl == 0) S.cnt[2] = n0 + nw;
    g.sync();
}

// The clamped window of side s around (cx, cy) (src/vbm3d.cpp:1045-1053).
__device__ __forceinline__ PWin make_window(const StepHead& P, int t, int cx, int cy, int s, int chain)
{
    const int half = (s - 1) / 2;
    const int x0 = max(0, cx - half), y0 = max(0, cy - half);
    const int x1 = min(P.W - P.k, cx + half), y1 = min(P.H - P.k, cy + half);
    PWin w;
    w.t = t;
    w.x0 = x0;
    w.y0 = y0;
    w.ww = x1 - x0 + 1;
    w.wh = y1 - y0 + 1;
    w.chain = chain;
    w.tile = 0;
    w.res = 0;
    w.base = (unsigned)t * P.whc + (unsigned)y0 * (unsigned)P.W + (unsigned)x0;
    w.seen = 0ull;
    return w;
}

// Block matching of reference patch r by the G lanes of group g (a warp,
// or half of one), with the group's shared-memory region ws laid out by L.
template <int K, int C, int G>
__device__ __forceinline__ void bm2_ref(const StepHead& P, const Layout& L, long long r, unsigned char* ws,
                                        const Grp<G>& g, const float* __restrict__ vid,
                                        const float* __restrict__ fflow, const float* __restrict__ bflow,
                                        unsigned* __restrict__ out_idx, float* __restrict__ out_dist,
                                        unsigned* __restrict__ out_nsimp, unsigned* __restrict__ out_nsx)
{
    constexpr int KK = K * K;
    const int Nb = P.Nb;
    const int gl = g.gl;
    Smem S;
    size_t off = 0;
    S.refp = reinterpret_cast<float2*>(ws + off);
    off = align16(off + sizeof(float2) * C * K * bm2_ref_row(K));
    S.tiles = reinterpret_cast<float*>(ws + off);
    off = align16(off + sizeof(float) * L.tile_floats);
    S.res = reinterpret_cast<Pair*>(ws + off);
    off = align16(off + sizeof(Pair) * L.res_cap);
    // the tie fallback's scratch shares the tile area: ties are sorted after
    // a phase's distances, and the next phase stages its tiles afterwards
    S.scr = reinterpret_cast<Pair*>(S.tiles);
    S.fc = reinterpret_cast<Pair*>(ws + off);
    off = align16(off + sizeof(Pair) * 2 * Nb * Nb);
    S.best = reinterpret_cast<Pair*>(ws + off);
    off = align16(off + sizeof(Pair) * P.bm_best_cap);
    S.wins = reinterpret_cast<Win*>(ws + off);
    off = align16(off + sizeof(Win) * P.bm_win_cap);
    S.pw = reinterpret_cast<PWin*>(ws + off);
    off = align16(off + sizeof(PWin) * 2 * Nb);
    S.cen = reinterpret_cast<unsigned*>(ws + off);
    off = align16(off + sizeof(unsigned) * 2 * kMaxNb);
    S.cnt = reinterpret_cast<int*>(ws + off);  // [0..2]: counters, [3..]: windows before phase window w

    int rx, ry, rt;
    ref_coords(P, r, rx, ry, rt);
    for (int e = gl; e < C * KK; e += G) {
        const int c = e / KK, pq = e - c * KK, py = pq / K, px = pq - py * K;
        const float v = __ldg(vid + (size_t)rt * P.whc + (size_t)c * P.wh + (size_t)(ry + py) * P.W + rx + px);
        S.refp[(c * K + py) * bm2_ref_row(K) + px] = make_float2(v, v);
    }
    if (gl == 0) {
        S.cnt[2] = 0;  // windows scanned
    }
    g.sync();

    // ---- phase 0: the reference frame (src/vbm3d.cpp:1114-1119)
    {
        const int pitch = bm2_pitch(P.Ns, K), plane = pitch * (P.Ns + K - 1);
        if (gl == 0) {
            PWin w = make_window(P, rt, rx, ry, P.Ns, 0);
            S.pw[0] = w;
            S.cnt[3] = 0;
        }
        g.sync();
        stage_tiles<K, C>(P, S, vid, 1, g, pitch, plane);
        phase_distances<K, C>(P, S, 1, g, rx, ry, rt, pitch, plane);
        register_windows(S, 1, g);
        int n0 = 0;
        select_window(P, S, S.pw[0], g, S.best, n0, S.scr);
        if (gl < Nb) {
            // the reference reads Nb entries here (src/vbm3d.cpp:1115-1119);
            // the host rejects grids whose corner window holds fewer
            S.cen[gl] = S.best[gl].i;          // forward chain centres
            S.cen[kMaxNb + gl] = S.best[gl].i; // backward chain centres
        }
        g.sync();
    }

    const int fend = min(rt + P.Nf, P.F - P.kt) - rt;
    const int bend = min(rt, P.Nf);
    const int nphase = max(fend, bend);
    int nbf = 0, nbb = 0;  // picks of the forward / backward chains so far
    Pair* bestf = S.best + Nb;
    Pair* bestb = S.best + Nb + Nb * P.Nf;
    const int pitch = bm2_pitch(P.Npr, K), plane = pitch * (P.Npr + K - 1);
    const int tile_sz = C * plane;
    for (int f = 1; f <= nphase; f++) {
        // windows of this phase, one per lane (nw <= 2 kMaxNb <= G): forward
        // step f (src/vbm3d.cpp:1126-1133), then backward step f (:1150-1157)
        const bool fa = f <= fend, ba = f <= bend;
        const int nw = (fa ? Nb : 0) + (ba ? Nb : 0);
        {
            PWin w;
            int n = 0;
            if (gl < nw) {
                const int chain = (fa && gl < Nb) ? 1 : 2;
                const int m = chain == 1 ? gl : gl - (fa ? Nb : 0);
                int px, py, pt;
                unpack_xyt(S.cen[(chain - 1) * kMaxNb + m], rt, px, py, pt);
                const float* flow = chain == 1 ? fflow : bflow;
                const int ft = chain == 1 ? pt : pt - 1;  // fflow(.., pt) / bflow(.., pt - 1)
                const float* fl = flow ? flow + (size_t)ft * 2 * P.wh : nullptr;
                const float fx = fl ? __ldg(fl + (size_t)(py + K / 2) * P.W + px + K / 2) : 0.f;
                px = min(max((int)((float)px + roundf(fx)), 0), P.W - K);
                const float fy = fl ? __ldg(fl + P.wh + (size_t)(py + K / 2) * P.W + px + K / 2) : 0.f;
                py = min(max((int)((float)py + roundf(fy)), 0), P.H - K);
                w = make_window(P, chain == 1 ? pt + 1 : pt - 1, px, py, P.Npr, chain);
                w.tile = bm2_tile_offset(gl, tile_sz);
                n = npos(w);
            }
            // exclusive prefix sum of the window sizes: result offsets
            int incl = n;
#pragma unroll
            for (int o = 1; o < G; o <<= 1) {
                const int v = g.shfl_up(incl, o);
                if (gl >= o) incl += v;
            }
            if (gl < nw) {
                w.res = incl - n;
                S.pw[gl] = w;
                S.cnt[3 + gl] = S.cnt[2] + gl;  // earlier windows: all registered + earlier in this phase
            }
            g.sync();
        }
        // this phase's windows must be visible to the seen test of later
        // windows of the same phase: register them first, then test each
        // window against the windows registered before it (S.cnt[3 + w])
        register_windows(S, nw, g);
        // seen masks: windows registered before each one, on its frame (up
        // to 64 windows, G per ballot)
        for (int w = 0; w < nw; w++) {
            const int lim = S.cnt[3 + w], wt = S.pw[w].t;
            unsigned long long bits = 0ull;
#pragma unroll
            for (int c = 0; c < 64 / G; c++) {
                const int wi = gl + G * c;
                bits |= (unsigned long long)g.ballot(wi < lim && S.wins[wi].t == wt) << (G * c);
            }
            if (gl == 0) S.pw[w].seen = bits;
        }
        g.sync();
        stage_tiles<K, C>(P, S, vid, nw, g, pitch, plane);
        phase_distances<K, C>(P, S, nw, g, rx, ry, rt, pitch, plane);

        // per chain: top-Nb of each window, then of their union
        int nfc2[2] = {0, 0};
        if (nw <= 4 && P.Npr * P.Npr <= 32) {
            if (nw <= 2) select_phase<G / 2>(P, S, nw, fa, g, nfc2[0], nfc2[1]);
            else select_phase<G / 4>(P, S, nw, fa, g, nfc2[0], nfc2[1]);
        } else {
            int w0 = 0;
            for (int chain = 1; chain <= 2; chain++) {
                if ((chain == 1 && f > fend) || (chain == 2 && f > bend)) continue;
                for (int m = 0; m < Nb; m++)
                    select_window(P, S, S.pw[w0 + m], g, S.fc + (chain - 1) * Nb * Nb, nfc2[chain - 1], S.scr);
                w0 += Nb;
            }
        }
        for (int chain = 1; chain <= 2; chain++) {
            if ((chain == 1 && f > fend) || (chain == 2 && f > bend)) continue;
            Pair* fc = S.fc + (chain - 1) * Nb * Nb;
            const int nfc = nfc2[chain - 1];
            const int m2 = min(Nb, nfc);
            small_partial_sort(fc, m2, nfc, g);
            Pair* dst = chain == 1 ? bestf + nbf : bestb + nbb;
            if (gl < m2) {
                S.cen[(chain - 1) * kMaxNb + gl] = fc[gl].i;
                dst[gl] = fc[gl];
            }
            if (chain == 1) nbf += m2;
            else nbb += m2;
            g.sync();
        }
    }

    // final selection (src/vbm3d.cpp:1169-1184): frame-t picks, forward picks,
    // backward picks, in that order
    Pair* lst = S.res;
    const int nb0 = Nb;  // frame-t picks: exactly Nb (the host validates the corner window)
    const int nbest = nb0 + nbf + nbb;
    for (int j = gl; j < nbest; j += G) {
        Pair e;
        if (j < nb0) e = S.best[j];
        else if (j < nb0 + nbf) e = bestf[j - nb0];
        else e = bestb[j - nb0 - nbf];
        lst[j] = e;
    }
    g.sync();
    const int nsimp = min(P.N, nbest);
    small_partial_sort(lst, nsimp, nbest, g);
    for (int j = gl; j < P.N; j += G) {
        unsigned oi = kNone;
        if (j < nsimp) {
            int x, y, t;
            unpack_xyt(lst[j].i, rt, x, y, t);
            oi = patch_index(P, x, y, t);
        }
        out_idx[(size_t)r * P.N + j] = oi;
        if (out_dist) out_dist[(size_t)r * P.N + j] = j < nsimp ? lst[j].d : 0.f;
    }
    if (gl == 0) {
        int thr = nsimp - 1;
        while (lst[thr].d > P.tau && thr > 0) thr--;
        unsigned pw2 = 1;
        while (pw2 * 2 <= (unsigned)(thr + 1)) pw2 *= 2;
        if (out_nsimp) out_nsimp[r] = (unsigned)nsimp;
        out_nsx[r] = pw2;
    }
}

}  // namespace

// Shared-memory layout of the staged kernel; warp_bytes == 0 when the
// shape is not handled by it.
inline Layout bm2_layout(const StepHead& P)
{
    Layout L{0, 0, 0, 0};
    if (!((P.k == 7 || P.k == 8) && (P.C == 1 || P.C == 3) && P.kt == 1 && P.bm_win_cap <= 64 && P.W <= 8192 &&
          P.H <= 8192 && P.Nf <= 16))
        return L;
    const int p0 = bm2_pitch(P.Ns, P.k), p1 = bm2_pitch(P.Npr, P.k);
    // phase 0: one Ns window; phase f: up to 2 Nb Npr windows in pairs; plus
    // the one-column over-read of the last slot of an odd-width window
    L.scr_cap = max(P.Ns * P.Ns, P.Npr * P.Npr);
    // (the tile area also holds the tie fallback's scratch of scr_cap pairs)
    L.tile_floats = max(max(P.C * p0 * (P.Ns + P.k - 1), P.Nb * bm2_pair_stride(P.C * p1 * (P.Npr + P.k - 1))) + 8,
                        2 * L.scr_cap);
    L.tile_floats = (L.tile_floats + 3) & ~3;
    L.res_cap = max(max(P.Ns * P.Ns, 2 * P.Nb * P.Npr * P.Npr), P.Nb * (1 + 2 * P.Nf));
    // the same sequence of 16-byte aligned regions as the kernel
    size_t off = align16(sizeof(float2) * P.C * P.k * bm2_ref_row(P.k));
    off = align16(off + sizeof(float) * L.tile_floats);
    off = align16(off + sizeof(Pair) * L.res_cap);
    off = align16(off + sizeof(Pair) * 2 * P.Nb * P.Nb);
    off = align16(off + sizeof(Pair) * P.bm_best_cap);
    off = align16(off + sizeof(Win) * P.bm_win_cap);
    off = align16(off + sizeof(PWin) * 2 * P.Nb);
    off = align16(off + sizeof(unsigned) * 2 * kMaxNb);
    off = align16(off + sizeof(int) * (3 + 2 * kMaxNb));
    // one-channel patches run two per warp, and the two half warps' shared
    // loads are one instruction: their workspaces 16 banks apart (stride
    // = 64 mod 128 bytes) put the second half's window loads, whose 15
    // addresses per half sit on the banks of the odd-pitch pattern, on
    // banks the first half's use for two lanes at most, and its 16-byte
    // reference loads on other banks
    if (P.C == 1)
        while ((off & 127) != 64) off += 16;
    if (off > 24 * 1024) return L;
    L.warp_bytes = (int)off;
    return L;
}

}  // namespace vbm3d
