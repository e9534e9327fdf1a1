// Device helpers shared by the filtering kernels (filter.cu), the batched
// work kernels (batch_kernels.cuh) and the linearised / adjoint kernels
// (linear.cu).
#pragma once

#include "common.cuh"

namespace vbm3d {

// ---------------------------------------------------------------- 1D ---

// haar_forward / haar_inverse (src/lib_transforms.cpp:453-512).  EXACT:
// the reference's (float)((double)s * SQRT2_INV) rounding (mul_sqrt2_inv),
// which the hard-threshold step needs for its keep / zero decisions to be
// the reference's; otherwise one float multiply by float(SQRT2_INV) (the
// Wiener step, whose gains are continuous in the coefficients and whose
// values differ from the reference's by float rounding anyway).
template <int N, bool EXACT = true>
__device__ __forceinline__ void haar_fwd(float* v)
{
    float tmp[N > 1 ? N : 1];
#pragma unroll
    for (int k = N / 2; k >= 1; k /= 2) {
#pragma unroll
        for (int i = 0; i < k; i++) {
            const float a = v[2 * i] + v[2 * i + 1], b = v[2 * i] - v[2 * i + 1];
            tmp[i] = EXACT ? mul_sqrt2_inv(a) : a * kS2iHi;
            tmp[i + k] = EXACT ? mul_sqrt2_inv(b) : b * kS2iHi;
        }
#pragma unroll
        for (int i = 0; i < 2 * k; i++) v[i] = tmp[i];
    }
}

template <int N, bool EXACT = true>
__device__ __forceinline__ void haar_inv(float* v)
{
    float tmp[N > 1 ? N : 1];
#pragma unroll
    for (int k = 1; k * 2 <= N; k *= 2) {
#pragma unroll
        for (int i = 0; i < k; i++) {
            const float a = v[i] + v[i + k], b = v[i] - v[i + k];
            tmp[2 * i] = EXACT ? mul_sqrt2_inv(a) : a * kS2iHi;
            tmp[2 * i + 1] = EXACT ? mul_sqrt2_inv(b) : b * kS2iHi;
        }
#pragma unroll
        for (int i = 0; i < 2 * k; i++) v[i] = tmp[i];
    }
}

// hadamard_transform (src/lib_transforms.cpp:410-440), unnormalised; the
// recursion pairs (2k, 2k+1) into (k, n/2 + k) at every level.
template <int N>
__device__ __forceinline__ void hadamard(float* v)
{
    if (N == 1) return;
    float tmp[N > 1 ? N : 1];
#pragma unroll
    for (int k = 0; k < N / 2; k++) {
        tmp[k] = v[2 * k] + v[2 * k + 1];
        tmp[N / 2 + k] = v[2 * k] - v[2 * k + 1];
    }
    hadamard<(N / 2 > 0 ? N / 2 : 1)>(tmp);
    hadamard<(N / 2 > 0 ? N / 2 : 1)>(tmp + N / 2);
#pragma unroll
    for (int k = 0; k < N; k++) v[k] = tmp[k];
}
template <>
__device__ __forceinline__ void hadamard<1>(float*) {}

__device__ __forceinline__ float warp_sum(float v)
{
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(kFull, v, off);
    return v;
}

// Where the aggregation adds: separate numerator / denominator arrays (two
// scalar reds per element), or one interleaved (numerator, denominator)
// float2 array (one red.global.add.v2.f32 per element).
struct AggTarget {
    float* num;
    float* den;
    float* pair;
    // deterministic two-pass aggregation (det_agg.cu): the weighted
    // estimates kaiser * w * est of reference r in est[r][c][n][k*k] and its
    // weights in wts[r][c], summed afterwards in the reference's order
    float* est = nullptr;
    float* wts = nullptr;
};

template <bool PAIR>
__device__ __forceinline__ void agg_add(const AggTarget& A, size_t o, float v, float kw)
{
    if (PAIR) {
        // no "memory" clobber: nothing in a filter kernel reads the
        // aggregation buffers, and the clobber would make the compiler
        // reload every operand of the loop after each reduction
        asm volatile("red.global.add.v2.f32 [%0], {%1, %2};" ::"l"(A.pair + 2 * o), "f"(v), "f"(kw));
    } else {
        atomicAdd(A.num + o, v);
        atomicAdd(A.den + o, kw);
    }
}

// ------------------------------------------------- register-resident ---
// One slice per lane for compile-time K: the k x k block lives in
// registers, loops are unrolled so every table entry is a constant-bank
// operand of the FMA/MUL that uses it.

// In-place passes over a K x K block held in registers, K temporaries.
// row_pass: x[i][v] = sum_j x[i][j] M[v][j]; col_pass: x[u][j] = sum_i
// M[u][i] x[i][j]; sums run from index 0 upwards.  EXACT selects separate
// multiply and add roundings (the reference's float loops); otherwise FMA.
template <int K, bool EXACT>
__device__ __forceinline__ void row_pass(float* x, const float* M)
{
#pragma unroll
    for (int i = 0; i < K; i++) {
        float y[K];
#pragma unroll
        for (int v = 0; v < K; v++) {
            float m = 0.f;
#pragma unroll
            for (int j = 0; j < K; j++) m = EXACT ? m + x[i * K + j] * M[v * K + j] : __fmaf_rn(x[i * K + j], M[v * K + j], m);
            y[v] = m;
        }
#pragma unroll
        for (int v = 0; v < K; v++) x[i * K + v] = y[v];
    }
}

template <int K, bool EXACT>
__device__ __forceinline__ void col_pass(float* x, const float* M)
{
#pragma unroll
    for (int j = 0; j < K; j++) {
        float y[K];
#pragma unroll
        for (int u = 0; u < K; u++) {
            float m = 0.f;
#pragma unroll
            for (int i = 0; i < K; i++) m = EXACT ? m + x[i * K + j] * M[u * K + i] : __fmaf_rn(M[u * K + i], x[i * K + j], m);
            y[u] = m;
        }
#pragma unroll
        for (int u = 0; u < K; u++) x[u * K + j] = y[u];
    }
}

// The DCT passes split into even and odd halves.  The DCT-II matrix
// M[u][j] = 2 cos(pi (j + 1/2) u / K) (REDFT10) satisfies
// M[u][K-1-j] = (-1)^u M[u][j], so the even outputs are sums over the
// folded inputs x[j] + x[K-1-j] (and the middle input of an odd K) and the
// odd outputs sums over the differences x[j] - x[K-1-j]: ceil(K/2) and
// floor(K/2) terms instead of K.  The DCT-III matrix (REDFT01, [out][in])
// satisfies M[K-1-i][u] = (-1)^u M[i][u], so outputs i and K-1-i are the
// sum and the difference of the products over the even and the odd inputs.
// Both use the first ceil(K/2) columns of the tables (fwd / inv) only, and
// about half the multiply-adds of a full matrix pass; the results equal the
// full passes' up to float rounding.
template <int K>
__device__ __forceinline__ void dct2_line(float (&v)[K], const float* M)
{
    constexpr int H = K / 2, NS = (K & 1) ? H + 1 : H;
    float s[NS], d[H > 0 ? H : 1];
#pragma unroll
    for (int j = 0; j < H; j++) {
        s[j] = v[j] + v[K - 1 - j];
        d[j] = v[j] - v[K - 1 - j];
    }
    if (K & 1) s[NS - 1] = v[H];
#pragma unroll
    for (int u = 0; u < K; u++) {
        float m = 0.f;
        if ((u & 1) == 0) {
#pragma unroll
            for (int j = 0; j < NS; j++) m = __fmaf_rn(s[j], M[u * K + j], m);
        } else {
#pragma unroll
            for (int j = 0; j < H; j++) m = __fmaf_rn(d[j], M[u * K + j], m);
        }
        v[u] = m;
    }
}

template <int K>
__device__ __forceinline__ void dct3_line(float (&v)[K], const float* M)
{
    constexpr int H = K / 2, NE = (K & 1) ? H + 1 : H;
    float e[NE], o[H > 0 ? H : 1];
#pragma unroll
    for (int i = 0; i < NE; i++) {
        float m = 0.f;
#pragma unroll
        for (int u = 0; u < K; u += 2) m = __fmaf_rn(v[u], M[i * K + u], m);
        e[i] = m;
    }
#pragma unroll
    for (int i = 0; i < H; i++) {
        float m = 0.f;
#pragma unroll
        for (int u = 1; u < K; u += 2) m = __fmaf_rn(v[u], M[i * K + u], m);
        o[i] = m;
    }
#pragma unroll
    for (int i = 0; i < H; i++) {
        v[i] = e[i] + o[i];
        v[K - 1 - i] = e[i] - o[i];
    }
    if (K & 1) v[H] = e[NE - 1];
}

// x <- (line transform) along the rows (ROWS) or the columns of a K x K
// block in registers.
template <int K, bool ROWS, bool INV>
__device__ __forceinline__ void dct_pass(float* x, const float* M)
{
#pragma unroll
    for (int a = 0; a < K; a++) {
        float v[K];
#pragma unroll
        for (int b = 0; b < K; b++) v[b] = ROWS ? x[a * K + b] : x[b * K + a];
        if (INV) dct3_line<K>(v, M);
        else dct2_line<K>(v, M);
#pragma unroll
        for (int b = 0; b < K; b++) {
            if (ROWS) x[a * K + b] = v[b];
            else x[b * K + a] = v[b];
        }
    }
}

// Forward 2D transform of slice g (stride-1 K*K floats in shared memory),
// through registers, result back in g.
template <int K, class TT>
__device__ __forceinline__ void slice_fwd2d(float* g, const StepHead& P, const TT& T)
{
    float x[K * K];
#pragma unroll
    for (int e = 0; e < K * K; e++) x[e] = g[e];
    if (K == 8 && P.T2D == kBIOR) {
        // bior_2d_forward (src/lib_transforms.cpp:158-176): t = X B^T (rows),
        // out[i][j] = sum_q t[q][i] B[j][q], i.e. the column pass gives out^T
        row_pass<K, true>(x, T.fwd);
        col_pass<K, true>(x, T.fwd);
#pragma unroll
        for (int i = 0; i < K; i++)
#pragma unroll
            for (int j = 0; j < K; j++) g[i * K + j] = x[j * K + i];
    } else {
        // REDFT10 along rows then columns, then coef_norm (src/vbm3d.cpp:1294-1302)
        dct_pass<K, true, false>(x, T.fwd);
        dct_pass<K, false, false>(x, T.fwd);
#pragma unroll
        for (int e = 0; e < K * K; e++) g[e] = x[e] * T.cn[e];
    }
}

template <int K, class TT>
__device__ __forceinline__ void slice_inv2d(float* g, const StepHead& P, const TT& T)
{
    float x[K * K];
#pragma unroll
    for (int e = 0; e < K * K; e++) x[e] = g[e];
    if (K == 8 && P.T2D == kBIOR) {
        // bior_2d_inverse (src/lib_transforms.cpp:294-320): temp = in^T;
        // t2 = temp B^T, computed as a column pass on `in` (gives t2^T);
        // then the row pass gives temp[i][j]; signal[j][i] = temp[i][j]
        col_pass<K, true>(x, T.inv);
        row_pass<K, true>(x, T.inv);
#pragma unroll
        for (int i = 0; i < K; i++)
#pragma unroll
            for (int j = 0; j < K; j++) g[j * K + i] = x[i * K + j];
    } else {
        // dct_2d_inv (src/vbm3d.cpp:1696-1709)
#pragma unroll
        for (int e = 0; e < K * K; e++) x[e] = x[e] * T.cni[e];
        dct_pass<K, true, true>(x, T.inv);
        dct_pass<K, false, true>(x, T.inv);
        const float coef = 1.0f / (float)(K * 2);
#pragma unroll
        for (int e = 0; e < K * K; e++) g[e] = coef * x[e];
    }
}

// ------------------------------------------------------ shared slices ---
// The same 2D transforms with LPS lanes per slice, for groups of at most
// 32 / LPS slices (filter_ref uses LPS = 4 for one-channel groups, which
// have at most 8): lane `part` of a
// slice owns its rows part, part + LPS, ... in the row pass and the same
// columns in the column pass.  Every output is the same sum as in row_pass
// / col_pass, over the same terms in the same order with the same
// rounding, so the results are bit-identical; the passes go through the
// slice in shared memory with a warp barrier between them, and a pass whose
// stores cross the lanes' lines (bior1.5's transposed outputs) computes all
// of its lines before any store.

template <int K, bool EXACT>
__device__ __forceinline__ float row_dot(const float* xr, const float* M, int v)
{
    float m = 0.f;
#pragma unroll
    for (int j = 0; j < K; j++) m = EXACT ? m + xr[j] * M[v * K + j] : __fmaf_rn(xr[j], M[v * K + j], m);
    return m;
}
template <int K, bool EXACT>
__device__ __forceinline__ float col_dot(const float* xc, const float* M, int u)
{
    float m = 0.f;
#pragma unroll
    for (int i = 0; i < K; i++) m = EXACT ? m + xc[i] * M[u * K + i] : __fmaf_rn(M[u * K + i], xc[i], m);
    return m;
}

// Row pass of the owned rows (in place; optional elementwise scale of the
// inputs first), and column pass of the owned columns into out[t][u].
// SPLIT: 0, the full matrix M (bior1.5 with EXACT); 1, the DCT-II and 2, the
// DCT-III through their even / odd halves (dct2_line / dct3_line).
template <int K, int LPS, bool EXACT, int SPLIT = 0>
__device__ __forceinline__ void rows_owned(float* s, int part, const float* M, const float* pre)
{
#pragma unroll
    for (int t = 0; t < (K + LPS - 1) / LPS; t++) {
        const int i = part + LPS * t;
        if (i >= K) continue;
        float xr[K], y[K];
#pragma unroll
        for (int j = 0; j < K; j++) xr[j] = pre ? s[i * K + j] * pre[i * K + j] : s[i * K + j];
        if (SPLIT == 1) dct2_line<K>(xr, M);
        if (SPLIT == 2) dct3_line<K>(xr, M);
#pragma unroll
        for (int v = 0; v < K; v++) y[v] = SPLIT ? xr[v] : row_dot<K, EXACT>(xr, M, v);
#pragma unroll
        for (int v = 0; v < K; v++) s[i * K + v] = y[v];
    }
}
template <int K, int LPS, bool EXACT, int SPLIT = 0>
__device__ __forceinline__ void cols_owned(const float* s, int part, const float* M, float (&out)[(K + LPS - 1) / LPS][K])
{
#pragma unroll
    for (int t = 0; t < (K + LPS - 1) / LPS; t++) {
        const int j = part + LPS * t;
        if (j >= K) continue;
        float xc[K];
#pragma unroll
        for (int i = 0; i < K; i++) xc[i] = s[i * K + j];
        if (SPLIT == 1) dct2_line<K>(xc, M);
        if (SPLIT == 2) dct3_line<K>(xc, M);
#pragma unroll
        for (int u = 0; u < K; u++) out[t][u] = SPLIT ? xc[u] : col_dot<K, EXACT>(xc, M, u);
    }
}

// slice_fwd2d over slices g + sl * SS, sl < nsl <= 32 / LPS.
template <int K, int LPS, int SS, class TT>
__device__ __forceinline__ void slices_fwd2d_shared(float* g, int nsl, int lane, const StepHead& P, const TT& T)
{
    constexpr int NL = (K + LPS - 1) / LPS;
    const int sl = lane / LPS, part = lane % LPS;
    const bool act = sl < nsl;
    float* s = g + sl * SS;
    const bool bior = K == 8 && P.T2D == kBIOR;
    float out[NL][K];
    if (act) {
        if (bior) rows_owned<K, LPS, true>(s, part, T.fwd, nullptr);
        else rows_owned<K, LPS, false, 1>(s, part, T.fwd, nullptr);
    }
    __syncwarp();
    if (act) {
        if (bior) cols_owned<K, LPS, true>(s, part, T.fwd, out);
        else cols_owned<K, LPS, false, 1>(s, part, T.fwd, out);
    }
    __syncwarp();  // every column read before the (transposed) stores
    if (act) {
#pragma unroll
        for (int t = 0; t < NL; t++) {
            const int j = part + LPS * t;
            if (j >= K) continue;
#pragma unroll
            for (int u = 0; u < K; u++) {
                if (bior) s[j * K + u] = out[t][u];  // out[u][j] stored transposed
                else s[u * K + j] = out[t][u] * T.cn[u * K + j];
            }
        }
    }
    __syncwarp();
}

// slice_inv2d over slices g + sl * SS, sl < nsl <= 32 / LPS.
template <int K, int LPS, int SS, class TT>
__device__ __forceinline__ void slices_inv2d_shared(float* g, int nsl, int lane, const StepHead& P, const TT& T)
{
    constexpr int NL = (K + LPS - 1) / LPS;
    const int sl = lane / LPS, part = lane % LPS;
    const bool act = sl < nsl;
    float* s = g + sl * SS;
    float out[NL][K];
    if (K == 8 && P.T2D == kBIOR) {
        // column pass first (each lane stores its own columns), then the row
        // pass with transposed stores
        if (act) cols_owned<K, LPS, true>(s, part, T.inv, out);
        __syncwarp();
        if (act) {
#pragma unroll
            for (int t = 0; t < NL; t++) {
                const int j = part + LPS * t;
                if (j >= K) continue;
#pragma unroll
                for (int u = 0; u < K; u++) s[u * K + j] = out[t][u];
            }
        }
        __syncwarp();
        if (act) {
#pragma unroll
            for (int t = 0; t < NL; t++) {
                const int i = part + LPS * t;
                if (i >= K) continue;
                float xr[K];
#pragma unroll
                for (int j = 0; j < K; j++) xr[j] = s[i * K + j];
#pragma unroll
                for (int v = 0; v < K; v++) out[t][v] = row_dot<K, true>(xr, T.inv, v);
            }
        }
        __syncwarp();  // every row read before the transposed stores
        if (act) {
#pragma unroll
            for (int t = 0; t < NL; t++) {
                const int i = part + LPS * t;
                if (i >= K) continue;
#pragma unroll
                for (int v = 0; v < K; v++) s[v * K + i] = out[t][v];
            }
        }
    } else {
        if (act) rows_owned<K, LPS, false, 2>(s, part, T.inv, T.cni);
        __syncwarp();
        if (act) cols_owned<K, LPS, false, 2>(s, part, T.inv, out);
        const float coef = 1.0f / (float)(K * 2);
        if (act) {
#pragma unroll
            for (int t = 0; t < NL; t++) {
                const int j = part + LPS * t;
                if (j >= K) continue;
#pragma unroll
                for (int u = 0; u < K; u++) s[u * K + j] = coef * out[t][u];
            }
        }
    }
    __syncwarp();
}

// Gathers the nsx patches of every channel into slices [c][n][K*K] of
// stride SS, lanes over consecutive pixels (each patch row is contiguous in
// memory, so a warp load touches a few rows instead of 32 patches).  idx[n]
// is the patch's linear index in channel 0; log2n = log2(nsx).  The copies
// are asynchronous (cp.async): the caller waits for them with
// cp_async_wait_all() and a __syncwarp before reading the slices, so that
// the gathers of one group (and of a second video) are in flight together.
template <int K, int SS>
__device__ __forceinline__ void gather_k(const StepHead& P, const float* __restrict__ vid, const unsigned* idx,
                                         int nsx, int log2n, float* g, int lane)
{
    constexpr int K2 = K * K, NG = 8;  // group sizes up to 8
    // lanes over the pixels of a patch, the group's slices in unrolled inner
    // loops: a lane's pixel offset is set once, the patch positions and the
    // clip's geometry are in registers before the first copy (cp_async4s);
    // offsets within a clip fit 32 bits (W * H * F * C < 2^32)
    unsigned pos[NG];
#pragma unroll
    for (int n = 0; n < NG; n++) pos[n] = n < nsx ? idx[n] : 0u;
    const unsigned W = (unsigned)P.W, wh = (unsigned)P.wh;
    const int C = P.C;
    const unsigned g0 = smem_addr(g);
#pragma unroll
    for (int pq0 = 0; pq0 < K2; pq0 += 32) {
        const int pq = pq0 + lane;
        if (pq < K2) {
            const int p = pq / K, q = pq - p * K;
            const unsigned off = (unsigned)p * W + (unsigned)q;
#pragma unroll
            for (int c = 0; c < kMaxC; c++) {
                if (c < C) {
                    const unsigned oc = (unsigned)c * wh + off;
                    const unsigned dc = g0 + 4u * (unsigned)((c << log2n) * SS + pq);
#pragma unroll
                    for (int n = 0; n < NG; n++)
                        if (n < nsx) cp_async4s(dc + 4u * (unsigned)(n * SS), vid + (pos[n] + oc));
                }
            }
        }
    }
}

// ---------------------------------------------------------------- 1D ---

// Step 1 shrinkage of one coefficient vector (all n at one (c, pq)):
// ht_filtering_haar / _hadamard (src/vbm3d.cpp:1405-1521).  Returns the
// number of kept coefficients.
template <int N>
__device__ __forceinline__ int ht_vector(float* g, int stride, bool is_dc_pos, float T, int T3D)
{
    float v[N];
#pragma unroll
    for (int n = 0; n < N; n++) v[n] = g[n * stride];
    int kept = 0;
    if (T3D == kHADAMARD) {
        hadamard<N>(v);
#pragma unroll
        for (int n = 0; n < N; n++) {
            if ((is_dc_pos && n == 0) || fabsf(v[n]) > T) kept++;
            else v[n] = 0.0f;
        }
        hadamard<N>(v);
        const float coef = 1.0f / (float)N;
#pragma unroll
        for (int n = 0; n < N; n++) v[n] = v[n] * coef;
    } else {
        haar_fwd<N>(v);
#pragma unroll
        for (int n = 0; n < N; n++) {
            if ((is_dc_pos && n == 0) || fabsf(v[n]) > T) kept++;
            else v[n] = 0.0f;
        }
        haar_inv<N>(v);
    }
#pragma unroll
    for (int n = 0; n < N; n++) g[n * stride] = v[n];
    return kept;
}

// Step 2 shrinkage: wiener_filtering_haar / _hadamard
// (src/vbm3d.cpp:1539-1666, DCWIENER on).  Writes the estimate into gb and
// returns the sum of squared Wiener coefficients.
template <int N>
__device__ __forceinline__ float wiener_vector(const float* gn, float* gb, int stride, float s2, int T3D)
{
    float vn[N], vb[N];
#pragma unroll
    for (int n = 0; n < N; n++) {
        vn[n] = gn[n * stride];
        vb[n] = gb[n * stride];
    }
    float wsum = 0.f;
    if (T3D == kHADAMARD) {
        hadamard<N>(vn);
        hadamard<N>(vb);
        const float coef = 1.0f / (float)N;
#pragma unroll
        for (int n = 0; n < N; n++) {
            float value = vb[n] * vb[n] * coef;
            value = value / (value + s2);
            vb[n] = vn[n] * value * coef;
            wsum = wsum + value * value;
        }
        hadamard<N>(vb);
    } else {
        haar_fwd<N, false>(vn);
        haar_fwd<N, false>(vb);
#pragma unroll
        for (int n = 0; n < N; n++) {
            float value = vb[n] * vb[n];
            value = __fdividef(value, value + s2);  // a gain in [0, 1): 2-ulp quotient
            vb[n] = vn[n] * value;
            wsum = wsum + value * value;
        }
        haar_inv<N, false>(vb);
    }
#pragma unroll
    for (int n = 0; n < N; n++) gb[n * stride] = vb[n];
    return wsum;
}

// 1D transform along the group, shrinkage and the per-channel weights of
// one group held in shared memory as slices [c][n][k*k] of stride ss; one
// coefficient vector (c, pq) per lane.
template <int STEP, int NMAX = 32, int K = 0, int SSK = 0>
__device__ __forceinline__ void group_1d(const StepHead& P, float* gA, float* gB, int nsx, int ss, int lane,
                                        float* wgt)
{
    // slices are laid out [c][n][ht][k*k] with stride ss; the coefficient
    // vector (c, ht, pq) runs over n with stride kt*ss.  Its index in the
    // reference's group_3D is pq + ht*k*k, so the group DC is pq = ht = 0.
    // K > 0: the register-resident path's compile-time k (kt == 1) and
    // slice stride SSK
    const int k2 = K ? K * K : P.k * P.k, kt = K ? 1 : P.kt, k2t = k2 * kt, C = P.C;
    const int ns = K ? SSK : kt * ss;
    if (K) ss = ns;
    float acc[kMaxC] = {0.f, 0.f, 0.f};
    for (int v = lane; v < C * k2t; v += 32) {
        const int c = v / k2t, rem = v - c * k2t, ht = K ? 0 : rem / k2, pq = rem - ht * k2;
        float* ga = gA + ((size_t)(c * nsx) * kt + ht) * ss + pq;
        float* gb = gB + ((size_t)(c * nsx) * kt + ht) * ss + pq;
        const bool dc = pq == 0 && ht == 0;
        if (STEP == 1) {
            const float T = P.lambda3D * P.sigma[c] * (P.T3D == kHADAMARD ? sqrtf((float)nsx) : 1.0f);
            int kept;
            switch (nsx) {
                case 1: kept = ht_vector<1>(ga, ns, dc, T, P.T3D); break;
                case 2: kept = ht_vector<2>(ga, ns, dc, T, P.T3D); break;
                case 4: kept = ht_vector<4>(ga, ns, dc, T, P.T3D); break;
                case 8: kept = ht_vector<(NMAX < 8 ? NMAX : 8)>(ga, ns, dc, T, P.T3D); break;
                case 16: kept = ht_vector<(NMAX < 16 ? NMAX : 16)>(ga, ns, dc, T, P.T3D); break;
                default: kept = ht_vector<NMAX>(ga, ns, dc, T, P.T3D); break;
            }
#pragma unroll
            for (int cc = 0; cc < kMaxC; cc++)
                if (cc == c) acc[cc] += (float)kept;
        } else {
            const float s2 = P.sigma[c] * P.sigma[c];
            float ws;
            switch (nsx) {
                case 1: ws = wiener_vector<1>(ga, gb, ns, s2, P.T3D); break;
                case 2: ws = wiener_vector<2>(ga, gb, ns, s2, P.T3D); break;
                case 4: ws = wiener_vector<4>(ga, gb, ns, s2, P.T3D); break;
                case 8: ws = wiener_vector<(NMAX < 8 ? NMAX : 8)>(ga, gb, ns, s2, P.T3D); break;
                case 16: ws = wiener_vector<(NMAX < 16 ? NMAX : 16)>(ga, gb, ns, s2, P.T3D); break;
                default: ws = wiener_vector<NMAX>(ga, gb, ns, s2, P.T3D); break;
            }
#pragma unroll
            for (int cc = 0; cc < kMaxC; cc++)
                if (cc == c) acc[cc] += ws;
        }
    }
#pragma unroll
    for (int c = 0; c < kMaxC; c++) {
        const float tot = warp_sum(acc[c]);  // counts are exact; Wiener sums reassociate
        const float s2 = P.sigma[c] * P.sigma[c];
        if (STEP == 2 && P.T3D == kHADAMARD) wgt[c] = tot > 0.0f ? 1.0f / (float)(s2 * tot) : 1.0f;
        else wgt[c] = 1.f / (float)(s2 * tot);
    }
    __syncwarp();

}

template <int K, int SS, class TT>
__device__ __forceinline__ void slice_fwd(const StepHead& P, const TT& T, float* g, int nsl, int lane)
{
    for (int sl = lane; sl < nsl; sl += 32) slice_fwd2d<K>(g + sl * SS, P, T);
}

// Filtering and aggregation of the group of reference patch r by one warp,
// register-resident transforms for compile-time K (kt == 1, N <= 8), with
// the warp's shared-memory region `base`.  T holds the kaiser / fwd / inv /
// cn / cni tables (StepParams, or the batched form's compact copy).
template <int STEP, int K, bool PAIR, int LPS, bool STORE = false, class TT>
__device__ __forceinline__ void filter_ref(const StepHead& P, const TT& T, long long r, float* base, int lane,
                                           const float* __restrict__ noisy, const float* __restrict__ basic,
                                           const unsigned* __restrict__ tab_idx, const unsigned* __restrict__ tab_nsx,
                                           const AggTarget& A)
{
    constexpr int K2 = K * K, SS = slice_stride(K, LPS);
    const int C = P.C;
    unsigned* idx = reinterpret_cast<unsigned*>(base);
    float* gA = base + kMaxN;               // noisy group
    float* gB = gA + (size_t)C * P.N * SS;  // basic group (step 2)

    const int nsx = (int)tab_nsx[r];
    const int log2n = __ffs(nsx) - 1;
    if (lane < nsx) idx[lane] = tab_idx[(size_t)r * P.N + lane];
    __syncwarp();
    const int nsl = C * nsx;

    gather_k<K, SS>(P, noisy, idx, nsx, log2n, gA, lane);
    if (STEP == 2) gather_k<K, SS>(P, basic, idx, nsx, log2n, gB, lane);
    cp_async_wait_all();
    __syncwarp();
    // 2D transforms: one slice (c, n) per lane in registers (LPS == 1), or
    // 4 lanes per slice through shared memory (LPS == 4: groups of at most 8
    // slices, such as every one-channel group; the kernels are instantiated
    // per mode, so each carries one form's registers); the barrier keeps the
    // compiler from interleaving the two groups' register transforms (two
    // blocks of k*k registers live at once)
    static_assert(LPS == 1 || LPS == 4, "slice modes");
    if (LPS == 4) {
        slices_fwd2d_shared<K, 4, SS>(gA, nsl, lane, P, T);
        if (STEP == 2) slices_fwd2d_shared<K, 4, SS>(gB, nsl, lane, P, T);
    } else {
        slice_fwd<K, SS>(P, T, gA, nsl, lane);
        if (STEP == 2) {
            __syncwarp();
            slice_fwd<K, SS>(P, T, gB, nsl, lane);
        }
        __syncwarp();
    }

    float wgt[kMaxC];
    group_1d<STEP, 8, K, SS>(P, gA, gB, nsx, SS, lane, wgt);  // the host sends N > 8 to the generic kernel

    // inverse 2D, as the forward one
    float* ge = STEP == 1 ? gA : gB;
    if (LPS == 4) {
        slices_inv2d_shared<K, 4, SS>(ge, nsl, lane, P, T);
    } else {
        for (int sl = lane; sl < nsl; sl += 32) slice_inv2d<K>(ge + sl * SS, P, T);
        __syncwarp();
    }

    // aggregation (src/vbm3d.cpp:612-650)
    constexpr int NG = 8;  // group sizes of this body (N <= 8, as group_1d)
    if (STORE) {
        // the products the reference adds, kept for the ordered second pass:
        // est[r][c][n][pq] = (kaiser[pq] * w_c) * est, the reference's
        // evaluation order of kai * w * e (src/vbm3d.cpp:641-643); lanes
        // over the pixels of a patch, as below
        float* er = A.est + (size_t)r * (size_t)(C * P.N * K2);
#pragma unroll
        for (int pq0 = 0; pq0 < K2; pq0 += 32) {
            const int pq = pq0 + lane;
            if (pq < K2) {
                const float kai = T.kaiser[pq];
#pragma unroll
                for (int c = 0; c < kMaxC; c++) {
                    if (c < C) {
                        const float kw = kai * wgt[c];
                        const float* gc = ge + (c << log2n) * SS + pq;
                        float* ec = er + c * P.N * K2 + pq;
#pragma unroll
                        for (int n = 0; n < NG; n++)
                            if (n < nsx) ec[n * K2] = kw * gc[n * SS];
                    }
                }
            }
        }
        if (lane == 0) {
#pragma unroll
            for (int c = 0; c < kMaxC; c++)
                if (c < C) A.wts[(size_t)r * C + c] = wgt[c];
        }
        return;
    }
    // lanes over the pixels of a patch, the group's slices in the inner
    // loops: a lane's pixel offset and Kaiser weight are set once, the
    // slice's channel weight and patch index are the same on every lane.
    // Offsets within a clip fit 32 bits (W * H * F * C < 2^32).
    unsigned pos[NG];
#pragma unroll
    for (int n = 0; n < NG; n++) pos[n] = n < nsx ? idx[n] : 0u;
    const unsigned W = (unsigned)P.W, wh = (unsigned)P.wh;
#pragma unroll
    for (int pq0 = 0; pq0 < K2; pq0 += 32) {
        const int pq = pq0 + lane;
        if (pq < K2) {
            const int p = pq / K, q = pq - p * K;
            const unsigned off = (unsigned)p * W + (unsigned)q;
            const float kai = T.kaiser[pq];
#pragma unroll
            for (int c = 0; c < kMaxC; c++) {
                if (c < C) {
                    const float kw = kai * wgt[c];
                    const float* gc = ge + (c << log2n) * SS + pq;
                    const unsigned oc = (unsigned)c * wh + off;
#pragma unroll
                    for (int n = 0; n < NG; n++)
                        if (n < nsx) agg_add<PAIR>(A, (size_t)(pos[n] + oc), kw * gc[n * SS], kw);
                }
            }
        }
    }
}

}  // namespace vbm3d
