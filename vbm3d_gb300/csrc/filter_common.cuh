// Device helpers shared by the filtering kernels (filter.cu) and the
// linearised / adjoint kernels (linear.cu).
#pragma once

#include "common.cuh"

namespace vbm3d {

// ---------------------------------------------------------------- 1D ---

// haar_forward / haar_inverse (src/lib_transforms.cpp:453-512).
template <int N>
__device__ __forceinline__ void haar_fwd(float* v)
{
    float tmp[N > 1 ? N : 1];
#pragma unroll
    for (int k = N / 2; k >= 1; k /= 2) {
#pragma unroll
        for (int i = 0; i < k; i++) {
            tmp[i] = mul_sqrt2_inv(v[2 * i] + v[2 * i + 1]);
            tmp[i + k] = mul_sqrt2_inv(v[2 * i] - v[2 * i + 1]);
        }
#pragma unroll
        for (int i = 0; i < 2 * k; i++) v[i] = tmp[i];
    }
}

template <int N>
__device__ __forceinline__ void haar_inv(float* v)
{
    float tmp[N > 1 ? N : 1];
#pragma unroll
    for (int k = 1; k * 2 <= N; k *= 2) {
#pragma unroll
        for (int i = 0; i < k; i++) {
            tmp[2 * i] = mul_sqrt2_inv(v[i] + v[i + k]);
            tmp[2 * i + 1] = mul_sqrt2_inv(v[i] - v[i + k]);
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
};

template <bool PAIR>
__device__ __forceinline__ void agg_add(const AggTarget& A, size_t o, float v, float kw)
{
    if (PAIR) {
        asm volatile("red.global.add.v2.f32 [%0], {%1, %2};" ::"l"(A.pair + 2 * o), "f"(v), "f"(kw) : "memory");
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

// Forward 2D transform of slice g (stride-1 K*K floats in shared memory),
// through registers, result back in g.
template <int K>
__device__ __forceinline__ void slice_fwd2d(float* g, const StepParams& P)
{
    float x[K * K];
#pragma unroll
    for (int e = 0; e < K * K; e++) x[e] = g[e];
    if (K == 8 && P.T2D == kBIOR) {
        // bior_2d_forward (src/lib_transforms.cpp:158-176): t = X B^T (rows),
        // out[i][j] = sum_q t[q][i] B[j][q], i.e. the column pass gives out^T
        row_pass<K, true>(x, P.fwd);
        col_pass<K, true>(x, P.fwd);
#pragma unroll
        for (int i = 0; i < K; i++)
#pragma unroll
            for (int j = 0; j < K; j++) g[i * K + j] = x[j * K + i];
    } else {
        // REDFT10 along rows then columns, then coef_norm (src/vbm3d.cpp:1294-1302)
        row_pass<K, false>(x, P.fwd);
        col_pass<K, false>(x, P.fwd);
#pragma unroll
        for (int e = 0; e < K * K; e++) g[e] = x[e] * P.cn[e];
    }
}

template <int K>
__device__ __forceinline__ void slice_inv2d(float* g, const StepParams& P)
{
    float x[K * K];
#pragma unroll
    for (int e = 0; e < K * K; e++) x[e] = g[e];
    if (K == 8 && P.T2D == kBIOR) {
        // bior_2d_inverse (src/lib_transforms.cpp:294-320): temp = in^T;
        // t2 = temp B^T, computed as a column pass on `in` (gives t2^T);
        // then the row pass gives temp[i][j]; signal[j][i] = temp[i][j]
        col_pass<K, true>(x, P.inv);
        row_pass<K, true>(x, P.inv);
#pragma unroll
        for (int i = 0; i < K; i++)
#pragma unroll
            for (int j = 0; j < K; j++) g[j * K + i] = x[i * K + j];
    } else {
        // dct_2d_inv (src/vbm3d.cpp:1696-1709)
#pragma unroll
        for (int e = 0; e < K * K; e++) x[e] = x[e] * P.cni[e];
        row_pass<K, false>(x, P.inv);
        col_pass<K, false>(x, P.inv);
        const float coef = 1.0f / (float)(K * 2);
#pragma unroll
        for (int e = 0; e < K * K; e++) g[e] = coef * x[e];
    }
}

// Gathers the nsx patches of every channel into slices [c][n][K*K] of
// stride SS, lanes over consecutive pixels (each patch row is contiguous in
// memory, so a warp load touches a few rows instead of 32 patches).  idx[n]
// is the patch's linear index in channel 0; log2n = log2(nsx).
template <int K, int SS>
__device__ __forceinline__ void gather_k(const StepParams& P, const float* __restrict__ vid, const unsigned* idx,
                                         int nsx, int log2n, float* g, int lane)
{
    constexpr int K2 = K * K;
    const int total = P.C * nsx * K2;
    for (int e = lane; e < total; e += 32) {
        const int sl = e / K2, pq = e - sl * K2;
        const int c = sl >> log2n, n = sl & (nsx - 1);
        const int p = pq / K, q = pq - p * K;
        g[sl * SS + pq] = __ldg(vid + idx[n] + (size_t)c * P.wh + (size_t)p * P.W + q);
    }
}

}  // namespace vbm3d
