// K-T + K-A: collaborative filtering of one group and its aggregation.
//
// Replaces, for one reference patch, dct_2d_process / bior_2d_process
// (src/vbm3d.cpp:1218-1386), the regrouping (:565-570), ht_filtering_* and
// wiener_filtering_* (:1405-1666), dct_2d_inv / bior_2d_inv (:1678-1731) and
// the aggregation loops (:612-650, :860-924).  One warp handles one group:
//
//  * the nsx patches of every channel are gathered into shared memory as
//    slices [c][n][k*k] (slice stride k*k + 1 to spread banks);
//  * the 2D transform runs one slice per lane: bior1.5 as the reference's
//    two basis-matrix passes in its float order (bit-identical), the DCT as
//    two float matrix passes followed by the reference's normalisation;
//  * the 1D Haar (or Walsh-Hadamard) transform along the group runs one
//    coefficient vector per lane, in registers, with the reference's
//    rounding, then hard thresholding (group DC always kept) or Wiener
//    shrinkage, then the inverse;
//  * per-channel weights follow the reference's formulas; the inverse 2D
//    transform runs one slice per lane and every pixel is added into the
//    numerator / denominator with a Kaiser window weight by red.global.add.
#include "filter_common.cuh"

namespace vbm3d {

// ---------------------------------------------------------------- 2D ---

// bior_2d_forward passes (src/lib_transforms.cpp:158-176): t[i][j] =
// sum_k x[i][k] B[j][k]; x[i][j] = sum_k t[k][i] B[j][k]; sums from k = 0.
__device__ __forceinline__ void bior_fwd8(float* x, float* t, const float* B)
{
    for (int i = 0; i < 8; i++)
        for (int j = 0; j < 8; j++) {
            float m = 0.f;
#pragma unroll
            for (int q = 0; q < 8; q++) m = m + x[i * 8 + q] * B[j * 8 + q];
            t[i * 8 + j] = m;
        }
    for (int i = 0; i < 8; i++)
        for (int j = 0; j < 8; j++) {
            float m = 0.f;
#pragma unroll
            for (int q = 0; q < 8; q++) m = m + t[q * 8 + i] * B[j * 8 + q];
            x[i * 8 + j] = m;
        }
}

// bior_2d_inverse (src/lib_transforms.cpp:294-320): transposed read, the
// same two passes with the inverse basis, transposed write.
__device__ __forceinline__ void bior_inv8(float* x, float* t, const float* B)
{
    for (int i = 0; i < 8; i++)
        for (int j = 0; j < 8; j++) {
            float m = 0.f;
#pragma unroll
            for (int q = 0; q < 8; q++) m = m + x[i + q * 8] * B[j * 8 + q];
            t[i * 8 + j] = m;
        }
    for (int i = 0; i < 8; i++)
        for (int j = 0; j < 8; j++) {
            float m = 0.f;
#pragma unroll
            for (int q = 0; q < 8; q++) m = m + t[q * 8 + i] * B[j * 8 + q];
            x[j * 8 + i] = m;
        }
}

// Orthonormal 2D DCT-II of a k x k block: FFTW REDFT10 along rows and
// columns, Y = D X D^T with D[u][j] = 2cos(pi (j + 1/2) u / k), then the
// reference's normalisation Y[u][v] * coef_norm[u*k + v] (src/vbm3d.cpp:1294-1302).
__device__ __forceinline__ void dct_fwd(float* x, float* t, const StepParams& P)
{
    const int k = P.k;
    for (int i = 0; i < k; i++)
        for (int v = 0; v < k; v++) {
            float m = 0.f;
            for (int j = 0; j < k; j++) m = __fmaf_rn(x[i * k + j], P.fwd[v * k + j], m);
            t[i * k + v] = m;
        }
    for (int u = 0; u < k; u++)
        for (int v = 0; v < k; v++) {
            float m = 0.f;
            for (int i = 0; i < k; i++) m = __fmaf_rn(P.fwd[u * k + i], t[i * k + v], m);
            x[u * k + v] = m * P.cn[u * k + v];
        }
}

// dct_2d_inv (src/vbm3d.cpp:1696-1709): Z = Y * coef_norm_inv, REDFT01 along
// both axes (X = E Z E^T, E[i][u] = u ? 2cos(pi u (i + 1/2) / k) : 1), times 1/(2k).
__device__ __forceinline__ void dct_inv(float* x, float* t, const StepParams& P)
{
    const int k = P.k;
    const float coef = 1.0f / (float)(k * 2);
    for (int u = 0; u < k; u++)
        for (int j = 0; j < k; j++) {
            float m = 0.f;
            for (int v = 0; v < k; v++) m = __fmaf_rn(x[u * k + v] * P.cni[u * k + v], P.inv[j * k + v], m);
            t[u * k + j] = m;
        }
    for (int i = 0; i < k; i++)
        for (int j = 0; j < k; j++) {
            float m = 0.f;
            for (int u = 0; u < k; u++) m = __fmaf_rn(P.inv[i * k + u], t[u * k + j], m);
            x[i * k + j] = coef * m;
        }
}

__device__ __forceinline__ void fwd2d(float* x, float* t, const StepParams& P)
{
    if (P.T2D == kBIOR) bior_fwd8(x, t, P.fwd);
    else dct_fwd(x, t, P);
}

__device__ __forceinline__ void inv2d(float* x, float* t, const StepParams& P)
{
    if (P.T2D == kBIOR) bior_inv8(x, t, P.inv);
    else dct_inv(x, t, P);
}

// ---------------------------------------------------------------- 1D ---

// Gather the nsx patches of all channels of `vid` into slices [c][n][k*k].
__device__ __forceinline__ void gather(const StepParams& P, const float* __restrict__ vid,
                                       const unsigned* idx, int nsx, int ss, float* g, int lane)
{
    const int k = P.k, k2 = k * k;
    const int total = P.C * nsx * k2;
    for (int e = lane; e < total; e += 32) {
        const int sl = e / k2, pq = e - sl * k2;
        const int c = sl / nsx, n = sl - c * nsx;
        const int p = pq / k, q = pq - p * k;
        int x, y, t;
        patch_coords(P, idx[n], x, y, t);
        g[sl * ss + pq] = __ldg(vid + (size_t)t * P.whc + (size_t)c * P.wh + (size_t)(y + p) * P.W + x + q);
    }
}

// temporal_transform / temporal_inv_transform (src/vbm3d.cpp:1866-1956):
// an orthonormal DCT-II along the kt slices of every (c, n, pq), for
// kt > 1 with the DCT 2D transform.  Forward: REDFT10 * norm, and the
// first coefficient times SQRT2_INV through double as in the reference;
// inverse: the first coefficient times SQRT2 through double, REDFT01, * norm.
__device__ void temporal_group(const StepParams& P, float* g, int nsx, int ss, int lane, bool inverse)
{
    const int kt = P.kt, k2 = P.k * P.k, total = P.C * nsx * k2;
    const float norm = (float)(1. / sqrt(2.0 * kt));
    const float pi = 3.14159265358979f;
    for (int v = lane; v < total; v += 32) {
        const int cn = v / k2, pq = v - cn * k2;  // cn = c * nsx + n
        float* base = g + (size_t)cn * kt * ss + pq;
        float in[kMaxKt], out[kMaxKt];
        for (int t = 0; t < kt; t++) in[t] = base[t * ss];
        if (!inverse) {
            for (int u = 0; u < kt; u++) {
                float m = 0.f;
                for (int t = 0; t < kt; t++) m = __fmaf_rn(in[t], 2.0f * cosf(pi * (t + 0.5f) * u / kt), m);
                const float y = m * norm;
                out[u] = u == 0 ? mul_sqrt2_inv(y) : y;
            }
        } else {
            in[0] = mul_sqrt2(in[0]);
            for (int t = 0; t < kt; t++) {
                float m = in[0];
                for (int u = 1; u < kt; u++) m = __fmaf_rn(in[u], 2.0f * cosf(pi * u * (t + 0.5f) / kt), m);
                out[t] = m * norm;
            }
        }
        for (int t = 0; t < kt; t++) base[t * ss] = out[t];
    }
}

// Any k <= 16 and kt <= 4: slices [c][n][ht] transformed in shared memory
// with runtime-sized loops; slice ht of patch n follows the patch's
// trajectory (patch_trajectory, src/vbm3d.cpp:378-425).
template <int STEP, bool PAIR>
__global__ void __launch_bounds__(128)
filter_kernel_generic(const StepParams P, const float* __restrict__ noisy, const float* __restrict__ basic,
                      const float* __restrict__ fflow, const unsigned* __restrict__ tab_idx,
                      const unsigned* __restrict__ tab_nsx, const AggTarget A, int warp_floats)
{
    extern __shared__ __align__(16) float fsm[];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const long long r = band_order_ref(P, P.ref_base + (long long)blockIdx.x * (blockDim.x >> 5) + wid);
    if (r >= P.nrefs) return;

    const int k = P.k, k2 = k * k, C = P.C, kt = P.kt;
    const int ss = k2 | 1;  // slice stride, odd: a lane per slice reads on distinct banks
    float* base = fsm + (size_t)wid * warp_floats;
    int* traj = reinterpret_cast<int*>(base);                // [n][ht]: top-left offset in channel 0
    float* gA = base + kMaxN * kMaxKt;                      // noisy group (step 1: the group)
    float* gT = gA + (size_t)C * P.N * kt * ss;             // per-slice scratch
    float* gB = gT + (size_t)C * P.N * kt * ss;             // basic group (step 2)

    const int nsx = (int)tab_nsx[r];
    if (lane < nsx) {
        int x, y, t, tx[kMaxKt], ty[kMaxKt];
        patch_coords(P, tab_idx[(size_t)r * P.N + lane], x, y, t);
        trajectory(P, fflow, x, y, t, tx, ty);
        for (int ht = 0; ht < kt; ht++) traj[lane * kMaxKt + ht] = (int)patch_index(P, tx[ht], ty[ht], t + ht);
    }
    __syncwarp();

    const int nsl = C * nsx * kt;  // slice sl = (c * nsx + n) * kt + ht
    for (int e = lane; e < nsl * k2; e += 32) {
        const int sl = e / k2, pq = e - sl * k2;
        const int cn = sl / kt, ht = sl - cn * kt, c = cn / nsx, n = cn - c * nsx;
        const int p = pq / k, q = pq - p * k;
        const size_t o = (size_t)traj[n * kMaxKt + ht] + (size_t)c * P.wh + (size_t)p * P.W + q;
        gA[sl * ss + pq] = __ldg(noisy + o);
        if (STEP == 2) gB[sl * ss + pq] = __ldg(basic + o);
    }
    __syncwarp();
    for (int sl = lane; sl < nsl; sl += 32) {
        fwd2d(gA + sl * ss, gT + sl * ss, P);
        if (STEP == 2) fwd2d(gB + sl * ss, gT + sl * ss, P);
    }
    __syncwarp();
    const bool temporal = kt > 1 && P.T2D != kBIOR;
    if (temporal) {
        temporal_group(P, gA, nsx, ss, lane, false);
        if (STEP == 2) temporal_group(P, gB, nsx, ss, lane, false);
        __syncwarp();
    }

    float wgt[kMaxC];
    group_1d<STEP>(P, gA, gB, nsx, ss, lane, wgt);

    float* ge = STEP == 1 ? gA : gB;
    if (temporal) {
        temporal_group(P, ge, nsx, ss, lane, true);
        __syncwarp();
    }
    for (int sl = lane; sl < nsl; sl += 32) inv2d(ge + sl * ss, gT + sl * ss, P);
    __syncwarp();

    // aggregation (src/vbm3d.cpp:612-650): num += kaiser * w * est; den += kaiser * w
    for (int e = lane; e < nsl * k2; e += 32) {
        const int sl = e / k2, pq = e - sl * k2;
        const int cn = sl / kt, ht = sl - cn * kt, c = cn / nsx, n = cn - c * nsx;
        const int p = pq / k, q = pq - p * k;
        const size_t o = (size_t)traj[n * kMaxKt + ht] + (size_t)c * P.wh + (size_t)p * P.W + q;
        const float kw = P.kaiser[pq] * wgt[c];
        agg_add<PAIR>(A, o, kw * ge[sl * ss + pq], kw);
    }
}

template <int STEP, int K, bool PAIR, int LPS, bool STORE = false>
__global__ void __launch_bounds__(128, 4)
filter_kernel_k(const StepParams P, const float* __restrict__ noisy, const float* __restrict__ basic,
                const unsigned* __restrict__ tab_idx, const unsigned* __restrict__ tab_nsx, const AggTarget A,
                int warp_floats)
{
    extern __shared__ __align__(16) float fsm[];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const long long r = band_order_ref(P, P.ref_base + (long long)blockIdx.x * (blockDim.x >> 5) + wid);
    if (r >= P.nrefs) return;
    filter_ref<STEP, K, PAIR, LPS, STORE>(P, P, r, fsm + (size_t)wid * warp_floats, lane, noisy, basic, tab_idx,
                                          tab_nsx, A);
}

namespace {

template <int STEP, int K, bool PAIR, int LPS, bool STORE = false>
cudaError_t launch_k_mode(const StepParams& P, const float* noisy, const float* basic, const unsigned* tab_idx,
                          const unsigned* tab_nsx, const AggTarget& A, long long count, cudaStream_t stream)
{
    const int warps = 4;
    constexpr int kSlice = slice_stride(K, LPS) > K * K + 1 ? slice_stride(K, LPS) : K * K + 1;
    const int wf = kMaxN + (STEP == 1 ? 1 : 2) * P.C * P.N * kSlice;
    const size_t smem = (size_t)warps * wf * sizeof(float);
    cudaError_t e = cudaFuncSetAttribute(filter_kernel_k<STEP, K, PAIR, LPS, STORE>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const long long blocks = (count + warps - 1) / warps;
    filter_kernel_k<STEP, K, PAIR, LPS, STORE><<<(unsigned)blocks, warps * 32, smem, stream>>>(P, noisy, basic,
                                                                                              tab_idx, tab_nsx, A, wf);
    return cudaGetLastError();
}

// One-channel groups (at most N <= 8 slices) take the shared-slice
// transforms, four lanes per slice; others one slice per lane.
template <int STEP, int K, bool PAIR>
cudaError_t launch_k(const StepParams& P, const float* noisy, const float* basic, const unsigned* tab_idx,
                     const unsigned* tab_nsx, const AggTarget& A, long long count, cudaStream_t stream)
{
    if (P.C == 1) return launch_k_mode<STEP, K, PAIR, 4>(P, noisy, basic, tab_idx, tab_nsx, A, count, stream);
    return launch_k_mode<STEP, K, PAIR, 1>(P, noisy, basic, tab_idx, tab_nsx, A, count, stream);
}

template <int STEP, bool PAIR>
cudaError_t launch_generic(const StepParams& P, const float* noisy, const float* basic, const float* fflow,
                           const unsigned* tab_idx, const unsigned* tab_nsx, const AggTarget& A, long long count,
                           cudaStream_t stream)
{
    // group(s) + scratch, kt slices per patch, plus the trajectories
    const int wf = kMaxN * kMaxKt + (STEP == 1 ? 2 : 3) * P.C * P.N * P.kt * (P.k * P.k + 1);
    int warps = 4;
    while (warps > 1 && (size_t)warps * wf * sizeof(float) > 200 * 1024) warps /= 2;
    const size_t smem = (size_t)warps * wf * sizeof(float);
    cudaError_t e = cudaFuncSetAttribute(filter_kernel_generic<STEP, PAIR>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const long long blocks = (count + warps - 1) / warps;
    filter_kernel_generic<STEP, PAIR><<<(unsigned)blocks, warps * 32, smem, stream>>>(P, noisy, basic, fflow,
                                                                                     tab_idx, tab_nsx, A, wf);
    return cudaGetLastError();
}

template <int STEP, bool PAIR>
cudaError_t dispatch(const StepParams& P, const float* noisy, const float* basic, const float* fflow,
                     const unsigned* tab_idx, const unsigned* tab_nsx, const AggTarget& A, long long count,
                     cudaStream_t stream)
{
    if (P.N <= 8 && P.kt == 1) {  // group sizes up to 8, 2D patches: the register-resident kernel
        switch (P.k) {
            case 7: return launch_k<STEP, 7, PAIR>(P, noisy, basic, tab_idx, tab_nsx, A, count, stream);
            case 8: return launch_k<STEP, 8, PAIR>(P, noisy, basic, tab_idx, tab_nsx, A, count, stream);
            default: break;
        }
    }
    return launch_generic<STEP, PAIR>(P, noisy, basic, fflow, tab_idx, tab_nsx, A, count, stream);
}

template <int STEP, int K>
cudaError_t launch_k_store(const StepParams& P, const float* noisy, const float* basic, const unsigned* tab_idx,
                           const unsigned* tab_nsx, const AggTarget& A, long long count, cudaStream_t stream)
{
    if (P.C == 1) return launch_k_mode<STEP, K, true, 4, true>(P, noisy, basic, tab_idx, tab_nsx, A, count, stream);
    return launch_k_mode<STEP, K, true, 1, true>(P, noisy, basic, tab_idx, tab_nsx, A, count, stream);
}

}  // namespace

// The filter of the deterministic two-pass aggregation: instead of adding
// into num / den, every group keeps its weighted estimates in est
// ([nrefs][C][N][k*k]) and its weights in wts ([nrefs][C]); det_agg.cu sums
// them in the reference's order.  k in {7, 8}, kt == 1, N <= 8.
cudaError_t launch_filter_store(int step, const StepParams& P, const float* noisy, const float* basic,
                                const unsigned* tab_idx, const unsigned* tab_nsx, float* est, float* wts,
                                long long count, cudaStream_t stream)
{
    AggTarget A{nullptr, nullptr, nullptr};
    A.est = est;
    A.wts = wts;
    if (P.N > 8 || P.kt != 1 || (P.k != 7 && P.k != 8)) return cudaErrorInvalidValue;
    if (step == 1)
        return P.k == 7 ? launch_k_store<1, 7>(P, noisy, basic, tab_idx, tab_nsx, A, count, stream)
                        : launch_k_store<1, 8>(P, noisy, basic, tab_idx, tab_nsx, A, count, stream);
    return P.k == 7 ? launch_k_store<2, 7>(P, noisy, basic, tab_idx, tab_nsx, A, count, stream)
                    : launch_k_store<2, 8>(P, noisy, basic, tab_idx, tab_nsx, A, count, stream);
}

// Aggregates into num / den when `pair` is NULL, else into the interleaved
// (num, den) array `pair` (2 floats per video value).
cudaError_t launch_filter(int step, const StepParams& P, const float* noisy, const float* basic,
                          const float* fflow, const unsigned* tab_idx, const unsigned* tab_nsx, float* num,
                          float* den, float* pair, long long count, cudaStream_t stream)
{
    const AggTarget A{num, den, pair};
    if (step == 1)
        return pair ? dispatch<1, true>(P, noisy, basic, fflow, tab_idx, tab_nsx, A, count, stream)
                    : dispatch<1, false>(P, noisy, basic, fflow, tab_idx, tab_nsx, A, count, stream);
    return pair ? dispatch<2, true>(P, noisy, basic, fflow, tab_idx, tab_nsx, A, count, stream)
                : dispatch<2, false>(P, noisy, basic, fflow, tab_idx, tab_nsx, A, count, stream);
}

}  // namespace vbm3d
