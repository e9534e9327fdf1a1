// Frozen linearisation of one collaborative-filtering step, and its adjoint.
//
// No counterpart in the reference.  With the block-matching groups, the
// hard-threshold masks (step 1) or the Wiener coefficients (step 2) and the
// aggregation weights frozen at the values the forward pass computes, each
// step is a linear map of its noisy input:
//   L x = [ sum_g S_g^T K w_g A_g (S_g x) ] / den,   A_g = G o Hinv o Lambda_g o Hf o F
// where S_g gathers the group's patches, F / G are the 2D forward / inverse
// transforms, Hf / Hinv the 1D transform along the group, Lambda_g the mask
// or Wiener gains, K the Kaiser window, w_g the group weights and den the
// forward pass's denominator.  Pixels with den == 0 fall back to the noisy
// value in step 1 (identity) and to the frozen basic estimate in step 2
// (constant), as run_vbm3d's division does (src/vbm3d.cpp:168-170, :198-202).
//
// The adjoint is L^T g = sum_g S_g^T F^T Hf^T Lambda_g Hinv^T G^T K w_g S_g (g / den)
// (+ g itself where den == 0 in step 1).  Haar is orthonormal and the
// reference's Walsh-Hadamard matrix is symmetric, so Hf^T / Hinv^T are the
// same 1D transforms in the forward order; F^T and G^T are the 2D transforms
// with transposed bases (bior1.5: F(X) = B X^T B^T, so F^T = F with B^T;
// DCT: F(X) = cn o (D X D^T), so F^T(Z) = D^T (cn o Z) D).
//
// Transforms are recomputed from the frozen inputs, never stored: the masks
// and gains come from the same float arithmetic as the forward kernels.
#include <cstring>

#include "filter_common.cuh"
#include "../../include/vbm3d_gb300.h"

namespace vbm3d {

cudaError_t launch_bm(const StepParams& P, const float* vid, const float* fflow, const float* bflow,
                      unsigned* out_idx, float* out_dist, unsigned* out_nsimp, unsigned* out_nsx,
                      long long count, cudaStream_t stream, unsigned long long* out_count);
int build_step_params(const vbm3d_params* p, vbm3d_dims d, float sigma, int color_space, StepParams& P);
void set_last_error(int status, const char* msg);

namespace {

// F^T: transpose of slice_fwd2d.
template <int K>
__device__ __forceinline__ void slice_fwd2d_T(float* g, const StepParams& P)
{
    float x[K * K];
#pragma unroll
    for (int e = 0; e < K * K; e++) x[e] = g[e];
    if (K == 8 && P.T2D == kBIOR) {
        row_pass<K, false>(x, P.fwdT);
        col_pass<K, false>(x, P.fwdT);
#pragma unroll
        for (int i = 0; i < K; i++)
#pragma unroll
            for (int j = 0; j < K; j++) g[i * K + j] = x[j * K + i];
    } else {
#pragma unroll
        for (int e = 0; e < K * K; e++) x[e] = x[e] * P.cn[e];
        // the transposed DCT-II matrix has the DCT-III's output symmetry:
        // its even / odd form (dct3_line) over the table fwdT
        dct_pass<K, true, true>(x, P.fwdT);
        dct_pass<K, false, true>(x, P.fwdT);
#pragma unroll
        for (int e = 0; e < K * K; e++) g[e] = x[e];
    }
}

// G^T: transpose of slice_inv2d.
template <int K>
__device__ __forceinline__ void slice_inv2d_T(float* g, const StepParams& P)
{
    float x[K * K];
#pragma unroll
    for (int e = 0; e < K * K; e++) x[e] = g[e];
    if (K == 8 && P.T2D == kBIOR) {
        col_pass<K, false>(x, P.invT);
        row_pass<K, false>(x, P.invT);
#pragma unroll
        for (int i = 0; i < K; i++)
#pragma unroll
            for (int j = 0; j < K; j++) g[j * K + i] = x[i * K + j];
    } else {
        // the transposed DCT-III matrix has the DCT-II's input symmetry
        dct_pass<K, true, false>(x, P.invT);
        dct_pass<K, false, false>(x, P.invT);
        const float coef = 1.0f / (float)(K * 2);
#pragma unroll
        for (int e = 0; e < K * K; e++) g[e] = coef * x[e] * P.cni[e];
    }
}

// Gains of one coefficient vector from the frozen source group (in place:
// the source values become the gains) and the weight statistic (kept count
// or sum of squared Wiener gains), with the forward kernels' arithmetic.
template <int STEP, int N>
__device__ __forceinline__ float gains_vector(float* gs, int stride, bool dc, float T, float s2, int T3D)
{
    float s[N];
#pragma unroll
    for (int n = 0; n < N; n++) s[n] = gs[n * stride];
    if (T3D == kHADAMARD) hadamard<N>(s);
    else haar_fwd<N>(s);
    float stat = 0.f;
    const float coef = 1.0f / (float)N;
#pragma unroll
    for (int n = 0; n < N; n++) {
        float lam;
        if (STEP == 1) {
            lam = ((dc && n == 0) || fabsf(s[n]) > T) ? 1.0f : 0.0f;
            stat += lam;
        } else if (T3D == kHADAMARD) {
            float value = s[n] * s[n] * coef;
            value = value / (value + s2);
            lam = value * coef;
            stat = stat + value * value;
        } else {
            float value = s[n] * s[n];
            value = value / (value + s2);
            lam = value;
            stat = stat + value * value;
        }
        gs[n * stride] = lam;
    }
    return stat;
}

// Applies Hinv o Lambda o Hf to one coefficient vector of x (in place).
template <int STEP, int N>
__device__ __forceinline__ void apply_vector(float* gx, const float* glam, int stride, int T3D)
{
    float v[N];
#pragma unroll
    for (int n = 0; n < N; n++) v[n] = gx[n * stride];
    if (T3D == kHADAMARD) {
        hadamard<N>(v);
#pragma unroll
        for (int n = 0; n < N; n++) v[n] = v[n] * glam[n * stride];
        hadamard<N>(v);
        if (STEP == 1) {
            const float coef = 1.0f / (float)N;
#pragma unroll
            for (int n = 0; n < N; n++) v[n] = v[n] * coef;
        }
    } else {
        haar_fwd<N>(v);
#pragma unroll
        for (int n = 0; n < N; n++) v[n] = v[n] * glam[n * stride];
        haar_inv<N>(v);
    }
#pragma unroll
    for (int n = 0; n < N; n++) gx[n * stride] = v[n];
}

// The group's pixels into shared memory, lanes over its flattened elements
// (c, n, p, q).  The filters' gather_k runs lanes over a patch's pixels with
// the patches in unrolled loops; in these kernels (168 registers at k = 8,
// no cap) that form measured 7-9 % slower per linearised application.
template <int K, int SS>
__device__ __forceinline__ void gather_flat(const StepHead& P, const float* __restrict__ vid, const unsigned* idx,
                                            int nsx, int log2n, float* g, int lane)
{
    constexpr int K2 = K * K;
    const int total = P.C * nsx * K2;
    const long long W = P.W, wh = P.wh;
    const unsigned g0 = smem_addr(g);
    for (int e = lane; e < total; e += 32) {
        const int sl = e / K2, pq = e - sl * K2;
        const int c = sl >> log2n, n = sl & (nsx - 1);
        const int p = pq / K, q = pq - p * K;
        cp_async4s(g0 + 4u * (unsigned)(sl * SS + pq), vid + idx[n] + c * wh + p * W + q);
    }
}

template <int STEP, int NMAX>
__device__ __forceinline__ void gains_group(const StepParams& P, float* gs, int nsx, int ss, int lane, float* wgt)
{
    const int k2 = P.k * P.k, C = P.C;
    float acc[kMaxC] = {0.f, 0.f, 0.f};
    for (int v = lane; v < C * k2; v += 32) {
        const int c = v / k2, pq = v - c * k2;
        float* g = gs + (size_t)(c * nsx) * ss + pq;
        const float T = P.lambda3D * P.sigma[c] * (P.T3D == kHADAMARD ? sqrtf((float)nsx) : 1.0f);
        const float s2 = P.sigma[c] * P.sigma[c];
        float st;
        switch (nsx) {
            case 1: st = gains_vector<STEP, 1>(g, ss, pq == 0, T, s2, P.T3D); break;
            case 2: st = gains_vector<STEP, 2>(g, ss, pq == 0, T, s2, P.T3D); break;
            case 4: st = gains_vector<STEP, 4>(g, ss, pq == 0, T, s2, P.T3D); break;
            default: st = gains_vector<STEP, NMAX>(g, ss, pq == 0, T, s2, P.T3D); break;
        }
        acc[c] += st;
    }
#pragma unroll
    for (int c = 0; c < kMaxC; c++) {
        const float tot = warp_sum(acc[c]);
        const float s2 = P.sigma[c] * P.sigma[c];
        if (STEP == 2 && P.T3D == kHADAMARD) wgt[c] = tot > 0.0f ? 1.0f / (float)(s2 * tot) : 1.0f;
        else wgt[c] = 1.f / (float)(s2 * tot);
    }
    __syncwarp();
}

template <int STEP, int NMAX>
__device__ __forceinline__ void apply_group(const StepParams& P, float* gx, const float* glam, int nsx, int ss,
                                            int lane)
{
    const int k2 = P.k * P.k, C = P.C;
    for (int v = lane; v < C * k2; v += 32) {
        const int c = v / k2, pq = v - c * k2;
        float* x = gx + (size_t)(c * nsx) * ss + pq;
        const float* l = glam + (size_t)(c * nsx) * ss + pq;
        switch (nsx) {
            case 1: apply_vector<STEP, 1>(x, l, ss, P.T3D); break;
            case 2: apply_vector<STEP, 2>(x, l, ss, P.T3D); break;
            case 4: apply_vector<STEP, 4>(x, l, ss, P.T3D); break;
            default: apply_vector<STEP, NMAX>(x, l, ss, P.T3D); break;
        }
    }
    __syncwarp();
}

// ADJ == false: the linearised step applied to x, into the interleaved
// (num, den) accumulator.  ADJ == true: the adjoint applied to gp = g / den,
// scatter-added into out.  `src` is the frozen source of the gains (noisy
// for step 1, basic for step 2).
template <int STEP, int K, bool ADJ>
__global__ void __launch_bounds__(128)
linear_kernel(const StepParams P, const float* __restrict__ src, const float* __restrict__ x,
              const unsigned* __restrict__ tab_idx, const unsigned* __restrict__ tab_nsx, float* __restrict__ out,
              int warp_floats)
{
    constexpr int K2 = K * K, SS = K2 | 1;  // odd: a lane per slice reads on distinct banks
    extern __shared__ __align__(16) float fsm[];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const long long r = (long long)blockIdx.x * (blockDim.x >> 5) + wid;
    if (r >= P.nrefs) return;
    const int C = P.C;
    float* base = fsm + (size_t)wid * warp_floats;
    unsigned* idx = reinterpret_cast<unsigned*>(base);
    float* gS = base + kMaxN;
    float* gX = gS + (size_t)C * P.N * SS;

    const int nsx = (int)tab_nsx[r];
    const int log2n = __ffs(nsx) - 1;
    if (lane < nsx) idx[lane] = tab_idx[(size_t)r * P.N + lane];
    __syncwarp();
    const int nsl = C * nsx;

    gather_flat<K, SS>(P, src, idx, nsx, log2n, gS, lane);
    cp_async_wait_all();
    __syncwarp();
    for (int sl = lane; sl < nsl; sl += 32) slice_fwd2d<K>(gS + sl * SS, P, P);
    __syncwarp();
    float wgt[kMaxC];
    gains_group<STEP, 8>(P, gS, nsx, SS, lane, wgt);

    if (!ADJ) {
        gather_flat<K, SS>(P, x, idx, nsx, log2n, gX, lane);
        cp_async_wait_all();
        __syncwarp();
        for (int sl = lane; sl < nsl; sl += 32) slice_fwd2d<K>(gX + sl * SS, P, P);
        __syncwarp();
        apply_group<STEP, 8>(P, gX, gS, nsx, SS, lane);
        for (int sl = lane; sl < nsl; sl += 32) slice_inv2d<K>(gX + sl * SS, P, P);
        __syncwarp();
        const AggTarget A{nullptr, nullptr, out};
        for (int e = lane; e < nsl * K2; e += 32) {
            const int sl = e / K2, pq = e - sl * K2;
            const int c = sl >> log2n, n = sl & (nsx - 1);
            const int p = pq / K, q = pq - p * K;
            const float kw = P.kaiser[pq] * wgt[c];
            agg_add<true>(A, idx[n] + (size_t)c * P.wh + (size_t)p * P.W + q, kw * gX[sl * SS + pq], kw);
        }
    } else {
        // adjoint of the Kaiser-weighted scatter: gather g/den times K w
        for (int e = lane; e < nsl * K2; e += 32) {
            const int sl = e / K2, pq = e - sl * K2;
            const int c = sl >> log2n, n = sl & (nsx - 1);
            const int p = pq / K, q = pq - p * K;
            const float kw = P.kaiser[pq] * wgt[c];
            gX[sl * SS + pq] = kw * __ldg(x + idx[n] + (size_t)c * P.wh + (size_t)p * P.W + q);
        }
        __syncwarp();
        for (int sl = lane; sl < nsl; sl += 32) slice_inv2d_T<K>(gX + sl * SS, P);
        __syncwarp();
        apply_group<STEP, 8>(P, gX, gS, nsx, SS, lane);
        for (int sl = lane; sl < nsl; sl += 32) slice_fwd2d_T<K>(gX + sl * SS, P);
        __syncwarp();
        // adjoint of the gather: scatter-add
        for (int e = lane; e < nsl * K2; e += 32) {
            const int sl = e / K2, pq = e - sl * K2;
            const int c = sl >> log2n, n = sl & (nsx - 1);
            const int p = pq / K, q = pq - p * K;
            atomicAdd(out + idx[n] + (size_t)c * P.wh + (size_t)p * P.W + q, gX[sl * SS + pq]);
        }
    }
}

// out = den == 0 ? (identity ? x : 0) : num / den, from the accumulator.
__global__ void lin_normalize(const float2* __restrict__ pair, const float* __restrict__ x, float* __restrict__ out,
                              size_t n, int identity)
{
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float2 v = pair[i];
        out[i] = v.y == 0 ? (identity ? x[i] : 0.f) : v.x / v.y;
    }
}

// gp = den == 0 ? 0 : g / den
__global__ void adj_prescale(const float* __restrict__ g, const float* __restrict__ den, float* __restrict__ gp,
                             size_t n)
{
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        gp[i] = den[i] == 0 ? 0.f : g[i] / den[i];
}

// out += (den == 0 ? g : 0)   (step 1's identity fallback)
__global__ void adj_fallback(const float* __restrict__ g, const float* __restrict__ den, float* __restrict__ out,
                             size_t n)
{
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        if (den[i] == 0) out[i] += g[i];
}

__global__ void take_den(const float2* __restrict__ pair, float* __restrict__ den, size_t n)
{
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        den[i] = pair[i].y;
}

int grid_1d(size_t n)
{
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const size_t want = (n + 255) / 256;
    const size_t cap = (size_t)sms * 8;
    return (int)(want < cap ? (want ? want : 1) : cap);
}

template <int STEP, int K, bool ADJ>
cudaError_t launch_lin(const StepParams& P, const float* src, const float* x, const unsigned* tab_idx,
                       const unsigned* tab_nsx, float* out, cudaStream_t s)
{
    const int warps = 4;
    const int wf = kMaxN + 2 * P.C * P.N * (K * K + 1);
    const size_t smem = (size_t)warps * wf * sizeof(float);
    cudaError_t e = cudaFuncSetAttribute(linear_kernel<STEP, K, ADJ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    const long long blocks = (P.nrefs + warps - 1) / warps;
    linear_kernel<STEP, K, ADJ><<<(unsigned)blocks, warps * 32, smem, s>>>(P, src, x, tab_idx, tab_nsx, out, wf);
    return cudaGetLastError();
}

cudaError_t dispatch_lin(int step, bool adj, const StepParams& P, const float* src, const float* x,
                         const unsigned* tab_idx, const unsigned* tab_nsx, float* out, cudaStream_t s)
{
#define VBM3D_LIN(ST, KV)                                                                              \
    if (step == ST && P.k == KV)                                                                       \
        return adj ? launch_lin<ST, KV, true>(P, src, x, tab_idx, tab_nsx, out, s)                      \
                   : launch_lin<ST, KV, false>(P, src, x, tab_idx, tab_nsx, out, s);
    VBM3D_LIN(1, 7)
    VBM3D_LIN(1, 8)
    VBM3D_LIN(2, 7)
    VBM3D_LIN(2, 8)
#undef VBM3D_LIN
    return cudaErrorInvalidValue;
}

}  // namespace

// Frozen state of one linearised step.
struct LinearState {
    int step;
    StepParams P;
    const float* noisy;
    const float* basic;
    unsigned* tab_idx;
    unsigned* tab_nsx;
    float* den;
    float* pair;
    float* gp;
    size_t n;
};

}  // namespace vbm3d

using namespace vbm3d;

struct vbm3d_linear {
    LinearState st;
};

extern "C" {

int vbm3d_linear_create(int step, const vbm3d_params* prms, const float* noisy, const float* basic,
                        const float* fflow, const float* bflow, vbm3d_dims dims, float sigma, int color_space,
                        vbm3d_linear** out, void* stream)
{
    if (!out || !noisy || (step == 2 && !basic) || (step != 1 && step != 2)) {
        vbm3d::set_last_error(VBM3D_ERR_INVALID_ARGUMENT, "vbm3d_linear_create: bad step or NULL pointer");
        return VBM3D_ERR_INVALID_ARGUMENT;
    }
    vbm3d::StepParams P;
    int rc = vbm3d::build_step_params(prms, dims, sigma, color_space, P);
    if (rc) return rc;
    if (!((P.k == 7 || P.k == 8) && P.kt == 1 && P.N <= 8)) {
        vbm3d::set_last_error(VBM3D_ERR_UNSUPPORTED, "the linearised step supports k in {7, 8}, kt == 1, N <= 8");
        return VBM3D_ERR_UNSUPPORTED;
    }
    cudaStream_t s = (cudaStream_t)stream;
    vbm3d_linear* L = new vbm3d_linear;
    LinearState& S = L->st;
    S.step = step;
    S.P = P;
    S.noisy = noisy;
    S.basic = basic;
    S.n = (size_t)P.whc * P.F;
    cudaError_t e = cudaMalloc(&S.tab_idx, sizeof(unsigned) * (size_t)P.nrefs * P.N);
    if (e == cudaSuccess) e = cudaMalloc(&S.tab_nsx, sizeof(unsigned) * (size_t)P.nrefs);
    if (e == cudaSuccess) e = cudaMalloc(&S.den, sizeof(float) * S.n);
    if (e == cudaSuccess) e = cudaMalloc(&S.pair, sizeof(float) * 2 * S.n);
    if (e == cudaSuccess) e = cudaMalloc(&S.gp, sizeof(float) * S.n);
    const float* src = step == 1 ? noisy : basic;
    // frozen groups: the forward pass's block matching
    if (e == cudaSuccess)
        e = vbm3d::launch_bm(P, src, fflow, bflow, S.tab_idx, nullptr, nullptr, S.tab_nsx, P.nrefs, s, nullptr);
    // frozen denominator: the linearised step applied to the noisy input is
    // the forward step itself, so its accumulator holds the forward den
    if (e == cudaSuccess) e = cudaMemsetAsync(S.pair, 0, sizeof(float) * 2 * S.n, s);
    if (e == cudaSuccess) e = dispatch_lin(step, false, P, src, noisy, S.tab_idx, S.tab_nsx, S.pair, s);
    if (e == cudaSuccess) {
        take_den<<<grid_1d(S.n), 256, 0, s>>>(reinterpret_cast<const float2*>(S.pair), S.den, S.n);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) {
        vbm3d::set_last_error(VBM3D_ERR_CUDA, cudaGetErrorString(e));
        cudaFree(S.tab_idx);
        cudaFree(S.tab_nsx);
        cudaFree(S.den);
        cudaFree(S.pair);
        cudaFree(S.gp);
        delete L;
        return e == cudaErrorMemoryAllocation ? VBM3D_ERR_OUT_OF_MEMORY : VBM3D_ERR_CUDA;
    }
    *out = L;
    return VBM3D_OK;
}

int vbm3d_linear_apply(vbm3d_linear* L, const float* x, float* out, int adjoint, void* stream)
{
    if (!L || !x || !out) {
        vbm3d::set_last_error(VBM3D_ERR_INVALID_ARGUMENT, "vbm3d_linear_apply: NULL pointer");
        return VBM3D_ERR_INVALID_ARGUMENT;
    }
    LinearState& S = L->st;
    cudaStream_t s = (cudaStream_t)stream;
    const float* src = S.step == 1 ? S.noisy : S.basic;
    cudaError_t e;
    if (!adjoint) {
        e = cudaMemsetAsync(S.pair, 0, sizeof(float) * 2 * S.n, s);
        if (e == cudaSuccess) e = dispatch_lin(S.step, false, S.P, src, x, S.tab_idx, S.tab_nsx, S.pair, s);
        if (e == cudaSuccess) {
            lin_normalize<<<grid_1d(S.n), 256, 0, s>>>(reinterpret_cast<const float2*>(S.pair), x, out, S.n,
                                                       S.step == 1);
            e = cudaGetLastError();
        }
    } else {
        adj_prescale<<<grid_1d(S.n), 256, 0, s>>>(x, S.den, S.gp, S.n);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemsetAsync(out, 0, sizeof(float) * S.n, s);
        if (e == cudaSuccess) e = dispatch_lin(S.step, true, S.P, src, S.gp, S.tab_idx, S.tab_nsx, out, s);
        if (e == cudaSuccess && S.step == 1) {
            adj_fallback<<<grid_1d(S.n), 256, 0, s>>>(x, S.den, out, S.n);
            e = cudaGetLastError();
        }
    }
    if (e != cudaSuccess) {
        vbm3d::set_last_error(VBM3D_ERR_CUDA, cudaGetErrorString(e));
        return VBM3D_ERR_CUDA;
    }
    return VBM3D_OK;
}

int vbm3d_linear_den(vbm3d_linear* L, const float** den)
{
    if (!L || !den) return VBM3D_ERR_INVALID_ARGUMENT;
    *den = L->st.den;
    return VBM3D_OK;
}

void vbm3d_linear_destroy(vbm3d_linear* L)
{
    if (!L) return;
    cudaFree(L->st.tab_idx);
    cudaFree(L->st.tab_nsx);
    cudaFree(L->st.den);
    cudaFree(L->st.pair);
    cudaFree(L->st.gp);
    delete L;
}

}  // extern "C"
