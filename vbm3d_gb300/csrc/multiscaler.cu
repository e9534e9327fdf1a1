// The multiscaler's DCT pyramid on the GPU (multiscaler/multiscaler.cpp:21-100,
// decompose.cpp / recompose.cpp type 0, merge_coarse.cpp): the pre- and
// post-processing of the reference's multiscale denoising script
// (src/utils/VBM3Ddenoising_multiscale.sh), which splits each frame into
// DCT levels, denoises every level with VBM3D and merges the levels back.
//
// Every transform is FFTW's unnormalised REDFT10 (DCT-II) or REDFT01
// (DCT-III) of a whole frame, per channel.  Here a 2D transform of P planes
// of R x W floats is two dense products with cosine matrices: along the
// rows, one (P*R) x W by W x W product; along the columns, P products of
// R x R by R x W.  The products run on a batched single-precision tiled
// kernel (128 x 128 tiles, 8 x 8 outputs per thread, two shared-memory
// stages, explicit FMA), the cosine matrices are generated on the device in
// double and rounded to float.  The reference computes the same transforms
// with FFTW in float; the results agree to float rounding (a few 1e-6 of the
// data's range), not bit for bit.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <vector>

#include "common.cuh"
#include "../../include/vbm3d_gb300.h"

namespace vbm3d {
void set_last_error(int status, const char* msg);
}

namespace vbm3d {
namespace ms {
namespace {

int fail(int status, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
int fail(int status, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    set_last_error(status, buf);
    return status;
}

#define MCK(call)                                                                                              \
    do {                                                                                                       \
        cudaError_t e_ = (call);                                                                               \
        if (e_ != cudaSuccess)                                                                                 \
            return fail(e_ == cudaErrorMemoryAllocation ? VBM3D_ERR_OUT_OF_MEMORY : VBM3D_ERR_CUDA, "%s: %s", \
                        #call, cudaGetErrorString(e_));                                                        \
    } while (0)

// ------------------------------------------------------------ kernels ---

// Even / odd split of a length-n transform, ne = ceil(n / 2), no = n / 2.
// FFTW's REDFT10 (DCT-II), Y[k] = 2 sum_j x[j] cos(pi (j + 1/2) k / n):
// the even outputs are a ne x ne product with the folded sums
// x[j] + x[n-1-j] (j < no; the middle sample once when n is odd), the odd
// outputs a no x no product with the differences x[j] - x[n-1-j] (the
// cosine is symmetric in j for even k and antisymmetric for odd k).
// REDFT01 (DCT-III), y[m] = x[0] + 2 sum_{k>=1} x[k] cos(pi k (m + 1/2) / n):
// for m < ne, E[m] over the even inputs and O[m] over the odd ones give
// y[m] = E + O and y[n-1-m] = E - O (the middle output is E).
// Half matrices, row = output index, generated in double:
//   forward: He[i][j] = 2 cos(pi (j+1/2) 2i / n) (ne x ne), then
//            Ho[i][j] = 2 cos(pi (j+1/2) (2i+1) / n) (no x no);
//   inverse: Ge[m][i] = (i == 0 ? 1 : 2 cos(pi 2i (m+1/2) / n)) (ne x ne), then
//            Go[m][i] = 2 cos(pi (2i+1) (m+1/2) / n) (ne x no).
// Rows of both half matrices are padded to multiples of 4 floats (and
// the second starts on such a multiple), so products load them 16 bytes at
// a time; the padding holds zeros and lies outside every product's K.
__host__ __device__ inline int pad4(int x) { return (x + 3) & ~3; }
struct HalfLayout {
    int ld1, ld2;       // row strides of the first (ne rows) and second matrix
    long long off2;     // start of the second
    long long total;    // floats of both
};
__host__ __device__ inline HalfLayout half_layout(int n, bool inverse)
{
    const int ne = (n + 1) / 2, no = n / 2;
    HalfLayout h;
    h.ld1 = pad4(ne);
    h.ld2 = pad4(no);
    h.off2 = (long long)ne * h.ld1;
    h.total = h.off2 + (long long)(inverse ? ne : no) * h.ld2;
    return h;
}

__global__ void half_matrices_kernel(float* __restrict__ M, int n, int inverse)
{
    const int ne = (n + 1) / 2, no = n / 2;
    const HalfLayout hl = half_layout(n, inverse != 0);
    const double pi = 3.14159265358979323846;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < hl.total;
         e += (long long)gridDim.x * blockDim.x) {
        double v = 0.0;
        if (e < hl.off2) {
            const int r = (int)(e / hl.ld1), c = (int)(e - (long long)r * hl.ld1);
            if (c < ne) {
                if (!inverse) v = 2.0 * cos(pi * (c + 0.5) * (2 * r) / n);
                else v = c == 0 ? 1.0 : 2.0 * cos(pi * (2 * c) * (r + 0.5) / n);
            }
        } else {
            const long long f = e - hl.off2;
            const int r = (int)(f / hl.ld2), c = (int)(f - (long long)r * hl.ld2);
            if (c < no) {
                if (!inverse) v = 2.0 * cos(pi * (c + 0.5) * (2 * r + 1) / n);
                else v = 2.0 * cos(pi * (2 * c + 1) * (r + 0.5) / n);
            }
        }
        M[e] = (float)v;
    }
}

// The even and odd columns of the top-left rows x n block of P planes
// (row stride ld, plane stride sp) as dense rows: ev (rows of ld_e),
// od (rows of ld_o), P rows-row planes one after the other.
__global__ void split_cols_kernel(const float* __restrict__ src, long long sp, int ld, int rows, int n,
                                  float* __restrict__ ev, int lde, float* __restrict__ od, int ldo)
{
    const int ne = (n + 1) / 2, no = n / 2;
    const long long p = blockIdx.y;
    const long long total = (long long)rows * ne;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(e / ne), i = (int)(e - (long long)r * ne);
        const float* x = src + p * sp + (long long)r * ld;
        const long long row = p * rows + r;
        ev[row * lde + i] = x[2 * i];
        if (i < no) od[row * ldo + i] = x[2 * i + 1];
    }
}

// Folds along rows: src rows of n floats (row stride lds) -> the sums
// (ne per row, row stride lse) and the differences (no per row, row
// stride lso).
__global__ void fold_rows_kernel(const float* __restrict__ src, int lds, long long rows, int n,
                                 float* __restrict__ sum, int lse, float* __restrict__ dif, int lso)
{
    const int ne = (n + 1) / 2, no = n / 2;
    const long long total = rows * ne;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const long long r = e / ne;
        const int j = (int)(e - r * ne);
        const float* x = src + r * lds;
        if (j < no) {
            const float a = x[j], b = x[n - 1 - j];
            sum[r * lse + j] = a + b;
            dif[r * lso + j] = a - b;
        } else {
            sum[r * lse + j] = x[j];  // the middle sample of an odd length
        }
    }
}

// Folds along columns, per plane: rows j and n-1-j of an n x w plane (row
// stride w, plane stride n w) -> sums (ne x w per plane) and differences
// (no x w per plane).
__global__ void fold_cols_kernel(const float* __restrict__ src, int n, int w, float* __restrict__ sum,
                                 float* __restrict__ dif)
{
    const int ne = (n + 1) / 2, no = n / 2;
    const long long p = blockIdx.y;
    const float* x = src + p * n * (long long)w;
    const long long total = (long long)ne * w;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int j = (int)(e / w), c = (int)(e - (long long)j * w);
        if (j < no) {
            const float a = x[(long long)j * w + c], b = x[(long long)(n - 1 - j) * w + c];
            sum[(p * ne + j) * w + c] = a + b;
            dif[(p * no + j) * w + c] = a - b;
        } else {
            sum[(p * ne + j) * w + c] = x[(long long)j * w + c];
        }
    }
}

// Combines along rows: E, O (rows of ne) -> y (rows of n, row stride ldy):
// y[m] = E[m] + O[m], y[n-1-m] = E[m] - O[m] (m < no), the middle y = E.
__global__ void combine_rows_kernel(const float* __restrict__ E, const float* __restrict__ O, long long rows, int n,
                                    float* __restrict__ y, int ldy)
{
    const int ne = (n + 1) / 2, no = n / 2;
    const long long total = rows * ne;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const long long r = e / ne;
        const int m = (int)(e - r * ne);
        const float a = E[r * ne + m];
        float* out = y + r * ldy;
        if (m < no) {
            const float b = O[r * ne + m];
            out[m] = a + b;
            out[n - 1 - m] = a - b;
        } else {
            out[m] = a;
        }
    }
}

// Combines along columns, per plane: E, O (ne x w per plane) -> y (n x w).
__global__ void combine_cols_kernel(const float* __restrict__ E, const float* __restrict__ O, int n, int w,
                                    float* __restrict__ y)
{
    const int ne = (n + 1) / 2, no = n / 2;
    const long long p = blockIdx.y;
    const long long total = (long long)ne * w;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int m = (int)(e / w), c = (int)(e - (long long)m * w);
        const float a = E[(p * ne + m) * w + c];
        float* out = y + p * n * (long long)w;
        if (m < no) {
            const float b = O[(p * ne + m) * w + c];
            out[(long long)m * w + c] = a + b;
            out[(long long)(n - 1 - m) * w + c] = a - b;
        } else {
            out[(long long)m * w + c] = a;
        }
    }
}

struct Gemm {
    const float* A;  // M x K, row stride lda, column stride ask, batch stride sA
    const float* B;  // K x N (row stride ldb), or N x K when BT
    float* C;        // M x N, row stride ldc, column stride csc
    long long sA, sB, sC;
    int lda, ldb, ldc;
    int ask, csc;
    int M, N, K;
    float div;  // divides every result when != 1
};

constexpr int BM = 128, BN = 128, BK = 16, kThreads = 256;
constexpr int AP = BM + 4, BP = BN + 4;  // padded shared rows (16-byte multiples)

// Eight consecutive values row[k .. k+8) of a row with column stride cs
// (zero past K), as two 16-byte loads when the row is 16-byte aligned and
// dense (VEC) and the four are in range.
template <bool VEC>
__device__ __forceinline__ void load8(const float* __restrict__ row, int k, int K, float* v, int cs = 1)
{
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const int kk = k + 4 * h;
        if (VEC && kk + 3 < K) {
            const float4 q = __ldg(reinterpret_cast<const float4*>(row + kk));
            v[4 * h] = q.x;
            v[4 * h + 1] = q.y;
            v[4 * h + 2] = q.z;
            v[4 * h + 3] = q.w;
        } else {
#pragma unroll
            for (int i = 0; i < 4; i++) v[4 * h + i] = kk + i < K ? __ldg(row + (long long)(kk + i) * cs) : 0.f;
        }
    }
}

// C[b] = A[b] op(B[b]) (op(B) = B^T when BT) in float with FMA, one
// 128 x 128 tile per block; each thread owns rows {4ty..4ty+3, 64+4ty..}
// and columns {4tx..4tx+3, 64+4tx..} of the tile.  The next K slice of 16
// is loaded into registers while the current one is multiplied from shared
// memory (two stages, one barrier per slice).  Loaders: A (and B^T) one
// row per lane (rows t mod 128, K half t / 128), stored transposed without
// bank conflicts; B one K row per 16 lanes.  VA / VB: 16-byte loads (the
// operand's rows are 16-byte aligned).
template <bool BT, bool VA, bool VB>
__global__ void __launch_bounds__(kThreads, 2) gemm_kernel(const Gemm g)
{
    __shared__ __align__(16) float As[2][BK][AP];
    __shared__ __align__(16) float Bs[2][BK][BP];
    const long long b = blockIdx.z;
    const float* __restrict__ A = g.A + b * g.sA;
    const float* __restrict__ B = g.B + b * g.sB;
    float* __restrict__ C = g.C + b * g.sC;
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    const int t = threadIdx.x;
    const int lr = t & 127, lk = (t >> 7) * 8;
    const int bk = t >> 4, bn = (t & 15) * 8;
    float ra[8], rb[8];
    auto load = [&](int k0) {
        const int m = m0 + lr;
        if (m < g.M) {
            load8<VA>(A + (long long)m * g.lda, k0 + lk, g.K, ra, g.ask);
        } else {
#pragma unroll
            for (int i = 0; i < 8; i++) ra[i] = 0.f;
        }
        if (BT) {
            const int n = n0 + lr;
            if (n < g.N) {
                load8<VB>(B + (long long)n * g.ldb, k0 + lk, g.K, rb);
            } else {
#pragma unroll
                for (int i = 0; i < 8; i++) rb[i] = 0.f;
            }
        } else {
            const int k = k0 + bk;
            if (k < g.K) {
                load8<VB>(B + (long long)k * g.ldb + n0, bn, g.N - n0, rb);
            } else {
#pragma unroll
                for (int i = 0; i < 8; i++) rb[i] = 0.f;
            }
        }
    };
    auto store = [&](int s) {
#pragma unroll
        for (int i = 0; i < 8; i++) As[s][lk + i][lr] = ra[i];
        if (BT) {
#pragma unroll
            for (int i = 0; i < 8; i++) Bs[s][lk + i][lr] = rb[i];
        } else {
            *reinterpret_cast<float4*>(&Bs[s][bk][bn]) = make_float4(rb[0], rb[1], rb[2], rb[3]);
            *reinterpret_cast<float4*>(&Bs[s][bk][bn + 4]) = make_float4(rb[4], rb[5], rb[6], rb[7]);
        }
    };
    const int tx = t & 15, ty = t >> 4;
    float acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; i++)
#pragma unroll
        for (int j = 0; j < 8; j++) acc[i][j] = 0.f;

    load(0);
    store(0);
    __syncthreads();
    int s = 0;
    for (int k0 = 0; k0 < g.K; k0 += BK) {
        const bool more = k0 + BK < g.K;
        if (more) load(k0 + BK);
#pragma unroll
        for (int kk = 0; kk < BK; kk++) {
            const float4 a0 = *reinterpret_cast<const float4*>(&As[s][kk][4 * ty]);
            const float4 a1 = *reinterpret_cast<const float4*>(&As[s][kk][64 + 4 * ty]);
            const float4 b0 = *reinterpret_cast<const float4*>(&Bs[s][kk][4 * tx]);
            const float4 b1 = *reinterpret_cast<const float4*>(&Bs[s][kk][64 + 4 * tx]);
            const float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
            const float c[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
            for (int i = 0; i < 8; i++)
#pragma unroll
                for (int j = 0; j < 8; j++) acc[i][j] = __fmaf_rn(a[i], c[j], acc[i][j]);
        }
        if (more) {
            store(s ^ 1);
            __syncthreads();
            s ^= 1;
        }
    }
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const int m = m0 + (i < 4 ? 4 * ty + i : 64 + 4 * ty + i - 4);
        if (m >= g.M) continue;
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const int n = n0 + (j < 4 ? 4 * tx + j : 64 + 4 * tx + j - 4);
            if (n < g.N) C[(long long)m * g.ldc + (long long)n * g.csc] = g.div != 1.f ? acc[i][j] / g.div : acc[i][j];
        }
    }
}

// dst[p][r][c] = src[p][r][c] for r < bh, c < bw (row strides ldd, lds;
// plane strides sd, ss).
__global__ void copy_block_kernel(float* __restrict__ dst, long long sd, int ldd, const float* __restrict__ src,
                                  long long ss, int lds, int bh, int bw)
{
    const long long p = blockIdx.y;
    const long long total = (long long)bh * bw;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(e / bw), c = (int)(e - (long long)r * bw);
        dst[p * sd + (long long)r * ldd + c] = src[p * ss + (long long)r * lds + c];
    }
}

// ---------------------------------------------------------------- host ---

int gemm(bool bt, const Gemm& g, int batch, cudaStream_t s)
{
    if (g.M <= 0 || g.N <= 0 || g.K <= 0 || batch <= 0) return VBM3D_OK;
    const dim3 grid((unsigned)((g.N + BN - 1) / BN), (unsigned)((g.M + BM - 1) / BM), (unsigned)batch);
    if (grid.y > 65535u || grid.z > 65535u) return fail(VBM3D_ERR_UNSUPPORTED, "matrix product too large");
    // 16-byte loads: every row of the operand starts on a 16-byte boundary
    auto rows16 = [](const float* p, int ld, long long sb) {
        return ((uintptr_t)p & 15) == 0 && (ld & 3) == 0 && (sb & 3) == 0;
    };
    const bool va = g.ask == 1 && rows16(g.A, g.lda, g.sA), vb = rows16(g.B, g.ldb, g.sB);
#define MS_GEMM(BT_, VA_, VB_) gemm_kernel<BT_, VA_, VB_><<<grid, kThreads, 0, s>>>(g)
    if (bt) {
        if (va && vb) MS_GEMM(true, true, true);
        else if (va) MS_GEMM(true, true, false);
        else if (vb) MS_GEMM(true, false, true);
        else MS_GEMM(true, false, false);
    } else {
        if (va && vb) MS_GEMM(false, true, true);
        else if (va) MS_GEMM(false, true, false);
        else if (vb) MS_GEMM(false, false, true);
        else MS_GEMM(false, false, false);
    }
#undef MS_GEMM
    MCK(cudaGetLastError());
    return VBM3D_OK;
}

int half_matrices(float* M, int n, bool inverse, cudaStream_t s)
{
    const long long total = half_layout(n, inverse).total;
    const unsigned blocks = (unsigned)std::min<long long>((total + 255) / 256, 4096);
    half_matrices_kernel<<<blocks, 256, 0, s>>>(M, n, inverse ? 1 : 0);
    MCK(cudaGetLastError());
    return VBM3D_OK;
}

unsigned elementwise_blocks(long long total) { return (unsigned)std::min<long long>((total + 255) / 256, 4096); }

// Scratch of one call: plane stacks, the fold buffer and the half
// matrices of every size the call uses.
struct Scratch {
    float* base = nullptr;
    cudaStream_t s = nullptr;
    ~Scratch()
    {
        if (base) cudaFreeAsync(base, s);
    }
};

// The fold / combine buffer of transforms up to R x W (P planes): two
// blocks, each room for P (R + 1) rows of both halves (padded: at most
// 2 pad4((W + 2) / 2) floats per row), so that the inverse's split columns
// (first block) and its row products (second block) never meet; the
// forward folds and the column phases fit in the two together.
size_t fold_block(int P, int R, int W) { return (size_t)P * (R + 1) * 2 * pad4((W + 2) / 2); }
size_t fold_floats(int P, int R, int W) { return 2 * fold_block(P, R, W); }
size_t up64(size_t x) { return (x + 63) & ~size_t(63); }

// 2D DCT (dct_inplace) of P planes of R x W (contiguous) into Y, each value
// divided by float(4 R W): along the rows, fold and two half products into
// T (even outputs at even columns, odd at odd); along the columns, fold
// and two half products into Y's even and odd rows.  Mw, Mr: the REDFT10
// half matrices of W and R (half_layout); F: fold_floats(P, R, W) scratch.
int dct2d(const float* X, int P, int R, int W, const float* Mw, const float* Mr, float* T, float* F, float* Y,
          cudaStream_t s)
{
    const int we = (W + 1) / 2, wo = W / 2, re = (R + 1) / 2, ro = R / 2;
    const HalfLayout hw = half_layout(W, false), hr = half_layout(R, false);
    const long long rows = (long long)P * R;
    float* Fs = F;
    float* Fd = F + rows * hw.ld1;
    fold_rows_kernel<<<elementwise_blocks(rows * we), 256, 0, s>>>(X, W, rows, W, Fs, hw.ld1, Fd, hw.ld2);
    MCK(cudaGetLastError());
    Gemm g{};
    g.ask = 1; g.csc = 2; g.div = 1.f;
    g.A = Fs; g.lda = hw.ld1; g.sA = 0;
    g.B = Mw; g.ldb = hw.ld1; g.sB = 0;
    g.C = T; g.ldc = W; g.sC = 0;
    g.M = (int)rows; g.N = we; g.K = we;
    int rc = gemm(true, g, 1, s);
    if (rc) return rc;
    if (wo) {
        g.A = Fd; g.lda = hw.ld2;
        g.B = Mw + hw.off2; g.ldb = hw.ld2;
        g.C = T + 1;
        g.N = wo; g.K = wo;
        if ((rc = gemm(true, g, 1, s))) return rc;
    }
    Fs = F;
    Fd = F + (long long)P * re * W;
    fold_cols_kernel<<<dim3(elementwise_blocks((long long)re * W), (unsigned)P), 256, 0, s>>>(T, R, W, Fs, Fd);
    MCK(cudaGetLastError());
    g = Gemm{};
    g.ask = 1; g.csc = 1; g.div = (float)(4 * R * W);
    g.A = Mr; g.lda = hr.ld1; g.sA = 0;
    g.B = Fs; g.ldb = W; g.sB = (long long)re * W;
    g.C = Y; g.ldc = 2 * W; g.sC = (long long)R * W;
    g.M = re; g.N = W; g.K = re;
    if ((rc = gemm(false, g, P, s)) || !ro) return rc;
    g.A = Mr + hr.off2; g.lda = hr.ld2;
    g.B = Fd; g.sB = (long long)ro * W;
    g.C = Y + W;
    g.M = ro; g.K = ro;
    return gemm(false, g, P, s);
}

// 2D inverse DCT (idct_inplace) of the top-left h x w block of P planes
// of coefficients (row stride ldy, plane stride sy) into Z (P planes of
// h x w, contiguous): along the rows, the block's even and odd columns
// split into dense rows, half products over each, and their combination
// into U; along the columns, half products over U's even and odd rows and
// their combination into Z.  Mw, Mh: REDFT01 half matrices (half_layout);
// U: P h w scratch; F: fold_floats(P, h, w).
int idct2d(const float* Y, long long sy, int ldy, int P, int h, int w, const float* Mw, const float* Mh, float* U,
           float* F, float* Z, cudaStream_t s)
{
    const int we = (w + 1) / 2, wo = w / 2, he = (h + 1) / 2, ho = h / 2;
    const HalfLayout hw = half_layout(w, true), hh = half_layout(h, true);
    const long long rows = (long long)P * h;
    const long long half = (long long)fold_block(P, h, w);
    // even / odd coefficient columns, then the two products into E and O
    float* Ye = F;
    float* Yo = F + rows * hw.ld1;
    split_cols_kernel<<<dim3(elementwise_blocks((long long)h * we), (unsigned)P), 256, 0, s>>>(
        Y, sy, ldy, h, w, Ye, hw.ld1, Yo, hw.ld2);
    MCK(cudaGetLastError());
    float* E = F + half;
    float* O = E + rows * we;
    Gemm g{};
    g.ask = 1; g.csc = 1; g.div = 1.f;
    g.A = Ye; g.lda = hw.ld1; g.sA = 0;
    g.B = Mw; g.ldb = hw.ld1; g.sB = 0;
    g.C = E; g.ldc = we; g.sC = 0;
    g.M = (int)rows; g.N = we; g.K = we;
    int rc = gemm(true, g, 1, s);
    if (rc) return rc;
    if (wo) {
        g.A = Yo; g.lda = hw.ld2;
        g.B = Mw + hw.off2; g.ldb = hw.ld2;
        g.C = O;
        g.K = wo;
        if ((rc = gemm(true, g, 1, s))) return rc;
    }
    combine_rows_kernel<<<elementwise_blocks(rows * we), 256, 0, s>>>(E, O, rows, w, U, w);
    MCK(cudaGetLastError());
    E = F;
    O = F + (long long)P * he * w;
    g = Gemm{};
    g.ask = 1; g.csc = 1; g.div = 1.f;
    g.A = Mh; g.lda = hh.ld1; g.sA = 0;
    g.B = U; g.ldb = 2 * w; g.sB = (long long)h * w;
    g.C = E; g.ldc = w; g.sC = (long long)he * w;
    g.M = he; g.N = w; g.K = he;
    if ((rc = gemm(false, g, P, s))) return rc;
    if (ho) {
        g.A = Mh + hh.off2; g.lda = hh.ld2;
        g.B = U + w;
        g.C = O;
        g.K = ho;
        if ((rc = gemm(false, g, P, s))) return rc;
    }
    combine_cols_kernel<<<dim3(elementwise_blocks((long long)he * w), (unsigned)P), 256, 0, s>>>(E, O, h, w, Z);
    MCK(cudaGetLastError());
    return VBM3D_OK;
}

int copy_block(float* dst, long long sd, int ldd, const float* src, long long ss, int lds, int P, int bh, int bw,
               cudaStream_t s)
{
    if (bh <= 0 || bw <= 0) return VBM3D_OK;
    const long long total = (long long)bh * bw;
    const unsigned bx = (unsigned)std::min<long long>((total + 255) / 256, 1024);
    copy_block_kernel<<<dim3(bx, (unsigned)P), 256, 0, s>>>(dst, sd, ldd, src, ss, lds, bh, bw);
    MCK(cudaGetLastError());
    return VBM3D_OK;
}

// Rows (or columns) that `for (j = 0; j < n * factor; ++j)` visits for an
// int n and a float factor: the product and the comparison are in float
// (recompose.cpp:45-46, merge_coarse.cpp:34-35).
int block_count(int n, float factor)
{
    const volatile float bound = (float)n * factor;
    int j = 0;
    while ((float)j < bound) j++;
    return j;
}

// Level sizes: halved by integer division per level (decompose.cpp:56-57).
void level_sizes(int H, int W, int levels, std::vector<int>& hs, std::vector<int>& ws)
{
    hs.assign(levels, 0);
    ws.assign(levels, 0);
    int h = H, w = W;
    for (int i = 0; i < levels; i++) {
        hs[i] = h;
        ws[i] = w;
        h /= 2;
        w /= 2;
    }
}

// Half matrices of the sizes a call uses (forward or inverse), laid out one
// after the other (offsets per size index).
struct MatSet {
    std::vector<int> n;
    std::vector<bool> inv;
    std::vector<size_t> off;
    size_t total = 0;
    int add(int size, bool inverse)
    {
        for (size_t i = 0; i < n.size(); i++)
            if (n[i] == size && inv[i] == inverse) return (int)i;
        n.push_back(size);
        inv.push_back(inverse);
        off.push_back(total);
        total += (size_t)((half_layout(size, inverse).total + 63) & ~63LL);
        return (int)n.size() - 1;
    }
};

int check_dims(unsigned width, unsigned height, unsigned planes, unsigned levels)
{
    if (!width || !height || !planes || !levels)
        return fail(VBM3D_ERR_INVALID_ARGUMENT, "empty image, no planes or no levels");
    if (levels > 30 || (height >> (levels - 1)) == 0 || (width >> (levels - 1)) == 0)
        return fail(VBM3D_ERR_INVALID_ARGUMENT, "%u levels leave an empty level of a %ux%u image", levels, width,
                    height);
    if ((unsigned long long)planes * height > 8000000ull || width > 65536 || height > 65536)
        return fail(VBM3D_ERR_UNSUPPORTED, "image stack too large for one call");
    return VBM3D_OK;
}

}  // namespace
}  // namespace ms
}  // namespace vbm3d

using namespace vbm3d::ms;

extern "C" {

int vbm3d_gpu_ms_decompose(const float* in, unsigned width, unsigned height, unsigned planes, unsigned levels,
                           float* const* out, void* stream)
{
    if (!in || !out) return fail(VBM3D_ERR_INVALID_ARGUMENT, "NULL pointer");
    int rc = check_dims(width, height, planes, levels);
    if (rc) return rc;
    for (unsigned i = 0; i < levels; i++)
        if (!out[i]) return fail(VBM3D_ERR_INVALID_ARGUMENT, "NULL output level %u", i);
    const int W = (int)width, H = (int)height, P = (int)planes, L = (int)levels;
    cudaStream_t s = (cudaStream_t)stream;
    std::vector<int> hs, ws;
    level_sizes(H, W, L, hs, ws);
    MatSet ms;
    const int iDw = ms.add(W, false), iDh = ms.add(H, false);
    std::vector<int> iEw(L), iEh(L);
    for (int i = 0; i < L; i++) {
        iEw[i] = ms.add(ws[i], true);
        iEh[i] = ms.add(hs[i], true);
    }
    const size_t plane = (size_t)P * H * W;
    Scratch sc;
    sc.s = s;
    const size_t fold = up64(fold_floats(P, H, W)), pl = up64(plane);
    MCK(cudaMallocAsync(&sc.base, (2 * pl + fold + ms.total) * sizeof(float), s));
    float* T = sc.base;
    float* Y = T + pl;
    float* F = Y + pl;
    float* mats = F + fold;
    for (size_t i = 0; i < ms.n.size(); i++)
        if ((rc = half_matrices(mats + ms.off[i], ms.n[i], ms.inv[i], s))) return rc;
    if ((rc = dct2d(in, P, H, W, mats + ms.off[iDw], mats + ms.off[iDh], T, F, Y, s))) return rc;
    for (int i = 0; i < L; i++)
        if ((rc = idct2d(Y, (long long)H * W, W, P, hs[i], ws[i], mats + ms.off[iEw[i]], mats + ms.off[iEh[i]], T,
                         F, out[i], s)))
            return rc;
    return VBM3D_OK;
}

int vbm3d_gpu_ms_recompose(const float* const* levels_in, unsigned width, unsigned height, unsigned planes,
                           unsigned levels, float factor, float* out, void* stream)
{
    if (!levels_in || !out) return fail(VBM3D_ERR_INVALID_ARGUMENT, "NULL pointer");
    int rc = check_dims(width, height, planes, levels);
    if (rc) return rc;
    for (unsigned i = 0; i < levels; i++)
        if (!levels_in[i]) return fail(VBM3D_ERR_INVALID_ARGUMENT, "NULL input level %u", i);
    if (!(factor <= 1.0f))
        return fail(VBM3D_ERR_INVALID_ARGUMENT, "recompose factor %g > 1 (the reference copies past the level)",
                    (double)factor);
    const int W = (int)width, H = (int)height, P = (int)planes, L = (int)levels;
    cudaStream_t s = (cudaStream_t)stream;
    std::vector<int> hs, ws;
    level_sizes(H, W, L, hs, ws);
    MatSet ms;
    std::vector<int> iDw(L), iDh(L);
    for (int i = 0; i < L; i++) {
        iDw[i] = ms.add(ws[i], false);
        iDh[i] = ms.add(hs[i], false);
    }
    const int iEw = ms.add(W, true), iEh = ms.add(H, true);
    const size_t plane = (size_t)P * H * W;
    Scratch sc;
    sc.s = s;
    const size_t fold = up64(fold_floats(P, H, W)), pl = up64(plane);
    MCK(cudaMallocAsync(&sc.base, (3 * pl + fold + ms.total) * sizeof(float), s));
    float* T = sc.base;
    float* Yo = T + pl;
    float* Yi = Yo + pl;
    float* F = Yi + pl;
    float* mats = F + fold;
    for (size_t i = 0; i < ms.n.size(); i++)
        if ((rc = half_matrices(mats + ms.off[i], ms.n[i], ms.inv[i], s))) return rc;
    // the DCT of level 0, then each coarser level's low frequencies over it
    if ((rc = dct2d(levels_in[0], P, H, W, mats + ms.off[iDw[0]], mats + ms.off[iDh[0]], T, F, Yo, s))) return rc;
    for (int i = 1; i < L; i++) {
        const int h = hs[i], w = ws[i];
        if ((rc = dct2d(levels_in[i], P, h, w, mats + ms.off[iDw[i]], mats + ms.off[iDh[i]], T, F, Yi, s)))
            return rc;
        const int bh = std::min(block_count(h, factor), h), bw = std::min(block_count(w, factor), w);
        if ((rc = copy_block(Yo, (long long)H * W, W, Yi, (long long)h * w, w, P, bh, bw, s))) return rc;
    }
    return idct2d(Yo, (long long)H * W, W, P, H, W, mats + ms.off[iEw], mats + ms.off[iEh], T, F, out, s);
}

int vbm3d_gpu_ms_merge_coarse(const float* fine, const float* coarse, unsigned width, unsigned height,
                              unsigned cwidth, unsigned cheight, unsigned planes, float factor, float* out,
                              void* stream)
{
    if (!fine || !coarse || !out) return fail(VBM3D_ERR_INVALID_ARGUMENT, "NULL pointer");
    int rc = check_dims(width, height, planes, 1);
    if (rc) return rc;
    if ((rc = check_dims(cwidth, cheight, planes, 1))) return rc;
    if (!(factor <= 1.0f))
        return fail(VBM3D_ERR_INVALID_ARGUMENT, "merge factor %g > 1 (the reference copies past the coarse image)",
                    (double)factor);
    const int W = (int)width, H = (int)height, P = (int)planes, cw = (int)cwidth, ch = (int)cheight;
    const int bh = block_count(ch, factor), bw = block_count(cw, factor);
    if (bh > H || bw > W)
        return fail(VBM3D_ERR_INVALID_ARGUMENT, "coarse block %dx%d larger than the fine image", bw, bh);
    cudaStream_t s = (cudaStream_t)stream;
    MatSet ms;
    const int iDw = ms.add(W, false), iDh = ms.add(H, false), iDcw = ms.add(cw, false), iDch = ms.add(ch, false);
    const int iEw = ms.add(W, true), iEh = ms.add(H, true);
    const size_t plane = (size_t)P * H * W, cplane = (size_t)P * ch * cw;
    Scratch sc;
    sc.s = s;
    const size_t big = up64(std::max(plane, cplane)), pl = up64(plane);
    const size_t fold = up64(std::max(fold_floats(P, H, W), fold_floats(P, ch, cw)));
    MCK(cudaMallocAsync(&sc.base, (pl + 2 * big + fold + ms.total) * sizeof(float), s));
    float* Yo = sc.base;
    float* Yc = Yo + pl;
    float* T = Yc + big;
    float* F = T + big;
    float* mats = F + fold;
    for (size_t i = 0; i < ms.n.size(); i++)
        if ((rc = half_matrices(mats + ms.off[i], ms.n[i], ms.inv[i], s))) return rc;
    if ((rc = dct2d(fine, P, H, W, mats + ms.off[iDw], mats + ms.off[iDh], T, F, Yo, s))) return rc;
    if ((rc = dct2d(coarse, P, ch, cw, mats + ms.off[iDcw], mats + ms.off[iDch], T, F, Yc, s))) return rc;
    if ((rc = copy_block(Yo, (long long)H * W, W, Yc, (long long)ch * cw, cw, P, std::min(bh, ch), std::min(bw, cw),
                         s)))
        return rc;
    return idct2d(Yo, (long long)H * W, W, P, H, W, mats + ms.off[iEw], mats + ms.off[iEh], T, F, out, s);
}

}  // extern "C"
