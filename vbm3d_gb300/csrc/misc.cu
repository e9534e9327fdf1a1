// K-N: numerator / denominator division and the colour transforms.
// Both are elementwise and HBM-bound: grid-stride loops over float4 where
// the pointers allow it.
#include "common.cuh"

namespace vbm3d {

// run_vbm3d's division (src/vbm3d.cpp:168-170, :198-202).
__global__ void normalize_kernel(const float* num, const float* __restrict__ den,
                                 const float* __restrict__ fb, float* out, size_t n)
{
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool vec = ((reinterpret_cast<uintptr_t>(num) | reinterpret_cast<uintptr_t>(den) |
                       reinterpret_cast<uintptr_t>(fb) | reinterpret_cast<uintptr_t>(out)) & 15) == 0;
    if (vec) {
        const size_t n4 = n / 4;
        for (size_t j = i; j < n4; j += stride) {
            const float4 a = reinterpret_cast<const float4*>(num)[j];
            const float4 b = reinterpret_cast<const float4*>(den)[j];
            const float4 f = reinterpret_cast<const float4*>(fb)[j];
            float4 o;
            o.x = b.x == 0 ? f.x : a.x / b.x;
            o.y = b.y == 0 ? f.y : a.y / b.y;
            o.z = b.z == 0 ? f.z : a.z / b.z;
            o.w = b.w == 0 ? f.w : a.w / b.w;
            reinterpret_cast<float4*>(out)[j] = o;
        }
        for (size_t j = n4 * 4 + i; j < n; j += stride) out[j] = den[j] == 0 ? fb[j] : num[j] / den[j];
    } else {
        for (size_t j = i; j < n; j += stride) out[j] = den[j] == 0 ? fb[j] : num[j] / den[j];
    }
}

// Interleaved (num, den) accumulator -> separate numerator / denominator.
__global__ void split_pair_kernel(const float2* __restrict__ pair, float* __restrict__ num, float* __restrict__ den,
                                  size_t n)
{
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float2 v = pair[i];
        num[i] = v.x;
        den[i] = v.y;
    }
}

// run_vbm3d's division read straight from the interleaved accumulator.
__global__ void normalize_pair_kernel(const float2* __restrict__ pair, const float* __restrict__ fb,
                                      float* __restrict__ out, size_t n)
{
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float2 v = pair[i];
        out[i] = v.y == 0 ? fb[i] : v.x / v.y;
    }
}

// transformColorSpace, 3 channels, in place (color3 in common.cuh).
__global__ void color_kernel(float* __restrict__ v, unsigned wh, unsigned frames, int forward)
{
    const size_t n = (size_t)wh * frames;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const size_t f = i / wh, k = i - f * wh;
        float* r = v + f * 3 * (size_t)wh + k;
        float* g = r + wh;
        float* b = g + wh;
        float o0 = *r, o1 = *g, o2 = *b;
        color3(o0, o1, o2, forward != 0);
        *r = o0;
        *g = o1;
        *b = o2;
    }
}

static int grid_for(size_t n, int threads)
{
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const size_t want = (n + threads - 1) / threads;
    const size_t cap = (size_t)sms * 8;  // 8 resident blocks of 256 threads per SM
    return (int)(want < cap ? (want ? want : 1) : cap);
}

cudaError_t launch_normalize(const float* num, const float* den, const float* fb, float* out, size_t n,
                             cudaStream_t s)
{
    normalize_kernel<<<grid_for(n / 4 + 1, 256), 256, 0, s>>>(num, den, fb, out, n);
    return cudaGetLastError();
}

cudaError_t launch_split_pair(const float* pair, float* num, float* den, size_t n, cudaStream_t s)
{
    split_pair_kernel<<<grid_for(n, 256), 256, 0, s>>>(reinterpret_cast<const float2*>(pair), num, den, n);
    return cudaGetLastError();
}

cudaError_t launch_normalize_pair(const float* pair, const float* fb, float* out, size_t n, cudaStream_t s)
{
    normalize_pair_kernel<<<grid_for(n, 256), 256, 0, s>>>(reinterpret_cast<const float2*>(pair), fb, out, n);
    return cudaGetLastError();
}

cudaError_t launch_color(float* v, unsigned wh, unsigned frames, int forward, cudaStream_t s)
{
    color_kernel<<<grid_for((size_t)wh * frames, 256), 256, 0, s>>>(v, wh, frames, forward);
    return cudaGetLastError();
}

}  // namespace vbm3d
