// Step-1 work kernels of the batched form (see batch.cu), one translation
// unit per step so that the two compile in parallel.
#include "batch_kernels.cuh"

namespace vbm3d {
namespace batched {

const void* work_kernel_step1(int phase, int cls)
{
    if (phase == 0) {
        switch (cls) {
            case 0: return reinterpret_cast<const void*>(batch_bm_kernel<1, 7, 1, 16>);
            case 1: return reinterpret_cast<const void*>(batch_bm_kernel<1, 7, 3, 32>);
            case 2: return reinterpret_cast<const void*>(batch_bm_kernel<1, 8, 1, 16>);
            case 3: return reinterpret_cast<const void*>(batch_bm_kernel<1, 8, 3, 32>);
            default: return nullptr;
        }
    }
    if (phase == 1) {
        switch (cls) {
            case 0: return reinterpret_cast<const void*>(batch_filter_kernel<1, 7, 1>);
            case 1:  // DCT and bior1.5 tables share the k = 8 kernels
            case 2: return reinterpret_cast<const void*>(batch_filter_kernel<1, 8, 1>);
            case 3: return reinterpret_cast<const void*>(batch_filter_kernel<1, 7, 4>);  // one channel
            case 4:
            case 5: return reinterpret_cast<const void*>(batch_filter_kernel<1, 8, 4>);
            default: return nullptr;
        }
    }
    return nullptr;
}

}  // namespace batched
}  // namespace vbm3d
