// Instantiations of the path kernel, plain FP64 form.
#include "hexo_paths.cuh"
#include "hexo_launch.h"

namespace hexo {

const void *paths_kernel_ptr_f64(uint32_t ppt, uint32_t unroll, bool cv) {
    if (cv) return ppt == 1 && unroll == 1 ? (const void *)paths_kernel<false, 1, 1, true> : nullptr;
    switch (ppt * 10u + unroll) {
    case 11: return (const void *)paths_kernel<false, 1, 1>;
    case 12: return (const void *)paths_kernel<false, 1, 2>;
    case 14: return (const void *)paths_kernel<false, 1, 4>;
    case 21: return (const void *)paths_kernel<false, 2, 1>;
    case 22: return (const void *)paths_kernel<false, 2, 2>;
    case 24: return (const void *)paths_kernel<false, 2, 4>;
    case 41: return (const void *)paths_kernel<false, 4, 1>;
    case 42: return (const void *)paths_kernel<false, 4, 2>;
    case 44: return (const void *)paths_kernel<false, 4, 4>;
    default: return nullptr;
    }
}

} // namespace hexo
