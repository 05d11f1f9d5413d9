// sfb_split.cu -- placeholder, replaced by the tcgen05 split-precision kernels.
#include "common.cuh"
namespace catana_gpu {
catana_status_t split_raw_accumulate(DeviceContext *, const double *, const double *, int64_t, int, int, double,
                                     const double *, double *, int *, cudaStream_t) {
    return CATANA_ERR_UNSUPPORTED;
}
}  // namespace catana_gpu
