// healpix.cu -- placeholder, replaced by the HEALPix kernels.
#include "common.cuh"
namespace catana_gpu {
catana_status_t healpix_bin_dev(DeviceContext *, int64_t, const double *, int64_t, int64_t *, double *, int *,
                                cudaStream_t) { return CATANA_ERR_UNSUPPORTED; }
catana_status_t healpix_ang2pix_dev(int64_t, const double *, const double *, int64_t, int64_t *, int *,
                                    cudaStream_t) { return CATANA_ERR_UNSUPPORTED; }
catana_status_t healpix_pix2ang_dev(int64_t, const int64_t *, int64_t, double *, double *, cudaStream_t) {
    return CATANA_ERR_UNSUPPORTED;
}
catana_status_t healpix_sfb_dev(DeviceContext *, int64_t, const int64_t *, const double *, int64_t, int, int, bool,
                                bool, const double *, double, double *, double *, int *, cudaStream_t) {
    return CATANA_ERR_UNSUPPORTED;
}
}  // namespace catana_gpu
