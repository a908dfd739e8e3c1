// FP64 instantiations of the fused Dslash kernel (4D/3D x recon 18/12 x isign).
#include "dslash_kernel.cuh"

namespace gbds {
cudaError_t launch_dslash_f64(const Geom &g, int recon, const void *gauge, const void *psi, void *res,
                              int isign, int cb, int block, int variant, cudaStream_t stream) {
    return launch_dslash_t<double>(g, recon, gauge, psi, res, isign, cb, block, variant, stream);
}
cudaError_t launch_dslash_xpay_f64(const Geom &g, int recon, const void *gauge, const void *psi, const void *x,
                                   double coef, void *res, double *partials, int isign, int cb, cudaStream_t stream) {
    return launch_dslash_xpay_t<double>(g, recon, gauge, psi, x, coef, res, partials, isign, cb, stream);
}
}  // namespace gbds
