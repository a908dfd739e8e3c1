// FP32 instantiations of the fused Dslash kernel (4D/3D x recon 18/12 x isign).
#include "dslash_kernel.cuh"

namespace gbds {
cudaError_t launch_dslash_f32(const Geom &g, int recon, const void *gauge, const void *psi, void *res,
                              int isign, int cb, int block, int variant, cudaStream_t stream) {
    return launch_dslash_t<float>(g, recon, gauge, psi, res, isign, cb, block, variant, stream);
}
int dslash_variants(int prec) { return prec == 32 ? Variants<float>::n : Variants<double>::n; }
cudaError_t launch_dslash_xpay_f32(const Geom &g, int recon, const void *gauge, const void *psi, const void *x,
                                   float coef, void *res, double *partials, int isign, int cb, cudaStream_t stream) {
    return launch_dslash_xpay_t<float>(g, recon, gauge, psi, x, coef, res, partials, isign, cb, stream);
}
}  // namespace gbds
