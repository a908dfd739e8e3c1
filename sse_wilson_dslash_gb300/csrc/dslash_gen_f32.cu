// Generalised Dslash, FP32 spinor storage (several right-hand sides).
#include "dslash_gen_impl.cuh"

namespace gbds {
cudaError_t launch_gen_f32(const Geom &g, int recon, int nrhs, const void *gauge, const void *psi, void *res, int isign,
                           int cb, const void *x, float coef, double *partials, cudaStream_t st, int variant) {
    return launch_gen_t<kFmtNative>(g, recon, nrhs, gauge, psi, res, isign, cb, x, coef, partials, st, variant);
}
cudaError_t launch_pack_gen_f32(const Geom &g, int nrhs, const float *packed, const int *table, int parity, void *out,
                                cudaStream_t st) {
    return launch_pack_gen_t<kFmtNative>(g, nrhs, packed, table, parity, out, st);
}
cudaError_t launch_unpack_gen_f32(const Geom &g, int nrhs, const void *in, const int *table, int parity, float *packed,
                                  cudaStream_t st) {
    return launch_unpack_gen_t<kFmtNative>(g, nrhs, in, table, parity, packed, st);
}
}  // namespace gbds
