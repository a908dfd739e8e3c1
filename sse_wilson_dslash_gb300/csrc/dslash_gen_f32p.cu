// Generalised Dslash, FP32 spinor storage in spin pairs (several right-hand
// sides; the fully packed kernel's operand layout).
#include "dslash_gen_impl.cuh"

namespace gbds {
cudaError_t launch_gen_f32p(const Geom &g, int recon, int nrhs, const void *gauge, const void *psi, void *res, int isign,
                            int cb, const void *x, float coef, double *partials, cudaStream_t st, int variant) {
    return launch_gen_t<kFmtF32Pairs>(g, recon, nrhs, gauge, psi, res, isign, cb, x, coef, partials, st, variant);
}
cudaError_t launch_gen_f32p_cg_update(const Geom &g, int recon, int nrhs, const void *gauge, const void *psi, int isign,
                                      int cb, const void *x, float coef, const RhsCgScalars *rsc, void *r,
                                      double *partials, cudaStream_t st) {
    return launch_gen_cg_update_t<kFmtF32Pairs>(g, recon, nrhs, gauge, psi, isign, cb, x, coef, rsc, r, partials, st);
}
cudaError_t launch_pack_gen_f32p(const Geom &g, int nrhs, const float *packed, const int *table, int parity, void *out,
                                 cudaStream_t st) {
    return launch_pack_gen_t<kFmtF32Pairs>(g, nrhs, packed, table, parity, out, st);
}
cudaError_t launch_unpack_gen_f32p(const Geom &g, int nrhs, const void *in, const int *table, int parity, float *packed,
                                   cudaStream_t st) {
    return launch_unpack_gen_t<kFmtF32Pairs>(g, nrhs, in, table, parity, packed, st);
}
}  // namespace gbds
