// Generalised Dslash, 16-bit spinor storage: bfloat16, and half with a
// per-spinor norm.
#include "dslash_gen_impl.cuh"

namespace gbds {
cudaError_t launch_gen_half(int fmt, const Geom &g, int recon, int nrhs, const void *gauge, const void *psi, void *res,
                            int isign, int cb, const void *x, float coef, double *partials, cudaStream_t st, int variant) {
    if (fmt == kFmtBF16)
        return launch_gen_t<kFmtBF16>(g, recon, nrhs, gauge, psi, res, isign, cb, x, coef, partials, st, variant);
    return launch_gen_t<kFmtF16N>(g, recon, nrhs, gauge, psi, res, isign, cb, x, coef, partials, st, variant);
}
cudaError_t launch_gen_h16(int fmt, const Geom &g, int recon, const void *gauge, const void *psi, void *res, int isign,
                           int cb, const void *x, float coef, double *partials, cudaStream_t st) {
    if (fmt == kFmtBF16) return launch_gen_h16_t<kFmtBF16>(g, recon, gauge, psi, res, isign, cb, x, coef, partials, st);
    return launch_gen_h16_t<kFmtF16N>(g, recon, gauge, psi, res, isign, cb, x, coef, partials, st);
}

// FP32 internal links -> FP16 internal links, element by element (same
// grouping, half the bytes).
__global__ void links_to_f16(const float *__restrict__ in, __half *out, size_t n) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = __float2half_rn(in[i]);
}

cudaError_t convert_links_f16(const void *gauge32, void *gauge16, size_t nfloats, cudaStream_t st) {
    links_to_f16<<<1024, 256, 0, st>>>(static_cast<const float *>(gauge32), static_cast<__half *>(gauge16), nfloats);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_pack_gen_half(int fmt, const Geom &g, int nrhs, const float *packed, const int *table, int parity,
                                 void *out, cudaStream_t st) {
    if (fmt == kFmtBF16) return launch_pack_gen_t<kFmtBF16>(g, nrhs, packed, table, parity, out, st);
    return launch_pack_gen_t<kFmtF16N>(g, nrhs, packed, table, parity, out, st);
}
cudaError_t launch_unpack_gen_half(int fmt, const Geom &g, int nrhs, const void *in, const int *table, int parity,
                                   float *packed, cudaStream_t st) {
    if (fmt == kFmtBF16) return launch_unpack_gen_t<kFmtBF16>(g, nrhs, in, table, parity, packed, st);
    return launch_unpack_gen_t<kFmtF16N>(g, nrhs, in, table, parity, packed, st);
}
}  // namespace gbds
