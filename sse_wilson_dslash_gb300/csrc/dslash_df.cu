// Double-float instantiations of the fused Dslash kernel (dfloat.cuh): FP64
// fields stored as (hi, lo) FP32 pairs and computed on the FP32 pipes, and
// the FP64 <-> double-float conversions of whole fields.
#include "dslash_kernel.cuh"

namespace gbds {

namespace {

// n complex elements (16 bytes each), in place or out of place
__global__ void f64_to_df_kernel(const double2 *in, float4 *out, size_t n) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = df_from_double2(in[i]);
}

__global__ void df_to_f64_kernel(const float4 *in, double2 *out, size_t n) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = df_to_double2(in[i]);
}

}  // namespace

int dslash_variants_df() { return Variants<dfloat>::n; }

cudaError_t launch_dslash_df(const Geom &g, int recon, const void *gauge, const void *psi, void *res, int isign,
                             int cb, int block, int variant, cudaStream_t stream) {
    return launch_dslash_t<dfloat>(g, recon, gauge, psi, res, isign, cb, block, variant, stream);
}

cudaError_t launch_dslash_xpay_df(const Geom &g, int recon, const void *gauge, const void *psi, const void *x,
                                  double coef, void *res, double *partials, int isign, int cb, cudaStream_t stream) {
    const float hi = (float)coef;
    const dfloat c(hi, (float)(coef - (double)hi));
    return launch_dslash_xpay_t<dfloat>(g, recon, gauge, psi, x, c, res, partials, isign, cb, stream);
}

cudaError_t launch_f64_to_df(const void *in, void *out, size_t n, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    f64_to_df_kernel<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(static_cast<const double2 *>(in),
                                                                       static_cast<float4 *>(out), n);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_df_to_f64(const void *in, void *out, size_t n, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    df_to_f64_kernel<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(static_cast<const float4 *>(in),
                                                                       static_cast<double2 *>(out), n);
    count_launch();
    return cudaGetLastError();
}

}  // namespace gbds
