// Double-float instantiations of the fused Dslash kernel (dfloat.cuh): FP64
// fields stored as (hi, lo) FP32 pairs and computed on the FP32 pipes, and
// the FP64 -> double-float conversion of whole fields (the way back is part
// of the unpack kernels).
#include "dslash_kernel.cuh"

namespace gbds {

namespace {

// n complex elements (16 bytes each), in place or out of place
__global__ void f64_to_df_kernel(const double2 *in, float4 *out, size_t n) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = df_from_double2(in[i]);
}

// ---------------------------------------------------------------------------
// Colour-split double-float Dslash (18-real links).  The one-thread-per-site
// kernel needs ~190 registers in double-float and runs latency-bound at 8-16
// warps per SM.  Here a CTA of three warps takes 32 consecutive sites and warp
// c computes colour c of their outputs: it loads colour c of the neighbour's
// four spins, projects it, and the three warps exchange the projected half
// spinors through shared memory (one barrier per hop, two buffers); each warp
// then needs only row c of U (forward) or column c of U (backward) and the
// four output spins of colour c, about half the registers, and every load and
// store stays coalesced over the 32 sites.
// ---------------------------------------------------------------------------

constexpr int kDf3Sites = 32;
constexpr int kDf3Minb = 8;  // CTAs of 96 threads per SM the registers are capped for (80, no spills)

__device__ __forceinline__ cx<dfloat> df_cx(float4 q) { return {dfloat(q.x, q.y), dfloat(q.z, q.w)}; }
__device__ __forceinline__ float4 df_f4(const cx<dfloat> &v) { return make_float4(v.r.hi, v.r.lo, v.i.hi, v.i.lo); }

// A sum of double-float products kept unnormalised: value = s + e, the
// products' high parts summed exactly by TwoSum into s and every rounding
// error (the products' low parts, the TwoSum errors) added into e.  12 FP32
// instructions a product against 15 for a double-float multiply-add, one
// TwoSum at the end; the error stays of order 2^-48 of the summed
// magnitudes, as in the double-float operations.
struct dsum {
    float s, e;
};

__device__ __forceinline__ dsum dsum_of(dfloat a) { return {a.hi, a.lo}; }

__device__ __forceinline__ void dsum_add_prod(dsum &a, dfloat x, dfloat y) {
    const float p = __fmul_rn(x.hi, y.hi);
    const float pe = df_prod_err(x, y, p);
    const dfloat t = df_two_sum(a.s, p);
    a.s = t.hi;
    a.e = __fadd_rn(a.e, __fadd_rn(t.lo, pe));
}

__device__ __forceinline__ dfloat dsum_value(dsum a) { return df_two_sum(a.s, a.e); }

// acc += m * v (CONJ: conj(m) * v) for the three colours j of a row
template <bool CONJ>
__device__ __forceinline__ void row_mac(const cx<dfloat> (&m)[3], const cx<dfloat> (&v)[3], cx<dfloat> &acc) {
    dsum re = dsum_of(acc.r), im = dsum_of(acc.i);
#pragma unroll
    for (int j = 0; j < 3; j++) {
        dsum_add_prod(re, m[j].r, v[j].r);
        dsum_add_prod(re, CONJ ? m[j].i : -m[j].i, CONJ ? v[j].i : v[j].i);
        dsum_add_prod(im, m[j].r, v[j].i);
        dsum_add_prod(im, CONJ ? -m[j].i : m[j].i, v[j].r);
    }
    acc = {dsum_value(re), dsum_value(im)};
}

// Colour c of the projected half spinor of psi(site), exchanged: hs[k][j]
// for all colours j on return.  Every thread of the CTA calls it (the
// barrier), inactive ones without loads.
template <int MU, int SIGMA>
__device__ __forceinline__ void df3_project(const float4 *__restrict__ psi, int stride, int site, int c, int lane,
                                            bool act, float4 (&sm)[2][3][kDf3Sites], cx<dfloat> (&hs)[2][3]) {
    using P = Proj<MU>;
    constexpr int f = SIGMA > 0 ? 0 : 1;
    if (act) {
        cx<dfloat> s[4];
#pragma unroll
        for (int sp = 0; sp < 4; sp++) s[sp] = df_cx(__ldg(psi + (size_t)(sp * 3 + c) * stride + site));
        sm[0][c][lane] = df_f4(cadd(s[0], mulc<P::a0 ^ f>(s[P::j0])));
        sm[1][c][lane] = df_f4(cadd(s[1], mulc<P::a1 ^ f>(s[P::j1])));
    }
    __syncthreads();
    if (act) {
#pragma unroll
        for (int k = 0; k < 2; k++)
#pragma unroll
            for (int j = 0; j < 3; j++) hs[k][j] = df_cx(sm[k][j][lane]);
    }
}

// Both hops of direction MU for colour c: the forward product's row c, then
// the backward one's FMA chains started from it (S = w_f + w_b) and
// D = 2 w_f - S, as in hop_pair_sd.
template <int ND, int ISIGN, int MU>
__device__ __forceinline__ void df3_dir(const DslashArgs<dfloat> &a, int h, int c, int lane, bool act, const Nbr &n,
                                        uint64_t pol, cx<dfloat> (&acc)[4], float4 (&sm)[2][2][3][kDf3Sites],
                                        int &buf) {
    using P = Proj<MU>;
    constexpr int f = ISIGN > 0 ? 0 : 1;
    const int stride = a.g.stride;
    cx<dfloat> hs[2][3], wf[2], w[2];
    df3_project<MU, ISIGN>(a.psi, stride, act ? n.f[MU] : 0, c, lane, act, sm[buf], hs);
    buf ^= 1;
    if (act) {
        const float4 *U = reinterpret_cast<const float4 *>(a.gauge + (size_t)(a.pt * ND + MU) * a.link_block_bytes);
        cx<dfloat> m[3];
#pragma unroll
        for (int j = 0; j < 3; j++) m[j] = df_cx(ld_once(U + (size_t)(c * 3 + j) * stride + h, pol));  // U_cj
#pragma unroll
        for (int k = 0; k < 2; k++) {
            wf[k] = {dfloat(), dfloat()};
            row_mac<false>(m, hs[k], wf[k]);
        }
    }
    df3_project<MU, -ISIGN>(a.psi, stride, act ? n.b[MU] : 0, c, lane, act, sm[buf], hs);
    buf ^= 1;
    if (act) {
        const int hb = n.b[MU];
        const float4 *U =
            reinterpret_cast<const float4 *>(a.gauge + (size_t)((1 - a.pt) * ND + MU) * a.link_block_bytes);
        cx<dfloat> m[3];
#pragma unroll
        for (int j = 0; j < 3; j++) m[j] = df_cx(ld_once(U + (size_t)(j * 3 + c) * stride + hb, pol));  // U_jc
#pragma unroll
        for (int k = 0; k < 2; k++) {
            w[k] = wf[k];
            row_mac<true>(m, hs[k], w[k]);  // (U^+)_cj = conj(U_jc)
        }
        // D = 2 w_f - S: the doubling is exact
        cx<dfloat> d[2];
#pragma unroll
        for (int k = 0; k < 2; k++)
            d[k] = {dfloat(2.f * wf[k].r.hi, 2.f * wf[k].r.lo) - w[k].r, dfloat(2.f * wf[k].i.hi, 2.f * wf[k].i.lo) - w[k].i};
        acc[0] = cadd(acc[0], w[0]);
        acc[1] = cadd(acc[1], w[1]);
        acc[2] = cadd(acc[2], mulc<P::b2 ^ f>(d[P::k2]));
        acc[3] = cadd(acc[3], mulc<P::b3 ^ f>(d[P::k3]));
    }
}

// res = Dslash psi (XPAY: res = x + coef Dslash psi), 18-real links
template <int ND, int ISIGN, bool XPAY>
__global__ void __launch_bounds__(3 * kDf3Sites, kDf3Minb)
    dslash_df3_kernel(const DslashArgs<dfloat> a, const float4 *__restrict__ x, dfloat coef) {
    __shared__ float4 sm[2][2][3][kDf3Sites];  // [buffer][half-spinor spin][colour][site]
    pdl_allow_next();
    const int lane = threadIdx.x & 31, c = threadIdx.x >> 5;
    const int h = blockIdx.x * kDf3Sites + lane;
    const bool act = h < a.g.Vh;
    Nbr n;
    if (act) neighbours<ND>(a.g, h, a.pt, n);
    const uint64_t pol = l2_evict_first_policy();
    pdl_wait_prev();
    cx<dfloat> acc[4];
#pragma unroll
    for (int sp = 0; sp < 4; sp++) acc[sp] = {dfloat(), dfloat()};
    int buf = 0;
    df3_dir<ND, ISIGN, 0>(a, h, c, lane, act, n, pol, acc, sm, buf);
    df3_dir<ND, ISIGN, 1>(a, h, c, lane, act, n, pol, acc, sm, buf);
    df3_dir<ND, ISIGN, 2>(a, h, c, lane, act, n, pol, acc, sm, buf);
    if constexpr (ND == 4) df3_dir<ND, ISIGN, 3>(a, h, c, lane, act, n, pol, acc, sm, buf);
    if (!act) return;
#pragma unroll
    for (int sp = 0; sp < 4; sp++) {
        const size_t i = (size_t)(sp * 3 + c) * a.g.stride + h;
        cx<dfloat> v = acc[sp];
        if constexpr (XPAY) {
            const cx<dfloat> xv = df_cx(__ldg(x + i));
            v = {fma(coef, v.r, xv.r), fma(coef, v.i, xv.i)};
        }
        __stcs(a.res + i, df_f4(v));
    }
}

template <bool XPAY>
cudaError_t launch_df3(const DslashArgs<dfloat> &a, int isign, const float4 *x, dfloat coef, cudaStream_t st) {
    const dim3 grid((a.g.Vh + kDf3Sites - 1) / kDf3Sites);
    const int threads = 3 * kDf3Sites;
    if (a.g.nd == 4) {
        if (isign > 0) launch_pdl(dslash_df3_kernel<4, 1, XPAY>, grid, threads, st, a, x, coef);
        else launch_pdl(dslash_df3_kernel<4, -1, XPAY>, grid, threads, st, a, x, coef);
    } else {
        if (isign > 0) launch_pdl(dslash_df3_kernel<3, 1, XPAY>, grid, threads, st, a, x, coef);
        else launch_pdl(dslash_df3_kernel<3, -1, XPAY>, grid, threads, st, a, x, coef);
    }
    count_launch();
    return cudaGetLastError();
}

DslashArgs<dfloat> df_args(const Geom &g, int recon, const void *gauge, const void *psi, void *res, int cb) {
    DslashArgs<dfloat> a;
    a.g = g;
    a.psi = static_cast<const float4 *>(psi);
    a.res = static_cast<float4 *>(res);
    a.gauge = static_cast<const char *>(gauge);
    a.link_block_bytes = (size_t)Field<dfloat>::link_vecs(recon) * g.stride * 16;
    a.pt = 1 - cb;
    return a;
}

dfloat to_df(double v) {
    const float hi = (float)v;
    return dfloat(hi, (float)(v - (double)hi));
}

}  // namespace

// Variant 0: the colour-split kernel (18-real links; 12-real links take the
// one-thread-per-site kernel capped for 4 CTAs); variants 1.. : the
// one-thread-per-site kernel with the register caps of Variants<dfloat>.
int dslash_variants_df() { return Variants<dfloat>::n; }

cudaError_t launch_dslash_df(const Geom &g, int recon, const void *gauge, const void *psi, void *res, int isign,
                             int cb, int block, int variant, cudaStream_t stream) {
    if (variant == 0) {
        if (recon == 18) return launch_df3<false>(df_args(g, recon, gauge, psi, res, cb), isign, nullptr, dfloat(), stream);
        variant = Variants<dfloat>::n - 1;
    }
    return launch_dslash_t<dfloat>(g, recon, gauge, psi, res, isign, cb, block, variant, stream);
}

cudaError_t launch_dslash_xpay_df(const Geom &g, int recon, const void *gauge, const void *psi, const void *x,
                                  double coef, void *res, double *partials, int isign, int cb, cudaStream_t stream) {
    if (recon == 18 && !partials)
        return launch_df3<true>(df_args(g, recon, gauge, psi, res, cb), isign, static_cast<const float4 *>(x),
                                to_df(coef), stream);
    return launch_dslash_xpay_t<dfloat>(g, recon, gauge, psi, x, to_df(coef), res, partials, isign, cb, stream);
}

cudaError_t launch_f64_to_df(const void *in, void *out, size_t n, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    f64_to_df_kernel<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(static_cast<const double2 *>(in),
                                                                       static_cast<float4 *>(out), n);
    count_launch();
    return cudaGetLastError();
}


}  // namespace gbds
