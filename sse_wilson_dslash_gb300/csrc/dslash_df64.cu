// FP64-class Dslash in float-float ("df64") arithmetic on the FP32 units.
//
// GB300 issues about two FP64 FMAs per SM clock, so the IEEE-FP64 Dslash is
// arithmetic-bound (~1.5 ms at 32^3x64 against a 0.24 ms memory floor).  Here
// every real is a pair of floats (hi, lo) with hi + lo carrying ~48
// significant bits (unit roundoff 2^-48 ~ 3.6e-15), and the arithmetic uses
// the error-free transformations of the double-float literature:
//   TwoSum (Knuth): s = a + b, e = (a - (s - bb)) + (b - bb), bb = s - a;
//   FastTwoSum (Dekker), |a| >= |b|: s = a + b, e = b - (s - a);
//   TwoProd via FMA: p = a * b, e = fma(a, b, -p);
//   double-float add: TwoSum of the high parts and TwoSum of the low parts,
//   folded together with two FastTwoSum renormalisations (the accurate form:
//   its error is bounded relative to the result even when the operands
//   cancel); multiply-add: TwoProd of the high parts plus the two cross
//   products, then the add.
// Fields keep the double layout's 16 bytes per complex: float4
// {re.hi, re.lo, im.hi, im.lo}.  The layout kernels below convert from and to
// IEEE doubles once per field; the Dslash itself runs no FP64 instruction.
#include <cuda_runtime.h>

#include "dslash_kernel.cuh"

namespace gbds {
namespace {

struct df {
    float hi, lo;
};

__device__ __forceinline__ df fast_two_sum(float a, float b) {
    const float s = a + b;
    return {s, b - (s - a)};
}

__device__ __forceinline__ df two_sum(float a, float b) {
    const float s = a + b;
    const float bb = s - a;
    return {s, (a - (s - bb)) + (b - bb)};
}

__device__ __forceinline__ df dadd(df a, df b) {
    const df s = two_sum(a.hi, b.hi);
    const df t = two_sum(a.lo, b.lo);
    df r = fast_two_sum(s.hi, s.lo + t.hi);
    return fast_two_sum(r.hi, r.lo + t.lo);
}

__device__ __forceinline__ df dneg(df a) { return {-a.hi, -a.lo}; }

// a * b + c
__device__ __forceinline__ df dfma(df a, df b, df c) {
    const float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    return dadd(fast_two_sum(p, e), c);
}

struct dcx {
    df r, i;
};

__device__ __forceinline__ dcx cxadd(dcx a, dcx b) { return {dadd(a.r, b.r), dadd(a.i, b.i)}; }

template <int CODE>
__device__ __forceinline__ dcx dmulc(dcx a) {
    if constexpr (CODE == 0) return a;
    else if constexpr (CODE == 1) return {dneg(a.r), dneg(a.i)};
    else if constexpr (CODE == 2) return {dneg(a.i), a.r};
    else return {a.i, dneg(a.r)};
}

__device__ __forceinline__ dcx ld(const float4 *p) {
    const float4 q = __ldg(p);
    return {{q.x, q.y}, {q.z, q.w}};
}

template <int MU, int SIGMA>
__device__ __forceinline__ void dproject(const dcx (&s)[4][3], dcx (&h)[2][3]) {
    using P = Proj<MU>;
    constexpr int f = SIGMA > 0 ? 0 : 1;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        h[0][c] = cxadd(s[0][c], dmulc<P::a0 ^ f>(s[P::j0][c]));
        h[1][c] = cxadd(s[1][c], dmulc<P::a1 ^ f>(s[P::j1][c]));
    }
}

template <int MU, int SIGMA>
__device__ __forceinline__ void dreconstruct(dcx (&acc)[4][3], const dcx (&w)[2][3]) {
    using P = Proj<MU>;
    constexpr int f = SIGMA > 0 ? 0 : 1;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        acc[0][c] = cxadd(acc[0][c], w[0][c]);
        acc[1][c] = cxadd(acc[1][c], w[1][c]);
        acc[2][c] = cxadd(acc[2][c], dmulc<P::b2 ^ f>(w[P::k2][c]));
        acc[3][c] = cxadd(acc[3][c], dmulc<P::b3 ^ f>(w[P::k3][c]));
    }
}

// w_k = U h_k or U^+ h_k; the link is read element by element to keep
// registers down (the loads hit L1 after the first half spinor).
template <bool DAG, int RECON>
__device__ __forceinline__ void dsu3(const float4 *__restrict__ lk, int stride, int h, const dcx (&hv)[2][3],
                                     dcx (&w)[2][3]) {
    dcx U[3][3];
    constexpr int n = RECON == 18 ? 9 : 6;
#pragma unroll
    for (int k = 0; k < n; k++) U[k / 3][k % 3] = ld(lk + (size_t)k * stride + h);
    if constexpr (RECON == 12) {
#pragma unroll
        for (int j = 0; j < 3; j++) {
            const int k = (j + 1) % 3, l = (j + 2) % 3;
            const dcx a = U[0][k], b = U[1][l], c = U[0][l], d = U[1][k];
            // conj(a b - c d)
            df re = dfma(a.r, b.r, dneg(dfma(a.i, b.i, {0.f, 0.f})));
            re = dfma(dneg(c.r), d.r, re);
            re = dfma(c.i, d.i, re);
            df im = dfma(a.r, b.i, dfma(a.i, b.r, {0.f, 0.f}));
            im = dfma(dneg(c.r), d.i, im);
            im = dfma(dneg(c.i), d.r, im);
            U[2][j] = {re, dneg(im)};
        }
    }
#pragma unroll
    for (int k = 0; k < 2; k++)
#pragma unroll
        for (int i = 0; i < 3; i++) {
            df re = {0.f, 0.f}, im = {0.f, 0.f};
#pragma unroll
            for (int j = 0; j < 3; j++) {
                const dcx m = DAG ? U[j][i] : U[i][j];
                const dcx v = hv[k][j];
                if (DAG) {
                    re = dfma(m.r, v.r, re);
                    re = dfma(m.i, v.i, re);
                    im = dfma(m.r, v.i, im);
                    im = dfma(dneg(m.i), v.r, im);
                } else {
                    re = dfma(m.r, v.r, re);
                    re = dfma(dneg(m.i), v.i, re);
                    im = dfma(m.r, v.i, im);
                    im = dfma(m.i, v.r, im);
                }
            }
            w[k][i] = {re, im};
        }
}

struct DfArgs {
    Geom g;
    const float4 *psi;
    float4 *res;
    const char *gauge;
    size_t link_block_bytes;
    int pt;
    const float4 *x;  // xpay: res = x + coef * D psi (nullptr: plain)
    df coef;
};

template <int ND, int RECON, int ISIGN, int MU>
__device__ __forceinline__ void dhop(const DfArgs &a, int h, const Nbr &n, dcx (&acc)[4][3]) {
    const int ps = 1 - a.pt;
    dcx s[4][3], hs[2][3], w[2][3];
#pragma unroll
    for (int k = 0; k < 12; k++) s[k / 3][k % 3] = ld(a.psi + (size_t)k * a.g.stride + n.f[MU]);
    dproject<MU, ISIGN>(s, hs);
    dsu3<false, RECON>(reinterpret_cast<const float4 *>(a.gauge + (size_t)(a.pt * ND + MU) * a.link_block_bytes),
                       a.g.stride, h, hs, w);
    dreconstruct<MU, ISIGN>(acc, w);
#pragma unroll
    for (int k = 0; k < 12; k++) s[k / 3][k % 3] = ld(a.psi + (size_t)k * a.g.stride + n.b[MU]);
    dproject<MU, -ISIGN>(s, hs);
    dsu3<true, RECON>(reinterpret_cast<const float4 *>(a.gauge + (size_t)(ps * ND + MU) * a.link_block_bytes),
                      a.g.stride, n.b[MU], hs, w);
    dreconstruct<MU, -ISIGN>(acc, w);
}

template <int ND, int RECON, int ISIGN>
__global__ void __launch_bounds__(128) dslash_df64_kernel(const DfArgs a) {
    const int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= a.g.Vh) return;
    Nbr n;
    neighbours<ND>(a.g, h, a.pt, n);
    dcx acc[4][3];
#pragma unroll
    for (int s = 0; s < 4; s++)
#pragma unroll
        for (int c = 0; c < 3; c++) acc[s][c] = {{0.f, 0.f}, {0.f, 0.f}};
    dhop<ND, RECON, ISIGN, 0>(a, h, n, acc);
    dhop<ND, RECON, ISIGN, 1>(a, h, n, acc);
    dhop<ND, RECON, ISIGN, 2>(a, h, n, acc);
    if constexpr (ND == 4) dhop<ND, RECON, ISIGN, 3>(a, h, n, acc);
#pragma unroll
    for (int k = 0; k < 12; k++) {
        dcx v = acc[k / 3][k % 3];
        if (a.x) {
            const dcx xv = ld(a.x + (size_t)k * a.g.stride + h);
            v = {dfma(a.coef, v.r, xv.r), dfma(a.coef, v.i, xv.i)};
        }
        __stcs(a.res + (size_t)k * a.g.stride + h, make_float4(v.r.hi, v.r.lo, v.i.hi, v.i.lo));
    }
}

// IEEE double <-> df64 pairs, elementwise over n doubles (a field's reals).
__global__ void to_df64(const double *__restrict__ in, float2 *out, size_t n) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const double x = in[i];
        const float hi = __double2float_rn(x);
        out[i] = make_float2(hi, __double2float_rn(x - (double)hi));
    }
}

__global__ void from_df64(const float2 *__restrict__ in, double *out, size_t n) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float2 v = in[i];
        out[i] = (double)v.x + (double)v.y;
    }
}

}  // namespace

cudaError_t launch_dslash_df64(const Geom &g, int recon, const void *gauge, const void *psi, void *res, int isign, int cb,
                               const void *x, double coef, cudaStream_t st) {
    DfArgs a;
    a.g = g;
    a.psi = static_cast<const float4 *>(psi);
    a.res = static_cast<float4 *>(res);
    a.gauge = static_cast<const char *>(gauge);
    a.link_block_bytes = (size_t)(recon == 18 ? 9 : 6) * 16 * g.stride;
    a.pt = 1 - cb;
    a.x = static_cast<const float4 *>(x);
    const float chi = (float)coef;
    a.coef = {chi, (float)(coef - (double)chi)};
    const dim3 grid((g.Vh + 127) / 128);
#define GBDS_DF(ND, R, S) dslash_df64_kernel<ND, R, S><<<grid, 128, 0, st>>>(a)
    if (g.nd == 4) {
        if (recon == 18) { if (isign > 0) GBDS_DF(4, 18, 1); else GBDS_DF(4, 18, -1); }
        else             { if (isign > 0) GBDS_DF(4, 12, 1); else GBDS_DF(4, 12, -1); }
    } else {
        if (recon == 18) { if (isign > 0) GBDS_DF(3, 18, 1); else GBDS_DF(3, 18, -1); }
        else             { if (isign > 0) GBDS_DF(3, 12, 1); else GBDS_DF(3, 12, -1); }
    }
#undef GBDS_DF
    count_launch();
    return cudaGetLastError();
}

// In-place conversion of a field of n doubles (IEEE <-> df64 pairs, same bytes).
cudaError_t convert_df64(void *field, size_t n, int to_df, cudaStream_t st) {
    if (to_df) to_df64<<<1024, 256, 0, st>>>(static_cast<const double *>(field), static_cast<float2 *>(field), n);
    else from_df64<<<1024, 256, 0, st>>>(static_cast<const float2 *>(field), static_cast<double *>(field), n);
    count_launch();
    return cudaGetLastError();
}

}  // namespace gbds
