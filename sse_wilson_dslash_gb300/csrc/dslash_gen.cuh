// Generalised Dslash: several right-hand sides per site and reduced-precision
// spinor storage, FP32 arithmetic, FP32 links (18 or 12 reals).
//
// Spinor field of one checkerboard with NRHS right-hand sides, element
// (component k, site h, rhs r) at  k * CS + h * NRHS + r,  CS = stride * NRHS:
// the right-hand-side index runs fastest, so the NRHS lanes that work on one
// site read one link (a broadcast load) and consecutive lanes read
// consecutive spinor words.  With NRHS right-hand sides a site's 2*nd links
// are read once for all of them: compulsory bytes per site and rhs are
// 2 s + 2 nd g / NRHS (s, g = spinor, link bytes).
//
// Storage formats (SpinorIO):
//   F32   6 float4 per spinor (96 B)
//   BF16  3 uint4 per spinor, 24 bfloat16 (48 B)
//   F16N  3 uint4 per spinor, 24 half scaled by a per-spinor float norm
//         stored after the components (48 + 4 B): value = half * norm,
//         norm = max |component|.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "dslash_kernel.cuh"

namespace gbds {

enum SpinorFormat { kFmtNative = 0, kFmtBF16 = 1, kFmtF16N = 2 };

// Load/store of one spinor at element index i, component stride cs (elements).
template <int FMT> struct Sio;

template <>
struct Sio<kFmtNative> {
    static constexpr int kBytes = 96;
    __device__ __forceinline__ static void load(const char *base, size_t cs, size_t i, cx<float> (&s)[4][3]) {
        const float4 *p = reinterpret_cast<const float4 *>(base);
        float v[24];
#pragma unroll
        for (int k = 0; k < 6; k++) {
            const float4 q = __ldg(p + k * cs + i);
            v[4 * k] = q.x; v[4 * k + 1] = q.y; v[4 * k + 2] = q.z; v[4 * k + 3] = q.w;
        }
#pragma unroll
        for (int j = 0; j < 12; j++) s[j / 3][j % 3] = {v[2 * j], v[2 * j + 1]};
    }
    __device__ __forceinline__ static void store(char *base, size_t cs, size_t i, const cx<float> (&s)[4][3]) {
        float4 *p = reinterpret_cast<float4 *>(base);
#pragma unroll
        for (int k = 0; k < 6; k++) {
            const cx<float> a = s[(2 * k) / 3][(2 * k) % 3], b = s[(2 * k + 1) / 3][(2 * k + 1) % 3];
            __stcs(p + k * cs + i, make_float4(a.r, a.i, b.r, b.i));
        }
    }
};

template <>
struct Sio<kFmtBF16> {
    static constexpr int kBytes = 48;
    __device__ __forceinline__ static void load(const char *base, size_t cs, size_t i, cx<float> (&s)[4][3]) {
        const uint4 *p = reinterpret_cast<const uint4 *>(base);
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const uint4 q = __ldg(p + k * cs + i);
            const unsigned w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
            for (int c = 0; c < 4; c++) {  // one complex per 32-bit word
                const __nv_bfloat162 b = *reinterpret_cast<const __nv_bfloat162 *>(&w[c]);
                const float2 f = __bfloat1622float2(b);
                const int j = 4 * k + c;
                s[j / 3][j % 3] = {f.x, f.y};
            }
        }
    }
    __device__ __forceinline__ static void store(char *base, size_t cs, size_t i, const cx<float> (&s)[4][3]) {
        uint4 *p = reinterpret_cast<uint4 *>(base);
#pragma unroll
        for (int k = 0; k < 3; k++) {
            unsigned w[4];
#pragma unroll
            for (int c = 0; c < 4; c++) {
                const int j = 4 * k + c;
                const __nv_bfloat162 b = __floats2bfloat162_rn(s[j / 3][j % 3].r, s[j / 3][j % 3].i);
                w[c] = *reinterpret_cast<const unsigned *>(&b);
            }
            __stcs(p + k * cs + i, make_uint4(w[0], w[1], w[2], w[3]));
        }
    }
};

template <>
struct Sio<kFmtF16N> {
    static constexpr int kBytes = 52;
    // norms follow the three uint4 component arrays
    __device__ __forceinline__ static const float *norms(const char *base, size_t cs) {
        return reinterpret_cast<const float *>(base + 3 * 16 * cs);
    }
    // the stored halves, not multiplied by the norm (values in [-1, 1])
    __device__ __forceinline__ static void load_raw(const char *base, size_t cs, size_t i, cx<float> (&s)[4][3]) {
        const uint4 *p = reinterpret_cast<const uint4 *>(base);
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const uint4 q = __ldg(p + k * cs + i);
            const unsigned w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
            for (int c = 0; c < 4; c++) {
                const float2 f = __half22float2(*reinterpret_cast<const __half2 *>(&w[c]));
                const int j = 4 * k + c;
                s[j / 3][j % 3] = {f.x, f.y};
            }
        }
    }
    __device__ __forceinline__ static void load(const char *base, size_t cs, size_t i, cx<float> (&s)[4][3]) {
        const uint4 *p = reinterpret_cast<const uint4 *>(base);
        const float nrm = __ldg(norms(base, cs) + i);
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const uint4 q = __ldg(p + k * cs + i);
            const unsigned w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
            for (int c = 0; c < 4; c++) {
                const __half2 b = *reinterpret_cast<const __half2 *>(&w[c]);
                const float2 f = __half22float2(b);
                const int j = 4 * k + c;
                s[j / 3][j % 3] = {f.x * nrm, f.y * nrm};
            }
        }
    }
    __device__ __forceinline__ static void store(char *base, size_t cs, size_t i, const cx<float> (&s)[4][3]) {
        float m = 0.f;
#pragma unroll
        for (int j = 0; j < 12; j++) m = fmaxf(m, fmaxf(fabsf(s[j / 3][j % 3].r), fabsf(s[j / 3][j % 3].i)));
        const float inv = m > 0.f ? 1.f / m : 0.f;
        uint4 *p = reinterpret_cast<uint4 *>(base);
#pragma unroll
        for (int k = 0; k < 3; k++) {
            unsigned w[4];
#pragma unroll
            for (int c = 0; c < 4; c++) {
                const int j = 4 * k + c;
                const __half2 b = __floats2half2_rn(s[j / 3][j % 3].r * inv, s[j / 3][j % 3].i * inv);
                w[c] = *reinterpret_cast<const unsigned *>(&b);
            }
            __stcs(p + k * cs + i, make_uint4(w[0], w[1], w[2], w[3]));
        }
        __stcs(reinterpret_cast<float *>(base + 3 * 16 * cs) + i, m);
    }
};

// Link loads: LFMT 0 = FP32 (float2 x 9 or float4 x 3), LFMT 1 = FP16 with the
// same component grouping (half2 x 9 or 4 x half in a uint2, x 3).  SU(3)
// entries are bounded by 1, so half needs no scaling.
template <int LFMT, int RECON>
__device__ __forceinline__ void load_link_g(const char *base, int stride, int h, cx<float> (&U)[3][3]) {
    if constexpr (LFMT == 0) {
        Field<float>::template load_link<RECON>(base, stride, h, U);
    } else if constexpr (RECON == 18) {
        const unsigned *p = reinterpret_cast<const unsigned *>(base);
#pragma unroll
        for (int k = 0; k < 9; k++) {
            const unsigned w = __ldg(p + (size_t)k * stride + h);
            const float2 f = __half22float2(*reinterpret_cast<const __half2 *>(&w));
            U[k / 3][k % 3] = {f.x, f.y};
        }
    } else {
        const uint2 *p = reinterpret_cast<const uint2 *>(base);
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const uint2 q = __ldg(p + (size_t)k * stride + h);
            const float2 a = __half22float2(*reinterpret_cast<const __half2 *>(&q.x));
            const float2 b = __half22float2(*reinterpret_cast<const __half2 *>(&q.y));
            U[(2 * k) / 3][(2 * k) % 3] = {a.x, a.y};
            U[(2 * k + 1) / 3][(2 * k + 1) % 3] = {b.x, b.y};
        }
        reconstruct_row2(U);
    }
}

struct GenArgs {
    Geom g;
    const char *psi;           // source checkerboard
    char *res;                 // target checkerboard
    const char *gauge;         // FP32 links, both checkerboards
    size_t link_block_bytes;   // one (parity, mu) block
    size_t cs;                 // component stride of the spinor arrays (elements) = stride * NRHS
    int nrhs;                  // right-hand sides (used when the kernel's NRHS is 0)
    int pt;                    // target parity
    // xpay epilogue: res = x + coef * D psi, |res|^2 partials
    const char *x;
    float coef;
    double *partials;
};

// NRHS > 0: compile-time count; NRHS == 0: a.nrhs at run time.
template <int NRHS>
__device__ __forceinline__ int nrhs_of(const GenArgs &a) { return NRHS > 0 ? NRHS : a.nrhs; }

template <int FMT, int RECON, int ISIGN, int NRHS, int MU, int LFMT>
__device__ __forceinline__ void gen_hop_pair(const GenArgs &a, int h, int r, const Nbr &n, cx<float> (&acc)[4][3]) {
    const int ps = 1 - a.pt;
    const int nr = nrhs_of<NRHS>(a);
    cx<float> s[4][3], hs[2][3], w[2][3], U[3][3];
    Sio<FMT>::load(a.psi, a.cs, (size_t)n.f[MU] * nr + r, s);
    load_link_g<LFMT, RECON>(a.gauge + (size_t)(a.pt * 4 + MU) * a.link_block_bytes, a.g.stride, h, U);
    project<MU, ISIGN>(s, hs);
    su3_mul<false>(U, hs, w);
    reconstruct<MU, ISIGN>(acc, w);
    Sio<FMT>::load(a.psi, a.cs, (size_t)n.b[MU] * nr + r, s);
    load_link_g<LFMT, RECON>(a.gauge + (size_t)(ps * 4 + MU) * a.link_block_bytes, a.g.stride, n.b[MU], U);
    project<MU, -ISIGN>(s, hs);
    su3_mul<true>(U, hs, w);
    reconstruct<MU, -ISIGN>(acc, w);
}

// Per-rhs sums over a 128-thread block of (site, rhs) threads, rhs fastest:
// partials[blockIdx.x * NRHS + r].  Lanes l and l + k NRHS of a warp hold
// the same rhs.
template <int NRHS>
__device__ __forceinline__ void block_sum_rhs(double *partials, float v) {
    static_assert(NRHS >= 2 && NRHS <= 32 && 32 % NRHS == 0, "NRHS must divide the warp");
#pragma unroll
    for (int o = 16; o >= NRHS; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __shared__ double ws[4][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane < NRHS) ws[w][lane] = (double)v;
    __syncthreads();
    if (threadIdx.x < NRHS)
        partials[(size_t)blockIdx.x * NRHS + threadIdx.x] =
            ws[0][threadIdx.x] + ws[1][threadIdx.x] + ws[2][threadIdx.x] + ws[3][threadIdx.x];
}

// ---------------------------------------------------------------------------
// Variant with the colour multiply in packed FP32x2 arithmetic (NRHS 8..32,
// FP32 links): each CTA first stages the eight links of each of its sites in
// shared memory as splats (Mr, Mr, -Mi, Mi) of M = U (forward hop) or
// M = U^dagger (backward hop), so that
//   w_i = sum_j (Mr, Mr) * (hr, hi) + (-Mi, Mi) * (hi, hr)
// is two __ffma2_rn per complex multiply-add with no operand moves; the nrhs
// threads of a site read each staged entry as a shared-memory broadcast.
// ---------------------------------------------------------------------------

// w_k = M h_k (k = 0, 1) from the staged splats M[i*3 + j]
__device__ __forceinline__ void su3_mul_splat(const float4 *M, const cx<float> (&h)[2][3], cx<float> (&w)[2][3]) {
    float2 hv[2][3], hs[2][3];
#pragma unroll
    for (int k = 0; k < 2; k++)
#pragma unroll
        for (int j = 0; j < 3; j++) {
            hv[k][j] = make_float2(h[k][j].r, h[k][j].i);
            hs[k][j] = make_float2(h[k][j].i, h[k][j].r);
        }
#pragma unroll
    for (int i = 0; i < 3; i++) {
        float2 w0 = make_float2(0.f, 0.f), w1 = make_float2(0.f, 0.f);
#pragma unroll
        for (int j = 0; j < 3; j++) {
            const float4 m = M[i * 3 + j];
            const float2 a = make_float2(m.x, m.y), b = make_float2(m.z, m.w);
            w0 = __ffma2_rn(a, hv[0][j], w0);
            w0 = __ffma2_rn(b, hs[0][j], w0);
            w1 = __ffma2_rn(a, hv[1][j], w1);
            w1 = __ffma2_rn(b, hs[1][j], w1);
        }
        w[0][i] = {w0.x, w0.y};
        w[1][i] = {w1.x, w1.y};
    }
}

template <int FMT, int RECON, int ISIGN, int NRHS, int EPI>
__global__ void __launch_bounds__(128, 6) dslash_gen2_kernel(const GenArgs a) {
    static_assert(NRHS >= 8 && NRHS <= 32, "8 to 32 right-hand sides");
    constexpr int P = 128 / NRHS;  // sites per CTA
    __shared__ float4 sL[P][8][9];
    const int t = threadIdx.x;
    const int p = t / NRHS, r = t % NRHS;
    const int h = blockIdx.x * P + p;
    const bool act = h < a.g.Vh;
    Nbr n;
    if (act) neighbours<4>(a.g, h, a.pt, n);
    if (act && r < 8) {
        // link r of the site: direction r / 2, forward (even r) or backward
        const int mu = r >> 1;
        const bool bwd = r & 1;
        const int nbm = mu == 0 ? n.b[0] : (mu == 1 ? n.b[1] : (mu == 2 ? n.b[2] : n.b[3]));
        const int lp = bwd ? 1 - a.pt : a.pt;
        cx<float> U[3][3];
        Field<float>::template load_link<RECON>(a.gauge + (size_t)(lp * 4 + mu) * a.link_block_bytes, a.g.stride,
                                                bwd ? nbm : h, U);
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) {
                // forward: M_ij = U_ij; backward: M_ij = conj(U_ji)
                const float mr = bwd ? U[j][i].r : U[i][j].r;
                const float mi = bwd ? -U[j][i].i : U[i][j].i;
                sL[p][r][i * 3 + j] = make_float4(mr, mr, -mi, mi);
            }
    }
    __syncthreads();
    float nrm = 0.f;
    if (act) {
        cx<float> acc[4][3];
#pragma unroll
        for (int s = 0; s < 4; s++)
#pragma unroll
            for (int c = 0; c < 3; c++) acc[s][c] = {0.f, 0.f};
#define GBDS_G2_HOP(MU)                                                              \
    {                                                                                \
        cx<float> sp[4][3], hs[2][3], w[2][3];                                       \
        Sio<FMT>::load(a.psi, a.cs, (size_t)n.f[MU] * NRHS + r, sp);                 \
        project<MU, ISIGN>(sp, hs);                                                  \
        su3_mul_splat(sL[p][2 * MU], hs, w);                                         \
        reconstruct<MU, ISIGN>(acc, w);                                              \
        Sio<FMT>::load(a.psi, a.cs, (size_t)n.b[MU] * NRHS + r, sp);                 \
        project<MU, -ISIGN>(sp, hs);                                                 \
        su3_mul_splat(sL[p][2 * MU + 1], hs, w);                                     \
        reconstruct<MU, -ISIGN>(acc, w);                                             \
    }
        GBDS_G2_HOP(0)
        GBDS_G2_HOP(1)
        GBDS_G2_HOP(2)
        GBDS_G2_HOP(3)
#undef GBDS_G2_HOP
        const size_t i = (size_t)h * NRHS + r;
        if constexpr (EPI) {
            cx<float> xv[4][3];
            Sio<FMT>::load(a.x, a.cs, i, xv);
#pragma unroll
            for (int s = 0; s < 4; s++)
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    acc[s][c].r = fmaf(a.coef, acc[s][c].r, xv[s][c].r);
                    acc[s][c].i = fmaf(a.coef, acc[s][c].i, xv[s][c].i);
                    nrm = fmaf(acc[s][c].r, acc[s][c].r, nrm);
                    nrm = fmaf(acc[s][c].i, acc[s][c].i, nrm);
                }
        }
        Sio<FMT>::store(a.res, a.cs, i, acc);
    }
    if constexpr (EPI == 2) {
        if (a.partials) block_sum_rhs<NRHS>(a.partials, nrm);
    }
}

// One thread per (site, rhs); 4D.  EPI = 1 adds the xpay epilogue
// (res = x + coef * D psi) with one |res|^2 partial per block; EPI = 2 the
// same with one partial per block and rhs (NRHS 2..32, 128-thread blocks).
template <int FMT, int RECON, int ISIGN, int NRHS, int EPI, int LFMT = 0>
__global__ void __launch_bounds__(128, 6) dslash_gen_kernel(const GenArgs a) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int nr = nrhs_of<NRHS>(a);
    const int h = t / nr, r = t - h * nr;
    float nrm = 0.f;
    if (h < a.g.Vh) {
        Nbr n;
        neighbours<4>(a.g, h, a.pt, n);
        cx<float> acc[4][3];
#pragma unroll
        for (int s = 0; s < 4; s++)
#pragma unroll
            for (int c = 0; c < 3; c++) acc[s][c] = {0.f, 0.f};
        gen_hop_pair<FMT, RECON, ISIGN, NRHS, 0, LFMT>(a, h, r, n, acc);
        gen_hop_pair<FMT, RECON, ISIGN, NRHS, 1, LFMT>(a, h, r, n, acc);
        gen_hop_pair<FMT, RECON, ISIGN, NRHS, 2, LFMT>(a, h, r, n, acc);
        gen_hop_pair<FMT, RECON, ISIGN, NRHS, 3, LFMT>(a, h, r, n, acc);
        const size_t i = (size_t)h * nr + r;
        if constexpr (EPI) {
            cx<float> xv[4][3];
            Sio<FMT>::load(a.x, a.cs, i, xv);
#pragma unroll
            for (int s = 0; s < 4; s++)
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    acc[s][c].r = fmaf(a.coef, acc[s][c].r, xv[s][c].r);
                    acc[s][c].i = fmaf(a.coef, acc[s][c].i, xv[s][c].i);
                    nrm = fmaf(acc[s][c].r, acc[s][c].r, nrm);
                    nrm = fmaf(acc[s][c].i, acc[s][c].i, nrm);
                }
        }
        Sio<FMT>::store(a.res, a.cs, i, acc);
    }
    if constexpr (EPI == 1) {
        if (a.partials) block_sum_to<float>(a.partials, nrm);
    } else if constexpr (EPI == 2) {
        if (a.partials) block_sum_rhs<NRHS>(a.partials, nrm);
    }
}

}  // namespace gbds
