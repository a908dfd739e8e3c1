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
//   F32   6 float4 per spinor (96 B): float4 k holds complex elements 2k and
//         2k + 1 (element j = spin * 3 + colour), as the single-rhs kernel
//   F32P  6 float4 per spinor (96 B) in spin pairs: float4 c (c = 0..2)
//         holds (s0_c.r, s1_c.r, s0_c.i, s1_c.i), float4 3 + c holds
//         (s2_c.r, s3_c.r, s2_c.i, s3_c.i) -- the operand pairs of the fully
//         packed kernel
//   BF16  3 uint4 per spinor, 24 bfloat16 (48 B)
//   F16N  3 uint4 per spinor, 24 half scaled by a per-spinor float norm
//         stored after the components (48 + 4 B): value = half * norm,
//         norm = max |component|.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <type_traits>

#include "dslash_kernel.cuh"

namespace gbds {

enum SpinorFormat { kFmtNative = 0, kFmtBF16 = 1, kFmtF16N = 2, kFmtF32Pairs = 3 };

// Load/store of one spinor at element index i, component stride cs (elements).
template <int FMT> struct Sio;

template <>
struct Sio<kFmtF32Pairs> {
    static constexpr int kBytes = 96;
    __device__ __forceinline__ static void load(const char *base, size_t cs, size_t i, cx<float> (&s)[4][3]) {
        const float4 *p = reinterpret_cast<const float4 *>(base);
#pragma unroll
        for (int k = 0; k < 6; k++) {
            const float4 q = __ldg(p + k * cs + i);
            const int a = k < 3 ? 0 : 2, c = k % 3;
            s[a][c] = {q.x, q.z};
            s[a + 1][c] = {q.y, q.w};
        }
    }
    __device__ __forceinline__ static void store(char *base, size_t cs, size_t i, const cx<float> (&s)[4][3]) {
        float4 *p = reinterpret_cast<float4 *>(base);
#pragma unroll
        for (int k = 0; k < 6; k++) {
            const int a = k < 3 ? 0 : 2, c = k % 3;
            __stcs(p + k * cs + i, make_float4(s[a][c].r, s[a + 1][c].r, s[a][c].i, s[a + 1][c].i));
        }
    }
};

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

// Per-rhs scalars of the batched CG, read by the fused update epilogue.
struct RhsCgScalars {
    double rr, pAp, alpha, beta;
    int active;
    int pad;
};

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
    // fused CG update (fully packed kernel, FP32 spin pairs): instead of
    // storing v = x + coef * D psi, r -= alpha_r v for active rhs, with
    // per-(block, rhs) |r|^2 partials
    const RhsCgScalars *rsc;
    float4 *rvec;
};

// NRHS > 0: compile-time count; NRHS == 0: a.nrhs at run time.
template <int NRHS>
__device__ __forceinline__ int nrhs_of(const GenArgs &a) { return NRHS > 0 ? NRHS : a.nrhs; }

__device__ __forceinline__ void prefetch_l2(const void *p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

// Site of logical index j in the multi-RHS kernels' traversal order.  With
// g.zblock = B (a divisor of Lz below Lz) the lattice is swept in z slabs of
// B (z, t) planes with t outside z inside each slab: (x, y) fastest, then z
// within the slab, then t, then the slab.  A source spinor is then read by
// CTAs at most ~2 B planes apart (2 Lz planes in the natural order), which
// keeps its eight reads in L2 when a plane of all right-hand sides is large;
// the planes next to a slab's z faces are read from DRAM twice.  B = 0: the
// natural (cb2) order.
__device__ __forceinline__ int gen_site(const Geom &g, int j) {
    const int B = g.zblock;
    if (B <= 0 || j >= g.Vh) return j;
    const int plane = g.Lxh * g.L[1];
    const int w = j % plane;
    int q = j / plane;
    const int zz = q % B;
    q /= B;
    const int t = q % g.L[3];
    const int z = (q / g.L[3]) * B + zz;
    return (t * g.L[2] + z) * plane + w;
}

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
// a + code * b on one complex held as an (r, i) pair: one packed FP32x2
// operation for a real coefficient (+1, -1); the imaginary ones (+i, -i)
// would need b's parts swapped, so they stay scalar.
template <int CODE>
__device__ __forceinline__ cx<float> cadd_code(cx<float> a, cx<float> b) {
    if constexpr (CODE >= 2) {
        return cadd(a, mulc<CODE>(b));
    } else {
        const float2 v = CODE == 0 ? __fadd2_rn(make_float2(a.r, a.i), make_float2(b.r, b.i))
                                   : __ffma2_rn(make_float2(b.r, b.i), make_float2(-1.f, -1.f), make_float2(a.r, a.i));
        return {v.x, v.y};
    }
}

template <int MU, int SIGMA>
__device__ __forceinline__ void project_pairs(const cx<float> (&s)[4][3], cx<float> (&h)[2][3]) {
    using P = Proj<MU>;
    constexpr int f = SIGMA > 0 ? 0 : 1;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        h[0][c] = cadd_code<P::a0 ^ f>(s[0][c], s[P::j0][c]);
        h[1][c] = cadd_code<P::a1 ^ f>(s[1][c], s[P::j1][c]);
    }
}

template <int MU, int SIGMA>
__device__ __forceinline__ void reconstruct_pairs(cx<float> (&acc)[4][3], const cx<float> (&w)[2][3]) {
    using P = Proj<MU>;
    constexpr int f = SIGMA > 0 ? 0 : 1;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        acc[0][c] = cadd_code<0>(acc[0][c], w[0][c]);
        acc[1][c] = cadd_code<0>(acc[1][c], w[1][c]);
        acc[2][c] = cadd_code<P::b2 ^ f>(acc[2][c], w[P::k2][c]);
        acc[3][c] = cadd_code<P::b3 ^ f>(acc[3][c], w[P::k3][c]);
    }
}

// Variant 1's projection and reconstruction: in (r, i) pairs for 16-bit
// storage (measured faster), scalar for FP32 storage (measured slower in
// pairs; the spin-pair layout has no (r, i) pairs in its registers).
template <int FMT, int MU, int SIGMA>
__device__ __forceinline__ void g2_project(const cx<float> (&s)[4][3], cx<float> (&h)[2][3]) {
    if constexpr (FMT == kFmtNative || FMT == kFmtF32Pairs) project<MU, SIGMA>(s, h);
    else project_pairs<MU, SIGMA>(s, h);
}

template <int FMT, int MU, int SIGMA>
__device__ __forceinline__ void g2_reconstruct(cx<float> (&acc)[4][3], const cx<float> (&w)[2][3]) {
    if constexpr (FMT == kFmtNative || FMT == kFmtF32Pairs) reconstruct<MU, SIGMA>(acc, w);
    else reconstruct_pairs<MU, SIGMA>(acc, w);
}

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
    pdl_allow_next();
    pdl_wait_prev();
    constexpr int P = 128 / NRHS;  // sites per CTA
    __shared__ float4 sL[P][8][9];
    const int t = threadIdx.x;
    const int p = t / NRHS, r = t % NRHS;
    const int h = gen_site(a.g, blockIdx.x * P + p);
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
        g2_project<FMT, MU, ISIGN>(sp, hs);                                          \
        su3_mul_splat(sL[p][2 * MU], hs, w);                                         \
        g2_reconstruct<FMT, MU, ISIGN>(acc, w);                                      \
        Sio<FMT>::load(a.psi, a.cs, (size_t)n.b[MU] * NRHS + r, sp);                 \
        g2_project<FMT, MU, -ISIGN>(sp, hs);                                         \
        su3_mul_splat(sL[p][2 * MU + 1], hs, w);                                     \
        g2_reconstruct<FMT, MU, -ISIGN>(acc, w);                                     \
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

// ---------------------------------------------------------------------------
// Fully packed variant (NRHS 8..32): projection, colour multiply and
// reconstruction all run on pairs holding the same part (real or imaginary)
// of the two spin halves,
//   R_c = (h0_c.r, h1_c.r),  I_c = (h0_c.i, h1_c.i),
// one __ffma2_rn / __fadd2_rn per two reals.  The 16-bit -> FP32 conversion
// writes each value straight into its pair; FP32 storage is laid out in
// these pairs in its F32P format (only mu = 0, 1, whose projection pairs
// spin 0 with 3 and 1 with 2, take moves).
//   projection  R_c = (s0_c.r, s1_c.r) + (g0, g1) * (part of s_j0_c, s_j1_c)
//   multiply    W_R = sum_j Mr R_j - Mi I_j,   W_I = sum_j Mr I_j + Mi R_j
//   upper       (acc0, acc1) += W
//   lower       (acc2, acc3) += (b2 w0, b3 w1) for mu = 2, 3 (k2, k3 = 0, 1)
//               (acc3, acc2) += (b3 w0, b2 w1) for mu = 0, 1 (k2, k3 = 1, 0)
// The lower pairs change order once, between mu = 1 and mu = 2.  Links are
// staged in shared memory as (Mr, Mr, Mi, Mi) of M = U or U^dagger.
// ---------------------------------------------------------------------------

// Re and Im of (code * s) in terms of the parts of s: code 0 (+1): (+r, +i),
// 1 (-1): (-r, -i), 2 (+i): (-i, +r), 3 (-i): (+i, -r).
template <int CODE>
struct CPart {
    static constexpr bool swap = CODE >= 2;  // the real part comes from s.i
    static constexpr float sre = (CODE == 0 || CODE == 3) ? 1.f : -1.f;
    static constexpr float sim = (CODE == 0 || CODE == 2) ? 1.f : -1.f;
};

// the 24 reals of a stored spinor, (s[j/3][j%3].r, .i) at 2j, 2j+1; returns
// the scale (the norm of half + norm, else 1)
template <int FMT>
__device__ __forceinline__ float load_reals(const char *base, size_t cs, size_t i, float (&v)[24]) {
    if constexpr (FMT == kFmtNative) {
        // float4 k holds complex elements 2k and 2k + 1: the reals in order
        const float4 *p = reinterpret_cast<const float4 *>(base);
#pragma unroll
        for (int k = 0; k < 6; k++) {
            const float4 q = __ldg(p + k * cs + i);
            v[4 * k] = q.x;
            v[4 * k + 1] = q.y;
            v[4 * k + 2] = q.z;
            v[4 * k + 3] = q.w;
        }
        return 1.f;
    } else if constexpr (FMT == kFmtF32Pairs) {
        // the pair layout: no moves for the projection's operand pairs
        const float4 *p = reinterpret_cast<const float4 *>(base);
#pragma unroll
        for (int k = 0; k < 6; k++) {
            const float4 q = __ldg(p + k * cs + i);
            const int a = k < 3 ? 0 : 2, c = k % 3;
            v[2 * (3 * a + c)] = q.x;
            v[2 * (3 * a + c) + 1] = q.z;
            v[2 * (3 * a + 3 + c)] = q.y;
            v[2 * (3 * a + 3 + c) + 1] = q.w;
        }
        return 1.f;
    } else {
        const uint4 *p = reinterpret_cast<const uint4 *>(base);
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const uint4 q = __ldg(p + k * cs + i);
            const unsigned w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
            for (int c = 0; c < 4; c++) {
                if constexpr (FMT == kFmtBF16) {
                    v[8 * k + 2 * c] = __uint_as_float(w[c] << 16);
                    v[8 * k + 2 * c + 1] = __uint_as_float(w[c] & 0xffff0000u);
                } else {
                    const float2 f = __half22float2(*reinterpret_cast<const __half2 *>(&w[c]));
                    v[8 * k + 2 * c] = f.x;
                    v[8 * k + 2 * c + 1] = f.y;
                }
            }
        }
        if constexpr (FMT == kFmtF16N) return __ldg(Sio<kFmtF16N>::norms(base, cs) + i);
        else return 1.f;
    }
}

// One hop: project v (scaled by nrm for half + norm), multiply by the staged
// M, add into the upper pairs U and the lower pairs L (order LORD: 0 =
// (acc2, acc3), 1 = (acc3, acc2)).
template <int MU, int SIG, int LORD, bool SCALE, typename SPLAT>
__device__ __forceinline__ void packed_hop(const float (&v)[24], float nrm, const SPLAT *M, float2 (&UR)[3],
                                           float2 (&UI)[3], float2 (&LR)[3], float2 (&LI)[3]) {
    using P = Proj<MU>;
    constexpr int f = SIG > 0 ? 0 : 1;
    using A0 = CPart<P::a0 ^ f>;
    using A1 = CPart<P::a1 ^ f>;
    using B2 = CPart<P::b2 ^ f>;
    using B3 = CPart<P::b3 ^ f>;
    static_assert(A0::swap == A1::swap && B2::swap == B3::swap, "both halves take the same parts");
    static_assert(LORD == 0 ? (P::k2 == 0 && P::k3 == 1) : (P::k2 == 1 && P::k3 == 0), "lower pair order");
    float2 R[3], I[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const int s0 = 2 * c, s1 = 2 * (3 + c), j0 = 2 * (3 * P::j0 + c), j1 = 2 * (3 * P::j1 + c);
        R[c] = __ffma2_rn(make_float2(v[j0 + (A0::swap ? 1 : 0)], v[j1 + (A1::swap ? 1 : 0)]),
                          make_float2(A0::sre, A1::sre), make_float2(v[s0], v[s1]));
        I[c] = __ffma2_rn(make_float2(v[j0 + (A0::swap ? 0 : 1)], v[j1 + (A1::swap ? 0 : 1)]),
                          make_float2(A0::sim, A1::sim), make_float2(v[s0 + 1], v[s1 + 1]));
        if constexpr (SCALE) {
            R[c] = __fmul2_rn(R[c], make_float2(nrm, nrm));
            I[c] = __fmul2_rn(I[c], make_float2(nrm, nrm));
        }
    }
#pragma unroll
    for (int i = 0; i < 3; i++) {
        float2 ar = make_float2(0.f, 0.f), br = make_float2(0.f, 0.f), ai = make_float2(0.f, 0.f);
#pragma unroll
        for (int j = 0; j < 3; j++) {
            float2 mr, mi;
            if constexpr (std::is_same_v<SPLAT, float4>) {
                const float4 m = M[i * 3 + j];
                mr = make_float2(m.x, m.y);
                mi = make_float2(m.z, m.w);
            } else {
                const float2 m = M[i * 3 + j];  // (Mr, Mi): the pairs formed in registers
                mr = make_float2(m.x, m.x);
                mi = make_float2(m.y, m.y);
            }
            ar = __ffma2_rn(mr, R[j], ar);
            br = __ffma2_rn(mi, I[j], br);
            ai = __ffma2_rn(mr, I[j], ai);
            ai = __ffma2_rn(mi, R[j], ai);
        }
        const float2 wr = __ffma2_rn(br, make_float2(-1.f, -1.f), ar);
        UR[i] = __fadd2_rn(UR[i], wr);
        UI[i] = __fadd2_rn(UI[i], ai);
        using X = std::conditional_t<LORD == 0, B2, B3>;  // first element of the lower pair
        using Y = std::conditional_t<LORD == 0, B3, B2>;
        LR[i] = __ffma2_rn(B2::swap ? ai : wr, make_float2(X::sre, Y::sre), LR[i]);
        LI[i] = __ffma2_rn(B2::swap ? wr : ai, make_float2(X::sim, Y::sim), LI[i]);
    }
}

template <int FMT, int RECON, int ISIGN, int NRHS, int EPI>
__global__ void __launch_bounds__(128, 5) dslash_gen3_kernel(const GenArgs a) {
    static_assert(NRHS >= 8 && NRHS <= 32, "8 to 32 right-hand sides");
    pdl_allow_next();
    pdl_wait_prev();
    constexpr int P = 128 / NRHS;  // sites per CTA
    constexpr bool SCALE = FMT == kFmtF16N;
    __shared__ float2 sL[P][8][9];  // (Mr, Mi) splats
    const int t = threadIdx.x;
    const int p = t / NRHS, r = t % NRHS;
    const int h = gen_site(a.g, blockIdx.x * P + p);
    const bool act = h < a.g.Vh;
    if constexpr (EPI >= 2 && FMT == kFmtF32Pairs) {
        // the epilogue's operands (x, and r for the CG update) toward L2 now:
        // their loads come after the hops, at the end of the thread
        if (act) {
            const size_t i = (size_t)h * NRHS + r;
#pragma unroll
            for (int k = 0; k < 6; k++) {
                prefetch_l2(reinterpret_cast<const float4 *>(a.x) + (size_t)k * a.cs + i);
                if constexpr (EPI == 3) prefetch_l2(a.rvec + (size_t)k * a.cs + i);
            }
        }
    }
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
                sL[p][r][i * 3 + j] = make_float2(mr, mi);
            }
    }
    __syncthreads();
    float nrm = 0.f;
    if (act) {
        float2 UR[3], UI[3], LR[3], LI[3];
#pragma unroll
        for (int c = 0; c < 3; c++) UR[c] = UI[c] = LR[c] = LI[c] = make_float2(0.f, 0.f);
#define GBDS_G3_HOP(MU, LORD)                                                                            \
    {                                                                                                    \
        float v[24];                                                                                     \
        float sc = load_reals<FMT>(a.psi, a.cs, (size_t)n.f[MU] * NRHS + r, v);                          \
        packed_hop<MU, ISIGN, LORD, SCALE>(v, sc, sL[p][2 * MU], UR, UI, LR, LI);                        \
        sc = load_reals<FMT>(a.psi, a.cs, (size_t)n.b[MU] * NRHS + r, v);                                \
        packed_hop<MU, -ISIGN, LORD, SCALE>(v, sc, sL[p][2 * MU + 1], UR, UI, LR, LI);                   \
    }
        GBDS_G3_HOP(0, 1)
        GBDS_G3_HOP(1, 1)
#pragma unroll
        for (int c = 0; c < 3; c++) {
            LR[c] = make_float2(LR[c].y, LR[c].x);
            LI[c] = make_float2(LI[c].y, LI[c].x);
        }
        GBDS_G3_HOP(2, 0)
        GBDS_G3_HOP(3, 0)
#undef GBDS_G3_HOP
        cx<float> acc[4][3];
#pragma unroll
        for (int c = 0; c < 3; c++) {
            acc[0][c] = {UR[c].x, UI[c].x};
            acc[1][c] = {UR[c].y, UI[c].y};
            acc[2][c] = {LR[c].x, LI[c].x};
            acc[3][c] = {LR[c].y, LI[c].y};
        }
        const size_t i = (size_t)h * NRHS + r;
        if constexpr (EPI == 3) {
            static_assert(FMT == kFmtF32Pairs, "the fused CG update works on FP32 spin pairs");
            const RhsCgScalars &sq = a.rsc[r];
            if (sq.active) {
                cx<float> xv[4][3];
                Sio<FMT>::load(a.x, a.cs, i, xv);
                const float al = (float)sq.alpha;
#pragma unroll
                for (int k = 0; k < 6; k++) {
                    const int s0 = k < 3 ? 0 : 2, c = k % 3;
                    // v in the spin-pair component order of float4 k
                    const float4 v = make_float4(fmaf(a.coef, acc[s0][c].r, xv[s0][c].r),
                                                 fmaf(a.coef, acc[s0 + 1][c].r, xv[s0 + 1][c].r),
                                                 fmaf(a.coef, acc[s0][c].i, xv[s0][c].i),
                                                 fmaf(a.coef, acc[s0 + 1][c].i, xv[s0 + 1][c].i));
                    float4 *rp = a.rvec + (size_t)k * a.cs + i;
                    const float4 ro = *rp;
                    const float4 rn = make_float4(fmaf(-al, v.x, ro.x), fmaf(-al, v.y, ro.y), fmaf(-al, v.z, ro.z),
                                                  fmaf(-al, v.w, ro.w));
                    *rp = rn;
                    nrm += rn.x * rn.x + rn.y * rn.y + rn.z * rn.z + rn.w * rn.w;
                }
            }
        } else {
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
    }
    if constexpr (EPI >= 2) {
        if (a.partials) block_sum_rhs<NRHS>(a.partials, nrm);
    }
}

// ---------------------------------------------------------------------------
// The fully packed hop with two right-hand sides per thread (variant 3):
// rhs r and r + NRHS / 2 of one site share every staged link splat, so each
// shared-memory load of M serves two outputs (half the broadcast wavefronts
// of variant 2), and each thread has two independent chains in flight.
// ---------------------------------------------------------------------------

template <int MU, int SIG, bool SCALE>
__device__ __forceinline__ void packed_project(const float (&v)[24], float nrm, float2 (&R)[3], float2 (&I)[3]) {
    using P = Proj<MU>;
    constexpr int f = SIG > 0 ? 0 : 1;
    using A0 = CPart<P::a0 ^ f>;
    using A1 = CPart<P::a1 ^ f>;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const int s0 = 2 * c, s1 = 2 * (3 + c), j0 = 2 * (3 * P::j0 + c), j1 = 2 * (3 * P::j1 + c);
        R[c] = __ffma2_rn(make_float2(v[j0 + (A0::swap ? 1 : 0)], v[j1 + (A1::swap ? 1 : 0)]),
                          make_float2(A0::sre, A1::sre), make_float2(v[s0], v[s1]));
        I[c] = __ffma2_rn(make_float2(v[j0 + (A0::swap ? 0 : 1)], v[j1 + (A1::swap ? 0 : 1)]),
                          make_float2(A0::sim, A1::sim), make_float2(v[s0 + 1], v[s1 + 1]));
        if constexpr (SCALE) {
            R[c] = __fmul2_rn(R[c], make_float2(nrm, nrm));
            I[c] = __fmul2_rn(I[c], make_float2(nrm, nrm));
        }
    }
}

// Both rhs of a thread: multiply by the staged M (each splat loaded once) and
// add into the upper and lower pairs, as packed_hop does for one rhs.
// FOLD: the real part's chain takes -Mi I directly (one FFMA2 fewer per
// output colour; measured faster for 16-bit storage, while FP32 spin pairs
// spill with it at the 128-register cap).
// M: the staged splats of the link, (Mr, Mr, Mi, Mi) as float4 or (Mr, Mi)
// as float2 (half the shared-memory traffic; the pairs are formed in
// registers)
template <int MU, int SIG, int LORD, bool FOLD, typename SPLAT>
__device__ __forceinline__ void packed_mul_recon2(const SPLAT *M, const float2 (&R)[2][3], const float2 (&I)[2][3],
                                                  float2 (&UR)[2][3], float2 (&UI)[2][3], float2 (&LR)[2][3],
                                                  float2 (&LI)[2][3]) {
    using P = Proj<MU>;
    constexpr int f = SIG > 0 ? 0 : 1;
    using B2 = CPart<P::b2 ^ f>;
    using B3 = CPart<P::b3 ^ f>;
    static_assert(B2::swap == B3::swap, "both halves take the same parts");
    static_assert(LORD == 0 ? (P::k2 == 0 && P::k3 == 1) : (P::k2 == 1 && P::k3 == 0), "lower pair order");
    using X = std::conditional_t<LORD == 0, B2, B3>;
    using Y = std::conditional_t<LORD == 0, B3, B2>;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        float2 ar[2], br[2], ai[2];
#pragma unroll
        for (int q = 0; q < 2; q++) ar[q] = br[q] = ai[q] = make_float2(0.f, 0.f);
#pragma unroll
        for (int j = 0; j < 3; j++) {
            float2 mr, mi;
            if constexpr (std::is_same_v<SPLAT, float4>) {
                const float4 m = M[i * 3 + j];
                mr = make_float2(m.x, m.y);
                mi = make_float2(m.z, m.w);
            } else {
                const float2 m = M[i * 3 + j];
                mr = make_float2(m.x, m.x);
                mi = make_float2(m.y, m.y);
            }
#pragma unroll
            for (int q = 0; q < 2; q++) {
                ar[q] = __ffma2_rn(mr, R[q][j], ar[q]);
                if constexpr (FOLD) ar[q] = __ffma2_rn(make_float2(-mi.x, -mi.y), I[q][j], ar[q]);
                else br[q] = __ffma2_rn(mi, I[q][j], br[q]);
                ai[q] = __ffma2_rn(mr, I[q][j], ai[q]);
                ai[q] = __ffma2_rn(mi, R[q][j], ai[q]);
            }
        }
#pragma unroll
        for (int q = 0; q < 2; q++) {
            const float2 wr = FOLD ? ar[q] : __ffma2_rn(br[q], make_float2(-1.f, -1.f), ar[q]);
            UR[q][i] = __fadd2_rn(UR[q][i], wr);
            UI[q][i] = __fadd2_rn(UI[q][i], ai[q]);
            LR[q][i] = __ffma2_rn(B2::swap ? ai[q] : wr, make_float2(X::sre, Y::sre), LR[q][i]);
            LI[q][i] = __ffma2_rn(B2::swap ? wr : ai[q], make_float2(X::sim, Y::sim), LI[q][i]);
        }
    }
}

template <int FMT, int RECON, int ISIGN, int NRHS>
__global__ void __launch_bounds__(128, 4) dslash_gen4_kernel(const GenArgs a) {
    static_assert(NRHS >= 8 && NRHS <= 32, "8 to 32 right-hand sides");
    pdl_allow_next();
    pdl_wait_prev();
    constexpr int H = NRHS / 2;    // threads per site
    constexpr int P = 128 / H;     // sites per CTA
    constexpr bool SCALE = FMT == kFmtF16N;
    __shared__ float2 sL[P][8][9];  // (Mr, Mi) splats
    const int t = threadIdx.x;
    const int p = t / H, r = t % H;  // this thread: rhs r and r + H of site p
    const int h = gen_site(a.g, blockIdx.x * P + p);
    const bool act = h < a.g.Vh;
    Nbr n;
    if (act) neighbours<4>(a.g, h, a.pt, n);
    // links l = r, r + H, ... < 8 of the site (H = 4 threads a site for 8 rhs):
    // direction l / 2, forward (even l) or backward
    for (int l = r; act && l < 8; l += H) {
        const int mu = l >> 1;
        const bool bwd = l & 1;
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
                sL[p][l][i * 3 + j] = make_float2(mr, mi);
            }
    }
    __syncthreads();
    if (!act) return;
    float2 UR[2][3], UI[2][3], LR[2][3], LI[2][3];
#pragma unroll
    for (int q = 0; q < 2; q++)
#pragma unroll
        for (int c = 0; c < 3; c++) UR[q][c] = UI[q][c] = LR[q][c] = LI[q][c] = make_float2(0.f, 0.f);
#define GBDS_G4_HOP(MU, LORD, NB, SIG, L)                                                              \
    {                                                                                                  \
        float2 R[2][3], I[2][3];                                                                       \
        _Pragma("unroll") for (int q = 0; q < 2; q++) {                                               \
            float v[24];                                                                               \
            const float sc = load_reals<FMT>(a.psi, a.cs, (size_t)(NB) * NRHS + r + q * H, v);         \
            packed_project<MU, SIG, SCALE>(v, sc, R[q], I[q]);                                         \
        }                                                                                              \
        packed_mul_recon2<MU, SIG, LORD, FMT == kFmtBF16 || FMT == kFmtF16N>(sL[p][L], R, I, UR, UI, LR, LI); \
    }
#define GBDS_G4_DIR(MU, LORD)                                   \
    GBDS_G4_HOP(MU, LORD, n.f[MU], ISIGN, 2 * MU)               \
    GBDS_G4_HOP(MU, LORD, n.b[MU], -ISIGN, 2 * MU + 1)
    GBDS_G4_DIR(0, 1)
    GBDS_G4_DIR(1, 1)
#pragma unroll
    for (int q = 0; q < 2; q++)
#pragma unroll
        for (int c = 0; c < 3; c++) {
            LR[q][c] = make_float2(LR[q][c].y, LR[q][c].x);
            LI[q][c] = make_float2(LI[q][c].y, LI[q][c].x);
        }
    GBDS_G4_DIR(2, 0)
    GBDS_G4_DIR(3, 0)
#undef GBDS_G4_DIR
#undef GBDS_G4_HOP
#pragma unroll
    for (int q = 0; q < 2; q++) {
        cx<float> acc[4][3];
#pragma unroll
        for (int c = 0; c < 3; c++) {
            acc[0][c] = {UR[q][c].x, UI[q][c].x};
            acc[1][c] = {UR[q][c].y, UI[q][c].y};
            acc[2][c] = {LR[q][c].x, LI[q][c].x};
            acc[3][c] = {LR[q][c].y, LI[q][c].y};
        }
        Sio<FMT>::store(a.res, a.cs, (size_t)h * NRHS + r + q * H, acc);
    }
}

// ---------------------------------------------------------------------------
// Variant 4 (16-bit storage): variant 3 with the neighbour spinors prefetched
// two hops ahead by cp.async into a per-thread ring of three shared-memory
// slots, so that up to three hops' loads are in flight without holding
// registers (variant 3 is latency-bound at four CTAs per SM).  Slot s, rhs q,
// 16-byte chunk c of thread t at ring[((s * 2 + q) * 3 + c) * 128 + t]
// (consecutive threads, consecutive 16 bytes); the half + norm format's
// norms follow.  Every thread reads back only what it copied itself, after
// its own cp.async.wait_group, and refills a slot one hop after reading it.
// ---------------------------------------------------------------------------

__device__ __forceinline__ uint32_t smem_addr_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void cp_async_16(void *dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_4(void *dst, const void *src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_addr_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

template <int FMT, int NRHS>
struct G5Smem {
    static constexpr int P = 256 / NRHS;  // sites per 128-thread CTA (two rhs a thread)
    // ring slots (hops prefetched SLOTS - 1 ahead) and the CTAs per SM the
    // registers are capped for: two slots at 5 CTAs measured slower (BF16,
    // 32 rhs, 24^3x48: 0.455 against 0.437 ms)
    static constexpr int SLOTS = 3;
    static constexpr int MINB = 4;
    static constexpr size_t link_bytes = (size_t)P * 8 * 9 * 8;  // (Mr, Mi) float2 splats
    static constexpr size_t ring_bytes = (size_t)SLOTS * 2 * 3 * 128 * 16;
    static constexpr size_t norm_bytes = FMT == kFmtF16N ? (size_t)SLOTS * 2 * 128 * 4 : 0;
    static constexpr size_t bytes = link_bytes + ring_bytes + norm_bytes;
};

// Copy hop K's two neighbour spinors of this thread into ring slot S.
template <int FMT, int NRHS, int K, int S>
__device__ __forceinline__ void g5_issue(const GenArgs &a, const Nbr &n, int r, uint4 *ring, float *rnorm) {
    constexpr int H = NRHS / 2;
    const int nb = (K & 1) ? n.b[K >> 1] : n.f[K >> 1];
    const uint4 *src = reinterpret_cast<const uint4 *>(a.psi);
    const int t = threadIdx.x;
#pragma unroll
    for (int q = 0; q < 2; q++) {
        const size_t i = (size_t)nb * NRHS + r + q * H;
#pragma unroll
        for (int c = 0; c < 3; c++) cp_async_16(ring + ((S * 2 + q) * 3 + c) * 128 + t, src + c * a.cs + i);
        if constexpr (FMT == kFmtF16N) cp_async_4(rnorm + (S * 2 + q) * 128 + t, Sio<kFmtF16N>::norms(a.psi, a.cs) + i);
    }
}

// The 24 reals of rhs q from ring slot S (as load_reals); returns the scale.
template <int FMT, int S>
__device__ __forceinline__ float g5_read(const uint4 *ring, const float *rnorm, int q, float (&v)[24]) {
    const int t = threadIdx.x;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const uint4 w4 = ring[((S * 2 + q) * 3 + k) * 128 + t];
        const unsigned w[4] = {w4.x, w4.y, w4.z, w4.w};
#pragma unroll
        for (int c = 0; c < 4; c++) {
            if constexpr (FMT == kFmtBF16) {
                v[8 * k + 2 * c] = __uint_as_float(w[c] << 16);
                v[8 * k + 2 * c + 1] = __uint_as_float(w[c] & 0xffff0000u);
            } else {
                const float2 f = __half22float2(*reinterpret_cast<const __half2 *>(&w[c]));
                v[8 * k + 2 * c] = f.x;
                v[8 * k + 2 * c + 1] = f.y;
            }
        }
    }
    if constexpr (FMT == kFmtF16N) return rnorm[(S * 2 + q) * 128 + t];
    else return 1.f;
}

template <int FMT, int RECON, int ISIGN, int NRHS>
__global__ void __launch_bounds__(128, G5Smem<FMT, NRHS>::MINB) dslash_gen5_kernel(const GenArgs a) {
    static_assert(FMT == kFmtBF16 || FMT == kFmtF16N, "16-bit storage");
    static_assert(NRHS >= 8 && NRHS <= 32, "8 to 32 right-hand sides");
    pdl_allow_next();
    pdl_wait_prev();
    using SM = G5Smem<FMT, NRHS>;
    constexpr int H = NRHS / 2;
    constexpr int P = SM::P;
    constexpr bool SCALE = FMT == kFmtF16N;
    extern __shared__ __align__(16) unsigned char g5s[];
    float2 (*sL)[8][9] = reinterpret_cast<float2 (*)[8][9]>(g5s);
    uint4 *ring = reinterpret_cast<uint4 *>(g5s + SM::link_bytes);
    float *rnorm = reinterpret_cast<float *>(g5s + SM::link_bytes + SM::ring_bytes);
    const int t = threadIdx.x;
    const int p = t / H, r = t % H;
    const int h = gen_site(a.g, blockIdx.x * P + p);
    const bool act = h < a.g.Vh;
    Nbr n;
    if (act) neighbours<4>(a.g, h, a.pt, n);
    constexpr int NS = SM::SLOTS, DIST = NS - 1;  // hop K + DIST is issued during hop K
    // the first DIST hops in flight during the link staging
    if (act) g5_issue<FMT, NRHS, 0, 0>(a, n, r, ring, rnorm);
    cp_async_commit();
    if constexpr (DIST > 1) {
        if (act) g5_issue<FMT, NRHS, 1, 1>(a, n, r, ring, rnorm);
        cp_async_commit();
    }
    for (int l = r; act && l < 8; l += H) {
        const int mu = l >> 1;
        const bool bwd = l & 1;
        const int nbm = mu == 0 ? n.b[0] : (mu == 1 ? n.b[1] : (mu == 2 ? n.b[2] : n.b[3]));
        const int lp = bwd ? 1 - a.pt : a.pt;
        cx<float> U[3][3];
        Field<float>::template load_link<RECON>(a.gauge + (size_t)(lp * 4 + mu) * a.link_block_bytes, a.g.stride,
                                                bwd ? nbm : h, U);
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) {
                const float mr = bwd ? U[j][i].r : U[i][j].r;
                const float mi = bwd ? -U[j][i].i : U[i][j].i;
                sL[p][l][i * 3 + j] = make_float2(mr, mi);
            }
    }
    __syncthreads();
    if (!act) {
        cp_async_wait<0>();
        return;
    }
    float2 UR[2][3], UI[2][3], LR[2][3], LI[2][3];
#pragma unroll
    for (int q = 0; q < 2; q++)
#pragma unroll
        for (int c = 0; c < 3; c++) UR[q][c] = UI[q][c] = LR[q][c] = LI[q][c] = make_float2(0.f, 0.f);
    // hop K = 2 mu + (0 forward, 1 backward) from slot K % NS; then slot
    // (K + DIST) % NS, read during hop K - 1, takes hop K + DIST
#define GBDS_G5_HOP(K, MU, LORD, SIG)                                                             \
    {                                                                                             \
        cp_async_wait<DIST - 1>();                                                                \
        float2 R[2][3], I[2][3];                                                                  \
        _Pragma("unroll") for (int q = 0; q < 2; q++) {                                          \
            float v[24];                                                                          \
            const float sc = g5_read<FMT, (K) % NS>(ring, rnorm, q, v);                           \
            packed_project<MU, SIG, SCALE>(v, sc, R[q], I[q]);                                    \
        }                                                                                         \
        if constexpr ((K) + DIST < 8)                                                             \
            g5_issue<FMT, NRHS, ((K) + DIST) & 7, ((K) + DIST) % NS>(a, n, r, ring, rnorm);       \
        cp_async_commit();                                                                        \
        packed_mul_recon2<MU, SIG, LORD, true>(sL[p][K], R, I, UR, UI, LR, LI);                   \
    }
    GBDS_G5_HOP(0, 0, 1, ISIGN)
    GBDS_G5_HOP(1, 0, 1, -ISIGN)
    GBDS_G5_HOP(2, 1, 1, ISIGN)
    GBDS_G5_HOP(3, 1, 1, -ISIGN)
#pragma unroll
    for (int q = 0; q < 2; q++)
#pragma unroll
        for (int c = 0; c < 3; c++) {
            LR[q][c] = make_float2(LR[q][c].y, LR[q][c].x);
            LI[q][c] = make_float2(LI[q][c].y, LI[q][c].x);
        }
    GBDS_G5_HOP(4, 2, 0, ISIGN)
    GBDS_G5_HOP(5, 2, 0, -ISIGN)
    GBDS_G5_HOP(6, 3, 0, ISIGN)
    GBDS_G5_HOP(7, 3, 0, -ISIGN)
#undef GBDS_G5_HOP
    cp_async_wait<0>();
#pragma unroll
    for (int q = 0; q < 2; q++) {
        cx<float> acc[4][3];
#pragma unroll
        for (int c = 0; c < 3; c++) {
            acc[0][c] = {UR[q][c].x, UI[q][c].x};
            acc[1][c] = {UR[q][c].y, UI[q][c].y};
            acc[2][c] = {LR[q][c].x, LI[q][c].x};
            acc[3][c] = {LR[q][c].y, LI[q][c].y};
        }
        Sio<FMT>::store(a.res, a.cs, (size_t)h * NRHS + r + q * H, acc);
    }
}

// One thread per (site, rhs); 4D.  EPI = 1 adds the xpay epilogue
// (res = x + coef * D psi) with one |res|^2 partial per block; EPI = 2 the
// same with one partial per block and rhs (NRHS 2..32, 128-thread blocks).
template <int FMT, int RECON, int ISIGN, int NRHS, int EPI, int LFMT = 0>
__global__ void __launch_bounds__(128, 6) dslash_gen_kernel(const GenArgs a) {
    pdl_allow_next();
    pdl_wait_prev();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int nr = nrhs_of<NRHS>(a);
    const int j = t / nr, r = t - j * nr;
    const int h = gen_site(a.g, j);
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
