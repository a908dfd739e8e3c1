// Fused Wilson Dslash kernel: gather + spin projection + SU(3) multiply +
// reconstruction + accumulation over all 2*nd hops of one output site, in
// registers, in one pass.
//
// Replaces, on the device, the reference's per-site SSE kernels
// (lib/site_dslash_32bit_scalar.c:23-3098, lib/site_dslash_64bit_scalar.c:20-4926),
// its decomp / decomp_hvv / mvv_recons / recons stage kernels
// (lib/decomp_32bit_parscalar.c, lib/decomp_hvv_32bit_parscalar.c,
// lib/mvv_recons_32bit_parscalar.c, lib/recons_32bit_parscalar.c) and its
// neighbour tables (lib/shift_tables_scalar.c:191-313): neighbours are
// computed from the site index with periodic wrap-around.
#pragma once

#include <cuda_runtime.h>

#include <type_traits>

#include "dfloat.cuh"
#include "gbds_internal.h"

namespace gbds {

template <typename T>
struct cx {
    T r, i;
};

// Multiply by a coefficient in {+1, -1, +i, -i} (codes 0, 1, 2, 3).
template <int CODE, typename T>
__device__ __forceinline__ cx<T> mulc(cx<T> a) {
    if constexpr (CODE == 0) return a;
    else if constexpr (CODE == 1) return {-a.r, -a.i};
    else if constexpr (CODE == 2) return {-a.i, a.r};
    else return {a.i, -a.r};
}

template <typename T>
__device__ __forceinline__ cx<T> cadd(cx<T> a, cx<T> b) { return {a.r + b.r, a.i + b.i}; }

// Half-spinor form of (1 - sigma*gamma_mu), DeGrand-Rossi basis, sigma = +1:
//   h0 = psi0 + a0*psi[j0], h1 = psi1 + a1*psi[j1]
//   after the colour multiply w = M h:  lower spin components r2 = b2*w[k2],
//   r3 = b3*w[k3].  sigma = -1 flips every coefficient (code ^ 1).
// mu=0: h0=psi0-i psi3, h1=psi1-i psi2; r2= i w1, r3= i w0
// mu=1: h0=psi0+psi3,   h1=psi1-psi2;   r2=-w1,   r3= w0
// mu=2: h0=psi0-i psi2, h1=psi1+i psi3; r2= i w0, r3=-i w1
// mu=3: h0=psi0-psi2,   h1=psi1-psi3;   r2=-w0,   r3=-w1
template <int MU> struct Proj;
template <> struct Proj<0> { static constexpr int j0 = 3, a0 = 3, j1 = 2, a1 = 3, k2 = 1, b2 = 2, k3 = 0, b3 = 2; };
template <> struct Proj<1> { static constexpr int j0 = 3, a0 = 0, j1 = 2, a1 = 1, k2 = 1, b2 = 1, k3 = 0, b3 = 0; };
template <> struct Proj<2> { static constexpr int j0 = 2, a0 = 3, j1 = 3, a1 = 2, k2 = 0, b2 = 2, k3 = 1, b3 = 3; };
template <> struct Proj<3> { static constexpr int j0 = 2, a0 = 1, j1 = 3, a1 = 1, k2 = 0, b2 = 1, k3 = 1, b3 = 1; };

template <int MU, int SIGMA, typename T>
__device__ __forceinline__ void project(const cx<T> (&s)[4][3], cx<T> (&h)[2][3]) {
    using P = Proj<MU>;
    constexpr int f = SIGMA > 0 ? 0 : 1;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        h[0][c] = cadd(s[0][c], mulc<P::a0 ^ f>(s[P::j0][c]));
        h[1][c] = cadd(s[1][c], mulc<P::a1 ^ f>(s[P::j1][c]));
    }
}

template <int MU, int SIGMA, typename T>
__device__ __forceinline__ void reconstruct(cx<T> (&acc)[4][3], const cx<T> (&w)[2][3]) {
    using P = Proj<MU>;
    constexpr int f = SIGMA > 0 ? 0 : 1;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        acc[0][c] = cadd(acc[0][c], w[0][c]);
        acc[1][c] = cadd(acc[1][c], w[1][c]);
        acc[2][c] = cadd(acc[2][c], mulc<P::b2 ^ f>(w[P::k2][c]));
        acc[3][c] = cadd(acc[3][c], mulc<P::b3 ^ f>(w[P::k3][c]));
    }
}

// w_k = U h_k  (DAG = false) or U^dagger h_k (DAG = true), k = 0, 1.
template <bool DAG, typename T>
__device__ __forceinline__ void su3_mul(const cx<T> (&U)[3][3], const cx<T> (&h)[2][3], cx<T> (&w)[2][3]) {
#pragma unroll
    for (int k = 0; k < 2; k++) {
#pragma unroll
        for (int i = 0; i < 3; i++) {
            T re = T(0), im = T(0);
#pragma unroll
            for (int j = 0; j < 3; j++) {
                const cx<T> m = DAG ? U[j][i] : U[i][j];
                const cx<T> v = h[k][j];
                if (DAG) {
                    re = fma(m.r, v.r, re); re = fma(m.i, v.i, re);
                    im = fma(m.r, v.i, im); im = fma(-m.i, v.r, im);
                } else {
                    re = fma(m.r, v.r, re); re = fma(-m.i, v.i, re);
                    im = fma(m.r, v.i, im); im = fma(m.i, v.r, im);
                }
            }
            w[k][i] = {re, im};
        }
    }
}

// w_k += U h_k (DAG = false) or U^dagger h_k (DAG = true): the FMA chains
// start from w.
template <bool DAG, typename T>
__device__ __forceinline__ void su3_mul_acc(const cx<T> (&U)[3][3], const cx<T> (&h)[2][3], cx<T> (&w)[2][3]) {
#pragma unroll
    for (int k = 0; k < 2; k++) {
#pragma unroll
        for (int i = 0; i < 3; i++) {
            T re = w[k][i].r, im = w[k][i].i;
#pragma unroll
            for (int j = 0; j < 3; j++) {
                const cx<T> m = DAG ? U[j][i] : U[i][j];
                const cx<T> v = h[k][j];
                if (DAG) {
                    re = fma(m.r, v.r, re); re = fma(m.i, v.i, re);
                    im = fma(m.r, v.i, im); im = fma(-m.i, v.r, im);
                } else {
                    re = fma(m.r, v.r, re); re = fma(-m.i, v.i, re);
                    im = fma(m.r, v.i, im); im = fma(m.i, v.r, im);
                }
            }
            w[k][i] = {re, im};
        }
    }
}

// Third row of an SU(3) matrix from the first two: row2 = conj(row0 x row1).
template <typename T>
__device__ __forceinline__ void reconstruct_row2(cx<T> (&U)[3][3]) {
#pragma unroll
    for (int j = 0; j < 3; j++) {
        const int k = (j + 1) % 3, l = (j + 2) % 3;
        // (a x b)_j = a_k b_l - a_l b_k
        const cx<T> a = U[0][k], b = U[1][l], c = U[0][l], d = U[1][k];
        T re = a.r * b.r - a.i * b.i - (c.r * d.r - c.i * d.i);
        T im = a.r * b.i + a.i * b.r - (c.r * d.i + c.i * d.r);
        U[2][j] = {re, -im};
    }
}

// ---------------------------------------------------------------------------
// Field access (structure-of-arrays, see gbdslash.h)
// ---------------------------------------------------------------------------

template <typename T> struct Field;

// The single right-hand-side operator reads every link once per
// application: it loads them without allocating in L1 and marks their L2
// lines first for eviction, so that L2 keeps the source spinors, which are
// read by eight neighbours.
__device__ __forceinline__ uint64_t l2_evict_first_policy() {
    uint64_t pol;
    asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}
__device__ __forceinline__ float2 ld_once(const float2 *p, uint64_t pol) {
    float2 v;
    asm("ld.global.nc.L1::no_allocate.L2::cache_hint.v2.f32 {%0, %1}, [%2], %3;" : "=f"(v.x), "=f"(v.y) : "l"(p), "l"(pol));
    return v;
}
__device__ __forceinline__ float4 ld_once(const float4 *p, uint64_t pol) {
    float4 v;
    asm("ld.global.nc.L1::no_allocate.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;"
        : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
        : "l"(p), "l"(pol));
    return v;
}

template <>
struct Field<float> {
    static constexpr int SPINOR_VECS = 6;  // float4
    __device__ __forceinline__ static void load_spinor(const float4 *__restrict__ p, int stride, int h,
                                                       cx<float> (&s)[4][3]) {
        float v[24];
#pragma unroll
        for (int k = 0; k < 6; k++) {
            float4 q = __ldg(p + k * stride + h);
            v[4 * k] = q.x; v[4 * k + 1] = q.y; v[4 * k + 2] = q.z; v[4 * k + 3] = q.w;
        }
#pragma unroll
        for (int sp = 0; sp < 4; sp++)
#pragma unroll
            for (int c = 0; c < 3; c++) s[sp][c] = {v[(sp * 3 + c) * 2], v[(sp * 3 + c) * 2 + 1]};
    }
    __device__ __forceinline__ static void store_spinor(float4 *__restrict__ p, int stride, int h,
                                                        const cx<float> (&s)[4][3]) {
        float v[24];
#pragma unroll
        for (int sp = 0; sp < 4; sp++)
#pragma unroll
            for (int c = 0; c < 3; c++) { v[(sp * 3 + c) * 2] = s[sp][c].r; v[(sp * 3 + c) * 2 + 1] = s[sp][c].i; }
#pragma unroll
        for (int k = 0; k < 6; k++) __stcs(p + k * stride + h, make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]));
    }
    // Link block base: vector elements per link for a recon.
    static constexpr int link_vecs(int recon) { return recon == 18 ? 9 : 3; }
    // ONCE: the caller reads each link once per launch (the single
    // right-hand-side operator); the hints are measured to cost the kernels
    // that read a link several times (several rhs, batches).
    template <int RECON, bool ONCE = false>
    __device__ __forceinline__ static void load_link(const void *__restrict__ base, int stride, int h,
                                                     cx<float> (&U)[3][3]) {
        const uint64_t pol = ONCE ? l2_evict_first_policy() : 0;
        if constexpr (RECON == 18) {
            const float2 *p = static_cast<const float2 *>(base);
#pragma unroll
            for (int k = 0; k < 9; k++) {
                float2 q = ONCE ? ld_once(p + k * stride + h, pol) : __ldg(p + k * stride + h);
                U[k / 3][k % 3] = {q.x, q.y};
            }
        } else {
            const float4 *p = static_cast<const float4 *>(base);
#pragma unroll
            for (int k = 0; k < 3; k++) {
                float4 q = ONCE ? ld_once(p + k * stride + h, pol) : __ldg(p + k * stride + h);
                U[(2 * k) / 3][(2 * k) % 3] = {q.x, q.y};
                U[(2 * k + 1) / 3][(2 * k + 1) % 3] = {q.z, q.w};
            }
            reconstruct_row2(U);
        }
    }
};

template <>
struct Field<double> {
    static constexpr int SPINOR_VECS = 12;  // double2
    __device__ __forceinline__ static void load_spinor(const double2 *__restrict__ p, int stride, int h,
                                                       cx<double> (&s)[4][3]) {
#pragma unroll
        for (int k = 0; k < 12; k++) {
            double2 q = __ldg(p + k * stride + h);
            s[k / 3][k % 3] = {q.x, q.y};
        }
    }
    __device__ __forceinline__ static void store_spinor(double2 *__restrict__ p, int stride, int h,
                                                        const cx<double> (&s)[4][3]) {
#pragma unroll
        for (int k = 0; k < 12; k++) __stcs(p + k * stride + h, make_double2(s[k / 3][k % 3].r, s[k / 3][k % 3].i));
    }
    static constexpr int link_vecs(int recon) { return recon == 18 ? 9 : 6; }
    template <int RECON, bool ONCE = false>
    __device__ __forceinline__ static void load_link(const void *__restrict__ base, int stride, int h,
                                                     cx<double> (&U)[3][3]) {
        const double2 *p = static_cast<const double2 *>(base);
        constexpr int n = RECON == 18 ? 9 : 6;
#pragma unroll
        for (int k = 0; k < n; k++) {
            double2 q = __ldg(p + k * stride + h);
            U[k / 3][k % 3] = {q.x, q.y};
        }
        if constexpr (RECON == 12) reconstruct_row2(U);
    }
};

// Double-float (dfloat.cuh): the FP64 layout with each double2 (one complex)
// as a float4 (re.hi, re.lo, im.hi, im.lo).
template <>
struct Field<dfloat> {
    static constexpr int SPINOR_VECS = 12;  // float4
    __device__ __forceinline__ static void load_spinor(const float4 *__restrict__ p, int stride, int h,
                                                       cx<dfloat> (&s)[4][3]) {
#pragma unroll
        for (int k = 0; k < 12; k++) {
            const float4 q = __ldg(p + k * stride + h);
            s[k / 3][k % 3] = {dfloat(q.x, q.y), dfloat(q.z, q.w)};
        }
    }
    __device__ __forceinline__ static void store_spinor(float4 *__restrict__ p, int stride, int h,
                                                        const cx<dfloat> (&s)[4][3]) {
#pragma unroll
        for (int k = 0; k < 12; k++) {
            const cx<dfloat> &v = s[k / 3][k % 3];
            __stcs(p + k * stride + h, make_float4(v.r.hi, v.r.lo, v.i.hi, v.i.lo));
        }
    }
    static constexpr int link_vecs(int recon) { return recon == 18 ? 9 : 6; }
    template <int RECON, bool ONCE = false>
    __device__ __forceinline__ static void load_link(const void *__restrict__ base, int stride, int h,
                                                     cx<dfloat> (&U)[3][3]) {
        const uint64_t pol = ONCE ? l2_evict_first_policy() : 0;
        const float4 *p = static_cast<const float4 *>(base);
        constexpr int n = RECON == 18 ? 9 : 6;
#pragma unroll
        for (int k = 0; k < n; k++) {
            const float4 q = ONCE ? ld_once(p + k * stride + h, pol) : __ldg(p + k * stride + h);
            U[k / 3][k % 3] = {dfloat(q.x, q.y), dfloat(q.z, q.w)};
        }
        if constexpr (RECON == 12) reconstruct_row2(U);
    }
};

template <typename T> struct VecOf;
template <> struct VecOf<float> { using S = float4; using G = float2; static constexpr int GB = 8; };
template <> struct VecOf<double> { using S = double2; using G = double2; static constexpr int GB = 16; };
template <> struct VecOf<dfloat> { using S = float4; using G = float4; static constexpr int GB = 16; };

// FP64 and double-float: the arithmetic is the limit (FP64 issue, or FP32
// issue at ~12 instructions a double-float operation), so the hop pairs
// share their reconstruction (hop_pair_sd).
template <typename T> struct Wide : std::false_type {};
template <> struct Wide<double> : std::true_type {};
template <> struct Wide<dfloat> : std::true_type {};

// Bytes of one gauge vector element (float2 / float4 / double2) per recon.
template <typename T, int RECON>
constexpr int gauge_vec_bytes() {
    return sizeof(T) == 4 ? (RECON == 18 ? 8 : 16) : 16;
}

// ---------------------------------------------------------------------------
// Neighbour indexing (periodic), internal site order of gbdslash.h
// ---------------------------------------------------------------------------

struct Nbr {
    int f[4], b[4];  // source-checkerboard index of x+mu / x-mu
};

template <int ND>
__device__ __forceinline__ void neighbours(const Geom &g, int h, int pt, Nbr &n) {
    const int Lxh = g.Lxh;
    if constexpr (ND == 4) {
        int r = h;
        const int xh = r % Lxh; r /= Lxh;
        const int y = r % g.L[1]; r /= g.L[1];
        const int z = r % g.L[2];
        const int t = r / g.L[2];
        const int x = 2 * xh + ((y + z + t + pt) & 1);
        const int row = h - xh;
        const int xp = (x + 1 == g.L[0]) ? 0 : x + 1;
        const int xm = (x == 0) ? g.L[0] - 1 : x - 1;
        n.f[0] = row + (xp >> 1);
        n.b[0] = row + (xm >> 1);
        const int sy = Lxh, sz = Lxh * g.L[1], st = sz * g.L[2];
        n.f[1] = (y + 1 == g.L[1]) ? h - (g.L[1] - 1) * sy : h + sy;
        n.b[1] = (y == 0) ? h + (g.L[1] - 1) * sy : h - sy;
        n.f[2] = (z + 1 == g.L[2]) ? h - (g.L[2] - 1) * sz : h + sz;
        n.b[2] = (z == 0) ? h + (g.L[2] - 1) * sz : h - sz;
        n.f[3] = (t + 1 == g.L[3]) ? h - (g.L[3] - 1) * st : h + st;
        n.b[3] = (t == 0) ? h + (g.L[3] - 1) * st : h - st;
    } else {
        const int Lt = g.L[3];
        int r = h / Lt;
        const int xh = r % Lxh; r /= Lxh;
        const int y = r % g.L[1];
        const int z = r / g.L[1];
        const int x = 2 * xh + ((y + z + pt) & 1);
        const int row = h - xh * Lt;
        const int xp = (x + 1 == g.L[0]) ? 0 : x + 1;
        const int xm = (x == 0) ? g.L[0] - 1 : x - 1;
        n.f[0] = row + (xp >> 1) * Lt;
        n.b[0] = row + (xm >> 1) * Lt;
        const int sy = Lt * Lxh, sz = sy * g.L[1];
        n.f[1] = (y + 1 == g.L[1]) ? h - (g.L[1] - 1) * sy : h + sy;
        n.b[1] = (y == 0) ? h + (g.L[1] - 1) * sy : h - sy;
        n.f[2] = (z + 1 == g.L[2]) ? h - (g.L[2] - 1) * sz : h + sz;
        n.b[2] = (z == 0) ? h + (g.L[2] - 1) * sz : h - sz;
        n.f[3] = n.b[3] = h;
    }
}

// ---------------------------------------------------------------------------
// The kernel
// ---------------------------------------------------------------------------

template <typename T>
struct DslashArgs {
    Geom g;
    const typename VecOf<T>::S *psi;  // source checkerboard (cb)
    typename VecOf<T>::S *res;        // target checkerboard (1-cb)
    const char *gauge;                // both checkerboards
    size_t link_block_bytes;          // bytes of one (parity, mu) block
    int pt;                           // target parity = 1 - cb
};

template <typename T, int ND, int RECON, int ISIGN, int MU>
__device__ __forceinline__ void hop_pair(const DslashArgs<T> &a, int h, const Nbr &n, cx<T> (&acc)[4][3]) {
    using F = Field<T>;
    const int ps = 1 - a.pt;
    cx<T> s[4][3], hs[2][3], w[2][3], U[3][3];
    // forward: U_mu(x) (1 - isign gamma_mu) psi(x + mu)
    F::load_spinor(a.psi, a.g.stride, n.f[MU], s);
    F::template load_link<RECON, true>(a.gauge + (size_t)(a.pt * ND + MU) * a.link_block_bytes, a.g.stride, h, U);
    project<MU, ISIGN>(s, hs);
    su3_mul<false>(U, hs, w);
    reconstruct<MU, ISIGN>(acc, w);
    // backward: U_mu(x - mu)^dagger (1 + isign gamma_mu) psi(x - mu)
    F::load_spinor(a.psi, a.g.stride, n.b[MU], s);
    F::template load_link<RECON, true>(a.gauge + (size_t)(ps * ND + MU) * a.link_block_bytes, a.g.stride, n.b[MU], U);
    project<MU, -ISIGN>(s, hs);
    su3_mul<true>(U, hs, w);
    reconstruct<MU, -ISIGN>(acc, w);
}

// FP64 and double-float (issue-bound): the backward coefficients of the
// lower spin components are the forward ones negated, so with S = w_f + w_b
// (the backward product's FMA chains start from w_f) and D = w_f - w_b =
// 2 w_f - S the hop pair adds S to the upper and c D to the lower
// components: 12 fewer operations per direction than two separate
// reconstructions.
template <typename T, int ND, int RECON, int ISIGN, int MU>
__device__ __forceinline__ void hop_pair_sd(const DslashArgs<T> &a, int h, const Nbr &n, cx<T> (&acc)[4][3]) {
    using F = Field<T>;
    using P = Proj<MU>;
    constexpr int f = ISIGN > 0 ? 0 : 1;  // the forward hop's sign flip
    const int ps = 1 - a.pt;
    cx<T> s[4][3], hs[2][3], w[2][3], U[3][3];
    F::load_spinor(a.psi, a.g.stride, n.f[MU], s);
    F::template load_link<RECON, true>(a.gauge + (size_t)(a.pt * ND + MU) * a.link_block_bytes, a.g.stride, h, U);
    project<MU, ISIGN>(s, hs);
    su3_mul<false>(U, hs, w);
    cx<T> wf[2][3];
#pragma unroll
    for (int k = 0; k < 2; k++)
#pragma unroll
        for (int c = 0; c < 3; c++) wf[k][c] = w[k][c];
    F::load_spinor(a.psi, a.g.stride, n.b[MU], s);
    F::template load_link<RECON, true>(a.gauge + (size_t)(ps * ND + MU) * a.link_block_bytes, a.g.stride, n.b[MU], U);
    project<MU, -ISIGN>(s, hs);
    su3_mul_acc<true>(U, hs, w);  // w = S
#pragma unroll
    for (int c = 0; c < 3; c++) {
        cx<T> d[2];
#pragma unroll
        for (int k = 0; k < 2; k++) d[k] = {fma(T(2), wf[k][c].r, -w[k][c].r), fma(T(2), wf[k][c].i, -w[k][c].i)};
        acc[0][c] = cadd(acc[0][c], w[0][c]);
        acc[1][c] = cadd(acc[1][c], w[1][c]);
        acc[2][c] = cadd(acc[2][c], mulc<P::b2 ^ f>(d[P::k2]));
        acc[3][c] = cadd(acc[3][c], mulc<P::b3 ^ f>(d[P::k3]));
    }
}

template <typename T, int ND, int RECON, int ISIGN, int MU>
__device__ __forceinline__ void hop_pair_any(const DslashArgs<T> &a, int h, const Nbr &n, cx<T> (&acc)[4][3]) {
    if constexpr (Wide<T>::value) hop_pair_sd<T, ND, RECON, ISIGN, MU>(a, h, n, acc);
    else hop_pair<T, ND, RECON, ISIGN, MU>(a, h, n, acc);
}

// MINB > 0 caps registers so that MINB blocks of 128 threads fit on an SM
// (launch with 128 threads); MINB == 0 leaves registers uncapped (<= 256 threads).
template <int MINB> struct Bounds { static constexpr int threads = 128, blocks = MINB; };
template <> struct Bounds<0> { static constexpr int threads = 256, blocks = 1; };

// Programmatic dependent launch: the next kernel launched on the stream with
// the programmatic-serialisation attribute may start its blocks once every
// block of this grid has started; it waits (griddepcontrol.wait) for this
// grid's completion and memory before its first global read.  Without the
// attribute both instructions are no-ops.
__device__ __forceinline__ void pdl_allow_next() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait_prev() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <typename T, int ND, int RECON, int ISIGN, int MINB>
__global__ void __launch_bounds__(Bounds<MINB>::threads, Bounds<MINB>::blocks) dslash_kernel(const DslashArgs<T> a) {
    pdl_allow_next();
    const int h = blockIdx.x * blockDim.x + threadIdx.x;
    Nbr n;
    if (h < a.g.Vh) neighbours<ND>(a.g, h, a.pt, n);  // index arithmetic only: overlaps the previous grid
    pdl_wait_prev();
    if (h >= a.g.Vh) return;
    cx<T> acc[4][3];
#pragma unroll
    for (int s = 0; s < 4; s++)
#pragma unroll
        for (int c = 0; c < 3; c++) acc[s][c] = {T(0), T(0)};
    hop_pair_any<T, ND, RECON, ISIGN, 0>(a, h, n, acc);
    hop_pair_any<T, ND, RECON, ISIGN, 1>(a, h, n, acc);
    hop_pair_any<T, ND, RECON, ISIGN, 2>(a, h, n, acc);
    if constexpr (ND == 4) hop_pair_any<T, ND, RECON, ISIGN, 3>(a, h, n, acc);
    Field<T>::store_spinor(a.res, a.g.stride, h, acc);
}

// Register-cap variants: index -> MINB (see Bounds).  FP32 and FP64 differ.
template <typename T> struct Variants;
template <> struct Variants<float> { static constexpr int n = 5; static constexpr int minb[5] = {0, 6, 7, 8, 10}; };
template <> struct Variants<double> { static constexpr int n = 3; static constexpr int minb[3] = {0, 3, 4}; };
// double-float at 32^3x64: 1.28 ms uncapped, 0.86 ms at 3 and 0.74 ms at 4
// CTAs of 128 threads per SM; 5 and 6 spill 1.2-1.9 KB and lose
template <> struct Variants<dfloat> { static constexpr int n = 3; static constexpr int minb[3] = {0, 3, 4}; };

// Launch with the programmatic-serialisation attribute (see pdl_wait_prev).
template <typename... P, typename... A>
void launch_pdl_smem(void (*kernel)(P...), dim3 grid, int block, size_t smem, cudaStream_t stream, const A &...args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    // a failed launch also sets the runtime's last error, which every
    // launcher returns through cudaGetLastError()
    (void)cudaLaunchKernelEx(&cfg, kernel, args...);
}

template <typename... P, typename... A>
void launch_pdl(void (*kernel)(P...), dim3 grid, int block, cudaStream_t stream, const A &...args) {
    launch_pdl_smem(kernel, grid, block, 0, stream, args...);
}

template <typename T, int MINB>
void launch_variant(const DslashArgs<T> &a, dim3 grid, int block, int nd, int recon, int isign, cudaStream_t stream) {
#define GBDS_LAUNCH(ND, R, S) launch_pdl(dslash_kernel<T, ND, R, S, MINB>, grid, block, stream, a)
    if (nd == 4) {
        if (recon == 18) { if (isign > 0) GBDS_LAUNCH(4, 18, 1); else GBDS_LAUNCH(4, 18, -1); }
        else             { if (isign > 0) GBDS_LAUNCH(4, 12, 1); else GBDS_LAUNCH(4, 12, -1); }
    } else {
        if (recon == 18) { if (isign > 0) GBDS_LAUNCH(3, 18, 1); else GBDS_LAUNCH(3, 18, -1); }
        else             { if (isign > 0) GBDS_LAUNCH(3, 12, 1); else GBDS_LAUNCH(3, 12, -1); }
    }
#undef GBDS_LAUNCH
}

// ---------------------------------------------------------------------------
// Dslash with an xpay epilogue and a norm reduction, for the even-odd
// operator M = 1 - kappa^2 D_eo D_oe:  out = x + coef * Dslash(psi), and
// partials[block] = sum over the block's sites of |out|^2 (for the CG's
// <p, M^+M p> = |M p|^2).  4D only.
// ---------------------------------------------------------------------------

template <typename T>
__device__ __forceinline__ void load_spinor_any(const typename VecOf<T>::S *p, int stride, int h, cx<T> (&s)[4][3]) {
    Field<T>::load_spinor(p, stride, h, s);
}

// Sum a per-thread float/double over the block into partials[blockIdx.x] (double).
template <typename T>
__device__ __forceinline__ void block_sum_to(double *partials, T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    __shared__ double warp_sums[32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) warp_sums[w] = (double)v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        const int nw = (blockDim.x + 31) >> 5;
        for (int i = 0; i < nw; i++) t += warp_sums[i];
        partials[blockIdx.x] = t;
    }
}

// double-float: the per-thread sum goes in as one double
__device__ __forceinline__ void block_sum_to(double *partials, dfloat v) {
    block_sum_to<double>(partials, (double)v.hi + (double)v.lo);
}

template <typename T, int RECON, int ISIGN, int MINB>
__global__ void __launch_bounds__(Bounds<MINB>::threads, Bounds<MINB>::blocks)
    dslash_xpay_kernel(const DslashArgs<T> a, const typename VecOf<T>::S *__restrict__ x, T coef, double *partials) {
    pdl_allow_next();
    pdl_wait_prev();
    const int h = blockIdx.x * blockDim.x + threadIdx.x;
    T nrm = T(0);
    if (h < a.g.Vh) {
        Nbr n;
        neighbours<4>(a.g, h, a.pt, n);
        cx<T> acc[4][3];
#pragma unroll
        for (int s = 0; s < 4; s++)
#pragma unroll
            for (int c = 0; c < 3; c++) acc[s][c] = {T(0), T(0)};
        hop_pair_any<T, 4, RECON, ISIGN, 0>(a, h, n, acc);
        hop_pair_any<T, 4, RECON, ISIGN, 1>(a, h, n, acc);
        hop_pair_any<T, 4, RECON, ISIGN, 2>(a, h, n, acc);
        hop_pair_any<T, 4, RECON, ISIGN, 3>(a, h, n, acc);
        cx<T> xv[4][3];
        load_spinor_any<T>(x, a.g.stride, h, xv);
#pragma unroll
        for (int s = 0; s < 4; s++)
#pragma unroll
            for (int c = 0; c < 3; c++) {
                acc[s][c].r = fma(coef, acc[s][c].r, xv[s][c].r);
                acc[s][c].i = fma(coef, acc[s][c].i, xv[s][c].i);
                nrm = fma(acc[s][c].r, acc[s][c].r, nrm);
                nrm = fma(acc[s][c].i, acc[s][c].i, nrm);
            }
        Field<T>::store_spinor(a.res, a.g.stride, h, acc);
    }
    if (partials) {
        if constexpr (std::is_same_v<T, dfloat>) block_sum_to(partials, nrm);
        else block_sum_to<T>(partials, nrm);
    }
}

template <typename T> struct XpayMinb;
template <> struct XpayMinb<float> { static constexpr int r18 = 6, r12 = 6; };
template <> struct XpayMinb<double> { static constexpr int r18 = 0, r12 = 0; };
template <> struct XpayMinb<dfloat> { static constexpr int r18 = 4, r12 = 4; };

// Grid blocks of an xpay launch (the size `partials` must have).
inline int xpay_blocks(const Geom &g) { return (g.Vh + 127) / 128; }

template <typename T>
cudaError_t launch_dslash_xpay_t(const Geom &g, int recon, const void *gauge, const void *psi, const void *x, T coef,
                                 void *res, double *partials, int isign, int cb, cudaStream_t stream) {
    DslashArgs<T> a;
    a.g = g;
    a.psi = static_cast<const typename VecOf<T>::S *>(psi);
    a.res = static_cast<typename VecOf<T>::S *>(res);
    a.gauge = static_cast<const char *>(gauge);
    const int vec_bytes = sizeof(T) == 4 ? (recon == 18 ? 8 : 16) : 16;
    a.link_block_bytes = (size_t)Field<T>::link_vecs(recon) * g.stride * vec_bytes;
    a.pt = 1 - cb;
    const dim3 grid(xpay_blocks(g));
    const auto *xv = static_cast<const typename VecOf<T>::S *>(x);
    constexpr int m18 = XpayMinb<T>::r18, m12 = XpayMinb<T>::r12;
    if (recon == 18) {
        if (isign > 0) launch_pdl(dslash_xpay_kernel<T, 18, 1, m18>, grid, 128, stream, a, xv, coef, partials);
        else launch_pdl(dslash_xpay_kernel<T, 18, -1, m18>, grid, 128, stream, a, xv, coef, partials);
    } else {
        if (isign > 0) launch_pdl(dslash_xpay_kernel<T, 12, 1, m12>, grid, 128, stream, a, xv, coef, partials);
        else launch_pdl(dslash_xpay_kernel<T, 12, -1, m12>, grid, 128, stream, a, xv, coef, partials);
    }
    count_launch();
    return cudaGetLastError();
}

// Variant I of Variants<T> (a template, so that the variant kernels are
// instantiated only in the translation units that launch them, and only
// those the list names).
template <typename T, int I = 0>
void launch_variant_index(const DslashArgs<T> &a, dim3 grid, int block, int nd, int recon, int isign, int variant,
                          cudaStream_t s) {
    if constexpr (I < Variants<T>::n) {
        if (variant == I) launch_variant<T, Variants<T>::minb[I]>(a, grid, block, nd, recon, isign, s);
        else launch_variant_index<T, I + 1>(a, grid, block, nd, recon, isign, variant, s);
    }
}

template <typename T>
cudaError_t launch_dslash_t(const Geom &g, int recon, const void *gauge, const void *psi, void *res,
                            int isign, int cb, int block, int variant, cudaStream_t stream) {
    DslashArgs<T> a;
    a.g = g;
    a.psi = static_cast<const typename VecOf<T>::S *>(psi);
    a.res = static_cast<typename VecOf<T>::S *>(res);
    a.gauge = static_cast<const char *>(gauge);
    const int vec_bytes = sizeof(T) == 4 ? (recon == 18 ? 8 : 16) : 16;
    a.link_block_bytes = (size_t)Field<T>::link_vecs(recon) * g.stride * vec_bytes;
    a.pt = 1 - cb;
    if (variant < 0 || variant >= Variants<T>::n) variant = 0;
    if (block <= 0) block = 128;
    if (Variants<T>::minb[variant] > 0) block = 128;  // the register cap assumes 128-thread blocks
    const dim3 grid((g.Vh + block - 1) / block);
    launch_variant_index<T>(a, grid, block, g.nd, recon, isign, variant, stream);
    count_launch();
    return cudaGetLastError();
}

}  // namespace gbds
