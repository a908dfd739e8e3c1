// Several right-hand sides with the SU(3) multiply on the tensor cores
// (tcgen05.mma, A in TMEM, accumulators in TMEM), 16-bit spinor storage.
//
// For one direction mu of one site, the colour multiplies of all NRHS
// right-hand sides are one real matrix product.  Row (site p, rhs r) of A
// holds, in K = 32 (bf16 or f16, four k-groups of 8), the projected half
// spinors of the neighbours: k-group 0 = forward half 0, 1 = forward half 1,
// 2 = backward half 0, 3 = backward half 1 (6 reals each, 2 zeros).  B holds,
// per site, 24 rows (the output columns of D):
//   rows 0..5   SUM  half 0:  [M_f | 0 | M_b | 0]
//   rows 6..11  SUM  half 1:  [0 | M_f | 0 | M_b]
//   rows 12..17 DIFF half 0:  [M_f | 0 | -M_b | 0]
//   rows 18..23 DIFF half 1:  [0 | M_f | 0 | -M_b]
// with M_f the real 6x6 form of U_mu(x) and M_b that of U_mu(x - mu)^dagger.
// The forward and backward projectors differ only in the sign of gamma_mu,
// so the upper spin components take the sums and the lower components
// (+-1 or +-i) times the differences.  One pair of MMAs (M = 128, N = 24 P,
// K = 2 x 16) serves both hops of a direction for P = 128 / NRHS sites; each
// row reads back only its own site's 24 columns of D.
//
// Kernel structure: persistent CTAs of 128 threads (thread t = row t) walk
// tiles of P sites, four rounds (mu = 0..3) per tile.  A round: projection
// of the neighbour spinors (loaded into registers during the round before)
// in packed 16-bit arithmetic, the A row to TMEM (tcgen05.st), the B rows of
// each site to shared memory (six link-row threads per site), the loads of
// the next round, one thread issuing the MMAs and waiting (bounded) on their
// mbarrier while the others wait at a CTA barrier, and the D rows read back
// (tcgen05.ld) and folded into the output spinor in registers (FP32).
//
// Shared-memory operand layout (B): K-major, no swizzle, core matrices of
// 8 rows x 16 bytes; element (row, k) at (row/8)*512 + (k/8)*128 +
// (row%8)*16 + (k%8)*2; descriptor leading (K) byte offset 128, stride
// (8-row) byte offset 512.  TMEM operand layout (A): lane = row, two 16-bit
// elements per 32-bit column, k ascending, even k in the low half.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>

#include "dslash_gen.cuh"

namespace gbds {
namespace {

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFF);
    d |= (uint64_t)(128 >> 4) << 16;  // K-direction core-matrix offset
    d |= (uint64_t)(512 >> 4) << 32;  // 8-row core-matrix offset
    d |= (uint64_t)1 << 46;           // descriptor version for tcgen05
    return d;
}

// Byte offset of the 16-byte core row (row, k-group kg) of the K = 32 B operand.
__device__ __forceinline__ int core_off(int row, int kg) { return (row >> 3) * 512 + kg * 128 + (row & 7) * 16; }

// Packed two-element 16-bit arithmetic (one complex number per 32 bits).
template <int FMT> struct Pk;
template <> struct Pk<kFmtBF16> {
    static constexpr uint32_t kOne = 0x3F80u;
    __device__ __forceinline__ static uint32_t fma2(uint32_t a, uint32_t b, uint32_t c) {
        const __nv_bfloat162 r = __hfma2(*reinterpret_cast<const __nv_bfloat162 *>(&a),
                                         *reinterpret_cast<const __nv_bfloat162 *>(&b),
                                         *reinterpret_cast<const __nv_bfloat162 *>(&c));
        return *reinterpret_cast<const uint32_t *>(&r);
    }
    __device__ __forceinline__ static uint32_t mul2(uint32_t a, uint32_t b) {
        const __nv_bfloat162 r = __hmul2(*reinterpret_cast<const __nv_bfloat162 *>(&a),
                                         *reinterpret_cast<const __nv_bfloat162 *>(&b));
        return *reinterpret_cast<const uint32_t *>(&r);
    }
    __device__ __forceinline__ static uint32_t pack(float a, float b) {
        const __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
        return *reinterpret_cast<const uint32_t *>(&v);
    }
};
template <> struct Pk<kFmtF16N> {
    static constexpr uint32_t kOne = 0x3C00u;
    __device__ __forceinline__ static uint32_t fma2(uint32_t a, uint32_t b, uint32_t c) {
        const __half2 r = __hfma2(*reinterpret_cast<const __half2 *>(&a), *reinterpret_cast<const __half2 *>(&b),
                                  *reinterpret_cast<const __half2 *>(&c));
        return *reinterpret_cast<const uint32_t *>(&r);
    }
    __device__ __forceinline__ static uint32_t mul2(uint32_t a, uint32_t b) {
        const __half2 r = __hmul2(*reinterpret_cast<const __half2 *>(&a), *reinterpret_cast<const __half2 *>(&b));
        return *reinterpret_cast<const uint32_t *>(&r);
    }
    __device__ __forceinline__ static uint32_t pack(float a, float b) {
        const __half2 v = __floats2half2_rn(a, b);
        return *reinterpret_cast<const uint32_t *>(&v);
    }
};

// Multiplier vector (re, im) for coefficient code 0: +1, 1: -1, 2: +i, 3: -i,
// applied to a half-swapped operand for codes 2 and 3.
template <int FMT, int CODE>
__device__ __forceinline__ constexpr uint32_t coef_vec() {
    constexpr uint32_t one = Pk<FMT>::kOne, neg = Pk<FMT>::kOne | 0x8000u;
    return CODE == 0 ? (one | (one << 16))
         : CODE == 1 ? (neg | (neg << 16))
         : CODE == 2 ? (neg | (one << 16))   // (re, im) -> (-im, re)
                     : (one | (neg << 16));  // (re, im) -> (im, -re)
}

template <int CODE>
__device__ __forceinline__ uint32_t coef_operand(uint32_t w) {
    return CODE >= 2 ? __byte_perm(w, 0, 0x1032) : w;  // swap re and im
}

// Both half spinors of one full spinor (w[3a + c] = spin a, colour c) for
// the projector (1 - SIGMA gamma_mu).
template <int FMT, int MU, int SIGMA>
__device__ __forceinline__ void project_packed(const uint4 (&q)[3], uint32_t (&h0)[3], uint32_t (&h1)[3]) {
    using P = Proj<MU>;
    constexpr int f = SIGMA > 0 ? 0 : 1;
    const uint32_t w[12] = {q[0].x, q[0].y, q[0].z, q[0].w, q[1].x, q[1].y, q[1].z, q[1].w, q[2].x, q[2].y, q[2].z, q[2].w};
    constexpr uint32_t v0 = coef_vec<FMT, P::a0 ^ f>(), v1 = coef_vec<FMT, P::a1 ^ f>();
#pragma unroll
    for (int c = 0; c < 3; c++) {
        h0[c] = Pk<FMT>::fma2(coef_operand<P::a0>(w[3 * P::j0 + c]), v0, w[c]);
        h1[c] = Pk<FMT>::fma2(coef_operand<P::a1>(w[3 * P::j1 + c]), v1, w[3 + c]);
    }
}

// n / d for 0 <= n < 2^31 by multiply-high: q = umulhi(n, m) >> s.
struct FastDiv {
    uint32_t d, m, s;
};

FastDiv make_fastdiv(uint32_t d) {
    FastDiv f{d, 0u, 0u};
    if (d <= 1) return f;
    uint32_t l = 0;
    while ((1ull << l) < d) l++;  // l = ceil(log2 d) >= 1
    // m = ceil(2^(31 + l) / d) < 2^32; error < 2^-l <= 1/d for n < 2^31
    f.m = (uint32_t)(((1ull << (31 + l)) + d - 1) / d);
    f.s = l - 1;
    return f;
}

__device__ __forceinline__ uint32_t fdiv(uint32_t n, const FastDiv &f) { return f.d <= 1 ? n : __umulhi(n, f.m) >> f.s; }

template <int NRHS>
struct TcShape {
    static constexpr int P = 128 / NRHS;                   // sites per tile
    static constexpr int N = 24 * P;                       // MMA N (D columns)
    static constexpr int ACOL = N;                         // first A column in TMEM
    static constexpr int COLS = N + 16 <= 128 ? 128 : 256;  // TMEM allocation
    static constexpr int B_BYTES = N * 64;
};

struct TcArgs {
    Geom g;
    FastDiv dx, dy, dz;  // Lx/2, Ly, Lz
    const char *psi, *gauge;
    char *res;
    size_t link_block_bytes;
    size_t cs;  // uint4 elements between the three spinor component arrays
    int pt;     // target checkerboard
    int ntiles;
    int *err;
};

// A target site and its coordinates.
struct Co {
    int h, x, y, z, t;
};

__device__ __forceinline__ Co coords(const TcArgs &a, int h) {
    Co c;
    c.h = h;
    const uint32_t r1 = fdiv((uint32_t)h, a.dx);
    const int xh = h - (int)r1 * a.g.Lxh;
    const uint32_t r2 = fdiv(r1, a.dy);
    c.y = (int)r1 - (int)r2 * a.g.L[1];
    c.t = (int)fdiv(r2, a.dz);
    c.z = (int)r2 - c.t * a.g.L[2];
    c.x = 2 * xh + ((c.y + c.z + c.t + a.pt) & 1);
    return c;
}

// Forward and backward neighbours of c in direction MU (periodic).
template <int MU>
__device__ __forceinline__ void nbr(const Geom &g, const Co &c, int &f, int &b) {
    if constexpr (MU == 0) {
        const int row = c.h - (c.x >> 1);
        const int xp = (c.x + 1 == g.L[0]) ? 0 : c.x + 1;
        const int xm = (c.x == 0) ? g.L[0] - 1 : c.x - 1;
        f = row + (xp >> 1);
        b = row + (xm >> 1);
    } else {
        const int L = g.L[MU];
        const int crd = MU == 1 ? c.y : (MU == 2 ? c.z : c.t);
        const int st = MU == 1 ? g.Lxh : (MU == 2 ? g.Lxh * g.L[1] : g.Lxh * g.L[1] * g.L[2]);
        f = (crd + 1 == L) ? c.h - (L - 1) * st : c.h + st;
        b = (crd == 0) ? c.h + (L - 1) * st : c.h - st;
    }
}

// One round's inputs of a thread, loaded a round ahead.
struct Raw {
    uint4 qf[3], qb[3];  // forward and backward neighbour spinors (rhs r)
    float nf, nb;        // their norms (half + norm format)
    float l[12];         // link data (link-row threads): recon 18 -> 3 complex, recon 12 -> rows 0 and 1
};

// Link-row thread: complex entries M[c][ci] (ci = 0..2) of M = U_mu(x)
// (dir 0) or U_mu(x - mu)^dagger (dir 1) from the loaded link data.
template <int RECON>
__device__ __forceinline__ void link_row(const float (&l)[12], int dir, int c, float (&mr)[3], float (&mi)[3]) {
    if constexpr (RECON == 18) {
        // loaded: U[c][ci] (dir 0) or U[ci][c] (dir 1)
        const float sg = dir == 0 ? 1.f : -1.f;
#pragma unroll
        for (int ci = 0; ci < 3; ci++) {
            mr[ci] = l[2 * ci];
            mi[ci] = sg * l[2 * ci + 1];
        }
    } else {
        cx<float> U[3][3];
#pragma unroll
        for (int k = 0; k < 6; k++) U[k / 3][k % 3] = {l[2 * k], l[2 * k + 1]};
        reconstruct_row2(U);
#pragma unroll
        for (int ci = 0; ci < 3; ci++) {
            // dir 0: U[c][ci]; dir 1: conj(U[ci][c])
            const cx<float> f = c == 0 ? U[0][ci] : (c == 1 ? U[1][ci] : U[2][ci]);
            const cx<float> b = c == 0 ? U[ci][0] : (c == 1 ? U[ci][1] : U[ci][2]);
            mr[ci] = dir == 0 ? f.r : b.r;
            mi[ci] = dir == 0 ? f.i : -b.i;
        }
    }
}

template <int N>
__device__ __forceinline__ void tmem_ld(uint32_t taddr, uint32_t *d);
template <>
__device__ __forceinline__ void tmem_ld<8>(uint32_t taddr, uint32_t *d) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(d[0]), "=r"(d[1]), "=r"(d[2]), "=r"(d[3]), "=r"(d[4]), "=r"(d[5]), "=r"(d[6]), "=r"(d[7])
                 : "r"(taddr));
}
template <>
__device__ __forceinline__ void tmem_ld<16>(uint32_t taddr, uint32_t *d) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                 : "=r"(d[0]), "=r"(d[1]), "=r"(d[2]), "=r"(d[3]), "=r"(d[4]), "=r"(d[5]), "=r"(d[6]), "=r"(d[7]),
                   "=r"(d[8]), "=r"(d[9]), "=r"(d[10]), "=r"(d[11]), "=r"(d[12]), "=r"(d[13]), "=r"(d[14]), "=r"(d[15])
                 : "r"(taddr));
}

template <int FMT, int RECON, int ISIGN, int NRHS>
struct TcCta {
    using S = TcShape<NRHS>;
    const TcArgs &a;
    int t, w, p, r, dir, c;
    bool item;  // link-row thread: B rows (dir, colour c) of its site
    unsigned char *B;
    const uint4 *ps;  // spinor base of rhs r

    __device__ __forceinline__ TcCta(const TcArgs &args, unsigned char *sb) : a(args), B(sb) {
        t = threadIdx.x;
        w = t >> 5;
        p = t / NRHS;
        r = t % NRHS;
        item = r < 6;
        dir = r / 3;
        c = r % 3;
        ps = reinterpret_cast<const uint4 *>(a.psi) + r;
    }

    template <int MU>
    __device__ __forceinline__ void load(const Co &co, bool act, Raw &raw) const {
        if (!act) {
#pragma unroll
            for (int k = 0; k < 3; k++) raw.qf[k] = raw.qb[k] = make_uint4(0, 0, 0, 0);
            raw.nf = raw.nb = 0.f;
#pragma unroll
            for (int k = 0; k < 12; k++) raw.l[k] = 0.f;
            return;
        }
        int f, b;
        nbr<MU>(a.g, co, f, b);
        const uint4 *pf = ps + (size_t)f * NRHS;
        const uint4 *pb = ps + (size_t)b * NRHS;
#pragma unroll
        for (int k = 0; k < 3; k++) {
            raw.qf[k] = __ldg(pf + k * a.cs);
            raw.qb[k] = __ldg(pb + k * a.cs);
        }
        if constexpr (FMT == kFmtF16N) {
            const float *nr = Sio<kFmtF16N>::norms(a.psi, a.cs) + r;
            raw.nf = __ldg(nr + (size_t)f * NRHS);
            raw.nb = __ldg(nr + (size_t)b * NRHS);
        }
        if (item) {
            const char *blk = a.gauge + (size_t)((dir == 0 ? a.pt : 1 - a.pt) * 4 + MU) * a.link_block_bytes;
            const size_t ls = (size_t)(dir == 0 ? co.h : b);
            const size_t stride = (size_t)a.g.stride;
            if constexpr (RECON == 18) {
                const float2 *pl = reinterpret_cast<const float2 *>(blk) + ls;
                const size_t step = (dir == 0 ? 1 : 3) * stride;
                const float2 *p0 = pl + (size_t)(dir == 0 ? 3 * c : c) * stride;
#pragma unroll
                for (int ci = 0; ci < 3; ci++) {
                    const float2 v = __ldg(p0 + ci * step);
                    raw.l[2 * ci] = v.x;
                    raw.l[2 * ci + 1] = v.y;
                }
            } else {
                const float4 *pl = reinterpret_cast<const float4 *>(blk) + ls;
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    const float4 v = __ldg(pl + k * stride);
                    raw.l[4 * k] = v.x;
                    raw.l[4 * k + 1] = v.y;
                    raw.l[4 * k + 2] = v.z;
                    raw.l[4 * k + 3] = v.w;
                }
            }
        }
    }

    // L1 prefetch of round MU's spinors and links (two rounds ahead of use,
    // one round ahead of the register loads, which then hit L1), for 16
    // right-hand sides.
    template <int MU>
    __device__ __forceinline__ void prefetch(const Co &co, bool act) const {
        // measured: pays off with two sites per warp (16 right-hand sides),
        // costs more issue slots than it saves with one (32)
        if constexpr (NRHS >= 32) return;
        if (!act) return;
        int f, b;
        nbr<MU>(a.g, co, f, b);
        const uint4 *pf = ps + (size_t)f * NRHS;
        const uint4 *pb = ps + (size_t)b * NRHS;
#pragma unroll
        for (int k = 0; k < 3; k++) {
            asm volatile("prefetch.global.L1 [%0];" ::"l"(pf + k * a.cs));
            asm volatile("prefetch.global.L1 [%0];" ::"l"(pb + k * a.cs));
        }
        if (item) {
            const char *blk = a.gauge + (size_t)((dir == 0 ? a.pt : 1 - a.pt) * 4 + MU) * a.link_block_bytes;
            const size_t ls = (size_t)(dir == 0 ? co.h : b);
            const size_t stride = (size_t)a.g.stride;
            if constexpr (RECON == 18) {
                const float2 *p0 = reinterpret_cast<const float2 *>(blk) + ls + (size_t)(dir == 0 ? 3 * c : c) * stride;
                const size_t step = (dir == 0 ? 1 : 3) * stride;
#pragma unroll
                for (int ci = 0; ci < 3; ci++) asm volatile("prefetch.global.L1 [%0];" ::"l"(p0 + ci * step));
            } else {
                const float4 *pl = reinterpret_cast<const float4 *>(blk) + ls;
#pragma unroll
                for (int k = 0; k < 3; k++) asm volatile("prefetch.global.L1 [%0];" ::"l"(pl + k * stride));
            }
        }
    }

    // The A row to TMEM and the B rows to shared memory; returns the D row
    // scale (half + norm).
    template <int MU>
    __device__ __forceinline__ float prep(const Raw &raw, uint32_t arow) const {
        uint32_t f0[3], f1[3], b0[3], b1[3];
        project_packed<FMT, MU, ISIGN>(raw.qf, f0, f1);   // forward hop: 1 - isign gamma_mu
        project_packed<FMT, MU, -ISIGN>(raw.qb, b0, b1);  // backward hop: 1 + isign gamma_mu
        float m = 1.f;
        if constexpr (FMT == kFmtF16N) {
            // one scale per A row: the larger of the two neighbour norms
            m = fmaxf(raw.nf, raw.nb);
            const float inv = m > 0.f ? 1.f / m : 0.f;
            const uint32_t sf = Pk<FMT>::pack(raw.nf * inv, raw.nf * inv);
            const uint32_t sb = Pk<FMT>::pack(raw.nb * inv, raw.nb * inv);
#pragma unroll
            for (int k = 0; k < 3; k++) {
                f0[k] = Pk<FMT>::mul2(f0[k], sf);
                f1[k] = Pk<FMT>::mul2(f1[k], sf);
                b0[k] = Pk<FMT>::mul2(b0[k], sb);
                b1[k] = Pk<FMT>::mul2(b1[k], sb);
            }
        }
        asm volatile(
            "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(
                arow),
            "r"(f0[0]), "r"(f0[1]), "r"(f0[2]), "r"(0u), "r"(f1[0]), "r"(f1[1]), "r"(f1[2]), "r"(0u), "r"(b0[0]),
            "r"(b0[1]), "r"(b0[2]), "r"(0u), "r"(b1[0]), "r"(b1[1]), "r"(b1[2]), "r"(0u));
        if (item) {
            float mr[3], mi[3];
            link_row<RECON>(raw.l, dir, c, mr, mi);
            const uint4 rr = make_uint4(Pk<FMT>::pack(mr[0], -mi[0]), Pk<FMT>::pack(mr[1], -mi[1]),
                                        Pk<FMT>::pack(mr[2], -mi[2]), 0u);
            const uint4 ri = make_uint4(Pk<FMT>::pack(mi[0], mr[0]), Pk<FMT>::pack(mi[1], mr[1]),
                                        Pk<FMT>::pack(mi[2], mr[2]), 0u);
            const uint32_t ng = dir == 0 ? 0u : 0x80008000u;  // the difference rows negate the backward block
            const uint4 nr = make_uint4(rr.x ^ ng, rr.y ^ ng, rr.z ^ ng, 0u);
            const uint4 ni = make_uint4(ri.x ^ ng, ri.y ^ ng, ri.z ^ ng, 0u);
            const int base = p * 24 + 2 * c;
#pragma unroll
            for (int hh = 0; hh < 2; hh++) {
                const int kg = dir * 2 + hh;
                *reinterpret_cast<uint4 *>(B + core_off(base + 6 * hh, kg)) = rr;
                *reinterpret_cast<uint4 *>(B + core_off(base + 6 * hh + 1, kg)) = ri;
                *reinterpret_cast<uint4 *>(B + core_off(base + 12 + 6 * hh, kg)) = nr;
                *reinterpret_cast<uint4 *>(B + core_off(base + 12 + 6 * hh + 1, kg)) = ni;
            }
        }
        return m;
    }

    // Fold one direction's sums and differences (24 values: sum h0, sum h1,
    // diff h0, diff h1, 3 complex each) into the output spinor.
    template <int MU>
    __device__ __forceinline__ void fold(const uint32_t (&d)[24], float m, cx<float> (&o)[4][3]) const {
        using P = Proj<MU>;
        constexpr int f = ISIGN > 0 ? 0 : 1;
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const cx<float> s0 = {__uint_as_float(d[2 * k]) * m, __uint_as_float(d[2 * k + 1]) * m};
            const cx<float> s1 = {__uint_as_float(d[6 + 2 * k]) * m, __uint_as_float(d[7 + 2 * k]) * m};
            const cx<float> d0 = {__uint_as_float(d[12 + 2 * k]) * m, __uint_as_float(d[13 + 2 * k]) * m};
            const cx<float> d1 = {__uint_as_float(d[18 + 2 * k]) * m, __uint_as_float(d[19 + 2 * k]) * m};
            o[0][k] = cadd(o[0][k], s0);
            o[1][k] = cadd(o[1][k], s1);
            o[2][k] = cadd(o[2][k], mulc<P::b2 ^ f>(P::k2 == 0 ? d0 : d1));
            o[3][k] = cadd(o[3][k], mulc<P::b3 ^ f>(P::k3 == 0 ? d0 : d1));
        }
    }

    // This row's 24 columns of D (its site's block).
    __device__ __forceinline__ void read_d(uint32_t tmem, uint32_t (&d)[24]) const {
        const uint32_t lane = (uint32_t)(32 * w) << 16;
        if constexpr (NRHS >= 32) {
            const uint32_t col = (uint32_t)(p * 24);  // one site per warp
            tmem_ld<16>(tmem + lane + col, d);
            tmem_ld<8>(tmem + lane + col + 16, d + 16);
        } else {
            // two sites per warp: read both blocks, keep this lane's
            const uint32_t col = (uint32_t)((32 * w / NRHS) * 24);
            uint32_t e[48];
            tmem_ld<16>(tmem + lane + col, e);
            tmem_ld<16>(tmem + lane + col + 16, e + 16);
            tmem_ld<16>(tmem + lane + col + 32, e + 32);
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            const bool hi = (t & 31) >= NRHS;
#pragma unroll
            for (int k = 0; k < 24; k++) d[k] = hi ? e[24 + k] : e[k];
        }
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    }
};

// Bounded wait for the phase of `parity` of an mbarrier: false if it has not
// completed after `polls` polls.
__device__ __forceinline__ bool wait_parity(uint32_t mbar, uint32_t parity, int polls = 1 << 20) {
    uint32_t done = 0;
    for (int it = 0; it < polls && !done; it++) {
        asm volatile(
            "{\n.reg .pred pw;\nmbarrier.try_wait.parity.shared::cta.b64 pw, [%1], %2;\nselp.u32 %0, 1, 0, pw;\n}"
            : "=r"(done)
            : "r"(mbar), "r"(parity)
            : "memory");
    }
    return done != 0;
}

// After a bounded wait that ran out: keep waiting for the same phase in up to
// `rounds` more bounded waits.  Returns the error code to record: 1 if the
// phase completed within them, 2 if it never did.
__device__ __forceinline__ int drain_after_timeout(uint32_t mbar, uint32_t parity, int polls, int rounds) {
    for (int r = 0; r < rounds; r++)
        if (wait_parity(mbar, parity, polls)) return 1;
    return 2;
}

template <int FMT, int RECON, int ISIGN, int NRHS>
__global__ void __launch_bounds__(128, 512 / TcShape<NRHS>::COLS) dslash_tc_kernel(const __grid_constant__ TcArgs a) {
    using S = TcShape<NRHS>;
    using Cta = TcCta<FMT, RECON, ISIGN, NRHS>;
    __shared__ __align__(128) unsigned char sB[S::B_BYTES];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tbase;
    Cta cta(a, sB);
    const int t = threadIdx.x;
    // rows and k-groups that no link-row thread writes stay zero
    for (int i = t; i < S::B_BYTES / 16; i += 128) reinterpret_cast<uint4 *>(sB)[i] = make_uint4(0, 0, 0, 0);
    if (cta.w == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tbase)),
                     "r"(S::COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (t == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&mbar)), "r"(1));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tbase;
    const uint32_t mb = smem_u32(&mbar);
    constexpr uint32_t fmt = FMT == kFmtBF16 ? 1u : 0u;
    constexpr uint32_t idesc =
        (1u << 4) | (fmt << 7) | (fmt << 10) | ((uint32_t)(S::N >> 3) << 17) | ((128u >> 4) << 24);
    const uint64_t bdesc0 = smem_desc(smem_u32(sB)), bdesc1 = smem_desc(smem_u32(sB) + 256);
    const uint32_t arow = tmem + ((uint32_t)(32 * cta.w) << 16) + S::ACOL;

    // grid-stride walk: at any time the CTAs work on one contiguous band of
    // sites, so a spinor's eight uses fall close together in time (L2 reuse)
    int tile = blockIdx.x;
    int h = tile * S::P + cta.p;
    bool act = tile < a.ntiles && h < a.g.Vh;
    Co co = coords(a, act ? h : 0);
    Raw raw;
    cta.template load<0>(co, act, raw);
    cta.template prefetch<1>(co, act);
    uint32_t phase = 0;
    bool bad = false;

    while (tile < a.ntiles) {
        const int ntile = tile + gridDim.x;
        const int nh = ntile * S::P + cta.p;
        const bool nact = ntile < a.ntiles && nh < a.g.Vh;
        Co nco = co;
        cx<float> o[4][3];
#pragma unroll
        for (int s = 0; s < 4; s++)
#pragma unroll
            for (int k = 0; k < 3; k++) o[s][k] = {0.f, 0.f};

#define GBDS_TC_ROUND(MU, NEXT_LOAD, NEXT_PREFETCH)                                                                            \
    {                                                                                                             \
        const float m = cta.template prep<MU>(raw, arow);                                                         \
        NEXT_LOAD;                                                                                                \
        NEXT_PREFETCH;                                                                                            \
        asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");                                              \
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");                                              \
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");                                          \
        __syncthreads();                                                                                          \
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");                                           \
        /* one thread issues the MMAs and waits for them; the others wait at */                                 \
        /* the barrier, which costs them no issue slots */                                                        \
        bool timed_out = false;                                                                                   \
        if (t == 0) {                                                                                             \
            asm volatile("{\n.reg .pred pd;\nsetp.ne.b32 pd, %4, 0;\n"                                            \
                         "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, pd;\n}" ::"r"(tmem),             \
                         "r"(tmem + S::ACOL), "l"(bdesc0), "r"(idesc), "r"(0));                                   \
            asm volatile("{\n.reg .pred pd;\nsetp.ne.b32 pd, %4, 0;\n"                                            \
                         "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, pd;\n}" ::"r"(tmem),             \
                         "r"(tmem + S::ACOL + 8), "l"(bdesc1), "r"(idesc), "r"(1));                               \
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mb)  \
                         : "memory");                                                                             \
            timed_out = !wait_parity(mb, phase);                                                                  \
        }                                                                                                         \
        phase ^= 1u;                                                                                              \
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");                                          \
        bad = __syncthreads_or(timed_out);                                                                        \
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");                                           \
        if (bad) break;                                                                                           \
        uint32_t d[24];                                                                                           \
        cta.read_d(tmem, d);                                                                                      \
        cta.template fold<MU>(d, m, o);                                                                           \
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");                                          \
    }

        GBDS_TC_ROUND(0, cta.template load<1>(co, act, raw), cta.template prefetch<2>(co, act))
        GBDS_TC_ROUND(1, cta.template load<2>(co, act, raw), cta.template prefetch<3>(co, act))
        GBDS_TC_ROUND(2, cta.template load<3>(co, act, raw),
                      (nco = coords(a, nact ? nh : 0), cta.template prefetch<0>(nco, nact)))
        GBDS_TC_ROUND(3, cta.template load<0>(nco, nact, raw), cta.template prefetch<1>(nco, nact))
#undef GBDS_TC_ROUND

        if (act) Sio<FMT>::store(a.res, a.cs, (size_t)h * NRHS + cta.r, o);
        tile = ntile;
        h = nh;
        act = nact;
        co = nco;
    }
    if (bad && t == 0) {
        // The MMAs whose wait ran out may still be in flight, and their
        // columns must not be freed under them.  Keep waiting, in bounded
        // rounds (16 more rounds of 2^20 polls at most), and record 2 instead
        // of 1 when they never completed.  The columns are freed in either
        // case: a CTA must release its TMEM before it exits, and columns it
        // kept would block every later tcgen05.alloc on this SM.
        atomicMax(a.err, drain_after_timeout(mb, phase ^ 1u, 1 << 20, 16));
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (cta.w == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(S::COLS));
}

template <int FMT, int RECON, int ISIGN, int NRHS>
cudaError_t launch_tc_t(TcArgs a, cudaStream_t st) {
    using S = TcShape<NRHS>;
    auto k = dslash_tc_kernel<FMT, RECON, ISIGN, NRHS>;
    // resident CTAs per SM, per device (computed once): 64K registers
    // (allocated per warp in steps of 256), 228 KB of shared memory (1 KB
    // reserved per CTA), 2048 threads, and the 512 TMEM columns
    constexpr int kMaxDev = 64;
    static std::atomic<int> resident[kMaxDev];  // SMs x CTAs per SM; 0 = not yet known
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    int slots = (dev >= 0 && dev < kMaxDev) ? resident[dev].load() : 0;
    if (slots == 0) {
        int sms = 0;
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaFuncAttributes fa;
        if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k);
        if (e != cudaSuccess) return e;
        const int regs = ((fa.numRegs * 32 + 255) / 256) * 256 * 4;
        int occ = 65536 / (regs > 0 ? regs : 1);
        const int by_smem = (228 * 1024) / ((int)fa.sharedSizeBytes + 1024);
        occ = occ < by_smem ? occ : by_smem;
        occ = occ < 16 ? occ : 16;
        occ = occ < 512 / S::COLS ? occ : 512 / S::COLS;
        occ = occ < 1 ? 1 : occ;
        slots = sms * occ;
        if (dev >= 0 && dev < kMaxDev) resident[dev].store(slots);
    }
    a.ntiles = (a.g.Vh + S::P - 1) / S::P;
    const int grid = a.ntiles < slots ? a.ntiles : slots;
    k<<<grid, 128, 0, st>>>(a);
    return cudaGetLastError();
}

// A wait that nothing completes: an mbarrier that no thread or copy arrives
// on.  The kernel's two steps after a timed-out MMA wait run on it: the
// bounded wait gives up, then the bounded drain gives up too.  flag = the code
// the Dslash kernel would record (2: the phase never completed), 0 if the
// first wait (wrongly) saw the phase complete.
__global__ void tc_wait_selftest_kernel(int polls, int *flag) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&bar)), "r"(1));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    const bool done = wait_parity(smem_u32(&bar), 0u, polls);
    const int code = done ? 0 : drain_after_timeout(smem_u32(&bar), 0u, polls, 4);
    if (threadIdx.x == 0) *flag = code;
}

}  // namespace

cudaError_t launch_tc_wait_selftest(int polls, int *flag, cudaStream_t st) {
    tc_wait_selftest_kernel<<<1, 32, 0, st>>>(polls, flag);
    return cudaGetLastError();
}

// fmt: kFmtBF16 or kFmtF16N; nrhs: 16 or 32; err: device int set to 1 if a
// wait on the tensor-core completion timed out.
cudaError_t launch_gen_tc(int fmt, const Geom &g, int recon, int nrhs, const void *gauge, const void *psi, void *res,
                          int isign, int cb, int *err, cudaStream_t st) {
    TcArgs a;
    a.g = g;
    a.dx = make_fastdiv((uint32_t)g.Lxh);
    a.dy = make_fastdiv((uint32_t)g.L[1]);
    a.dz = make_fastdiv((uint32_t)g.L[2]);
    a.psi = static_cast<const char *>(psi);
    a.res = static_cast<char *>(res);
    a.gauge = static_cast<const char *>(gauge);
    a.link_block_bytes = (size_t)recon * 4 * g.stride;
    a.cs = (size_t)g.stride * nrhs;
    a.pt = 1 - cb;
    a.ntiles = 0;
    a.err = err;
    cudaError_t e = cudaErrorInvalidValue;
#define GBDS_TC(F, R, S, N) e = launch_tc_t<F, R, S, N>(a, st)
#define GBDS_TC_N(F, R, S) do { if (nrhs == 32) GBDS_TC(F, R, S, 32); else if (nrhs == 16) GBDS_TC(F, R, S, 16); } while (0)
#define GBDS_TC_S(F, R) do { if (isign > 0) GBDS_TC_N(F, R, 1); else GBDS_TC_N(F, R, -1); } while (0)
#define GBDS_TC_R(F) do { if (recon == 18) GBDS_TC_S(F, 18); else GBDS_TC_S(F, 12); } while (0)
    if (fmt == kFmtBF16) GBDS_TC_R(kFmtBF16);
    else if (fmt == kFmtF16N) GBDS_TC_R(kFmtF16N);
#undef GBDS_TC_R
#undef GBDS_TC_S
#undef GBDS_TC_N
#undef GBDS_TC
    count_launch();
    return e;
}

}  // namespace gbds
