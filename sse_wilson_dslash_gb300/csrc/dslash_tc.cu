// Several right-hand sides with the SU(3) multiply on the tensor cores
// (tcgen05.mma, accumulators in TMEM), 16-bit spinor storage.
//
// For one hop of one site, the colour multiply of all NRHS right-hand sides
// is a real matrix product: with H the projected half spinors as rows
// (rhs r, spin half s) of 6 reals (3 colours x re/im) and U the link in its
// real 6x6 form,  W^T = H^T U^T  (rows (r, s), 6 output reals).  One
// tcgen05.mma (M = 128, K = 16, kind::f16: bf16 or f16 operands, FP32
// accumulation) takes P = 128 / (2 NRHS) sites at once: A holds the P blocks
// of 2 NRHS rows; B holds the P links side by side (N = 8 P: 6 used columns
// per site), so block (p, p) of D is site p's result and the other blocks are
// not read.  K = 16 carries the 6 used reals plus zeros.
//
// A CTA of 128 threads owns P consecutive sites; thread t is A row t:
// (site p, rhs r, spin half s).  Per round of HR hops it loads and projects
// the neighbour spinors (CUDA cores), writes its A rows, writes the links
// into B, and one thread issues HR MMAs into HR column blocks of TMEM and
// commits them to an mbarrier; after the (bounded) wait every thread reads
// its D row back with tcgen05.ld and reconstructs the four spin components
// (CUDA cores).  Spin halves s = 0, 1 of one rhs sit in adjacent lanes and
// combine their partial lower spin components with a shuffle at the end.
//
// Operand layout in shared memory: K-major, no swizzle, core matrices of
// 8 rows x 16 bytes; element (row, k) at ((row/8)*2 + k/8)*128 + (row%8)*16 +
// (k%8)*2; descriptors with leading (K) byte offset 128 and stride (8-row)
// byte offset 256.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "dslash_gen.cuh"

namespace gbds {
namespace {

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFF);
    d |= (uint64_t)(128 >> 4) << 16;  // K-direction core-matrix offset
    d |= (uint64_t)(256 >> 4) << 32;  // 8-row core-matrix offset
    d |= (uint64_t)1 << 46;           // descriptor version for tcgen05
    return d;
}

// Offset of the first 16 bytes (k = 0..7) of row r in a K-major operand.
__device__ __forceinline__ int row_off(int r) { return (r / 8) * 256 + (r % 8) * 16; }

template <int FMT>
__device__ __forceinline__ uint32_t pack2(float a, float b) {
    if constexpr (FMT == kFmtBF16) {
        const __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
        return *reinterpret_cast<const uint32_t *>(&v);
    } else {
        const __half2 v = __floats2half2_rn(a, b);
        return *reinterpret_cast<const uint32_t *>(&v);
    }
}

template <int NRHS, int HR>
struct TcShape {
    static constexpr int P = 128 / (2 * NRHS);  // sites per CTA
    static constexpr int N = 8 * P;             // MMA N
    static constexpr int COLS = HR * N;         // TMEM columns
    static constexpr int A_BYTES = 128 * 32;
    static constexpr int B_BYTES = N * 32;
    static constexpr int SMEM = HR * (A_BYTES + B_BYTES);
};

struct TcArgs {
    Geom g;
    const char *psi, *gauge;
    char *res;
    size_t link_block_bytes;
    size_t cs;
    int pt;
    int *err;
};

// Hop index 0..7 -> (mu, forward?)
template <int FMT, int RECON, int ISIGN, int NRHS, int HOP>
__device__ __forceinline__ void tc_prepare(const TcArgs &a, bool active, int h, int r, int s, int p, int j,
                                           const Nbr &n, unsigned char *A, unsigned char *B) {
    constexpr int MU = HOP / 2;
    constexpr bool FWD = (HOP % 2) == 0;
    constexpr int SIGMA = FWD ? ISIGN : -ISIGN;
    using Pj = Proj<MU>;
    constexpr int f = SIGMA > 0 ? 0 : 1;
    const int t = threadIdx.x;
    // --- A row: projected half spinor component s of the neighbour, rhs r
    uint4 row = make_uint4(0, 0, 0, 0);
    if (active) {
        const int nb = FWD ? n.f[MU] : n.b[MU];
        cx<float> sp[4][3];
        // half + norm: the normalised halves go to the tensor core and the
        // norm scales the result rows afterwards
        if constexpr (FMT == kFmtF16N) Sio<FMT>::load_raw(a.psi, a.cs, (size_t)nb * NRHS + r, sp);
        else Sio<FMT>::load(a.psi, a.cs, (size_t)nb * NRHS + r, sp);
        cx<float> hv[3];
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const cx<float> h0 = cadd(sp[0][c], mulc<Pj::a0 ^ f>(sp[Pj::j0][c]));
            const cx<float> h1 = cadd(sp[1][c], mulc<Pj::a1 ^ f>(sp[Pj::j1][c]));
            hv[c] = s == 0 ? h0 : h1;
        }
        row = make_uint4(pack2<FMT>(hv[0].r, hv[0].i), pack2<FMT>(hv[1].r, hv[1].i), pack2<FMT>(hv[2].r, hv[2].i), 0u);
    }
    *reinterpret_cast<uint4 *>(A + row_off(t)) = row;
    // --- B row j of site p: output real j = 2*c + (0 re, 1 im) over input reals k = 2*ci + (0 re, 1 im)
    if (j < 8) {
        uint4 brow = make_uint4(0, 0, 0, 0);
        if (active && j < 6) {
            cx<float> U[3][3];
            const int lh = FWD ? h : n.b[MU];
            const int lp = FWD ? a.pt : 1 - a.pt;
            Field<float>::template load_link<RECON>(a.gauge + (size_t)(lp * 4 + MU) * a.link_block_bytes, a.g.stride, lh, U);
            const int c = j / 2;
            const bool im = j & 1;
            float v[6];
#pragma unroll
            for (int ci = 0; ci < 3; ci++) {
                // M = U (forward) or U^dagger (backward); M[c][ci]
                const float mr = FWD ? U[c][ci].r : U[ci][c].r;
                const float mi = FWD ? U[c][ci].i : -U[ci][c].i;
                // re out: mr*hr - mi*hi ; im out: mi*hr + mr*hi
                v[2 * ci] = im ? mi : mr;
                v[2 * ci + 1] = im ? mr : -mi;
            }
            brow = make_uint4(pack2<FMT>(v[0], v[1]), pack2<FMT>(v[2], v[3]), pack2<FMT>(v[4], v[5]), 0u);
        }
        *reinterpret_cast<uint4 *>(B + row_off(p * 8 + j)) = brow;
    }
}

template <int ISIGN, int HOP>
__device__ __forceinline__ void tc_reconstruct(int s, const cx<float> (&w)[3], cx<float> (&up)[3], cx<float> (&l2)[3],
                                               cx<float> (&l3)[3]) {
    constexpr int MU = HOP / 2;
    constexpr bool FWD = (HOP % 2) == 0;
    constexpr int SIGMA = FWD ? ISIGN : -ISIGN;
    using Pj = Proj<MU>;
    constexpr int f = SIGMA > 0 ? 0 : 1;
    // this half spinor (index s) feeds upper component s and the lower
    // component whose source index (k2 or k3) equals s
    const bool to2 = (Pj::k2 == s);
#pragma unroll
    for (int c = 0; c < 3; c++) {
        up[c] = cadd(up[c], w[c]);
        const cx<float> c2 = mulc<Pj::b2 ^ f>(w[c]);
        const cx<float> c3 = mulc<Pj::b3 ^ f>(w[c]);
        if (to2) l2[c] = cadd(l2[c], c2);
        else l3[c] = cadd(l3[c], c3);
    }
}

template <int FMT, int RECON, int ISIGN, int NRHS, int HR>
__global__ void __launch_bounds__(128) dslash_tc_kernel(const TcArgs a) {
    using S = TcShape<NRHS, HR>;
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tbase;
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    const int p = t / (2 * NRHS), loc = t % (2 * NRHS), r = loc / 2, s = loc % 2, j = loc;
    const int h = blockIdx.x * S::P + p;
    const bool active = h < a.g.Vh;
    unsigned char *Abuf = smem;
    unsigned char *Bbuf = smem + HR * S::A_BYTES;
    // zero the operand buffers once (the k = 8..15 core matrices stay zero)
    for (int i = t; i < S::SMEM / 16; i += 128) reinterpret_cast<uint4 *>(smem)[i] = make_uint4(0, 0, 0, 0);
    if (w == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tbase)),
                     "r"(S::COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (t == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&mbar)), "r"(1));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    Nbr n;
    if (active) neighbours<4>(a.g, active ? h : 0, a.pt, n);
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = tbase;
    constexpr uint32_t idesc = (1u << 4) | ((FMT == kFmtBF16 ? 1u : 0u) << 7) | ((FMT == kFmtBF16 ? 1u : 0u) << 10) |
                               ((uint32_t)(S::N >> 3) << 17) | ((128u >> 4) << 24);
    cx<float> up[3], l2[3], l3[3];
#pragma unroll
    for (int c = 0; c < 3; c++) up[c] = l2[c] = l3[c] = {0.f, 0.f};
    float nrm_scale[8];
    bool ok = true;
#pragma unroll
    for (int round = 0; round < 8 / HR; round++) {
        // ---- operands for HR hops
#pragma unroll
        for (int q = 0; q < HR; q++) {
            const int hop = round * HR + q;
#define GBDS_PREP(H) \
    if (hop == H) tc_prepare<FMT, RECON, ISIGN, NRHS, H>(a, active, h, r, s, p, j, n, Abuf + q * S::A_BYTES, Bbuf + q * S::B_BYTES)
            GBDS_PREP(0); GBDS_PREP(1); GBDS_PREP(2); GBDS_PREP(3); GBDS_PREP(4); GBDS_PREP(5); GBDS_PREP(6); GBDS_PREP(7);
#undef GBDS_PREP
        }
        if constexpr (FMT == kFmtF16N) {
            // the tensor core multiplies normalised halves; scale D rows by the
            // neighbour spinor's norm afterwards
#pragma unroll
            for (int q = 0; q < HR; q++) {
                const int hop = round * HR + q, mu = hop / 2;
                float v = 0.f;
                if (active) {
                    const int nb = (hop % 2 == 0) ? n.f[mu] : n.b[mu];
                    v = __ldg(Sio<kFmtF16N>::norms(a.psi, a.cs) + (size_t)nb * NRHS + r);
                }
                nrm_scale[q] = v;
            }
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;");
        if (t == 0) {
#pragma unroll
            for (int q = 0; q < HR; q++) {
                const uint64_t ad = smem_desc(smem_u32(Abuf + q * S::A_BYTES));
                const uint64_t bd = smem_desc(smem_u32(Bbuf + q * S::B_BYTES));
                asm volatile("{\n.reg .pred pd;\nsetp.ne.b32 pd, %4, 0;\ntcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, pd;\n}" ::"r"(
                                 tmem + q * S::N),
                             "l"(ad), "l"(bd), "r"(idesc), "r"(0));
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(&mbar)));
        }
        // bounded wait for this round's MMAs; the whole CTA agrees on the outcome
        uint32_t done = 0;
        for (int it = 0; it < (1 << 20) && !done; it++) {
            asm volatile("{\n.reg .pred pw;\nmbarrier.try_wait.parity.shared::cta.b64 pw, [%1], %2;\nselp.u32 %0, 1, 0, pw;\n}"
                         : "=r"(done)
                         : "r"(smem_u32(&mbar)), "r"(round & 1));
        }
        if (!__syncthreads_and(done)) {
            ok = false;
            if (t == 0) atomicExch(a.err, 1);
            break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        // ---- read back and reconstruct
        const int pw = (32 * w) / (2 * NRHS);  // site block of this warp's rows
#pragma unroll
        for (int q = 0; q < HR; q++) {
            uint32_t d[8];
            const uint32_t taddr = tmem + ((uint32_t)(32 * w) << 16) + q * S::N + pw * 8;
            asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                         : "=r"(d[0]), "=r"(d[1]), "=r"(d[2]), "=r"(d[3]), "=r"(d[4]), "=r"(d[5]), "=r"(d[6]), "=r"(d[7])
                         : "r"(taddr));
            asm volatile("tcgen05.wait::ld.sync.aligned;");
            const float sc = FMT == kFmtF16N ? nrm_scale[q] : 1.f;
            cx<float> wv[3];
#pragma unroll
            for (int c = 0; c < 3; c++) wv[c] = {__uint_as_float(d[2 * c]) * sc, __uint_as_float(d[2 * c + 1]) * sc};
            const int hop = round * HR + q;
#define GBDS_REC(H) if (hop == H) tc_reconstruct<ISIGN, H>(s, wv, up, l2, l3)
            GBDS_REC(0); GBDS_REC(1); GBDS_REC(2); GBDS_REC(3); GBDS_REC(4); GBDS_REC(5); GBDS_REC(6); GBDS_REC(7);
#undef GBDS_REC
        }
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncthreads();  // everyone has read TMEM and the operands before the next round
        asm volatile("tcgen05.fence::after_thread_sync;");
    }
    // ---- combine the spin halves of each rhs and store
    if (ok) {
        cx<float> out[4][3];
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const cx<float> o_up = {__shfl_xor_sync(0xffffffffu, up[c].r, 1), __shfl_xor_sync(0xffffffffu, up[c].i, 1)};
            const cx<float> o_l2 = {__shfl_xor_sync(0xffffffffu, l2[c].r, 1), __shfl_xor_sync(0xffffffffu, l2[c].i, 1)};
            const cx<float> o_l3 = {__shfl_xor_sync(0xffffffffu, l3[c].r, 1), __shfl_xor_sync(0xffffffffu, l3[c].i, 1)};
            out[0][c] = s == 0 ? up[c] : o_up;
            out[1][c] = s == 0 ? o_up : up[c];
            out[2][c] = cadd(l2[c], o_l2);
            out[3][c] = cadd(l3[c], o_l3);
        }
        if (active && s == 0) Sio<FMT>::store(a.res, a.cs, (size_t)h * NRHS + r, out);
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (w == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(S::COLS));
}

template <int FMT, int RECON, int ISIGN, int NRHS, int HR>
cudaError_t launch_tc_t(const TcArgs &a, cudaStream_t st) {
    using S = TcShape<NRHS, HR>;
    auto k = dslash_tc_kernel<FMT, RECON, ISIGN, NRHS, HR>;
    // at most 4 CTAs per SM: 4 x S::COLS <= 512 TMEM columns
    const int smem = S::SMEM < 48 * 1024 ? 48 * 1024 : S::SMEM;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    const unsigned grid = (unsigned)((a.g.Vh + S::P - 1) / S::P);
    k<<<grid, 128, smem, st>>>(a);
    return cudaGetLastError();
}

}  // namespace

// fmt: kFmtBF16 or kFmtF16N; nrhs: 16 or 32; err: device int set to 1 if a
// wait on the tensor-core completion timed out.
cudaError_t launch_gen_tc(int fmt, const Geom &g, int recon, int nrhs, const void *gauge, const void *psi, void *res,
                          int isign, int cb, int *err, cudaStream_t st) {
    TcArgs a;
    a.g = g;
    a.psi = static_cast<const char *>(psi);
    a.res = static_cast<char *>(res);
    a.gauge = static_cast<const char *>(gauge);
    a.link_block_bytes = (size_t)recon * 4 * g.stride;
    a.cs = (size_t)g.stride * nrhs;
    a.pt = 1 - cb;
    a.err = err;
    cudaError_t e = cudaErrorInvalidValue;
#define GBDS_TC(F, R, S, N) e = launch_tc_t<F, R, S, N, (N == 32 ? 8 : 4)>(a, st)
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
