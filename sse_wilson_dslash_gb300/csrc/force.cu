// Gradient of L = Re <chi, Dslash(isign) psi> with respect to the links.
//
// psi lives on checkerboard cb, chi on 1-cb (pt = 1-cb).  Every link of the
// lattice enters L exactly once:
//   links at sites x of checkerboard pt, forward hop:  chi(x)^+ U_mu(x) P- psi(x+mu)
//     -> G = sum_s chi_s(x) (x) conj(phi_s),   phi = (1 - isign g_mu) psi(x+mu)
//   links at sites x of checkerboard cb, backward hop to y = x+mu:
//        chi(y)^+ U_mu(x)^+ P+ psi(x)
//     -> G = sum_s phi'_s (x) conj(chi_s(y)),  phi' = (1 + isign g_mu) psi(x)
// G is the complex gradient (dL/dRe U + i dL/dIm U).  The lower spin
// components of phi are multiples of the upper ones, so each G is two colour
// outer products of half spinors after folding chi onto two components.
// mode 0 writes G; mode 1 writes the su(3) force F = TA(G U^+)
// (traceless anti-Hermitian part), the derivative along U -> exp(eps X) U:
//   dL/deps = Re tr(F^+ X) for X in su(3).
// The neighbour projections are recomputed here, not stored by the forward
// operator.  Output: the packed gauge layout, f[s][mu][j][i] = F_ij.
#include <cuda_runtime.h>

#include <cstdint>

#include "dslash_kernel.cuh"

namespace gbds {
namespace {

template <typename T> struct Cplx { T r, i; };

// xi_k = chi_k + sum over the lower components s that reconstruct from
// upper component k of conj(coefficient) * chi_s  (projector (1 - SIGMA g_mu)).
template <int MU, int SIGMA, typename T>
__device__ __forceinline__ void fold(const cx<T> (&chi)[4][3], cx<T> (&xi)[2][3]) {
    using P = Proj<MU>;
    constexpr int f = SIGMA > 0 ? 0 : 1;
    constexpr int c2 = P::b2 ^ f, c3 = P::b3 ^ f;
    // conjugate coefficient codes: +-1 unchanged, +-i swapped
    constexpr int cc2 = c2 >= 2 ? (c2 ^ 1) : c2, cc3 = c3 >= 2 ? (c3 ^ 1) : c3;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        xi[0][c] = chi[0][c];
        xi[1][c] = chi[1][c];
        if constexpr (P::k2 == 0) xi[0][c] = cadd(xi[0][c], mulc<cc2>(chi[2][c]));
        else xi[1][c] = cadd(xi[1][c], mulc<cc2>(chi[2][c]));
        if constexpr (P::k3 == 0) xi[0][c] = cadd(xi[0][c], mulc<cc3>(chi[3][c]));
        else xi[1][c] = cadd(xi[1][c], mulc<cc3>(chi[3][c]));
    }
}

// G += a (x) conj(b) for colour vectors a, b
template <typename T>
__device__ __forceinline__ void outer_acc(cx<T> (&G)[3][3], const cx<T> (&a)[3], const cx<T> (&b)[3]) {
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) {
            G[i][j].r += a[i].r * b[j].r + a[i].i * b[j].i;
            G[i][j].i += a[i].i * b[j].r - a[i].r * b[j].i;
        }
}

// F = TA(M), M = G U^+ with G = sum_s a_s (x) conj(b_s): M = sum_s a_s (x)
// conj(U b_s), so two SU(3) matrix-vector products and two outer products
// (144 real FMA) instead of G and then G U^+ (180): the FP64 kernel, which
// is FP64-issue bound (16^4: 0.219 -> 0.165 ms).
template <typename T>
__device__ __forceinline__ void traceless_antihermitian_of_GUdag(const cx<T> (&a)[2][3], const cx<T> (&b)[2][3],
                                                                 const cx<T> (&U)[3][3], cx<T> (&F)[3][3]) {
    cx<T> c[2][3];  // c_s = U b_s
#pragma unroll
    for (int s = 0; s < 2; s++)
#pragma unroll
        for (int j = 0; j < 3; j++) {
            T re = 0, im = 0;
#pragma unroll
            for (int k = 0; k < 3; k++) {
                re = fma(U[j][k].r, b[s][k].r, re);
                re = fma(-U[j][k].i, b[s][k].i, re);
                im = fma(U[j][k].r, b[s][k].i, im);
                im = fma(U[j][k].i, b[s][k].r, im);
            }
            c[s][j] = {re, im};
        }
    cx<T> M[3][3];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) M[i][j] = {T(0), T(0)};
    outer_acc(M, a[0], c[0]);
    outer_acc(M, a[1], c[1]);
    const T tr_im = (M[0][0].i + M[1][1].i + M[2][2].i) / T(3);
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) {
            // (M - M^+)/2
            F[i][j] = {(M[i][j].r - M[j][i].r) / T(2), (M[i][j].i + M[j][i].i) / T(2)};
        }
#pragma unroll
    for (int i = 0; i < 3; i++) F[i][i].i -= tr_im;
}

// F = TA(G U^+) from G itself (the FP32 kernel, memory- and latency-bound,
// measured faster in this form)
template <typename T>
__device__ __forceinline__ void traceless_antihermitian_of_GUdag(const cx<T> (&G)[3][3], const cx<T> (&U)[3][3],
                                                                 cx<T> (&F)[3][3]) {
    cx<T> M[3][3];  // M = G U^+
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) {
            T re = 0, im = 0;
#pragma unroll
            for (int k = 0; k < 3; k++) {  // G_ik conj(U_jk)
                re += G[i][k].r * U[j][k].r + G[i][k].i * U[j][k].i;
                im += G[i][k].i * U[j][k].r - G[i][k].r * U[j][k].i;
            }
            M[i][j] = {re, im};
        }
    const T tr_im = (M[0][0].i + M[1][1].i + M[2][2].i) / T(3);
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) F[i][j] = {(M[i][j].r - M[j][i].r) / T(2), (M[i][j].i + M[j][i].i) / T(2)};
#pragma unroll
    for (int i = 0; i < 3; i++) F[i][i].i -= tr_im;
}

struct ForceArgs {
    Geom g;
    const char *gauge;        // internal, both checkerboards
    size_t link_block_bytes;
    const void *psi;          // internal, checkerboard cb
    const void *chi;          // internal, checkerboard pt
    const int *table;         // caller layout (nullptr: canonical)
    void *out;                // packed [V][4][3][3][2]
    int pt;                   // target checkerboard (chi's)
    int mode;                 // 0: G, 1: TA(G U^+)
    double coef;
    int accumulate;
};

// Sites per CTA: 128 in FP32, 64 in FP64, so that the staged output of a CTA
// (2 links x 18 reals per site at a time) is 18 KB of shared memory either
// way; FP32 caps registers for 7 CTAs per SM.
template <typename T> struct ForceTile {
    static constexpr int sites = sizeof(T) == 4 ? 128 : 64;
    static constexpr int min_blocks = sizeof(T) == 4 ? 7 : 1;
};

// R = G (mode 0) or TA(G U^+) (mode 1) of link (p, h, MU), times coef, into
// o[(3j+i)*2 + 0/1] = R_ij: the packed transposed order of the output.
template <typename T, int ISIGN, int MU>
__device__ __forceinline__ void force_link(const ForceArgs &a, int p, int h, const Nbr &n, const cx<T> (&own)[4][3],
                                           T *o) {
    using F = Field<T>;
    using V = typename VecOf<T>::S;
    // G = sum_s ga_s (x) conj(gb_s)
    cx<T> s[4][3], ga[2][3], gb[2][3];
    if (p == a.pt) {
        // forward hop at x: xi from chi(x) (own), half spinor of psi(x + mu)
        fold<MU, ISIGN>(own, ga);
        F::load_spinor(static_cast<const V *>(a.psi), a.g.stride, n.f[MU], s);
        project<MU, ISIGN>(s, gb);
    } else {
        // backward hop into y = x + mu: half spinor of psi(x) (own), xi from chi(y)
        project<MU, -ISIGN>(own, ga);
        F::load_spinor(static_cast<const V *>(a.chi), a.g.stride, n.f[MU], s);
        fold<MU, -ISIGN>(s, gb);
    }
    cx<T> R[3][3];
    if (a.mode == 1) {
        cx<T> U[3][3];
        F::template load_link<18>(a.gauge + (size_t)(p * 4 + MU) * a.link_block_bytes, a.g.stride, h, U);
        if constexpr (sizeof(T) == 8) {
            traceless_antihermitian_of_GUdag(ga, gb, U, R);
        } else {
            cx<T> G[3][3];
#pragma unroll
            for (int i = 0; i < 3; i++)
#pragma unroll
                for (int j = 0; j < 3; j++) G[i][j] = {T(0), T(0)};
            outer_acc(G, ga[0], gb[0]);
            outer_acc(G, ga[1], gb[1]);
            traceless_antihermitian_of_GUdag(G, U, R);
        }
    } else {
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) R[i][j] = {T(0), T(0)};
        outer_acc(R, ga[0], gb[0]);
        outer_acc(R, ga[1], gb[1]);
    }
    const T c = (T)a.coef;
#pragma unroll
    for (int j = 0; j < 3; j++)
#pragma unroll
        for (int i = 0; i < 3; i++) {
            o[(j * 3 + i) * 2] = c * R[i][j].r;
            o[(j * 3 + i) * 2 + 1] = c * R[i][j].i;
        }
}

// One thread per site of checkerboard p = blockIdx.y (both checkerboards in
// one launch; they own disjoint links), all four links of the site.  The
// site's own spinor (chi on checkerboard pt, psi on cb) is loaded once for
// the four links.  The results go out in two halves (links 0-1, then 2-3),
// each staged in shared memory and written with 16-byte stores: in the
// canonical layout a CTA's sites are one contiguous run of the packed output
// and each half a 36-real block per site; with a caller layout each warp
// writes its sites' blocks one site at a time.
template <typename T, int ISIGN, int HALF>
__device__ __forceinline__ void force_half(const ForceArgs &a, int p, int h0, int h, const Nbr &n,
                                           const cx<T> (&own)[4][3], T *stage) {
    using Q = typename VecOf<T>::S;  // 16-byte vector: float4 or double2
    constexpr int NS = ForceTile<T>::sites;
    constexpr int QPS = 72 * (int)sizeof(T) / 16;  // 16-byte vectors per site
    constexpr int QH = QPS / 2;                    // per half
    if (h < a.g.Vh) {
        T *st = stage + threadIdx.x * 36;
        force_link<T, ISIGN, 2 * HALF>(a, p, h, n, own, st);
        force_link<T, ISIGN, 2 * HALF + 1>(a, p, h, n, own, st + 18);
    }
    __syncthreads();
    const int nsites = min(NS, a.g.Vh - h0);
    const Q *sq = reinterpret_cast<const Q *>(stage);
    Q *out = static_cast<Q *>(a.out);
    if (!a.table) {
        Q *dst = out + (size_t)(p * a.g.Vh + h0) * QPS + HALF * QH;
        for (int i = threadIdx.x; i < nsites * QH; i += NS) {
            const int s = i / QH, j = i - s * QH;
            Q v = sq[i];
            Q *d = dst + (size_t)s * QPS + j;
            if (a.accumulate) {
                const Q w = *d;
                if constexpr (sizeof(T) == 4) v = make_float4(w.x + v.x, w.y + v.y, w.z + v.z, w.w + v.w);
                else v = make_double2(w.x + v.x, w.y + v.y);
            }
            *d = v;
        }
    } else {
        const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        for (int k = w * 32; k < min(nsites, w * 32 + 32); k++) {
            Q *dst = out + (size_t)a.table[p * a.g.Vh + h0 + k] * QPS + HALF * QH;
            for (int i = lane; i < QH; i += 32) {
                Q v = sq[k * QH + i];
                if (a.accumulate) {
                    const Q w2 = dst[i];
                    if constexpr (sizeof(T) == 4) v = make_float4(w2.x + v.x, w2.y + v.y, w2.z + v.z, w2.w + v.w);
                    else v = make_double2(w2.x + v.x, w2.y + v.y);
                }
                dst[i] = v;
            }
        }
    }
    __syncthreads();  // the staging area is refilled by the next half
}

template <typename T, int ISIGN>
__global__ void __launch_bounds__(ForceTile<T>::sites, ForceTile<T>::min_blocks) force_kernel(const ForceArgs a) {
    using F = Field<T>;
    using V = typename VecOf<T>::S;
    constexpr int NS = ForceTile<T>::sites;
    __shared__ __align__(16) T stage[NS * 36];
    const int p = blockIdx.y;
    const int h0 = blockIdx.x * NS;
    const int h = h0 + threadIdx.x;
    Nbr n;
    cx<T> own[4][3];
    if (h < a.g.Vh) {
        neighbours<4>(a.g, h, p, n);
        F::load_spinor(static_cast<const V *>(p == a.pt ? a.chi : a.psi), a.g.stride, h, own);
    }
    force_half<T, ISIGN, 0>(a, p, h0, h, n, own, stage);
    force_half<T, ISIGN, 1>(a, p, h0, h, n, own, stage);
}

}  // namespace
}  // namespace gbds

using namespace gbds;

extern "C" int gbds_op_force(gbds_op op, const void *gauge, const void *psi, const void *chi, int isign, int cb,
                             int mode, double coef, int accumulate, void *force_packed, void *stream) {
    if (!op) return set_error(GBDS_ERROR_NOT_INITIALIZED, "op is NULL");
    if (op->g.nd != 4 || op->nrhs != 1 || op->format != GBDS_SPINOR_NATIVE || op->recon != 18)
        return set_error(GBDS_ERROR_UNSUPPORTED, "the force needs a 4D, single right-hand side, native, recon 18 operator");
    if (isign != 1 && isign != -1) return set_error(GBDS_ERROR_INVALID_VALUE, "isign must be +1 or -1");
    if (cb != 0 && cb != 1) return set_error(GBDS_ERROR_INVALID_VALUE, "cb must be 0 or 1");
    if (mode != 0 && mode != 1) return set_error(GBDS_ERROR_INVALID_VALUE, "mode must be 0 (gradient) or 1 (su(3) force)");
    if (!gauge || !psi || !chi || !force_packed) return set_error(GBDS_ERROR_INVALID_VALUE, "NULL field pointer");
    ForceArgs a;
    a.g = op->g;
    a.gauge = static_cast<const char *>(gauge);
    a.link_block_bytes = (size_t)18 * (op->prec == 32 ? 4 : 8) * op->g.stride;
    a.psi = psi;
    a.chi = chi;
    a.table = op->d_site_table;
    a.out = force_packed;
    a.pt = 1 - cb;
    a.mode = mode;
    a.coef = coef;
    a.accumulate = accumulate ? 1 : 0;
    if ((reinterpret_cast<uintptr_t>(force_packed) & 15u) != 0)
        return set_error(GBDS_ERROR_INVALID_VALUE, "force_packed must be 16-byte aligned");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (op->prec == 32) {
        constexpr int ns = ForceTile<float>::sites;
        const dim3 grid((op->g.Vh + ns - 1) / ns, 2);
        if (isign > 0) force_kernel<float, 1><<<grid, ns, 0, st>>>(a);
        else force_kernel<float, -1><<<grid, ns, 0, st>>>(a);
    } else {
        constexpr int ns = ForceTile<double>::sites;
        const dim3 grid((op->g.Vh + ns - 1) / ns, 2);
        if (isign > 0) force_kernel<double, 1><<<grid, ns, 0, st>>>(a);
        else force_kernel<double, -1><<<grid, ns, 0, st>>>(a);
    }
    count_launch();
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GBDS_SUCCESS : cuda_error(e, "gbds_op_force");
}
