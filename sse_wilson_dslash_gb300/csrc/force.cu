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
        for (int j = 0; j < 3; j++) {
            // (M - M^+)/2
            F[i][j] = {(M[i][j].r - M[j][i].r) / T(2), (M[i][j].i + M[j][i].i) / T(2)};
        }
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

template <typename T, int ISIGN, int MU>
__device__ __forceinline__ void force_link(const ForceArgs &a, int p, int h, const Nbr &n) {
    using F = Field<T>;
    using V = typename VecOf<T>::S;
    const V *psi = static_cast<const V *>(a.psi);
    const V *chi = static_cast<const V *>(a.chi);
    cx<T> G[3][3];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) G[i][j] = {T(0), T(0)};
    cx<T> s[4][3], hs[2][3], xi[2][3];
    if (p == a.pt) {
        // forward hop at x: xi from chi(x), half spinor of psi(x + mu)
        F::load_spinor(chi, a.g.stride, h, s);
        fold<MU, ISIGN>(s, xi);
        F::load_spinor(psi, a.g.stride, n.f[MU], s);
        project<MU, ISIGN>(s, hs);
        outer_acc(G, xi[0], hs[0]);
        outer_acc(G, xi[1], hs[1]);
    } else {
        // backward hop into y = x + mu: half spinor of psi(x), xi from chi(y)
        F::load_spinor(psi, a.g.stride, h, s);
        project<MU, -ISIGN>(s, hs);
        F::load_spinor(chi, a.g.stride, n.f[MU], s);
        fold<MU, -ISIGN>(s, xi);
        outer_acc(G, hs[0], xi[0]);
        outer_acc(G, hs[1], xi[1]);
    }
    cx<T> R[3][3];
    if (a.mode == 1) {
        cx<T> U[3][3];
        F::template load_link<18>(a.gauge + (size_t)(p * 4 + MU) * a.link_block_bytes, a.g.stride, h, U);
        traceless_antihermitian_of_GUdag(G, U, R);
    } else {
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) R[i][j] = G[i][j];
    }
    const int i_int = p * a.g.Vh + h;
    const int site = a.table ? a.table[i_int] : i_int;
    T *o = static_cast<T *>(a.out) + ((size_t)site * 4 + MU) * 18;
    const T c = (T)a.coef;
#pragma unroll
    for (int j = 0; j < 3; j++)
#pragma unroll
        for (int i = 0; i < 3; i++) {  // packed transposed: o[j][i] = R_ij
            T *d = o + (j * 3 + i) * 2;
            if (a.accumulate) {
                d[0] += c * R[i][j].r;
                d[1] += c * R[i][j].i;
            } else {
                d[0] = c * R[i][j].r;
                d[1] = c * R[i][j].i;
            }
        }
}

// One thread per site of checkerboard p; all four links of the site.
template <typename T, int ISIGN>
__global__ void __launch_bounds__(128) force_kernel(const ForceArgs a, int p) {
    const int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= a.g.Vh) return;
    Nbr n;
    neighbours<4>(a.g, h, p, n);
    force_link<T, ISIGN, 0>(a, p, h, n);
    force_link<T, ISIGN, 1>(a, p, h, n);
    force_link<T, ISIGN, 2>(a, p, h, n);
    force_link<T, ISIGN, 3>(a, p, h, n);
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
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const dim3 grid((op->g.Vh + 127) / 128);
    for (int p = 0; p < 2; p++) {
        if (op->prec == 32) {
            if (isign > 0) force_kernel<float, 1><<<grid, 128, 0, st>>>(a, p);
            else force_kernel<float, -1><<<grid, 128, 0, st>>>(a, p);
        } else {
            if (isign > 0) force_kernel<double, 1><<<grid, 128, 0, st>>>(a, p);
            else force_kernel<double, -1><<<grid, 128, 0, st>>>(a, p);
        }
        count_launch();
    }
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GBDS_SUCCESS : cuda_error(e, "gbds_op_force");
}
