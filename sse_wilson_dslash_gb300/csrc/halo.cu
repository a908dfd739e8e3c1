// Domain decomposition along t: the Dslash of one rank's sub-lattice with the
// time direction split across ranks (gbds_op_pack_faces /
// gbds_op_dslash_halo in gbdslash.h).
//
// Replaces the reference's parscalar halo path
// (lib/sse_su3dslash_32bit_parscalar.c:967-1095 face buffers,
// :1203-1284 communication overlapped with the interior, the decomp /
// decomp_hvv stages that fill the send buffers and the mvv_recons / recons
// stages that consume the received ones, lib/shift_tables_parscalar.c for
// the face tables).  Here the other three directions stay periodic on the
// device and only t crosses ranks:
//
//   * a target site x on the last local time slice takes its forward t hop
//     from the next rank: that rank sends the projected half spinor
//     (1 - isign g_t) psi(y) of its first time slice (12 reals a site), and
//     the receiver multiplies by its own U_t(x) and reconstructs;
//   * a target site on the first local slice takes its backward t hop from the
//     previous rank, which owns U_t(x - t): it sends U_t(y)^+ (1 + isign g_t)
//     psi(y) of its last time slice, and the receiver only reconstructs.
//
// Face buffers hold one checkerboard of a time slice, S = Lz Ly Lx / 2 half
// spinors, in the slice's site order, structure-of-arrays: FP32 3 float4
// components (reals 4k..4k+3 of h[2][3][2]), FP64 6 double2 (complex k).
// With an even local Lt the local parity equals the global one, and the
// receiving index of a face site is its offset within the time slice.
#include <cuda_runtime.h>

#include <cstdint>

#include "dslash_kernel.cuh"

namespace gbds {
namespace {

template <typename T> struct Face;
template <>
struct Face<float> {
    __device__ __forceinline__ static void store(float4 *f, int S, int s, const cx<float> (&h)[2][3]) {
        f[s] = make_float4(h[0][0].r, h[0][0].i, h[0][1].r, h[0][1].i);
        f[S + s] = make_float4(h[0][2].r, h[0][2].i, h[1][0].r, h[1][0].i);
        f[2 * S + s] = make_float4(h[1][1].r, h[1][1].i, h[1][2].r, h[1][2].i);
    }
    __device__ __forceinline__ static void load(const float4 *f, int S, int s, cx<float> (&h)[2][3]) {
        const float4 a = __ldg(f + s), b = __ldg(f + S + s), c = __ldg(f + 2 * S + s);
        h[0][0] = {a.x, a.y}; h[0][1] = {a.z, a.w}; h[0][2] = {b.x, b.y};
        h[1][0] = {b.z, b.w}; h[1][1] = {c.x, c.y}; h[1][2] = {c.z, c.w};
    }
};
template <>
struct Face<double> {
    __device__ __forceinline__ static void store(double2 *f, int S, int s, const cx<double> (&h)[2][3]) {
#pragma unroll
        for (int k = 0; k < 6; k++) f[k * S + s] = make_double2(h[k / 3][k % 3].r, h[k / 3][k % 3].i);
    }
    __device__ __forceinline__ static void load(const double2 *f, int S, int s, cx<double> (&h)[2][3]) {
#pragma unroll
        for (int k = 0; k < 6; k++) {
            const double2 q = __ldg(f + k * S + s);
            h[k / 3][k % 3] = {q.x, q.y};
        }
    }
};

template <typename T>
DslashArgs<T> make_args(const Geom &g, int recon, const void *gauge, const void *psi, void *res, int cb) {
    DslashArgs<T> a;
    a.g = g;
    a.psi = static_cast<const typename VecOf<T>::S *>(psi);
    a.res = static_cast<typename VecOf<T>::S *>(res);
    a.gauge = static_cast<const char *>(gauge);
    const int vec_bytes = sizeof(T) == 4 ? (recon == 18 ? 8 : 16) : 16;
    a.link_block_bytes = (size_t)Field<T>::link_vecs(recon) * g.stride * vec_bytes;
    a.pt = 1 - cb;
    return a;
}

// Send buffers of the source field psi (checkerboard cb = 1 - a.pt):
// blockIdx.y 0 -> to_prev: (1 - isign g_t) psi on the first time slice;
// blockIdx.y 1 -> to_next: U_t^+ (1 + isign g_t) psi on the last time slice.
template <typename T, int RECON, int ISIGN>
__global__ void __launch_bounds__(128) pack_faces_kernel(const DslashArgs<T> a, int S, typename VecOf<T>::S *to_prev,
                                                         typename VecOf<T>::S *to_next) {
    using F = Field<T>;
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    cx<T> sp[4][3], hs[2][3];
    if (blockIdx.y == 0) {
        F::load_spinor(a.psi, a.g.stride, s, sp);
        project<3, ISIGN>(sp, hs);
        Face<T>::store(to_prev, S, s, hs);
    } else {
        const int h = (a.g.L[3] - 1) * S + s;
        const int ps = 1 - a.pt;
        F::load_spinor(a.psi, a.g.stride, h, sp);
        project<3, -ISIGN>(sp, hs);
        cx<T> U[3][3], w[2][3];
        F::template load_link<RECON>(a.gauge + (size_t)(ps * 4 + 3) * a.link_block_bytes, a.g.stride, h, U);
        su3_mul<true>(U, hs, w);
        Face<T>::store(to_next, S, s, w);
    }
}

template <typename T>
struct HaloArgs {
    DslashArgs<T> a;
    const typename VecOf<T>::S *from_prev;  // backward t hops of the first slice
    const typename VecOf<T>::S *from_next;  // forward t hops of the last slice
    int S;                                  // sites of one checkerboard of a time slice
    int first_a, count_a, first_b, total;   // sites [first_a, +count_a) then [first_b, ...)
};

template <typename T, int RECON, int ISIGN>
__device__ __forceinline__ void halo_hop_t(const HaloArgs<T> &ha, int h, int t, const Nbr &n, cx<T> (&acc)[4][3]) {
    using F = Field<T>;
    const DslashArgs<T> &a = ha.a;
    const int Lt = a.g.L[3];
    const int ps = 1 - a.pt;
    cx<T> s[4][3], hs[2][3], w[2][3], U[3][3];
    // forward: U_t(x) (1 - isign g_t) psi(x + t), the half spinor from the next rank on the last slice
    if (t == Lt - 1) {
        Face<T>::load(ha.from_next, ha.S, h - (Lt - 1) * ha.S, hs);
    } else {
        F::load_spinor(a.psi, a.g.stride, n.f[3], s);
        project<3, ISIGN>(s, hs);
    }
    F::template load_link<RECON, true>(a.gauge + (size_t)(a.pt * 4 + 3) * a.link_block_bytes, a.g.stride, h, U);
    su3_mul<false>(U, hs, w);
    reconstruct<3, ISIGN>(acc, w);
    // backward: U_t(x - t)^+ (1 + isign g_t) psi(x - t), received whole on the first slice
    if (t == 0) {
        Face<T>::load(ha.from_prev, ha.S, h, w);
    } else {
        F::load_spinor(a.psi, a.g.stride, n.b[3], s);
        F::template load_link<RECON, true>(a.gauge + (size_t)(ps * 4 + 3) * a.link_block_bytes, a.g.stride, n.b[3], U);
        project<3, -ISIGN>(s, hs);
        su3_mul<true>(U, hs, w);
    }
    reconstruct<3, -ISIGN>(acc, w);
}

template <typename T, int RECON, int ISIGN, int MINB>
__global__ void __launch_bounds__(Bounds<MINB>::threads, Bounds<MINB>::blocks) dslash_halo_kernel(const HaloArgs<T> ha) {
    pdl_allow_next();
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    const bool act = idx < ha.total;
    const int h = idx < ha.count_a ? ha.first_a + idx : ha.first_b + (idx - ha.count_a);
    Nbr n;
    if (act) neighbours<4>(ha.a.g, h, ha.a.pt, n);
    pdl_wait_prev();
    if (!act) return;
    cx<T> acc[4][3];
#pragma unroll
    for (int s = 0; s < 4; s++)
#pragma unroll
        for (int c = 0; c < 3; c++) acc[s][c] = {T(0), T(0)};
    hop_pair_any<T, 4, RECON, ISIGN, 0>(ha.a, h, n, acc);
    hop_pair_any<T, 4, RECON, ISIGN, 1>(ha.a, h, n, acc);
    hop_pair_any<T, 4, RECON, ISIGN, 2>(ha.a, h, n, acc);
    halo_hop_t<T, RECON, ISIGN>(ha, h, h / ha.S, n, acc);
    Field<T>::store_spinor(ha.a.res, ha.a.g.stride, h, acc);
}

// FP32: the register cap of the single-rhs kernel's default variant (6
// blocks of 128 threads per SM); FP64: uncapped.
template <typename T> struct HaloMinb { static constexpr int v = sizeof(T) == 4 ? 6 : 0; };

template <typename T>
cudaError_t launch_pack_faces_t(const Geom &g, int recon, const void *gauge, const void *psi, int isign, int cb,
                                void *to_prev, void *to_next, cudaStream_t st) {
    const DslashArgs<T> a = make_args<T>(g, recon, gauge, psi, nullptr, cb);
    const int S = g.Vh / g.L[3];
    auto *tp = static_cast<typename VecOf<T>::S *>(to_prev);
    auto *tn = static_cast<typename VecOf<T>::S *>(to_next);
    const dim3 grid((S + 127) / 128, 2);
    if (recon == 18) {
        if (isign > 0) pack_faces_kernel<T, 18, 1><<<grid, 128, 0, st>>>(a, S, tp, tn);
        else pack_faces_kernel<T, 18, -1><<<grid, 128, 0, st>>>(a, S, tp, tn);
    } else {
        if (isign > 0) pack_faces_kernel<T, 12, 1><<<grid, 128, 0, st>>>(a, S, tp, tn);
        else pack_faces_kernel<T, 12, -1><<<grid, 128, 0, st>>>(a, S, tp, tn);
    }
    count_launch();
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_halo_t(const Geom &g, int recon, const void *gauge, const void *psi, const void *from_prev,
                          const void *from_next, void *res, int isign, int cb, int part, cudaStream_t st) {
    HaloArgs<T> ha;
    ha.a = make_args<T>(g, recon, gauge, psi, res, cb);
    ha.from_prev = static_cast<const typename VecOf<T>::S *>(from_prev);
    ha.from_next = static_cast<const typename VecOf<T>::S *>(from_next);
    const int Lt = g.L[3], S = g.Vh / Lt;
    ha.S = S;
    if (part == GBDS_HALO_INTERIOR) {
        ha.first_a = S, ha.count_a = (Lt - 2) * S, ha.first_b = 0, ha.total = ha.count_a;
    } else if (part == GBDS_HALO_BOUNDARY) {
        ha.first_a = 0, ha.count_a = S, ha.first_b = (Lt - 1) * S, ha.total = 2 * S;
    } else {
        ha.first_a = 0, ha.count_a = g.Vh, ha.first_b = 0, ha.total = g.Vh;
    }
    if (ha.total == 0) return cudaSuccess;  // no interior slice when Lt = 2
    constexpr int MINB = HaloMinb<T>::v;
    const dim3 grid((ha.total + 127) / 128);
    if (recon == 18) {
        if (isign > 0) launch_pdl(dslash_halo_kernel<T, 18, 1, MINB>, grid, 128, st, ha);
        else launch_pdl(dslash_halo_kernel<T, 18, -1, MINB>, grid, 128, st, ha);
    } else {
        if (isign > 0) launch_pdl(dslash_halo_kernel<T, 12, 1, MINB>, grid, 128, st, ha);
        else launch_pdl(dslash_halo_kernel<T, 12, -1, MINB>, grid, 128, st, ha);
    }
    count_launch();
    return cudaGetLastError();
}

bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

int check_halo_op(gbds_op op) {
    if (!op) return set_error(GBDS_ERROR_NOT_INITIALIZED, "op is NULL");
    if (op->g.nd != 4 || op->nrhs != 1 || op->format != GBDS_SPINOR_NATIVE)
        return set_error(GBDS_ERROR_UNSUPPORTED,
                         "the split-t operator needs a 4D, single right-hand side, native-format operator");
    return GBDS_SUCCESS;
}

}  // namespace
}  // namespace gbds

using namespace gbds;

extern "C" size_t gbds_op_face_bytes(gbds_op op) {
    if (!op || op->g.nd != 4) return 0;
    const size_t S = (size_t)op->g.Vh / op->g.L[3];
    return S * 12 * (op->prec == 32 ? 4 : 8);
}

extern "C" int gbds_op_pack_faces(gbds_op op, const void *gauge, const void *psi, int isign, int cb, void *to_prev,
                                  void *to_next, void *stream) {
    int rc = check_halo_op(op);
    if (rc != GBDS_SUCCESS) return rc;
    if (isign != 1 && isign != -1) return GBDS_SUCCESS;
    if (cb != 0 && cb != 1) return set_error(GBDS_ERROR_INVALID_VALUE, "cb must be 0 or 1");
    if (!gauge || !psi || !to_prev || !to_next) return set_error(GBDS_ERROR_INVALID_VALUE, "NULL pointer");
    if (!aligned16(gauge) || !aligned16(psi) || !aligned16(to_prev) || !aligned16(to_next))
        return set_error(GBDS_ERROR_INVALID_VALUE, "fields and faces must be 16-byte aligned");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = op->prec == 32 ? launch_pack_faces_t<float>(op->g, op->recon, gauge, psi, isign, cb, to_prev, to_next, st)
                                   : launch_pack_faces_t<double>(op->g, op->recon, gauge, psi, isign, cb, to_prev, to_next, st);
    return e == cudaSuccess ? GBDS_SUCCESS : cuda_error(e, "gbds_op_pack_faces");
}

extern "C" int gbds_op_dslash_halo(gbds_op op, const void *gauge, const void *psi, const void *from_prev,
                                   const void *from_next, void *res, int isign, int cb, int part, void *stream) {
    int rc = check_halo_op(op);
    if (rc != GBDS_SUCCESS) return rc;
    if (isign != 1 && isign != -1) return GBDS_SUCCESS;
    if (cb != 0 && cb != 1) return set_error(GBDS_ERROR_INVALID_VALUE, "cb must be 0 or 1");
    if (part != GBDS_HALO_ALL && part != GBDS_HALO_INTERIOR && part != GBDS_HALO_BOUNDARY)
        return set_error(GBDS_ERROR_INVALID_VALUE, "part must be GBDS_HALO_ALL, _INTERIOR or _BOUNDARY");
    const bool faces = part != GBDS_HALO_INTERIOR;
    if (!gauge || !psi || !res || (faces && (!from_prev || !from_next)))
        return set_error(GBDS_ERROR_INVALID_VALUE, "NULL pointer");
    if (!aligned16(gauge) || !aligned16(psi) || !aligned16(res) ||
        (faces && (!aligned16(from_prev) || !aligned16(from_next))))
        return set_error(GBDS_ERROR_INVALID_VALUE, "fields and faces must be 16-byte aligned");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = op->prec == 32
                        ? launch_halo_t<float>(op->g, op->recon, gauge, psi, from_prev, from_next, res, isign, cb, part, st)
                        : launch_halo_t<double>(op->g, op->recon, gauge, psi, from_prev, from_next, res, isign, cb, part, st);
    return e == cudaSuccess ? GBDS_SUCCESS : cuda_error(e, "gbds_op_dslash_halo");
}
