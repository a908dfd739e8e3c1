// Layout kernels: the reference's packed host layout <-> the internal
// structure-of-arrays layout, with an optional site permutation for callers
// whose site order is not the canonical one.
//
// These replace, on the device, the reference's gauge packers
// (lib/packer_nopad.c:29-45, lib/qdp_packer_nopad.cc:7-19,
// lib/qdp_packer_3d.cc:13-22) as the step between the caller's arrays and the
// operator, and the reference's site_table indirection
// (lib/shift_tables_scalar.c:240-263).
#include <cuda_runtime.h>

#include "gbds_internal.h"

namespace gbds {

namespace {

// Spinors move as 16-byte units: FP32 = 6 units (float4), FP64 = 12 (double2).
// `site0` is subtracted from the caller index before addressing `packed`, so
// a buffer that holds only sites [site0, site0 + Vh) can be used.
__global__ void pack_spinor_kernel(const uint4 *__restrict__ packed, const int *__restrict__ table, int site0,
                                   int parity, int Vh, int stride, int units, uint4 *__restrict__ soa) {
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= (long long)units * Vh) return;
    const int k = (int)(tid / Vh), h = (int)(tid % Vh);
    const int i = parity * Vh + h;
    const int c = table ? __ldg(table + i) : i;
    soa[(size_t)k * stride + h] = __ldg(packed + (size_t)(c - site0) * units + k);
}

__global__ void unpack_spinor_kernel(const uint4 *__restrict__ soa, const int *__restrict__ table, int site0,
                                     int parity, int Vh, int stride, int units, uint4 *__restrict__ packed) {
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= (long long)units * Vh) return;
    const int h = (int)(tid / units), k = (int)(tid % units);
    const int i = parity * Vh + h;
    const int c = table ? __ldg(table + i) : i;
    packed[(size_t)(c - site0) * units + k] = __ldg(soa + (size_t)k * stride + h);
}

// One thread per (parity, mu, h): reads the packed 3x3 link (transposed,
// u[j][i] = U_ij), writes the internal components.
template <typename T, int RECON>
__global__ void pack_gauge_kernel(const T *__restrict__ packed, const int *__restrict__ table,
                                  Geom g, char *__restrict__ gauge, size_t block_bytes) {
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long n = 2LL * g.nd * g.Vh;
    if (tid >= n) return;
    const int h = (int)(tid % g.Vh);
    const int pm = (int)(tid / g.Vh);  // p * nd + mu
    const int p = pm / g.nd, mu = pm % g.nd;
    const int i = p * g.Vh + h;
    const int c = table ? __ldg(table + i) : i;
    const T *src = packed + ((size_t)c * 4 + mu) * 18;
    T U[3][3][2];
#pragma unroll
    for (int j = 0; j < 3; j++)
#pragma unroll
        for (int ii = 0; ii < 3; ii++) {
            U[ii][j][0] = src[(j * 3 + ii) * 2];
            U[ii][j][1] = src[(j * 3 + ii) * 2 + 1];
        }
    char *blk = gauge + (size_t)pm * block_bytes;
    if constexpr (sizeof(T) == 4 && RECON == 18) {
        float2 *d = reinterpret_cast<float2 *>(blk);
#pragma unroll
        for (int k = 0; k < 9; k++) d[(size_t)k * g.stride + h] = make_float2(U[k / 3][k % 3][0], U[k / 3][k % 3][1]);
    } else if constexpr (sizeof(T) == 4 && RECON == 12) {
        float4 *d = reinterpret_cast<float4 *>(blk);
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const int a = 2 * k, b = 2 * k + 1;
            d[(size_t)k * g.stride + h] = make_float4(U[a / 3][a % 3][0], U[a / 3][a % 3][1],
                                                      U[b / 3][b % 3][0], U[b / 3][b % 3][1]);
        }
    } else {
        double2 *d = reinterpret_cast<double2 *>(blk);
        constexpr int nk = RECON == 18 ? 9 : 6;
#pragma unroll
        for (int k = 0; k < nk; k++) d[(size_t)k * g.stride + h] = make_double2(U[k / 3][k % 3][0], U[k / 3][k % 3][1]);
    }
}

inline unsigned blocks_for(long long n, int threads) { return (unsigned)((n + threads - 1) / threads); }

}  // namespace

size_t spinor_bytes(const Geom &g, int prec) { return (size_t)24 * (prec == 32 ? 4 : 8) * g.stride; }

size_t gauge_block_bytes(const Geom &g, int prec, int recon) {
    return (size_t)recon * (prec == 32 ? 4 : 8) * g.stride;
}

size_t gauge_bytes(const Geom &g, int prec, int recon) { return 2 * (size_t)g.nd * gauge_block_bytes(g, prec, recon); }

cudaError_t launch_pack_spinor(const Geom &g, int prec, const void *psi_packed, const int *site_table,
                               int site0, int parity, void *spinor, cudaStream_t stream) {
    const int units = prec == 32 ? 6 : 12;
    const long long n = (long long)units * g.Vh;
    pack_spinor_kernel<<<blocks_for(n, 256), 256, 0, stream>>>(static_cast<const uint4 *>(psi_packed), site_table,
                                                               site0, parity, g.Vh, g.stride, units,
                                                               static_cast<uint4 *>(spinor));
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_unpack_spinor(const Geom &g, int prec, const void *spinor, const int *site_table,
                                 int site0, int parity, void *psi_packed, cudaStream_t stream) {
    const int units = prec == 32 ? 6 : 12;
    const long long n = (long long)units * g.Vh;
    unpack_spinor_kernel<<<blocks_for(n, 256), 256, 0, stream>>>(static_cast<const uint4 *>(spinor), site_table,
                                                                 site0, parity, g.Vh, g.stride, units,
                                                                 static_cast<uint4 *>(psi_packed));
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_pack_gauge(const Geom &g, int prec, int recon, const void *u_packed, const int *site_table,
                              void *gauge, cudaStream_t stream) {
    const long long n = 2LL * g.nd * g.Vh;
    const size_t bb = gauge_block_bytes(g, prec, recon);
    char *dst = static_cast<char *>(gauge);
    const unsigned nb = blocks_for(n, 128);
    if (prec == 32) {
        const float *src = static_cast<const float *>(u_packed);
        if (recon == 18) pack_gauge_kernel<float, 18><<<nb, 128, 0, stream>>>(src, site_table, g, dst, bb);
        else pack_gauge_kernel<float, 12><<<nb, 128, 0, stream>>>(src, site_table, g, dst, bb);
    } else {
        const double *src = static_cast<const double *>(u_packed);
        if (recon == 18) pack_gauge_kernel<double, 18><<<nb, 128, 0, stream>>>(src, site_table, g, dst, bb);
        else pack_gauge_kernel<double, 12><<<nb, 128, 0, stream>>>(src, site_table, g, dst, bb);
    }
    count_launch();
    return cudaGetLastError();
}

}  // namespace gbds
