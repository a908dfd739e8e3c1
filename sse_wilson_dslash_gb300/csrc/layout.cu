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

#include <cstring>

#include "dfloat.cuh"
#include "gbds_internal.h"

namespace gbds {

namespace {

// DF: the internal FP64 field is stored as double-float (dfloat.cuh); one
// 16-byte unit is one complex either way
template <bool DF>
__device__ __forceinline__ uint4 to_internal(uint4 v) {
    if constexpr (DF) {
        double2 d;
        memcpy(&d, &v, 16);
        const float4 f = df_from_double2(d);
        memcpy(&v, &f, 16);
    }
    return v;
}

template <bool DF>
__device__ __forceinline__ uint4 to_packed(uint4 v) {
    if constexpr (DF) {
        float4 f;
        memcpy(&f, &v, 16);
        const double2 d = df_to_double2(f);
        memcpy(&v, &d, 16);
    }
    return v;
}

// Spinors move as 16-byte units: FP32 = 6 units (float4), FP64 = 12 (double2).
// `site0` is subtracted from the caller index before addressing `packed`, so
// a buffer that holds only sites [site0, site0 + Vh) can be used.
template <bool DF>
__global__ void pack_spinor_kernel(const uint4 *__restrict__ packed, const int *__restrict__ table, int site0,
                                   int parity, int Vh, int stride, int units, uint4 *__restrict__ soa) {
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= (long long)units * Vh) return;
    const int k = (int)(tid / Vh), h = (int)(tid % Vh);
    const int i = parity * Vh + h;
    const int c = table ? __ldg(table + i) : i;
    soa[(size_t)k * stride + h] = to_internal<DF>(__ldg(packed + (size_t)(c - site0) * units + k));
}

template <bool DF>
__global__ void unpack_spinor_kernel(const uint4 *__restrict__ soa, const int *__restrict__ table, int site0,
                                     int parity, int Vh, int stride, int units, uint4 *__restrict__ packed) {
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= (long long)units * Vh) return;
    const int h = (int)(tid / units), k = (int)(tid % units);
    const int i = parity * Vh + h;
    const int c = table ? __ldg(table + i) : i;
    packed[(size_t)(c - site0) * units + k] = to_packed<DF>(__ldg(soa + (size_t)k * stride + h));
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

// ---------------------------------------------------------------------------
// Canonical-order kernels staged through shared memory.  Every access to the
// packed array is a contiguous, fully coalesced run, so these also work well
// when the packed array is host memory read or written directly by the GPU
// (pinned memory, or pageable memory on a coherent NVLink-C2C host).  Plain
// loads and stores are used on the packed side (it may be host memory).
// ---------------------------------------------------------------------------

constexpr int kSpinorTile = 128;  // sites per block
constexpr int kGaugeTile = 32;

// packed: first site of checkerboard `parity` (sites [0, Vh) of that half).
template <int UNITS, bool DF = false>
__global__ void __launch_bounds__(128) pack_spinor_tile(const uint4 *packed, int Vh, int stride, uint4 *__restrict__ soa) {
    __shared__ uint4 sm[kSpinorTile * UNITS];
    const int h0 = blockIdx.x * kSpinorTile;
    const int n = min(kSpinorTile, Vh - h0);
    const uint4 *src = packed + (size_t)h0 * UNITS;
    for (int e = threadIdx.x; e < n * UNITS; e += blockDim.x) sm[e] = src[e];
    __syncthreads();
    for (int e = threadIdx.x; e < n * UNITS; e += blockDim.x) {
        const int k = e / n, t = e - k * n;
        soa[(size_t)k * stride + h0 + t] = to_internal<DF>(sm[t * UNITS + k]);
    }
}

template <int UNITS, bool DF = false>
__global__ void __launch_bounds__(128) unpack_spinor_tile(const uint4 *__restrict__ soa, int Vh, int stride, uint4 *packed) {
    __shared__ uint4 sm[kSpinorTile * UNITS];
    const int h0 = blockIdx.x * kSpinorTile;
    const int n = min(kSpinorTile, Vh - h0);
    for (int e = threadIdx.x; e < n * UNITS; e += blockDim.x) {
        const int k = e / n, t = e - k * n;
        sm[t * UNITS + k] = to_packed<DF>(__ldg(soa + (size_t)k * stride + h0 + t));
    }
    __syncthreads();
    uint4 *dst = packed + (size_t)h0 * UNITS;
    for (int e = threadIdx.x; e < n * UNITS; e += blockDim.x) dst[e] = sm[e];
}

// Gauge: block of kGaugeTile consecutive caller sites (canonical order, both
// checkerboards), only the first nd links of each site are read.  Units of 8
// bytes (one float2 / one double) keep the 3D skip of mu = 3 exact.
template <typename T, int RECON>
__global__ void __launch_bounds__(128) pack_gauge_tile(const unsigned long long *packed, Geom g, char *__restrict__ gauge,
                                                        size_t block_bytes) {
    constexpr int SITE_UNITS = 4 * 18 * sizeof(T) / 8;  // 8-byte units per site (4 links)
    constexpr int LINK_UNITS = 18 * sizeof(T) / 8;
    __shared__ unsigned long long sm[kGaugeTile * SITE_UNITS];
    const int i0 = blockIdx.x * kGaugeTile;
    const int n = min(kGaugeTile, g.V - i0);
    const int used = g.nd * LINK_UNITS;  // leading units of each site that are read
    const unsigned long long *src = packed + (size_t)i0 * SITE_UNITS;
    for (int e = threadIdx.x; e < n * used; e += blockDim.x) {
        const int t = e / used, u = e - t * used;
        sm[t * SITE_UNITS + u] = src[(size_t)t * SITE_UNITS + u];
    }
    __syncthreads();
    const T *st = reinterpret_cast<const T *>(sm);
    constexpr int C = sizeof(T) == 4 ? (RECON == 18 ? 9 : 3) : (RECON == 18 ? 9 : 6);
    for (int e = threadIdx.x; e < n * g.nd * C; e += blockDim.x) {
        const int t = e % n, rest = e / n;
        const int mu = rest / C, k = rest % C;
        const int i = i0 + t;
        const int p = i >= g.Vh ? 1 : 0, h = i - p * g.Vh;
        const T *m = st + (size_t)t * 72 + mu * 18;  // m[(3j+i)*2] = U_ij
        char *blk = gauge + (size_t)(p * g.nd + mu) * block_bytes;
        if constexpr (sizeof(T) == 4 && RECON == 18) {
            const int r = k / 3, c = k % 3;
            reinterpret_cast<float2 *>(blk)[(size_t)k * g.stride + h] = make_float2(m[(3 * c + r) * 2], m[(3 * c + r) * 2 + 1]);
        } else if constexpr (sizeof(T) == 4) {
            const int a = 2 * k, b = 2 * k + 1;  // complex components (row-major over rows 0, 1)
            reinterpret_cast<float4 *>(blk)[(size_t)k * g.stride + h] =
                make_float4(m[(3 * (a % 3) + a / 3) * 2], m[(3 * (a % 3) + a / 3) * 2 + 1],
                            m[(3 * (b % 3) + b / 3) * 2], m[(3 * (b % 3) + b / 3) * 2 + 1]);
        } else {
            const int r = k / 3, c = k % 3;
            reinterpret_cast<double2 *>(blk)[(size_t)k * g.stride + h] = make_double2(m[(3 * c + r) * 2], m[(3 * c + r) * 2 + 1]);
        }
    }
}

}  // namespace

size_t spinor_bytes(const Geom &g, int prec) { return (size_t)24 * (prec == 32 ? 4 : 8) * g.stride; }

size_t gauge_block_bytes(const Geom &g, int prec, int recon) {
    return (size_t)recon * (prec == 32 ? 4 : 8) * g.stride;
}

size_t gauge_bytes(const Geom &g, int prec, int recon) { return 2 * (size_t)g.nd * gauge_block_bytes(g, prec, recon); }

cudaError_t launch_pack_spinor(const Geom &g, int prec, const void *psi_packed, const int *site_table,
                               int site0, int parity, void *spinor, cudaStream_t stream, bool df) {
    const int units = prec == 32 ? 6 : 12;
    df = df && prec == 64;
    if (!site_table) {
        // canonical: the checkerboard is the contiguous run [parity*Vh, parity*Vh + Vh) - site0
        const uint4 *src = static_cast<const uint4 *>(psi_packed) + (size_t)(parity * g.Vh - site0) * units;
        const unsigned nb = blocks_for(g.Vh, kSpinorTile);
        uint4 *dst = static_cast<uint4 *>(spinor);
        if (prec == 32) pack_spinor_tile<6><<<nb, 128, 0, stream>>>(src, g.Vh, g.stride, dst);
        else if (df) pack_spinor_tile<12, true><<<nb, 128, 0, stream>>>(src, g.Vh, g.stride, dst);
        else pack_spinor_tile<12><<<nb, 128, 0, stream>>>(src, g.Vh, g.stride, dst);
        count_launch();
        return cudaGetLastError();
    }
    const long long n = (long long)units * g.Vh;
    auto k = df ? pack_spinor_kernel<true> : pack_spinor_kernel<false>;
    k<<<blocks_for(n, 256), 256, 0, stream>>>(static_cast<const uint4 *>(psi_packed), site_table, site0, parity, g.Vh,
                                              g.stride, units, static_cast<uint4 *>(spinor));
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_unpack_spinor(const Geom &g, int prec, const void *spinor, const int *site_table,
                                 int site0, int parity, void *psi_packed, cudaStream_t stream, bool df) {
    const int units = prec == 32 ? 6 : 12;
    df = df && prec == 64;
    const uint4 *src = static_cast<const uint4 *>(spinor);
    if (!site_table) {
        uint4 *dst = static_cast<uint4 *>(psi_packed) + (size_t)(parity * g.Vh - site0) * units;
        const unsigned nb = blocks_for(g.Vh, kSpinorTile);
        if (prec == 32) unpack_spinor_tile<6><<<nb, 128, 0, stream>>>(src, g.Vh, g.stride, dst);
        else if (df) unpack_spinor_tile<12, true><<<nb, 128, 0, stream>>>(src, g.Vh, g.stride, dst);
        else unpack_spinor_tile<12><<<nb, 128, 0, stream>>>(src, g.Vh, g.stride, dst);
        count_launch();
        return cudaGetLastError();
    }
    const long long n = (long long)units * g.Vh;
    auto k = df ? unpack_spinor_kernel<true> : unpack_spinor_kernel<false>;
    k<<<blocks_for(n, 256), 256, 0, stream>>>(src, site_table, site0, parity, g.Vh, g.stride, units,
                                              static_cast<uint4 *>(psi_packed));
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_pack_gauge(const Geom &g, int prec, int recon, const void *u_packed, const int *site_table,
                              void *gauge, cudaStream_t stream) {
    const long long n = 2LL * g.nd * g.Vh;
    const size_t bb = gauge_block_bytes(g, prec, recon);
    char *dst = static_cast<char *>(gauge);
    if (!site_table) {
        const unsigned long long *src = static_cast<const unsigned long long *>(u_packed);
        const unsigned nt = blocks_for(g.V, kGaugeTile);
        if (prec == 32) {
            if (recon == 18) pack_gauge_tile<float, 18><<<nt, 128, 0, stream>>>(src, g, dst, bb);
            else pack_gauge_tile<float, 12><<<nt, 128, 0, stream>>>(src, g, dst, bb);
        } else {
            if (recon == 18) pack_gauge_tile<double, 18><<<nt, 128, 0, stream>>>(src, g, dst, bb);
            else pack_gauge_tile<double, 12><<<nt, 128, 0, stream>>>(src, g, dst, bb);
        }
        count_launch();
        return cudaGetLastError();
    }
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
