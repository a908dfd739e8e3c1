// Launchers and layout kernels of the generalised Dslash (dslash_gen.cuh),
// instantiated per storage format by dslash_gen_f32.cu / dslash_gen_half.cu.
#pragma once

#include <atomic>

#include "dslash_gen.cuh"

namespace gbds {

// packed: FP32 [nrhs][V][4][3][2] in caller order; thread per (h, r).
template <int FMT>
__global__ void pack_gen_kernel(const float *__restrict__ packed, const int *__restrict__ table, int parity, Geom g,
                                int nrhs, size_t cs, char *out) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)g.Vh * nrhs) return;
    const int h = (int)(t / nrhs), r = (int)(t % nrhs);
    const int i = parity * g.Vh + h;
    const int c = table ? __ldg(table + i) : i;
    const float *src = packed + ((size_t)r * g.V + c) * 24;
    cx<float> s[4][3];
#pragma unroll
    for (int j = 0; j < 12; j++) s[j / 3][j % 3] = {src[2 * j], src[2 * j + 1]};
    Sio<FMT>::store(out, cs, (size_t)h * nrhs + r, s);
}

template <int FMT>
__global__ void unpack_gen_kernel(const char *in, const int *__restrict__ table, int parity, Geom g, int nrhs, size_t cs,
                                  float *packed) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)g.Vh * nrhs) return;
    const int h = (int)(t / nrhs), r = (int)(t % nrhs);
    const int i = parity * g.Vh + h;
    const int c = table ? __ldg(table + i) : i;
    cx<float> s[4][3];
    Sio<FMT>::load(in, cs, (size_t)h * nrhs + r, s);
    float *dst = packed + ((size_t)r * g.V + c) * 24;
#pragma unroll
    for (int j = 0; j < 12; j++) {
        dst[2 * j] = s[j / 3][j % 3].r;
        dst[2 * j + 1] = s[j / 3][j % 3].i;
    }
}

// EPI: 0 none, 1 xpay (nrhs 1), 2 xpay with per-rhs partials (nrhs 2..32,
// powers of two)
template <int FMT, int RECON, int ISIGN, int EPI>
void launch_gen_nrhs(const GenArgs &a, int nrhs, dim3 grid, cudaStream_t st) {
    constexpr int E1 = EPI == 1 ? 1 : 0;  // nrhs 1 takes the single-sum epilogue
    switch (nrhs) {
    case 1: if constexpr (EPI != 2) launch_pdl(dslash_gen_kernel<FMT, RECON, ISIGN, 1, E1>, grid, 128, st, a); break;
    case 2: if constexpr (EPI != 1) launch_pdl(dslash_gen_kernel<FMT, RECON, ISIGN, 2, EPI>, grid, 128, st, a); break;
    case 4: if constexpr (EPI != 1) launch_pdl(dslash_gen_kernel<FMT, RECON, ISIGN, 4, EPI>, grid, 128, st, a); break;
    case 8: if constexpr (EPI != 1) launch_pdl(dslash_gen_kernel<FMT, RECON, ISIGN, 8, EPI>, grid, 128, st, a); break;
    case 16: if constexpr (EPI != 1) launch_pdl(dslash_gen_kernel<FMT, RECON, ISIGN, 16, EPI>, grid, 128, st, a); break;
    case 32: if constexpr (EPI != 1) launch_pdl(dslash_gen_kernel<FMT, RECON, ISIGN, 32, EPI>, grid, 128, st, a); break;
    default: if constexpr (EPI == 0) launch_pdl(dslash_gen_kernel<FMT, RECON, ISIGN, 0, 0>, grid, 128, st, a); break;
    }
}

// nrhs 1 with FP16 links (the 16-bit inner solver's operator)
template <int FMT>
cudaError_t launch_gen_h16_t(const Geom &g, int recon, const void *gauge, const void *psi, void *res, int isign, int cb,
                             const void *x, float coef, double *partials, cudaStream_t st) {
    GenArgs a;
    a.g = g;
    a.psi = static_cast<const char *>(psi);
    a.res = static_cast<char *>(res);
    a.gauge = static_cast<const char *>(gauge);
    a.link_block_bytes = (size_t)recon * 2 * g.stride;
    a.cs = (size_t)g.stride;
    a.nrhs = 1;
    a.pt = 1 - cb;
    a.x = static_cast<const char *>(x);
    a.coef = coef;
    a.partials = partials;
    const dim3 grid((unsigned)((g.Vh + 127) / 128));
#define GBDS_H(R, S, E) launch_pdl(dslash_gen_kernel<FMT, R, S, 1, E, 1>, grid, 128, st, a)
    if (x) {
        if (recon == 18) { if (isign > 0) GBDS_H(18, 1, 1); else GBDS_H(18, -1, 1); }
        else             { if (isign > 0) GBDS_H(12, 1, 1); else GBDS_H(12, -1, 1); }
    } else {
        if (recon == 18) { if (isign > 0) GBDS_H(18, 1, 0); else GBDS_H(18, -1, 0); }
        else             { if (isign > 0) GBDS_H(12, 1, 0); else GBDS_H(12, -1, 0); }
    }
#undef GBDS_H
    count_launch();
    return cudaGetLastError();
}

template <int FMT, int RECON, int ISIGN, int EPI>
void launch_gen2_nrhs(const GenArgs &a, int nrhs, cudaStream_t st) {
    const unsigned vh = (unsigned)a.g.Vh;
    switch (nrhs) {
    case 8: launch_pdl(dslash_gen2_kernel<FMT, RECON, ISIGN, 8, EPI>, dim3((vh + 15) / 16), 128, st, a); break;
    case 16: launch_pdl(dslash_gen2_kernel<FMT, RECON, ISIGN, 16, EPI>, dim3((vh + 7) / 8), 128, st, a); break;
    default: launch_pdl(dslash_gen2_kernel<FMT, RECON, ISIGN, 32, EPI>, dim3((vh + 3) / 4), 128, st, a); break;
    }
}

template <int FMT, int RECON, int ISIGN, int EPI>
void launch_gen3_nrhs(const GenArgs &a, int nrhs, cudaStream_t st) {
    const unsigned vh = (unsigned)a.g.Vh;
    switch (nrhs) {
    case 8: launch_pdl(dslash_gen3_kernel<FMT, RECON, ISIGN, 8, EPI>, dim3((vh + 15) / 16), 128, st, a); break;
    case 16: launch_pdl(dslash_gen3_kernel<FMT, RECON, ISIGN, 16, EPI>, dim3((vh + 7) / 8), 128, st, a); break;
    default: launch_pdl(dslash_gen3_kernel<FMT, RECON, ISIGN, 32, EPI>, dim3((vh + 3) / 4), 128, st, a); break;
    }
}

template <int FMT, int RECON, int ISIGN>
void launch_gen4_nrhs(const GenArgs &a, int nrhs, cudaStream_t st) {
    const unsigned vh = (unsigned)a.g.Vh;
    switch (nrhs) {
    case 8: launch_pdl(dslash_gen4_kernel<FMT, RECON, ISIGN, 8>, dim3((vh + 31) / 32), 128, st, a); break;
    case 16: launch_pdl(dslash_gen4_kernel<FMT, RECON, ISIGN, 16>, dim3((vh + 15) / 16), 128, st, a); break;
    default: launch_pdl(dslash_gen4_kernel<FMT, RECON, ISIGN, 32>, dim3((vh + 7) / 8), 128, st, a); break;
    }
}

// Variant 4 (16-bit storage): dynamic shared memory above the 48 KB default,
// allowed once per kernel instance and device before its first launch there.
template <int FMT, int RECON, int ISIGN, int NRHS>
void launch_gen5_one(const GenArgs &a, cudaStream_t st) {
    using SM = G5Smem<FMT, NRHS>;
    auto k = dslash_gen5_kernel<FMT, RECON, ISIGN, NRHS>;
    constexpr int kMaxDev = 64;
    static std::atomic<bool> ready[kMaxDev];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return;  // the error stays the runtime's last error
    if (dev < 0 || dev >= kMaxDev || !ready[dev].load()) {
        if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SM::bytes) != cudaSuccess) return;
        if (dev >= 0 && dev < kMaxDev) ready[dev].store(true);
    }
    const unsigned vh = (unsigned)a.g.Vh;
    launch_pdl_smem(k, dim3((vh + SM::P - 1) / SM::P), 128, SM::bytes, st, a);
}

template <int FMT, int RECON, int ISIGN>
void launch_gen5_nrhs(const GenArgs &a, int nrhs, cudaStream_t st) {
    switch (nrhs) {
    case 8: launch_gen5_one<FMT, RECON, ISIGN, 8>(a, st); break;
    case 16: launch_gen5_one<FMT, RECON, ISIGN, 16>(a, st); break;
    default: launch_gen5_one<FMT, RECON, ISIGN, 32>(a, st); break;
    }
}

template <int FMT>
cudaError_t launch_gen_t(const Geom &g, int recon, int nrhs, const void *gauge, const void *psi, void *res, int isign,
                         int cb, const void *x, float coef, double *partials, cudaStream_t st, int variant = 0) {
    GenArgs a;
    a.g = g;
    a.psi = static_cast<const char *>(psi);
    a.res = static_cast<char *>(res);
    a.gauge = static_cast<const char *>(gauge);
    a.link_block_bytes = (size_t)recon * 4 * g.stride;
    a.cs = (size_t)g.stride * nrhs;
    a.nrhs = nrhs;
    a.pt = 1 - cb;
    a.x = static_cast<const char *>(x);
    a.coef = coef;
    a.partials = partials;
    const long long n = (long long)g.Vh * nrhs;
    const dim3 grid((unsigned)((n + 127) / 128));
    const bool epi = x != nullptr;
    // the xpay epilogue takes nrhs 1 or a power of two up to 32
    if (epi && (nrhs > 32 || (nrhs & (nrhs - 1)) != 0)) return cudaErrorInvalidValue;
    const bool packed_nrhs = nrhs == 8 || nrhs == 16 || nrhs == 32;
    const bool v2 = variant == 1 && packed_nrhs;
    // variant 2 (fully packed, every format: the native FP32 layout holds
    // the reals in order and the pairs are formed in registers; its xpay
    // epilogue serves the batched solver's FP32-pair fields); like variant 1,
    // it falls back to the plain kernel otherwise
    const bool v3 = (variant >= 2 && variant <= 4) && packed_nrhs && (FMT == kFmtF32Pairs || !epi);
    // variant 3: the fully packed kernel with two rhs per thread (no
    // epilogue; with one, variant 2 runs); variant 4: the same with cp.async
    // prefetching (16-bit storage; variant 3 for the FP32 formats)
    const bool v5 = variant == 4 && packed_nrhs && (FMT == kFmtBF16 || FMT == kFmtF16N) && !epi;
    const bool v4 = (variant == 3 || variant == 4) && packed_nrhs && !epi;
#define GBDS_GEN(R, S)                                                   \
    do {                                                                 \
        if constexpr (FMT == kFmtBF16 || FMT == kFmtF16N) {              \
            if (v5) {                                                    \
                launch_gen5_nrhs<FMT, R, S>(a, nrhs, st);                \
                break;                                                   \
            }                                                            \
        }                                                                \
        if (v4) {                                                        \
            launch_gen4_nrhs<FMT, R, S>(a, nrhs, st);                    \
            break;                                                       \
        }                                                                \
        if (v3) {                                                        \
            if constexpr (FMT == kFmtF32Pairs) {                         \
                if (epi) launch_gen3_nrhs<FMT, R, S, 2>(a, nrhs, st);    \
                else launch_gen3_nrhs<FMT, R, S, 0>(a, nrhs, st);        \
            } else {                                                     \
                launch_gen3_nrhs<FMT, R, S, 0>(a, nrhs, st);             \
            }                                                            \
            break;                                                       \
        }                                                                \
        if (v2 && epi) launch_gen2_nrhs<FMT, R, S, 2>(a, nrhs, st);      \
        else if (v2) launch_gen2_nrhs<FMT, R, S, 0>(a, nrhs, st);        \
        else if (epi && nrhs == 1) launch_gen_nrhs<FMT, R, S, 1>(a, nrhs, grid, st);  \
        else if (epi) launch_gen_nrhs<FMT, R, S, 2>(a, nrhs, grid, st);  \
        else launch_gen_nrhs<FMT, R, S, 0>(a, nrhs, grid, st);           \
    } while (0)
    if (recon == 18) { if (isign > 0) GBDS_GEN(18, 1); else GBDS_GEN(18, -1); }
    else             { if (isign > 0) GBDS_GEN(12, 1); else GBDS_GEN(12, -1); }
#undef GBDS_GEN
    count_launch();
    return cudaGetLastError();
}

// The batched CG's fused update (fully packed kernel, FP32 spin pairs, nrhs
// 8, 16 or 32): r -= alpha_r (x + coef D psi) for the active rhs of rsc,
// with per-(128-element block, rhs) |r|^2 partials; nothing else is stored.
template <int FMT>
cudaError_t launch_gen_cg_update_t(const Geom &g, int recon, int nrhs, const void *gauge, const void *psi, int isign,
                                   int cb, const void *x, float coef, const RhsCgScalars *rsc, void *r, double *partials,
                                   cudaStream_t st) {
    if (nrhs != 8 && nrhs != 16 && nrhs != 32) return cudaErrorInvalidValue;
    GenArgs a;
    a.g = g;
    a.psi = static_cast<const char *>(psi);
    a.res = nullptr;
    a.gauge = static_cast<const char *>(gauge);
    a.link_block_bytes = (size_t)recon * 4 * g.stride;
    a.cs = (size_t)g.stride * nrhs;
    a.nrhs = nrhs;
    a.pt = 1 - cb;
    a.x = static_cast<const char *>(x);
    a.coef = coef;
    a.partials = partials;
    a.rsc = rsc;
    a.rvec = static_cast<float4 *>(r);
    if (recon == 18) {
        if (isign > 0) launch_gen3_nrhs<FMT, 18, 1, 3>(a, nrhs, st);
        else launch_gen3_nrhs<FMT, 18, -1, 3>(a, nrhs, st);
    } else {
        if (isign > 0) launch_gen3_nrhs<FMT, 12, 1, 3>(a, nrhs, st);
        else launch_gen3_nrhs<FMT, 12, -1, 3>(a, nrhs, st);
    }
    count_launch();
    return cudaGetLastError();
}

template <int FMT>
cudaError_t launch_pack_gen_t(const Geom &g, int nrhs, const float *packed, const int *table, int parity, void *out,
                              cudaStream_t st) {
    const long long n = (long long)g.Vh * nrhs;
    pack_gen_kernel<FMT><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(packed, table, parity, g, nrhs,
                                                                      (size_t)g.stride * nrhs, static_cast<char *>(out));
    count_launch();
    return cudaGetLastError();
}

template <int FMT>
cudaError_t launch_unpack_gen_t(const Geom &g, int nrhs, const void *in, const int *table, int parity, float *packed,
                                cudaStream_t st) {
    const long long n = (long long)g.Vh * nrhs;
    unpack_gen_kernel<FMT><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(static_cast<const char *>(in), table, parity, g,
                                                                        nrhs, (size_t)g.stride * nrhs, packed);
    count_launch();
    return cudaGetLastError();
}

}  // namespace gbds
