// Even-odd preconditioned Wilson solver on one GPU.
//
//   M = 1 - kappa^2 D_eo D_oe   on checkerboard 0 (even sites), D = the
//   Dslash of this library (D_oe: even source -> odd target, cb = 0;
//   D_eo: odd source -> even target, cb = 1); M^+ is the same with isign = -1.
//
// CG on the normal equations A x = c, A = M^+ M, c = M^+ b.
//   inner_prec 64: all-FP64 CG.
//   inner_prec 32: FP32 CG (FP32 fields, FP32 arithmetic, per-block sums in
//                  FP64) inside FP64 defect correction: the residual
//                  r = b - M x, the solution update and all global norms stay
//                  in FP64 on the GPU; the inner right-hand side M^+ r is
//                  formed in FP32 (two FP64 Dslash applications per cycle
//                  instead of four).  The normal-equation solve keeps
//                  r = c - A x in FP64.
//   inner_prec 16 / 17: the same with the CG's direction p and the operator's
//                  intermediates (M p, A p, D_oe p) stored as half with a
//                  per-site norm (16) or bfloat16 (17), FP16 links, FP32
//                  arithmetic; the CG's solution and residual stay FP32.
// The reference library provides only D; a caller such as Chroma builds M and
// its solvers around it (tests/dslashm_w.cc states D the same way).  Scalars
// of the iteration (rr, pAp, alpha, beta) live in device memory and are
// computed by the kernels themselves; the host reads rr only to test
// convergence.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <vector>

#include "dslash_gen.cuh"

namespace gbds {
namespace {

struct Scalars {
    double rr;        // |r|^2 of the running CG
    double pAp;       // <p, A p> = |M p|^2
    double alpha, beta;
    double outer_rr;  // |r|^2 of the FP64 defect-correction residual
    double norm;      // scratch result of a norm
};

constexpr int kThreads = 128;

inline int blocks(const Geom &g) { return (g.Vh + kThreads - 1) / kThreads; }

template <typename T> using SV = typename VecOf<T>::S;  // float4 / double2
template <typename T> constexpr int nvec() { return sizeof(T) == 4 ? 6 : 12; }

__device__ __forceinline__ float4 axpy_v(float a, float4 x, float4 y) {
    return make_float4(fmaf(a, x.x, y.x), fmaf(a, x.y, y.y), fmaf(a, x.z, y.z), fmaf(a, x.w, y.w));
}
__device__ __forceinline__ double2 axpy_v(double a, double2 x, double2 y) {
    return make_double2(fma(a, x.x, y.x), fma(a, x.y, y.y));
}
__device__ __forceinline__ float norm_v(float4 v) { return v.x * v.x + v.y * v.y + v.z * v.z + v.w * v.w; }
__device__ __forceinline__ double norm_v(double2 v) { return v.x * v.x + v.y * v.y; }

// x += alpha p;  r -= alpha Ap;  partial |r|^2
template <typename T>
__global__ void __launch_bounds__(kThreads) cg_update(SV<T> *x, SV<T> *r, const SV<T> *__restrict__ p,
                                                     const SV<T> *__restrict__ Ap, const Scalars *sc, int Vh, int stride,
                                                     double *partials) {
    pdl_allow_next();
    pdl_wait_prev();
    const int h = blockIdx.x * blockDim.x + threadIdx.x;
    T nrm = 0;
    if (h < Vh) {
        const T a = (T)sc->alpha;
#pragma unroll
        for (int k = 0; k < nvec<T>(); k++) {
            const size_t i = (size_t)k * stride + h;
            x[i] = axpy_v(a, p[i], x[i]);
            const SV<T> rn = axpy_v(-a, Ap[i], r[i]);
            r[i] = rn;
            nrm += norm_v(rn);
        }
    }
    block_sum_to<T>(partials, nrm);
}

// p = r + beta p
template <typename T>
__global__ void __launch_bounds__(kThreads) cg_xpay(const SV<T> *__restrict__ r, SV<T> *p, const Scalars *sc, int Vh,
                                                   int stride) {
    pdl_allow_next();
    pdl_wait_prev();
    const int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= Vh) return;
    const T b = (T)sc->beta;
#pragma unroll
    for (int k = 0; k < nvec<T>(); k++) {
        const size_t i = (size_t)k * stride + h;
        p[i] = axpy_v(b, p[i], r[i]);
    }
}

// r = c - v; partial |r|^2  (FP64 defect residual)
__global__ void __launch_bounds__(kThreads) xmy_norm(const double2 *__restrict__ c, const double2 *__restrict__ v,
                                                    double2 *r, int Vh, int stride, double *partials) {
    const int h = blockIdx.x * blockDim.x + threadIdx.x;
    double nrm = 0;
    if (h < Vh) {
#pragma unroll
        for (int k = 0; k < 12; k++) {
            const size_t i = (size_t)k * stride + h;
            const double2 d = make_double2(c[i].x - v[i].x, c[i].y - v[i].y);
            r[i] = d;
            nrm += norm_v(d);
        }
    }
    block_sum_to<double>(partials, nrm);
}

// r = c - v for v in double-float (the outer residual's M x); partial |r|^2
__global__ void __launch_bounds__(kThreads) xmy_norm_df(const double2 *__restrict__ c, const float4 *__restrict__ v,
                                                       double2 *r, int Vh, int stride, double *partials) {
    const int h = blockIdx.x * blockDim.x + threadIdx.x;
    double nrm = 0;
    if (h < Vh) {
#pragma unroll
        for (int k = 0; k < 12; k++) {
            const size_t i = (size_t)k * stride + h;
            const double2 m = df_to_double2(v[i]);
            const double2 d = make_double2(c[i].x - m.x, c[i].y - m.y);
            r[i] = d;
            nrm += norm_v(d);
        }
    }
    block_sum_to<double>(partials, nrm);
}

// partial |v|^2, and optionally dst = v
template <typename T>
__global__ void __launch_bounds__(kThreads) norm_copy(const SV<T> *__restrict__ v, SV<T> *dst, SV<T> *dst2, int Vh,
                                                     int stride, double *partials) {
    const int h = blockIdx.x * blockDim.x + threadIdx.x;
    T nrm = 0;
    if (h < Vh) {
#pragma unroll
        for (int k = 0; k < nvec<T>(); k++) {
            const size_t i = (size_t)k * stride + h;
            const SV<T> a = v[i];
            if (dst) dst[i] = a;
            if (dst2) dst2[i] = a;
            nrm += norm_v(a);
        }
    }
    block_sum_to<T>(partials, nrm);
}

template <typename T>
__global__ void __launch_bounds__(kThreads) zero_field(SV<T> *v, int Vh, int stride) {
    const int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= Vh) return;
    const SV<T> z = {};
#pragma unroll
    for (int k = 0; k < nvec<T>(); k++) v[(size_t)k * stride + h] = z;
}

// r32 = r64 / sqrt(outer_rr);  p32 = r32
__global__ void __launch_bounds__(kThreads) demote_residual(const double2 *__restrict__ r64, float4 *r32, float4 *p32,
                                                           const Scalars *sc, int Vh, int stride) {
    const int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= Vh) return;
    const double s = 1.0 / sqrt(sc->outer_rr);
#pragma unroll
    for (int k = 0; k < 6; k++) {
        const double2 a = r64[(size_t)(2 * k) * stride + h], b = r64[(size_t)(2 * k + 1) * stride + h];
        const float4 f = make_float4((float)(a.x * s), (float)(a.y * s), (float)(b.x * s), (float)(b.y * s));
        r32[(size_t)k * stride + h] = f;
        p32[(size_t)k * stride + h] = f;
    }
}

// x64 += sqrt(outer_rr) * e32
__global__ void __launch_bounds__(kThreads) promote_update(const float4 *__restrict__ e32, double2 *x64,
                                                          const Scalars *sc, int Vh, int stride) {
    const int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= Vh) return;
    const double s = sqrt(sc->outer_rr);
#pragma unroll
    for (int k = 0; k < 6; k++) {
        const float4 e = e32[(size_t)k * stride + h];
        double2 &a = x64[(size_t)(2 * k) * stride + h];
        double2 &b = x64[(size_t)(2 * k + 1) * stride + h];
        a.x = fma(s, (double)e.x, a.x);
        a.y = fma(s, (double)e.y, a.y);
        b.x = fma(s, (double)e.z, b.x);
        b.y = fma(s, (double)e.w, b.y);
    }
}

// r32 = inv * r64
__global__ void __launch_bounds__(kThreads) demote_scaled(const double2 *__restrict__ r64, double inv, float4 *r32,
                                                         int Vh, int stride) {
    const int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= Vh) return;
#pragma unroll
    for (int k = 0; k < 6; k++) {
        const double2 a = r64[(size_t)(2 * k) * stride + h], b = r64[(size_t)(2 * k + 1) * stride + h];
        r32[(size_t)k * stride + h] =
            make_float4((float)(a.x * inv), (float)(a.y * inv), (float)(b.x * inv), (float)(b.y * inv));
    }
}

// r32 = a * v;  p32 = r32
__global__ void __launch_bounds__(kThreads) scale_copy(const float4 *__restrict__ v, float a, float4 *r32, float4 *p32,
                                                      int Vh, int stride) {
    const int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= Vh) return;
#pragma unroll
    for (int k = 0; k < 6; k++) {
        const float4 x = v[(size_t)k * stride + h];
        const float4 y = make_float4(a * x.x, a * x.y, a * x.z, a * x.w);
        r32[(size_t)k * stride + h] = y;
        p32[(size_t)k * stride + h] = y;
    }
}

// x64 += s * e32
__global__ void __launch_bounds__(kThreads) promote_scaled(const float4 *__restrict__ e32, double s, double2 *x64, int Vh,
                                                          int stride) {
    const int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= Vh) return;
#pragma unroll
    for (int k = 0; k < 6; k++) {
        const float4 e = e32[(size_t)k * stride + h];
        double2 &a = x64[(size_t)(2 * k) * stride + h];
        double2 &b = x64[(size_t)(2 * k + 1) * stride + h];
        a.x = fma(s, (double)e.x, a.x);
        a.y = fma(s, (double)e.y, a.y);
        b.x = fma(s, (double)e.z, b.x);
        b.y = fma(s, (double)e.w, b.y);
    }
}

// --- 16-bit direction vectors (Sio formats), FP32 solution and residual ---

// float4 component k of a spinor holds complexes 2k and 2k+1
__device__ __forceinline__ float4 pair(const cx<float> (&s)[4][3], int k) {
    const cx<float> a = s[(2 * k) / 3][(2 * k) % 3], b = s[(2 * k + 1) / 3][(2 * k + 1) % 3];
    return make_float4(a.r, a.i, b.r, b.i);
}

// x += alpha p;  r -= alpha Ap;  partial |r|^2   (p, Ap 16-bit)
template <int FMT>
__global__ void __launch_bounds__(kThreads) cg_update_h(float4 *x, float4 *r, const char *p, const char *Ap,
                                                       const Scalars *sc, int Vh, int stride, double *partials) {
    pdl_allow_next();
    pdl_wait_prev();
    const int h = blockIdx.x * blockDim.x + threadIdx.x;
    float nrm = 0.f;
    if (h < Vh) {
        const float a = (float)sc->alpha;
        cx<float> ps[4][3], aps[4][3];
        Sio<FMT>::load(p, stride, h, ps);
        Sio<FMT>::load(Ap, stride, h, aps);
#pragma unroll
        for (int k = 0; k < 6; k++) {
            const size_t i = (size_t)k * stride + h;
            x[i] = axpy_v(a, pair(ps, k), x[i]);
            const float4 rn = axpy_v(-a, pair(aps, k), r[i]);
            r[i] = rn;
            nrm += norm_v(rn);
        }
    }
    block_sum_to<float>(partials, nrm);
}

// p = r + beta p   (p 16-bit)
template <int FMT>
__global__ void __launch_bounds__(kThreads) cg_xpay_h(const float4 *__restrict__ r, char *p, const Scalars *sc, int Vh,
                                                     int stride) {
    pdl_allow_next();
    pdl_wait_prev();
    const int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= Vh) return;
    const float b = (float)sc->beta;
    cx<float> ps[4][3];
    Sio<FMT>::load(p, stride, h, ps);
#pragma unroll
    for (int k = 0; k < 6; k++) {
        const float4 rv = r[(size_t)k * stride + h];
        cx<float> &u = ps[(2 * k) / 3][(2 * k) % 3];
        cx<float> &v = ps[(2 * k + 1) / 3][(2 * k + 1) % 3];
        u = {fmaf(b, u.r, rv.x), fmaf(b, u.i, rv.y)};
        v = {fmaf(b, v.r, rv.z), fmaf(b, v.i, rv.w)};
    }
    Sio<FMT>::store(p, stride, h, ps);
}

// r32 = r64 / sqrt(outer_rr);  p = r32 (16-bit)
template <int FMT>
__global__ void __launch_bounds__(kThreads) demote_residual_h(const double2 *__restrict__ r64, float4 *r32, char *p,
                                                             const Scalars *sc, int Vh, int stride) {
    const int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= Vh) return;
    const double s = 1.0 / sqrt(sc->outer_rr);
    cx<float> ps[4][3];
#pragma unroll
    for (int k = 0; k < 6; k++) {
        const double2 a = r64[(size_t)(2 * k) * stride + h], b = r64[(size_t)(2 * k + 1) * stride + h];
        const float4 f = make_float4((float)(a.x * s), (float)(a.y * s), (float)(b.x * s), (float)(b.y * s));
        r32[(size_t)k * stride + h] = f;
        ps[(2 * k) / 3][(2 * k) % 3] = {f.x, f.y};
        ps[(2 * k + 1) / 3][(2 * k + 1) % 3] = {f.z, f.w};
    }
    Sio<FMT>::store(p, stride, h, ps);
}

// r32 = a * v;  p = r32 (16-bit)
template <int FMT>
__global__ void __launch_bounds__(kThreads) scale_copy_h(const float4 *__restrict__ v, float a, float4 *r32, char *p,
                                                        int Vh, int stride) {
    const int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= Vh) return;
    cx<float> ps[4][3];
#pragma unroll
    for (int k = 0; k < 6; k++) {
        const float4 x = v[(size_t)k * stride + h];
        const float4 f = make_float4(a * x.x, a * x.y, a * x.z, a * x.w);
        r32[(size_t)k * stride + h] = f;
        ps[(2 * k) / 3][(2 * k) % 3] = {f.x, f.y};
        ps[(2 * k + 1) / 3][(2 * k + 1) % 3] = {f.z, f.w};
    }
    Sio<FMT>::store(p, stride, h, ps);
}

enum FinishMode { kAlpha = 0, kBeta = 1, kSetRR = 2, kOuterRR = 3, kNorm = 4 };

// Deterministic sum of the block partials (fixed order), then the scalar step.
__global__ void __launch_bounds__(1024) finish(const double *partials, int n, Scalars *sc, int mode) {
    pdl_allow_next();
    pdl_wait_prev();
    __shared__ double buf[1024];
    double t = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) t += partials[i];
    buf[threadIdx.x] = t;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) buf[threadIdx.x] += buf[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x != 0) return;
    const double sum = buf[0];
    switch (mode) {
    case kAlpha: sc->pAp = sum; sc->alpha = sum > 0 ? sc->rr / sum : 0.0; break;
    case kBeta: sc->beta = sc->rr > 0 ? sum / sc->rr : 0.0; sc->rr = sum; break;
    case kSetRR: sc->rr = sum; break;
    case kOuterRR: sc->outer_rr = sum; break;
    default: sc->norm = sum; break;
    }
}

__global__ void f64_to_f32(const double *__restrict__ a, float *b, size_t n) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}

}  // namespace
}  // namespace gbds

using namespace gbds;

struct gbds_solver_s {
    Geom g;
    gbds_solver_params prm;
    void *gauge64 = nullptr;  // FP64, recon 18
    void *gauge32 = nullptr;  // FP32, inner recon
    // mixed solves with outer_double_float: the outer residual's operator in
    // double-float (dfloat.cuh) on the FP32 pipes: the links, and the
    // solution converted for it
    void *gauge_df = nullptr, *xdf = nullptr;
    // FP64 fields (checkerboard 0 except t64: checkerboard 1)
    void *b64 = nullptr, *c64 = nullptr, *x64 = nullptr, *r64 = nullptr, *p64 = nullptr, *Ap64 = nullptr,
         *Mp64 = nullptr, *t64 = nullptr;
    // FP32 inner fields
    void *e32 = nullptr, *r32 = nullptr, *p32 = nullptr, *Ap32 = nullptr, *Mp32 = nullptr, *t32 = nullptr;
    // 16-bit inner fields and FP16 links (inner_prec 16 / 17)
    void *p16 = nullptr, *Ap16 = nullptr, *Mp16 = nullptr, *t16 = nullptr, *gauge16 = nullptr;
    int fmt16 = 0;
    double *partials = nullptr;
    Scalars *sc = nullptr;    // device
    Scalars *hsc = nullptr;   // pinned host copy
    bool have_gauge = false;
};

namespace {

// Dslash launches through the precision-specific entry points (the kernels are
// instantiated once, in dslash_f32.cu / dslash_f64.cu).
template <typename T>
cudaError_t dslash(const Geom &g, int recon, const void *gauge, const void *psi, void *res, int isign, int cb,
                   int block, int variant, cudaStream_t st) {
    if constexpr (sizeof(T) == 4) return launch_dslash_f32(g, recon, gauge, psi, res, isign, cb, block, variant, st);
    else return launch_dslash_f64(g, recon, gauge, psi, res, isign, cb, block, variant, st);
}

template <typename T>
cudaError_t dslash_xpay(const Geom &g, int recon, const void *gauge, const void *psi, const void *x, T coef, void *res,
                        double *partials, int isign, int cb, cudaStream_t st) {
    if constexpr (sizeof(T) == 4) return launch_dslash_xpay_f32(g, recon, gauge, psi, x, coef, res, partials, isign, cb, st);
    else return launch_dslash_xpay_f64(g, recon, gauge, psi, x, coef, res, partials, isign, cb, st);
}

cudaError_t finish_on(gbds_solver s, int mode, cudaStream_t st) {
    launch_pdl(finish, dim3(1), 1024, st, s->partials, blocks(s->g), s->sc, mode);
    count_launch();
    return cudaGetLastError();
}

// out_e = in_e - kappa^2 D_eo(isign) D_oe(isign) in_e  (partials: |out|^2)
template <typename T>
cudaError_t apply_M(gbds_solver s, const void *gauge, int recon, const void *in, void *tmp, void *out, int isign,
                    double *partials, cudaStream_t st) {
    const Geom &g = s->g;
    const double k2 = s->prm.kappa * s->prm.kappa;
    const int variant = (sizeof(T) == 4 && recon == 18) ? 1 : 0;
    const int block = (sizeof(T) == 4 && recon == 12) ? 64 : 128;
    cudaError_t e = dslash<T>(g, recon, gauge, in, tmp, isign, 0, block, variant, st);
    if (e != cudaSuccess) return e;
    return dslash_xpay<T>(g, recon, gauge, tmp, in, (T)(-k2), out, partials, isign, 1, st);
}

// The outer residual's operator in double-float (outer_double_float): out
// (double-float, in the storage of an FP64 field) = M in for the FP64 field
// `in`, which is converted into xdf first.  About 48 significant bits: the
// residual b - M x is exact to ~1e-14 |b|, far below the tolerances the
// defect correction reaches, at a fraction of the FP64 operator's time (GB300
// issues FP64 at 1/64 of the FP32 rate).  By default the FP64 operator forms
// the residual.
constexpr int kDfVariant = 0;  // the colour-split kernel (dslash_df.cu)

cudaError_t apply_M_df(gbds_solver s, const void *in64, void *out_df, int isign, cudaStream_t st) {
    const Geom &g = s->g;
    const double k2 = s->prm.kappa * s->prm.kappa;
    cudaError_t e = launch_f64_to_df(in64, s->xdf, spinor_bytes(g, 64) / 16, st);
    if (e == cudaSuccess) e = launch_dslash_df(g, 18, s->gauge_df, s->xdf, s->t64, isign, 0, 128, kDfVariant, st);
    if (e != cudaSuccess) return e;
    return launch_dslash_xpay_df(g, 18, s->gauge_df, s->t64, s->xdf, -k2, out_df, nullptr, isign, 1, st);
}

// Fields within FP32's exponent range (the double-float operator's): |b|^2
// well inside it, else the FP64 operator forms the residual.
bool df_range(double b2) { return b2 > 1e-50 && b2 < 1e50; }

// r = b - M x (FP64 fields), partial |r|^2 in s->partials
cudaError_t outer_residual(gbds_solver s, const void *b64, const void *x64, void *r64, bool df, cudaStream_t st) {
    const Geom &g = s->g;
    const int nb = blocks(g);
    cudaError_t e;
    if (df && s->gauge_df) {
        e = apply_M_df(s, x64, s->Mp64, +1, st);
        if (e != cudaSuccess) return e;
        xmy_norm_df<<<nb, kThreads, 0, st>>>(static_cast<const double2 *>(b64), static_cast<const float4 *>(s->Mp64),
                                             static_cast<double2 *>(r64), g.Vh, g.stride, s->partials);
    } else {
        e = apply_M<double>(s, s->gauge64, 18, x64, s->t64, s->Mp64, +1, nullptr, st);
        if (e != cudaSuccess) return e;
        xmy_norm<<<nb, kThreads, 0, st>>>(static_cast<const double2 *>(b64), static_cast<const double2 *>(s->Mp64),
                                          static_cast<double2 *>(r64), g.Vh, g.stride, s->partials);
    }
    count_launch();
    return cudaGetLastError();
}

// A low-precision inner solve whose residual has not dropped below 0.9 of its
// best value for 96 iterations has reached the accuracy its storage allows:
// the defect correction takes over from there.
bool stagnated(double rr, int k, double &best, int &best_k) {
    if (rr < 0.81 * best) {
        best = rr;
        best_k = k;
        return false;
    }
    return k - best_k >= 96;
}

cudaError_t read_scalars(gbds_solver s, cudaStream_t st) {
    cudaError_t e = cudaMemcpyAsync(s->hsc, s->sc, sizeof(Scalars), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return e;
}

// CG on A = M^+ M with x, r, p prepared (x = 0, r = p = rhs, sc->rr = |rhs|^2).
// Stops when rr <= target_rr or after max_iter iterations.
template <typename T>
cudaError_t cg(gbds_solver s, const void *gauge, int recon, void *x, void *r, void *p, void *Ap, void *Mp, void *t,
               double target_rr, int max_iter, int *iters, cudaStream_t st) {
    const Geom &g = s->g;
    const int nb = blocks(g);
    const int check_every = sizeof(T) == 4 ? 4 : 1;
    cudaError_t e = cudaSuccess;
    int k = 0;
    double best = 1e300;
    int best_k = 0;
    while (k < max_iter) {
        e = apply_M<T>(s, gauge, recon, p, t, Mp, +1, s->partials, st);
        if (e == cudaSuccess) e = finish_on(s, kAlpha, st);
        if (e == cudaSuccess) e = apply_M<T>(s, gauge, recon, Mp, t, Ap, -1, nullptr, st);
        if (e == cudaSuccess) {
            launch_pdl(cg_update<T>, dim3(nb), kThreads, st, static_cast<SV<T> *>(x), static_cast<SV<T> *>(r),
                       static_cast<const SV<T> *>(p), static_cast<const SV<T> *>(Ap), (const Scalars *)s->sc, g.Vh,
                       g.stride, s->partials);
            count_launch();
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = finish_on(s, kBeta, st);
        if (e == cudaSuccess) {
            launch_pdl(cg_xpay<T>, dim3(nb), kThreads, st, static_cast<const SV<T> *>(r), static_cast<SV<T> *>(p),
                       (const Scalars *)s->sc, g.Vh, g.stride);
            count_launch();
            e = cudaGetLastError();
        }
        if (e != cudaSuccess) break;
        k++;
        if (k % check_every == 0 || k == max_iter) {
            e = read_scalars(s, st);
            if (e != cudaSuccess) break;
            if (!(s->hsc->rr > target_rr)) break;  // converged (or NaN: stop)
            if (sizeof(T) == 4 && stagnated(s->hsc->rr, k, best, best_k)) break;
        }
    }
    *iters = k;
    return e;
}

// The 16-bit operator: out = in - kappa^2 D_eo D_oe in, FP16 links.
cudaError_t apply_M_h(gbds_solver s, const void *in, void *tmp, void *out, int isign, double *partials, cudaStream_t st) {
    const Geom &g = s->g;
    const float k2 = (float)(s->prm.kappa * s->prm.kappa);
    cudaError_t e = launch_gen_h16(s->fmt16, g, s->prm.inner_recon, s->gauge16, in, tmp, isign, 0, nullptr, 0.f, nullptr, st);
    if (e != cudaSuccess) return e;
    return launch_gen_h16(s->fmt16, g, s->prm.inner_recon, s->gauge16, tmp, out, isign, 1, in, -k2, partials, st);
}

template <int FMT>
cudaError_t cg_h(gbds_solver s, double target_rr, int max_iter, int *iters, cudaStream_t st) {
    const Geom &g = s->g;
    const int nb = blocks(g);
    cudaError_t e = cudaSuccess;
    int k = 0;
    double best = 1e300;
    int best_k = 0;
    while (k < max_iter) {
        e = apply_M_h(s, s->p16, s->t16, s->Mp16, +1, s->partials, st);
        if (e == cudaSuccess) e = finish_on(s, kAlpha, st);
        if (e == cudaSuccess) e = apply_M_h(s, s->Mp16, s->t16, s->Ap16, -1, nullptr, st);
        if (e == cudaSuccess) {
            launch_pdl(cg_update_h<FMT>, dim3(nb), kThreads, st, static_cast<float4 *>(s->e32),
                       static_cast<float4 *>(s->r32), static_cast<const char *>(s->p16),
                       static_cast<const char *>(s->Ap16), (const Scalars *)s->sc, g.Vh, g.stride, s->partials);
            count_launch();
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = finish_on(s, kBeta, st);
        if (e == cudaSuccess) {
            launch_pdl(cg_xpay_h<FMT>, dim3(nb), kThreads, st, static_cast<const float4 *>(s->r32),
                       static_cast<char *>(s->p16), (const Scalars *)s->sc, g.Vh, g.stride);
            count_launch();
            e = cudaGetLastError();
        }
        if (e != cudaSuccess) break;
        k++;
        if (k % 4 == 0 || k == max_iter) {
            e = read_scalars(s, st);
            if (e != cudaSuccess) break;
            if (!(s->hsc->rr > target_rr)) break;
            if (stagnated(s->hsc->rr, k, best, best_k)) break;
        }
    }
    *iters = k;
    return e;
}

template <typename T>
cudaError_t norm_into(gbds_solver s, const void *v, void *dst, void *dst2, int mode, cudaStream_t st) {
    norm_copy<T><<<blocks(s->g), kThreads, 0, st>>>(static_cast<const SV<T> *>(v), static_cast<SV<T> *>(dst),
                                                     static_cast<SV<T> *>(dst2), s->g.Vh, s->g.stride, s->partials);
    count_launch();
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? finish_on(s, mode, st) : e;
}

template <typename T>
cudaError_t zero(gbds_solver s, void *v, cudaStream_t st) {
    zero_field<T><<<blocks(s->g), kThreads, 0, st>>>(static_cast<SV<T> *>(v), s->g.Vh, s->g.stride);
    count_launch();
    return cudaGetLastError();
}

void release(gbds_solver s) {
    void *bufs[] = {s->gauge64, s->gauge32, s->gauge_df, s->xdf, s->b64, s->c64, s->x64, s->r64, s->p64, s->Ap64,
                    s->Mp64, s->t64,
                    s->e32, s->r32, s->p32, s->Ap32, s->Mp32, s->t32, s->p16, s->Ap16, s->Mp16, s->t16, s->gauge16,
                    s->partials, s->sc};
    for (void *b : bufs)
        if (b) cudaFree(b);
    if (s->hsc) cudaFreeHost(s->hsc);
}

}  // namespace

extern "C" int gbds_solver_create(gbds_solver *out, const int dims[4], const gbds_solver_params *p) {
    if (!out || !p) return set_error(GBDS_ERROR_INVALID_VALUE, "NULL argument");
    *out = nullptr;
    if (p->inner_prec != 64 && p->inner_prec != 32 && p->inner_prec != 16 && p->inner_prec != 17)
        return set_error(GBDS_ERROR_INVALID_VALUE, "inner_prec must be 64, 32, 16 or 17");
    if (p->inner_recon != 18 && p->inner_recon != 12) return set_error(GBDS_ERROR_INVALID_VALUE, "inner_recon must be 18 or 12");
    if (!(p->tol > 0) || p->max_iter <= 0 || !(p->kappa > 0))
        return set_error(GBDS_ERROR_INVALID_VALUE, "tol, max_iter and kappa must be positive");
    Geom g;
    int rc = make_geom(dims, 4, &g);
    if (rc != GBDS_SUCCESS) return rc;
    gbds_solver s = new (std::nothrow) gbds_solver_s;
    if (!s) return set_error(GBDS_ERROR_OUT_OF_MEMORY, "host allocation failed");
    s->g = g;
    s->prm = *p;
    if (!(s->prm.inner_tol > 0 && s->prm.inner_tol < 1)) s->prm.inner_tol = 1e-5;
    const size_t f64 = spinor_bytes(g, 64), f32 = spinor_bytes(g, 32);
    cudaError_t e = cudaSuccess;
    void **d64[] = {&s->b64, &s->c64, &s->x64, &s->r64, &s->p64, &s->Ap64, &s->Mp64, &s->t64};
    for (void **b : d64)
        if (e == cudaSuccess) e = cudaMalloc(b, f64);
    if (p->inner_prec == 32) {
        void **d32[] = {&s->e32, &s->r32, &s->p32, &s->Ap32, &s->Mp32, &s->t32};
        for (void **b : d32)
            if (e == cudaSuccess) e = cudaMalloc(b, f32);
        if (e == cudaSuccess) e = cudaMalloc(&s->gauge32, gauge_bytes(g, 32, p->inner_recon));
    } else if (p->inner_prec == 16 || p->inner_prec == 17) {
        s->fmt16 = p->inner_prec == 16 ? kFmtF16N : kFmtBF16;
        const size_t f16 = (size_t)gen_spinor_bytes(s->fmt16) * g.stride;
        void **d32[] = {&s->e32, &s->r32, &s->Mp32, &s->t32};
        for (void **b : d32)
            if (e == cudaSuccess) e = cudaMalloc(b, f32);
        void **d16[] = {&s->p16, &s->Ap16, &s->Mp16, &s->t16};
        for (void **b : d16)
            if (e == cudaSuccess) e = cudaMalloc(b, f16);
        if (e == cudaSuccess) e = cudaMalloc(&s->gauge32, gauge_bytes(g, 32, p->inner_recon));
        if (e == cudaSuccess) e = cudaMalloc(&s->gauge16, gauge_bytes(g, 32, p->inner_recon) / 2);
    }
    if (e == cudaSuccess) e = cudaMalloc(&s->gauge64, gauge_bytes(g, 64, 18));
    const bool df = p->inner_prec != 64 && p->outer_double_float;
    if (e == cudaSuccess && df) e = cudaMalloc(&s->gauge_df, gauge_bytes(g, 64, 18));
    if (e == cudaSuccess && df) e = cudaMalloc(&s->xdf, f64);
    if (e == cudaSuccess) e = cudaMalloc(&s->partials, sizeof(double) * (size_t)blocks(g));
    if (e == cudaSuccess) e = cudaMalloc(&s->sc, sizeof(Scalars));
    if (e == cudaSuccess) e = cudaMallocHost(&s->hsc, sizeof(Scalars));
    if (e != cudaSuccess) {
        release(s);
        delete s;
        return cuda_error(e, "gbds_solver_create");
    }
    *out = s;
    return GBDS_SUCCESS;
}

extern "C" int gbds_solver_destroy(gbds_solver s) {
    if (!s) return GBDS_SUCCESS;
    cudaDeviceSynchronize();
    release(s);
    delete s;
    return GBDS_SUCCESS;
}

extern "C" int gbds_solver_set_gauge(gbds_solver s, const double *u_packed, void *stream) {
    if (!s) return set_error(GBDS_ERROR_NOT_INITIALIZED, "solver is NULL");
    if (!u_packed || (reinterpret_cast<uintptr_t>(u_packed) & 15u))
        return set_error(GBDS_ERROR_INVALID_VALUE, "u_packed must be a 16-byte aligned device pointer");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = launch_pack_gauge(s->g, 64, 18, u_packed, nullptr, s->gauge64, st);
    if (e == cudaSuccess && s->gauge_df) e = launch_f64_to_df(s->gauge64, s->gauge_df, gauge_bytes(s->g, 64, 18) / 16, st);
    if (e == cudaSuccess && s->prm.inner_prec != 64) {
        const size_t n = (size_t)s->g.V * 72;
        float *tmp = nullptr;
        e = cudaMallocAsync(reinterpret_cast<void **>(&tmp), n * sizeof(float), st);
        if (e == cudaSuccess) {
            f64_to_f32<<<1024, 256, 0, st>>>(u_packed, tmp, n);
            count_launch();
            e = cudaGetLastError();
            if (e == cudaSuccess) e = launch_pack_gauge(s->g, 32, s->prm.inner_recon, tmp, nullptr, s->gauge32, st);
            if (e == cudaSuccess && s->gauge16)
                e = convert_links_f16(s->gauge32, s->gauge16, gauge_bytes(s->g, 32, s->prm.inner_recon) / 4, st);
            cudaFreeAsync(tmp, st);
        }
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_error(e, "gbds_solver_set_gauge");
    s->have_gauge = true;
    return GBDS_SUCCESS;
}

extern "C" int gbds_solver_apply(gbds_solver s, const double *x_packed, double *y_packed, int dagger, void *stream) {
    if (!s) return set_error(GBDS_ERROR_NOT_INITIALIZED, "solver is NULL");
    if (!s->have_gauge) return set_error(GBDS_ERROR_NOT_INITIALIZED, "gbds_solver_set_gauge has not been called");
    if (!x_packed || !y_packed) return set_error(GBDS_ERROR_INVALID_VALUE, "NULL field pointer");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = launch_pack_spinor(s->g, 64, x_packed, nullptr, 0, 0, s->b64, st);
    if (e == cudaSuccess) e = apply_M<double>(s, s->gauge64, 18, s->b64, s->t64, s->Mp64, dagger ? -1 : 1, nullptr, st);
    if (e == cudaSuccess) e = launch_unpack_spinor(s->g, 64, s->Mp64, nullptr, 0, 0, y_packed, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return e == cudaSuccess ? GBDS_SUCCESS : cuda_error(e, "gbds_solver_apply");
}

static int solve_impl(gbds_solver s, const double *b_packed, double *x_packed, gbds_solver_stats *stats, void *stream,
                      bool normal);

extern "C" int gbds_solver_solve(gbds_solver s, const double *b_packed, double *x_packed, gbds_solver_stats *stats,
                                 void *stream) {
    return solve_impl(s, b_packed, x_packed, stats, stream, false);
}

extern "C" int gbds_solver_solve_normal(gbds_solver s, const double *c_packed, double *x_packed, gbds_solver_stats *stats,
                                        void *stream) {
    return solve_impl(s, c_packed, x_packed, stats, stream, true);
}

// Mixed-precision solve of M x = b by defect correction on the true
// residual: each cycle forms r = b - M x in FP64 (two FP64 Dslash
// applications, or the double-float operator with outer_double_float), then
// c = M^+ r in FP32 (the normal-equation right-hand side
// for the inner CG and, through |c|, the stopping test |M^+ (b - M x)| <=
// tol |M^+ b|: the cancellation is in the FP64 subtraction, so |c| carries
// FP32 relative accuracy of its own size), then the inner CG on M^+ M and
// x += |c| e in FP64.
static int solve_mixed(gbds_solver s, const double *b_packed, double *x_packed, gbds_solver_stats *stats,
                       cudaStream_t st, std::chrono::steady_clock::time_point t0) {
    const Geom &g = s->g;
    const int nb = blocks(g);
    const double tol2 = s->prm.tol * s->prm.tol;
    const bool half = s->prm.inner_prec != 32;
    gbds_solver_stats out = {};
    cudaError_t e = launch_pack_spinor(g, 64, b_packed, nullptr, 0, 0, s->b64, st);
    if (e == cudaSuccess) e = norm_into<double>(s, s->b64, s->r64, nullptr, kOuterRR, st);  // r = b
    if (e == cudaSuccess) e = zero<double>(s, s->x64, st);
    if (e == cudaSuccess) e = read_scalars(s, st);
    if (e != cudaSuccess) return cuda_error(e, "gbds_solver_solve");
    const double b2 = s->hsc->outer_rr;
    double r2 = b2;   // |b - M x|^2, FP64
    double c2 = 0;    // |M^+ b|^2
    double n2 = 0;    // |M^+ (b - M x)|^2
    int total = 0;
    bool stop = false;
    while (b2 > 0) {
        // c = M^+ (r / |r|) in FP32 and |c|^2
        demote_scaled<<<nb, kThreads, 0, st>>>(static_cast<const double2 *>(s->r64), 1.0 / std::sqrt(r2),
                                               static_cast<float4 *>(s->r32), g.Vh, g.stride);
        count_launch();
        e = cudaGetLastError();
        if (e == cudaSuccess)
            e = apply_M<float>(s, s->gauge32, s->prm.inner_recon, s->r32, s->t32, s->Mp32, -1, s->partials, st);
        if (e == cudaSuccess) e = finish_on(s, kNorm, st);
        if (e == cudaSuccess) e = read_scalars(s, st);
        if (e != cudaSuccess) break;
        const double s2 = s->hsc->norm;
        n2 = r2 * s2;
        if (out.cycles == 0) c2 = n2;
        if (stop || !(n2 > tol2 * c2) || total >= s->prm.max_iter || !(s2 > 0)) break;
        // inner CG on A e = c / |c|, from e = 0
        const float inv = (float)(1.0 / std::sqrt(s2));
        if (!half)
            scale_copy<<<nb, kThreads, 0, st>>>(static_cast<const float4 *>(s->Mp32), inv, static_cast<float4 *>(s->r32),
                                                static_cast<float4 *>(s->p32), g.Vh, g.stride);
        else if (s->fmt16 == kFmtF16N)
            scale_copy_h<kFmtF16N><<<nb, kThreads, 0, st>>>(static_cast<const float4 *>(s->Mp32), inv,
                                                            static_cast<float4 *>(s->r32), static_cast<char *>(s->p16),
                                                            g.Vh, g.stride);
        else
            scale_copy_h<kFmtBF16><<<nb, kThreads, 0, st>>>(static_cast<const float4 *>(s->Mp32), inv,
                                                            static_cast<float4 *>(s->r32), static_cast<char *>(s->p16),
                                                            g.Vh, g.stride);
        count_launch();
        e = cudaGetLastError();
        if (e == cudaSuccess) e = zero<float>(s, s->e32, st);
        if (e == cudaSuccess) e = norm_into<float>(s, s->r32, nullptr, nullptr, kSetRR, st);
        if (e != cudaSuccess) break;
        double delta = s->prm.inner_tol;
        const double need = 0.5 * s->prm.tol * std::sqrt(c2 / n2);
        if (need > delta) delta = need;
        int it = 0;
        if (!half)
            e = cg<float>(s, s->gauge32, s->prm.inner_recon, s->e32, s->r32, s->p32, s->Ap32, s->Mp32, s->t32,
                          delta * delta, s->prm.max_iter - total, &it, st);
        else if (s->fmt16 == kFmtF16N)
            e = cg_h<kFmtF16N>(s, delta * delta, s->prm.max_iter - total, &it, st);
        else
            e = cg_h<kFmtBF16>(s, delta * delta, s->prm.max_iter - total, &it, st);
        total += it;
        out.cycles++;
        if (e != cudaSuccess) break;
        // x += |c| e (the correction A^-1 M^+ r);  r = b - M x on FP64 fields
        // (the FP64 operator, or the double-float one with outer_double_float)
        promote_scaled<<<nb, kThreads, 0, st>>>(static_cast<const float4 *>(s->e32), std::sqrt(n2),
                                                static_cast<double2 *>(s->x64), g.Vh, g.stride);
        count_launch();
        e = cudaGetLastError();
        if (e == cudaSuccess) e = outer_residual(s, s->b64, s->x64, s->r64, df_range(b2), st);
        if (e == cudaSuccess) e = finish_on(s, kOuterRR, st);
        if (e == cudaSuccess) e = read_scalars(s, st);
        if (e != cudaSuccess) break;
        const double prev = r2;
        r2 = s->hsc->outer_rr;
        if (!(r2 < prev) || !(r2 > 0)) stop = true;  // no progress (or NaN, or exact): measure once more, then stop
    }
    if (e == cudaSuccess) e = launch_unpack_spinor(g, 64, s->x64, nullptr, 0, 0, x_packed, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_error(e, "gbds_solver_solve");
    out.iterations = total;
    out.residual = c2 > 0 ? std::sqrt(n2 / c2) : 0.0;
    out.true_residual = b2 > 0 ? std::sqrt(r2 / b2) : 0.0;
    out.converged = out.residual <= s->prm.tol ? 1 : 0;
    out.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (stats) *stats = out;
    return GBDS_SUCCESS;
}

static int solve_impl(gbds_solver s, const double *b_packed, double *x_packed, gbds_solver_stats *stats, void *stream,
                      bool normal) {
    if (!s) return set_error(GBDS_ERROR_NOT_INITIALIZED, "solver is NULL");
    if (!s->have_gauge) return set_error(GBDS_ERROR_NOT_INITIALIZED, "gbds_solver_set_gauge has not been called");
    if (!b_packed || !x_packed) return set_error(GBDS_ERROR_INVALID_VALUE, "NULL field pointer");
    if ((reinterpret_cast<uintptr_t>(b_packed) | reinterpret_cast<uintptr_t>(x_packed)) & 15u)
        return set_error(GBDS_ERROR_INVALID_VALUE, "fields must be 16-byte aligned");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const auto t0 = std::chrono::steady_clock::now();
    if (!normal && s->prm.inner_prec != 64) return solve_mixed(s, b_packed, x_packed, stats, st, t0);
    gbds_solver_stats out = {};
    const Geom &g = s->g;
    const double tol2 = s->prm.tol * s->prm.tol;
    // b, c = M^+ b, |c|^2
    cudaError_t e = launch_pack_spinor(g, 64, b_packed, nullptr, 0, 0, normal ? s->c64 : s->b64, st);
    if (e == cudaSuccess) {
        if (normal) e = norm_into<double>(s, s->c64, nullptr, nullptr, kOuterRR, st);
        else e = apply_M<double>(s, s->gauge64, 18, s->b64, s->t64, s->c64, -1, s->partials, st);
    }
    if (e == cudaSuccess && !normal) e = finish_on(s, kOuterRR, st);
    if (e == cudaSuccess) e = zero<double>(s, s->x64, st);
    if (e == cudaSuccess) e = read_scalars(s, st);
    if (e != cudaSuccess) return cuda_error(e, "gbds_solver_solve");
    const double c2 = s->hsc->outer_rr;
    double outer_rr = c2;
    int total = 0;
    bool have_residual = false;  // r64 = c - A x and Mp64 = M x are current
    if (c2 > 0) {
        if (s->prm.inner_prec == 64) {
            // all-FP64 CG: r = p = c
            e = norm_into<double>(s, s->c64, s->r64, s->p64, kSetRR, st);
            int it = 0;
            if (e == cudaSuccess)
                e = cg<double>(s, s->gauge64, 18, s->x64, s->r64, s->p64, s->Ap64, s->Mp64, s->t64, tol2 * c2,
                               s->prm.max_iter, &it, st);
            total = it;
            out.cycles = 1;
        } else {
            // FP64 defect correction around FP32 CG; r64 starts as c.
            e = norm_into<double>(s, s->c64, s->r64, nullptr, kOuterRR, st);
            const bool half = s->prm.inner_prec != 32;
            while (e == cudaSuccess && outer_rr > tol2 * c2 && total < s->prm.max_iter) {
                const int nb = blocks(g);
                if (!half) {
                    demote_residual<<<nb, kThreads, 0, st>>>(static_cast<const double2 *>(s->r64),
                                                             static_cast<float4 *>(s->r32), static_cast<float4 *>(s->p32),
                                                             s->sc, g.Vh, g.stride);
                } else if (s->fmt16 == kFmtF16N) {
                    demote_residual_h<kFmtF16N><<<nb, kThreads, 0, st>>>(static_cast<const double2 *>(s->r64),
                                                                         static_cast<float4 *>(s->r32),
                                                                         static_cast<char *>(s->p16), s->sc, g.Vh, g.stride);
                } else {
                    demote_residual_h<kFmtBF16><<<nb, kThreads, 0, st>>>(static_cast<const double2 *>(s->r64),
                                                                         static_cast<float4 *>(s->r32),
                                                                         static_cast<char *>(s->p16), s->sc, g.Vh, g.stride);
                }
                count_launch();
                e = cudaGetLastError();
                if (e == cudaSuccess) e = zero<float>(s, s->e32, st);
                if (e == cudaSuccess) e = norm_into<float>(s, s->r32, nullptr, nullptr, kSetRR, st);
                if (e != cudaSuccess) break;
                // inner target: the requested reduction, but no further than the outer goal needs
                double delta = s->prm.inner_tol;
                const double need = 0.5 * s->prm.tol * std::sqrt(c2 / outer_rr);
                if (need > delta) delta = need;
                int it = 0;
                if (!half)
                    e = cg<float>(s, s->gauge32, s->prm.inner_recon, s->e32, s->r32, s->p32, s->Ap32, s->Mp32, s->t32,
                                  delta * delta, s->prm.max_iter - total, &it, st);
                else if (s->fmt16 == kFmtF16N)
                    e = cg_h<kFmtF16N>(s, delta * delta, s->prm.max_iter - total, &it, st);
                else
                    e = cg_h<kFmtBF16>(s, delta * delta, s->prm.max_iter - total, &it, st);
                total += it;
                out.cycles++;
                if (e != cudaSuccess) break;
                promote_update<<<nb, kThreads, 0, st>>>(static_cast<const float4 *>(s->e32), static_cast<double2 *>(s->x64),
                                                        s->sc, g.Vh, g.stride);
                count_launch();
                e = cudaGetLastError();
                // true residual r = c - A x in FP64
                if (e == cudaSuccess) e = apply_M<double>(s, s->gauge64, 18, s->x64, s->t64, s->Mp64, +1, nullptr, st);
                if (e == cudaSuccess) e = apply_M<double>(s, s->gauge64, 18, s->Mp64, s->t64, s->Ap64, -1, nullptr, st);
                if (e == cudaSuccess) {
                    xmy_norm<<<nb, kThreads, 0, st>>>(static_cast<const double2 *>(s->c64), static_cast<const double2 *>(s->Ap64),
                                                      static_cast<double2 *>(s->r64), g.Vh, g.stride, s->partials);
                    count_launch();
                    e = cudaGetLastError();
                }
                if (e == cudaSuccess) e = finish_on(s, kOuterRR, st);
                if (e == cudaSuccess) e = read_scalars(s, st);
                if (e != cudaSuccess) break;
                have_residual = true;
                const double prev = outer_rr;
                outer_rr = s->hsc->outer_rr;
                if (!(outer_rr < prev)) break;  // no progress (or NaN): stop
            }
        }
    }
    if (e != cudaSuccess) return cuda_error(e, "gbds_solver_solve");
    // FP64 checks: |c - A x| / |c| and |b - M x| / |b|.  The defect-correction
    // loop leaves both r = c - A x (norm in outer_rr) and M x (in Mp64) from
    // its last cycle; the FP64 CG's recursive residual is not the true one, so
    // there they are computed here.
    const int nb = blocks(g);
    double final_rr = outer_rr;
    if (!have_residual) {
        e = apply_M<double>(s, s->gauge64, 18, s->x64, s->t64, s->Mp64, +1, nullptr, st);
        if (e == cudaSuccess) e = apply_M<double>(s, s->gauge64, 18, s->Mp64, s->t64, s->Ap64, -1, nullptr, st);
        if (e == cudaSuccess) {
            xmy_norm<<<nb, kThreads, 0, st>>>(static_cast<const double2 *>(s->c64), static_cast<const double2 *>(s->Ap64),
                                              static_cast<double2 *>(s->r64), g.Vh, g.stride, s->partials);
            count_launch();
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = finish_on(s, kOuterRR, st);
        if (e == cudaSuccess) e = read_scalars(s, st);
        final_rr = s->hsc->outer_rr;
    }
    if (!normal) {
        if (e == cudaSuccess) {
            xmy_norm<<<nb, kThreads, 0, st>>>(static_cast<const double2 *>(s->b64), static_cast<const double2 *>(s->Mp64),
                                              static_cast<double2 *>(s->p64), g.Vh, g.stride, s->partials);
            count_launch();
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = finish_on(s, kNorm, st);
        if (e == cudaSuccess) e = norm_into<double>(s, s->b64, nullptr, nullptr, kOuterRR, st);
        if (e == cudaSuccess) e = read_scalars(s, st);
    } else {
        s->hsc->norm = final_rr;
        s->hsc->outer_rr = c2;
    }
    if (e == cudaSuccess) e = launch_unpack_spinor(g, 64, s->x64, nullptr, 0, 0, x_packed, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_error(e, "gbds_solver_solve");
    out.iterations = total;
    out.residual = c2 > 0 ? std::sqrt(final_rr / c2) : 0.0;
    out.true_residual = s->hsc->outer_rr > 0 ? std::sqrt(s->hsc->norm / s->hsc->outer_rr) : 0.0;
    out.converged = out.residual <= s->prm.tol ? 1 : 0;
    out.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (stats) *stats = out;
    return GBDS_SUCCESS;
}

// ---------------------------------------------------------------------------
// Batched solve: nrhs independent systems M x_k = b_k on one gauge field.
// The inner FP32 CGs of all right-hand sides advance in lockstep on the
// multi-RHS operator (rhs fastest in memory: every link load serves all of
// them), each with its own scalars and its own stopping point; a converged
// right-hand side is masked out of the vector updates.  The FP64 defect
// correction (residual, solution update, norms) is done per right-hand side
// with the FP64 operator.
// ---------------------------------------------------------------------------

namespace gbds {
namespace {

using BScalars = RhsCgScalars;  // rr, pAp, alpha, beta, active (dslash_gen.cuh)

enum BFinish { kBAlpha = 0, kBBeta = 1, kBSetRR = 2 };

// r -= alpha_r Ap;  per-rhs partial |r|^2  (active rhs only; the matching
// x += alpha_r p happens in bcg_xpay, which reads p anyway)
template <int NRHS>
__global__ void __launch_bounds__(128) bcg_update(float4 *r, const float4 *__restrict__ Ap, const BScalars *sc, long long n,
                                                 size_t cs, double *partials) {
    pdl_allow_next();
    pdl_wait_prev();
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int q = (int)(t % NRHS);
    float nrm = 0.f;
    if (t < n && sc[q].active) {
        const float a = (float)sc[q].alpha;
#pragma unroll
        for (int k = 0; k < 6; k++) {
            const size_t i = (size_t)k * cs + (size_t)t;
            const float4 rn = axpy_v(-a, Ap[i], r[i]);
            r[i] = rn;
            nrm += norm_v(rn);
        }
    }
    block_sum_rhs<NRHS>(partials, nrm);
}

// x += alpha_r p;  p = r + beta_r p  (active rhs only)
template <int NRHS>
__global__ void __launch_bounds__(128) bcg_xpay(float4 *x, const float4 *__restrict__ r, float4 *p, const BScalars *sc,
                                               long long n, size_t cs) {
    pdl_allow_next();
    pdl_wait_prev();
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int q = (int)(t % NRHS);
    if (!sc[q].active) return;
    const float a = (float)sc[q].alpha, b = (float)sc[q].beta;
#pragma unroll
    for (int k = 0; k < 6; k++) {
        const size_t i = (size_t)k * cs + (size_t)t;
        const float4 pv = p[i];
        x[i] = axpy_v(a, pv, x[i]);
        p[i] = axpy_v(b, pv, r[i]);
    }
}

// per-rhs partial |v|^2
template <int NRHS>
__global__ void __launch_bounds__(128) bnorm(const float4 *__restrict__ v, long long n, size_t cs, double *partials) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    float nrm = 0.f;
    if (t < n) {
#pragma unroll
        for (int k = 0; k < 6; k++) nrm += norm_v(v[(size_t)k * cs + (size_t)t]);
    }
    block_sum_rhs<NRHS>(partials, nrm);
}

// Per-rhs sums of the (block, rhs) partials in two fixed-order stages.
// Stage 1: block j of the grid sums rows [j*rows, (j+1)*rows) for every rhs
// (thread t takes rhs t % nrhs: coalesced reads) into partials2[j][rhs].
constexpr int kBRows = 1024;  // partial rows per stage-1 block
__global__ void __launch_bounds__(256) bfinish1(const double *partials, int nrows, int nrhs, double *partials2) {
    pdl_allow_next();
    pdl_wait_prev();
    __shared__ double buf[256];
    const int q = threadIdx.x % nrhs, lanes = 256 / nrhs;  // nrhs divides 256
    const int row0 = blockIdx.x * kBRows;
    const int row1 = min(row0 + kBRows, nrows);
    double t = 0;
    for (int i = row0 + threadIdx.x / nrhs; i < row1; i += lanes) t += partials[(size_t)i * nrhs + q];
    buf[threadIdx.x] = t;
    __syncthreads();
    if (threadIdx.x < nrhs) {
        double s = 0;
        for (int j = 0; j < lanes; j++) s += buf[j * nrhs + threadIdx.x];
        partials2[(size_t)blockIdx.x * nrhs + threadIdx.x] = s;
    }
}

// Stage 2: per rhs (thread), the sum over the stage-1 blocks, then the
// scalar step.
__global__ void __launch_bounds__(32) bfinish2(const double *partials2, int nblocks2, int nrhs, BScalars *sc, int mode) {
    pdl_allow_next();
    pdl_wait_prev();
    const int q = threadIdx.x;
    if (q >= nrhs) return;
    double sum = 0;
    for (int j = 0; j < nblocks2; j++) sum += partials2[(size_t)j * nrhs + q];
    BScalars &c = sc[q];
    switch (mode) {
    case kBAlpha:
        if (c.active) {
            c.pAp = sum;
            c.alpha = sum > 0 ? c.rr / sum : 0.0;
        }
        break;
    case kBBeta:
        if (c.active) {
            c.beta = c.rr > 0 ? sum / c.rr : 0.0;
            c.rr = sum;
        }
        break;
    default: c.rr = sum; break;
    }
}

// r = p = scale_q * v (scale in sc[q].beta; zero for inactive rhs)
template <int NRHS>
__global__ void __launch_bounds__(128) bscale_copy(const float4 *__restrict__ v, const BScalars *sc, float4 *r, float4 *p,
                                                  long long n, size_t cs) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int q = (int)(t % NRHS);
    const float a = sc[q].active ? (float)sc[q].beta : 0.f;
#pragma unroll
    for (int k = 0; k < 6; k++) {
        const size_t i = (size_t)k * cs + (size_t)t;
        const float4 x = v[i];
        const float4 y = make_float4(a * x.x, a * x.y, a * x.z, a * x.w);
        r[i] = y;
        p[i] = y;
    }
}

// The per-rhs FP64 fields of all rhs and a scale for each, in the kernel
// parameters (512 bytes).
struct RhsFields {
    double2 *v[32];
    double s[32];
};

// All columns of the multi-RHS inner fields in one launch.  A CTA of 256
// threads takes 32 sites: lane = site (coalesced reads of the per-rhs FP64
// fields), warp w the rhs w, w + 8, ...
constexpr int kBXSites = 32;

// r = p = s_q r64_q (s_q = 1 / |r64_q|), or 0 where s_q = 0; each component
// passes through a [site][rhs] tile in shared memory, so that the
// interleaved (site, rhs) stores are contiguous too
__global__ void __launch_bounds__(256) bdemote_all(const RhsFields f, float4 *r, float4 *p, int Vh, int stride,
                                                  int nrhs, size_t cs) {
    __shared__ float4 tile[kBXSites][33];  // padded: lanes of one rhs hit different banks
    const int base = blockIdx.x * kBXSites;
    const int h = base + (threadIdx.x & 31);
    const int n = min(kBXSites, Vh - base) * nrhs;  // (site, rhs) entries of this CTA
#pragma unroll 1
    for (int k = 0; k < 6; k++) {
        // the inner fields are FP32 spin pairs: float4 k holds complex
        // elements e0 and e0 + 3 (spins 0/1 or 2/3 of colour k % 3) as (e0.r,
        // e1.r, e0.i, e1.i)
        const int e0 = (k < 3 ? 0 : 6) + k % 3;
        if (h < Vh) {
            for (int q = threadIdx.x >> 5; q < nrhs; q += 8) {
                const double inv = f.s[q];
                float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
                if (inv != 0.0) {
                    const double2 *r64 = f.v[q];
                    const double2 a = r64[(size_t)e0 * stride + h], b = r64[(size_t)(e0 + 3) * stride + h];
                    v = make_float4((float)(a.x * inv), (float)(b.x * inv), (float)(a.y * inv), (float)(b.y * inv));
                }
                tile[threadIdx.x & 31][q] = v;
            }
        }
        __syncthreads();
        for (int j = threadIdx.x; j < n; j += blockDim.x) {
            const float4 v = tile[j / nrhs][j % nrhs];
            const size_t i = (size_t)k * cs + (size_t)base * nrhs + j;
            r[i] = v;
            p[i] = v;
        }
        __syncthreads();
    }
}

// x64_q += s_q * column q of e for the rhs with s_q != 0
__global__ void __launch_bounds__(256) bpromote_all(const float4 *__restrict__ e, const RhsFields f, int Vh, int stride,
                                                   int nrhs, size_t cs) {
    const int h = blockIdx.x * kBXSites + (threadIdx.x & 31);
    if (h >= Vh) return;
    for (int q = threadIdx.x >> 5; q < nrhs; q += 8) {
        const double s = f.s[q];
        if (s == 0.0) continue;
        double2 *x64 = f.v[q];
#pragma unroll
        for (int k = 0; k < 6; k++) {
            const int e0 = (k < 3 ? 0 : 6) + k % 3;  // the pair layout, as in bdemote_all
            const float4 v = e[(size_t)k * cs + (size_t)h * nrhs + q];
            double2 &a = x64[(size_t)e0 * stride + h];
            double2 &b = x64[(size_t)(e0 + 3) * stride + h];
            a.x = fma(s, (double)v.x, a.x);
            a.y = fma(s, (double)v.z, a.y);
            b.x = fma(s, (double)v.y, b.x);
            b.y = fma(s, (double)v.w, b.y);
        }
    }
}

}  // namespace
}  // namespace gbds

struct gbds_bsolver_s {
    gbds_solver s1 = nullptr;  // FP64 gauge, FP64 operator temporaries, FP32 links, reductions
    Geom gm{};                 // s1's geometry with the multi-RHS kernels' site order
    int nrhs = 0;
    std::vector<void *> b64, x64, r64;  // per rhs, FP64, checkerboard 0
    void *e = nullptr, *r = nullptr, *p = nullptr, *Ap = nullptr, *Mp = nullptr, *t = nullptr;  // multi-RHS FP32
    double *bpartials = nullptr, *bpartials2 = nullptr;
    BScalars *bsc = nullptr, *hbsc = nullptr;
};

namespace {

long long bcount(gbds_bsolver b) { return (long long)b->s1->g.Vh * b->nrhs; }
int bblocks(gbds_bsolver b) { return (int)((bcount(b) + 127) / 128); }
size_t bcs(gbds_bsolver b) { return (size_t)b->s1->g.stride * b->nrhs; }

#define GBDS_BN(NR, CALL) \
    switch (NR) {         \
    case 2: CALL(2); break; \
    case 4: CALL(4); break; \
    case 8: CALL(8); break; \
    case 16: CALL(16); break; \
    default: CALL(32); break; \
    }

int bblocks2(gbds_bsolver b) { return (bblocks(b) + kBRows - 1) / kBRows; }

cudaError_t bfinish_on(gbds_bsolver b, int mode, cudaStream_t st) {
    launch_pdl(bfinish1, dim3(bblocks2(b)), 256, st, b->bpartials, bblocks(b), b->nrhs, b->bpartials2);
    launch_pdl(bfinish2, dim3(1), 32, st, b->bpartials2, bblocks2(b), b->nrhs, b->bsc, mode);
    count_launch(2);
    return cudaGetLastError();
}

// out = in - kappa^2 D_eo D_oe in for all rhs (partials: per-rhs |out|^2)
cudaError_t apply_Mb(gbds_bsolver b, const void *in, void *out, int isign, double *partials, cudaStream_t st) {
    gbds_solver s = b->s1;
    const float k2 = (float)(s->prm.kappa * s->prm.kappa);
    // inner fields in FP32 spin pairs: the fully packed FP32x2 kernel from 16
    // rhs on (measured faster there), two rhs a thread where there is no
    // epilogue
    const int v = b->nrhs >= 16 ? 2 : 0;
    cudaError_t e = launch_gen_f32p(b->gm, s->prm.inner_recon, b->nrhs, s->gauge32, in, b->t, isign, 0, nullptr, 0.f,
                                    nullptr, st, v ? 3 : 0);
    if (e != cudaSuccess) return e;
    return launch_gen_f32p(b->gm, s->prm.inner_recon, b->nrhs, s->gauge32, b->t, out, isign, 1, in, -k2, partials, st, v);
}

// The fully packed operator (16, 32 rhs) fuses the CG's r -= alpha Ap into
// M^+'s second launch: Ap is never stored.
bool fused_update(gbds_bsolver b) { return b->nrhs == 16 || b->nrhs == 32; }

// r -= alpha_r M^+ in for all active rhs, per-rhs |r|^2 partials
cudaError_t apply_Mb_dagger_update(gbds_bsolver b, const void *in, cudaStream_t st) {
    gbds_solver s = b->s1;
    const float k2 = (float)(s->prm.kappa * s->prm.kappa);
    cudaError_t e =
        launch_gen_f32p(b->gm, s->prm.inner_recon, b->nrhs, s->gauge32, in, b->t, -1, 0, nullptr, 0.f, nullptr, st, 3);
    if (e != cudaSuccess) return e;
    return launch_gen_f32p_cg_update(b->gm, s->prm.inner_recon, b->nrhs, s->gauge32, b->t, -1, 1, in, -k2, b->bsc, b->r,
                                     b->bpartials, st);
}

cudaError_t read_bscalars(gbds_bsolver b, cudaStream_t st) {
    cudaError_t e = cudaMemcpyAsync(b->hbsc, b->bsc, sizeof(BScalars) * b->nrhs, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return e;
}

// Lockstep CG on the active right-hand sides (x = e = 0, r = p = residual,
// rr set); each stops at rr <= target[q] or when it stagnates.
cudaError_t bcg(gbds_bsolver b, const std::vector<double> &target, int max_iter, std::vector<int> &iters,
                cudaStream_t st) {
    const long long n = bcount(b);
    const int nb = bblocks(b);
    const size_t cs = bcs(b);
    const int nr = b->nrhs;
    std::vector<double> best(nr, 1e300);
    std::vector<int> best_k(nr, 0);
    cudaError_t e = read_bscalars(b, st);
    int k = 0;
    while (e == cudaSuccess && k < max_iter) {
        bool any = false;
        for (int q = 0; q < nr; q++) any |= b->hbsc[q].active != 0;
        if (!any) break;
        e = apply_Mb(b, b->p, b->Mp, +1, b->bpartials, st);
        if (e == cudaSuccess) e = bfinish_on(b, kBAlpha, st);
        if (e == cudaSuccess && fused_update(b)) {
            e = apply_Mb_dagger_update(b, b->Mp, st);
        } else if (e == cudaSuccess) {
            e = apply_Mb(b, b->Mp, b->Ap, -1, nullptr, st);
        }
        if (e == cudaSuccess && !fused_update(b)) {
#define GBDS_UPD(NR)                                                                                      \
    launch_pdl(bcg_update<NR>, dim3(nb), 128, st, static_cast<float4 *>(b->r), static_cast<const float4 *>(b->Ap), \
               (const BScalars *)b->bsc, n, cs, b->bpartials)
            GBDS_BN(nr, GBDS_UPD)
#undef GBDS_UPD
            count_launch();
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = bfinish_on(b, kBBeta, st);
        if (e == cudaSuccess) {
#define GBDS_XP(NR)                                                                                         \
    launch_pdl(bcg_xpay<NR>, dim3(nb), 128, st, static_cast<float4 *>(b->e), static_cast<const float4 *>(b->r), \
               static_cast<float4 *>(b->p), (const BScalars *)b->bsc, n, cs)
            GBDS_BN(nr, GBDS_XP)
#undef GBDS_XP
            count_launch();
            e = cudaGetLastError();
        }
        if (e != cudaSuccess) break;
        k++;
        for (int q = 0; q < nr; q++)
            if (b->hbsc[q].active) iters[q]++;
        if (k % 4 == 0 || k == max_iter) {
            e = read_bscalars(b, st);
            if (e != cudaSuccess) break;
            bool changed = false;
            for (int q = 0; q < nr; q++) {
                BScalars &c = b->hbsc[q];
                if (!c.active) continue;
                if (!(c.rr > target[q]) || stagnated(c.rr, k, best[q], best_k[q])) {
                    c.active = 0;  // converged, stagnated or NaN
                    changed = true;
                }
            }
            if (changed) {
                e = cudaMemcpyAsync(b->bsc, b->hbsc, sizeof(BScalars) * nr, cudaMemcpyHostToDevice, st);
                if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            }
        }
    }
    return e;
}

void brelease(gbds_bsolver b) {
    for (auto *v : {&b->b64, &b->x64, &b->r64})
        for (void *p : *v)
            if (p) cudaFree(p);
    void *bufs[] = {b->e, b->r, b->p, b->Ap, b->Mp, b->t, b->bpartials, b->bpartials2, b->bsc};
    for (void *p : bufs)
        if (p) cudaFree(p);
    if (b->hbsc) cudaFreeHost(b->hbsc);
    if (b->s1) gbds_solver_destroy(b->s1);
}

}  // namespace

extern "C" int gbds_bsolver_create(gbds_bsolver *out, const int dims[4], int nrhs, const gbds_solver_params *p) {
    if (!out || !p) return set_error(GBDS_ERROR_INVALID_VALUE, "NULL argument");
    *out = nullptr;
    if (nrhs != 2 && nrhs != 4 && nrhs != 8 && nrhs != 16 && nrhs != 32)
        return set_error(GBDS_ERROR_INVALID_VALUE, "nrhs must be 2, 4, 8, 16 or 32");
    if (p->inner_prec != 32) return set_error(GBDS_ERROR_UNSUPPORTED, "the batched solver runs an FP32 inner CG (inner_prec 32)");
    gbds_bsolver b = new (std::nothrow) gbds_bsolver_s;
    if (!b) return set_error(GBDS_ERROR_OUT_OF_MEMORY, "host allocation failed");
    b->nrhs = nrhs;
    int rc = gbds_solver_create(&b->s1, dims, p);
    if (rc != GBDS_SUCCESS) {
        delete b;
        return rc;
    }
    const Geom &g = b->s1->g;
    b->gm = g;
    b->gm.zblock = gen_zblock(g, nrhs, GBDS_SPINOR_F32_PAIRS, p->inner_recon);
    const size_t f64 = spinor_bytes(g, 64), f32m = spinor_bytes(g, 32) * nrhs;
    cudaError_t e = cudaSuccess;
    for (auto *v : {&b->b64, &b->x64, &b->r64}) {
        v->assign(nrhs, nullptr);
        for (int q = 0; q < nrhs && e == cudaSuccess; q++) e = cudaMalloc(&(*v)[q], f64);
    }
    void **bufs[] = {&b->e, &b->r, &b->p, &b->Mp, &b->t};
    for (void **x : bufs)
        if (e == cudaSuccess) e = cudaMalloc(x, f32m);
    if (e == cudaSuccess && !fused_update(b)) e = cudaMalloc(&b->Ap, f32m);  // else never stored
    if (e == cudaSuccess) e = cudaMalloc(&b->bpartials, sizeof(double) * (size_t)bblocks(b) * nrhs);
    if (e == cudaSuccess) e = cudaMalloc(&b->bpartials2, sizeof(double) * (size_t)bblocks2(b) * nrhs);
    if (e == cudaSuccess) e = cudaMalloc(&b->bsc, sizeof(BScalars) * nrhs);
    if (e == cudaSuccess) e = cudaMallocHost(&b->hbsc, sizeof(BScalars) * nrhs);
    if (e != cudaSuccess) {
        brelease(b);
        delete b;
        return cuda_error(e, "gbds_bsolver_create");
    }
    *out = b;
    return GBDS_SUCCESS;
}

extern "C" int gbds_bsolver_destroy(gbds_bsolver b) {
    if (!b) return GBDS_SUCCESS;
    cudaDeviceSynchronize();
    brelease(b);
    delete b;
    return GBDS_SUCCESS;
}

extern "C" int gbds_bsolver_set_gauge(gbds_bsolver b, const double *u_packed, void *stream) {
    if (!b) return set_error(GBDS_ERROR_NOT_INITIALIZED, "solver is NULL");
    return gbds_solver_set_gauge(b->s1, u_packed, stream);
}

extern "C" int gbds_bsolver_solve(gbds_bsolver b, const double *b_packed, double *x_packed, gbds_solver_stats *stats,
                                  void *stream) {
    if (!b) return set_error(GBDS_ERROR_NOT_INITIALIZED, "solver is NULL");
    gbds_solver s = b->s1;
    if (!s->have_gauge) return set_error(GBDS_ERROR_NOT_INITIALIZED, "gbds_bsolver_set_gauge has not been called");
    if (!b_packed || !x_packed) return set_error(GBDS_ERROR_INVALID_VALUE, "NULL field pointer");
    if ((reinterpret_cast<uintptr_t>(b_packed) | reinterpret_cast<uintptr_t>(x_packed)) & 15u)
        return set_error(GBDS_ERROR_INVALID_VALUE, "fields must be 16-byte aligned");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const auto t0 = std::chrono::steady_clock::now();
    const Geom &g = s->g;
    const int nr = b->nrhs;
    const long long n = bcount(b);
    const size_t cs = bcs(b);
    const double tol2 = s->prm.tol * s->prm.tol;
    const size_t vlen = (size_t)g.V * 24;  // doubles per packed right-hand side
    // per rhs: |b|^2, |b - M x|^2 (FP64), |M^+ b|^2, |M^+ (b - M x)|^2
    std::vector<double> b2(nr, 0.0), r2(nr, 0.0), c2(nr, 0.0), n2(nr, 0.0);
    std::vector<int> iters(nr, 0), cycles(nr, 0);
    std::vector<char> live(nr, 0);  // still being solved
    std::vector<char> last(nr, 0);  // no progress in the last cycle: measure once more, then stop
    cudaError_t e = cudaSuccess;
    for (int q = 0; q < nr && e == cudaSuccess; q++) {
        e = launch_pack_spinor(g, 64, b_packed + q * vlen, nullptr, 0, 0, b->b64[q], st);
        if (e == cudaSuccess) e = norm_into<double>(s, b->b64[q], b->r64[q], nullptr, kOuterRR, st);  // r = b
        if (e == cudaSuccess) e = zero<double>(s, b->x64[q], st);
        if (e == cudaSuccess) e = read_scalars(s, st);
        if (e != cudaSuccess) break;
        b2[q] = r2[q] = s->hsc->outer_rr;
        live[q] = b2[q] > 0;
    }
    int total = 0;
    bool first = true;
    while (e == cudaSuccess) {
        // c_q = M^+ (r_q / |r_q|) in FP32 for all right-hand sides at once, and |c_q|^2
        {
            RhsFields f{};
            for (int q = 0; q < nr; q++) {
                f.v[q] = static_cast<double2 *>(b->r64[q]);
                f.s[q] = live[q] ? 1.0 / std::sqrt(r2[q]) : 0.0;
            }
            bdemote_all<<<(g.Vh + kBXSites - 1) / kBXSites, 256, 0, st>>>(
                f, static_cast<float4 *>(b->r), static_cast<float4 *>(b->p), g.Vh, g.stride, nr, cs);
            count_launch();
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = apply_Mb(b, b->r, b->Mp, -1, b->bpartials, st);
        for (int q = 0; q < nr; q++) b->hbsc[q] = BScalars{};
        if (e == cudaSuccess) e = cudaMemcpyAsync(b->bsc, b->hbsc, sizeof(BScalars) * nr, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = bfinish_on(b, kBSetRR, st);
        if (e == cudaSuccess) e = read_bscalars(b, st);
        if (e != cudaSuccess) break;
        std::vector<double> target(nr, 0.0);
        bool any = false;
        for (int q = 0; q < nr; q++) {
            const double s2 = b->hbsc[q].rr;
            BScalars &c = b->hbsc[q];
            c = BScalars{};
            if (!live[q]) continue;
            n2[q] = r2[q] * s2;
            if (first) c2[q] = n2[q];
            if (last[q] || !(n2[q] > tol2 * c2[q]) || total >= s->prm.max_iter || !(s2 > 0)) {
                live[q] = 0;  // converged, stalled, or nothing left to solve
                continue;
            }
            double delta = s->prm.inner_tol;
            const double need = 0.5 * s->prm.tol * std::sqrt(c2[q] / n2[q]);
            if (need > delta) delta = need;
            target[q] = delta * delta;
            c.active = 1;
            c.beta = 1.0 / std::sqrt(s2);  // scale of the inner right-hand side
            any = true;
        }
        first = false;
        if (!any) break;
        // inner CG on A e_q = c_q / |c_q| from e = 0
        e = cudaMemcpyAsync(b->bsc, b->hbsc, sizeof(BScalars) * nr, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) {
#define GBDS_SC(NR)                                                                                                  \
    bscale_copy<NR><<<bblocks(b), 128, 0, st>>>(static_cast<const float4 *>(b->Mp), b->bsc, static_cast<float4 *>(b->r), \
                                                static_cast<float4 *>(b->p), n, cs)
            GBDS_BN(nr, GBDS_SC)
#undef GBDS_SC
            count_launch();
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaMemsetAsync(b->e, 0, spinor_bytes(g, 32) * nr, st);
        if (e == cudaSuccess) {
#define GBDS_NRM(NR) bnorm<NR><<<bblocks(b), 128, 0, st>>>(static_cast<const float4 *>(b->r), n, cs, b->bpartials)
            GBDS_BN(nr, GBDS_NRM)
#undef GBDS_NRM
            count_launch();
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = bfinish_on(b, kBSetRR, st);
        std::vector<int> it(nr, 0);
        if (e == cudaSuccess) e = bcg(b, target, s->prm.max_iter - total, it, st);
        if (e != cudaSuccess) break;
        int most = 0;
        for (int q = 0; q < nr; q++) {
            if (target[q] == 0.0) continue;
            iters[q] += it[q];
            cycles[q]++;
            most = std::max(most, it[q]);
        }
        total += most;
        // x_q += |c_q| e_q (all rhs in one launch);  r_q = b_q - M x_q in FP64
        {
            RhsFields f{};
            for (int q = 0; q < nr; q++) {
                f.v[q] = static_cast<double2 *>(b->x64[q]);
                f.s[q] = target[q] == 0.0 ? 0.0 : std::sqrt(n2[q]);
            }
            bpromote_all<<<(g.Vh + kBXSites - 1) / kBXSites, 256, 0, st>>>(static_cast<const float4 *>(b->e), f, g.Vh,
                                                                           g.stride, nr, cs);
            count_launch();
            e = cudaGetLastError();
        }
        for (int q = 0; q < nr && e == cudaSuccess; q++) {
            if (target[q] == 0.0) continue;
            e = outer_residual(s, b->b64[q], b->x64[q], b->r64[q], df_range(b2[q]), st);
            if (e == cudaSuccess) e = finish_on(s, kOuterRR, st);
            if (e == cudaSuccess) e = read_scalars(s, st);
            if (e != cudaSuccess) break;
            const double prev = r2[q];
            r2[q] = s->hsc->outer_rr;
            if (!(r2[q] < prev) || !(r2[q] > 0)) last[q] = 1;  // no progress (or NaN, or exact)
        }
    }
    for (int q = 0; q < nr && e == cudaSuccess; q++)
        e = launch_unpack_spinor(g, 64, b->x64[q], nullptr, 0, 0, x_packed + q * vlen, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_error(e, "gbds_bsolver_solve");
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (stats) {
        for (int q = 0; q < nr; q++) {
            gbds_solver_stats &o = stats[q];
            o.iterations = iters[q];
            o.cycles = cycles[q];
            o.residual = c2[q] > 0 ? std::sqrt(n2[q] / c2[q]) : 0.0;
            o.true_residual = b2[q] > 0 ? std::sqrt(r2[q] / b2[q]) : 0.0;
            o.converged = o.residual <= s->prm.tol ? 1 : 0;
            o.seconds = secs;
        }
    }
    return GBDS_SUCCESS;
}
