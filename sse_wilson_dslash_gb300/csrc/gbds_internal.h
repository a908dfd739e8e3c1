// Internal declarations shared by the translation units of libgbdslash.so.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <string>

#include "gbdslash.h"

namespace gbds {

// Lattice geometry as the kernels see it.
// 36 bytes: the uneven-batch kernel reads an array of descriptors holding a
// Geom from its parameters by a run-time index, and a larger stride cost it
// register spills and 50 % of its speed.
struct Geom {
    int L[4];      // Lx, Ly, Lz, Lt
    short nd;      // 4 or 3
    short zblock;  // site order of the multi-RHS kernels: z slabs of this
                   // many planes, t swept inside each (0: natural; gen_site)
    int Lxh;       // Lx / 2
    int V;         // full volume
    int Vh;        // sites per checkerboard
    int stride;    // elements between consecutive components of a field
};
static_assert(sizeof(Geom) == 36, "Geom is part of the uneven batch's parameter block");

// Record an error message for gbds_get_last_error() and return `code`.
int set_error(int code, const std::string &msg);
int cuda_error(cudaError_t e, const char *where);
void count_launch(int n = 1);

// Launchers (defined in dslash_f32.cu / dslash_f64.cu / layout.cu).
// All pointers are device pointers; `stream` is a cudaStream_t.
// block: threads per block (0 = default); variant: register-cap variant
// (0 = uncapped; see Variants<T> in dslash_kernel.cuh).
cudaError_t launch_dslash_f32(const Geom &g, int recon, const void *gauge, const void *psi,
                              void *res, int isign, int cb, int block, int variant, cudaStream_t stream);
cudaError_t launch_dslash_f64(const Geom &g, int recon, const void *gauge, const void *psi,
                              void *res, int isign, int cb, int block, int variant, cudaStream_t stream);
int dslash_variants(int prec);

// res = x + coef * Dslash(psi) (4D; res and x on checkerboard 1-cb); if
// partials != nullptr, partials[b] = sum of |res|^2 over launch block b
// (there are (Vh + 127) / 128 blocks).
cudaError_t launch_dslash_xpay_f32(const Geom &g, int recon, const void *gauge, const void *psi, const void *x,
                                   float coef, void *res, double *partials, int isign, int cb, cudaStream_t stream);
cudaError_t launch_dslash_xpay_f64(const Geom &g, int recon, const void *gauge, const void *psi, const void *x,
                                   double coef, void *res, double *partials, int isign, int cb, cudaStream_t stream);

// Double-float (dslash_df.cu, dfloat.cuh): FP64 fields stored as (hi, lo)
// FP32 pairs, 16 bytes a complex as in FP64, computed on the FP32 pipes.
int dslash_variants_df();
cudaError_t launch_dslash_df(const Geom &g, int recon, const void *gauge, const void *psi, void *res, int isign,
                             int cb, int block, int variant, cudaStream_t stream);
cudaError_t launch_dslash_xpay_df(const Geom &g, int recon, const void *gauge, const void *psi, const void *x,
                                  double coef, void *res, double *partials, int isign, int cb, cudaStream_t stream);
// n complex elements FP64 -> double-float; in place allowed
cudaError_t launch_f64_to_df(const void *in, void *out, size_t n, cudaStream_t stream);

// site0: first caller site held by the packed buffer (0 for a full lattice).
// df (prec 64): the internal field is double-float (dfloat.cuh).
cudaError_t launch_pack_spinor(const Geom &g, int prec, const void *psi_packed, const int *site_table,
                               int site0, int parity, void *spinor, cudaStream_t stream, bool df = false);
cudaError_t launch_unpack_spinor(const Geom &g, int prec, const void *spinor, const int *site_table,
                                 int site0, int parity, void *psi_packed, cudaStream_t stream, bool df = false);
cudaError_t launch_pack_gauge(const Geom &g, int prec, int recon, const void *u_packed,
                              const int *site_table, void *gauge, cudaStream_t stream);

// Generalised Dslash (dslash_gen_*.cu): FP32 arithmetic and links, nrhs in
// {1,2,4,8,16,32}, spinor formats 0 FP32, 1 BF16, 2 FP16 + norm, 3 FP32 in
// spin pairs.  x != nullptr selects the xpay epilogue res = x + coef * D psi
// with |res|^2 partials (one per 128-thread block for nrhs 1, one per block
// and rhs otherwise).
// variant 1: the colour multiply in packed FP32x2 arithmetic on links staged
// per CTA (nrhs 8, 16, 32; other counts take variant 0).  variant 2 (formats
// 1, 2, 3): the whole hop in packed FP32x2 (nrhs 8, 16, 32).
cudaError_t launch_gen_f32(const Geom &g, int recon, int nrhs, const void *gauge, const void *psi, void *res, int isign,
                           int cb, const void *x, float coef, double *partials, cudaStream_t st, int variant = 0);
cudaError_t launch_gen_f32p(const Geom &g, int recon, int nrhs, const void *gauge, const void *psi, void *res, int isign,
                            int cb, const void *x, float coef, double *partials, cudaStream_t st, int variant = 0);
cudaError_t launch_gen_half(int fmt, const Geom &g, int recon, int nrhs, const void *gauge, const void *psi, void *res,
                            int isign, int cb, const void *x, float coef, double *partials, cudaStream_t st, int variant = 0);
// packed: FP32 [nrhs][V][4][3][2], caller order
cudaError_t launch_pack_gen_f32(const Geom &g, int nrhs, const float *packed, const int *table, int parity, void *out,
                                cudaStream_t st);
cudaError_t launch_unpack_gen_f32(const Geom &g, int nrhs, const void *in, const int *table, int parity, float *packed,
                                  cudaStream_t st);
cudaError_t launch_pack_gen_f32p(const Geom &g, int nrhs, const float *packed, const int *table, int parity, void *out,
                                 cudaStream_t st);
cudaError_t launch_unpack_gen_f32p(const Geom &g, int nrhs, const void *in, const int *table, int parity, float *packed,
                                   cudaStream_t st);
cudaError_t launch_pack_gen_half(int fmt, const Geom &g, int nrhs, const float *packed, const int *table, int parity,
                                 void *out, cudaStream_t st);
cudaError_t launch_unpack_gen_half(int fmt, const Geom &g, int nrhs, const void *in, const int *table, int parity,
                                   float *packed, cudaStream_t st);
// The batched CG's fused update on FP32 spin pairs (nrhs 8, 16, 32):
// r -= alpha_q (x + coef D psi) for the active rhs q of rsc, per-(128-element
// block, rhs) |r|^2 partials; nothing else is stored.
struct RhsCgScalars;
cudaError_t launch_gen_f32p_cg_update(const Geom &g, int recon, int nrhs, const void *gauge, const void *psi, int isign,
                                      int cb, const void *x, float coef, const RhsCgScalars *rsc, void *r,
                                      double *partials, cudaStream_t st);
inline int gen_spinor_bytes(int fmt) { return (fmt == 0 || fmt == 3) ? 96 : (fmt == 1 ? 48 : 52); }
// z slab of the multi-RHS kernels' site order for nrhs right-hand sides in
// format fmt with recon-real FP32 links (0: the natural order)
int gen_zblock(const Geom &g, int nrhs, int fmt, int recon);
// Tensor-core form (dslash_tc.cu): fmt 1 / 2, nrhs 16 or 32, FP32 links
// converted to the 16-bit operand type; err set to 1 on a timed-out wait.
cudaError_t launch_gen_tc(int fmt, const Geom &g, int recon, int nrhs, const void *gauge, const void *psi, void *res,
                          int isign, int cb, int *err, cudaStream_t st);
// The tensor-core kernel's bounded mbarrier wait on a barrier nothing
// completes; flag = 1 when the wait gave up.
cudaError_t launch_tc_wait_selftest(int polls, int *flag, cudaStream_t st);
// nrhs 1, 16-bit spinors (fmt 1 / 2) with FP16 links: gauge is the FP32
// internal gauge converted by convert_links_f16 (recon * 2 bytes per link
// per site-stride).
cudaError_t launch_gen_h16(int fmt, const Geom &g, int recon, const void *gauge, const void *psi, void *res, int isign,
                           int cb, const void *x, float coef, double *partials, cudaStream_t st);
cudaError_t convert_links_f16(const void *gauge32, void *gauge16, size_t nfloats, cudaStream_t st);

// Sizes in bytes of the internal fields.
size_t spinor_bytes(const Geom &g, int prec);
size_t gauge_bytes(const Geom &g, int prec, int recon);

// Validate dims for an nd-dimensional operator and fill a Geom.
int make_geom(const int dims[4], int nd, Geom *g);

}  // namespace gbds

struct gbds_op_s {
    gbds::Geom g;
    int prec;
    int recon;
    int block;
    int variant;
    int nrhs;    // right-hand sides per site (1 = the plain operator)
    int format;  // spinor storage: 0 native (prec), 1 bfloat16, 2 half + per-spinor norm
    int tensor_cores;  // 16-bit formats, nrhs 16/32: colour multiply on tcgen05
    int *d_err;        // device flag of the tensor-core kernel's bounded waits
    int *d_site_table;  // device copy of the layout table, or nullptr (canonical)
};
