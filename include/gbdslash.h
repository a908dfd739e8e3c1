/*
 * gbdslash.h -- GB300-native Wilson Dslash: extended C ABI.
 *
 * The drop-in libraries libgbdslash32.so / libgbdslash64.so export the
 * reference's own entry points (see sse_dslash.h and sse_dslash_3d.h in this
 * directory).  This header is the layer underneath them, exported by
 * libgbdslash.so:
 *
 *   1. precision-suffixed forms of every reference entry point
 *      (gbds_sse_*_f32 / _f64), so FP32 and FP64 can be used in one process;
 *   2. an operator handle that works on DEVICE pointers and CUDA streams, with
 *      the fields held in the library's structure-of-arrays layout
 *      (described below), optional 12-real gauge compression and status codes;
 *   3. switches for the legacy host-pointer path.
 *
 * Everything is plain C: pointers, ints and sizes.  A CUDA stream is passed
 * as `void*` (a cudaStream_t; NULL = the legacy default stream).
 *
 * Operator (identical to the reference, lib/sse_su3dslash_32bit_scalar.c:39-64):
 *
 *   res(x) = sum_{mu<nd} U_mu(x) (1 - isign g_mu) psi(x+mu)
 *                      + U_mu(x-mu)^dag (1 + isign g_mu) psi(x-mu)
 *
 * on the sites x of checkerboard 1-cb, where cb is the checkerboard of the
 * source, periodic boundaries, DeGrand-Rossi gamma matrices.  nd = 4 uses the
 * 4D parity (x+y+z+t)&1; nd = 3 is the spatial operator with parity
 * (x+y+z)&1 (lib/sse_su3dslash_32bit_scalar_3d.c).
 *
 * Internal layout (one checkerboard of a spinor, "SoA"):
 *   site order within a checkerboard: nd=4: h = ((t*Lz+z)*Ly+y)*(Lx/2) + x/2
 *                                     nd=3: h = t + Lt*(x/2 + (Lx/2)*(y+Ly*z))
 *   FP32: 6 arrays of float4, array k holds reals 4k..4k+3 of the packed
 *         spinor [4 spin][3 colour][2]; element (k, h) at k*stride + h.
 *   FP64: 12 arrays of double2 (one complex each), element (k, h) at
 *         k*stride + h.
 *   stride = gbds_op_stride(): Vh rounded up to a multiple of 64.
 * Gauge field (both checkerboards): block (p, mu) for p in {0,1}, mu < nd, at
 *   offset (p*nd + mu) * C * stride elements, C components per link:
 *   recon 18: 9 complex U_ij (i row, j column), component 3i+j;
 *   recon 12: rows 0 and 1 only (6 complex); row 2 is rebuilt as
 *             conj(row0 x row1) in the kernel (exact for SU(3) links).
 *   FP32 uses float2 per complex for recon 18 and float4 pairs for recon 12;
 *   FP64 uses double2 per complex.
 */
#ifndef GBDSLASH_H
#define GBDSLASH_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBDS_VERSION_MAJOR 0
#define GBDS_VERSION_MINOR 1

/* Status codes returned by the extended API. */
typedef enum gbds_status {
    GBDS_SUCCESS = 0,
    GBDS_ERROR_INVALID_VALUE = 1,   /* bad argument (dims, isign, cb, pointer, size) */
    GBDS_ERROR_NOT_INITIALIZED = 2, /* handle or legacy state not set up            */
    GBDS_ERROR_CUDA = 3,            /* a CUDA runtime call failed                   */
    GBDS_ERROR_OUT_OF_MEMORY = 4,   /* device or pinned host allocation failed      */
    GBDS_ERROR_UNSUPPORTED = 5      /* valid request the library does not implement */
} gbds_status;

/* Storage precisions and gauge compressions. */
#define GBDS_PREC_F32 32
#define GBDS_PREC_F64 64
#define GBDS_RECON_18 18
#define GBDS_RECON_12 12

/* Text of the last error raised on the calling thread ("" if none). */
const char *gbds_get_last_error(void);

/* ------------------------------------------------------------------------ */
/* Operator handle (device pointers)                                         */
/* ------------------------------------------------------------------------ */

typedef struct gbds_op_s *gbds_op;

/* Create an operator for lattice dims[4] = {Lx, Ly, Lz, Lt}.
 * nd = 4: all four dims even; nd = 3: Lx, Ly, Lz even (Lt any >= 1).
 * prec: GBDS_PREC_F32 or GBDS_PREC_F64.  recon: GBDS_RECON_18 or _12.
 * Does not allocate device memory. */
int gbds_op_create(gbds_op *op, const int dims[4], int nd, int prec, int recon);
int gbds_op_destroy(gbds_op op);

/* Storage formats of spinor fields (gbds_op_create_ex). */
#define GBDS_SPINOR_NATIVE 0   /* FP32 float4 or FP64 double2, as prec        */
#define GBDS_SPINOR_BF16 1     /* 24 bfloat16 per spinor (48 B)                */
#define GBDS_SPINOR_F16_NORM 2 /* 24 half scaled by a per-spinor float norm (52 B) */
#define GBDS_SPINOR_F32_PAIRS 3 /* FP32 in spin pairs (96 B): 16-byte component c
                                  * (0..2) = (s0c.r, s1c.r, s0c.i, s1c.i), 3 + c =
                                  * (s2c.r, s3c.r, s2c.i, s3c.i); the operand
                                  * layout of the fully packed kernel (variant 2) */
#define GBDS_SPINOR_DOUBLE_FLOAT 4 /* prec 64, one rhs: every double of the
                                    * spinor and gauge fields held as an
                                    * unevaluated FP32 sum hi + lo (48 of its
                                    * 53 significant bits, FP32 exponent
                                    * range), each complex one 16-byte
                                    * (re.hi, re.lo, im.hi, im.lo) unit in
                                    * the FP64 layout's place; the operator
                                    * runs in double-float arithmetic on the
                                    * FP32 pipes.  pack/unpack take and give
                                    * FP64 arrays. */

/* As gbds_op_create, for nrhs right-hand sides per site (1..32; powers of two
 * have specialised kernels) and a spinor storage format.
 * GBDS_SPINOR_DOUBLE_FLOAT needs prec 64 and nrhs 1 (nd 3 or 4; fields of
 * FP64 size; not for the force or the split-t entry points).  nrhs > 1 or
 * any other format except GBDS_SPINOR_NATIVE needs prec 32 and nd 4;
 * arithmetic is FP32.  A field then holds nrhs spinors per
 * site, element (k, h, r) at k*stride*nrhs + h*nrhs + r (k: 16-byte component,
 * h: site, r: right-hand side), half formats followed by one float norm per
 * (h, r).  pack/unpack take FP32 packed arrays [nrhs][V][4][3][2]; the gauge
 * field is the FP32 one of gbds_op_pack_gauge, shared by all right-hand
 * sides, so each link is read once per site for all nrhs of them. */
int gbds_op_create_ex(gbds_op *op, const int dims[4], int nd, int prec, int recon, int nrhs, int format);
int gbds_op_nrhs(gbds_op op);

/* 16-bit spinor formats with 16 or 32 right-hand sides: do the colour
 * multiply of each hop on the tensor cores (tcgen05.mma, FP32 accumulation in
 * TMEM) for all right-hand sides of a few sites at once; the links enter as
 * bfloat16 (GBDS_SPINOR_BF16) or half (GBDS_SPINOR_F16_NORM) operands.
 * Spin projection and reconstruction stay on the CUDA cores.  gbds_op_check
 * synchronises and reports a tensor-core launch whose bounded wait for its
 * MMAs ran out (it then wrote nothing for those sites). */
int gbds_op_set_tensor_cores(gbds_op op, int on);
int gbds_op_check(gbds_op op);
/* Diagnostic: runs the tensor-core kernel's bounded mbarrier wait, with
 * `polls` polls, on a barrier that nothing completes, then the bounded drain
 * the kernel runs before it releases its tensor memory (4 more waits of
 * `polls` polls), and returns GBDS_SUCCESS when both gave up and reported the
 * code of MMAs that never completed (the context stays usable).  No
 * reference counterpart. */
int gbds_tc_wait_selftest(int polls);

/* Caller site layout for pack/unpack: site_table[i] = caller linear index of
 * internal site i (i = p*Vh + h, internal order above), n = V entries, a
 * permutation of [0, V).  NULL (or the identity) selects the canonical
 * layout, in which the caller's order equals the internal order (QDP++ cb2
 * for nd = 4, cb3d for nd = 3).  Copies the table to the device. */
int gbds_op_set_layout(gbds_op op, const int *site_table, int n);
/* 1 if the operator uses the canonical layout (no permutation). */
int gbds_op_is_canonical(gbds_op op);

size_t gbds_op_spinor_bytes(gbds_op op); /* one checkerboard, internal layout */
size_t gbds_op_gauge_bytes(gbds_op op);  /* both checkerboards                */
int gbds_op_geometry(gbds_op op, int *volume, int *volume_cb, int *stride);

/* Packed (reference layout) device arrays <-> internal layout.
 *   u_packed:   [V][4][3][3][2] reals, u[s][mu][j][i] = U_mu(s)_ij, caller order
 *   psi_packed: [V][4][3][2] reals, caller order (full lattice)
 * pack_spinor reads the sites of checkerboard `parity`; unpack_spinor writes
 * only those sites of psi_packed. */
int gbds_op_pack_gauge(gbds_op op, const void *u_packed, void *gauge, void *stream);
int gbds_op_pack_spinor(gbds_op op, const void *psi_packed, int parity, void *spinor, void *stream);
int gbds_op_unpack_spinor(gbds_op op, const void *spinor, int parity, void *psi_packed, void *stream);

/* res (checkerboard 1-cb) = Dslash psi (checkerboard cb), internal layout.
 * isign +1: D, -1: D^dagger; any other isign is a no-op (returns
 * GBDS_SUCCESS), as in the reference.  cb must be 0 or 1. */
int gbds_op_dslash(gbds_op op, const void *gauge, const void *psi, void *res,
                   int isign, int cb, void *stream);
/* Stream ordering: the Dslash, solver and uneven-batch kernels use
 * programmatic dependent launch.  Each waits (griddepcontrol.wait) for the previous grid on its
 * stream before its first global read, and lets the next grid launched with
 * cudaLaunchAttributeProgrammaticStreamSerialization start early.  Kernels
 * launched without that attribute, copies and events are ordered as usual.
 * A caller kernel launched with the attribute after one of these must itself
 * wait (cudaGridDependencySynchronize) before reading their output. */

/* Launch tuning of gbds_op_dslash: threads per block (0 = default 128; a
 * multiple of 32 up to 256) and a kernel variant.  Single rhs: 0 = registers
 * uncapped; 1.. = variants that cap registers for more resident warps, which
 * launch 128-thread blocks.  Several rhs or 16-bit storage: 0 = the plain
 * multi-RHS kernel, 1 = the packed FP32x2 form (8, 16, 32 rhs; the block
 * size is fixed at 128), 2 = projection, multiply and reconstruction all in
 * packed FP32x2 (8, 16, 32 rhs; 128-thread blocks; every storage format),
 * 3 = variant 2 with two rhs per thread, which share each staged link (the
 * default from 16 rhs on for both FP32 layouts), and for the 16-bit formats
 * 4 = variant 3 with each thread's neighbour spinors prefetched two hops
 * ahead by cp.async into shared memory (their default from 16 rhs on).
 * Variants 1 to 4 run the plain kernel for other counts of rhs (variant 4 on
 * the FP32 formats runs variant 3).
 * gbds_op_num_variants gives the count.  Used by the autotuner. */
int gbds_op_set_tuning(gbds_op op, int threads, int variant);
int gbds_op_get_tuning(gbds_op op, int *threads, int *variant);
int gbds_op_num_variants(gbds_op op);

/* Site order of the multi-RHS CUDA-core kernels (operators with several
 * right-hand sides or 16-bit storage; the tensor-core kernel keeps its own
 * tile order).  zblock = B, a divisor of the z extent: the lattice is swept
 * in z slabs of B (z, t) planes, t outside z within each slab, so that a
 * source spinor's eight reads stay within about 2 B planes and hit L2; 0 or
 * Lz: the natural checkerboard order; -1: the default, the largest slab whose
 * reuse span fits in a fixed share of L2 (natural order when the whole
 * lattice's span fits); gbds_op_autotune times the orders.  Outputs are
 * bit-identical in every order; only the grouping of per-block partial sums
 * (the solver epilogues' norms) follows it.  Storage layouts do not change.
 * get: the slab in use (0 = natural order). */
int gbds_op_set_site_order(gbds_op op, int zblock);
int gbds_op_get_site_order(gbds_op op, int *zblock);

/* Time every (block, variant) candidate of gbds_op_dslash on the caller's
 * fields (res is overwritten), keep the fastest for this operator and cache
 * it process-wide for its (dims, nd, prec, recon, nrhs, format); a later call
 * for the same shape takes the cached choice without timing.  Operators with
 * several right-hand sides (or 16-bit storage) have these candidates: 0 the
 * plain multi-RHS kernel, 1 the colour multiply in packed FP32x2 arithmetic
 * on links staged per CTA (8, 16 or 32 rhs), 2 the whole hop in packed
 * FP32x2 (8, 16, 32 rhs), 3 the same with two rhs per thread, for the 16-bit
 * formats 4 (3 with cp.async prefetching)
 * and, for 16-bit formats with 16 or 32 rhs, the tensor-core kernel
 * (gbds_op_set_tensor_cores); for a CUDA-core pick it then times the site
 * order (gbds_op_set_site_order): the natural order and z slabs of Lz/8
 * planes and up.  Synchronises `stream`. */
int gbds_op_autotune(gbds_op op, const void *gauge, const void *psi, void *res, void *stream);

/* Number of kernels this library has launched in this process (all kinds). */
long long gbds_kernel_launch_count(void);

/* ------------------------------------------------------------------------ */
/* Packed-layout Dslash that allocates nothing                               */
/* ------------------------------------------------------------------------ */
/* No counterpart in the reference.  For callers that must not allocate
 * device memory themselves or have the library do it: code whose device
 * memory belongs to a framework's own pool allocator, code running under a
 * fixed device-memory budget, and latency-critical loops that cannot afford
 * the device-wide synchronisation that cudaFree implies.  Such callers still
 * need the operator on the reference's packed layout, which goes through
 * structure-of-arrays copies of the gauge field and of both spinor
 * checkerboards; here those copies live in one file-scope device array of
 * GBDS_NOALLOC_SCRATCH_BYTES (12 MiB) that every GPU which loads this part of
 * the library holds until the process exits.
 *
 *   u_packed, psi_packed, res_packed: DEVICE pointers, 16-byte aligned, in the
 *     reference's packed layouts (u[V][4][3][3][2], psi/res[V][4][3][2]) and
 *     the QDP++ site order (cb2 for nd = 4, cb3d for nd = 3).
 *   Writes the sites of checkerboard 1-cb of res_packed, like
 *   sse_su3dslash_wilson; isign other than +1/-1 does nothing.
 *   Lattices above GBDS_NOALLOC_MAX_SITES sites are rejected with
 *   GBDS_ERROR_INVALID_VALUE.  No cudaMalloc, cudaFree or other allocating
 *   call is made.
 *   The first call on each device looks up that device's address of the
 *   array (cudaGetSymbolAddress) with the device current; make that first call
 *   before any stream capture.  The address is kept for the life of the
 *   process, so a cudaDeviceReset between calls is not supported.
 *   All calls share the array and it keeps the last call's contents (every
 *   element a call reads it has written first).  Calls that overlap on the
 *   GPU -- different streams, or different host threads -- race on it: issue
 *   them in order on one stream. */
#define GBDS_NOALLOC_MAX_SITES 32768
#define GBDS_NOALLOC_SCRATCH_BYTES 12582912
int gbds_dslash_packed_noalloc_f32(const int dims[4], int nd, const float *u_packed, const float *psi_packed,
                                   float *res_packed, int isign, int cb, void *stream);

/* ------------------------------------------------------------------------ */
/* Uneven batches                                                            */
/* ------------------------------------------------------------------------ */
/* Several lattices -- each with its own size, FP32 gauge field, spinors,
 * number of right-hand sides, isign and cb -- applied by one persistent
 * kernel launch (no counterpart in the reference).  Fields are the internal
 * ones of gbds_op_create_ex(dims, 4, 32, recon, nrhs, format) for the item's
 * dims and nrhs (gauge from gbds_op_pack_gauge, spinors from
 * gbds_op_pack_spinor); recon and format are common to the batch.  The work
 * list (tiles of (site, rhs) pairs) is built at create time; each CTA of the
 * launch walks it with a fixed stride, so no CTA waits on another and the
 * launch can be captured in a CUDA graph (gbds_batch_capture_graph; later
 * gbds_batch_launch calls replay the graph).  Pointers are fixed at create
 * time.  At most 32 lattices per batch (the descriptors travel in the kernel
 * parameters). */
typedef struct gbds_batch_item {
    int dims[4];
    int nrhs;
    int isign;
    int cb;
    const void *gauge;
    const void *psi;
    void *res;
} gbds_batch_item;

typedef struct gbds_batch_s *gbds_batch;

int gbds_batch_create(gbds_batch *b, const gbds_batch_item *items, int n, int recon, int format);
int gbds_batch_destroy(gbds_batch b);
/* Schedule: threads per tile (multiple of 32, <= 256), resident CTAs (0 =
 * one per tile), order 0 (lattice after lattice) or 1 (interleaved). */
int gbds_batch_set_schedule(gbds_batch b, int tile_threads, int resident_ctas, int order);
int gbds_batch_get_schedule(gbds_batch b, int *tile_threads, int *resident_ctas, int *order, int *ntiles);
/* Time the candidate schedules on the batch's own fields (res is overwritten)
 * and keep the fastest.  Drops a captured graph. */
int gbds_batch_autotune(gbds_batch b, void *stream);
int gbds_batch_capture_graph(gbds_batch b, void *stream);
int gbds_batch_launch(gbds_batch b, void *stream);

/* ------------------------------------------------------------------------ */
/* Adjoint and force                                                         */
/* ------------------------------------------------------------------------ */
/* For L = Re <chi, Dslash(isign) psi> (psi: internal field on checkerboard
 * cb, chi: on 1-cb; no counterpart in the reference):
 *   dL/dpsi = Dslash(-isign) chi  -- gbds_op_dslash with -isign, source 1-cb;
 *   dL/dU   -- this call, for every link of the lattice (forward hops own the
 *              links on checkerboard 1-cb, backward hops those on cb):
 *     mode 0: G = dL/dRe U + i dL/dIm U, the complex gradient;
 *     mode 1: F = TA(G U^+), the traceless anti-Hermitian (su(3)) force, so
 *             that along U -> exp(eps X) U, dL/deps = Re tr(F^+ X).
 * Written to force_packed, FP32/FP64 as the operator, in the packed gauge
 * layout [V][4][3][3][2] with f[s][mu][j][i] = R_ij (R = G or F), caller
 * order; accumulate = 1 adds coef * R to it, 0 stores coef * R.
 * Needs a 4D, single right-hand side, native-format, recon 18 operator. */
int gbds_op_force(gbds_op op, const void *gauge, const void *psi, const void *chi, int isign, int cb, int mode,
                  double coef, int accumulate, void *force_packed, void *stream);

/* ------------------------------------------------------------------------ */
/* Time direction split across ranks (domain decomposition)                  */
/* ------------------------------------------------------------------------ */
/* Replaces the reference's parscalar halo exchange
 * (lib/sse_su3dslash_32bit_parscalar.c:967-1095 face buffers, :1203-1284
 * communication overlapped with the interior; lib/shift_tables_parscalar.c).
 * The operator of gbds_op_create is one rank's sub-lattice dims[4], with the
 * global lattice split into equal slabs along t (dims[3] even, so local and
 * global parities agree); x, y and z stay periodic within the rank.  Per
 * application:
 *   1. gbds_op_pack_faces fills the two send buffers from the source psi
 *      (checkerboard cb):
 *        to_prev: (1 - isign g_t) psi on the first local time slice, the
 *                 previous rank's forward t hops (12 reals a face site);
 *        to_next: U_t^+ (1 + isign g_t) psi on the last local time slice,
 *                 the next rank's backward t hops (the sender owns U_t);
 *   2. the caller moves to_prev to the previous rank's from_next and to_next
 *      to the next rank's from_prev (NCCL send/recv, MPI, peer copies; a
 *      single rank passes its own buffers across);
 *   3. gbds_op_dslash_halo computes res on checkerboard 1-cb; part
 *      GBDS_HALO_INTERIOR needs no face and can run while the faces travel,
 *      GBDS_HALO_BOUNDARY then does the first and last time slices,
 *      GBDS_HALO_ALL does both in one launch.
 * Face buffers: gbds_op_face_bytes each, 16-byte aligned, device memory.
 * Needs a 4D, single right-hand side, native-format operator. */
#define GBDS_HALO_ALL 0
#define GBDS_HALO_INTERIOR 1
#define GBDS_HALO_BOUNDARY 2
size_t gbds_op_face_bytes(gbds_op op);
int gbds_op_pack_faces(gbds_op op, const void *gauge, const void *psi, int isign, int cb, void *to_prev,
                       void *to_next, void *stream);
int gbds_op_dslash_halo(gbds_op op, const void *gauge, const void *psi, const void *from_prev, const void *from_next,
                        void *res, int isign, int cb, int part, void *stream);

/* ------------------------------------------------------------------------ */
/* Even-odd preconditioned Wilson solver                                     */
/* ------------------------------------------------------------------------ */
/* M = 1 - kappa^2 D_eo D_oe on checkerboard 0 (even sites), D the operator
 * above (D_oe: cb = 0 source, D_eo: cb = 1 source); M^+ uses isign = -1.
 * CG on A = M^+ M, right-hand side c = M^+ b.  No counterpart in the
 * reference, which provides only D; its callers (Chroma) build M and the
 * solvers around it. */

typedef struct gbds_solver_s *gbds_solver;

typedef struct gbds_solver_params {
    double kappa;     /* hopping parameter */
    double tol;       /* stop when |c - A x| <= tol |c| (FP64) */
    int max_iter;     /* CG iterations, all cycles together */
    int inner_prec;   /* 64: all-FP64 CG; 32: FP32 CG inside FP64 defect correction;
                         16 / 17: as 32 with the CG direction and operator
                         intermediates in half + per-site norm (16) or
                         bfloat16 (17), FP16 links, FP32 arithmetic */
    int inner_recon;  /* 18 or 12: gauge compression of the FP32 operator */
    double inner_tol; /* residual reduction per defect-correction cycle (e.g. 1e-5) */
    int outer_double_float; /* mixed-precision solves: 0 (default) forms the
                               outer residual b - M x with the FP64 operator;
                               1 with the operator in double-float arithmetic
                               on the FP32 pipes (GBDS_SPINOR_DOUBLE_FLOAT:
                               ~1e-14 of |b|, 2.9x the FP64 operator's speed
                               on GB300); fields, update and norms stay FP64,
                               and the FP64 operator still serves sources
                               with |b|^2 outside [1e-50, 1e50] */
} gbds_solver_params;

typedef struct gbds_solver_stats {
    int iterations;       /* CG iterations in total */
    int cycles;           /* defect-correction cycles (1 for FP64 CG) */
    int converged;        /* residual <= tol */
    double residual;      /* |c - A x| / |c| = |M^+ (b - M x)| / |M^+ b|: for the
                             mixed-precision solves b - M x is formed on FP64
                             fields (the FP64 operator, or the double-float one
                             with outer_double_float) and M^+ applied in FP32
                             (FP32 relative accuracy of the residual's own
                             size); FP64 throughout for the FP64 CG and the
                             normal-equation solve */
    double true_residual; /* |b - M x| / |b| on FP64 fields, as above */
    double seconds;       /* wall time of the solve, including its syncs */
} gbds_solver_stats;

/* Allocates its fields on the current device. */
int gbds_solver_create(gbds_solver *s, const int dims[4], const gbds_solver_params *p);
int gbds_solver_destroy(gbds_solver s);
/* u_packed: FP64 device array [V][4][3][3][2] (reference layout, QDP++ cb2
 * order); kept in FP64 for the outer residual and in FP32 for the inner CG. */
int gbds_solver_set_gauge(gbds_solver s, const double *u_packed, void *stream);
/* y = M x (dagger = 0) or M^+ x (dagger = 1) on the even sites of FP64
 * device arrays [V][4][3][2] in cb2 order; odd sites of y are not written. */
int gbds_solver_apply(gbds_solver s, const double *x_packed, double *y_packed, int dagger, void *stream);
/* Solve M x = b on the even sites (b, x as in gbds_solver_apply; x is
 * written on the even sites only; it starts from zero). */
int gbds_solver_solve(gbds_solver s, const double *b_packed, double *x_packed, gbds_solver_stats *stats,
                      void *stream);
/* Solve the normal equations M^+ M x = c directly (c given on the even sites;
 * stats->true_residual then reports |c - M^+ M x| / |c|). */
int gbds_solver_solve_normal(gbds_solver s, const double *c_packed, double *x_packed, gbds_solver_stats *stats,
                             void *stream);

/* Batched solve (no reference counterpart): nrhs (2, 4, 8, 16 or 32)
 * independent systems M x_q = b_q on one gauge field.  The inner FP32 CGs of
 * all right-hand sides advance together on the multi-RHS operator (each link
 * load serves every right-hand side), each with its own scalars and stopping
 * point; the FP64 defect correction runs per right-hand side.  params as for
 * gbds_solver_create with inner_prec 32.  b_packed, x_packed: FP64 device
 * arrays [nrhs][V][4][3][2] (cb2 order, even sites used / written); stats:
 * nrhs entries (seconds: the whole batch). */
typedef struct gbds_bsolver_s *gbds_bsolver;
int gbds_bsolver_create(gbds_bsolver *s, const int dims[4], int nrhs, const gbds_solver_params *p);
int gbds_bsolver_destroy(gbds_bsolver s);
int gbds_bsolver_set_gauge(gbds_bsolver s, const double *u_packed, void *stream);
int gbds_bsolver_solve(gbds_bsolver s, const double *b_packed, double *x_packed, gbds_solver_stats *stats, void *stream);

/* ------------------------------------------------------------------------ */
/* Reference entry points with precision suffixes                            */
/* ------------------------------------------------------------------------ */
/* Same arguments and behaviour as init_sse_su3dslash & co.
 * (include/sse_dslash.h:13-36, include/sse_dslash_3d.h:13-33 of the
 * reference); u, psi and res are HOST pointers in the packed layout. */

void gbds_sse_init_f32(const int *latt_size,
                       void (*getSiteCoords)(int coord[], int node, int linearsite),
                       int (*getLinearSiteIndex)(const int coord[]),
                       int (*nodeNumber)(const int coord[]));
void gbds_sse_free_f32(void);
void gbds_sse_wilson_f32(float *u, float *psi, float *res, int isign, int cb);
void gbds_sse_init_3d_f32(const int *latt_size,
                          void (*getSiteCoords)(int coord[], int node, int linearsite),
                          int (*getLinearSiteIndex)(const int coord[]),
                          int (*nodeNumber)(const int coord[]));
void gbds_sse_free_3d_f32(void);
void gbds_sse_wilson_3d_f32(float *u, float *psi, float *res, int isign, int cb);
void gbds_pack_gauge_field_f32(int volume, float *u, float *u_tmp);
void gbds_unpack_gauge_field_f32(int volume, float *u_tmp, float *u);

void gbds_sse_init_f64(const int *latt_size,
                       void (*getSiteCoords)(int coord[], int node, int linearsite),
                       int (*getLinearSiteIndex)(const int coord[]),
                       int (*nodeNumber)(const int coord[]));
void gbds_sse_free_f64(void);
void gbds_sse_wilson_f64(double *u, double *psi, double *res, int isign, int cb);
void gbds_sse_init_3d_f64(const int *latt_size,
                          void (*getSiteCoords)(int coord[], int node, int linearsite),
                          int (*getLinearSiteIndex)(const int coord[]),
                          int (*nodeNumber)(const int coord[]));
void gbds_sse_free_3d_f64(void);
void gbds_sse_wilson_3d_f64(double *u, double *psi, double *res, int isign, int cb);
void gbds_pack_gauge_field_f64(int volume, double *u, double *u_tmp);
void gbds_unpack_gauge_field_f64(int volume, double *u_tmp, double *u);

/* ------------------------------------------------------------------------ */
/* QDP++ site-order callbacks                                                */
/* ------------------------------------------------------------------------ */
/* Ready-made getSiteCoords / getLinearSiteIndex / nodeNumber for callers of
 * init_sse_su3dslash* that do not link QDP++: they describe the QDP++ cb2
 * order (nd = 4) or cb3d order (nd = 3) of the lattice selected by
 * gbds_layout_select (process-wide; select before the init call that uses
 * them).  With these callbacks the drop-in runs without any permutation. */
int gbds_layout_select(int nd, const int dims[4]);
void gbds_layout_site_coords(int coord[], int node, int linearsite);
int gbds_layout_linear_site_index(const int coord[]);
int gbds_layout_node_number(const int coord[]);

/* ------------------------------------------------------------------------ */
/* Legacy host-pointer path: switches and state                              */
/* ------------------------------------------------------------------------ */

/* On an error in a legacy init (odd dimension, bad layout, allocation
 * failure) the reference prints to stderr and calls exit(1)
 * (lib/sse_su3dslash_32bit_scalar.c:103-110).  That is the default here too;
 * set 0 to print and return instead, leaving the library uninitialised. */
int gbds_legacy_set_exit_on_error(int on);

/* Gauge residency: with 1, a legacy apply whose `u` pointer equals the
 * previous call's skips the host->device copy and repacking of the gauge
 * field.  The caller promises not to change the contents behind that pointer
 * until gbds_legacy_invalidate_gauge() is called.  Default 0 (every call
 * reads `u`, like the reference). */
int gbds_legacy_set_gauge_cache(int on);
int gbds_legacy_invalidate_gauge(void);

/* Gauge compression used by the legacy path (18 = exact copy of the links;
 * 12 = two rows, third rebuilt; only valid for SU(3) links).  Default 18.
 * Takes effect at the next init. */
int gbds_legacy_set_recon(int recon);

/* How the legacy path reaches the caller's host arrays (canonical layouts):
 * 0 (default) - where the GPU can address them (pinned or registered memory,
 *               device or managed memory, or pageable memory on a host whose
 *               pages the GPU translates, as on NVLink-C2C Grace systems) the
 *               layout kernels read u/psi and write res in place;
 *               otherwise as 1;
 * 1           - stage every array through cudaMemcpyAsync. */
int gbds_legacy_set_host_access(int mode);
/* Path taken by the last legacy apply: 1 direct, 0 staged, -1 none yet. */
int gbds_legacy_last_path(void);

/* Refcount of a legacy context: prec 32/64, nd 4/3 (0 = not initialised). */
int gbds_legacy_refcount(int prec, int nd);

#ifdef __cplusplus
}
#endif

#endif /* GBDSLASH_H */
