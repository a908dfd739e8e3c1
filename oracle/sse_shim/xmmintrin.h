/*
 * Portable stand-in for <xmmintrin.h> -- TEST INFRASTRUCTURE ONLY.
 *
 * Lets the reference scalar library (the CPU implementation of the Wilson
 * Dslash this project replaces) be compiled from its own sources on hosts
 * without x86 SSE, e.g. the aarch64 (Grace) host of a GB300: oracle/Makefile
 * puts this directory first on the include path, so the reference's
 * `#include <xmmintrin.h>` (include/types32.h, include/types64.h,
 * lib/site_dslash_32bit_scalar.c, lib/site_dslash_64bit_scalar.c) resolves
 * here.
 *
 * It implements only the SSE/SSE2 intrinsics (and the prefetch hint) the
 * reference's scalar build uses, each with the semantics of Intel's published intrinsic definitions,
 * on GCC vector extensions (no x86 instructions, no inline assembly).  Every
 * lane operation is a single IEEE-754 operation in the same order as the SSE
 * instruction; compiled with -ffp-contract=off (no fused multiply-add), the
 * results equal the SSE build's bit for bit, which tests/test_sse_shim.py checks
 * on x86 hosts where both builds exist.
 *
 * Types: __m128 (4 x float), __m128d (2 x double), __m64 (8 bytes).
 */
#ifndef GBDS_SSE_SHIM_XMMINTRIN_H
#define GBDS_SSE_SHIM_XMMINTRIN_H

#if !defined(__GNUC__)
#error "the SSE shim needs GCC vector extensions"
#endif

typedef float __m128 __attribute__((vector_size(16), aligned(16)));
typedef double __m128d __attribute__((vector_size(16), aligned(16)));
typedef int __m64 __attribute__((vector_size(8), aligned(8)));
/* unaligned 8-byte view for the *_pi loads and stores */
typedef float gbds_shim_v2f __attribute__((vector_size(8), aligned(4)));
typedef int gbds_shim_v4i __attribute__((vector_size(16)));
typedef long long gbds_shim_v2l __attribute__((vector_size(16)));

#define GBDS_SHIM_INLINE static __inline__ __attribute__((always_inline, unused))

/* ---- single precision (SSE) ------------------------------------------- */

/* lane-wise a + b, a - b, a * b */
GBDS_SHIM_INLINE __m128 _mm_add_ps(__m128 a, __m128 b) { return a + b; }
GBDS_SHIM_INLINE __m128 _mm_sub_ps(__m128 a, __m128 b) { return a - b; }
GBDS_SHIM_INLINE __m128 _mm_mul_ps(__m128 a, __m128 b) { return a * b; }

/* bitwise exclusive or of the 128 bits (used to flip signs) */
GBDS_SHIM_INLINE __m128 _mm_xor_ps(__m128 a, __m128 b) {
    return (__m128)((gbds_shim_v4i)a ^ (gbds_shim_v4i)b);
}

/* 16-byte aligned load / store of 4 floats */
GBDS_SHIM_INLINE __m128 _mm_load_ps(const float *p) { return *(const __m128 *)p; }
GBDS_SHIM_INLINE void _mm_store_ps(float *p, __m128 a) { *(__m128 *)p = a; }

/* {p[0], 0, 0, 0} */
GBDS_SHIM_INLINE __m128 _mm_load_ss(const float *p) { return (__m128){p[0], 0.0f, 0.0f, 0.0f}; }

/* replace lanes 0,1 (loadl) or 2,3 (loadh) of a by the two floats at p */
GBDS_SHIM_INLINE __m128 _mm_loadl_pi(__m128 a, const __m64 *p) {
    const gbds_shim_v2f v = *(const gbds_shim_v2f *)p;
    return (__m128){v[0], v[1], a[2], a[3]};
}
GBDS_SHIM_INLINE __m128 _mm_loadh_pi(__m128 a, const __m64 *p) {
    const gbds_shim_v2f v = *(const gbds_shim_v2f *)p;
    return (__m128){a[0], a[1], v[0], v[1]};
}

/* store lanes 0,1 (storel) or 2,3 (storeh) of a to the two floats at p */
GBDS_SHIM_INLINE void _mm_storel_pi(__m64 *p, __m128 a) { *(gbds_shim_v2f *)p = (gbds_shim_v2f){a[0], a[1]}; }
GBDS_SHIM_INLINE void _mm_storeh_pi(__m64 *p, __m128 a) { *(gbds_shim_v2f *)p = (gbds_shim_v2f){a[2], a[3]}; }

/* result lanes 0,1 from a, lanes 2,3 from b; lane k takes the element of
 * bits 2k..2k+1 of imm (a compile-time constant) */
#define _mm_shuffle_ps(a, b, imm)                                                                  \
    ((__m128)__builtin_shuffle((__m128)(a), (__m128)(b),                                            \
                               (gbds_shim_v4i){(imm) & 3, ((imm) >> 2) & 3, 4 + (((imm) >> 4) & 3), \
                                               4 + (((imm) >> 6) & 3)}))

/* cache hint for a read of the line holding p (no effect on results):
 * T0 keeps it in every cache level, NTA in none */
#define _MM_HINT_NTA 0
#define _MM_HINT_T2 1
#define _MM_HINT_T1 2
#define _MM_HINT_T0 3
#define _mm_prefetch(p, hint) __builtin_prefetch((const void *)(p), 0, (hint))

/* ---- double precision (SSE2) ------------------------------------------ */

GBDS_SHIM_INLINE __m128d _mm_add_pd(__m128d a, __m128d b) { return a + b; }
GBDS_SHIM_INLINE __m128d _mm_sub_pd(__m128d a, __m128d b) { return a - b; }
GBDS_SHIM_INLINE __m128d _mm_mul_pd(__m128d a, __m128d b) { return a * b; }

GBDS_SHIM_INLINE __m128d _mm_xor_pd(__m128d a, __m128d b) {
    return (__m128d)((gbds_shim_v2l)a ^ (gbds_shim_v2l)b);
}

GBDS_SHIM_INLINE __m128d _mm_load_pd(const double *p) { return *(const __m128d *)p; }
GBDS_SHIM_INLINE void _mm_store_pd(double *p, __m128d a) { *(__m128d *)p = a; }

/* {p[0], 0} */
GBDS_SHIM_INLINE __m128d _mm_load_sd(const double *p) { return (__m128d){p[0], 0.0}; }

/* {a[0], b[0]} */
GBDS_SHIM_INLINE __m128d _mm_unpacklo_pd(__m128d a, __m128d b) { return (__m128d){a[0], b[0]}; }

/* {a[bit 0 of imm], b[bit 1 of imm]} */
#define _mm_shuffle_pd(a, b, imm) \
    ((__m128d)__builtin_shuffle((__m128d)(a), (__m128d)(b), (gbds_shim_v2l){(imm) & 1, 2 + (((imm) >> 1) & 1)}))

#endif /* GBDS_SSE_SHIM_XMMINTRIN_H */
