/*
 * sse_config.h -- drop-in configuration header.
 *
 * Selects the real type of the drop-in API the way the reference does
 * (include/sse_config.h:34-41 of the reference): SSE_PRECISION 32 -> float,
 * 64 -> double.  Link against libgbdslash32.so or libgbdslash64.so to match.
 * Defaults to 32 when the including code does not define SSE_PRECISION.
 */
#ifndef SSE_CONFIG_H
#define SSE_CONFIG_H

#ifndef SSE_PRECISION
#ifdef GBDS_SHIM_PREC
#define SSE_PRECISION GBDS_SHIM_PREC
#else
#define SSE_PRECISION 32
#endif
#endif

#if SSE_PRECISION == 32
typedef float SSEREAL;
#elif SSE_PRECISION == 64
typedef double SSEREAL;
#else
#error "SSE_PRECISION must be 32 or 64"
#endif

#endif
