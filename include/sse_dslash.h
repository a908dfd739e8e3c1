/*
 * sse_dslash.h -- drop-in declarations of the reference's 4D Wilson Dslash
 * API (include/sse_dslash.h:13-36 of the reference), implemented on the GPU by
 * libgbdslash32.so (SSEREAL = float) and libgbdslash64.so (double).
 *
 * Behaviour, as in the reference scalar build:
 *  - init is reference counted: a second init only increments the count and
 *    the first lattice stays (lib/sse_su3dslash_32bit_scalar.c:95-99); free
 *    decrements and releases at zero (:126-140).
 *  - every lattice extent must be even; otherwise init prints to stderr and
 *    calls exit(1) (:103-110) (gbds_legacy_set_exit_on_error(0) makes it
 *    return instead).
 *  - the layout callbacks are called during init only; nodeNumber is unused.
 *  - sse_su3dslash_wilson writes the sites of checkerboard 1-cb of res, where
 *    cb is the checkerboard of the source psi (:159-180); sites of
 *    checkerboard cb of res are not touched.  isign = +1 applies D, -1 applies
 *    D^dagger, anything else does nothing.
 *  - u, psi and res are host pointers to the packed arrays:
 *      u   [V][4][3][3][2]  with u[s][mu][j][i] = U_mu(s)_ij
 *      psi [V][4][3][2], res the same, in the caller's linear site order.
 *  - unlike the reference, a call before init prints an error and returns.
 */
#ifndef SSE_DSLASH_H
#define SSE_DSLASH_H

#include "sse_config.h"

#ifdef __cplusplus
extern "C" {
#endif

void init_sse_su3dslash(const int *latt_size,
                        void (*getSiteCoords)(int coord[], int node, int linearsite),
                        int (*getLinearSiteIndex)(const int coord[]),
                        int (*nodeNumber)(const int coord[]));

void free_sse_su3dslash(void);

void sse_su3dslash_wilson(SSEREAL *u, SSEREAL *psi, SSEREAL *res, int isign, int cb);

/* A no-op, as in the reference's scalar build. */
void sse_su3dslash_prepost_receives(void);

/* Gauge reorder from SZIN order u[mu][cb][site] to u_tmp[cb][site][mu]
 * (lib/packer_nopad.c:29-45; volume = sites per checkerboard), and its
 * companion, which copies u_tmp to u index for index (lib/packer_nopad.c:47-69). */
void pack_gauge_field(int volume, SSEREAL (*u)[3][3][2], SSEREAL (*u_tmp)[3][3][2]);
void unpack_gauge_field(int volume, SSEREAL (*u_tmp)[3][3][2], SSEREAL (*u)[3][3][2]);

#ifdef __cplusplus
}
#endif

#endif
