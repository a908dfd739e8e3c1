/*
 * sse_dslash_3d.h -- drop-in declarations of the reference's spatial (3D)
 * Wilson Dslash API (include/sse_dslash_3d.h:13-33 of the reference).
 *
 * Same contract as sse_dslash.h, with these differences (as in the reference,
 * lib/sse_su3dslash_32bit_scalar_3d.c):
 *  - hops in mu = 0, 1, 2 only; the checkerboard is (x+y+z)&1;
 *  - only extents 0, 1, 2 must be even; the time extent may be odd;
 *  - the gauge array still holds four links per site (the 3D packer keeps
 *    all four mu, lib/qdp_packer_3d.cc:13-22); mu = 3 is not read.
 *  - 4D and 3D have separate state and reference counts.
 */
#ifndef SSE_DSLASH3D_H
#define SSE_DSLASH3D_H

#include "sse_config.h"

#ifdef __cplusplus
extern "C" {
#endif

void init_sse_su3dslash_3d(const int *latt_size,
                           void (*getSiteCoords)(int coord[], int node, int linearsite),
                           int (*getLinearSiteIndex)(const int coord[]),
                           int (*nodeNumber)(const int coord[]));

void free_sse_su3dslash_3d(void);

void sse_su3dslash_wilson_3d(SSEREAL *u, SSEREAL *psi, SSEREAL *res, int isign, int cb);

#ifdef __cplusplus
}
#endif

#endif
