/*
 * Drop-in shim: exports the reference library's entry points under their own
 * names for one precision, forwarding to libgbdslash.so.  Compiled twice:
 *   -DGBDS_SHIM_PREC=32 -> libgbdslash32.so  (SSEREAL = float)
 *   -DGBDS_SHIM_PREC=64 -> libgbdslash64.so  (SSEREAL = double)
 * as the reference builds liblevel3.a once per precision
 * (configure.ac --enable-precision, include/sse_config.h:34-41).
 */
#include "sse_dslash.h"
#include "sse_dslash_3d.h"
#include "gbdslash.h"

#if GBDS_SHIM_PREC == 32
#define GBDS_FWD(name) name##_f32
#else
#define GBDS_FWD(name) name##_f64
#endif

/* include/sse_dslash.h:13-17 */
void init_sse_su3dslash(const int *latt_size, void (*getSiteCoords)(int coord[], int node, int linearsite),
                        int (*getLinearSiteIndex)(const int coord[]), int (*nodeNumber)(const int coord[]))
{
    GBDS_FWD(gbds_sse_init)(latt_size, getSiteCoords, getLinearSiteIndex, nodeNumber);
}

/* include/sse_dslash.h:20 */
void free_sse_su3dslash(void) { GBDS_FWD(gbds_sse_free)(); }

/* include/sse_dslash.h:32 */
void sse_su3dslash_wilson(SSEREAL *u, SSEREAL *psi, SSEREAL *res, int isign, int cb)
{
    GBDS_FWD(gbds_sse_wilson)(u, psi, res, isign, cb);
}

/* include/sse_dslash.h:36 -- a no-op in the scalar build
 * (lib/sse_su3dslash_32bit_scalar.c:77-80) and here: there is no halo. */
void sse_su3dslash_prepost_receives(void) {}

/* include/sse_dslash_3d.h:13-17 */
void init_sse_su3dslash_3d(const int *latt_size, void (*getSiteCoords)(int coord[], int node, int linearsite),
                           int (*getLinearSiteIndex)(const int coord[]), int (*nodeNumber)(const int coord[]))
{
    GBDS_FWD(gbds_sse_init_3d)(latt_size, getSiteCoords, getLinearSiteIndex, nodeNumber);
}

/* include/sse_dslash_3d.h:21 */
void free_sse_su3dslash_3d(void) { GBDS_FWD(gbds_sse_free_3d)(); }

/* include/sse_dslash_3d.h:33 */
void sse_su3dslash_wilson_3d(SSEREAL *u, SSEREAL *psi, SSEREAL *res, int isign, int cb)
{
    GBDS_FWD(gbds_sse_wilson_3d)(u, psi, res, isign, cb);
}

/* lib/packer_nopad.c:29-45 */
void pack_gauge_field(int volume, SSEREAL (*u)[3][3][2], SSEREAL (*u_tmp)[3][3][2])
{
    GBDS_FWD(gbds_pack_gauge_field)(volume, (SSEREAL *)u, (SSEREAL *)u_tmp);
}

/* lib/packer_nopad.c:47-69 */
void unpack_gauge_field(int volume, SSEREAL (*u_tmp)[3][3][2], SSEREAL (*u)[3][3][2])
{
    GBDS_FWD(gbds_unpack_gauge_field)(volume, (SSEREAL *)u_tmp, (SSEREAL *)u);
}
