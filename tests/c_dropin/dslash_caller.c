/*
 * A plain C caller of the drop-in, written the way a QDP++/Chroma code calls
 * the reference (tests/testDslashFull.cc:72-99 of the reference): its own
 * cb2 layout callbacks, init_sse_su3dslash, sse_su3dslash_wilson for every
 * (isign, cb), free_sse_su3dslash.  Built with
 *   cc -DSSE_PRECISION=32|64 -I include dslash_caller.c -lgbdslash32|64
 * Writes u, psi and the four results to the file named by argv[5] (raw
 * SSEREAL arrays, in this order) for the test to compare with the oracle.
 * Usage: dslash_caller Lx Ly Lz Lt out.bin
 */
#include <stdio.h>
#include <stdlib.h>

#include "sse_dslash.h"

static int L[4];

/* QDP++ cb2 order: linear = parity * V/2 + ((t*Lz + z)*Ly + y)*(Lx/2) + x/2 */
static int lin_index(const int c[]) {
    const int V = L[0] * L[1] * L[2] * L[3];
    const int par = (c[0] + c[1] + c[2] + c[3]) & 1;
    return par * (V / 2) + ((c[3] * L[2] + c[2]) * L[1] + c[1]) * (L[0] / 2) + c[0] / 2;
}

static void site_coords(int c[], int node, int linear) {
    (void)node;
    const int Vh = L[0] * L[1] * L[2] * L[3] / 2;
    const int par = linear >= Vh;
    int r = linear - par * Vh;
    const int xh = r % (L[0] / 2);
    r /= L[0] / 2;
    c[1] = r % L[1];
    r /= L[1];
    c[2] = r % L[2];
    c[3] = r / L[2];
    /* x parity makes the site parity come out right */
    c[0] = 2 * xh + ((par + c[1] + c[2] + c[3]) & 1);
}

static int node_number(const int c[]) {
    (void)c;
    return 0;
}

/* deterministic uniform(-1, 1) numbers (64-bit LCG) */
static unsigned long long state = 88172645463325252ULL;
static double uniform(void) {
    state = state * 6364136223846793005ULL + 1442695040888963407ULL;
    return (double)(state >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

int main(int argc, char **argv) {
    if (argc != 6) {
        fprintf(stderr, "usage: %s Lx Ly Lz Lt out.bin\n", argv[0]);
        return 2;
    }
    for (int mu = 0; mu < 4; mu++) L[mu] = atoi(argv[1 + mu]);
    const int V = L[0] * L[1] * L[2] * L[3];
    SSEREAL *u = malloc(sizeof(SSEREAL) * (size_t)V * 72);
    SSEREAL *psi = malloc(sizeof(SSEREAL) * (size_t)V * 24);
    SSEREAL *res = malloc(sizeof(SSEREAL) * (size_t)V * 24 * 4);
    if (!u || !psi || !res) return 3;
    /* any complex 3x3 entries exercise the operator (no unitarity needed) */
    for (size_t i = 0; i < (size_t)V * 72; i++) u[i] = (SSEREAL)uniform();
    for (size_t i = 0; i < (size_t)V * 24; i++) psi[i] = (SSEREAL)uniform();
    for (size_t i = 0; i < (size_t)V * 24 * 4; i++) res[i] = (SSEREAL)0;

    init_sse_su3dslash(L, site_coords, lin_index, node_number);
    int k = 0;
    for (int isign = 1; isign >= -1; isign -= 2)
        for (int cb = 0; cb < 2; cb++, k++) sse_su3dslash_wilson(u, psi, res + (size_t)k * V * 24, isign, cb);
    free_sse_su3dslash();

    FILE *f = fopen(argv[5], "wb");
    if (!f) return 4;
    fwrite(u, sizeof(SSEREAL), (size_t)V * 72, f);
    fwrite(psi, sizeof(SSEREAL), (size_t)V * 24, f);
    fwrite(res, sizeof(SSEREAL), (size_t)V * 24 * 4, f);
    fclose(f);
    free(u);
    free(psi);
    free(res);
    return 0;
}
