/*
 * dslash_oracle.c -- CPU oracle for the Wilson hopping term (Dslash).
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker used by tests/,
 * __graft_entry__.smoke() and the CPU-baseline leg of bench.py.  It is never
 * linked into the product libraries and the product path never calls it.
 *
 * It restates, in plain C, the operator applied by the reference library
 * JeffersonLab/sse_wilson_dslash:
 *
 *   res(x) = sum_mu  U_mu(x)        (1 - isign*gamma_mu) psi(x+mu)
 *                  + U_mu(x-mu)^dag (1 + isign*gamma_mu) psi(x-mu)
 *
 * for every site x of checkerboard 1-cb (cb = checkerboard of the SOURCE),
 * periodic in every direction, mu = 0..3 (4D) or 0..2 (3D, spatial only).
 *   - operator comment block: lib/sse_su3dslash_32bit_scalar.c:39-64
 *   - QDP++ statement of the same operator: tests/dslashm_w.cc:13-123,
 *     tests/dslash_3d_w.cc:9-111
 *   - target checkerboard is 1-cb: lib/sse_su3dslash_32bit_scalar.c:159-180
 *   - packed link layout u[site][mu][j][i] = U_mu(site)_{ij} (the QDP++ packer
 *     stores the transpose): lib/qdp_packer_nopad.cc:7-19, and the 3D packer
 *     keeps all four mu: lib/qdp_packer_3d.cc:13-22
 *   - gamma matrices: DeGrand-Rossi basis, as encoded by the sign/shuffle
 *     masks of lib/site_dslash_32bit_scalar.c:60-171
 *
 * Three restatements live here:
 *   orc_dslash_plain  full 4x4 gamma matrices, FP64, one site at a time; the
 *                     most literal form of the formula above.
 *   orc_dslash_port_* half-spinor projection + SU(3) multiply + reconstruction,
 *                     driven by a site table and neighbour tables built from
 *                     the caller's layout exactly as the reference does
 *                     (lib/shift_tables_scalar.c:191-305,
 *                     lib/shift_tables_scalar_3d.c:207-325), OpenMP over
 *                     sites like lib/dispatch_scalar.c:37-67.  float and
 *                     double arithmetic.  This is the CPU baseline.
 *   layout callbacks  getSiteCoords / getLinearSiteIndex / nodeNumber for the
 *                     QDP++ cb2 (4D), cb3d (3D), lexicographic and arbitrary
 *                     permuted layouts, usable by the reference library and by
 *                     the drop-in library alike.
 */
#include <stdlib.h>
#include <string.h>
#include <stdio.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------ */
/* Canonical site orders                                                     */
/* ------------------------------------------------------------------------ */

/* QDP++ cb2 (4D): lin = p*V/2 + ((t*Lz+z)*Ly+y)*(Lx/2) + x/2,
 * p = (x+y+z+t)&1.  Same order as the reference traversal
 * (lib/shift_tables_scalar.c:99-123, :240-263). */
static int cb2_linear(const int L[4], const int c[4])
{
    int V = L[0] * L[1] * L[2] * L[3];
    int p = (c[0] + c[1] + c[2] + c[3]) & 1;
    return p * (V / 2) + ((c[3] * L[2] + c[2]) * L[1] + c[1]) * (L[0] / 2) + c[0] / 2;
}

static void cb2_coords(const int L[4], int lin, int c[4])
{
    int Vh = L[0] * L[1] * L[2] * L[3] / 2;
    int p = lin / Vh, r = lin % Vh;
    int xh = r % (L[0] / 2); r /= (L[0] / 2);
    c[1] = r % L[1]; r /= L[1];
    c[2] = r % L[2]; r /= L[2];
    c[3] = r;
    c[0] = 2 * xh + ((p + c[1] + c[2] + c[3]) & 1);
}

/* QDP++ cb3d (3D): lin = p3*V/2 + t + Lt*(x/2 + (Lx/2)*(y + Ly*z)),
 * p3 = (x+y+z)&1, t fastest (lib/shift_tables_scalar_3d.c:97-141). */
static int cb3d_linear(const int L[4], const int c[4])
{
    int V = L[0] * L[1] * L[2] * L[3];
    int p = (c[0] + c[1] + c[2]) & 1;
    return p * (V / 2) + c[3] + L[3] * (c[0] / 2 + (L[0] / 2) * (c[1] + L[1] * c[2]));
}

static void cb3d_coords(const int L[4], int lin, int c[4])
{
    int Vh = L[0] * L[1] * L[2] * L[3] / 2;
    int p = lin / Vh, r = lin % Vh;
    c[3] = r % L[3]; r /= L[3];
    int xh = r % (L[0] / 2); r /= (L[0] / 2);
    c[1] = r % L[1]; r /= L[1];
    c[2] = r;
    c[0] = 2 * xh + ((p + c[1] + c[2]) & 1);
}

static int lex_index(const int L[4], const int c[4])
{
    return c[0] + L[0] * (c[1] + L[1] * (c[2] + L[2] * c[3]));
}

static void lex_coords(const int L[4], int lex, int c[4])
{
    c[0] = lex % L[0]; lex /= L[0];
    c[1] = lex % L[1]; lex /= L[1];
    c[2] = lex % L[2]; lex /= L[2];
    c[3] = lex;
}

/* ------------------------------------------------------------------------ */
/* Layout callbacks (one process-wide "current layout")                     */
/* ------------------------------------------------------------------------ */

enum { ORC_LAYOUT_CB2 = 0, ORC_LAYOUT_CB3D = 1, ORC_LAYOUT_LEX = 2, ORC_LAYOUT_PERM = 3 };

static int g_kind = ORC_LAYOUT_CB2;
static int g_L[4] = {2, 2, 2, 2};
static int *g_perm = NULL;      /* lex -> linear (PERM layout) */
static int *g_iperm = NULL;     /* linear -> lex */
static long g_callback_calls = 0;

/* Select the layout the callbacks below describe.  For ORC_LAYOUT_PERM,
 * lin_of_lex[lex] gives the linear index of the lexicographic site lex and
 * must be a permutation of [0, V). Returns 0 on success. */
int orc_layout_set(int kind, const int dims[4], const int *lin_of_lex)
{
    int V = dims[0] * dims[1] * dims[2] * dims[3];
    memcpy(g_L, dims, sizeof(g_L));
    g_kind = kind;
    free(g_perm); free(g_iperm);
    g_perm = g_iperm = NULL;
    if (kind == ORC_LAYOUT_PERM) {
        g_perm = (int *)malloc(sizeof(int) * (size_t)V);
        g_iperm = (int *)malloc(sizeof(int) * (size_t)V);
        if (!g_perm || !g_iperm) return 1;
        for (int i = 0; i < V; i++) g_iperm[i] = -1;
        for (int i = 0; i < V; i++) {
            int l = lin_of_lex[i];
            if (l < 0 || l >= V || g_iperm[l] != -1) return 2;
            g_perm[i] = l;
            g_iperm[l] = i;
        }
    }
    g_callback_calls = 0;
    return 0;
}

long orc_layout_callback_calls(void) { return g_callback_calls; }

int orc_get_linear_site_index(const int coord[])
{
    g_callback_calls++;
    switch (g_kind) {
    case ORC_LAYOUT_CB2: return cb2_linear(g_L, coord);
    case ORC_LAYOUT_CB3D: return cb3d_linear(g_L, coord);
    case ORC_LAYOUT_LEX: return lex_index(g_L, coord);
    default: return g_perm[lex_index(g_L, coord)];
    }
}

void orc_get_site_coords(int coord[], int node, int linear)
{
    (void)node;
    g_callback_calls++;
    switch (g_kind) {
    case ORC_LAYOUT_CB2: cb2_coords(g_L, linear, coord); break;
    case ORC_LAYOUT_CB3D: cb3d_coords(g_L, linear, coord); break;
    case ORC_LAYOUT_LEX: lex_coords(g_L, linear, coord); break;
    default: lex_coords(g_L, g_iperm[linear], coord); break;
    }
}

int orc_node_number(const int coord[]) { (void)coord; return 0; }

/* Fill lin_of_lex[V] for a layout kind (CB2, CB3D, LEX). */
void orc_layout_table(int kind, const int dims[4], int *lin_of_lex)
{
    int V = dims[0] * dims[1] * dims[2] * dims[3];
    for (int lex = 0; lex < V; lex++) {
        int c[4];
        lex_coords(dims, lex, c);
        lin_of_lex[lex] = kind == ORC_LAYOUT_CB2 ? cb2_linear(dims, c)
                        : kind == ORC_LAYOUT_CB3D ? cb3d_linear(dims, c)
                        : lex;
    }
}

/* ------------------------------------------------------------------------ */
/* Plain FP64 restatement with full gamma matrices                           */
/* ------------------------------------------------------------------------ */

typedef struct { double re, im; } cplx;

static inline cplx cmul(cplx a, cplx b) { cplx r = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; return r; }
static inline cplx cadd(cplx a, cplx b) { cplx r = {a.re + b.re, a.im + b.im}; return r; }
static inline cplx conjc(cplx a) { cplx r = {a.re, -a.im}; return r; }

/* gamma[mu][row][col], DeGrand-Rossi basis. */
static const cplx GAMMA[4][4][4] = {
    /* gamma_0: (0,3)=i (1,2)=i (2,1)=-i (3,0)=-i */
    {{{0,0},{0,0},{0,0},{0,1}}, {{0,0},{0,0},{0,1},{0,0}}, {{0,0},{0,-1},{0,0},{0,0}}, {{0,-1},{0,0},{0,0},{0,0}}},
    /* gamma_1: (0,3)=-1 (1,2)=1 (2,1)=1 (3,0)=-1 */
    {{{0,0},{0,0},{0,0},{-1,0}}, {{0,0},{0,0},{1,0},{0,0}}, {{0,0},{1,0},{0,0},{0,0}}, {{-1,0},{0,0},{0,0},{0,0}}},
    /* gamma_2: (0,2)=i (1,3)=-i (2,0)=-i (3,1)=i */
    {{{0,0},{0,0},{0,1},{0,0}}, {{0,0},{0,0},{0,0},{0,-1}}, {{0,-1},{0,0},{0,0},{0,0}}, {{0,0},{0,1},{0,0},{0,0}}},
    /* gamma_3: (0,2)=1 (1,3)=1 (2,0)=1 (3,1)=1 */
    {{{0,0},{0,0},{1,0},{0,0}}, {{0,0},{0,0},{0,0},{1,0}}, {{1,0},{0,0},{0,0},{0,0}}, {{0,0},{1,0},{0,0},{0,0}}},
};

/* Link U_mu(site)_{ij} from the packed array u[site][4][3][3][2] (transposed). */
static inline cplx link_elem(const double *u, int site, int mu, int i, int j)
{
    const double *p = u + (((size_t)site * 4 + mu) * 9 + (size_t)j * 3 + i) * 2;
    cplx r = {p[0], p[1]};
    return r;
}

static inline cplx spin_elem(const double *psi, int site, int s, int c)
{
    const double *p = psi + ((size_t)site * 12 + (size_t)s * 3 + c) * 2;
    cplx r = {p[0], p[1]};
    return r;
}

/* acc[s][i] += sum_j M_ij * sum_s' P[s][s'] psi[s'][j], with M = U or U^dag and
 * P = 1 + sgn*gamma_mu. */
static void add_hop(cplx acc[4][3], const double *u, int lsite, int mu, int dagger,
                    const double *psi, int nsite, double sgn)
{
    cplx proj[4][3];
    for (int s = 0; s < 4; s++)
        for (int c = 0; c < 3; c++) {
            cplx v = spin_elem(psi, nsite, s, c);
            for (int t = 0; t < 4; t++) {
                cplx g = GAMMA[mu][s][t];
                if (g.re == 0.0 && g.im == 0.0) continue;
                cplx gs = {sgn * g.re, sgn * g.im};
                v = cadd(v, cmul(gs, spin_elem(psi, nsite, t, c)));
            }
            proj[s][c] = v;
        }
    for (int s = 0; s < 4; s++)
        for (int i = 0; i < 3; i++) {
            cplx sum = {0, 0};
            for (int j = 0; j < 3; j++) {
                cplx m = dagger ? conjc(link_elem(u, lsite, mu, j, i)) : link_elem(u, lsite, mu, i, j);
                sum = cadd(sum, cmul(m, proj[s][j]));
            }
            acc[s][i] = cadd(acc[s][i], sum);
        }
}

/* Apply the operator in FP64 on the caller's layout.
 *   nd        4 (4D, parity x+y+z+t) or 3 (3D, parity x+y+z, mu = 0..2)
 *   lin_of_lex caller linear index of each lexicographic site (V ints)
 *   u, psi, res  packed arrays in the caller's order (see file header)
 * Only sites of parity 1-cb are written.  isign outside {+1,-1} writes
 * nothing (the reference dispatches neither worker:
 * lib/sse_su3dslash_32bit_scalar.c:162-179). */
void orc_dslash_plain(int nd, const int dims[4], const int *lin_of_lex,
                      const double *u, const double *psi, double *res, int isign, int cb)
{
    if (isign != 1 && isign != -1) return;
    int V = dims[0] * dims[1] * dims[2] * dims[3];
    int target = 1 - cb;
#pragma omp parallel for schedule(static)
    for (int lex = 0; lex < V; lex++) {
        int c[4];
        lex_coords(dims, lex, c);
        int par = (nd == 4 ? c[0] + c[1] + c[2] + c[3] : c[0] + c[1] + c[2]) & 1;
        if (par != target) continue;
        cplx acc[4][3];
        memset(acc, 0, sizeof(acc));
        int site = lin_of_lex[lex];
        for (int mu = 0; mu < nd; mu++) {
            int cf[4], cbk[4];
            memcpy(cf, c, sizeof(cf)); memcpy(cbk, c, sizeof(cbk));
            cf[mu] = (c[mu] + 1) % dims[mu];
            cbk[mu] = (c[mu] - 1 + dims[mu]) % dims[mu];
            int fs = lin_of_lex[lex_index(dims, cf)];
            int bs = lin_of_lex[lex_index(dims, cbk)];
            add_hop(acc, u, site, mu, 0, psi, fs, -(double)isign);
            add_hop(acc, u, bs, mu, 1, psi, bs, +(double)isign);
        }
        double *out = res + (size_t)site * 24;
        for (int s = 0; s < 4; s++)
            for (int i = 0; i < 3; i++) {
                out[(s * 3 + i) * 2] = acc[s][i].re;
                out[(s * 3 + i) * 2 + 1] = acc[s][i].im;
            }
    }
}

/* ------------------------------------------------------------------------ */
/* Table-driven half-spinor restatement (the CPU baseline)                   */
/* ------------------------------------------------------------------------ */

typedef struct {
    int nd;
    int V, Vh;
    int *site_table;   /* traversal index -> caller linear index       */
    int *bwd;          /* [traversal][mu] caller index of x - mu       */
    int *fwd;          /* [traversal][mu] caller index of x + mu       */
} orc_tables;

/* Build the site table and neighbour tables for a layout (lin_of_lex) in the
 * canonical traversal order of the operator: cb2 order for nd=4, cb3d order
 * for nd=3 (lib/shift_tables_scalar.c:240-302, lib/shift_tables_scalar_3d.c:256-325). */
orc_tables *orc_tables_new(int nd, const int dims[4], const int *lin_of_lex)
{
    orc_tables *t = (orc_tables *)calloc(1, sizeof(orc_tables));
    if (!t) return NULL;
    t->nd = nd;
    t->V = dims[0] * dims[1] * dims[2] * dims[3];
    t->Vh = t->V / 2;
    t->site_table = (int *)malloc(sizeof(int) * (size_t)t->V);
    t->bwd = (int *)malloc(sizeof(int) * (size_t)t->V * 4);
    t->fwd = (int *)malloc(sizeof(int) * (size_t)t->V * 4);
    if (!t->site_table || !t->bwd || !t->fwd) {
        free(t->site_table); free(t->bwd); free(t->fwd); free(t);
        return NULL;
    }
    for (int idx = 0; idx < t->V; idx++) {
        int c[4];
        if (nd == 4) cb2_coords(dims, idx, c); else cb3d_coords(dims, idx, c);
        t->site_table[idx] = lin_of_lex[lex_index(dims, c)];
        for (int mu = 0; mu < 4; mu++) {
            int cf[4], cbk[4];
            memcpy(cf, c, sizeof(cf)); memcpy(cbk, c, sizeof(cbk));
            cf[mu] = (c[mu] + 1) % dims[mu];
            cbk[mu] = (c[mu] - 1 + dims[mu]) % dims[mu];
            t->fwd[idx * 4 + mu] = lin_of_lex[lex_index(dims, cf)];
            t->bwd[idx * 4 + mu] = lin_of_lex[lex_index(dims, cbk)];
        }
    }
    return t;
}

void orc_tables_free(orc_tables *t)
{
    if (!t) return;
    free(t->site_table); free(t->bwd); free(t->fwd); free(t);
}

/* Spin projection (1 - sigma*gamma_mu) psi for sigma = +1, in half-spinor form:
 *   h0 = psi0 + a0*psi_j0, h1 = psi1 + a1*psi_j1;   after the SU(3) multiply
 *   w0, w1 = M h0, M h1 and the lower components are r2 = b2*w_k2, r3 = b3*w_k3.
 * sigma = -1 flips every coefficient.  Derived from the gamma matrices above. */
static const struct { int j0, a0, j1, a1, k2, b2, k3, b3; } PROJ[4] = {
    /* mu=0: h0=psi0-i psi3, h1=psi1-i psi2; r2= i w1, r3= i w0 */ {3, 3, 2, 3, 1, 2, 0, 2},
    /* mu=1: h0=psi0+psi3,   h1=psi1-psi2;   r2=-w1,   r3= w0   */ {3, 0, 2, 1, 1, 1, 0, 0},
    /* mu=2: h0=psi0-i psi2, h1=psi1+i psi3; r2= i w0, r3=-i w1 */ {2, 3, 3, 2, 0, 2, 1, 3},
    /* mu=3: h0=psi0-psi2,   h1=psi1-psi3;   r2=-w0,   r3=-w1   */ {2, 1, 3, 1, 0, 1, 1, 1},
};

/* One template, instantiated for float and double arithmetic.
 *
 * The hop works on 4-wide vectors (GCC vector extensions, portable) that hold
 * one colour of two spin components as (re, im, re, im): the two upper spin
 * components of the half spinor, or of the accumulator, or its two lower
 * ones.  For each direction both projection coefficients are real or both
 * imaginary, and so are both reconstruction coefficients, so each step is a
 * lane permutation, a constant sign vector and an add.  The colour multiply
 * is w_i = sum_j Re(M_ij) h_j + Im(M_ij) (i h_j).                            */
#define ORC_PORT(REAL, NAME, IREAL)                                                 \
typedef REAL NAME##_v __attribute__((vector_size(4 * sizeof(REAL))));              \
typedef IREAL NAME##_m __attribute__((vector_size(4 * sizeof(REAL))));             \
/* {a.re, a.im, b.re, b.im} of the complex numbers at a and b */                     \
static inline __attribute__((always_inline))                                       \
NAME##_v NAME##_pair(const REAL *a, const REAL *b)                                   \
{ return (NAME##_v){a[0], a[1], b[0], b[1]}; }                                       \
/* code * v for each complex of v (both codes real or both imaginary):        \
 * 0: +1, 1: -1, 2: +i, 3: -i                                                  */   \
static inline __attribute__((always_inline))                                       \
NAME##_v NAME##_coef(NAME##_v v, const int ca, const int cb)                         \
{                                                                                    \
    const REAL sar = (ca == 0 || ca == 3) ? 1 : -1, sai = (ca == 0 || ca == 2) ? 1 : -1; \
    const REAL sbr = (cb == 0 || cb == 3) ? 1 : -1, sbi = (cb == 0 || cb == 2) ? 1 : -1; \
    if (ca >= 2) v = __builtin_shuffle(v, (NAME##_m){1, 0, 3, 2});                   \
    return v * (NAME##_v){sar, sai, sbr, sbi};                                       \
}                                                                                    \
/* always inlined with constant dagger, mu and sigma: the coefficient codes   \
 * and the PROJ entries fold to constants, as in the reference's one site     \
 * kernel per direction and sign (lib/site_dslash_32bit_scalar.c:23-3098) */   \
static inline __attribute__((always_inline))                                       \
void NAME##_hop(NAME##_v up[3], NAME##_v lo[3], const REAL *ps, const REAL *lk,     \
                const int dagger, const int mu, const int sigma)                   \
{                                                                                    \
    const int f = sigma < 0;                                                         \
    const int a0 = PROJ[mu].a0 ^ f, a1 = PROJ[mu].a1 ^ f;                            \
    const int b2 = PROJ[mu].b2 ^ f, b3 = PROJ[mu].b3 ^ f;                            \
    const int j0 = PROJ[mu].j0, j1 = PROJ[mu].j1;                                    \
    NAME##_v h[3], ih[3];                                                            \
    for (int c = 0; c < 3; c++) {                                                    \
        /* (h0_c, h1_c) = (psi0_c + a0 psi_j0,c, psi1_c + a1 psi_j1,c) */            \
        h[c] = NAME##_pair(ps + 2 * c, ps + 6 + 2 * c) +                             \
               NAME##_coef(NAME##_pair(ps + 6 * j0 + 2 * c, ps + 6 * j1 + 2 * c), a0, a1); \
        ih[c] = NAME##_coef(h[c], 2, 2);                                             \
    }                                                                                \
    for (int i = 0; i < 3; i++) {                                                    \
        NAME##_v w = {0, 0, 0, 0};                                                   \
        for (int j = 0; j < 3; j++) {                                                \
            /* M = U: M_ij = U_ij = lk[3j+i];  M = U^+: M_ij = conj(U_ji) = conj(lk[3i+j]) */ \
            const REAL *m = dagger ? lk + 2 * (3 * i + j) : lk + 2 * (3 * j + i);    \
            w += m[0] * h[j] + (dagger ? -m[1] : m[1]) * ih[j];                      \
        }                                                                            \
        up[i] += w;                                                                  \
        /* lower pair (r2, r3) = (b2 w_k2, b3 w_k3); (k2, k3) is (1, 0) or (0, 1) */  \
        const NAME##_v wl = PROJ[mu].k2 == 1 ? __builtin_shuffle(w, (NAME##_m){2, 3, 0, 1}) : w; \
        lo[i] += NAME##_coef(wl, b2, b3);                                            \
    }                                                                                \
}                                                                                    \
/* Both hops of direction MU (forward: U_mu(x), backward: U_mu(x-mu)^+) */          \
static inline __attribute__((always_inline))                                       \
void NAME##_dir(NAME##_v up[3], NAME##_v lo[3], const orc_tables *t, const REAL *u,  \
                const REAL *psi, int ix, int site, const int mu, const int sg)      \
{                                                                                    \
    int fs = t->fwd[ix * 4 + mu], bs = t->bwd[ix * 4 + mu];                          \
    NAME##_hop(up, lo, psi + (size_t)fs * 24, u + ((size_t)site * 4 + mu) * 18, 0, mu, sg); \
    NAME##_hop(up, lo, psi + (size_t)bs * 24, u + ((size_t)bs * 4 + mu) * 18, 1, mu, -sg);  \
}                                                                                    \
/* One target site (traversal index ix), the directions unrolled */                 \
static inline __attribute__((always_inline))                                       \
void NAME##_site(const orc_tables *t, const REAL *u, const REAL *psi, REAL *res,    \
                 int ix, int nd, const int sg)                                       \
{                                                                                    \
    NAME##_v up[3] = {{0, 0, 0, 0}, {0, 0, 0, 0}, {0, 0, 0, 0}};                    \
    NAME##_v lo[3] = {{0, 0, 0, 0}, {0, 0, 0, 0}, {0, 0, 0, 0}};                    \
    int site = t->site_table[ix];                                                    \
    NAME##_dir(up, lo, t, u, psi, ix, site, 0, sg);                                  \
    NAME##_dir(up, lo, t, u, psi, ix, site, 1, sg);                                  \
    NAME##_dir(up, lo, t, u, psi, ix, site, 2, sg);                                  \
    if (nd == 4) NAME##_dir(up, lo, t, u, psi, ix, site, 3, sg);                     \
    REAL *r = res + (size_t)site * 24; /* [spin][colour][re, im] */                  \
    for (int c = 0; c < 3; c++) {                                                    \
        r[2 * c] = up[c][0];      r[2 * c + 1] = up[c][1];                           \
        r[6 + 2 * c] = up[c][2];  r[6 + 2 * c + 1] = up[c][3];                       \
        r[12 + 2 * c] = lo[c][0]; r[12 + 2 * c + 1] = lo[c][1];                      \
        r[18 + 2 * c] = lo[c][2]; r[18 + 2 * c + 1] = lo[c][3];                      \
    }                                                                                \
}                                                                                    \
/* Target sites [first, first+count) of checkerboard 1-cb, in traversal order  \
 * (a bounded slice of one application, for timing on the host).  */               \
void orc_dslash_port_range_##NAME(const orc_tables *t, const REAL *u,                \
                                  const REAL *psi, REAL *res, int isign, int cb,     \
                                  int first, int count, int nthreads)                \
{                                                                                    \
    if (isign != 1 && isign != -1) return;                                           \
    if (first < 0) first = 0;                                                        \
    if (count > t->Vh - first) count = t->Vh - first;                                \
    if (count <= 0) return;                                                          \
    int target = 1 - cb;                                                             \
    int lo = target * t->Vh + first, hi = lo + count;                                \
    int nd = t->nd;                                                                  \
    if (nthreads <= 0) nthreads = 1;                                                 \
    if (isign == 1) {                                                                \
        _Pragma("omp parallel for schedule(static) num_threads(nthreads)")           \
        for (int ix = lo; ix < hi; ix++) NAME##_site(t, u, psi, res, ix, nd, 1);     \
    } else {                                                                         \
        _Pragma("omp parallel for schedule(static) num_threads(nthreads)")           \
        for (int ix = lo; ix < hi; ix++) NAME##_site(t, u, psi, res, ix, nd, -1);    \
    }                                                                                \
}                                                                                    \
void orc_dslash_port_##NAME(const orc_tables *t, const REAL *u, const REAL *psi,     \
                            REAL *res, int isign, int cb, int nthreads)              \
{                                                                                    \
    orc_dslash_port_range_##NAME(t, u, psi, res, isign, cb, 0, t->Vh, nthreads);     \
}

ORC_PORT(float, f32, int)
ORC_PORT(double, f64, long long)

int orc_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
