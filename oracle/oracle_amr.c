/*
 * oracle_amr.c -- TEST INFRASTRUCTURE ONLY (part of oracle/_build/libahforacle.so).
 *
 * A CPU restatement of AHF's AMR hierarchy (src/main.c:614-648;
 * src/libamr_serial: gen_domgrids / gen_AMRhierarchy / gen_refgrid in
 * generate_grids.c, refine_grid / ref_pquad / ref_cquad / ref_nquad /
 * test_node in refine_grid.c, get_TSCnodes / search_TSCplane /
 * search_TSCcolumn in get_nnodes.c, ll in lltools.c, relink in relink.c,
 * zero_dens / assign_npart in density.c), default build: TSC, periodic in
 * x, y and z, no NP_LIMIT, non-MULTIMASS.
 *
 * A grid is kept as the reference keeps it, as runs ("segments"): a grid is
 * a list of plane runs along z; each plane a list of row runs along y; each
 * row a list of node runs along x.  The segmentation matters: a node's
 * neighbours along x and y are only looked for inside its own run (or across
 * the periodic boundary), along z inside its plane run, and the refinement
 * passes skip the ends of runs.  Particle lists are kept in the reference's
 * order (ll prepends; relink moves matches to the head of the fine list), so
 * the float node densities are summed in the reference's order.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct { int64_t x0, len, node0, row; } nseg_t;       /* a run of nodes along x in one row   */
typedef struct { int64_t y, plane, cq, s0, ns; } row_t;        /* a row: its node runs s0 .. s0+ns-1 */
typedef struct { int64_t y0, len, row0, plane; } cseg_t;       /* a run of rows along y in one plane  */
typedef struct { int64_t z, pq, c0, nc; } plane_t;             /* a plane: its row runs c0 .. c0+nc-1 */
typedef struct { int64_t z0, len, plane0; } pseg_t;            /* a run of planes along z             */

typedef struct {
  int64_t l1;
  pseg_t *P; int64_t nP, capP;
  plane_t *pl; int64_t npl, cappl;
  cseg_t *C; int64_t nC, capC;
  row_t *R; int64_t nR, capR;
  nseg_t *N; int64_t nN, capN;
  int64_t nnodes;
  int64_t *nz, *ny, *nx, *nseg;    /* per node: coordinates and its run      */
  float *dens;                      /* per node: density (float, as flouble)  */
  int64_t *head;                    /* per node: first particle of its list   */
} grid_t;

#define GROW(a, n, cap)                                                   \
  do {                                                                    \
    if ((n) >= (cap)) {                                                   \
      (cap) = (cap) ? 2 * (cap) : 64;                                     \
      (a) = realloc((a), (size_t)(cap) * sizeof(*(a)));                   \
      if (!(a)) abort();                                                  \
    }                                                                     \
  } while (0)

static void grid_free(grid_t *g)
{
  free(g->P); free(g->pl); free(g->C); free(g->R); free(g->N);
  free(g->nz); free(g->ny); free(g->nx); free(g->nseg); free(g->dens); free(g->head);
  memset(g, 0, sizeof *g);
}

/* node arrays from the run structure (quad order: planes, row runs, rows,
 * node runs, nodes) */
static void grid_index(grid_t *g)
{
  int64_t n = 0;
  for (int64_t s = 0; s < g->nN; s++) { g->N[s].node0 = n; n += g->N[s].len; }
  g->nnodes = n;
  g->nz = malloc((n ? n : 1) * sizeof(int64_t)); g->ny = malloc((n ? n : 1) * sizeof(int64_t));
  g->nx = malloc((n ? n : 1) * sizeof(int64_t)); g->nseg = malloc((n ? n : 1) * sizeof(int64_t));
  g->dens = malloc((n ? n : 1) * sizeof(float)); g->head = malloc((n ? n : 1) * sizeof(int64_t));
  if (!g->nz || !g->ny || !g->nx || !g->nseg || !g->dens || !g->head) abort();
  for (int64_t s = 0; s < g->nN; s++) {
    const row_t *r = &g->R[g->N[s].row];
    for (int64_t k = 0; k < g->N[s].len; k++) {
      const int64_t i = g->N[s].node0 + k;
      g->nz[i] = g->pl[r->plane].z; g->ny[i] = r->y; g->nx[i] = g->N[s].x0 + k; g->nseg[i] = s;
      g->head[i] = -1;
    }
  }
}

/* the run of row r holding x, searched as the reference walks a row's runs;
 * -1 when x is in none */
static int64_t find_nseg(const grid_t *g, int64_t r, int64_t x)
{
  const row_t *R = &g->R[r];
  if (R->ns == 0) return -1;
  int64_t s = R->s0;
  while (x >= g->N[s].x0 + g->N[s].len && s + 1 < R->s0 + R->ns) s++;
  return (x >= g->N[s].x0 && x < g->N[s].x0 + g->N[s].len) ? s : -1;
}

/* the row run of plane p holding y; -1 when y is in none */
static int64_t find_cseg(const grid_t *g, int64_t p, int64_t y)
{
  const plane_t *P = &g->pl[p];
  if (P->nc == 0) return -1;
  int64_t c = P->c0;
  while (y >= g->C[c].y0 + g->C[c].len && c + 1 < P->c0 + P->nc) c++;
  return (y >= g->C[c].y0 && y < g->C[c].y0 + g->C[c].len) ? c : -1;
}

static int64_t row_of(const grid_t *g, int64_t c, int64_t y) { return g->C[c].row0 + (y - g->C[c].y0); }
static int64_t node_at(const grid_t *g, int64_t s, int64_t x) { return g->N[s].node0 + (x - g->N[s].x0); }

/* search_TSCcolumn: col[1] set; col[0], col[2] along x inside run s, or
 * across the periodic boundary through the row's last / first run */
static void tsc_column(const grid_t *g, int64_t c, int64_t s, int64_t col[3], int64_t y, int64_t x)
{
  const int64_t l1 = g->l1, r = row_of(g, c, y);
  const nseg_t *S = &g->N[s];
  if (x < S->x0 + S->len - 1) col[2] = col[1] + 1;
  else if (x == l1 - 1) {
    const nseg_t *F = &g->N[g->R[r].s0];
    col[2] = (F->x0 == 0 && F->len > 0) ? F->node0 : -1;
  } else col[2] = -1;
  if (x > S->x0) col[0] = col[1] - 1;
  else if (x == 0) {
    const nseg_t *L = &g->N[g->R[r].s0 + g->R[r].ns - 1];
    col[0] = (L->x0 + L->len == l1 && L->len > 0) ? L->node0 + L->len - 1 : -1;
  } else col[0] = -1;
}

static void null_col(int64_t col[3]) { col[0] = col[1] = col[2] = -1; }
static void null_plane(int64_t pl[3][3]) { for (int j = 0; j < 3; j++) null_col(pl[j]); }

/* search_TSCplane: pl[1][1] set (row run c, node run s of plane p) */
static void tsc_plane(const grid_t *g, int64_t p, int64_t c, int64_t s, int64_t pl[3][3], int64_t y, int64_t x)
{
  const int64_t l1 = g->l1;
  const cseg_t *C = &g->C[c];
  tsc_column(g, c, s, pl[1], y, x);
  /* row y + 1 */
  if (y < C->y0 + C->len - 1) {
    const int64_t s1 = find_nseg(g, row_of(g, c, y + 1), x);
    if (s1 >= 0) { pl[2][1] = node_at(g, s1, x); tsc_column(g, c, s1, pl[2], y + 1, x); }
    else null_col(pl[2]);
  } else if (y == l1 - 1) {
    const int64_t c1 = g->pl[p].c0;
    if (g->C[c1].y0 == 0) {
      const int64_t s1 = find_nseg(g, g->C[c1].row0, x);
      if (s1 >= 0) { pl[2][1] = node_at(g, s1, x); tsc_column(g, c1, s1, pl[2], 0, x); }
      else null_col(pl[2]);
    } else null_col(pl[2]);
  } else null_col(pl[2]);
  /* row y - 1 */
  if (y > C->y0) {
    const int64_t s1 = find_nseg(g, row_of(g, c, y - 1), x);
    if (s1 >= 0) { pl[0][1] = node_at(g, s1, x); tsc_column(g, c, s1, pl[0], y - 1, x); }
    else null_col(pl[0]);
  } else if (y == 0) {
    const int64_t c1 = find_cseg(g, p, l1 - 1);
    if (c1 >= 0) {
      const int64_t s1 = find_nseg(g, row_of(g, c1, l1 - 1), x);
      if (s1 >= 0) { pl[0][1] = node_at(g, s1, x); tsc_column(g, c1, s1, pl[0], l1 - 1, x); }
      else null_col(pl[0]);
    } else null_col(pl[0]);
  } else null_col(pl[0]);
}

/* plane p2 (a neighbour plane): the node at (y, x) found through the plane's
 * row runs and the row's node runs, then its plane of neighbours */
static void tsc_other_plane(const grid_t *g, int64_t p2, int64_t pl[3][3], int64_t y, int64_t x)
{
  const int64_t c2 = find_cseg(g, p2, y);
  if (c2 < 0) { null_plane(pl); return; }
  const int64_t s2 = find_nseg(g, row_of(g, c2, y), x);
  if (s2 < 0) { null_plane(pl); return; }
  pl[1][1] = node_at(g, s2, x);
  tsc_plane(g, p2, c2, s2, pl, y, x);
}

/* get_TSCnodes: the 27 nodes around node i as t[k][j][q] (z, y, x; 1 =
 * centre), -1 where the reference finds none */
static void tsc_nodes(const grid_t *g, int64_t i, int64_t t[3][3][3])
{
  const int64_t l1 = g->l1, s = g->nseg[i], r = g->N[s].row, p = g->R[r].plane, c = g->R[r].cq;
  const int64_t z = g->nz[i], y = g->ny[i], x = g->nx[i];
  const pseg_t *P = &g->P[g->pl[p].pq];
  t[1][1][1] = i;
  tsc_plane(g, p, c, s, t[1], y, x);
  /* plane z - 1 */
  if (z > P->z0) tsc_other_plane(g, p - 1, t[0], y, x);
  else if (z == 0) {
    int64_t q = 0;
    while (l1 - 1 >= g->P[q].z0 + g->P[q].len && q + 1 < g->nP) q++;
    if (l1 - 1 >= g->P[q].z0 && l1 - 1 < g->P[q].z0 + g->P[q].len)
      tsc_other_plane(g, g->P[q].plane0 + (l1 - 1 - g->P[q].z0), t[0], y, x);
    else null_plane(t[0]);
  } else null_plane(t[0]);
  /* plane z + 1 */
  if (z < P->z0 + P->len - 1) tsc_other_plane(g, p + 1, t[2], y, x);
  else if (z == l1 - 1) {
    if (g->P[0].z0 == 0) tsc_other_plane(g, g->P[0].plane0, t[2], y, x);
    else null_plane(t[2]);
  } else null_plane(t[2]);
}

static int tsc_all(int64_t t[3][3][3])
{
  for (int k = 0; k < 3; k++)
    for (int j = 0; j < 3; j++)
      for (int q = 0; q < 3; q++)
        if (t[k][j][q] < 0) return 0;
  return 1;
}

/* test_node (refine_grid.c:113-137): all 27 TSC nodes present and one of
 * the nine (z, y) x two (x, x + 1) at or above the threshold
 * critdens - mean_dens */
static int test_node(const grid_t *g, int64_t i, double thr)
{
  int64_t t[3][3][3];
  tsc_nodes(g, i, t);
  if (!tsc_all(t)) return 0;
  for (int k = 0; k < 3; k++)
    for (int j = 0; j < 3; j++)
      for (int q = 1; q < 3; q++)
        if ((double)g->dens[t[k][j][q]] >= thr) return 1;
  return 0;
}

/* the fine runs of one row: (x0, len) pairs */
typedef struct { int64_t *x0, *len; int64_t n, cap; } rowbuf_t;

static void row_emit(rowbuf_t *b, int64_t x0, int64_t len)
{
  if (b->n >= b->cap) {
    b->cap = b->cap ? 2 * b->cap : 8;
    b->x0 = realloc(b->x0, (size_t)b->cap * sizeof(int64_t));
    b->len = realloc(b->len, (size_t)b->cap * sizeof(int64_t));
    if (!b->x0 || !b->len) abort();
  }
  b->x0[b->n] = x0;
  b->len[b->n] = len;
  b->n++;
}

static void row_free(rowbuf_t *b) { free(b->x0); free(b->len); memset(b, 0, sizeof *b); }

/* ref_nquad (refine_grid.c:155-305) on the node runs of row r from run s */
static int ref_nquad(const grid_t *g, int64_t r, int64_t s, double thr, rowbuf_t *out)
{
  const int64_t l1 = g->l1, last = g->R[r].s0 + g->R[r].ns - 1;
  const nseg_t *S = &g->N[s];
  int state = 0, refever = 0, refined = 0;
  int64_t xlen = 0, start = 0, xoffset = 1;
  if (S->x0 == 0) {
    const nseg_t *L = &g->N[last];
    if (L->x0 + L->len == l1) {
      if (L->len > 0 && test_node(g, L->node0 + L->len - 1, thr)) { state = 1; refever = 1; start = 0; }
      xoffset = 0;
    }
  }
  int64_t idx = xoffset;
  for (; idx < S->len - 1; idx++) {
    const int64_t i = S->node0 + idx, x = S->x0 + idx;
    if (test_node(g, i, thr)) {
      if (!state) { state = 1; refever = 1; start = 2 * x; }
      xlen += 2;
    } else if (state) {
      int64_t t[3][3][3];
      state = 0;
      tsc_nodes(g, i, t);
      if (tsc_all(t)) xlen += 2;
      row_emit(out, start, xlen);
      xlen = 0;
    }
  }
  const int64_t xe = S->x0 + idx;
  if (s < last) {
    if (state) row_emit(out, start, xlen);
    refined = ref_nquad(g, r, s + 1, thr, out);
  } else if (S->x0 + S->len == l1 && idx < S->len && test_node(g, S->node0 + idx, thr)) {
    if (!state) { refever = 1; start = 2 * xe; }
    xlen += 2;
    row_emit(out, start, xlen);
  } else if (state) {
    row_emit(out, start, xlen);
  }
  return refever || refined;
}

/* the fine row runs of one plane: runs of rows, each row its node runs */
typedef struct {
  int64_t *cy0, *cr0, *cnr; int64_t nc, capc;       /* row runs: first y, first row, rows      */
  int64_t *ry, *rs0, *rns; int64_t nr, capr;        /* rows: y, first node run, node runs      */
  int64_t *sx0, *slen; int64_t ns, caps;            /* node runs                               */
  int open;
} planebuf_t;

static void *grow(void *a, int64_t *cap, int64_t n, size_t sz)
{
  if (n < *cap) return a;
  *cap = *cap ? 2 * *cap : 16;
  a = realloc(a, (size_t)*cap * sz);
  if (!a) abort();
  return a;
}

static void pb_open(planebuf_t *b, int64_t y0)
{
  int64_t c = b->capc;
  b->cy0 = grow(b->cy0, &c, b->nc, sizeof(int64_t)); c = b->capc;
  b->cr0 = grow(b->cr0, &c, b->nc, sizeof(int64_t)); c = b->capc;
  b->cnr = grow(b->cnr, &c, b->nc, sizeof(int64_t));
  b->capc = c;
  b->cy0[b->nc] = y0; b->cr0[b->nc] = b->nr; b->cnr[b->nc] = 0;
  b->nc++;
  b->open = 1;
}

static void pb_row(planebuf_t *b, int64_t y, const rowbuf_t *r)
{
  int64_t c = b->capr;
  b->ry = grow(b->ry, &c, b->nr, sizeof(int64_t)); c = b->capr;
  b->rs0 = grow(b->rs0, &c, b->nr, sizeof(int64_t)); c = b->capr;
  b->rns = grow(b->rns, &c, b->nr, sizeof(int64_t));
  b->capr = c;
  b->ry[b->nr] = y; b->rs0[b->nr] = b->ns; b->rns[b->nr] = r->n;
  b->nr++;
  for (int64_t k = 0; k < r->n; k++) {
    int64_t cs = b->caps;
    b->sx0 = grow(b->sx0, &cs, b->ns, sizeof(int64_t)); cs = b->caps;
    b->slen = grow(b->slen, &cs, b->ns, sizeof(int64_t));
    b->caps = cs;
    b->sx0[b->ns] = r->x0[k]; b->slen[b->ns] = r->len[k];
    b->ns++;
  }
  b->cnr[b->nc - 1]++;
}

static void pb_free(planebuf_t *b)
{
  free(b->cy0); free(b->cr0); free(b->cnr); free(b->ry); free(b->rs0); free(b->rns); free(b->sx0); free(b->slen);
  memset(b, 0, sizeof *b);
}

/* ref_cquad (refine_grid.c:310-604) on the row runs of plane p from run c.
 * Whether the rows wrap periodically is judged, as the reference does
 * (fst_cquad = coa_pquad->loc), from the first and last row runs of the
 * FIRST plane of p's plane run, whichever plane p is. */
static int ref_cquad(const grid_t *g, int64_t p, int64_t c, double thr, planebuf_t *out)
{
  const int64_t l1 = g->l1;
  const plane_t *P = &g->pl[p], *P0 = &g->pl[g->P[P->pq].plane0];
  const cseg_t *C = &g->C[c], *fst = &g->C[P0->c0], *lst = &g->C[P0->c0 + P0->nc - 1];
  int64_t ylow = 1, yup = -1;
  if (fst->y0 == 0 && lst->y0 + lst->len == l1) {
    if (C->y0 == 0 && C->y0 + C->len == l1) { ylow = 0; yup = 0; }
    else if (C->y0 == 0) { ylow = 0; yup = -1; }
    else if (C->y0 + C->len == l1) { ylow = 1; yup = 0; }
  }
  int state = 0, refever = 0, refined = 0;
  int64_t idx = ylow;
  for (; idx < C->len - 1 + yup; idx++) {
    const int64_t y = C->y0 + idx, r = C->row0 + idx;
    rowbuf_t rb = {0};
    if (ref_nquad(g, r, g->R[r].s0, thr, &rb)) {
      if (!state) { state = 1; refever = 1; pb_open(out, 2 * y); }
      pb_row(out, 2 * y, &rb);
      pb_row(out, 2 * y + 1, &rb);
    } else if (state) {
      state = 0;
    }
    row_free(&rb);
  }
  const int64_t ye = C->y0 + idx;
  if (c < P->c0 + P->nc - 1) {
    refined = ref_cquad(g, p, c + 1, thr, out);
  } else if (C->y0 + C->len == l1 && idx < C->len) {
    rowbuf_t rb = {0};
    const int64_t r = C->row0 + idx;
    if (ref_nquad(g, r, g->R[r].s0, thr, &rb)) {
      if (!state) { refever = 1; pb_open(out, 2 * ye); }
      pb_row(out, 2 * ye, &rb);
      pb_row(out, 2 * ye + 1, &rb);
    }
    row_free(&rb);
  }
  return refever || refined;
}

/* a refined plane (2 z or 2 z + 1) into the fine grid, as the current plane
 * run's next plane */
static void fine_plane(grid_t *f, int64_t z, const planebuf_t *b)
{
  GROW(f->pl, f->npl, f->cappl);
  const int64_t p = f->npl++;
  f->pl[p].z = z; f->pl[p].pq = f->nP - 1; f->pl[p].c0 = f->nC; f->pl[p].nc = b->nc;
  f->P[f->nP - 1].len++;
  for (int64_t c = 0; c < b->nc; c++) {
    GROW(f->C, f->nC, f->capC);
    const int64_t ci = f->nC++;
    f->C[ci].y0 = b->cy0[c]; f->C[ci].len = b->cnr[c]; f->C[ci].row0 = f->nR; f->C[ci].plane = p;
    for (int64_t r = b->cr0[c]; r < b->cr0[c] + b->cnr[c]; r++) {
      GROW(f->R, f->nR, f->capR);
      const int64_t ri = f->nR++;
      f->R[ri].y = b->ry[r]; f->R[ri].plane = p; f->R[ri].cq = ci; f->R[ri].s0 = f->nN; f->R[ri].ns = b->rns[r];
      for (int64_t s = b->rs0[r]; s < b->rs0[r] + b->rns[r]; s++) {
        GROW(f->N, f->nN, f->capN);
        f->N[f->nN].x0 = b->sx0[s]; f->N[f->nN].len = b->slen[s]; f->N[f->nN].row = ri; f->N[f->nN].node0 = 0;
        f->nN++;
      }
    }
  }
}

static void fine_open(grid_t *f, int64_t z0)
{
  GROW(f->P, f->nP, f->capP);
  f->P[f->nP].z0 = z0; f->P[f->nP].len = 0; f->P[f->nP].plane0 = f->npl;
  f->nP++;
}

/* ref_pquad (refine_grid.c:609-800) on the plane runs of grid g from run q */
static int ref_pquad(const grid_t *g, int64_t q, double thr, grid_t *f)
{
  const int64_t l1 = g->l1;
  const pseg_t *Q = &g->P[q], *fst = &g->P[0], *lst = &g->P[g->nP - 1];
  int64_t zlow = 1, zup = -1;
  if (fst->z0 == 0 && lst->z0 + lst->len == l1) {
    if (Q->z0 == 0 && Q->z0 + Q->len == l1) { zlow = 0; zup = 0; }
    else if (Q->z0 == 0) { zlow = 0; zup = -1; }
    else if (Q->z0 + Q->len == l1) { zlow = 1; zup = 0; }
  }
  int state = 0, refever = 0, refined = 0;
  int64_t idx = zlow;
  for (; idx < Q->len - 1 + zup; idx++) {
    const int64_t z = Q->z0 + idx, p = Q->plane0 + idx;
    planebuf_t pb = {0};
    if (ref_cquad(g, p, g->pl[p].c0, thr, &pb)) {
      if (!state) { state = 1; refever = 1; fine_open(f, 2 * z); }
      fine_plane(f, 2 * z, &pb);
      fine_plane(f, 2 * z + 1, &pb);
    } else if (state) {
      state = 0;
    }
    pb_free(&pb);
  }
  const int64_t ze = Q->z0 + idx;
  if (q < g->nP - 1) {
    refined = ref_pquad(g, q + 1, thr, f);
  } else if (Q->z0 + Q->len == l1 && idx < Q->len) {
    planebuf_t pb = {0};
    const int64_t p = Q->plane0 + idx;
    if (ref_cquad(g, p, g->pl[p].c0, thr, &pb)) {
      if (!state) { refever = 1; fine_open(f, 2 * ze); }
      fine_plane(f, 2 * ze, &pb);
      fine_plane(f, 2 * ze + 1, &pb);
    }
    pb_free(&pb);
  }
  return refever || refined;
}

/* the node of grid g at (z, y, x), through its runs; -1 when absent */
static int64_t find_node(const grid_t *g, int64_t z, int64_t y, int64_t x)
{
  int64_t q = 0;
  while (z >= g->P[q].z0 + g->P[q].len && q + 1 < g->nP) q++;
  if (z < g->P[q].z0 || z >= g->P[q].z0 + g->P[q].len) return -1;
  const int64_t c = find_cseg(g, g->P[q].plane0 + (z - g->P[q].z0), y);
  if (c < 0) return -1;
  const int64_t s = find_nseg(g, row_of(g, c, y), x);
  return s < 0 ? -1 : node_at(g, s, x);
}

/* relink (relink.c:31-290): for each fine node in order whose 27 TSC nodes
 * all exist, the particles of its coarse parent's list lying within half a
 * fine cell of its centre (inclusive) leave that list, keeping the others'
 * order, and are prepended to the fine node's list.  Returns their number. */
static int64_t relink(grid_t *g, grid_t *f, const float *pos[3], int64_t *next)
{
  const double l1 = (double)f->l1, shift = 0.5 / l1;
  int64_t moved = 0;
  for (int64_t i = 0; i < f->nnodes; i++) {
    const int64_t j = find_node(g, f->nz[i] / 2, f->ny[i] / 2, f->nx[i] / 2);
    if (j < 0 || g->head[j] < 0) continue;
    int64_t t[3][3][3];
    tsc_nodes(f, i, t);
    if (!tsc_all(t)) continue;
    const double cx = (double)f->nx[i] / l1 + shift, cy = (double)f->ny[i] / l1 + shift,
                 cz = (double)f->nz[i] / l1 + shift;
    int64_t prev = -1, cur = g->head[j];
    while (cur >= 0) {
      const int64_t nx = next[cur];
      if (fabs((double)pos[0][cur] - cx) <= shift && fabs((double)pos[1][cur] - cy) <= shift &&
          fabs((double)pos[2][cur] - cz) <= shift) {
        if (prev < 0) g->head[j] = nx; else next[prev] = nx;
        next[cur] = f->head[i];
        f->head[i] = cur;
        moved++;
      } else {
        prev = cur;
      }
      cur = nx;
    }
  }
  return moved;
}

static double f1mod_amr(double x) { return x >= 2.0 ? x - 2.0 : (x >= 1.0 ? x - 1.0 : x); }

/* zero_dens + assign_npart (density.c:238-443): -mean_dens everywhere, then
 * every particle of every node's list (nodes in order) adds its TSC weights
 * to the TSC nodes that exist.  Returns the particles assigned. */
static int64_t assign_npart(grid_t *g, const float *pos[3], const int64_t *next, double m2d)
{
  const double l1 = (double)g->l1, shift = 0.5 / l1;
  int64_t np = 0;
  for (int64_t i = 0; i < g->nnodes; i++) g->dens[i] = (float)(-1.0);
  for (int64_t i = 0; i < g->nnodes; i++) {
    if (g->head[i] < 0) continue;
    int64_t t[3][3][3];
    tsc_nodes(g, i, t);
    const int64_t cc[3] = {g->nx[i], g->ny[i], g->nz[i]};
    double centre[3];
    for (int d = 0; d < 3; d++) centre[d] = f1mod_amr(((double)cc[d] / l1 + shift) + 1.0);
    for (int64_t p = g->head[i]; p >= 0; p = next[p]) {
      np++;
      double w[3][3];
      for (int d = 0; d < 3; d++) {
        double sep = ((double)pos[d][p] - centre[d]) * l1;
        if (fabs(sep) > 0.5 * l1) {
          const double a = f1mod_amr(((double)pos[d][p] + 0.5) + 1.0);
          const double b = f1mod_amr((centre[d] + 0.5) + 1.0);
          sep = (a - b) * l1;
        }
        w[d][1] = 0.75 - sep * sep;
        w[d][0] = ((0.5 - sep) * (0.5 - sep)) / 2;
        w[d][2] = ((0.5 + sep) * (0.5 + sep)) / 2;
      }
      for (int k = 0; k < 3; k++)
        for (int j = 0; j < 3; j++)
          for (int q = 0; q < 3; q++)
            if (t[k][j][q] >= 0) g->dens[t[k][j][q]] += m2d * w[2][k] * w[1][j] * w[0][q];
    }
  }
  return np;
}

/* The same densities as a gather (the formulation a GPU kernel can use
 * without atomics): the (target, source, stencil slot) pairs of every
 * source's TSC nodes, ordered by target and then source (stable in slot);
 * each target starts at -mean_dens and adds, source by source in node
 * order, each source particle's weight in list order.  Float additions in
 * the same order as assign_npart's scatter, so the result is identical;
 * returns the number of nodes whose density differs from g->dens. */
typedef struct { int64_t t, s; int slot; } tpair_t;

static int cmp_tpair(const void *a, const void *b)
{
  const tpair_t *p = a, *q = b;
  if (p->t != q->t) return p->t < q->t ? -1 : 1;
  if (p->s != q->s) return p->s < q->s ? -1 : 1;
  return p->slot - q->slot;
}

static int64_t gather_mismatch(const grid_t *g, const float *pos[3], const int64_t *next, double m2d)
{
  const double l1 = (double)g->l1, shift = 0.5 / l1;
  tpair_t *pr = malloc((size_t)(g->nnodes ? g->nnodes : 1) * 27 * sizeof(tpair_t));
  float *out = malloc((size_t)(g->nnodes ? g->nnodes : 1) * sizeof(float));
  if (!pr || !out) return -1;
  int64_t np = 0;
  for (int64_t s = 0; s < g->nnodes; s++) {
    if (g->head[s] < 0) continue;
    int64_t t[3][3][3];
    tsc_nodes(g, s, t);
    for (int k = 0; k < 27; k++)
      if (t[k / 9][(k / 3) % 3][k % 3] >= 0) { pr[np].t = t[k / 9][(k / 3) % 3][k % 3]; pr[np].s = s; pr[np].slot = k; np++; }
  }
  qsort(pr, (size_t)np, sizeof(tpair_t), cmp_tpair);
  for (int64_t i = 0; i < g->nnodes; i++) out[i] = (float)(-1.0);
  for (int64_t e = 0; e < np; e++) {
    const int64_t s = pr[e].s, tt = pr[e].t;
    const int k = pr[e].slot / 9, j = (pr[e].slot / 3) % 3, q = pr[e].slot % 3;
    const int64_t cc[3] = {g->nx[s], g->ny[s], g->nz[s]};
    double centre[3];
    for (int d = 0; d < 3; d++) centre[d] = f1mod_amr(((double)cc[d] / l1 + shift) + 1.0);
    for (int64_t p = g->head[s]; p >= 0; p = next[p]) {
      double w[3][3];
      for (int d = 0; d < 3; d++) {
        double sep = ((double)pos[d][p] - centre[d]) * l1;
        if (fabs(sep) > 0.5 * l1) {
          const double a = f1mod_amr(((double)pos[d][p] + 0.5) + 1.0);
          const double b = f1mod_amr((centre[d] + 0.5) + 1.0);
          sep = (a - b) * l1;
        }
        w[d][1] = 0.75 - sep * sep;
        w[d][0] = ((0.5 - sep) * (0.5 - sep)) / 2;
        w[d][2] = ((0.5 + sep) * (0.5 + sep)) / 2;
      }
      out[tt] += m2d * w[2][k] * w[1][j] * w[0][q];
    }
  }
  int64_t bad = 0;
  for (int64_t i = 0; i < g->nnodes; i++) bad += memcmp(&out[i], &g->dens[i], sizeof(float)) != 0;
  free(pr);
  free(out);
  return bad;
}

/* The hierarchy (main.c:614-648, gen_AMRhierarchy): the ngrid_dom^3 domain
 * grid (one run per plane, row and node line), particles linked to it by ll
 * (cell trunc(l1 x), a cell index above l1 - 1 folded to 0; each particle
 * prepended in input order), densities; then, while the finest grid is
 * below ngrid_max, a refinement (threshold critdens - mean_dens, critdens =
 * NperDomCell masstodens on the domain grid and NperRefCell masstodens on the
 * others, masstodens = ngrid_dom^3 / n times 8 per level), relink, densities,
 * and the grid kept only with at least MIN_NNODES = 125 nodes.
 * levels[3 g + 0..2] = nodes per dimension, nodes, particles assigned of
 * grid g; returns the number of grids (at most max_levels reported), or -1. */
#define MAX_GRIDS 40

static int64_t *g_gather_check;   /* when set: gather-vs-scatter mismatches, summed over grids */

static int build_hierarchy(uint64_t n, const float *x, const float *y, const float *z, int ngrid_dom, int ngrid_max,
                           double nth_dom, double nth_ref, grid_t *grids, int64_t *levels, int max_levels,
                           int64_t **next_out)
{
  const float *pos[3] = {x, y, z};
  const int64_t L = ngrid_dom;
  int64_t *next = malloc((n ? n : 1) * sizeof(int64_t));
  if (!next || n == 0) return -1;
  memset(grids, 0, MAX_GRIDS * sizeof(grid_t));
  grid_t *d = &grids[0];
  d->l1 = L;
  fine_open(d, 0);
  for (int64_t zz = 0; zz < L; zz++) {
    GROW(d->pl, d->npl, d->cappl);
    const int64_t p = d->npl++;
    d->pl[p].z = zz; d->pl[p].pq = 0; d->pl[p].c0 = d->nC; d->pl[p].nc = 1;
    d->P[0].len++;
    GROW(d->C, d->nC, d->capC);
    const int64_t c = d->nC++;
    d->C[c].y0 = 0; d->C[c].len = L; d->C[c].row0 = d->nR; d->C[c].plane = p;
    for (int64_t yy = 0; yy < L; yy++) {
      GROW(d->R, d->nR, d->capR);
      const int64_t r = d->nR++;
      d->R[r].y = yy; d->R[r].plane = p; d->R[r].cq = c; d->R[r].s0 = d->nN; d->R[r].ns = 1;
      GROW(d->N, d->nN, d->capN);
      d->N[d->nN].x0 = 0; d->N[d->nN].len = L; d->N[d->nN].row = r;
      d->nN++;
    }
  }
  grid_index(d);
  for (uint64_t i = 0; i < n; i++) {
    int64_t c[3];
    for (int k = 0; k < 3; k++) {
      unsigned long v = (unsigned long)((double)L * (double)pos[k][i]);
      if (v > (unsigned long)(L - 1)) v = 0;
      c[k] = (int64_t)v;
    }
    const int64_t node = (c[2] * L + c[1]) * L + c[0];
    next[i] = d->head[node];
    d->head[node] = (int64_t)i;
  }
  const double dl = (double)L;
  double m2d = (dl * dl * dl) / (double)n;
  int64_t np = assign_npart(d, pos, next, m2d);
  if (g_gather_check) *g_gather_check += gather_mismatch(d, pos, next, m2d);
  int ng = 1;
  if (max_levels > 0) { levels[0] = L; levels[1] = d->nnodes; levels[2] = np; }
  double thr = nth_dom * m2d - 1.0;
  while (ng < MAX_GRIDS) {
    grid_t *c = &grids[ng - 1], *f = &grids[ng];
    if (c->l1 >= ngrid_max) break;
    f->l1 = 2 * c->l1;
    if (!ref_pquad(c, 0, thr, f)) { grid_free(f); break; }
    grid_index(f);
    relink(c, f, pos, next);
    const double m2f = m2d * 8.0;
    np = assign_npart(f, pos, next, m2f);
    if (g_gather_check) *g_gather_check += gather_mismatch(f, pos, next, m2f);
    if (f->nnodes < 125) { grid_free(f); break; }
    if (ng < max_levels) { levels[3 * ng] = f->l1; levels[3 * ng + 1] = f->nnodes; levels[3 * ng + 2] = np; }
    ng++;
    m2d = m2f;
    thr = nth_ref * m2d - 1.0;
  }
  if (next_out) *next_out = next;
  else free(next);
  return ng;
}

int ahforacle_amr_levels(uint64_t n, const float *x, const float *y, const float *z, int ngrid_dom,
                         int ngrid_max, double nth_dom, double nth_ref, int64_t *levels, int max_levels)
{
  grid_t grids[MAX_GRIDS];
  const int ng = build_hierarchy(n, x, y, z, ngrid_dom, ngrid_max, nth_dom, nth_ref, grids, levels, max_levels, NULL);
  for (int g = 0; g < ng; g++) grid_free(&grids[g]);
  return ng;
}

/* Grid `level` of that hierarchy: nodes (z, y, x) in run order and their
 * densities.  Returns the number of nodes, -3 when more than max_nodes, -4
 * when there is no such grid. */
int64_t ahforacle_amr_nodes(uint64_t n, const float *x, const float *y, const float *z, int ngrid_dom,
                            int ngrid_max, double nth_dom, double nth_ref, int level, int64_t *zyx, double *dens,
                            int64_t max_nodes)
{
  grid_t grids[MAX_GRIDS];
  int64_t lv[3 * MAX_GRIDS];
  const int ng = build_hierarchy(n, x, y, z, ngrid_dom, ngrid_max, nth_dom, nth_ref, grids, lv, MAX_GRIDS, NULL);
  int64_t count = level < ng ? 0 : -4;
  if (level < ng) {
    const grid_t *g = &grids[level];
    if (g->nnodes > max_nodes) count = -3;
    else {
      for (int64_t i = 0; i < g->nnodes; i++) {
        zyx[3 * i] = g->nz[i]; zyx[3 * i + 1] = g->ny[i]; zyx[3 * i + 2] = g->nx[i];
        dens[i] = (double)g->dens[i];
      }
      count = g->nnodes;
    }
  }
  for (int g = 0; g < ng; g++) grid_free(&grids[g]);
  return count;
}


/* Every grid of that hierarchy at once: grid g's nodes and densities at
 * offsets counts[0] + ... + counts[g - 1] of zyx (3 per node) and dens;
 * counts[g] its node count.  Returns the number of grids, -3 when more than
 * max_total nodes or max_grids grids. */
int ahforacle_amr_all_nodes(uint64_t n, const float *x, const float *y, const float *z, int ngrid_dom,
                            int ngrid_max, double nth_dom, double nth_ref, int64_t *zyx, double *dens,
                            int64_t max_total, int64_t *counts, int max_grids)
{
  grid_t grids[MAX_GRIDS];
  int64_t lv[3 * MAX_GRIDS];
  const int ng = build_hierarchy(n, x, y, z, ngrid_dom, ngrid_max, nth_dom, nth_ref, grids, lv, MAX_GRIDS, NULL);
  int rc = ng;
  int64_t at = 0;
  for (int g = 0; g < ng && rc >= 0; g++) {
    if (g >= max_grids || at + grids[g].nnodes > max_total) { rc = -3; break; }
    for (int64_t i = 0; i < grids[g].nnodes; i++, at++) {
      zyx[3 * at] = grids[g].nz[i]; zyx[3 * at + 1] = grids[g].ny[i]; zyx[3 * at + 2] = grids[g].nx[i];
      dens[at] = (double)grids[g].dens[i];
    }
    counts[g] = grids[g].nnodes;
  }
  for (int g = 0; g < ng; g++) grid_free(&grids[g]);
  return rc;
}

/* Checks a property of the hierarchy a GPU version can build on: each
 * node's particle list is in input-index order, descending on grids 0, 2,
 * 4, ... and ascending on grids 1, 3, ... (ll prepends in index order;
 * relink reverses the matches it moves).  Each grid is checked as the finest
 * of a hierarchy stopped there, before another relink takes particles from
 * it.  Returns the number of out-of-order pairs over all grids, or -1. */
int64_t ahforacle_amr_list_order_violations(uint64_t n, const float *x, const float *y, const float *z,
                                            int ngrid_dom, int ngrid_max, double nth_dom, double nth_ref)
{
  grid_t grids[MAX_GRIDS];
  int64_t lv[3 * MAX_GRIDS], bad = 0;
  for (int level = 0; level < MAX_GRIDS && ((int64_t)ngrid_dom << level) <= ngrid_max; level++) {
    int64_t *next = NULL;
    const int ng = build_hierarchy(n, x, y, z, ngrid_dom, (int)((int64_t)ngrid_dom << level), nth_dom, nth_ref,
                                   grids, lv, MAX_GRIDS, &next);
    if (ng < 0) return -1;
    const grid_t *g = &grids[ng - 1];
    const int desc = ((ng - 1) % 2) == 0;
    for (int64_t i = 0; i < g->nnodes; i++)
      for (int64_t p = g->head[i]; p >= 0 && next[p] >= 0; p = next[p])
        if (desc ? !(p > next[p]) : !(p < next[p])) bad++;
    for (int k = 0; k < ng; k++) grid_free(&grids[k]);
    free(next);
    if (ng - 1 < level) break;   /* the hierarchy stopped earlier */
  }
  return bad;
}


/* Builds the hierarchy and recomputes every grid's densities in the gather
 * formulation (gather_mismatch); returns the number of nodes, over all
 * grids, whose gathered density differs from the scattered one, or -1. */
int64_t ahforacle_amr_gather_mismatches(uint64_t n, const float *x, const float *y, const float *z, int ngrid_dom,
                                        int ngrid_max, double nth_dom, double nth_ref)
{
  grid_t grids[MAX_GRIDS];
  int64_t lv[3 * MAX_GRIDS], bad = 0;
  g_gather_check = &bad;
  const int ng = build_hierarchy(n, x, y, z, ngrid_dom, ngrid_max, nth_dom, nth_ref, grids, lv, MAX_GRIDS, NULL);
  g_gather_check = NULL;
  for (int k = 0; k < ng; k++) grid_free(&grids[k]);
  return ng < 0 ? -1 : bad;
}
