// amr_tree.cu -- AHF's AMR hierarchy below the domain grid (libamr_serial):
// the refinement of a grid kept as runs, relink, and the TSC densities of
// the refined grid, level after level (gen_AMRhierarchy,
// src/libamr_serial/generate_grids.c:278; refine_grid.c; relink.c;
// get_nnodes.c; density.c:238).
//
// A grid is held as the reference holds it: runs of planes along z, each
// plane a list of row runs along y, each row a list of node runs along x.
// The segmentation decides which neighbours exist for the TSC stencil (a
// node's x neighbours are looked for only inside its own node run or across
// the periodic face, its y neighbours only inside its row run, its z
// neighbours only inside its plane run) and which nodes the refinement
// tests (the state machines skip the ends of runs), so it is kept exactly,
// in device arrays:
//   plane runs  {z0, len, first plane}
//   planes      {z, plane run, first row run, row runs}
//   row runs    {y0, len, first row, plane}
//   rows        {y, plane, row run, first node run, node runs}
//   node runs   {x0, len, first node, row}
//   nodes       ascending (z, y, x): key (z l1 + y) l1 + x, node run.
// Everything is in ascending order, so a node index is its rank by key.
//
// One refinement (refine_grid, refine_grid.c:899, ref_pquad / ref_cquad /
// ref_nquad :155-800, test_node :113-137):
//   k_ag_tsc    the 27 TSC nodes of every node (get_TSCnodes,
//               get_nnodes.c), and whether all exist;
//   k_ag_test   test_node: all 27 exist and one of the 18 at dx in {0, 1} is
//               at or above critdens - mean_dens;
//   k_ag_rows   per coarse row, the node-run state machine (ref_nquad): the
//               fine node runs it emits and whether it refines (count, then
//               emit at the scanned offsets);
//   k_ag_planes per coarse plane, the row-run state machine (ref_cquad): its
//               fine row runs and the coarse rows it refines;
//   k_ag_pquad  one thread: the plane-run state machine (ref_pquad), the fine
//               planes in order and every count and offset of the fine grid;
//   k_ag_fplanes, k_ag_fnodes  the fine grid's arrays.
// Relink (relink.c:31-290): a particle of a coarse node's list moves to the
// first of the node's children, in node order, whose 27 TSC nodes exist and
// whose cell (half a fine cell about its centre, inclusive) holds it.  The
// moved particles are ordered by fine node (a stable radix sort): within a
// node they come in input order, and the reference's list order is that or
// its reverse (ll prepends in input order, relink prepends what it moves),
// descending on grids 0, 2, 4, ... and ascending on grids 1, 3, ...
// Densities (assign_npart, density.c:238): every node starts at -1 (minus
// the mean density); the reference visits the nodes in order and adds each
// listed particle's m2d w_z w_y w_x (double) to the float density of its 27
// TSC nodes.  Here as a gather: one thread per target finds its sources
// through its own stencil (and the few one-sided pairs the runs make, listed
// beforehand), orders them by node index and adds their particles in list
// order -- the same float additions in the same order, so the floats are
// identical.
#include <cstdint>

#include "common.cuh"
#include "amr_tree.cuh"
#include "amr_sum.cuh"

namespace ahfgpu {

constexpr int kAgT = 256;

// ---------------------------------------------------------------------------
// neighbour search through the runs (get_TSCnodes / search_TSCplane /
// search_TSCcolumn): each walk visits the runs in order, as the reference
// does, so a run of length zero takes part in the search as it does there

// the node run of row r holding x; -1 when none does
__device__ int ag_find_nseg(const AGrid& g, int r, int x) {
  const ARow R = g.R[r];
  if (R.ns == 0) return -1;
  int s = R.s0;
  while (x >= g.N[s].x0 + g.N[s].len && s + 1 < R.s0 + R.ns) s++;
  return (x >= g.N[s].x0 && x < g.N[s].x0 + g.N[s].len) ? s : -1;
}

// the row run of plane p holding y; -1 when none does
__device__ int ag_find_cseg(const AGrid& g, int p, int y) {
  const APlane P = g.pl[p];
  if (P.nc == 0) return -1;
  int c = P.c0;
  while (y >= g.C[c].y0 + g.C[c].len && c + 1 < P.c0 + P.nc) c++;
  return (y >= g.C[c].y0 && y < g.C[c].y0 + g.C[c].len) ? c : -1;
}

__device__ __forceinline__ int ag_row_of(const AGrid& g, int c, int y) { return g.C[c].r0 + (y - g.C[c].y0); }
__device__ __forceinline__ int ag_node_at(const AGrid& g, int s, int x) { return g.N[s].n0 + (x - g.N[s].x0); }

// the x neighbours of the node at (y, x) in node run s of row run c; col[1]
// is the node itself
__device__ void ag_column(const AGrid& g, int c, int s, int* col, int y, int x) {
  const int r = ag_row_of(g, c, y);
  const ANRun S = g.N[s];
  if (x < S.x0 + S.len - 1) col[2] = col[1] + 1;
  else if (x == g.l1 - 1) {
    const ANRun F = g.N[g.R[r].s0];
    col[2] = (F.x0 == 0 && F.len > 0) ? F.n0 : -1;
  } else col[2] = -1;
  if (x > S.x0) col[0] = col[1] - 1;
  else if (x == 0) {
    const ANRun L = g.N[g.R[r].s0 + g.R[r].ns - 1];
    col[0] = (L.x0 + L.len == g.l1 && L.len > 0) ? L.n0 + L.len - 1 : -1;
  } else col[0] = -1;
}

__device__ __forceinline__ void ag_null3(int* c) { c[0] = c[1] = c[2] = -1; }
__device__ __forceinline__ void ag_null9(int* p) {
  for (int k = 0; k < 9; k++) p[k] = -1;
}

// the 3 x 3 (y, x) neighbours in plane p of the node at (y, x) (node run s
// of row run c); pl[4] is the node itself, pl[3 j + q] the node at
// (y + j - 1, x + q - 1)
__device__ void ag_plane(const AGrid& g, int p, int c, int s, int* pl, int y, int x) {
  const int l1 = g.l1;
  const ACRun C = g.C[c];
  ag_column(g, c, s, pl + 3, y, x);
  // row y + 1
  if (y < C.y0 + C.len - 1) {
    const int s1 = ag_find_nseg(g, ag_row_of(g, c, y + 1), x);
    if (s1 >= 0) { pl[7] = ag_node_at(g, s1, x); ag_column(g, c, s1, pl + 6, y + 1, x); }
    else ag_null3(pl + 6);
  } else if (y == l1 - 1) {
    const int c1 = g.pl[p].c0;
    if (g.C[c1].y0 == 0) {
      const int s1 = ag_find_nseg(g, g.C[c1].r0, x);
      if (s1 >= 0) { pl[7] = ag_node_at(g, s1, x); ag_column(g, c1, s1, pl + 6, 0, x); }
      else ag_null3(pl + 6);
    } else ag_null3(pl + 6);
  } else ag_null3(pl + 6);
  // row y - 1
  if (y > C.y0) {
    const int s1 = ag_find_nseg(g, ag_row_of(g, c, y - 1), x);
    if (s1 >= 0) { pl[1] = ag_node_at(g, s1, x); ag_column(g, c, s1, pl, y - 1, x); }
    else ag_null3(pl);
  } else if (y == 0) {
    const int c1 = ag_find_cseg(g, p, l1 - 1);
    if (c1 >= 0) {
      const int s1 = ag_find_nseg(g, ag_row_of(g, c1, l1 - 1), x);
      if (s1 >= 0) { pl[1] = ag_node_at(g, s1, x); ag_column(g, c1, s1, pl, l1 - 1, x); }
      else ag_null3(pl);
    } else ag_null3(pl);
  } else ag_null3(pl);
}

// a neighbour plane p2: the node at (y, x) through its row runs and node
// runs, then its plane of neighbours
__device__ void ag_other_plane(const AGrid& g, int p2, int* pl, int y, int x) {
  const int c2 = ag_find_cseg(g, p2, y);
  if (c2 < 0) { ag_null9(pl); return; }
  const int s2 = ag_find_nseg(g, ag_row_of(g, c2, y), x);
  if (s2 < 0) { ag_null9(pl); return; }
  pl[4] = ag_node_at(g, s2, x);
  ag_plane(g, p2, c2, s2, pl, y, x);
}

// the 27 TSC nodes of node i: t[9 k + 3 j + q] at (z + k - 1, y + j - 1,
// x + q - 1), -1 where the reference finds none
__device__ void ag_tsc_nodes(const AGrid& g, int i, int* t) {
  const int l1 = g.l1, s = g.nseg[i];
  const ANRun S = g.N[s];
  const ARow R = g.R[S.row];
  const int p = R.pl, c = R.cq;
  const APlane PL = g.pl[p];
  const APRun Q = g.P[PL.pq];
  const int z = PL.z, y = R.y, x = S.x0 + (i - S.n0);
  t[13] = i;
  ag_plane(g, p, c, s, t + 9, y, x);
  // plane z - 1
  if (z > Q.z0) ag_other_plane(g, p - 1, t, y, x);
  else if (z == 0) {
    int q = 0;
    while (l1 - 1 >= g.P[q].z0 + g.P[q].len && q + 1 < g.nP) q++;
    if (l1 - 1 >= g.P[q].z0 && l1 - 1 < g.P[q].z0 + g.P[q].len)
      ag_other_plane(g, g.P[q].pl0 + (l1 - 1 - g.P[q].z0), t, y, x);
    else ag_null9(t);
  } else ag_null9(t);
  // plane z + 1
  if (z < Q.z0 + Q.len - 1) ag_other_plane(g, p + 1, t + 18, y, x);
  else if (z == l1 - 1) {
    if (g.P[0].z0 == 0) ag_other_plane(g, g.P[0].pl0, t + 18, y, x);
    else ag_null9(t + 18);
  } else ag_null9(t + 18);
}

// flag bits of a node
constexpr uint8_t kAgTest = 1;   // test_node: refine around it
constexpr uint8_t kAgAll = 2;    // all 27 TSC nodes exist

__global__ void __launch_bounds__(kAgT) k_ag_tsc(AGrid g, int* __restrict__ tsc, uint8_t* __restrict__ flag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.nn) return;
  int t[27];
  ag_tsc_nodes(g, i, t);
  bool all = true;
  for (int k = 0; k < 27; k++) {
    tsc[(int64_t)i * 27 + k] = t[k];
    all = all && t[k] >= 0;
  }
  flag[i] = all ? kAgAll : 0;
}

__global__ void __launch_bounds__(kAgT) k_ag_test(int nn, const int* __restrict__ tsc, const float* __restrict__ dens,
                                                  double thr, uint8_t* __restrict__ flag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nn) return;
  uint8_t f = flag[i] & kAgAll;
  if (f) {
    const int* t = tsc + (int64_t)i * 27;
    bool hit = false;
    for (int k = 0; k < 3 && !hit; k++)
      for (int j = 0; j < 3 && !hit; j++)
        for (int q = 1; q < 3 && !hit; q++) hit = (double)dens[t[9 * k + 3 * j + q]] >= thr;
    if (hit) f |= kAgTest;
  }
  flag[i] = f;
}

// ---------------------------------------------------------------------------
// the refinement state machines

// ref_nquad over the node runs of coarse row r: the fine node runs (x0, len)
// it emits, in order; returns whether the row refines.  Counts when out is
// null.
__device__ bool ag_row_machine(const AGrid& g, const uint8_t* __restrict__ flag, int r, int2* out, int* nrun,
                               int* nnode) {
  const int l1 = g.l1;
  const ARow R = g.R[r];
  const int last = R.s0 + R.ns - 1;
  bool any = false;
  int cnt = 0, nodes = 0;
  auto emit = [&](int start, int len) {
    if (out) out[cnt] = make_int2(start, len);
    cnt++;
    nodes += len;
  };
  for (int s = R.s0; s <= last; s++) {
    const ANRun S = g.N[s];
    bool state = false, refever = false;
    int xlen = 0, start = 0, xoffset = 1;
    if (S.x0 == 0) {
      const ANRun L = g.N[last];
      if (L.x0 + L.len == l1) {
        if (L.len > 0 && (flag[L.n0 + L.len - 1] & kAgTest)) { state = true; refever = true; start = 0; }
        xoffset = 0;
      }
    }
    int idx = xoffset;
    for (; idx < S.len - 1; idx++) {
      const int i = S.n0 + idx, x = S.x0 + idx;
      if (flag[i] & kAgTest) {
        if (!state) { state = true; refever = true; start = 2 * x; }
        xlen += 2;
      } else if (state) {
        state = false;
        if (flag[i] & kAgAll) xlen += 2;
        emit(start, xlen);
        xlen = 0;
      }
    }
    const int xe = S.x0 + idx;
    if (s < last) {
      if (state) emit(start, xlen);
    } else if (S.x0 + S.len == l1 && idx < S.len && (flag[S.n0 + idx] & kAgTest)) {
      if (!state) { refever = true; start = 2 * xe; }
      xlen += 2;
      emit(start, xlen);
    } else if (state) {
      emit(start, xlen);
    }
    any = any || refever;
  }
  *nrun = cnt;
  *nnode = nodes;
  return any;
}

__global__ void __launch_bounds__(kAgT) k_ag_rows(AGrid g, const uint8_t* __restrict__ flag, uint32_t* __restrict__ nrun,
                                                  uint32_t* __restrict__ nnode, uint8_t* __restrict__ rref) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= g.nR) return;
  int a, b;
  rref[r] = ag_row_machine(g, flag, r, nullptr, &a, &b) ? 1 : 0;
  nrun[r] = (uint32_t)a;
  nnode[r] = (uint32_t)b;
}

__global__ void __launch_bounds__(kAgT) k_ag_rows_emit(AGrid g, const uint8_t* __restrict__ flag,
                                                       const uint32_t* __restrict__ run_off, int2* __restrict__ runs) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= g.nR) return;
  int a, b;
  ag_row_machine(g, flag, r, runs + run_off[r], &a, &b);
}

// ref_cquad over the row runs of coarse plane p: the fine row runs (y0,
// rows) and the refined coarse rows, in order; returns whether the plane
// refines.  Whether rows wrap periodically is judged from the first and last
// row runs of the first plane of p's plane run, as the reference does.
__device__ bool ag_plane_machine(const AGrid& g, const uint8_t* __restrict__ rref, const uint32_t* __restrict__ rrun,
                                 const uint32_t* __restrict__ rnode, int p, int2* rr_out, int* sel_out,
                                 APlaneOut* o) {
  const int l1 = g.l1;
  const APlane P = g.pl[p];
  const APlane P0 = g.pl[g.P[P.pq].pl0];
  const ACRun fst = g.C[P0.c0], lst = g.C[P0.c0 + P0.nc - 1];
  bool any = false;
  uint32_t nc = 0, nsel = 0, nrun = 0, nnode = 0;
  auto open = [&](int y0) {
    if (rr_out) rr_out[nc] = make_int2(y0, 0);
    nc++;
  };
  auto add = [&](int r) {
    if (sel_out) sel_out[nsel] = r;
    if (rr_out) rr_out[nc - 1].y += 2;
    nsel++;
    nrun += rrun[r];
    nnode += rnode[r];
  };
  const int clast = P.c0 + P.nc - 1;
  for (int c = P.c0; c <= clast; c++) {
    const ACRun C = g.C[c];
    int ylow = 1, yup = -1;
    if (fst.y0 == 0 && lst.y0 + lst.len == l1) {
      if (C.y0 == 0 && C.y0 + C.len == l1) { ylow = 0; yup = 0; }
      else if (C.y0 == 0) { ylow = 0; yup = -1; }
      else if (C.y0 + C.len == l1) { ylow = 1; yup = 0; }
    }
    bool state = false, refever = false;
    int idx = ylow;
    for (; idx < C.len - 1 + yup; idx++) {
      const int y = C.y0 + idx, r = C.r0 + idx;
      if (rref[r]) {
        if (!state) { state = true; refever = true; open(2 * y); }
        add(r);
      } else if (state) {
        state = false;
      }
    }
    const int ye = C.y0 + idx;
    if (c < clast) {
      // the next row run starts afresh
    } else if (C.y0 + C.len == l1 && idx < C.len) {
      const int r = C.r0 + idx;
      if (rref[r]) {
        if (!state) { refever = true; open(2 * ye); }
        add(r);
      }
    }
    any = any || refever;
  }
  o->nc = nc;
  o->nsel = nsel;
  o->nrun = nrun;
  o->nnode = nnode;
  return any;
}

__global__ void __launch_bounds__(kAgT) k_ag_planes(AGrid g, const uint8_t* __restrict__ rref,
                                                    const uint32_t* __restrict__ rrun,
                                                    const uint32_t* __restrict__ rnode, uint8_t* __restrict__ pref,
                                                    APlaneOut* __restrict__ po, uint32_t* __restrict__ pnc,
                                                    uint32_t* __restrict__ pnsel) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= g.npl) return;
  APlaneOut o;
  pref[p] = ag_plane_machine(g, rref, rrun, rnode, p, nullptr, nullptr, &o) ? 1 : 0;
  po[p] = o;
  pnc[p] = o.nc;
  pnsel[p] = o.nsel;
}

__global__ void __launch_bounds__(kAgT) k_ag_planes_emit(AGrid g, const uint8_t* __restrict__ rref,
                                                         const uint32_t* __restrict__ rrun,
                                                         const uint32_t* __restrict__ rnode,
                                                         const uint32_t* __restrict__ rr_off,
                                                         const uint32_t* __restrict__ sel_off, int2* __restrict__ rr,
                                                         int* __restrict__ sel) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= g.npl) return;
  APlaneOut o;
  ag_plane_machine(g, rref, rrun, rnode, p, rr + rr_off[p], sel + sel_off[p], &o);
}

// ref_pquad over the plane runs of the coarse grid (one thread): the fine
// planes (2 z, 2 z + 1 of each refined coarse plane) in order with their
// plane runs, and the offsets of every fine plane's row runs, rows, node
// runs and nodes
__global__ void k_ag_pquad(AGrid g, const uint8_t* __restrict__ pref, const APlaneOut* __restrict__ po,
                           APRun* __restrict__ fP, AFPlane* __restrict__ fpl, AFineTotals* __restrict__ tot) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  const int l1 = g.l1;
  const APRun fst = g.P[0], lst = g.P[g.nP - 1];
  int nP = 0, npl = 0;
  int64_t nC = 0, nR = 0, nN = 0, nn = 0;
  bool any = false;
  auto fopen = [&](int z0) {
    fP[nP].z0 = z0;
    fP[nP].len = 0;
    fP[nP].pl0 = npl;
    fP[nP].pad = 0;
    nP++;
  };
  auto fplane = [&](int z, int p) {
    const APlaneOut o = po[p];
    AFPlane f;
    f.z = z; f.cp = p; f.pq = nP - 1;
    f.c0 = (int)nC; f.r0 = (int)nR; f.s0 = (int)nN; f.n0 = (int)nn; f.pad = 0;
    fpl[npl++] = f;
    fP[nP - 1].len++;
    nC += o.nc;
    nR += 2 * (int64_t)o.nsel;
    nN += 2 * (int64_t)o.nrun;
    nn += 2 * (int64_t)o.nnode;
  };
  for (int q = 0; q < g.nP; q++) {
    const APRun Q = g.P[q];
    int zlow = 1, zup = -1;
    if (fst.z0 == 0 && lst.z0 + lst.len == l1) {
      if (Q.z0 == 0 && Q.z0 + Q.len == l1) { zlow = 0; zup = 0; }
      else if (Q.z0 == 0) { zlow = 0; zup = -1; }
      else if (Q.z0 + Q.len == l1) { zlow = 1; zup = 0; }
    }
    bool state = false, refever = false;
    int idx = zlow;
    for (; idx < Q.len - 1 + zup; idx++) {
      const int z = Q.z0 + idx, p = Q.pl0 + idx;
      if (pref[p]) {
        if (!state) { state = true; refever = true; fopen(2 * z); }
        fplane(2 * z, p);
        fplane(2 * z + 1, p);
      } else if (state) {
        state = false;
      }
    }
    const int ze = Q.z0 + idx;
    if (q < g.nP - 1) {
      // the next plane run starts afresh
    } else if (Q.z0 + Q.len == l1 && idx < Q.len) {
      const int p = Q.pl0 + idx;
      if (pref[p]) {
        if (!state) { refever = true; fopen(2 * ze); }
        fplane(2 * ze, p);
        fplane(2 * ze + 1, p);
      }
    }
    any = any || refever;
  }
  tot->refined = any ? 1 : 0;
  tot->nP = nP;
  tot->npl = npl;
  tot->err = (nC > 0x7fffffff || nR > 0x7fffffff || nN > 0x7fffffff || nn > 0x7fffffff) ? 1 : 0;
  tot->nC = (int)nC;
  tot->nR = (int)nR;
  tot->nN = (int)nN;
  tot->nn = (int)nn;
}

// the fine grid's planes, row runs, rows and node runs: one thread per fine
// plane copies its coarse plane's refined rows (each twice, as rows 2 y and
// 2 y + 1) with their fine node runs
__global__ void __launch_bounds__(kAgT) k_ag_fplanes(int npl_f, const AFPlane* __restrict__ fpl,
                                                     const uint32_t* __restrict__ rr_off,
                                                     const uint32_t* __restrict__ sel_off,
                                                     const APlaneOut* __restrict__ po, const int2* __restrict__ rr,
                                                     const int* __restrict__ sel, const AGrid gc,
                                                     const uint32_t* __restrict__ run_off,
                                                     const int2* __restrict__ runs, APlane* __restrict__ pl,
                                                     ACRun* __restrict__ C, ARow* __restrict__ R,
                                                     ANRun* __restrict__ N) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= npl_f) return;
  const AFPlane F = fpl[f];
  const APlaneOut o = po[F.cp];
  pl[f] = APlane{F.z, F.pq, F.c0, (int)o.nc};
  int row = F.r0, nrun = F.s0, node = F.n0;
  const int2* myrr = rr + rr_off[F.cp];
  const int* mysel = sel + sel_off[F.cp];
  int k = 0;   // selected coarse row
  for (uint32_t c = 0; c < o.nc; c++) {
    const int2 cr = myrr[c];   // (fine y0, fine rows)
    C[F.c0 + c] = ACRun{cr.x, cr.y, row, f};
    for (int h = 0; h < cr.y / 2; h++, k++) {
      const int r = mysel[k];
      const int y = gc.R[r].y;
      const int2* rruns = runs + run_off[r];
      const int nr = (int)(run_off[r + 1] - run_off[r]);
      for (int half = 0; half < 2; half++) {
        ARow Rw;
        Rw.y = 2 * y + half; Rw.pl = f; Rw.cq = F.c0 + (int)c; Rw.s0 = nrun; Rw.ns = nr;
        Rw.pad0 = Rw.pad1 = Rw.pad2 = 0;
        R[row] = Rw;
        for (int s = 0; s < nr; s++) {
          N[nrun] = ANRun{rruns[s].x, rruns[s].y, node, row};
          node += rruns[s].y;
          nrun++;
        }
        row++;
      }
    }
  }
}

// the nodes of every fine node run: key and run
__global__ void __launch_bounds__(kAgT) k_ag_fnodes(int nN, int l1, const ANRun* __restrict__ N,
                                                    const ARow* __restrict__ R, const APlane* __restrict__ pl,
                                                    uint64_t* __restrict__ key, int* __restrict__ nseg) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nN) return;
  const ANRun S = N[s];
  const ARow Rw = R[S.row];
  const uint64_t base = ((uint64_t)pl[Rw.pl].z * (uint64_t)l1 + (uint64_t)Rw.y) * (uint64_t)l1;
  for (int k = 0; k < S.len; k++) {
    key[S.n0 + k] = base + (uint64_t)(S.x0 + k);
    nseg[S.n0 + k] = s;
  }
}

// the domain grid as runs: one plane run of l1 planes, each plane one row
// run of l1 rows, each row one node run of l1 nodes
__global__ void __launch_bounds__(kAgT) k_ag_domain(int l1, APRun* __restrict__ P, APlane* __restrict__ pl,
                                                    ACRun* __restrict__ C, ARow* __restrict__ R,
                                                    ANRun* __restrict__ N, uint64_t* __restrict__ key,
                                                    int* __restrict__ nseg) {
  const int64_t nn = (int64_t)l1 * l1 * l1;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) P[0] = APRun{0, l1, 0, 0};
  if (i < l1) {
    pl[i] = APlane{(int)i, 0, (int)i, 1};
    C[i] = ACRun{0, l1, (int)i * l1, (int)i};
  }
  if (i < (int64_t)l1 * l1) {
    const int z = (int)(i / l1), y = (int)(i % l1);
    ARow Rw;
    Rw.y = y; Rw.pl = z; Rw.cq = z; Rw.s0 = (int)i; Rw.ns = 1; Rw.pad0 = Rw.pad1 = Rw.pad2 = 0;
    R[i] = Rw;
    N[i] = ANRun{0, l1, (int)(i * l1), (int)i};
  }
  if (i < nn) {
    key[i] = (uint64_t)i;
    nseg[i] = (int)(i / l1);
  }
}

// ---------------------------------------------------------------------------
// relink

// the node of key `want` (keys ascend with the node index), or -1
__device__ __forceinline__ int ag_find_key(const uint64_t* __restrict__ key, int nn, uint64_t want) {
  int lo = 0, hi = nn;   // first key >= want
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (key[mid] < want) lo = mid + 1;
    else hi = mid;
  }
  return (lo < nn && key[lo] == want) ? lo : -1;
}

// the first child of every refined coarse node, with the nodes of its fine
// row and plane: a fine node with even (z, y, x) is child (0, 0, 0) of the
// coarse node at half its coordinates.  child[c] = {i0, R, P, 0}; i0 = -1
// where the coarse node is not refined (set before the launch).
__global__ void __launch_bounds__(kAgT) k_ag_child0(AGrid gf, const uint64_t* __restrict__ ckey, int nnc,
                                                    int4* __restrict__ child) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= gf.nn) return;
  const uint64_t k = gf.key[i], L = (uint64_t)gf.l1;
  const uint64_t x = k % L, y = (k / L) % L, z = k / (L * L);
  if ((x | y | z) & 1ull) return;
  const uint64_t Lc = L / 2;
  const uint64_t want = ((z / 2) * Lc + y / 2) * Lc + x / 2;
  const int c = ag_find_key(ckey, nnc, want);
  if (c < 0) return;
  const ARow Rw = gf.R[gf.N[gf.nseg[i]].row];
  const ANRun Rl = gf.N[Rw.s0 + Rw.ns - 1];
  const int rlen = Rl.n0 + Rl.len - gf.N[Rw.s0].n0;
  const APlane Pl = gf.pl[Rw.pl];
  const ACRun C0 = gf.C[Pl.c0], C1 = gf.C[Pl.c0 + Pl.nc - 1];
  const ARow Rf = gf.R[C0.r0], Rz = gf.R[C1.r0 + C1.len - 1];
  const ANRun Pz = gf.N[Rz.s0 + Rz.ns - 1];
  const int plen = Pz.n0 + Pz.len - gf.N[Rf.s0].n0;
  child[c] = make_int4(i, rlen, plen, 0);
}

// the fine node each listed particle of the coarse grid moves to, or -1.
// Slot k of the coarse lists holds particle ord[k] of coarse node cnode[k].
// The children of a refined node are a 2 x 2 x 2 block (fine node runs
// start and end on even x, fine rows and planes come in identical pairs), so
// child (a, b, c) is i0 + a P + b R + c, i0 the first child, R and P the
// nodes of its fine row and plane; each child is checked against its key and
// searched for where that layout would not give it.  i0, R and P come from
// the coarse nodes' child table (k_ag_child0): the particles are in coarse
// node order, so neighbouring threads read the same entries.
__global__ void __launch_bounds__(kAgT) k_ag_relink(uint32_t np, const uint32_t* __restrict__ ord,
                                                    const uint64_t* __restrict__ cnode,
                                                    const uint64_t* __restrict__ ckey, int l1c, AGrid gf,
                                                    const int4* __restrict__ child, const double* __restrict__ cen,
                                                    const uint8_t* __restrict__ fflag, const float* __restrict__ x,
                                                    const float* __restrict__ y, const float* __restrict__ z,
                                                    int* __restrict__ dest, uint32_t* __restrict__ moved) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= np) return;
  const uint64_t ck = ckey ? ckey[cnode[k]] : cnode[k];
  const uint64_t L = (uint64_t)l1c;
  const int cx = (int)(ck % L), cy = (int)((ck / L) % L), cz = (int)(ck / (L * L));
  const int l1f = 2 * l1c;
  const uint64_t Lf = (uint64_t)l1f;
  const double dl = (double)l1f, shift = 0.5 / dl;
  const uint64_t base = ((uint64_t)(2 * cz) * Lf + (uint64_t)(2 * cy)) * Lf + (uint64_t)(2 * cx);
  int to = -1;
  const int4 ch = child[cnode[k]];
  const int i0 = ch.x;
  if (i0 >= 0) {
    const int rlen = ch.y, plen = ch.z;
    const uint32_t p = ord[k];
    const double px = (double)x[p], py = (double)y[p], pz = (double)z[p];
    for (int a = 0; a < 2 && to < 0; a++)
      for (int b = 0; b < 2 && to < 0; b++)
        for (int c = 0; c < 2 && to < 0; c++) {
          const uint64_t want = base + ((uint64_t)a * Lf + (uint64_t)b) * Lf + (uint64_t)c;
          int i = i0 + a * plen + b * rlen + c;
          if (i >= gf.nn || gf.key[i] != want) i = ag_find_key(gf.key, gf.nn, want);
          if (i < 0 || !(fflag[i] & kAgAll)) continue;
          const int fz = 2 * cz + a, fy = 2 * cy + b, fx = 2 * cx + c;
          if (fabs(px - cen[fx]) <= shift && fabs(py - cen[fy]) <= shift && fabs(pz - cen[fz]) <= shift) to = i;
        }
  }
  dest[k] = to;
  moved[k] = to >= 0 ? 1u : 0u;
}

// the moved particles as (fine node, particle) pairs at their scanned places
__global__ void __launch_bounds__(kAgT) k_ag_compact(uint32_t np, const int* __restrict__ dest,
                                                     const uint32_t* __restrict__ off, const uint32_t* __restrict__ ord,
                                                     uint64_t* __restrict__ fkey_out, uint32_t* __restrict__ fidx_out,
                                                     uint32_t* __restrict__ count) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= np || dest[k] < 0) return;
  const uint32_t o = off[k];
  fkey_out[o] = (uint64_t)dest[k];
  fidx_out[o] = ord[k];
  atomicAdd(&count[dest[k]], 1u);
}

// ---------------------------------------------------------------------------
// densities

__device__ __forceinline__ double ag_fold(double v) { return v >= 2.0 ? v - 2.0 : (v >= 1.0 ? v - 1.0 : v); }

__device__ __forceinline__ double ag_w(double sep, int o) {
  if (o == 0) return 0.75 - sep * sep;
  if (o < 0) return ((0.5 - sep) * (0.5 - sep)) / 2;
  return ((0.5 + sep) * (0.5 + sep)) / 2;
}

__device__ __forceinline__ double ag_sep(float p, double centre, double dl1) {
  double sep = ((double)p - centre) * dl1;
  if (fabs(sep) > 0.5 * dl1) {
    const double a = ag_fold(((double)p + 0.5) + 1.0);
    const double b = ag_fold((centre + 0.5) + 1.0);
    sep = (a - b) * dl1;
  }
  return sep;
}

// per grid index c of a level: the node centre c / l1 + 1 / (2 l1) (relink's
// half-cell test) and its fold((...) + 1) (the weights), formed as the
// reference forms them -- one FP64 division per index instead of several per
// particle
__global__ void __launch_bounds__(kAgT) k_ag_centres(int l1, double* __restrict__ cen, double* __restrict__ cfold) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= l1) return;
  const double dl = (double)l1, shift = 0.5 / dl;
  const double v = (double)c / dl + shift;
  cen[c] = v;
  cfold[c] = ag_fold(v + 1.0);
}

// each listed particle's TSC factors in list-slot order: w[3 oz + oy] =
// (m2d * w_z(oz - 1)) * w_y(oy - 1) and w[9 + ox] = w_x(ox - 1) at column
// o * np + k (the first two products of the reference's left-to-right
// m2d * w_z * w_y * w_x formed once)
__global__ void __launch_bounds__(kAgT) k_ag_weights(int l1, double m2d, uint32_t np, const uint64_t* __restrict__ node,
                                                     const uint64_t* __restrict__ nkey,
                                                     const uint32_t* __restrict__ ord, const float* __restrict__ x,
                                                     const float* __restrict__ y, const float* __restrict__ z,
                                                     const double* __restrict__ cfold, double* __restrict__ w) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= np) return;
  const double dl1 = (double)l1;
  const uint64_t key = nkey[node[k]];
  const uint64_t L = (uint64_t)l1;
  const int cx = (int)(key % L), cy = (int)((key / L) % L), cz = (int)(key / (L * L));
  const uint32_t i = ord[k];
  const double sx = ag_sep(x[i], cfold[cx], dl1);
  const double sy = ag_sep(y[i], cfold[cy], dl1);
  const double sz = ag_sep(z[i], cfold[cz], dl1);
  const uint64_t n = np;
#pragma unroll
  for (int oz = 0; oz < 3; oz++) {
    const double az = m2d * ag_w(sz, oz - 1);
#pragma unroll
    for (int oy = 0; oy < 3; oy++) w[(uint64_t)(3 * oz + oy) * n + k] = az * ag_w(sy, oy - 1);
  }
#pragma unroll
  for (int o = 0; o < 3; o++) w[(uint64_t)(9 + o) * n + k] = ag_w(sx, o - 1);
}

// The sources of a target.  Source s adds to the 27 nodes of its stencil;
// a target t reads the same relation back through its own stencil: the
// node s at t's slot j reaches t at s's mirrored slot 26 - j when
// tsc[s][26 - j] == t.  Where the run segmentation makes the relation
// one-sided (s finds t, t does not find s at the mirrored slot), the pair is
// an "extra" of t, listed per target here: pass 0 counts them per target,
// pass 1 writes (s, slot) at the target's scanned place (in any order; the
// density kernel orders every target's sources by node index).
__global__ void __launch_bounds__(kAgT) k_ag_extras(int nn, const uint32_t* __restrict__ start,
                                                    const int* __restrict__ tsc, int pass,
                                                    uint32_t* __restrict__ ecount, const uint32_t* __restrict__ eoff,
                                                    uint32_t* __restrict__ efill, uint64_t* __restrict__ extra) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nn || start[s + 1] == start[s]) return;
  for (int k = 0; k < 27; k++) {
    const int t = tsc[(int64_t)s * 27 + k];
    if (t < 0 || tsc[(int64_t)t * 27 + (26 - k)] == s) continue;
    if (pass == 0) atomicAdd(&ecount[t], 1u);
    else extra[eoff[t] + atomicAdd(&efill[t], 1u)] = (uint64_t)s * 32u + (uint64_t)k;
  }
}

// One warp per target: -1, then its sources in node order, each source's
// particles in list order (descending slots when `desc`).  Lane j < 27 takes
// the node at the target's stencil slot j when it has particles: such a node
// has all 27 of its TSC nodes (relink moves particles only into those), so
// its own slot 26 - j is the node at the target's coordinates, the target.
// The listed one-sided sources follow; the candidates are ranked by node
// index (a target has at most 27 sources, one per stencil position), laid
// out in shared memory with their term offsets, and summed by amr_warp_sum.
__global__ void __launch_bounds__(kAgT) k_ag_dens(int nn, const int* __restrict__ tsc,
                                                  const uint32_t* __restrict__ eoff,
                                                  const uint64_t* __restrict__ extra,
                                                  const uint32_t* __restrict__ start, const double* __restrict__ w,
                                                  uint32_t np, int desc, float* __restrict__ dens,
                                                  int* __restrict__ err) {
  __shared__ AmrSrc sh[kAgT / 32][32];
  __shared__ int cs[kAgT / 32][32];
  __shared__ uint32_t ck[kAgT / 32][32];
  const unsigned FULL = 0xffffffffu, lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
  const int t = (int)(blockIdx.x * (kAgT / 32) + wid);
  if (t >= nn) return;   // uniform over the warp
  int s = -1;
  uint32_t slot = 0;
  if (lane < 27u) {
    const int c = tsc[(int64_t)t * 27 + lane];
    if (c >= 0 && start[c + 1] > start[c]) {
      s = c;
      slot = 26u - lane;
    }
  }
  const unsigned reg = __ballot_sync(FULL, s >= 0);
  const int nreg = __popc(reg);
  if (s >= 0) {
    const int at = __popc(reg & ((1u << lane) - 1u));
    cs[wid][at] = s;
    ck[wid][at] = slot;
  }
  const uint32_t e0 = eoff[t], ne = eoff[t + 1] - e0;
  int total = nreg + (int)ne;
  if (total > 27) {
    if (lane == 0u) atomicExch(err, 1);
    total = 27;
  }
  if ((int)lane < total - nreg) {
    const uint64_t e = extra[e0 + lane];
    cs[wid][nreg + (int)lane] = (int)(e >> 5);
    ck[wid][nreg + (int)lane] = (uint32_t)(e & 31u);
  }
  __syncwarp();
  // rank by node index (distinct), the source's slots, then term offsets
  uint32_t s0 = 0, cnt = 0;
  int rank = 0, my = -1;
  uint32_t myslot = 0;
  // the stencil slots give ascending node indices unless the stencil
  // crosses a periodic face (or extras were appended): rank only then
  const bool inorder = (int)lane + 1 >= total || cs[wid][lane] < cs[wid][lane + 1];
  const bool sorted = __all_sync(FULL, inorder);
  if ((int)lane < total) {
    my = cs[wid][lane];
    myslot = ck[wid][lane];
    if (sorted) rank = (int)lane;
    else
      for (int k = 0; k < total; k++) rank += cs[wid][k] < my ? 1 : 0;
    s0 = start[my];
    cnt = start[my + 1] - s0;
  }
  // counts in rank order: each lane reads the count of the rank-th source
  __syncwarp();
  if ((int)lane < total) ck[wid][rank] = cnt;
  __syncwarp();
  uint32_t rc = (int)lane < total ? ck[wid][lane] : 0u;
  uint32_t inc = rc;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const uint32_t v = __shfl_up_sync(FULL, inc, off);
    if ((int)lane >= off) inc += v;
  }
  const uint32_t cum_rank = inc - rc;   // term offset of the source of rank `lane`
  const uint32_t nterm = __shfl_sync(FULL, inc, 31);
  // each source's entry at its rank, with the offset of that rank
  const uint32_t mycum = __shfl_sync(FULL, cum_rank, rank & 31);
  if ((int)lane < total) sh[wid][rank] = AmrSrc{s0, cnt, myslot, mycum};
  __syncwarp();
  float d = (float)(-1.0);
  if (nterm) d = desc ? amr_warp_sum<true>(sh[wid], total, nterm, w, np)
                      : amr_warp_sum<false>(sh[wid], total, nterm, w, np);
  if (lane == 0u) dens[t] = d;
}

// node coordinates (z, y, x) from the keys
__global__ void __launch_bounds__(kAgT) k_ag_zyx(int nn, int l1, const uint64_t* __restrict__ key,
                                                 int32_t* __restrict__ zyx) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nn) return;
  const uint64_t k = key[i], L = (uint64_t)l1;
  zyx[3 * (int64_t)i] = (int32_t)(k / (L * L));
  zyx[3 * (int64_t)i + 1] = (int32_t)((k / L) % L);
  zyx[3 * (int64_t)i + 2] = (int32_t)(k % L);
}

// ---------------------------------------------------------------------------
// launch wrappers

static unsigned ag_blocks(int64_t n) { return (unsigned)((n + kAgT - 1) / kAgT); }

void ag_domain(int l1, APRun* P, APlane* pl, ACRun* C, ARow* R, ANRun* N, uint64_t* key, int* nseg,
               cudaStream_t st) {
  k_ag_domain<<<ag_blocks((int64_t)l1 * l1 * l1), kAgT, 0, st>>>(l1, P, pl, C, R, N, key, nseg);
}

void ag_tsc(const AGrid& g, int* tsc, uint8_t* flag, cudaStream_t st) {
  if (g.nn > 0) k_ag_tsc<<<ag_blocks(g.nn), kAgT, 0, st>>>(g, tsc, flag);
}

void ag_test(int nn, const int* tsc, const float* dens, double thr, uint8_t* flag, cudaStream_t st) {
  if (nn > 0) k_ag_test<<<ag_blocks(nn), kAgT, 0, st>>>(nn, tsc, dens, thr, flag);
}

void ag_rows(const AGrid& g, const uint8_t* flag, uint32_t* nrun, uint32_t* nnode, uint8_t* rref, cudaStream_t st) {
  if (g.nR > 0) k_ag_rows<<<ag_blocks(g.nR), kAgT, 0, st>>>(g, flag, nrun, nnode, rref);
}

void ag_rows_emit(const AGrid& g, const uint8_t* flag, const uint32_t* run_off, int2* runs, cudaStream_t st) {
  if (g.nR > 0) k_ag_rows_emit<<<ag_blocks(g.nR), kAgT, 0, st>>>(g, flag, run_off, runs);
}

void ag_planes(const AGrid& g, const uint8_t* rref, const uint32_t* rrun, const uint32_t* rnode, uint8_t* pref,
               APlaneOut* po, uint32_t* pnc, uint32_t* pnsel, cudaStream_t st) {
  if (g.npl > 0) k_ag_planes<<<ag_blocks(g.npl), kAgT, 0, st>>>(g, rref, rrun, rnode, pref, po, pnc, pnsel);
}

void ag_planes_emit(const AGrid& g, const uint8_t* rref, const uint32_t* rrun, const uint32_t* rnode,
                    const uint32_t* rr_off, const uint32_t* sel_off, int2* rr, int* sel, cudaStream_t st) {
  if (g.npl > 0)
    k_ag_planes_emit<<<ag_blocks(g.npl), kAgT, 0, st>>>(g, rref, rrun, rnode, rr_off, sel_off, rr, sel);
}

void ag_pquad(const AGrid& g, const uint8_t* pref, const APlaneOut* po, APRun* fP, AFPlane* fpl, AFineTotals* tot,
              cudaStream_t st) {
  k_ag_pquad<<<1, 32, 0, st>>>(g, pref, po, fP, fpl, tot);
}

void ag_fplanes(int npl_f, const AFPlane* fpl, const uint32_t* rr_off, const uint32_t* sel_off, const APlaneOut* po,
                const int2* rr, const int* sel, const AGrid& gc, const uint32_t* run_off, const int2* runs,
                APlane* pl, ACRun* C, ARow* R, ANRun* N, cudaStream_t st) {
  if (npl_f > 0)
    k_ag_fplanes<<<ag_blocks(npl_f), kAgT, 0, st>>>(npl_f, fpl, rr_off, sel_off, po, rr, sel, gc, run_off, runs, pl,
                                                     C, R, N);
}

void ag_fnodes(int nN, int l1, const ANRun* N, const ARow* R, const APlane* pl, uint64_t* key, int* nseg,
               cudaStream_t st) {
  if (nN > 0) k_ag_fnodes<<<ag_blocks(nN), kAgT, 0, st>>>(nN, l1, N, R, pl, key, nseg);
}

void ag_child0(const AGrid& gf, const uint64_t* ckey, int nnc, int4* child, cudaStream_t st) {
  if (gf.nn > 0) k_ag_child0<<<ag_blocks(gf.nn), kAgT, 0, st>>>(gf, ckey, nnc, child);
}

void ag_relink(uint32_t np, const uint32_t* ord, const uint64_t* cnode, const uint64_t* ckey, int l1c,
               const AGrid& gf, const int4* child, const double* cen, const uint8_t* fflag, const float* x,
               const float* y, const float* z, int* dest, uint32_t* moved, cudaStream_t st) {
  if (np > 0)
    k_ag_relink<<<ag_blocks(np), kAgT, 0, st>>>(np, ord, cnode, ckey, l1c, gf, child, cen, fflag, x, y, z, dest,
                                                 moved);
}

void ag_compact(uint32_t np, const int* dest, const uint32_t* off, const uint32_t* ord, uint64_t* fkey_out,
                uint32_t* fidx_out, uint32_t* count, cudaStream_t st) {
  if (np > 0) k_ag_compact<<<ag_blocks(np), kAgT, 0, st>>>(np, dest, off, ord, fkey_out, fidx_out, count);
}

void ag_centres(int l1, double* cen, double* cfold, cudaStream_t st) {
  if (l1 > 0) k_ag_centres<<<ag_blocks(l1), kAgT, 0, st>>>(l1, cen, cfold);
}

void ag_weights(int l1, double m2d, uint32_t np, const uint64_t* node, const uint64_t* nkey, const uint32_t* ord,
                const float* x, const float* y, const float* z, const double* cfold, double* w, cudaStream_t st) {
  if (np > 0) k_ag_weights<<<ag_blocks(np), kAgT, 0, st>>>(l1, m2d, np, node, nkey, ord, x, y, z, cfold, w);
}

void ag_extras(int nn, const uint32_t* start, const int* tsc, int pass, uint32_t* ecount, const uint32_t* eoff,
               uint32_t* efill, uint64_t* extra, cudaStream_t st) {
  if (nn > 0) k_ag_extras<<<ag_blocks(nn), kAgT, 0, st>>>(nn, start, tsc, pass, ecount, eoff, efill, extra);
}

void ag_dens(int nn, const int* tsc, const uint32_t* eoff, const uint64_t* extra, const uint32_t* start,
             const double* w, uint32_t np, int desc, float* dens, int* err, cudaStream_t st) {
  if (nn > 0)
    k_ag_dens<<<(unsigned)(((int64_t)nn + kAgT / 32 - 1) / (kAgT / 32)), kAgT, 0, st>>>(nn, tsc, eoff, extra, start, w,
                                                                                       np, desc, dens, err);
}

void ag_zyx(int nn, int l1, const uint64_t* key, int32_t* zyx, cudaStream_t st) {
  if (nn > 0) k_ag_zyx<<<ag_blocks(nn), kAgT, 0, st>>>(nn, l1, key, zyx);
}

}  // namespace ahfgpu
