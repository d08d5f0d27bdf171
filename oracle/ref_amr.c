/*
 * ref_amr.c -- TEST INFRASTRUCTURE ONLY (oracle/_ref/libahfref_amr.so).
 *
 * Runs the reference's own AMR hierarchy on a snapshot given as float
 * positions, the way src/main.c:614-648 sets it up: the domain grids
 * (gen_domgrids, libamr_serial/generate_grids.c:24), the particles linked to
 * the domain grid (ll, libamr_serial/lltools.c:32), their number density on
 * it (zero_dens / assign_npart, libamr_serial/density.c), then the recursive
 * refinement (gen_AMRhierarchy, generate_grids.c:278) under the NperDomCell /
 * NperRefCell criteria.  All reference sources are compiled unchanged.
 *
 * Result per grid of the hierarchy: its nodes per dimension (l1dim), the
 * number of nodes it holds and the number of particles assigned to it
 * (gridls.size.no_nodes / no_part, as assign_npart leaves them).  This is the
 * oracle of the AMR-hierarchy row; the haloes built from the hierarchy come
 * after ahf_gridinfo and are not reported here.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "common.h"
#include "libamr_serial/amr_serial.h"

/* globals normally defined in src/common.c and src/main.c */
info_timing   timing;
info_global   global;
info_io       io;
info_ahf      ahf;
info_energy   energy;
info_Pk       PkSpectrum;
info_gadget   gadget;
param_simu    simu;
global_io_t   global_io;
global_info_t global_info;
SRINDEX      *spatialRefIndex;
int          *numIsoRef;
int           totnumIsoRef;

/* levels[3 * g + 0..2] = l1dim, no_nodes, no_part of grid g; returns the
 * number of grids (at most max_levels reported) or a negative error */
int ahfref_amr_levels(uint64_t n, const float *x, const float *y, const float *z, int ngrid_dom, int ngrid_max,
                      double nth_dom, double nth_ref, int64_t *levels, int max_levels)
{
  FILE *log = fopen("/dev/null", "w");
  io.logfile = log ? log : stderr;
  partptr p = (partptr)calloc(n ? n : 1, sizeof(part));
  if (!p) return -1;
  for (uint64_t i = 0; i < n; i++) {
    p[i].pos[0] = x[i];
    p[i].pos[1] = y[i];
    p[i].pos[2] = z[i];
    p[i].id = (part_id_t)i;
  }
  simu.no_part = n;
  simu.no_vpart = (double)n;
  simu.NGRID_DOM = ngrid_dom;
  simu.NGRID_MIN = ngrid_dom;
  simu.NGRID_MAX = ngrid_max;
  simu.Nth_dom = nth_dom;
  simu.Nth_ref = nth_ref;
  simu.boxsize = 1.0;
  simu.mean_dens = 1.0;
  global.super_t = 1.0;
  global.fst_part = p;
  global.no_part = n;
  global_info.fst_part = p;
  global_info.no_part = n;

  int no_grids = 0;
  gridls *grid_list = gen_domgrids(&no_grids);
  ll(n, p, global.dom_grid);
  zero_dens(global.dom_grid);
  assign_npart(global.dom_grid);
  global.fst_cycle = TRUE;
  gen_AMRhierarchy(&grid_list, &no_grids);

  for (int g = 0; g < no_grids && g < max_levels; g++) {
    levels[3 * g + 0] = (int64_t)grid_list[g].l1dim;
    levels[3 * g + 1] = (int64_t)grid_list[g].size.no_nodes;
    levels[3 * g + 2] = (int64_t)grid_list[g].size.no_part;
  }
  /* the grids' quads are left to process exit: this harness runs once per
   * process (the reference frees them only at the end of a run) */
  free(p);
  global.fst_part = NULL;
  if (log) fclose(log);
  io.logfile = NULL;
  return no_grids;
}

/* The domain grid's node densities straight after assign_npart (TSC
 * assignment, libamr_serial/density.c:238-420), before any refinement:
 * dens[(z * l1 + y) * l1 + x] for the ngrid_dom^3 nodes, read from the
 * grid's quads.  Returns the number of nodes written, or a negative error. */
int64_t ahfref_domain_dens(uint64_t n, const float *x, const float *y, const float *z, int ngrid_dom,
                           double *dens)
{
  FILE *log = fopen("/dev/null", "w");
  io.logfile = log ? log : stderr;
  partptr p = (partptr)calloc(n ? n : 1, sizeof(part));
  if (!p) return -1;
  for (uint64_t i = 0; i < n; i++) {
    p[i].pos[0] = x[i];
    p[i].pos[1] = y[i];
    p[i].pos[2] = z[i];
    p[i].id = (part_id_t)i;
  }
  simu.no_part = n;
  simu.no_vpart = (double)n;
  simu.NGRID_DOM = ngrid_dom;
  simu.NGRID_MIN = ngrid_dom;
  simu.NGRID_MAX = ngrid_dom;
  simu.Nth_dom = 5.0;
  simu.Nth_ref = 5.0;
  simu.boxsize = 1.0;
  simu.mean_dens = 1.0;
  global.super_t = 1.0;
  int no_grids = 0;
  gridls *grid_list = gen_domgrids(&no_grids);
  gridls *g = global.dom_grid;
  ll(n, p, g);
  zero_dens(g);
  assign_npart(g);
  const long l1 = (long)g->l1dim;
  int64_t count = 0;
  for (pqptr pq = g->pquad; pq != NULL; pq = pq->next) {
    long zz = pq->z;
    for (cqptr cq = pq->loc; cq < pq->loc + pq->length; cq++, zz++)
      for (cqptr icq = cq; icq != NULL; icq = icq->next) {
        long yy = icq->y;
        for (nqptr nq = icq->loc; nq < icq->loc + icq->length; nq++, yy++)
          for (nqptr inq = nq; inq != NULL; inq = inq->next) {
            long xx = inq->x;
            for (nptr nd = inq->loc; nd < inq->loc + inq->length; nd++, xx++) {
              if (zz < 0 || zz >= l1 || yy < 0 || yy >= l1 || xx < 0 || xx >= l1) return -2;
              dens[(zz * l1 + yy) * l1 + xx] = (double)nd->dens;
              count++;
            }
          }
      }
  }
  (void)grid_list;
  free(p);
  if (log) fclose(log);
  io.logfile = NULL;
  return count;
}

/* The first refinement alone: the domain grid (ngrid_dom^3), its densities,
 * then gen_AMRhierarchy with NGRID_MAX = 2 ngrid_dom, so at most one finer
 * grid is made.  Its nodes' coordinates (fine-grid units) go to
 * zyx[3 k + 0..2] in the order of its quads.  Returns the number of nodes
 * (0 when nothing was refined), -3 when more than max_nodes. */
int64_t ahfref_first_refinement(uint64_t n, const float *x, const float *y, const float *z, int ngrid_dom,
                                double nth_dom, double nth_ref, int64_t *zyx, int64_t max_nodes)
{
  FILE *log = fopen("/dev/null", "w");
  io.logfile = log ? log : stderr;
  partptr p = (partptr)calloc(n ? n : 1, sizeof(part));
  if (!p) return -1;
  for (uint64_t i = 0; i < n; i++) {
    p[i].pos[0] = x[i];
    p[i].pos[1] = y[i];
    p[i].pos[2] = z[i];
    p[i].id = (part_id_t)i;
  }
  simu.no_part = n;
  simu.no_vpart = (double)n;
  simu.NGRID_DOM = ngrid_dom;
  simu.NGRID_MIN = ngrid_dom;
  simu.NGRID_MAX = 2 * ngrid_dom;
  simu.Nth_dom = nth_dom;
  simu.Nth_ref = nth_ref;
  simu.boxsize = 1.0;
  simu.mean_dens = 1.0;
  global.super_t = 1.0;
  global.fst_part = p;
  global.no_part = n;
  int no_grids = 0;
  gridls *grid_list = gen_domgrids(&no_grids);
  ll(n, p, global.dom_grid);
  zero_dens(global.dom_grid);
  assign_npart(global.dom_grid);
  global.fst_cycle = TRUE;
  gen_AMRhierarchy(&grid_list, &no_grids);
  int64_t count = 0;
  if (no_grids > 1) {
    gridls *g = grid_list + 1;
    for (pqptr pq = g->pquad; pq != NULL; pq = pq->next) {
      long zz = pq->z;
      for (cqptr cq = pq->loc; cq < pq->loc + pq->length; cq++, zz++)
        for (cqptr icq = cq; icq != NULL; icq = icq->next) {
          long yy = icq->y;
          for (nqptr nq = icq->loc; nq < icq->loc + icq->length; nq++, yy++)
            for (nqptr inq = nq; inq != NULL; inq = inq->next) {
              long xx = inq->x;
              for (nptr nd = inq->loc; nd < inq->loc + inq->length; nd++, xx++) {
                if (count >= max_nodes) return -3;
                zyx[3 * count + 0] = zz;
                zyx[3 * count + 1] = yy;
                zyx[3 * count + 2] = xx;
                count++;
              }
            }
        }
    }
  }
  free(p);
  global.fst_part = NULL;
  if (log) fclose(log);
  io.logfile = NULL;
  return count;
}

/* Grid `level` of the hierarchy ahfref_amr_levels builds: its nodes in the
 * order of its quads, zyx[3 k + 0..2], and their densities as the last
 * assign_npart left them.  Returns the number of nodes, -3 when more than
 * max_nodes, -4 when the hierarchy has no such grid. */
int64_t ahfref_amr_nodes(uint64_t n, const float *x, const float *y, const float *z, int ngrid_dom, int ngrid_max,
                         double nth_dom, double nth_ref, int level, int64_t *zyx, double *dens, int64_t max_nodes)
{
  FILE *log = fopen("/dev/null", "w");
  io.logfile = log ? log : stderr;
  partptr p = (partptr)calloc(n ? n : 1, sizeof(part));
  if (!p) return -1;
  for (uint64_t i = 0; i < n; i++) {
    p[i].pos[0] = x[i];
    p[i].pos[1] = y[i];
    p[i].pos[2] = z[i];
    p[i].id = (part_id_t)i;
  }
  simu.no_part = n;
  simu.no_vpart = (double)n;
  simu.NGRID_DOM = ngrid_dom;
  simu.NGRID_MIN = ngrid_dom;
  simu.NGRID_MAX = ngrid_max;
  simu.Nth_dom = nth_dom;
  simu.Nth_ref = nth_ref;
  simu.boxsize = 1.0;
  simu.mean_dens = 1.0;
  global.super_t = 1.0;
  global.fst_part = p;
  global.no_part = n;
  int no_grids = 0;
  gridls *grid_list = gen_domgrids(&no_grids);
  ll(n, p, global.dom_grid);
  zero_dens(global.dom_grid);
  assign_npart(global.dom_grid);
  global.fst_cycle = TRUE;
  gen_AMRhierarchy(&grid_list, &no_grids);
  if (level >= no_grids) return -4;
  gridls *g = grid_list + level;
  int64_t count = 0;
  for (pqptr pq = g->pquad; pq != NULL; pq = pq->next) {
    long zz = pq->z;
    for (cqptr cq = pq->loc; cq < pq->loc + pq->length; cq++, zz++)
      for (cqptr icq = cq; icq != NULL; icq = icq->next) {
        long yy = icq->y;
        for (nqptr nq = icq->loc; nq < icq->loc + icq->length; nq++, yy++)
          for (nqptr inq = nq; inq != NULL; inq = inq->next) {
            long xx = inq->x;
            for (nptr nd = inq->loc; nd < inq->loc + inq->length; nd++, xx++) {
              if (count >= max_nodes) return -3;
              zyx[3 * count + 0] = zz;
              zyx[3 * count + 1] = yy;
              zyx[3 * count + 2] = xx;
              dens[count] = (double)nd->dens;
              count++;
            }
          }
      }
  }
  if (log) fclose(log);
  io.logfile = NULL;
  return count;
}
