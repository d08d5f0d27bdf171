/*
 * ref_radii.c -- TEST INFRASTRUCTURE ONLY (oracle/_ref/libahfref_radii.so).
 *
 * Runs the reference's gather-radius loop, which sits at the end of
 * spatialRef2halos (src/libahf/ahf_halos.c:2405-3057, loop :2987-3051),
 * through the reference function itself, compiled unchanged.  This file
 * includes ahf_halos.c so that its file-static halos[], numHalos and
 * gridl1dim, and its spatREF type, are in reach; the library is therefore
 * built without a separate ahf_halos.o.
 *
 * spatialRef2halos turns a tree of isolated refinements into haloes.  The
 * tree built here has two levels: level 0 holds one refinement whose
 * daughter is level-1 refinement 0 and whose substructures are level-1
 * refinements 1..n-1, every level-1 refinement ends there.  The function
 * then makes halo 0 the host (centre and particles of level-1 refinement 0,
 * plus the level-0 particles; R_vir stays at its initial -1) and halo h >= 1
 * a subhalo (centre and particles of level-1 refinement h, R_vir its
 * closeRefDist), orders them by particle count and runs the loop.  The
 * caller's counts, centres and R_vir go in as those fields; the gather
 * radii and the R_vir each halo carried come back.
 */
#include "libahf/ahf_halos.c"

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

int ahfref_gather_radii(int64_t nh, const uint64_t *npart, const double *cx, const double *cy, const double *cz,
                        const double *rvir, double max_gather_rad_box, double *rad, double *rvir_used)
{
  if (nh < 1) return -1;
  FILE *log = fopen("/dev/null", "w");
  io.logfile = log ? log : stderr;
  simu.boxsize = 1.0;
  simu.MaxGatherRad = max_gather_rad_box;

  double grid_dims[2] = {64.0, 128.0};
  gridl1dim = grid_dims;
  int iso[2] = {1, (int)nh};
  numIsoRef = iso;
  totnumIsoRef = 1 + (int)nh;

  SPATIALREF *l0 = (SPATIALREF *)calloc(1, sizeof(SPATIALREF));
  SPATIALREF *l1 = (SPATIALREF *)calloc((size_t)nh, sizeof(SPATIALREF));
  INDEX *sub = (INDEX *)calloc((size_t)nh, sizeof(INDEX));
  if (!l0 || !l1 || !sub) return -1;
  for (int64_t k = 0; k < nh; k++) {
    sub[k].refLevel = 1;
    sub[k].isoRefIndex = (int)k;
  }
  l0->numNodes = 1;
  l0->numParts = (long)npart[0];
  l0->numSubStruct = nh > 1 ? (int)nh : 1;   /* the daughter plus n-1 substructures */
  l0->subStruct = sub;
  l0->daughter.refLevel = 1;
  l0->daughter.isoRefIndex = 0;
  l0->haloIndex = -1;
  for (int64_t j = 0; j < nh; j++) {
    l1[j].numNodes = 1;
    l1[j].numParDom = 1;
    l1[j].numSubStruct = 0;
    l1[j].centre.x = cx[j];
    l1[j].centre.y = cy[j];
    l1[j].centre.z = cz[j];
    l1[j].numParts = j ? (long)npart[j] : 0;
    l1[j].closeRefDist = rvir[j];
    l1[j].daughter.refLevel = -1;
    l1[j].daughter.isoRefIndex = -1;
    l1[j].haloIndex = -1;
  }
  SPATIALREF *tree[2] = {l0, l1};
  int ok = spatialRef2halos(2, tree);
  int rc = (ok && numHalos == (int)nh) ? 0 : -2;
  for (int64_t h = 0; rc == 0 && h < nh; h++) {
    if (halos[h].npart != (long unsigned)npart[h]) rc = -3;
    rad[h] = halos[h].gatherRad;
    rvir_used[h] = halos[h].R_vir;
  }
  for (int h = 0; h < MAX(totnumIsoRef + 1, numHalos); h++) free(halos[h].subStruct);
  free(halos);
  halos = NULL;
  numHalos = 0;
  gridl1dim = NULL;
  numIsoRef = NULL;
  free(sub);
  free(l1);
  free(l0);
  if (log) fclose(log);
  io.logfile = NULL;
  return rc;
}
