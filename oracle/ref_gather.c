/*
 * ref_gather.c -- TEST INFRASTRUCTURE ONLY (part of oracle/_ref/libahfref*.so).
 * Runs the reference's own particle gather, ahf_halos_sfc_gatherParts
 * (src/libahf/ahf_halos_sfc.c:171-412, compiled unchanged), on a snapshot
 * given as float arrays, the way AHF sets it up: every particle gets its
 * Hilbert key at BITS_PER_DIMENSION (sfc_curve_calcKey, as
 * src/main.c:342-352 does), the particles are sorted by key with
 * cmp_sfckey_part (main.c:353-356), global_info.fst_part/no_part/ctype point
 * at them (startrun.c:617), and each halo's centre and gatherRad go into a
 * HALO that the gather fills.
 *
 * Result: CSR lists of ORIGINAL particle indices (position in the input
 * arrays), each halo's list in the reference's gather order.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "libahf/ahf_halos_sfc.h"
#include "libsfc/sfc_curve.h"
#include "libutility/specific.h"
#include "common.h"
#include "tdef.h"

int ahfref_gather(uint64_t n, const float *x, const float *y, const float *z, int64_t nhalo,
                  const double *cx, const double *cy, const double *cz, const double *rad,
                  uint64_t *out_off, uint64_t **out_idx)
{
  partptr p = (partptr)calloc(n ? n : 1, sizeof(part));
  if (!p) return -1;
  for (uint64_t i = 0; i < n; i++) {
    p[i].pos[0] = x[i];
    p[i].pos[1] = y[i];
    p[i].pos[2] = z[i];
    p[i].sfckey = sfc_curve_calcKey(SFC_CURVE_HILBERT, (double)p[i].pos[0], (double)p[i].pos[1],
                                    (double)p[i].pos[2], BITS_PER_DIMENSION);
    p[i].id = (part_id_t)i;
  }
  qsort(p, (size_t)n, sizeof(part), &cmp_sfckey_part);
  global_info.fst_part = p;
  global_info.no_part = n;
  global_info.ctype = SFC_CURVE_HILBERT;
  uint64_t cap = 1024, used = 0;
  uint64_t *idx = (uint64_t *)malloc(cap * sizeof(uint64_t));
  if (!idx) { free(p); return -1; }
  out_off[0] = 0;
  for (int64_t h = 0; h < nhalo; h++) {
    HALO halo;
    memset(&halo, 0, sizeof halo);
    halo.pos.x = cx[h];
    halo.pos.y = cy[h];
    halo.pos.z = cz[h];
    halo.gatherRad = rad[h];
    halo.npart = 0;
    halo.ipart = NULL;
    ahf_halos_sfc_gatherParts(&halo);
    if (used + halo.npart > cap) {
      while (used + halo.npart > cap) cap *= 2;
      uint64_t *t = (uint64_t *)realloc(idx, cap * sizeof(uint64_t));
      if (!t) { free(idx); free(p); free(halo.ipart); return -1; }
      idx = t;
    }
    for (uint64_t j = 0; j < halo.npart; j++) idx[used + j] = (uint64_t)p[halo.ipart[j]].id;
    used += halo.npart;
    out_off[h + 1] = used;
    free(halo.ipart);
  }
  free(p);
  global_info.fst_part = NULL;
  global_info.no_part = 0;
  *out_idx = idx;
  return 0;
}

void ahfref_gather_free(uint64_t *idx) { free(idx); }

/* The reference's keying and sort alone (main.c:342-356): keys[k] and
 * order[k] = original index of the k-th particle after the qsort by
 * cmp_sfckey_part.  Equal keys come out in the order the C library's qsort
 * leaves them. */
int ahfref_sfc_sort(uint64_t n, const float *x, const float *y, const float *z, uint64_t *keys, uint64_t *order)
{
  partptr p = (partptr)calloc(n ? n : 1, sizeof(part));
  if (!p) return -1;
  for (uint64_t i = 0; i < n; i++) {
    p[i].pos[0] = x[i];
    p[i].pos[1] = y[i];
    p[i].pos[2] = z[i];
    p[i].sfckey = sfc_curve_calcKey(SFC_CURVE_HILBERT, (double)p[i].pos[0], (double)p[i].pos[1],
                                    (double)p[i].pos[2], BITS_PER_DIMENSION);
    p[i].id = (part_id_t)i;
  }
  qsort(p, (size_t)n, sizeof(part), &cmp_sfckey_part);
  for (uint64_t k = 0; k < n; k++) {
    keys[k] = (uint64_t)p[k].sfckey;
    order[k] = (uint64_t)p[k].id;
  }
  free(p);
  return 0;
}

/* One key: sfc_curve_calcKey(SFC_CURVE_HILBERT, x, y, z, bits). */
uint64_t ahfref_sfc_key(double x, double y, double z, unsigned bits)
{
  return (uint64_t)sfc_curve_calcKey(SFC_CURVE_HILBERT, x, y, z, bits);
}
