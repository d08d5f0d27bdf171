/*
 * ref_writer.c -- TEST INFRASTRUCTURE ONLY (part of oracle/_ref/libahfref*.so).
 * Runs the reference's own AHF_particles writer, ahf_io_WriteParticles
 * (src/libahf/ahf_io.c:178-212, WriteParticlesLegacy :1095-1175, compiled
 * unchanged), on haloes given as kept particle lists: global.fst_part holds
 * the particles (their ids), each HALO its npart and ipart, idx the output
 * order, simu.AHF_MINPART the cut.  The file it writes is read back into a
 * malloc()ed buffer: <prefix>.AHF_particles, or in the -DAHFbinary build
 * (libahfref_bin.so) <prefix>.AHF_particles_bin, written by
 * ahf_binwrite_particles (ahf_io.c:1733-1855); its text companion
 * <prefix>.AHF_particles_info is removed.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "libahf/ahf_io.h"
#include "common.h"
#include "tdef.h"

int ahfref_write_particles(uint64_t npart_total, const uint64_t *ids, const float *w, int64_t nhalo,
                           const uint64_t *member_off, const uint64_t *member, const uint64_t *halo_npart,
                           const int64_t *order, int64_t minpart, const char *prefix,
                           unsigned char **out, uint64_t *nbytes)
{
  partptr p = (partptr)calloc(npart_total ? npart_total : 1, sizeof(part));
  HALO *halos = (HALO *)calloc(nhalo ? nhalo : 1, sizeof(HALO));
  unsigned long *idx = (unsigned long *)calloc(nhalo ? nhalo : 1, sizeof(unsigned long));
  if (!p || !halos || !idx) return -1;
  for (uint64_t i = 0; i < npart_total; i++) {
    p[i].id = (part_id_t)ids[i];
#ifdef MULTIMASS
    p[i].weight = w ? w[i] : 1.0f;
#else
    (void)w;
#endif
  }
  for (int64_t h = 0; h < nhalo; h++) {
    uint64_t k = member_off[h + 1] - member_off[h];
    halos[h].npart = halo_npart[h];
    halos[h].ipart = (unsigned long *)malloc((k ? k : 1) * sizeof(unsigned long));
    for (uint64_t j = 0; j < k; j++) halos[h].ipart[j] = (unsigned long)member[member_off[h] + j];
    idx[h] = (unsigned long)order[h];
  }
  global.fst_part = p;
  global.no_part = npart_total;
  simu.AHF_MINPART = (int)minpart;
  ahf_io_WriteParticles(prefix, halos, idx, (int)nhalo);
  for (int64_t h = 0; h < nhalo; h++) free(halos[h].ipart);
  free(halos);
  free(idx);
  free(p);
  global.fst_part = NULL;
  global.no_part = 0;
  char fn[4096];
#ifdef AHFbinary
  snprintf(fn, sizeof fn, "%s.AHF_particles_info", prefix);
  remove(fn);
  snprintf(fn, sizeof fn, "%s.AHF_particles_bin", prefix);
#else
  snprintf(fn, sizeof fn, "%s.AHF_particles", prefix);
#endif
  FILE *f = fopen(fn, "rb");
  if (!f) return -2;
  fseek(f, 0, SEEK_END);
  long sz = ftell(f);
  fseek(f, 0, SEEK_SET);
  unsigned char *buf = (unsigned char *)malloc(sz > 0 ? (size_t)sz : 1);
  if (!buf || fread(buf, 1, (size_t)sz, f) != (size_t)sz) { fclose(f); free(buf); return -3; }
  fclose(f);
  remove(fn);
  *out = buf;
  *nbytes = (uint64_t)sz;
  return 0;
}

void ahfref_write_free(unsigned char *buf) { free(buf); }
