/*
 * ref_harness.c -- drives the UNMODIFIED reference AHF routines on a batch.
 *
 * TEST INFRASTRUCTURE ONLY.  Compiled (by oracle/Makefile) together with the
 * reference's own src/libahf/ahf_halos.c and src/libutility/{general,
 * specific,alloc_struct,cosmology}.c, straight from the reference tree, into
 * oracle/_ref/libahfref.so.  It fills global.fst_part, simu.*, global.* and
 * the unit factors of src/libahf/ahf_halos.c:163 from an ahfgpu_batch,
 * builds one HALO per list, and calls the reference's
 *   sort_halo_particles -> rem_outsideRvir(.,0) -> rem_unbound ->
 *   rem_outsideRvir(.,1) -> HaloProfiles
 * in the order of src/libahf/ahf_halos_sfc.c:140-156.  Results are packed into
 * an ahfgpu_result so they compare field by field with the restatement
 * (ahf_oracle.c) and the GPU library.  Nothing here is the product.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>

#include "common.h"
#include "libahf/ahf_halos.h"
#include "libutility/alloc_struct.h"

#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/ahfgpu.h"

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

static double pget(const HALOPROFILE *pr, int f, int i)
{
  switch (f) {
  case AHFGPU_PROF_R: return pr->r[i];
  case AHFGPU_PROF_NPART: return (double)pr->npart[i];
  case AHFGPU_PROF_NVPART: return pr->nvpart[i];
  case AHFGPU_PROF_OVDENS: return pr->ovdens[i];
  case AHFGPU_PROF_DENS: return pr->dens[i];
  case AHFGPU_PROF_V2_CIRC: return pr->v2_circ[i];
  case AHFGPU_PROF_V_ESC2: return pr->v_esc2[i];
  case AHFGPU_PROF_SIG_V: return pr->sig_v[i];
  case AHFGPU_PROF_EKIN: return pr->Ekin[i];
  case AHFGPU_PROF_EPOT: return pr->Epot[i];
  case AHFGPU_PROF_LX: return pr->Lx[i];
  case AHFGPU_PROF_LY: return pr->Ly[i];
  case AHFGPU_PROF_LZ: return pr->Lz[i];
  case AHFGPU_PROF_AXIS1: return pr->axis1[i];
  case AHFGPU_PROF_E1X: return pr->E1x[i];
  case AHFGPU_PROF_E1Y: return pr->E1y[i];
  case AHFGPU_PROF_E1Z: return pr->E1z[i];
  case AHFGPU_PROF_AXIS2: return pr->axis2[i];
  case AHFGPU_PROF_E2X: return pr->E2x[i];
  case AHFGPU_PROF_E2Y: return pr->E2y[i];
  case AHFGPU_PROF_E2Z: return pr->E2z[i];
  case AHFGPU_PROF_AXIS3: return pr->axis3[i];
  case AHFGPU_PROF_E3X: return pr->E3x[i];
  case AHFGPU_PROF_E3Y: return pr->E3y[i];
  case AHFGPU_PROF_E3Z: return pr->E3z[i];
  }
  return 0.0;
}

int ahfref_multimass(void)
{
#ifdef MULTIMASS
  return 1;
#else
  return 0;
#endif
}

int ahfref_construct_halos(const ahfgpu_params *prm, const ahfgpu_batch *b, ahfgpu_result *res,
                           int nthreads)
{
  int64_t nh = b->nhalo;
  uint64_t N = nh ? b->off[nh] : 0;
  memset(res, 0, sizeof(*res));
#ifdef MULTIMASS
  if (!b->w) return AHFGPU_ERR_INVALID;
#else
  if (b->w) return AHFGPU_ERR_INVALID;
#endif
  part *parts = (part *)calloc(N ? N : 1, sizeof(part));
  for (uint64_t e = 0; e < N; e++) {
    parts[e].pos[0] = b->x[e]; parts[e].pos[1] = b->y[e]; parts[e].pos[2] = b->z[e];
    parts[e].mom[0] = b->vx[e]; parts[e].mom[1] = b->vy[e]; parts[e].mom[2] = b->vz[e];
#ifdef MULTIMASS
    parts[e].weight = b->w[e];
#endif
    parts[e].id = b->gidx ? b->gidx[e] : e;
  }
  io.logfile = stderr;
  global.fst_part = parts;
  global.no_part = N;
  global.ovlim = prm->ovlim;
  global.rho_vir = prm->rho_vir;
  simu.AHF_MINPART = (int)prm->MINPART;
  simu.AHF_VTUNE = prm->VescTune;
  r_fac = prm->r_fac; x_fac = prm->x_fac; v_fac = prm->v_fac; m_fac = prm->m_fac;
  rho_fac = prm->rho_fac; phi_fac = prm->phi_fac; Hubble = prm->Hubble;

  HALO *hs = (HALO *)calloc(nh ? nh : 1, sizeof(HALO));
  uint32_t *flags = (uint32_t *)calloc(nh ? nh : 1, sizeof(uint32_t));
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic) num_threads(nthreads)
#endif
  for (int64_t i = 0; i < nh; i++) {
    HALO *h = &hs[i];
    uint32_t f = 0;
    uint64_t n = b->off[i + 1] - b->off[i];
    h->pos.x = b->cx[i]; h->pos.y = b->cy[i]; h->pos.z = b->cz[i];
    h->npart = n;
    h->ipart = (long unsigned *)malloc((n ? n : 1) * sizeof(long unsigned));
    for (uint64_t j = 0; j < n; j++) h->ipart[j] = b->off[i] + j;
    if (n == 0) { flags[i] = AHFGPU_HALO_EMPTY; continue; }
    long unsigned mp = (long unsigned)simu.AHF_MINPART;
    if (h->npart >= mp) f |= AHFGPU_HALO_RAN_SORT | AHFGPU_HALO_RAN_RVIR0;
    sort_halo_particles(h);
    rem_outsideRvir(h, 0);
    if (h->npart >= mp) f |= AHFGPU_HALO_RAN_UNBIND;
    rem_unbound(h);
    if (h->npart >= mp) f |= AHFGPU_HALO_RAN_RVIR1;
    rem_outsideRvir(h, 1);
    if (h->npart >= mp) f |= AHFGPU_HALO_RAN_PROFILE;
    HaloProfiles(h);
    flags[i] = f;
  }

  res->nhalo = nh;
  res->halo = (ahfgpu_halo *)calloc(nh ? nh : 1, sizeof(ahfgpu_halo));
  res->member_off = (uint64_t *)calloc(nh + 1, sizeof(uint64_t));
  res->prof_off = (uint64_t *)calloc(nh + 1, sizeof(uint64_t));
  for (int64_t i = 0; i < nh; i++) {
    int nb = (flags[i] & AHFGPU_HALO_RAN_PROFILE) ? hs[i].prof.nbins : 0;
    res->member_off[i + 1] = res->member_off[i] + hs[i].npart;
    res->prof_off[i + 1] = res->prof_off[i] + (uint64_t)nb;
  }
  res->member = (uint64_t *)malloc((res->member_off[nh] ? res->member_off[nh] : 1) * sizeof(uint64_t));
  res->prof = (double *)malloc((res->prof_off[nh] ? res->prof_off[nh] : 1) * AHFGPU_PROF_NFIELDS * sizeof(double));
  for (int64_t i = 0; i < nh; i++) {
    HALO *h = &hs[i];
    ahfgpu_halo *o = &res->halo[i];
    o->npart = h->npart;
    o->flags = flags[i];
    int ranprof = (flags[i] & AHFGPU_HALO_RAN_PROFILE) != 0;
    o->nbins = ranprof ? h->prof.nbins : 0;
    o->M_vir = h->M_vir; o->R_vir = h->R_vir; o->ovdens = h->ovdens; o->Phi0 = h->Phi0;
    o->vel[0] = h->vel.x; o->vel[1] = h->vel.y; o->vel[2] = h->vel.z;
    o->sigV = h->sigV; o->v_esc2 = h->v_esc2; o->V2_max = h->V2_max; o->R_max = h->R_max; o->r2 = h->r2;
    o->lambda = h->lambda; o->lambdaE = h->lambdaE; o->Ekin = h->Ekin; o->Epot = h->Epot; o->SurfP = h->SurfP;
    o->pos_com[0] = h->pos_com.x; o->pos_com[1] = h->pos_com.y; o->pos_com[2] = h->pos_com.z;
    o->com_offset = h->com_offset;
    o->pos_mbp[0] = h->pos_mbp.x; o->pos_mbp[1] = h->pos_mbp.y; o->pos_mbp[2] = h->pos_mbp.z;
    o->vel_mbp[0] = h->vel_mbp.x; o->vel_mbp[1] = h->vel_mbp.y; o->vel_mbp[2] = h->vel_mbp.z;
    o->mbp_offset = h->mbp_offset;
    if (ranprof && h->mbp_offset == -1.0) o->flags |= AHFGPU_HALO_NO_MBP;
    o->AngMom[0] = h->AngMom.x; o->AngMom[1] = h->AngMom.y; o->AngMom[2] = h->AngMom.z;
    o->axis[0] = h->axis.x; o->axis[1] = h->axis.y; o->axis[2] = h->axis.z;
    o->E1[0] = h->E1.x; o->E1[1] = h->E1.y; o->E1[2] = h->E1.z;
    o->E2[0] = h->E2.x; o->E2[1] = h->E2.y; o->E2[2] = h->E2.z;
    o->E3[0] = h->E3.x; o->E3[1] = h->E3.y; o->E3[2] = h->E3.z;
    o->fMhires = h->fMhires; o->cNFW = h->cNFW; o->R1 = h->R1; o->cR1 = h->cR1;
    for (uint64_t j = 0; j < h->npart; j++)
      res->member[res->member_off[i] + j] = b->gidx ? b->gidx[h->ipart[j]] : h->ipart[j];
    for (int k = 0; k < o->nbins; k++)
      for (int f = 0; f < AHFGPU_PROF_NFIELDS; f++)
        res->prof[(res->prof_off[i] + k) * AHFGPU_PROF_NFIELDS + f] = pget(&h->prof, f, k);
    if (ranprof) dest_profile(h);
    free(h->ipart);
  }
  res->stats.n_particles_in = N;
  res->stats.n_kept = res->member_off[nh];
  free(hs); free(flags); free(parts);
  return AHFGPU_OK;
}

void ahfref_result_free(ahfgpu_result *r)
{
  free(r->halo); free(r->member_off); free(r->member); free(r->prof_off); free(r->prof);
  memset(r, 0, sizeof(*r));
}
