/*
 * ahf_gpu_shim.c -- AHF-side binding of the GB300 stage (libahfgpu.so).
 *
 * Compiled into AHF with -DAHF_GPU (and -I<AHF>/src), it replaces the per-halo
 * loop of ahf_halos() (src/libahf/ahf_halos.c:504-510):
 *
 *     for (i = 0; i < numHalos; i++)  ahf_halos_sfc_constructHalo(halos + i);
 *
 * by one call, ahfgpu_shim_construct_halos(halos, numHalos), which
 *   1. does for every halo what ahf_halos_sfc_constructHalo
 *      (src/libahf/ahf_halos_sfc.c:118-169) does before its sort: skip a halo
 *      whose preliminary npart is 0 (:122), reset npart/ipart/nll/ll
 *      (:126-129) and gather its particles (ahf_halos_sfc_gatherParts, :137);
 *   2. packs the gathered lists into one ahfgpu_batch (positions, momenta,
 *      MULTIMASS weights, the ipart indices as gidx, the halo centres) and
 *      makes ONE ahfgpu_construct_halos call: sort_halo_particles,
 *      rem_outsideRvir(.,0), rem_unbound, rem_outsideRvir(.,1) and
 *      HaloProfiles for every halo;
 *   3. writes the results back into HALO exactly where those five functions
 *      write: ipart/npart always (the kept list in radial order, malloc'ed as
 *      AHF frees it, ahf_halos.c:897); M_vir, R_vir, ovdens, Phi0 when
 *      rem_outsideRvir(.,0) ran; every HaloProfiles field and the profile
 *      arrays (c_profile, freed by dest_profile) when HaloProfiles ran.
 *      (HALO.R_edge, which HaloProfiles computes but AHF no longer writes
 *      out, is left as it was.)
 *
 * The form comes from the environment: AHFGPU_MODE = plain (default; halo by
 * halo in FP64, bit-exact), batched (FP64, one launch) or fp32c (batched
 * FP32-compensated).  AHFGPU_DEVICE selects the GPU (default 0).  Any
 * library error is printed with its message and returned; the caller maps a
 * non-zero return to common_terminate(EXIT_FAILURE) as AHF does on failure.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "common.h"
#include "param.h"
#include "tdef.h"
#include "libahf/ahf_halos_sfc.h"
#include "libutility/alloc_struct.h"

#include "ahfgpu.h"

/* the unit factors of ahf_halos() (file-scope globals of ahf_halos.c:163) */
extern double r_fac, x_fac, v_fac, m_fac, rho_fac, phi_fac, Hubble;

static int shim_fail(int rc, const char *what)
{
  char msg[512];
  ahfgpu_last_error(msg, sizeof msg);
  fprintf(stderr, "ahfgpu: %s failed (%d): %s\n", what, rc, msg);
  return rc;
}

static ahfgpu_mode shim_mode(void)
{
  const char *m = getenv("AHFGPU_MODE");
  if (m && strcmp(m, "batched") == 0) return AHFGPU_BATCHED_FP64;
  if (m && strcmp(m, "fp32c") == 0) return AHFGPU_BATCHED_FP32C;
  return AHFGPU_PLAIN_FP64;
}

/* HaloProfiles' integral properties and profile arrays (ahf_halos.c:3961-5261) */
static void shim_write_profiles(HALO *halo, const ahfgpu_halo *r, const double *rows)
{
  int b;
  halo->vel.x = r->vel[0];  halo->vel.y = r->vel[1];  halo->vel.z = r->vel[2];
  halo->M_vir = r->M_vir;
  halo->sigV = r->sigV;     halo->v_esc2 = r->v_esc2;
  halo->V2_max = r->V2_max; halo->R_max = r->R_max;  halo->r2 = r->r2;
  halo->lambda = r->lambda; halo->lambdaE = r->lambdaE;
  halo->Ekin = r->Ekin;     halo->Epot = r->Epot;    halo->SurfP = r->SurfP;
  halo->pos_com.x = r->pos_com[0]; halo->pos_com.y = r->pos_com[1]; halo->pos_com.z = r->pos_com[2];
  halo->com_offset = r->com_offset;
  halo->pos_mbp.x = r->pos_mbp[0]; halo->pos_mbp.y = r->pos_mbp[1]; halo->pos_mbp.z = r->pos_mbp[2];
  halo->vel_mbp.x = r->vel_mbp[0]; halo->vel_mbp.y = r->vel_mbp[1]; halo->vel_mbp.z = r->vel_mbp[2];
  halo->mbp_offset = r->mbp_offset;
  halo->AngMom.x = r->AngMom[0]; halo->AngMom.y = r->AngMom[1]; halo->AngMom.z = r->AngMom[2];
  halo->axis.x = r->axis[0]; halo->axis.y = r->axis[1]; halo->axis.z = r->axis[2];
  halo->E1.x = r->E1[0]; halo->E1.y = r->E1[1]; halo->E1.z = r->E1[2];
  halo->E2.x = r->E2[0]; halo->E2.y = r->E2[1]; halo->E2.z = r->E2[2];
  halo->E3.x = r->E3[0]; halo->E3.y = r->E3[1]; halo->E3.z = r->E3[2];
  halo->fMhires = r->fMhires;
  halo->cNFW = r->cNFW;
  halo->R1 = r->R1;
  halo->cR1 = r->cR1;
  c_profile(halo, r->nbins);
  for (b = 0; b < r->nbins; b++) {
    const double *f = rows + (size_t)b * AHFGPU_PROF_NFIELDS;
    halo->prof.r[b]       = f[AHFGPU_PROF_R];
    halo->prof.npart[b]   = (long unsigned)f[AHFGPU_PROF_NPART];
    halo->prof.nvpart[b]  = f[AHFGPU_PROF_NVPART];
    halo->prof.ovdens[b]  = f[AHFGPU_PROF_OVDENS];
    halo->prof.dens[b]    = f[AHFGPU_PROF_DENS];
    halo->prof.v2_circ[b] = f[AHFGPU_PROF_V2_CIRC];
    halo->prof.v_esc2[b]  = f[AHFGPU_PROF_V_ESC2];
    halo->prof.sig_v[b]   = f[AHFGPU_PROF_SIG_V];
    halo->prof.Ekin[b]    = f[AHFGPU_PROF_EKIN];
    halo->prof.Epot[b]    = f[AHFGPU_PROF_EPOT];
    halo->prof.Lx[b]      = f[AHFGPU_PROF_LX];
    halo->prof.Ly[b]      = f[AHFGPU_PROF_LY];
    halo->prof.Lz[b]      = f[AHFGPU_PROF_LZ];
    halo->prof.axis1[b]   = f[AHFGPU_PROF_AXIS1];
    halo->prof.E1x[b]     = f[AHFGPU_PROF_E1X];
    halo->prof.E1y[b]     = f[AHFGPU_PROF_E1Y];
    halo->prof.E1z[b]     = f[AHFGPU_PROF_E1Z];
    halo->prof.axis2[b]   = f[AHFGPU_PROF_AXIS2];
    halo->prof.E2x[b]     = f[AHFGPU_PROF_E2X];
    halo->prof.E2y[b]     = f[AHFGPU_PROF_E2Y];
    halo->prof.E2z[b]     = f[AHFGPU_PROF_E2Z];
    halo->prof.axis3[b]   = f[AHFGPU_PROF_AXIS3];
    halo->prof.E3x[b]     = f[AHFGPU_PROF_E3X];
    halo->prof.E3y[b]     = f[AHFGPU_PROF_E3Y];
    halo->prof.E3z[b]     = f[AHFGPU_PROF_E3Z];
  }
}

int ahfgpu_shim_construct_halos(HALO *halos, int numHalos)
{
  static int inited = 0;
  int          rc, i;
  int64_t      nb = 0, k;
  uint64_t     n = 0;
  int         *which;
  uint64_t    *off = NULL, *gidx = NULL;
  float       *buf = NULL, *x, *y, *z, *vx, *vy, *vz, *w = NULL;
  double      *cen = NULL;
  ahfgpu_params prm;
  ahfgpu_batch  b;
  ahfgpu_result res;

  if (!inited) {
    const char *d = getenv("AHFGPU_DEVICE");
    if ((rc = ahfgpu_init(d ? atoi(d) : 0)) != AHFGPU_OK) return shim_fail(rc, "ahfgpu_init");
    inited = 1;
  }

  /* 1. gather (ahf_halos_sfc.c:122-137) for every halo that has particles */
  which = (int *)malloc((size_t)(numHalos > 0 ? numHalos : 1) * sizeof(int));
  if (!which) return AHFGPU_ERR_OOM;
  for (i = 0; i < numHalos; i++)
    if (halos[i].npart != 0) which[nb++] = i;
#ifdef _OPENMP
#  pragma omp parallel for schedule(dynamic)
#endif
  for (k = 0; k < nb; k++) {
    HALO *halo = halos + which[k];
    halo->nll = 0;
    halo->ll = NULL;
    halo->npart = 0;
    halo->ipart = NULL;
    ahf_halos_sfc_gatherParts(halo);
  }

  /* 2. one CSR batch: SoA floats, ipart as gidx, centres */
  off = (uint64_t *)malloc((size_t)(nb + 1) * sizeof(uint64_t));
  if (!off) { free(which); return AHFGPU_ERR_OOM; }
  off[0] = 0;
  for (k = 0; k < nb; k++) off[k + 1] = off[k] + halos[which[k]].npart;
  n = off[nb];
#ifdef MULTIMASS
  buf = (float *)malloc((size_t)(n > 0 ? n : 1) * 7 * sizeof(float));
#else
  buf = (float *)malloc((size_t)(n > 0 ? n : 1) * 6 * sizeof(float));
#endif
  gidx = (uint64_t *)malloc((size_t)(n > 0 ? n : 1) * sizeof(uint64_t));
  cen = (double *)malloc((size_t)(nb > 0 ? nb : 1) * 3 * sizeof(double));
  if (!buf || !gidx || !cen) { free(which); free(off); free(buf); free(gidx); free(cen); return AHFGPU_ERR_OOM; }
  x = buf; y = x + n; z = y + n; vx = z + n; vy = vx + n; vz = vy + n;
#ifdef MULTIMASS
  w = vz + n;
#endif
#ifdef _OPENMP
#  pragma omp parallel for schedule(dynamic)
#endif
  for (k = 0; k < nb; k++) {
    const HALO *halo = halos + which[k];
    uint64_t j, o = off[k];
    for (j = 0; j < halo->npart; j++) {
      const part *p = global.fst_part + halo->ipart[j];
      x[o + j] = p->pos[X];  y[o + j] = p->pos[Y];  z[o + j] = p->pos[Z];
      vx[o + j] = p->mom[X]; vy[o + j] = p->mom[Y]; vz[o + j] = p->mom[Z];
#ifdef MULTIMASS
      w[o + j] = p->weight;
#endif
      gidx[o + j] = halo->ipart[j];
    }
    cen[k] = halo->pos.x;
    cen[nb + k] = halo->pos.y;
    cen[2 * nb + k] = halo->pos.z;
  }
  memset(&b, 0, sizeof b);
  b.nhalo = nb;
  b.off = off;
  b.x = x; b.y = y; b.z = z; b.vx = vx; b.vy = vy; b.vz = vz; b.w = w;
  b.gidx = gidx;
  b.cx = cen; b.cy = cen + nb; b.cz = cen + 2 * nb;
  prm.VescTune = simu.AHF_VTUNE;
  prm.MINPART = simu.AHF_MINPART;
  prm.ovlim = global.ovlim;
  prm.rho_vir = global.rho_vir;
  prm.r_fac = r_fac; prm.x_fac = x_fac; prm.v_fac = v_fac; prm.m_fac = m_fac;
  prm.rho_fac = rho_fac; prm.phi_fac = phi_fac; prm.Hubble = Hubble;

  rc = ahfgpu_construct_halos(&prm, &b, &res, shim_mode());
  free(buf); free(gidx); free(cen); free(off);
  if (rc != AHFGPU_OK) { free(which); return shim_fail(rc, "ahfgpu_construct_halos"); }
  if (getenv("AHFGPU_LOG"))
    fprintf(stderr, "ahfgpu: %lld haloes, %llu particles in, %llu kept, %llu equal radial keys, "
            "%llu replayed haloes, %.3f ms on the device\n", (long long)nb,
            (unsigned long long)res.stats.n_particles_in, (unsigned long long)res.stats.n_kept,
            (unsigned long long)res.stats.n_key_ties, (unsigned long long)res.stats.n_replay_halos,
            res.stats.ms_device);

  /* 3. write back where the five functions write */
  for (k = 0; k < nb; k++) {
    HALO *halo = halos + which[k];
    const ahfgpu_halo *r = res.halo + k;
    const uint64_t m0 = res.member_off[k], nk = res.member_off[k + 1] - m0;
    uint64_t j;
    free(halo->ipart);
    halo->ipart = NULL;
    halo->npart = nk;
    if (nk > 0) {
      halo->ipart = (long unsigned *)malloc(nk * sizeof(long unsigned));
      if (!halo->ipart) { ahfgpu_result_free(&res); free(which); return AHFGPU_ERR_OOM; }
      for (j = 0; j < nk; j++) halo->ipart[j] = (long unsigned)res.member[m0 + j];
    }
    if (r->flags & AHFGPU_HALO_RAN_RVIR0) {
      halo->M_vir = r->M_vir;
      halo->R_vir = r->R_vir;
      halo->ovdens = r->ovdens;
      halo->Phi0 = r->Phi0;
    }
    if (r->flags & AHFGPU_HALO_RAN_PROFILE)
      shim_write_profiles(halo, r, res.prof + res.prof_off[k] * AHFGPU_PROF_NFIELDS);
  }
  ahfgpu_result_free(&res);
  free(which);
  return AHFGPU_OK;
}
