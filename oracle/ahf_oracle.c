/*
 * ahf_oracle.c -- CPU restatement of AHF's per-halo unbinding + property
 * stage, used as the parity oracle of the GPU library.
 *
 * TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke()
 * as the checker and by bench.py's CPU-baseline leg.  The product never
 * calls it.
 *
 * Each function restates one reference routine (cited file:line, paths
 * inside the AHF source tree) in the reference's own operation order, in
 * FP64 with FP contraction off, so that results are bit-identical to the
 * reference wherever the reference is deterministic.  Two routines of the
 * reference are Numerical-Recipes code (indexx, jacobi); they are NOT
 * restated: the radial sort here is a stable merge sort on (key, list
 * position) and the 3x3 eigen-solver is a cyclic Jacobi written from the
 * textbook rotation formulas.  Consequences: (i) exactly equal radial keys
 * and exactly equal |mom|^2 among the innermost MINPART/2 particles are
 * ordered by list position (the reference's order for such ties is that of
 * its quicksort); (ii) eigenvectors agree with the reference up to sign.
 */
#include "ahf_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* src/param.h:125 and :124 (single-precision build), src/param.h:45       */
#define OR_MACHINE_ZERO 5e-16
#define OR_ZERO         1e-6
#define OR_GRAV         4.3006485e-9
/* src/libahf/ahf_halos.c:3985 FourPiThird with PI of src/libutility/utility.h */
#define OR_PI           3.14159265358979323846264338
/* src/param.h:26 AHF_Rmax_r2_NIGNORE with AHFparticle_Rmax_r2 on (define.h) */
#define OR_NIGNORE      5
#define OR_HIRES_W      1.0  /* src/param.h:16 AHF_HIRES_DM_WEIGHT */

typedef struct {
  const ahfgpu_params *p;
  const ahfgpu_batch  *b;
  double cx, cy, cz;
  /* current member list: batch entry indices */
  uint64_t *ipart;
  uint64_t  npart;
  /* outputs */
  ahfgpu_halo out;
  double     *prof;   /* [nbins][NFIELDS] */
} halo_work;

static inline double wgt(const ahfgpu_batch *b, uint64_t e)
{
  return b->w ? (double)b->w[e] : 1.0;
}

/* signed offset with both periodic wraps (ahf_halos.c:3505-3516) */
static inline double wrap_s(double d)
{
  if (d > 0.5) d -= 1.0;
  if (d < -0.5) d += 1.0;
  return d;
}

/* fabs + single wrap (ahf_halos.c:3381-3389, 3838-3845) */
static inline double wrap_a(double d)
{
  d = fabs(d);
  if (d > 0.5) d -= 1.0;
  return d;
}

static inline double sq(double a) { return a * a; }

/* ------------------------------------------------------------------------
 * sort_halo_particles, src/libahf/ahf_halos.c:5786-5894: key dR^2 with the
 * signed wrap (:5816-5843), ascending (:5846), permute ipart (:5850-5856).
 * Own stable merge sort; ties keep list order.
 * ---------------------------------------------------------------------- */
static uint64_t merge_sort_by_key(uint64_t n, const double *key, uint64_t *ord, uint64_t *tmp)
{
  uint64_t ties = 0;
  for (uint64_t width = 1; width < n; width *= 2) {
    for (uint64_t lo = 0; lo < n; lo += 2 * width) {
      uint64_t mid = lo + width < n ? lo + width : n;
      uint64_t hi = lo + 2 * width < n ? lo + 2 * width : n;
      uint64_t i = lo, j = mid, k = lo;
      while (i < mid && j < hi) {
        if (key[ord[j]] < key[ord[i]]) tmp[k++] = ord[j++];
        else tmp[k++] = ord[i++];
      }
      while (i < mid) tmp[k++] = ord[i++];
      while (j < hi) tmp[k++] = ord[j++];
    }
    memcpy(ord, tmp, n * sizeof(uint64_t));
  }
  for (uint64_t i = 1; i < n; i++)
    if (key[ord[i]] == key[ord[i - 1]]) ties++;
  return ties;
}

static uint64_t sort_halo_particles(halo_work *h)
{
  const ahfgpu_batch *b = h->b;
  uint64_t n = h->npart;
  if (n < (uint64_t)h->p->MINPART) return 0;
  double *key = (double *)malloc(n * sizeof(double));
  uint64_t *ord = (uint64_t *)malloc(n * sizeof(uint64_t));
  uint64_t *tmp = (uint64_t *)malloc(n * sizeof(uint64_t));
  uint64_t *np = (uint64_t *)malloc(n * sizeof(uint64_t));
  for (uint64_t i = 0; i < n; i++) {
    uint64_t e = h->ipart[i];
    double dX = wrap_s((double)b->x[e] - h->cx);
    double dY = wrap_s((double)b->y[e] - h->cy);
    double dZ = wrap_s((double)b->z[e] - h->cz);
    key[i] = (sq(dX) + sq(dY)) + sq(dZ);
    ord[i] = i;
  }
  uint64_t ties = merge_sort_by_key(n, key, ord, tmp);
  for (uint64_t i = 0; i < n; i++) np[i] = h->ipart[ord[i]];
  memcpy(h->ipart, np, n * sizeof(uint64_t));
  free(key); free(ord); free(tmp); free(np);
  h->out.flags |= AHFGPU_HALO_RAN_SORT;
  return ties;
}

/* distance of a member, fabs form (identical value to the signed form) */
static inline double member_dist(const halo_work *h, uint64_t e)
{
  const ahfgpu_batch *b = h->b;
  double dX = wrap_a((double)b->x[e] - h->cx);
  double dY = wrap_a((double)b->y[e] - h->cy);
  double dZ = wrap_a((double)b->z[e] - h->cz);
  return sqrt((sq(dX) + sq(dY)) + sq(dZ));
}

/* ------------------------------------------------------------------------
 * rem_outsideRvir, src/libahf/ahf_halos.c:3687-3889 (AHFprofilerise off):
 * walk outwards while ovdens >= ovlim; the first failing particle is kept
 * (:3818-3861).  Phi0 reset on the first call (:3870-3871).
 * ---------------------------------------------------------------------- */
static void rem_outsideRvir(halo_work *h, int icall)
{
  const ahfgpu_params *p = h->p;
  if (h->npart < (uint64_t)p->MINPART) return;
  double ovdens_vir = p->ovlim;
  uint64_t j = 0, nsph = 0;
  double M = 0.0, R = -1.0, ov = 2 * ovdens_vir;
  while (j < h->npart && ov >= ovdens_vir) {
    uint64_t e = h->ipart[j];
    M += wgt(h->b, e);
    R = member_dist(h, e);
    double V = 4. * OR_PI / 3. * (R * R * R);
    ov = M / V * p->rho_fac / p->rho_vir;
    nsph++;
    j++;
  }
  h->npart = nsph;
  h->out.M_vir = M;
  h->out.R_vir = R;
  h->out.ovdens = ov;
  if (icall == 0) h->out.Phi0 = 0.0;
  h->out.flags |= icall == 0 ? AHFGPU_HALO_RAN_RVIR0 : AHFGPU_HALO_RAN_RVIR1;
}

/* ------------------------------------------------------------------------
 * rem_unbound, src/libahf/ahf_halos.c:3292-3607.
 * ---------------------------------------------------------------------- */
static void rem_unbound(halo_work *h)
{
  const ahfgpu_params *p = h->p;
  const ahfgpu_batch *b = h->b;
  if (h->npart < (uint64_t)p->MINPART) return;
  double v2_tune = sq(p->VescTune);
  uint64_t no_vbulk = (uint64_t)(p->MINPART / 2);
  uint64_t nremove = 4;
  int niter = 0;
  double R_vir = 0.0;            /* reference: uninitialised until a bound particle */
  uint64_t *bound = (uint64_t *)malloc((h->npart ? h->npart : 1) * sizeof(uint64_t));

  h->out.flags |= AHFGPU_HALO_RAN_UNBIND;
  while (nremove > 3) {
    niter++;
    /* Phi0 pass, :3343-3426 */
    double I_now = 0.0, I_prev = 0.0, d_prev = 0.0, M_r = 0.0, Phi0 = 0.0, dist = 0.0;
    for (uint64_t j = 0; j < h->npart; j++) {
      uint64_t e = h->ipart[j];
      M_r += wgt(b, e);
      dist = member_dist(h, e);
      if (dist > OR_MACHINE_ZERO) {
        I_now = M_r / sq(dist);
        double I_mid = (I_now + I_prev) / 2.;
        double dr = dist - d_prev;
        Phi0 += I_mid * dr;
      }
      d_prev = dist;
      I_prev = I_now;
    }
    Phi0 += M_r / dist;                                /* :3423 */
    h->out.Phi0 = Phi0;

    /* bulk-velocity seed, :3441-3470 */
    uint64_t js;
    if (niter == 1) {
      /* rank no_vbulk/2 (1-based) of float |mom|^2 among the innermost
       * no_vbulk members; ties by list position. */
      float m2[64];
      uint64_t pos[64];
      uint64_t nv = no_vbulk < 64 ? no_vbulk : 64;
      for (uint64_t j = 0; j < nv; j++) {
        uint64_t e = h->ipart[j];
        float mx = b->vx[e], my = b->vy[e], mz = b->vz[e];
        volatile float t = mx * mx;
        t = t + my * my;
        t = t + mz * mz;
        m2[j] = t;
        pos[j] = j;
      }
      for (uint64_t i = 1; i < nv; i++) {          /* stable insertion sort */
        float kv = m2[i]; uint64_t kp = pos[i]; uint64_t k = i;
        while (k > 0 && m2[k - 1] > kv) { m2[k] = m2[k - 1]; pos[k] = pos[k - 1]; k--; }
        m2[k] = kv; pos[k] = kp;
      }
      js = pos[no_vbulk / 2 - 1];
    } else {
      js = 0;
    }
    uint64_t es = h->ipart[js];
    double w0 = wgt(b, es);
    double M_vel = w0;
    double VXc = w0 * b->vx[es], VYc = w0 * b->vy[es], VZc = w0 * b->vz[es];

    /* bound pass, :3478-3583 */
    nremove = 0;
    I_now = 0.0; I_prev = 0.0; d_prev = 0.0; M_r = 0.0;
    double M_vir = 0.0, Phi = 0.0;
    uint64_t nb = 0;
    for (uint64_t j = 0; j < h->npart; j++) {
      uint64_t e = h->ipart[j];
      double weight = wgt(b, e);
      M_r += weight;
      double dX = wrap_s((double)b->x[e] - h->cx);
      double dY = wrap_s((double)b->y[e] - h->cy);
      double dZ = wrap_s((double)b->z[e] - h->cz);
      dist = sqrt((sq(dX) + sq(dY)) + sq(dZ));
      double v_esc2;
      if (dist > OR_MACHINE_ZERO) {
        I_now = M_r / sq(dist);
        double I_mid = (I_now + I_prev) / 2.;
        double dr = dist - d_prev;
        Phi += I_mid * dr;
        v_esc2 = (2 * fabs(Phi - Phi0) * p->phi_fac);
      } else {
        v_esc2 = 1e30;
      }
      double VXp = (double)b->vx[e], VYp = (double)b->vy[e], VZp = (double)b->vz[e];
      double dVX = (VXp - VXc / M_vel) * p->v_fac + p->Hubble * (dX) * p->r_fac;
      double dVY = (VYp - VYc / M_vel) * p->v_fac + p->Hubble * (dY) * p->r_fac;
      double dVZ = (VZp - VZc / M_vel) * p->v_fac + p->Hubble * (dZ) * p->r_fac;
      double vel2 = (sq(dVX) + sq(dVY)) + sq(dVZ);
      if (vel2 > v2_tune * v_esc2) {
        nremove++;
      } else {
        M_vel += weight;
        VXc += weight * b->vx[e];
        VYc += weight * b->vy[e];
        VZc += weight * b->vz[e];
        bound[nb++] = e;
        M_vir += weight;
        R_vir = dist;
      }
      I_prev = I_now;
      d_prev = dist;
    }
    memcpy(h->ipart, bound, nb * sizeof(uint64_t));
    if (nb == 0) h->out.flags |= AHFGPU_HALO_NOBOUND;
    h->npart = nb;
    h->out.M_vir = M_vir;
    h->out.R_vir = R_vir;
    if (((double)(h->npart)) < ((double)(p->MINPART))) break;
  }
  h->out.niter = niter;
  free(bound);
}

/* ------------------------------------------------------------------------
 * Numerics used by HaloProfiles
 * ---------------------------------------------------------------------- */

/* smooth3, src/libutility/general.c:548-573 */
static void smooth3(double *data, int64_t nbins, int nsmooth, double *tmp)
{
  if (nsmooth == 0 || nbins < 3) return;
  for (int j = 0; j < nsmooth; j++) {
    tmp[0] = (data[0] + data[1]) / 2.;
    for (int64_t i = 1; i < nbins - 1; i++)
      tmp[i] = (data[i - 1] + data[i] + data[i + 1]) / 3.;
    tmp[nbins - 1] = (data[nbins - 1] + data[nbins - 2]) / 2.;
    memcpy(data, tmp, (size_t)nbins * sizeof(double));
  }
}

/* find_max, src/libutility/general.c:608-650: first strict maximum of the
 * smoothed copy over [0, nbins-2]; the right-hand approach of the reference
 * revisits only indices already scanned and never moves the pick.         */
static void find_max(const double *x, const double *y_raw, int64_t nbins, int ismooth,
                     double *x_max, double *y_max)
{
  double *y = (double *)malloc((size_t)(nbins > 0 ? nbins : 1) * sizeof(double));
  double *tmp = (double *)malloc((size_t)(nbins > 0 ? nbins : 1) * sizeof(double));
  memcpy(y, y_raw, (size_t)nbins * sizeof(double));
  smooth3(y, nbins, ismooth, tmp);
  double ymax = -10.0;
  int64_t i0 = nbins - 1;
  for (int64_t i = 0; i < nbins - 1; i++)
    if (y[i] > ymax) { ymax = y[i]; i0 = i; }
  int64_t i1 = i0;
  for (int64_t i = (nbins - 1 + i0) / 2; i > i0; i--)
    if (y[i] > ymax) { ymax = y[i]; i1 = i; }
  *x_max = (x[i0] + x[i1]) / 2;
  *y_max = (y_raw[i0] + y_raw[i1]) / 2;
  free(y); free(tmp);
}

/* Symmetric 3x3 eigen-decomposition by cyclic Jacobi rotations
 * (Golub & Van Loan, "Matrix Computations", sym.schur2 + cyclic sweep).
 * On return d[k] are eigenvalues and column k of v the eigenvector.       */
static void jacobi3(const double a_in[3][3], double d[3], double v[3][3])
{
  double a[3][3];
  memcpy(a, a_in, sizeof(a));
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) v[i][j] = (i == j) ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 64; sweep++) {
    double off = fabs(a[0][1]) + fabs(a[0][2]) + fabs(a[1][2]);
    if (off == 0.0) break;
    for (int pp = 0; pp < 2; pp++) {
      for (int qq = pp + 1; qq < 3; qq++) {
        double apq = a[pp][qq];
        if (apq == 0.0) continue;
        double app = a[pp][pp], aqq = a[qq][qq];
        /* negligible element relative to both diagonal entries */
        if (sweep > 3 && fabs(app) + 100.0 * fabs(apq) == fabs(app) &&
            fabs(aqq) + 100.0 * fabs(apq) == fabs(aqq)) {
          a[pp][qq] = a[qq][pp] = 0.0;
          continue;
        }
        double tau = (aqq - app) / (2.0 * apq);
        double t = (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
        double c = 1.0 / sqrt(1.0 + t * t);
        double s = t * c;
        /* A <- J^T A J with J the (pp,qq) rotation [c s; -s c] */
        for (int k = 0; k < 3; k++) {
          double akp = a[k][pp], akq = a[k][qq];
          a[k][pp] = c * akp - s * akq;
          a[k][qq] = s * akp + c * akq;
        }
        for (int k = 0; k < 3; k++) {
          double apk = a[pp][k], aqk = a[qq][k];
          a[pp][k] = c * apk - s * aqk;
          a[qq][k] = s * apk + c * aqk;
        }
        a[pp][qq] = a[qq][pp] = 0.0;
        for (int k = 0; k < 3; k++) {
          double vkp = v[k][pp], vkq = v[k][qq];
          v[k][pp] = c * vkp - s * vkq;
          v[k][qq] = s * vkp + c * vkq;
        }
      }
    }
  }
  for (int k = 0; k < 3; k++) d[k] = a[k][k];
}

/* get_axes, src/libutility/specific.c:135-178: eigenvalues descending
 * (axis1 largest); column 0/1/2 of itensor = eigenvector of axis1/2/3.     */
static void get_axes(double it[3][3], double *axis1, double *axis2, double *axis3)
{
  double d[3], v[3][3];
  jacobi3((const double (*)[3])it, d, v);
  int o[3] = {0, 1, 2};
  for (int i = 1; i < 3; i++) {                 /* stable, descending */
    int k = o[i], j = i;
    while (j > 0 && d[o[j - 1]] < d[k]) { o[j] = o[j - 1]; j--; }
    o[j] = k;
  }
  *axis1 = d[o[0]]; *axis2 = d[o[1]]; *axis3 = d[o[2]];
  for (int c = 0; c < 3; c++)
    for (int r = 0; r < 3; r++) it[r][c] = v[r][o[c]];
}

/* binning_parameter, src/libutility/specific.c:259-322 */
static void binning_parameter(const halo_work *h, int *nbins, double *dist_min, double *dist_max)
{
  const ahfgpu_batch *b = h->b;
  int nb = (int)(6.2 * (log10((double)h->npart)) - 3.5);
  nb *= 1;
  if (nb < 2) nb = 2;
  *nbins = nb;
  long npart = (long)floor(((double)h->p->MINPART / 10.) + 0.5);
  *dist_min = -1.0;
  while (npart < (long)h->npart - 1 && *dist_min < OR_MACHINE_ZERO) {
    uint64_t e = h->ipart[npart];
    double dX = fabs(b->x[e] - h->cx), dY = fabs(b->y[e] - h->cy), dZ = fabs(b->z[e] - h->cz);
    if (dX > 0.5) dX = 1.0 - dX;
    if (dY > 0.5) dY = 1.0 - dY;
    if (dZ > 0.5) dZ = 1.0 - dZ;
    *dist_min = sqrt((sq(dX) + sq(dY)) + sq(dZ));
    npart++;
  }
  uint64_t e = h->ipart[h->npart - 1];
  double dX = fabs(b->x[e] - h->cx), dY = fabs(b->y[e] - h->cy), dZ = fabs(b->z[e] - h->cz);
  if (dX > 0.5) dX = 1.0 - dX;
  if (dY > 0.5) dY = 1.0 - dY;
  if (dZ > 0.5) dZ = 1.0 - dZ;
  *dist_max = sqrt((sq(dX) + sq(dY)) + sq(dZ));
  if (*dist_min < OR_MACHINE_ZERO) *dist_min = *dist_max / 2.;
}

/* calc_cNFW, src/libutility/specific.c:2041-2072 (bisection on [2.2,100]) */
static double cnfw_root(double c, double v2r) { return 0.216 * c / (log(1 + c) - c / (1 + c)) - v2r; }
static double calc_cNFW(double V2_max, double V2_vir)
{
  double r = V2_max / V2_vir;
  if (r <= 1 || r > 5.9) return -1;
  double a = 2.2, bb = 100, c;
  while (bb - a > 1e-3) {
    c = (a + bb) / 2;
    if (cnfw_root(a, r) * cnfw_root(c, r) > 0) a = c; else bb = c;
  }
  return (a + bb) / 2.0;
}

/* calc_R1 / calc_cR1, src/libutility/specific.c:1977-2018 */
static double cr1_root(double c, double R1)
{
  return (c - 2.0 * log(1.0 + c) + c / (1.0 + c)) / (c * (log(1.0 + c) - c / (1.0 + c))) - R1;
}
static double calc_R1(const double *prof, int nbins)
{
#define PR(i, f) prof[(size_t)(i) * AHFGPU_PROF_NFIELDS + (f)]
  double r0h = PR(0, AHFGPU_PROF_R) / 2.0;
  double R1 = (r0h * r0h * r0h) * PR(0, AHFGPU_PROF_DENS) * (PR(0, AHFGPU_PROF_R));
  for (int i = 1; i < nbins; i++) {
    double rmid = (PR(i, AHFGPU_PROF_R) + PR(i - 1, AHFGPU_PROF_R)) / 2.0;
    double dr = PR(i, AHFGPU_PROF_R) - PR(i - 1, AHFGPU_PROF_R);
    R1 += (rmid * rmid * rmid) * PR(i, AHFGPU_PROF_DENS) * dr;
  }
#undef PR
  return 4 * OR_PI * R1;
}
static double calc_cR1(double R1)
{
  if (R1 <= 0.19 || 0.585 <= R1) return -1.0;
  double a = 1.0, bb = 500.0, c;
  while (bb - a > 1e-3) {
    c = (a + bb) / 2;
    if (cr1_root(a, R1) * cr1_root(c, R1) > 0) a = c; else bb = c;
  }
  return (a + bb) / 2.0;
}

/* calc_lambdaE, src/libahf/ahf_halos.c:3937-3953 */
static double calc_lambdaE(const ahfgpu_params *p, double absL, double Mhalo, double Mass,
                           double Ekin, double Epot)
{
  double t1 = sqrt(p->m_fac * Mhalo);
  t1 = t1 * t1 * t1;
  double t2 = Ekin * p->m_fac * (p->v_fac * p->v_fac);
  double t3 = Epot * p->m_fac * p->phi_fac;
  t2 = fabs(t2 + t3);
  t2 = sqrt(t2);
  t1 = t2 / t1;
  t2 = p->m_fac * p->r_fac * p->v_fac * absL;
  t2 = t2 / (p->m_fac * Mass);
  t3 = t1 * t2;
  return t3 / OR_GRAV;
}

/* ------------------------------------------------------------------------
 * HaloProfiles, src/libahf/ahf_halos.c:3961-5261 (default flags:
 * AHFparticle_Rmax_r2, no GAS_PARTICLES, no AHFshellshape).
 * ---------------------------------------------------------------------- */
static void HaloProfiles(halo_work *h)
{
  const ahfgpu_params *p = h->p;
  const ahfgpu_batch *b = h->b;
  if (h->npart < (uint64_t)p->MINPART) return;
  const double FourPiThird = 4. * OR_PI / 3.;
  int nbins;
  double dist_min, dist_max;
  binning_parameter(h, &nbins, &dist_min, &dist_max);
  double ldist_min = log10(dist_min), ldist_max = log10(dist_max);
  double ldr = (ldist_max - ldist_min) / (double)nbins;
  h->prof = (double *)calloc((size_t)nbins * AHFGPU_PROF_NFIELDS, sizeof(double));
  h->out.nbins = nbins;
  uint64_t n = h->npart;
  double *Vcirc2 = (double *)calloc(n, sizeof(double));
  double *dens_r2 = (double *)calloc(n, sizeof(double));
  double *ovdens = (double *)calloc(n, sizeof(double));
  double *radius = (double *)calloc(n, sizeof(double));

  double Phi0 = h->out.Phi0, Phi = 0.0, pre_dist = 0.0, I_prev = 0.0, I_now = 0.0;
  uint64_t npart = 0;
  double M_prev = 0, V_prev = 0.0, M_sphere_prev = 0.0, prev_dist = 0.0;
  double M_sphere = 0.0, VXc = 0.0, VYc = 0.0, VZc = 0.0;
  double a11 = 0, a22 = 0, a33 = 0, a12 = 0, a13 = 0, a23 = 0;
  double sig_v = 0, Lx = 0, Ly = 0, Lz = 0, CoM[3] = {0, 0, 0};
  double Epot = 0, Ekin = 0, Emin = 1e30, v_esc2 = 0.0;
  int64_t mb = -1;
  double M_hires = 0.0, M_lores = 0.0;
  const double Xc = h->cx, Yc = h->cy, Zc = h->cz;
  uint64_t jpart = 0;
  double cur_dist = -1.0;

  for (int ibin = 0; ibin < nbins; ibin++) {
    double lcur_rad = ldist_min + ((double)ibin + 1) * ldr;
    double cur_rad = pow(10., lcur_rad);
    if (ibin == nbins - 1) cur_rad = dist_max + OR_ZERO;
    while (cur_dist < cur_rad && jpart < n) {
      uint64_t e = h->ipart[jpart];
      npart++;
      double weight = wgt(b, e);
      if (b->w) {
        if (fabs(weight - OR_HIRES_W) < OR_ZERO) M_hires += weight;
        else if (weight > OR_HIRES_W) M_lores += weight;
      } else {
        M_hires += weight;
      }
      M_sphere += weight;
      double dX = wrap_s((double)b->x[e] - Xc);
      double dY = wrap_s((double)b->y[e] - Yc);
      double dZ = wrap_s((double)b->z[e] - Zc);
      cur_dist = sqrt((sq(dX) + sq(dY)) + sq(dZ));
      CoM[0] += weight * (Xc + dX);
      CoM[1] += weight * (Yc + dY);
      CoM[2] += weight * (Zc + dZ);
      a11 += weight * dX * dX;
      a22 += weight * dY * dY;
      a33 += weight * dZ * dZ;
      a12 += weight * dX * dY;
      a13 += weight * dX * dZ;
      a23 += weight * dY * dZ;
      VXc += weight * b->vx[e];
      VYc += weight * b->vy[e];
      VZc += weight * b->vz[e];
      double VXp = (double)b->vx[e], VYp = (double)b->vy[e], VZp = (double)b->vz[e];
      double dVX = (VXp - VXc / M_sphere);
      double dVY = (VYp - VYc / M_sphere);
      double dVZ = (VZp - VZc / M_sphere);
      Lx += weight * (dY * dVZ - dZ * dVY);
      Ly += weight * (dZ * dVX - dX * dVZ);
      Lz += weight * (dX * dVY - dY * dVX);
      dVX += p->Hubble * dX * p->r_fac / p->v_fac;
      dVY += p->Hubble * dY * p->r_fac / p->v_fac;
      dVZ += p->Hubble * dZ * p->r_fac / p->v_fac;
      double Tpart = weight * ((sq(dVX) + sq(dVY)) + sq(dVZ));
      double Upart;
      if (cur_dist > OR_MACHINE_ZERO) {
        I_now = M_sphere / sq(cur_dist);
        double I_mid = (I_now + I_prev) / 2.;
        Phi += I_mid * (cur_dist - pre_dist);
        Upart = (Phi - Phi0) * weight;
      } else {
        Upart = (Phi - Phi0) * weight;
      }
      v_esc2 = 2 * fabs(Upart) / weight;
      I_prev = I_now;
      pre_dist = cur_dist;
      Epot += Upart;
      sig_v += Tpart;
      Ekin += Tpart;
      double Epart = (0.5 * Tpart + Upart);
      if (Epart < Emin) { Emin = Epart; mb = (int64_t)e; }
      radius[jpart] = cur_dist;
      ovdens[jpart] = M_sphere / (FourPiThird * (cur_dist * cur_dist * cur_dist));
      double dV = FourPiThird * ((cur_dist * cur_dist * cur_dist) - (prev_dist * prev_dist * prev_dist));
      double dM = M_sphere - M_sphere_prev;
      Vcirc2[jpart] = M_sphere / cur_dist;
      M_sphere_prev = M_sphere;
      double rm = (cur_dist + prev_dist) / 2.;
      dens_r2[jpart] = dM / dV * (rm * rm);
      prev_dist = cur_dist;
      jpart++;
    }
    double Volume = FourPiThird * (cur_rad * cur_rad * cur_rad);
    double dM = M_sphere - M_prev;
    double dV = Volume - V_prev;
    double itensor[3][3], axis1, axis2, axis3;
    if (npart > 10) {
      itensor[0][0] = a11; itensor[1][1] = a22; itensor[2][2] = a33;
      itensor[0][1] = a12; itensor[1][0] = a12;
      itensor[0][2] = a13; itensor[2][0] = a13;
      itensor[1][2] = a23; itensor[2][1] = a23;
      get_axes(itensor, &axis1, &axis2, &axis3);
    } else {
      memset(itensor, 0, sizeof(itensor));
      axis1 = 1; axis2 = 0; axis3 = 0;
    }
    double *row = h->prof + (size_t)ibin * AHFGPU_PROF_NFIELDS;
    row[AHFGPU_PROF_R] = cur_rad;
    row[AHFGPU_PROF_NPART] = (double)npart;
    row[AHFGPU_PROF_NVPART] = M_sphere;
    row[AHFGPU_PROF_OVDENS] = M_sphere / Volume;
    row[AHFGPU_PROF_DENS] = dV > 0 ? dM / dV : 0.0;
    row[AHFGPU_PROF_V2_CIRC] = M_sphere / cur_rad;
    row[AHFGPU_PROF_V_ESC2] = v_esc2;
    row[AHFGPU_PROF_SIG_V] = sqrt(sig_v / M_sphere);
    row[AHFGPU_PROF_EKIN] = 0.5 * Ekin;
    row[AHFGPU_PROF_EPOT] = 0.5 * Epot;
    row[AHFGPU_PROF_LX] = Lx;
    row[AHFGPU_PROF_LY] = Ly;
    row[AHFGPU_PROF_LZ] = Lz;
    row[AHFGPU_PROF_E1X] = itensor[0][0];
    row[AHFGPU_PROF_E1Y] = itensor[1][0];
    row[AHFGPU_PROF_E1Z] = itensor[2][0];
    row[AHFGPU_PROF_E2X] = itensor[0][1];
    row[AHFGPU_PROF_E2Y] = itensor[1][1];
    row[AHFGPU_PROF_E2Z] = itensor[2][1];
    row[AHFGPU_PROF_E3X] = itensor[0][2];
    row[AHFGPU_PROF_E3Y] = itensor[1][2];
    row[AHFGPU_PROF_E3Z] = itensor[2][2];
    row[AHFGPU_PROF_AXIS1] = 1.0;
    if (axis1 > 0.) {
      row[AHFGPU_PROF_AXIS2] = sqrt(axis2 / axis1);
      row[AHFGPU_PROF_AXIS3] = sqrt(axis3 / axis1);
    } else {
      row[AHFGPU_PROF_AXIS2] = 0.0;
      row[AHFGPU_PROF_AXIS3] = 0.0;
    }
    M_prev = M_sphere;
    V_prev = Volume;
  }
  for (int k = 0; k < 3; k++) CoM[k] = fmod(CoM[k] / M_sphere + 1., 1.);

  double x_max, y_max, r2, R_max;
  int64_t np5 = (int64_t)n - OR_NIGNORE;
  find_max(radius + OR_NIGNORE, dens_r2 + OR_NIGNORE, np5, 3, &x_max, &y_max);
  r2 = x_max;
  find_max(radius + OR_NIGNORE, Vcirc2 + OR_NIGNORE, np5, 1, &x_max, &y_max);
  R_max = x_max;
  int64_t ib = 0;
  while (radius[ib] < x_max && ib < (int64_t)n - 1) ib++;
  double M_max = ovdens[ib] * FourPiThird * (radius[ib] * radius[ib] * radius[ib]);
  double V_max = M_max / R_max;
  free(ovdens); free(Vcirc2); free(radius); free(dens_r2);

  const double *last = h->prof + (size_t)(nbins - 1) * AHFGPU_PROF_NFIELDS;
  Lx = last[AHFGPU_PROF_LX]; Ly = last[AHFGPU_PROF_LY]; Lz = last[AHFGPU_PROF_LZ];
  double absAngMom = sqrt((sq(Lx) + sq(Ly)) + sq(Lz));
  ahfgpu_halo *o = &h->out;
  o->M_vir = M_sphere;
  o->vel[0] = VXc / M_sphere; o->vel[1] = VYc / M_sphere; o->vel[2] = VZc / M_sphere;
  o->R_max = R_max;
  o->V2_max = V_max;
  o->r2 = r2;
  o->sigV = last[AHFGPU_PROF_SIG_V];
  o->v_esc2 = last[AHFGPU_PROF_V_ESC2];
  o->Ekin = last[AHFGPU_PROF_EKIN];
  o->Epot = last[AHFGPU_PROF_EPOT];
  o->axis[0] = last[AHFGPU_PROF_AXIS1]; o->axis[1] = last[AHFGPU_PROF_AXIS2]; o->axis[2] = last[AHFGPU_PROF_AXIS3];
  o->E1[0] = last[AHFGPU_PROF_E1X]; o->E1[1] = last[AHFGPU_PROF_E1Y]; o->E1[2] = last[AHFGPU_PROF_E1Z];
  o->E2[0] = last[AHFGPU_PROF_E2X]; o->E2[1] = last[AHFGPU_PROF_E2Y]; o->E2[2] = last[AHFGPU_PROF_E2Z];
  o->E3[0] = last[AHFGPU_PROF_E3X]; o->E3[1] = last[AHFGPU_PROF_E3Y]; o->E3[2] = last[AHFGPU_PROF_E3Z];
  if (absAngMom > 0) {
    o->AngMom[0] = Lx / absAngMom; o->AngMom[1] = Ly / absAngMom; o->AngMom[2] = Lz / absAngMom;
    o->lambda = absAngMom / o->M_vir / sqrt(2. * o->M_vir * o->R_vir);
    o->lambda *= p->v_fac * sqrt(p->r_fac / (OR_GRAV * p->m_fac));
    o->lambdaE = calc_lambdaE(p, absAngMom, o->M_vir, o->M_vir, o->Ekin, o->Epot);
  } else {
    o->AngMom[0] = o->AngMom[1] = o->AngMom[2] = 0.0;
    o->lambda = 0.0;
    o->lambdaE = 0.0;
  }
  o->cNFW = calc_cNFW(o->V2_max, o->M_vir / o->R_vir);
  o->R1 = calc_R1(h->prof, nbins) / o->M_vir / o->R_vir;
  o->cR1 = calc_cR1(o->R1);
  {
    const double *pl = h->prof + (size_t)(nbins - 2) * AHFGPU_PROF_NFIELDS;
    double Ts = 2.0 * (last[AHFGPU_PROF_EKIN] - pl[AHFGPU_PROF_EKIN]);
    double frad = fabs(pl[AHFGPU_PROF_R] / last[AHFGPU_PROF_R]);
    o->SurfP = -0.125 * ((1. + frad) * (1. + frad) * (1. + frad)) / (1. - (frad * frad * frad)) * Ts;
  }
  o->fMhires = M_hires > 0 ? M_hires / (M_hires + M_lores) : 0.0;
  if (mb >= 0) {
    double dX = fabs(b->x[mb] - Xc), dY = fabs(b->y[mb] - Yc), dZ = fabs(b->z[mb] - Zc);
    if (dX > 0.5) dX -= 1.0;
    if (dY > 0.5) dY -= 1.0;
    if (dZ > 0.5) dZ -= 1.0;
    o->mbp_offset = sqrt((sq(dX) + sq(dY)) + sq(dZ));
    o->pos_mbp[0] = b->x[mb]; o->pos_mbp[1] = b->y[mb]; o->pos_mbp[2] = b->z[mb];
    o->vel_mbp[0] = b->vx[mb]; o->vel_mbp[1] = b->vy[mb]; o->vel_mbp[2] = b->vz[mb];
  } else {
    o->mbp_offset = -1.0;
    o->flags |= AHFGPU_HALO_NO_MBP;
  }
  {
    double dX = fabs(CoM[0] - Xc), dY = fabs(CoM[1] - Yc), dZ = fabs(CoM[2] - Zc);
    if (dX > 0.5) dX -= 1.0;
    if (dY > 0.5) dY -= 1.0;
    if (dZ > 0.5) dZ -= 1.0;
    o->com_offset = sqrt((sq(dX) + sq(dY)) + sq(dZ));
  }
  o->pos_com[0] = CoM[0]; o->pos_com[1] = CoM[1]; o->pos_com[2] = CoM[2];
  o->flags |= AHFGPU_HALO_RAN_PROFILE;
}

/* ahf_halos_sfc_constructHalo minus the gather, src/libahf/ahf_halos_sfc.c:118-169 */
static uint64_t construct_halo(halo_work *h)
{
  uint64_t ties = 0;
  if (h->npart == 0) { h->out.flags |= AHFGPU_HALO_EMPTY; return 0; }
  ties = sort_halo_particles(h);
  rem_outsideRvir(h, 0);
  rem_unbound(h);
  rem_outsideRvir(h, 1);
  HaloProfiles(h);
  h->out.npart = h->npart;
  return ties;
}

int ahforacle_max_threads(void)
{
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

int ahforacle_construct_halos(const ahfgpu_params *params, const ahfgpu_batch *batch,
                              ahfgpu_result *res, int nthreads)
{
  if (!params || !batch || !res || batch->nhalo < 0 || !batch->off) return AHFGPU_ERR_INVALID;
  if (params->MINPART < 4 || params->MINPART > 128) return AHFGPU_ERR_INVALID;
  int64_t nh = batch->nhalo;
  memset(res, 0, sizeof(*res));
  res->nhalo = nh;
  halo_work *hw = (halo_work *)calloc((size_t)(nh > 0 ? nh : 1), sizeof(halo_work));
  if (!hw) return AHFGPU_ERR_OOM;
  uint64_t ties = 0;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic) num_threads(nthreads) reduction(+:ties)
#endif
  for (int64_t i = 0; i < nh; i++) {
    halo_work *h = &hw[i];
    h->p = params;
    h->b = batch;
    h->cx = batch->cx[i]; h->cy = batch->cy[i]; h->cz = batch->cz[i];
    uint64_t o0 = batch->off[i], o1 = batch->off[i + 1];
    h->npart = o1 - o0;
    h->ipart = (uint64_t *)malloc((h->npart ? h->npart : 1) * sizeof(uint64_t));
    for (uint64_t j = 0; j < h->npart; j++) h->ipart[j] = o0 + j;
    ties += construct_halo(h);
  }
  /* pack */
  res->halo = (ahfgpu_halo *)calloc((size_t)(nh > 0 ? nh : 1), sizeof(ahfgpu_halo));
  res->member_off = (uint64_t *)calloc((size_t)nh + 1, sizeof(uint64_t));
  res->prof_off = (uint64_t *)calloc((size_t)nh + 1, sizeof(uint64_t));
  for (int64_t i = 0; i < nh; i++) {
    res->member_off[i + 1] = res->member_off[i] + hw[i].npart;
    res->prof_off[i + 1] = res->prof_off[i] + (uint64_t)hw[i].out.nbins;
  }
  res->member = (uint64_t *)malloc((res->member_off[nh] ? res->member_off[nh] : 1) * sizeof(uint64_t));
  res->prof = (double *)malloc((res->prof_off[nh] ? res->prof_off[nh] : 1) * AHFGPU_PROF_NFIELDS * sizeof(double));
  for (int64_t i = 0; i < nh; i++) {
    halo_work *h = &hw[i];
    h->out.npart = h->npart;
    res->halo[i] = h->out;
    for (uint64_t j = 0; j < h->npart; j++)
      res->member[res->member_off[i] + j] = batch->gidx ? batch->gidx[h->ipart[j]] : h->ipart[j];
    if (h->out.nbins)
      memcpy(res->prof + res->prof_off[i] * AHFGPU_PROF_NFIELDS, h->prof,
             (size_t)h->out.nbins * AHFGPU_PROF_NFIELDS * sizeof(double));
    free(h->ipart);
    free(h->prof);
  }
  free(hw);
  res->stats.n_particles_in = nh ? batch->off[nh] : 0;
  res->stats.n_kept = res->member_off[nh];
  res->stats.n_key_ties = ties;
  return AHFGPU_OK;
}

void ahforacle_result_free(ahfgpu_result *r)
{
  if (!r) return;
  free(r->halo); free(r->member_off); free(r->member); free(r->prof_off); free(r->prof);
  memset(r, 0, sizeof(*r));
}


/* ---------------------------------------------------------------------------
 * Particle gather, src/libahf/ahf_halos_sfc.c:171-412.  The reference visits
 * the 3x3x3 cells (at the coarsest level whose cells exceed 1.001 gatherRad,
 * local_getSuitableBits :236-255) around the centre's cell, which contain
 * the whole gather sphere, and keeps each particle with
 * islessequal(dist2, gatherRad2) (:329-332), dist2 from LOCAL_CAL_DXYZ
 * (:69-78) on the float position promoted to double.  The kept set is
 * therefore every particle within the radius; this restatement lists it in
 * ascending particle index (the reference's order follows its SFC cells).
 * Candidate particles come from a uniform grid (below), a superset of the
 * sphere; the kept set is decided by the reference's test alone.
 */
static double gather_d2(float px, float py, float pz, double cx, double cy, double cz)
{
  double dx = fabs((double)px - cx), dy = fabs((double)py - cy), dz = fabs((double)pz - cz);
  if (dx > 0.5) dx = 1.0 - dx;
  if (dy > 0.5) dy = 1.0 - dy;
  if (dz > 0.5) dz = 1.0 - dz;
  return dx * dx + dy * dy + dz * dz;
}

/* Candidates come from a uniform grid of G^3 cells (about half the median
 * radius, 8..256 per axis), scanned one cell beyond each sphere; the test
 * itself is the reference's.  Lists in ascending particle index.          */
static int gather_cell(float x, int G)
{
  int c = (int)((double)x * (double)G);
  return c < 0 ? 0 : (c >= G ? G - 1 : c);
}

static int cmp_u64(const void *a, const void *b)
{
  uint64_t x = *(const uint64_t *)a, y = *(const uint64_t *)b;
  return x < y ? -1 : x > y;
}

static double median_radius(const double *rad, int64_t nhalo)
{
  double *t = (double *)malloc((size_t)(nhalo > 0 ? nhalo : 1) * sizeof(double));
  if (!t) return 0.5;
  memcpy(t, rad, (size_t)nhalo * sizeof(double));
  for (int64_t i = 1; i < nhalo; i++) {           /* insertion sort is enough here */
    double v = t[i];
    int64_t j = i;
    while (j > 0 && t[j - 1] > v) { t[j] = t[j - 1]; j--; }
    t[j] = v;
  }
  double m = nhalo > 0 ? t[nhalo / 2] : 0.5;
  free(t);
  return m;
}

/* one halo's matches, ascending; returns the count (buf NULL: count only) */
static uint64_t gather_one(const float *x, const float *y, const float *z, const uint64_t *start,
                           const uint64_t *order, int G, double cx, double cy, double cz, double r,
                           uint64_t *buf)
{
  const double r2 = r * r, cc[3] = {cx, cy, cz};
  int lo[3], nd[3];
  for (int d = 0; d < 3; d++) {
    long long a = (long long)floor((cc[d] - r) * G) - 1, b = (long long)floor((cc[d] + r) * G) + 1;
    if (!(r >= 0.0) || b - a + 1 >= G) { lo[d] = 0; nd[d] = G; }
    else { lo[d] = (int)(((a % G) + G) % G); nd[d] = (int)(b - a + 1); }
  }
  uint64_t k = 0;
  for (int i = 0; i < nd[0]; i++)
    for (int j = 0; j < nd[1]; j++)
      for (int l = 0; l < nd[2]; l++) {
        uint64_t c = ((uint64_t)((lo[0] + i) % G) * G + (uint64_t)((lo[1] + j) % G)) * G + (uint64_t)((lo[2] + l) % G);
        for (uint64_t q = start[c]; q < start[c + 1]; q++) {
          uint64_t p = order[q];
          if (gather_d2(x[p], y[p], z[p], cx, cy, cz) <= r2) {
            if (buf) buf[k] = p;
            k++;
          }
        }
      }
  if (buf) qsort(buf, (size_t)k, sizeof(uint64_t), cmp_u64);
  return k;
}

int ahforacle_gather(uint64_t n, const float *x, const float *y, const float *z, int64_t nhalo,
                     const double *cx, const double *cy, const double *cz, const double *rad,
                     uint64_t *out_off, uint64_t **out_idx)
{
  const double rmed = median_radius(rad, nhalo);
  int G = rmed > 0 ? (int)fmin(256.0, fmax(8.0, floor(2.0 / rmed))) : 8;
  const uint64_t m = (uint64_t)G * G * G;
  uint64_t *start = (uint64_t *)calloc(m + 1, sizeof(uint64_t));
  uint64_t *order = (uint64_t *)malloc((size_t)(n ? n : 1) * sizeof(uint64_t));
  uint64_t *cnt = (uint64_t *)calloc((size_t)(nhalo > 0 ? nhalo : 1), sizeof(uint64_t));
  if (!start || !order || !cnt) { free(start); free(order); free(cnt); return -1; }
  /* counting sort of the particles by cell (particle order within a cell) */
  for (uint64_t i = 0; i < n; i++) {
    uint64_t c = ((uint64_t)gather_cell(x[i], G) * G + (uint64_t)gather_cell(y[i], G)) * G + (uint64_t)gather_cell(z[i], G);
    start[c + 1]++;
  }
  for (uint64_t c = 0; c < m; c++) start[c + 1] += start[c];
  {
    uint64_t *fill = (uint64_t *)malloc((size_t)m * sizeof(uint64_t));
    if (!fill) { free(start); free(order); free(cnt); return -1; }
    memcpy(fill, start, (size_t)m * sizeof(uint64_t));
    for (uint64_t i = 0; i < n; i++) {
      uint64_t c = ((uint64_t)gather_cell(x[i], G) * G + (uint64_t)gather_cell(y[i], G)) * G + (uint64_t)gather_cell(z[i], G);
      order[fill[c]++] = i;
    }
    free(fill);
  }
#pragma omp parallel for schedule(dynamic)
  for (int64_t h = 0; h < nhalo; h++) cnt[h] = gather_one(x, y, z, start, order, G, cx[h], cy[h], cz[h], rad[h], NULL);
  out_off[0] = 0;
  for (int64_t h = 0; h < nhalo; h++) out_off[h + 1] = out_off[h] + cnt[h];
  uint64_t tot = nhalo > 0 ? out_off[nhalo] : 0;
  uint64_t *idx = (uint64_t *)malloc((size_t)(tot ? tot : 1) * sizeof(uint64_t));
  if (!idx) { free(start); free(order); free(cnt); return -1; }
#pragma omp parallel for schedule(dynamic)
  for (int64_t h = 0; h < nhalo; h++)
    gather_one(x, y, z, start, order, G, cx[h], cy[h], cz[h], rad[h], idx + out_off[h]);
  free(start); free(order); free(cnt);
  *out_idx = idx;
  return 0;
}

void ahforacle_gather_free(uint64_t *idx) { free(idx); }


/* ---------------------------------------------------------------------------
 * Gather radii, src/libahf/ahf_halos.c:2987-3051.  The reference walks the
 * haloes in order of decreasing particle count and, for each, every halo
 * before it with strictly more particles: the smallest periodic squared
 * distance (LOCAL-style fold at 0.5, dx*dx + dy*dy + dz*dz) starting from
 * 1e11 (:2535), then sqrt(.) * 0.5, max_rad when there is no such halo, then
 * MAX with R_vir and MIN with max_rad = MIN(MaxGatherRad / boxsize, 1/4).
 * The set of candidates does not depend on how ties in the count are
 * ordered, so a plain scan over all haloes restates it.                    */
void ahforacle_gather_radii(int64_t nhalo, const uint64_t *npart, const double *cx, const double *cy,
                            const double *cz, const double *rvir, double max_gather_rad_box, double *rad)
{
  const double maxr = max_gather_rad_box < 0.25 ? max_gather_rad_box : 0.25;
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t i = 0; i < nhalo; i++) {
    double best = 100000000000.0;
    int64_t count = 0;
    for (int64_t j = 0; j < nhalo; j++) {
      if (j == i || !(npart[j] > npart[i])) continue;
      double dx = fabs(cx[i] - cx[j]), dy = fabs(cy[i] - cy[j]), dz = fabs(cz[i] - cz[j]);
      if (dx > 0.5) dx = 1.0 - dx;
      if (dy > 0.5) dy = 1.0 - dy;
      if (dz > 0.5) dz = 1.0 - dz;
      double d2 = dx * dx + dy * dy + dz * dz;
      if (d2 < best) best = d2;
      count++;
    }
    double r = sqrt(best) * 0.5;
    if (count == 0) r = maxr;
    r = r > rvir[i] ? r : rvir[i];
    r = r < maxr ? r : maxr;
    rad[i] = r;
  }
}


/* ---------------------------------------------------------------------------
 * AHF_particles, WriteParticlesLegacy (src/libahf/ahf_io.c:1095-1175), default
 * build (no GAS_PARTICLES, SUSSING2013 or AHFnewHaloIDs): the header holds
 * the good-halo count (written as 0, rewritten with "%15lu" after the rewind
 * :1167-1170, so the first line is that count and the original newline).   */
#include <inttypes.h>
#include <stdio.h>

int ahforacle_write_particles(const uint64_t *ids, const float *w, int64_t nhalo, const uint64_t *member_off,
                              const uint64_t *member, const uint64_t *halo_npart, const int64_t *order,
                              int64_t minpart, unsigned char **out, uint64_t *nbytes)
{
  uint64_t cap = 1 << 20, used = 0;
  char *buf = (char *)malloc(cap);
  if (!buf) return -1;
  unsigned long good = 0;
  for (int64_t j = 0; j < nhalo; j++)
    if ((int64_t)halo_npart[order[j]] >= minpart) good++;
  char line[96];
#define PUT(...)                                                             \
  do {                                                                       \
    int n_ = snprintf(line, sizeof line, __VA_ARGS__);                       \
    if (used + (uint64_t)n_ > cap) {                                         \
      while (used + (uint64_t)n_ > cap) cap *= 2;                            \
      char *t_ = (char *)realloc(buf, cap);                                  \
      if (!t_) { free(buf); return -1; }                                     \
      buf = t_;                                                              \
    }                                                                        \
    memcpy(buf + used, line, (size_t)n_);                                    \
    used += (uint64_t)n_;                                                    \
  } while (0)
  PUT("%15lu\n", good);
  for (int64_t j = 0; j < nhalo; j++) {
    const int64_t i = order[j];
    if (!((int64_t)halo_npart[i] >= minpart)) continue;
    PUT("%lu %10ld\n", (unsigned long)halo_npart[i], (long)j);
    for (uint64_t k = member_off[i]; k < member_off[i] + halo_npart[i]; k++) {
      const uint64_t e = member[k];
      PUT("%" PRIu64 "\t%d\n", ids[e], w ? (int)w[e] : (int)(-(-1.0)));
    }
  }
#undef PUT
  *out = (unsigned char *)buf;
  *nbytes = used;
  return 0;
}


/* ---------------------------------------------------------------------------
 * AHF_particles_bin, ahf_binwrite_particles (src/libahf/ahf_io.c:1733-1855,
 * AHFbinary build, no GAS_PARTICLES or AHFnewHaloIDs): int32 1, uint64 the
 * number of haloes written (written as 0, put back after the rewind
 * :1842-1844), uint32 2 (columns); per halo j of the output order with at
 * least minpart particles, uint64 npart and uint64 j, then per kept particle
 * uint64 id and int32 1.  Native byte order, fwrite of each field: no
 * padding, 16 + 12 npart bytes per halo.                                    */
static void put_bytes(unsigned char *buf, uint64_t *used, const void *v, size_t n)
{
  memcpy(buf + *used, v, n);
  *used += n;
}

int ahforacle_write_particles_bin(const uint64_t *ids, int64_t nhalo, const uint64_t *member_off,
                                  const uint64_t *member, const uint64_t *halo_npart, const int64_t *order,
                                  int64_t minpart, unsigned char **out, uint64_t *nbytes)
{
  uint64_t total = 16, good = 0;
  for (int64_t j = 0; j < nhalo; j++)
    if ((int64_t)halo_npart[order[j]] >= minpart) {
      good++;
      total += 16 + 12 * halo_npart[order[j]];
    }
  unsigned char *buf = (unsigned char *)malloc(total);
  if (!buf) return -1;
  uint64_t used = 0;
  const int32_t one = 1;
  const uint32_t ncol = 2;
  put_bytes(buf, &used, &one, 4);
  put_bytes(buf, &used, &good, 8);
  put_bytes(buf, &used, &ncol, 4);
  for (int64_t j = 0; j < nhalo; j++) {
    const int64_t i = order[j];
    if (!((int64_t)halo_npart[i] >= minpart)) continue;
    const uint64_t np = halo_npart[i], hj = (uint64_t)j;
    put_bytes(buf, &used, &np, 8);
    put_bytes(buf, &used, &hj, 8);
    for (uint64_t k = member_off[i]; k < member_off[i] + np; k++) {
      put_bytes(buf, &used, &ids[member[k]], 8);
      put_bytes(buf, &used, &one, 4);
    }
  }
  *out = buf;
  *nbytes = used;
  return 0;
}


/* ---------------------------------------------------------------------------
 * Hilbert keys and the particle sort (src/main.c:342-356).
 * sfc_curve_calcKey(SFC_CURVE_HILBERT, ...) (libsfc/sfc_curve.c:79-91) maps
 * a position in [0,1]^3 to grid coordinates c_d = trunc(x_d 2^bits), capped
 * at 2^bits - 1 (libsfc/hilbert_util.c:69-92), and those to the index of the
 * cell on the Hilbert curve of libsfc/hilbert.c (hilbert_c2i, :197-240).
 * That curve, restated per level from the most significant bit: with g_b the
 * 3-bit group (bit b of c_0, c_1, c_2 as bits 0, 1, 2) and G_b = g_b ^
 * g_{b+1} (g_bits = 0), each level emits r_b = rotr3(G_b ^ flip, rot); then
 * flip = 1 << rot, and rot advances by 1, plus 1 or 2 when the lowest set
 * bit of r_b is bit 0 or bit 1 (mod 3); rot and flip start at 0.  The
 * emitted index has bit 2 of every level but the top one inverted and is
 * then Gray-decoded (prefix XOR from the top).  The sort: ascending key; the
 * reference's qsort leaves equal keys in its C library's order, the
 * restatement by original index.                                          */
uint64_t ahforacle_sfc_key(double x, double y, double z, unsigned bits)
{
  const uint64_t max = (uint64_t)1 << bits;
  const double v[3] = {x, y, z};
  uint64_t c[3];
  for (int d = 0; d < 3; d++) {
    c[d] = (uint64_t)trunc(v[d] * (double)max);
    if (c[d] == max) c[d] = max - 1;
  }
  uint64_t key = 0;
  unsigned rot = 0, flip = 0, gup = 0;
  for (int b = (int)bits - 1; b >= 0; b--) {
    const unsigned g = (unsigned)(((c[0] >> b) & 1u) | (((c[1] >> b) & 1u) << 1) | (((c[2] >> b) & 1u) << 2));
    const unsigned t = (g ^ gup ^ flip) & 7u;
    const unsigned r = ((t >> rot) | (t << (3u - rot))) & 7u;
    key = (key << 3) | r;
    flip = 1u << rot;
    const unsigned low = r & (0u - r) & 3u;
    rot += 1u + (low == 1u ? 1u : 0u) + (low == 2u ? 2u : 0u);
    if (rot >= 3u) rot -= 3u;
    gup = g;
  }
  for (unsigned b = 0; b + 1 < bits; b++) key ^= (uint64_t)4 << (3 * b);
  for (unsigned s = 1; s < 3 * bits; s *= 2) key ^= key >> s;
  return key;
}

typedef struct {
  uint64_t key, idx;
} keyidx_t;

static int cmp_keyidx(const void *a, const void *b)
{
  const keyidx_t *p = (const keyidx_t *)a, *q = (const keyidx_t *)b;
  if (p->key != q->key) return p->key < q->key ? -1 : 1;
  return p->idx < q->idx ? -1 : (p->idx > q->idx);
}

int ahforacle_sfc_sort(uint64_t n, const float *x, const float *y, const float *z, unsigned bits, uint64_t *keys,
                       uint64_t *order)
{
  keyidx_t *a = (keyidx_t *)malloc((n ? n : 1) * sizeof(keyidx_t));
  if (!a) return -1;
  for (uint64_t i = 0; i < n; i++) {
    a[i].key = ahforacle_sfc_key((double)x[i], (double)y[i], (double)z[i], bits);
    a[i].idx = i;
  }
  qsort(a, (size_t)n, sizeof(keyidx_t), cmp_keyidx);
  for (uint64_t k = 0; k < n; k++) {
    keys[k] = a[k].key;
    order[k] = a[k].idx;
  }
  free(a);
  return 0;
}


/* ---------------------------------------------------------------------------
 * The domain grid's TSC number density (assign_npart,
 * src/libamr_serial/density.c:238-420, default TSC build, periodic, float
 * node densities), the first step of the AMR hierarchy: every node starts
 * at -mean_dens = -1 (zero_dens); the nodes are visited in z, y, x order
 * and, within a node, its particles in linked-list order (ll() prepends, so
 * descending input index); each particle adds masstodens w_z w_y w_x to the
 * 27 nodes around its own (periodic), with separations d measured from the
 * node centre (x + 1/2)/l1 in cells, wrapped through f1mod when |d| > l1/2,
 * and TSC weights 0.75 - d^2, (1/2 - d)^2 / 2, (1/2 + d)^2 / 2.  Each
 * addition is the reference's float += double.                            */
static double f1mod_ref(double x) { return x >= 2.0 ? x - 2.0 : (x >= 1.0 ? x - 1.0 : x); }

int ahforacle_domain_dens(uint64_t n, const float *x, const float *y, const float *z, int l1, double *dens_out)
{
  const size_t nn = (size_t)l1 * (size_t)l1 * (size_t)l1;
  float *dens = (float *)malloc(nn * sizeof(float));
  uint64_t *start = (uint64_t *)calloc(nn + 1, sizeof(uint64_t));
  uint64_t *cell = (uint64_t *)malloc((n ? n : 1) * sizeof(uint64_t));
  uint64_t *list = (uint64_t *)malloc((n ? n : 1) * sizeof(uint64_t));
  if (!dens || !start || !cell || !list) return -1;
  const float *pos[3] = {x, y, z};
  for (uint64_t i = 0; i < n; i++) {
    unsigned long c[3];
    for (int d = 0; d < 3; d++) {
      c[d] = (unsigned long)((double)l1 * (double)pos[d][i]);
      if (c[d] > (unsigned long)(l1 - 1)) c[d] = 0;
    }
    cell[i] = ((uint64_t)c[2] * (uint64_t)l1 + c[1]) * (uint64_t)l1 + c[0];
    start[cell[i] + 1]++;
  }
  for (size_t k = 0; k < nn; k++) start[k + 1] += start[k];
  {
    uint64_t *fill = (uint64_t *)malloc((nn ? nn : 1) * sizeof(uint64_t));
    if (!fill) return -1;
    memcpy(fill, start, nn * sizeof(uint64_t));
    for (uint64_t i = n; i-- > 0;) list[fill[cell[i]]++] = i;   /* descending index within a node */
    free(fill);
  }
  for (size_t k = 0; k < nn; k++) dens[k] = (float)(-1.0);
  const double dl1 = (double)l1;
  const double m2d = (dl1 * dl1 * dl1) / (double)n;
  const double shift = 0.5 / dl1;
  for (long zz = 0; zz < l1; zz++)
    for (long yy = 0; yy < l1; yy++)
      for (long xx = 0; xx < l1; xx++) {
        const size_t node = ((size_t)zz * l1 + yy) * l1 + xx;
        const long cc[3] = {xx, yy, zz};
        double centre[3];
        for (int d = 0; d < 3; d++) centre[d] = f1mod_ref(((double)cc[d] / dl1 + shift) + 1.0);
        for (uint64_t s = start[node]; s < start[node + 1]; s++) {
          const uint64_t i = list[s];
          double w[3][3];   /* w[d][0..2]: weights of the nodes below, at, above along axis d */
          for (int d = 0; d < 3; d++) {
            double sep = ((double)pos[d][i] - centre[d]) * dl1;
            if (fabs(sep) > 0.5 * dl1) {
              const double a = f1mod_ref(((double)pos[d][i] + 0.5) + 1.0);
              const double b = f1mod_ref((centre[d] + 0.5) + 1.0);
              sep = (a - b) * dl1;
            }
            w[d][1] = 0.75 - sep * sep;
            w[d][0] = ((0.5 - sep) * (0.5 - sep)) / 2;
            w[d][2] = ((0.5 + sep) * (0.5 + sep)) / 2;
          }
          for (int k = 0; k < 3; k++)
            for (int j = 0; j < 3; j++)
              for (int q = 0; q < 3; q++) {
                const size_t t = ((size_t)((zz + k - 1 + l1) % l1) * l1 + (size_t)((yy + j - 1 + l1) % l1)) * l1 +
                                 (size_t)((xx + q - 1 + l1) % l1);
                dens[t] += m2d * w[2][k] * w[1][j] * w[0][q];
              }
        }
      }
  for (size_t k = 0; k < nn; k++) dens_out[k] = (double)dens[k];
  free(dens);
  free(start);
  free(cell);
  free(list);
  return 0;
}


/* The first refinement of the domain grid (gen_refgrid -> refine_grid,
 * src/libamr_serial/generate_grids.c:126 and refine_grid.c:113-609, default
 * build, periodic), restated as a rule on the full l1^3 domain grid: a coarse
 * node is flagged (test_node, :113-137) when any node at dz, dy in {-1,0,1}
 * and dx in {0,1} has density >= critdens - mean_dens, critdens = NperDomCell
 * l1^3 / n; along x, ref_nquad's runs also cover the node after a flagged
 * one (x - 1 flagged), wrapping at x = 0 but not at x = l1 - 1; every
 * covered coarse node becomes 2x2x2 fine nodes (ref_cquad/ref_pquad mirror
 * each refined row and plane); the grid is kept only with at least
 * MIN_NNODES = 125 fine nodes (assign_npart, density.c:215).  Output: the
 * fine nodes' (z, y, x) in ascending order; returns their number (0 when no
 * grid is kept), -1 on allocation failure, -2 when more than max_nodes.    */
int64_t ahforacle_first_refinement(uint64_t n, const float *x, const float *y, const float *z, int l1,
                                   double nth_dom, int64_t *zyx, int64_t max_nodes)
{
  const size_t nn = (size_t)l1 * l1 * l1;
  double *dens = (double *)malloc(nn * sizeof(double));
  unsigned char *hit = (unsigned char *)calloc(nn, 1), *flag = (unsigned char *)calloc(nn, 1);
  if (!dens || !hit || !flag) return -1;
  if (ahforacle_domain_dens(n, x, y, z, l1, dens) != 0) return -1;
  const double dl1 = (double)l1;
  const double crit = nth_dom * ((dl1 * dl1 * dl1) / (double)n);
  for (size_t k = 0; k < nn; k++) hit[k] = dens[k] >= crit - 1.0;
#define NODE(zz, yy, xx) ((((size_t)(((zz) + l1) % l1)) * l1 + (size_t)(((yy) + l1) % l1)) * l1 + (size_t)(((xx) + l1) % l1))
  for (long zz = 0; zz < l1; zz++)
    for (long yy = 0; yy < l1; yy++)
      for (long xx = 0; xx < l1; xx++) {
        unsigned char f = 0;
        for (int dz = -1; dz <= 1 && !f; dz++)
          for (int dy = -1; dy <= 1 && !f; dy++)
            for (int dx = 0; dx <= 1 && !f; dx++) f = hit[NODE(zz + dz, yy + dy, xx + dx)];
        flag[NODE(zz, yy, xx)] = f;
      }
  int64_t count = 0;
  for (long zz = 0; zz < l1; zz++)
    for (int a = 0; a < 2; a++)
      for (long yy = 0; yy < l1; yy++)
        for (int b = 0; b < 2; b++)
          for (long xx = 0; xx < l1; xx++) {
            const int cov = flag[NODE(zz, yy, xx)] || (xx != l1 - 1 && flag[NODE(zz, yy, xx - 1)]);
            if (!cov) continue;
            for (int c = 0; c < 2; c++) {
              if (count >= max_nodes) return -2;
              zyx[3 * count + 0] = 2 * zz + a;
              zyx[3 * count + 1] = 2 * yy + b;
              zyx[3 * count + 2] = 2 * xx + c;
              count++;
            }
          }
#undef NODE
  free(dens);
  free(hit);
  free(flag);
  return count >= 125 ? count : 0;
}
