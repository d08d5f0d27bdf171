// finish.cuh -- per-bin and per-halo finishing of HaloProfiles shared by
// the FP64 and the FP32-compensated forms: 3x3 eigen-solver, concentration
// root finders, profile rows and integral properties.  All FP64, in the
// reference's operation order (the including unit is compiled without FMA
// contraction).
#pragma once

#include <cmath>

#include "common.cuh"

namespace ahfgpu {

struct Bin {
  double npart, M, Lx, Ly, Lz, T, U, a11, a22, a33, a12, a13, a23, vesc2;
};

// ---------------------------------------------------------------------------
// numerics of the per-bin / per-halo finish (one thread)

// symmetric 3x3 eigen-decomposition by cyclic Jacobi rotations (Golub & Van
// Loan, sym.schur2 + cyclic sweep); column k of v is the eigenvector of d[k]
static __device__ void jacobi3(const double ain[3][3], double d[3], double v[3][3]) {
  double a[3][3];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) { a[i][j] = ain[i][j]; v[i][j] = (i == j) ? 1.0 : 0.0; }
  for (int sweep = 0; sweep < 64; sweep++) {
    double off = fabs(a[0][1]) + fabs(a[0][2]) + fabs(a[1][2]);
    if (off == 0.0) break;
    for (int pp = 0; pp < 2; pp++) {
      for (int qq = pp + 1; qq < 3; qq++) {
        double apq = a[pp][qq];
        if (apq == 0.0) continue;
        double app = a[pp][pp], aqq = a[qq][qq];
        if (sweep > 3 && fabs(app) + 100.0 * fabs(apq) == fabs(app) &&
            fabs(aqq) + 100.0 * fabs(apq) == fabs(aqq)) {
          a[pp][qq] = a[qq][pp] = 0.0;
          continue;
        }
        double tau = (aqq - app) / (2.0 * apq);
        double t = (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
        double cs = 1.0 / sqrt(1.0 + t * t);
        double sn = t * cs;
        for (int k = 0; k < 3; k++) {
          double akp = a[k][pp], akq = a[k][qq];
          a[k][pp] = cs * akp - sn * akq;
          a[k][qq] = sn * akp + cs * akq;
        }
        for (int k = 0; k < 3; k++) {
          double apk = a[pp][k], aqk = a[qq][k];
          a[pp][k] = cs * apk - sn * aqk;
          a[qq][k] = sn * apk + cs * aqk;
        }
        a[pp][qq] = a[qq][pp] = 0.0;
        for (int k = 0; k < 3; k++) {
          double vkp = v[k][pp], vkq = v[k][qq];
          v[k][pp] = cs * vkp - sn * vkq;
          v[k][qq] = sn * vkp + cs * vkq;
        }
      }
    }
  }
  for (int k = 0; k < 3; k++) d[k] = a[k][k];
}

// the same cyclic Jacobi in FP32 (the FP32-compensated form, whose inertia
// sums are themselves FP32-accurate): about one sixteenth of the FP64 cost
static __device__ void jacobi3f(const double ain[3][3], double dout[3], double vout[3][3]) {
  float a[3][3], v[3][3];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) { a[i][j] = (float)ain[i][j]; v[i][j] = (i == j) ? 1.f : 0.f; }
  for (int sweep = 0; sweep < 32; sweep++) {
    float off = fabsf(a[0][1]) + fabsf(a[0][2]) + fabsf(a[1][2]);
    if (off == 0.f) break;
    for (int pp = 0; pp < 2; pp++) {
      for (int qq = pp + 1; qq < 3; qq++) {
        float apq = a[pp][qq];
        if (apq == 0.f) continue;
        float app = a[pp][pp], aqq = a[qq][qq];
        if (sweep > 3 && fabsf(app) + 100.f * fabsf(apq) == fabsf(app) &&
            fabsf(aqq) + 100.f * fabsf(apq) == fabsf(aqq)) {
          a[pp][qq] = a[qq][pp] = 0.f;
          continue;
        }
        float tau = (aqq - app) / (2.f * apq);
        float t = (tau >= 0.f ? 1.f : -1.f) / (fabsf(tau) + sqrtf(1.f + tau * tau));
        float cs = 1.f / sqrtf(1.f + t * t);
        float sn = t * cs;
        for (int k = 0; k < 3; k++) {
          float akp = a[k][pp], akq = a[k][qq];
          a[k][pp] = cs * akp - sn * akq;
          a[k][qq] = sn * akp + cs * akq;
        }
        for (int k = 0; k < 3; k++) {
          float apk = a[pp][k], aqk = a[qq][k];
          a[pp][k] = cs * apk - sn * aqk;
          a[qq][k] = sn * apk + cs * aqk;
        }
        a[pp][qq] = a[qq][pp] = 0.f;
        for (int k = 0; k < 3; k++) {
          float vkp = v[k][pp], vkq = v[k][qq];
          v[k][pp] = cs * vkp - sn * vkq;
          v[k][qq] = sn * vkp + cs * vkq;
        }
      }
    }
  }
  for (int k = 0; k < 3; k++) {
    dout[k] = (double)a[k][k];
    for (int j = 0; j < 3; j++) vout[k][j] = (double)v[k][j];
  }
}

// get_axes, src/libutility/specific.c:135-178 (own eigen-solver)
static __device__ void get_axes(double it[3][3], double* a1, double* a2, double* a3, bool f32 = false) {
  double d[3], v[3][3];
  if (f32) jacobi3f(it, d, v); else jacobi3(it, d, v);
  int ord[3] = {0, 1, 2};
  for (int i = 1; i < 3; i++) {
    int k = ord[i], j = i;
    while (j > 0 && d[ord[j - 1]] < d[k]) { ord[j] = ord[j - 1]; j--; }
    ord[j] = k;
  }
  *a1 = d[ord[0]]; *a2 = d[ord[1]]; *a3 = d[ord[2]];
  for (int cc = 0; cc < 3; cc++)
    for (int r = 0; r < 3; r++) it[r][cc] = v[r][ord[cc]];
}

static __device__ double cnfw_root(double cc, double v2r) { return 0.216 * cc / (log(1 + cc) - cc / (1 + cc)) - v2r; }
// calc_cNFW, src/libutility/specific.c:2041-2072
static __device__ double calc_cNFW(double V2_max, double V2_vir) {
  double r = V2_max / V2_vir;
  if (r <= 1 || r > 5.9) return -1;
  double a = 2.2, b = 100, cc;
  while (b - a > 1e-3) {
    cc = (a + b) / 2;
    if (cnfw_root(a, r) * cnfw_root(cc, r) > 0) a = cc; else b = cc;
  }
  return (a + b) / 2.0;
}
static __device__ double cr1_root(double cc, double R1) {
  return (cc - 2.0 * log(1.0 + cc) + cc / (1.0 + cc)) / (cc * (log(1.0 + cc) - cc / (1.0 + cc))) - R1;
}
// calc_cR1, src/libutility/specific.c:1993-2018
static __device__ double calc_cR1(double R1) {
  if (R1 <= 0.19 || 0.585 <= R1) return -1.0;
  double a = 1.0, b = 500.0, cc;
  while (b - a > 1e-3) {
    cc = (a + b) / 2;
    if (cr1_root(a, R1) * cr1_root(cc, R1) > 0) a = cc; else b = cc;
  }
  return (a + b) / 2.0;
}


// One profile row of HaloProfiles' per-bin block (ahf_halos.c:4632-4868)
// from bin b's cumulative record R, its outer edge, and the previous bin's
// mass and edge (has_prev false for the first bin).
// f32eig: FP32 eigen-solver (FP32-compensated form)
static __device__ __forceinline__ void bin_row(const Bin& R, double cur_rad, bool has_prev, double Mprev_in,
                                               double edge_prev, double* row, bool f32eig) {
  const double FPT = 4. * kPi / 3.;
  double Volume = FPT * (cur_rad * cur_rad * cur_rad);
  double Mprev = has_prev ? Mprev_in : 0.0;
  double Vprev = has_prev ? FPT * (edge_prev * edge_prev * edge_prev) : 0.0;
  double dM = R.M - Mprev;
  double dV = Volume - Vprev;
  double it[3][3], ax1, ax2, ax3;
  if (R.npart > 10) {
    it[0][0] = R.a11; it[1][1] = R.a22; it[2][2] = R.a33;
    it[0][1] = R.a12; it[1][0] = R.a12;
    it[0][2] = R.a13; it[2][0] = R.a13;
    it[1][2] = R.a23; it[2][1] = R.a23;
    get_axes(it, &ax1, &ax2, &ax3, f32eig);
  } else {
    for (int x = 0; x < 3; x++)
      for (int y = 0; y < 3; y++) it[x][y] = 0.0;
    ax1 = 1; ax2 = 0; ax3 = 0;
  }
  row[AHFGPU_PROF_R] = cur_rad;
  row[AHFGPU_PROF_NPART] = R.npart;
  row[AHFGPU_PROF_NVPART] = R.M;
  row[AHFGPU_PROF_OVDENS] = R.M / Volume;
  row[AHFGPU_PROF_DENS] = dV > 0 ? dM / dV : 0.0;
  row[AHFGPU_PROF_V2_CIRC] = R.M / cur_rad;
  row[AHFGPU_PROF_V_ESC2] = R.vesc2;
  row[AHFGPU_PROF_SIG_V] = sqrt(R.T / R.M);
  row[AHFGPU_PROF_EKIN] = 0.5 * R.T;
  row[AHFGPU_PROF_EPOT] = 0.5 * R.U;
  row[AHFGPU_PROF_LX] = R.Lx;
  row[AHFGPU_PROF_LY] = R.Ly;
  row[AHFGPU_PROF_LZ] = R.Lz;
  row[AHFGPU_PROF_E1X] = it[0][0]; row[AHFGPU_PROF_E1Y] = it[1][0]; row[AHFGPU_PROF_E1Z] = it[2][0];
  row[AHFGPU_PROF_E2X] = it[0][1]; row[AHFGPU_PROF_E2Y] = it[1][1]; row[AHFGPU_PROF_E2Z] = it[2][1];
  row[AHFGPU_PROF_E3X] = it[0][2]; row[AHFGPU_PROF_E3Y] = it[1][2]; row[AHFGPU_PROF_E3Z] = it[2][2];
  row[AHFGPU_PROF_AXIS1] = 1.0;
  if (ax1 > 0.) {
    row[AHFGPU_PROF_AXIS2] = sqrt(ax2 / ax1);
    row[AHFGPU_PROF_AXIS3] = sqrt(ax3 / ax1);
  } else {
    row[AHFGPU_PROF_AXIS2] = 0.0;
    row[AHFGPU_PROF_AXIS3] = 0.0;
  }
}

// FP32C hands the bin records and the integral properties' inputs to a
// post-pass over all haloes (fp32c_finish_kernel): each bin's record and
// outer edge wait in the bin's own profile row (the row is then computed in
// place), the per-halo inputs in W.fin.
enum : int { kFinM = 0, kFinVX, kFinVY, kFinVZ, kFinCX, kFinCY, kFinCZ, kFinMhi, kFinMlo, kFinMbe, kFinR2, kFinRmax,
             kFinVmax };

__device__ __forceinline__ void stash_bin(double* row, const Bin& R, double edge) {
  row[0] = R.npart; row[1] = R.M; row[2] = R.Lx; row[3] = R.Ly; row[4] = R.Lz; row[5] = R.T; row[6] = R.U;
  row[7] = R.a11; row[8] = R.a22; row[9] = R.a33; row[10] = R.a12; row[11] = R.a13; row[12] = R.a23;
  row[13] = R.vesc2; row[14] = edge;
}

__device__ __forceinline__ void load_bin(const double* row, Bin& R, double& edge) {
  R.npart = row[0]; R.M = row[1]; R.Lx = row[2]; R.Ly = row[3]; R.Lz = row[4]; R.T = row[5]; R.U = row[6];
  R.a11 = row[7]; R.a22 = row[8]; R.a33 = row[9]; R.a12 = row[10]; R.a13 = row[11]; R.a23 = row[12];
  R.vesc2 = row[13]; edge = row[14];
}

// Profile rows of HaloProfiles' per-bin block from the cumulative bin
// records; one thread per bin.
static __device__ void write_bin_rows(const Bin* bins, const double* edge, int nbins, double* rows,
                                      bool f32eig = false) {
  for (int b = threadIdx.x; b < nbins; b += blockDim.x)
    bin_row(bins[b], edge[b], b > 0, b > 0 ? bins[b - 1].M : 0.0, b > 0 ? edge[b - 1] : 0.0,
            rows + (uint64_t)b * AHFGPU_PROF_NFIELDS, f32eig);
}

// Integral properties at the end of HaloProfiles (ahf_halos.c:4870-5018),
// one thread.  cNFW and cR1 (bisections) are filled afterwards for all
// haloes at once by concentration_kernel.  cM.. are the totals over the final members, mbe the entry of
// the most bound particle (-1: none).
static __device__ void finish_scalars(const double* rows, int nbins, double cM, double cVX, double cVY, double cVZ,
                               double cCx, double cCy, double cCz, double Mhi, double Mlo, long long mbe,
                               double r2, double R_max, double V_max, const DevParams& P, const DevBatch& B,
                               double hcx, double hcy, double hcz, ahfgpu_halo& hout) {
    const double* last = rows + (uint64_t)(nbins - 1) * AHFGPU_PROF_NFIELDS;
    const double* pl = rows + (uint64_t)(nbins - 2) * AHFGPU_PROF_NFIELDS;
    double Lx = last[AHFGPU_PROF_LX], Ly = last[AHFGPU_PROF_LY], Lz = last[AHFGPU_PROF_LZ];
    double absL = sqrt((Lx * Lx + Ly * Ly) + Lz * Lz);
    double Msph = cM;
    hout.M_vir = Msph;
    hout.vel[0] = cVX / Msph; hout.vel[1] = cVY / Msph; hout.vel[2] = cVZ / Msph;
    hout.R_max = R_max;
    hout.V2_max = V_max;
    hout.r2 = r2;
    hout.sigV = last[AHFGPU_PROF_SIG_V];
    hout.v_esc2 = last[AHFGPU_PROF_V_ESC2];
    hout.Ekin = last[AHFGPU_PROF_EKIN];
    hout.Epot = last[AHFGPU_PROF_EPOT];
    hout.axis[0] = last[AHFGPU_PROF_AXIS1]; hout.axis[1] = last[AHFGPU_PROF_AXIS2]; hout.axis[2] = last[AHFGPU_PROF_AXIS3];
    hout.E1[0] = last[AHFGPU_PROF_E1X]; hout.E1[1] = last[AHFGPU_PROF_E1Y]; hout.E1[2] = last[AHFGPU_PROF_E1Z];
    hout.E2[0] = last[AHFGPU_PROF_E2X]; hout.E2[1] = last[AHFGPU_PROF_E2Y]; hout.E2[2] = last[AHFGPU_PROF_E2Z];
    hout.E3[0] = last[AHFGPU_PROF_E3X]; hout.E3[1] = last[AHFGPU_PROF_E3Y]; hout.E3[2] = last[AHFGPU_PROF_E3Z];
    if (absL > 0) {
      hout.AngMom[0] = Lx / absL; hout.AngMom[1] = Ly / absL; hout.AngMom[2] = Lz / absL;
      hout.lambda = absL / hout.M_vir / sqrt(2. * hout.M_vir * hout.R_vir);
      hout.lambda *= P.v_fac * sqrt(P.r_fac / (kGrav * P.m_fac));
      // calc_lambdaE, ahf_halos.c:3937-3953
      double t1 = sqrt(P.m_fac * hout.M_vir);
      t1 = t1 * t1 * t1;
      double t2 = hout.Ekin * P.m_fac * (P.v_fac * P.v_fac);
      double t3 = hout.Epot * P.m_fac * P.phi_fac;
      t2 = fabs(t2 + t3);
      t2 = sqrt(t2);
      t1 = t2 / t1;
      t2 = P.m_fac * P.r_fac * P.v_fac * absL;
      t2 = t2 / (P.m_fac * hout.M_vir);
      t3 = t1 * t2;
      hout.lambdaE = t3 / kGrav;
    } else {
      hout.AngMom[0] = hout.AngMom[1] = hout.AngMom[2] = 0.0;
      hout.lambda = 0.0;
      hout.lambdaE = 0.0;
    }
    {
      // calc_R1, src/libutility/specific.c:1977-1991
      double r0h = rows[AHFGPU_PROF_R] / 2.0;
      double R1 = (r0h * r0h * r0h) * rows[AHFGPU_PROF_DENS] * (rows[AHFGPU_PROF_R]);
      for (int b = 1; b < nbins; b++) {
        const double* rb = rows + (uint64_t)b * AHFGPU_PROF_NFIELDS;
        const double* ra = rb - AHFGPU_PROF_NFIELDS;
        double rmid = (rb[AHFGPU_PROF_R] + ra[AHFGPU_PROF_R]) / 2.0;
        double drr = rb[AHFGPU_PROF_R] - ra[AHFGPU_PROF_R];
        R1 += (rmid * rmid * rmid) * rb[AHFGPU_PROF_DENS] * drr;
      }
      hout.R1 = 4 * kPi * R1 / hout.M_vir / hout.R_vir;
    }
    {
      double Ts = 2.0 * (last[AHFGPU_PROF_EKIN] - pl[AHFGPU_PROF_EKIN]);
      double frad = fabs(pl[AHFGPU_PROF_R] / last[AHFGPU_PROF_R]);
      hout.SurfP = -0.125 * ((1. + frad) * (1. + frad) * (1. + frad)) / (1. - (frad * frad * frad)) * Ts;
    }
    hout.fMhires = Mhi > 0 ? Mhi / (Mhi + Mlo) : 0.0;
    if (mbe >= 0) {
      uint64_t e = (uint64_t)mbe;
      double dX = fabs(B.x[e] - hcx), dY = fabs(B.y[e] - hcy), dZ = fabs(B.z[e] - hcz);
      if (dX > 0.5) dX -= 1.0;
      if (dY > 0.5) dY -= 1.0;
      if (dZ > 0.5) dZ -= 1.0;
      hout.mbp_offset = sqrt((dX * dX + dY * dY) + dZ * dZ);
      hout.pos_mbp[0] = B.x[e]; hout.pos_mbp[1] = B.y[e]; hout.pos_mbp[2] = B.z[e];
      hout.vel_mbp[0] = B.vx[e]; hout.vel_mbp[1] = B.vy[e]; hout.vel_mbp[2] = B.vz[e];
    } else {
      hout.mbp_offset = -1.0;
      hout.flags |= AHFGPU_HALO_NO_MBP;
    }
    double CoM[3] = {fmod(cCx / Msph + 1., 1.), fmod(cCy / Msph + 1., 1.), fmod(cCz / Msph + 1., 1.)};
    {
      double dX = fabs(CoM[0] - hcx), dY = fabs(CoM[1] - hcy), dZ = fabs(CoM[2] - hcz);
      if (dX > 0.5) dX -= 1.0;
      if (dY > 0.5) dY -= 1.0;
      if (dZ > 0.5) dZ -= 1.0;
      hout.com_offset = sqrt((dX * dX + dY * dY) + dZ * dZ);
    }
    hout.pos_com[0] = CoM[0]; hout.pos_com[1] = CoM[1]; hout.pos_com[2] = CoM[2];
}

}  // namespace ahfgpu
