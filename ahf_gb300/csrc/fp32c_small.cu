// fp32c_small.cu -- the small lists of the batched FP32C form, one list per
// thread, in FP64 in the reference's sequential order.
//
// A list of a few hundred entries is too short for a CTA: the CTA path runs
// the whole block-parallel code (about a megabyte of instructions, barriers
// around every serial section) for ~100 particles, and instruction fetch and
// barriers, not arithmetic, set its time.  Here each lane of a warp takes one
// halo (32 consecutive haloes of the size-sorted queue per warp, so the lanes'
// lists have similar lengths) and runs the five functions of
// ahf_halos_sfc_constructHalo (src/libahf/ahf_halos_sfc.c:140-156) as plain
// loops, exactly as the reference orders its operations:
//
//   sort_halo_particles  ahf_halos.c:5786-5894 (dR^2 with the signed wrap; a
//                        stable merge sort: ties in list order)
//   rem_outsideRvir(.,0) :3687-3889 (walk out while ovdens >= ovlim; the first
//                        failing particle kept)
//   rem_unbound          :3292-3607 (Phi0 pass, the bulk-velocity seed, the
//                        bound pass with the running bound-only bulk
//                        velocity, until at most 3 are removed)
//   rem_outsideRvir(.,1)
//   HaloProfiles         :3961-5261 (binning_parameter, specific.c:259-322;
//                        the per-particle pass; find_max/smooth3,
//                        general.c:548-650)
//
// so the kept lists and every sum are the reference's, bit for bit.  The
// per-bin records and the integral properties' inputs go to the FP32C
// post-pass (fp32c_finish_kernel) like the CTA path's, which forms the
// profile rows and the properties.
//
// Work space: per warp a region of per-slot arrays, element i of lane l at
// [i * 32 + l] (a lane's loop over its list reads one element per lane per
// step: coalesced across the warp), for lists of at most `nmax` entries.
#include <cstdint>

#include "common.cuh"
#include "finish.cuh"

namespace ahfgpu {

constexpr int kSmallT = 128;               // threads per block (4 warps)
// per-slot arrays of the work space: doubles, floats, 32-bit indices
enum : int { kSD_KEY = 0, kSD_DX, kSD_DY, kSD_DZ, kSD_D, kSD_OVD, kSD_VC2, kSD_DR2, kSD_Y, kSD_T, kSmallDoubles };
enum : int { kSF_VX = 0, kSF_VY, kSF_VZ, kSF_W, kSmallFloats };
enum : int { kSU_ORD = 0, kSU_TMP, kSmallU32 };
constexpr size_t kSmallSlotBytes = kSmallDoubles * 8 + kSmallFloats * 4 + kSmallU32 * 4;

size_t fp32c_small_bytes_per_warp(uint64_t nmax) { return (size_t)32 * nmax * kSmallSlotBytes; }

struct SmallLane {
  double* d[kSmallDoubles];
  float* f[kSmallFloats];
  uint32_t* u[kSmallU32];
  int lane;
  __device__ __forceinline__ double& D(int a, uint32_t i) const { return d[a][(size_t)i * 32 + lane]; }
  __device__ __forceinline__ float& F(int a, uint32_t i) const { return f[a][(size_t)i * 32 + lane]; }
  __device__ __forceinline__ uint32_t& U(int a, uint32_t i) const { return u[a][(size_t)i * 32 + lane]; }
};

// smooth3 (general.c:548-573) in place on y[0..m) (work array a), tmp b
__device__ static void small_smooth3(const SmallLane& L, int a, int b, int64_t m, int ns) {
  if (ns == 0 || m < 3) return;
  for (int j = 0; j < ns; j++) {
    L.D(b, 0) = (L.D(a, 0) + L.D(a, 1)) / 2.;
    for (int64_t i = 1; i < m - 1; i++) L.D(b, (uint32_t)i) = (L.D(a, (uint32_t)(i - 1)) + L.D(a, (uint32_t)i) + L.D(a, (uint32_t)(i + 1))) / 3.;
    L.D(b, (uint32_t)(m - 1)) = (L.D(a, (uint32_t)(m - 1)) + L.D(a, (uint32_t)(m - 2))) / 2.;
    for (int64_t i = 0; i < m; i++) L.D(a, (uint32_t)i) = L.D(b, (uint32_t)i);
  }
}

// find_max (general.c:608-650) of y = raw[kNignore..kNignore+m) smoothed ns
// times; x = radius at the same ranks; returns x_max
__device__ static double small_find_max(const SmallLane& L, int raw, int64_t m, int ns) {
  for (int64_t i = 0; i < m; i++) L.D(kSD_Y, (uint32_t)i) = L.D(raw, (uint32_t)(i + kNignore));
  small_smooth3(L, kSD_Y, kSD_T, m, ns);
  double ymax = -10.0;
  int64_t i0 = m - 1;
  for (int64_t i = 0; i < m - 1; i++)
    if (L.D(kSD_Y, (uint32_t)i) > ymax) { ymax = L.D(kSD_Y, (uint32_t)i); i0 = i; }
  int64_t i1 = i0;
  for (int64_t i = (m - 1 + i0) / 2; i > i0; i--)
    if (L.D(kSD_Y, (uint32_t)i) > ymax) { ymax = L.D(kSD_Y, (uint32_t)i); i1 = i; }
  // radius of rank r is kept in kSD_KEY from HaloProfiles on
  return (L.D(kSD_KEY, (uint32_t)(i0 + kNignore)) + L.D(kSD_KEY, (uint32_t)(i1 + kNignore))) / 2;
}

__device__ static void small_halo(int h, const DevParams& P, const DevBatch& B, const Work& W, const SmallLane& L) {
  const uint64_t o = B.off[h];
  const uint32_t n = (uint32_t)(B.off[h + 1] - o);
  const double cx = B.cx[h], cy = B.cy[h], cz = B.cz[h];
  ahfgpu_halo& H = W.halo[h];   // zeroed by the host before the launch
  if (n == 0) { H.flags = AHFGPU_HALO_EMPTY; return; }
  if ((int64_t)n < P.MINPART) {
    // nothing runs: the gathered list passes through
    for (uint32_t i = 0; i < n; i++) W.mem_stage[o + i] = o + i;
    H.npart = n;
    return;
  }
  // ---- sort_halo_particles
  for (uint32_t i = 0; i < n; i++) {
    const uint64_t e = o + i;
    const double dX = wrap_s((double)B.x[e] - cx), dY = wrap_s((double)B.y[e] - cy), dZ = wrap_s((double)B.z[e] - cz);
    L.D(kSD_KEY, i) = (dX * dX + dY * dY) + dZ * dZ;
    L.U(kSU_ORD, i) = i;
  }
  int src = kSU_ORD, dst = kSU_TMP;
  for (uint32_t width = 1; width < n; width *= 2) {
    for (uint32_t lo = 0; lo < n; lo += 2 * width) {
      const uint32_t mid = min(lo + width, n), hi = min(lo + 2 * width, n);
      uint32_t i = lo, j = mid, k = lo;
      while (i < mid && j < hi) {
        const uint32_t a = L.U(src, i), b = L.U(src, j);
        if (L.D(kSD_KEY, b) < L.D(kSD_KEY, a)) { L.U(dst, k++) = b; j++; }
        else { L.U(dst, k++) = a; i++; }
      }
      while (i < mid) L.U(dst, k++) = L.U(src, i++);
      while (j < hi) L.U(dst, k++) = L.U(src, j++);
    }
    int t = src; src = dst; dst = t;
  }
  if (src != kSU_ORD)
    for (uint32_t i = 0; i < n; i++) L.U(kSU_ORD, i) = L.U(kSU_TMP, i);
  unsigned long long ties = 0;
  for (uint32_t i = 1; i < n; i++)
    if (L.D(kSD_KEY, L.U(kSU_ORD, i)) == L.D(kSD_KEY, L.U(kSU_ORD, i - 1))) ties++;
  if (ties) atomicAdd(&W.counters[2], ties);
  // the list in radial order: offsets, distance, momenta, weight
  for (uint32_t i = 0; i < n; i++) {
    const uint64_t e = o + L.U(kSU_ORD, i);
    const double dX = wrap_s((double)B.x[e] - cx), dY = wrap_s((double)B.y[e] - cy), dZ = wrap_s((double)B.z[e] - cz);
    L.D(kSD_DX, i) = dX; L.D(kSD_DY, i) = dY; L.D(kSD_DZ, i) = dZ;
    L.D(kSD_D, i) = sqrt((dX * dX + dY * dY) + dZ * dZ);
    L.F(kSF_VX, i) = B.vx[e]; L.F(kSF_VY, i) = B.vy[e]; L.F(kSF_VZ, i) = B.vz[e];
    L.F(kSF_W, i) = B.w ? B.w[e] : 1.f;
  }
  // from here: kSU_ORD[rank] = local entry index; kSU_TMP = member list (ranks)
  const double FPT = 4. * kPi / 3.;
  uint32_t flags = AHFGPU_HALO_RAN_SORT | AHFGPU_HALO_RAN_RVIR0;
  // ---- rem_outsideRvir(.,0)
  uint32_t npart;
  {
    uint32_t j = 0;
    double M = 0.0, R = -1.0, ov = 2 * P.ovlim;
    while (j < n && ov >= P.ovlim) {
      M += (double)L.F(kSF_W, j);
      R = L.D(kSD_D, j);
      const double V = 4. * kPi / 3. * (R * R * R);
      ov = M / V * P.rho_fac / P.rho_vir;
      j++;
    }
    npart = j;
    H.M_vir = M; H.R_vir = R; H.ovdens = ov; H.Phi0 = 0.0;
  }
  for (uint32_t k = 0; k < npart; k++) L.U(kSU_TMP, k) = k;
  // ---- rem_unbound
  if ((int64_t)npart >= P.MINPART) {
    flags |= AHFGPU_HALO_RAN_UNBIND;
    const uint64_t no_vbulk = (uint64_t)(P.MINPART / 2);
    uint32_t nremove = 4;
    int niter = 0;
    double R_vir = 0.0;
    while (nremove > 3) {
      niter++;
      double I_now = 0.0, I_prev = 0.0, d_prev = 0.0, M_r = 0.0, Phi0 = 0.0, dist = 0.0;
      for (uint32_t j = 0; j < npart; j++) {
        const uint32_t s = L.U(kSU_TMP, j);
        M_r += (double)L.F(kSF_W, s);
        dist = L.D(kSD_D, s);
        if (dist > kMachineZero) {
          I_now = M_r / (dist * dist);
          const double I_mid = (I_now + I_prev) / 2.;
          const double dr = dist - d_prev;
          Phi0 += I_mid * dr;
        }
        d_prev = dist;
        I_prev = I_now;
      }
      Phi0 += M_r / dist;
      H.Phi0 = Phi0;
      // bulk-velocity seed: rank no_vbulk/2 (1-based) of the float |mom|^2
      // of the innermost no_vbulk members (ties by position), else the
      // innermost member
      uint32_t js = 0;
      if (niter == 1) {
        float m2[64];
        uint32_t pos[64];
        const uint32_t nv = (uint32_t)(no_vbulk < 64 ? no_vbulk : 64);
        for (uint32_t j = 0; j < nv; j++) {
          const uint32_t s = L.U(kSU_TMP, j);
          const float mx = L.F(kSF_VX, s), my = L.F(kSF_VY, s), mz = L.F(kSF_VZ, s);
          m2[j] = __fadd_rn(__fadd_rn(__fmul_rn(mx, mx), __fmul_rn(my, my)), __fmul_rn(mz, mz));
          pos[j] = j;
        }
        for (uint32_t i = 1; i < nv; i++) {
          const float kv = m2[i];
          const uint32_t kp = pos[i];
          uint32_t k = i;
          while (k > 0 && m2[k - 1] > kv) { m2[k] = m2[k - 1]; pos[k] = pos[k - 1]; k--; }
          m2[k] = kv;
          pos[k] = kp;
        }
        js = pos[no_vbulk / 2 - 1];
      }
      const uint32_t ss = L.U(kSU_TMP, js);
      const double w0 = (double)L.F(kSF_W, ss);
      double M_vel = w0;
      double VXc = w0 * (double)L.F(kSF_VX, ss), VYc = w0 * (double)L.F(kSF_VY, ss), VZc = w0 * (double)L.F(kSF_VZ, ss);
      nremove = 0;
      I_now = 0.0; I_prev = 0.0; d_prev = 0.0; M_r = 0.0;
      double M_vir = 0.0, Phi = 0.0;
      uint32_t nb = 0;
      for (uint32_t j = 0; j < npart; j++) {
        const uint32_t s = L.U(kSU_TMP, j);
        const double weight = (double)L.F(kSF_W, s);
        M_r += weight;
        const double dX = L.D(kSD_DX, s), dY = L.D(kSD_DY, s), dZ = L.D(kSD_DZ, s);
        dist = L.D(kSD_D, s);
        double v_esc2;
        if (dist > kMachineZero) {
          I_now = M_r / (dist * dist);
          const double I_mid = (I_now + I_prev) / 2.;
          const double dr = dist - d_prev;
          Phi += I_mid * dr;
          v_esc2 = (2 * fabs(Phi - Phi0) * P.phi_fac);
        } else {
          v_esc2 = 1e30;
        }
        const double VXp = (double)L.F(kSF_VX, s), VYp = (double)L.F(kSF_VY, s), VZp = (double)L.F(kSF_VZ, s);
        const double dVX = (VXp - VXc / M_vel) * P.v_fac + P.Hubble * (dX) * P.r_fac;
        const double dVY = (VYp - VYc / M_vel) * P.v_fac + P.Hubble * (dY) * P.r_fac;
        const double dVZ = (VZp - VZc / M_vel) * P.v_fac + P.Hubble * (dZ) * P.r_fac;
        const double vel2 = (dVX * dVX + dVY * dVY) + dVZ * dVZ;
        if (vel2 > P.v2_tune * v_esc2) {
          nremove++;
        } else {
          M_vel += weight;
          VXc += weight * VXp;
          VYc += weight * VYp;
          VZc += weight * VZp;
          L.U(kSU_TMP, nb++) = s;   // nb <= j: the member list compacts in place
          M_vir += weight;
          R_vir = dist;
        }
        I_prev = I_now;
        d_prev = dist;
      }
      if (nb == 0) flags |= AHFGPU_HALO_NOBOUND;
      npart = nb;
      H.M_vir = M_vir;
      H.R_vir = R_vir;
      if (((double)npart) < ((double)P.MINPART)) break;
    }
    H.niter = niter;
  }
  // ---- rem_outsideRvir(.,1)
  if ((int64_t)npart >= P.MINPART) {
    flags |= AHFGPU_HALO_RAN_RVIR1;
    uint32_t j = 0;
    double M = 0.0, R = -1.0, ov = 2 * P.ovlim;
    while (j < npart && ov >= P.ovlim) {
      const uint32_t s = L.U(kSU_TMP, j);
      M += (double)L.F(kSF_W, s);
      R = L.D(kSD_D, s);
      const double V = 4. * kPi / 3. * (R * R * R);
      ov = M / V * P.rho_fac / P.rho_vir;
      j++;
    }
    npart = j;
    H.M_vir = M; H.R_vir = R; H.ovdens = ov;
  }
  // ---- HaloProfiles
  if ((int64_t)npart >= P.MINPART) {
    const uint32_t n2 = npart;
    // binning_parameter (the reference's fabs / 1 - d wrap: the same distances)
    int nbins = (int)(6.2 * (log10((double)n2)) - 3.5);
    if (nbins < 2) nbins = 2;
    if (nbins > kMaxBins) nbins = kMaxBins;
    long npb = (long)floor(((double)P.MINPART / 10.) + 0.5);
    double dist_min = -1.0;
    while (npb < (long)n2 - 1 && dist_min < kMachineZero) { dist_min = L.D(kSD_D, L.U(kSU_TMP, (uint32_t)npb)); npb++; }
    const double dist_max = L.D(kSD_D, L.U(kSU_TMP, n2 - 1));
    if (dist_min < kMachineZero) dist_min = dist_max / 2.;
    const double ldist_min = log10(dist_min), ldist_max = log10(dist_max);
    const double ldr = (ldist_max - ldist_min) / (double)nbins;
    double* rows = W.prof_stage + W.prof_cap_off[h] * AHFGPU_PROF_NFIELDS;
    double Phi0 = H.Phi0, Phi = 0.0, pre_dist = 0.0, I_prev = 0.0, I_now = 0.0;
    double npp = 0;
    double M_sphere_prev = 0.0, prev_dist = 0.0, M_sphere = 0.0, VXc = 0.0, VYc = 0.0, VZc = 0.0;
    double a11 = 0, a22 = 0, a33 = 0, a12 = 0, a13 = 0, a23 = 0;
    double sig_v = 0, Lx = 0, Ly = 0, Lz = 0, CoM0 = 0, CoM1 = 0, CoM2 = 0;
    double Epot = 0, Emin = 1e30, v_esc2 = 0.0;
    long long mb = -1;
    double M_hires = 0.0, M_lores = 0.0;
    uint32_t jpart = 0;
    double cur_dist = -1.0;
    const double Hrv = P.Hubble;   // Hubble * d * r_fac / v_fac, in the reference's order below
    for (int ibin = 0; ibin < nbins; ibin++) {
      const double lcur_rad = ldist_min + ((double)ibin + 1) * ldr;
      double cur_rad = pow(10., lcur_rad);
      if (ibin == nbins - 1) cur_rad = dist_max + kZero;
      while (cur_dist < cur_rad && jpart < n2) {
        const uint32_t s = L.U(kSU_TMP, jpart);
        npp += 1;
        const double weight = (double)L.F(kSF_W, s);
        if (B.w) {
          if (fabs(weight - 1.0) < kZero) M_hires += weight;
          else if (weight > 1.0) M_lores += weight;
        } else {
          M_hires += weight;
        }
        M_sphere += weight;
        const double dX = L.D(kSD_DX, s), dY = L.D(kSD_DY, s), dZ = L.D(kSD_DZ, s);
        cur_dist = L.D(kSD_D, s);
        CoM0 += weight * (cx + dX);
        CoM1 += weight * (cy + dY);
        CoM2 += weight * (cz + dZ);
        a11 += weight * dX * dX;
        a22 += weight * dY * dY;
        a33 += weight * dZ * dZ;
        a12 += weight * dX * dY;
        a13 += weight * dX * dZ;
        a23 += weight * dY * dZ;
        const double VXp = (double)L.F(kSF_VX, s), VYp = (double)L.F(kSF_VY, s), VZp = (double)L.F(kSF_VZ, s);
        VXc += weight * VXp;
        VYc += weight * VYp;
        VZc += weight * VZp;
        double dVX = (VXp - VXc / M_sphere);
        double dVY = (VYp - VYc / M_sphere);
        double dVZ = (VZp - VZc / M_sphere);
        Lx += weight * (dY * dVZ - dZ * dVY);
        Ly += weight * (dZ * dVX - dX * dVZ);
        Lz += weight * (dX * dVY - dY * dVX);
        dVX += Hrv * dX * P.r_fac / P.v_fac;
        dVY += Hrv * dY * P.r_fac / P.v_fac;
        dVZ += Hrv * dZ * P.r_fac / P.v_fac;
        const double Tpart = weight * ((dVX * dVX + dVY * dVY) + dVZ * dVZ);
        double Upart;
        if (cur_dist > kMachineZero) {
          I_now = M_sphere / (cur_dist * cur_dist);
          const double I_mid = (I_now + I_prev) / 2.;
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
        const double Epart = (0.5 * Tpart + Upart);
        if (Epart < Emin) { Emin = Epart; mb = (long long)(o + L.U(kSU_ORD, s)); }
        // per-rank arrays: radius over the sort keys (no longer needed)
        L.D(kSD_KEY, jpart) = cur_dist;
        L.D(kSD_OVD, jpart) = M_sphere / (FPT * (cur_dist * cur_dist * cur_dist));
        const double dV = FPT * ((cur_dist * cur_dist * cur_dist) - (prev_dist * prev_dist * prev_dist));
        const double dM = M_sphere - M_sphere_prev;
        L.D(kSD_VC2, jpart) = M_sphere / cur_dist;
        M_sphere_prev = M_sphere;
        const double rm = (cur_dist + prev_dist) / 2.;
        L.D(kSD_DR2, jpart) = dM / dV * (rm * rm);
        prev_dist = cur_dist;
        jpart++;
      }
      Bin R;
      R.npart = npp; R.M = M_sphere; R.Lx = Lx; R.Ly = Ly; R.Lz = Lz; R.T = sig_v; R.U = Epot;
      R.a11 = a11; R.a22 = a22; R.a33 = a33; R.a12 = a12; R.a13 = a13; R.a23 = a23; R.vesc2 = v_esc2;
      stash_bin(rows + (uint64_t)ibin * AHFGPU_PROF_NFIELDS, R, cur_rad);
    }
    const int64_t np5 = (int64_t)n2 - kNignore;
    const double r2 = small_find_max(L, kSD_DR2, np5, 3);
    const double R_max = small_find_max(L, kSD_VC2, np5, 1);
    int64_t ib = 0;
    while (L.D(kSD_KEY, (uint32_t)ib) < R_max && ib < (int64_t)n2 - 1) ib++;
    const double rb = L.D(kSD_KEY, (uint32_t)ib);
    const double M_max = L.D(kSD_OVD, (uint32_t)ib) * FPT * (rb * rb * rb);
    const double V_max = M_max / R_max;
    double* fin = W.fin + (uint64_t)h * kFinStride;
    fin[kFinM] = M_sphere;
    fin[kFinVX] = VXc; fin[kFinVY] = VYc; fin[kFinVZ] = VZc;
    fin[kFinCX] = CoM0; fin[kFinCY] = CoM1; fin[kFinCZ] = CoM2;
    fin[kFinMhi] = M_hires; fin[kFinMlo] = M_lores;
    fin[kFinMbe] = __longlong_as_double(mb);
    fin[kFinR2] = r2; fin[kFinRmax] = R_max; fin[kFinVmax] = V_max;
    H.nbins = nbins;
    flags |= AHFGPU_HALO_RAN_PROFILE;
  }
  // the kept list in radial order, as entry indices
  for (uint32_t k = 0; k < npart; k++) W.mem_stage[o + k] = o + L.U(kSU_ORD, L.U(kSU_TMP, k));
  H.npart = npart;
  H.flags = flags;
}

// Persistent warps: lane 0 takes 32 queue positions at a time.  `scratch`
// holds kSmallSlotBytes * 32 * nmax bytes per warp of the grid.
__global__ void __launch_bounds__(kSmallT) fp32c_small_kernel(DevParams P, DevBatch B, Work W, unsigned char* scratch,
                                                               uint32_t nmax) {
  const int lane = threadIdx.x & 31;
  const uint64_t warp = ((uint64_t)blockIdx.x * kSmallT + threadIdx.x) >> 5;
  const size_t stride = (size_t)32 * nmax;
  unsigned char* base = scratch + warp * stride * kSmallSlotBytes;
  SmallLane L;
  L.lane = lane;
  for (int a = 0; a < kSmallDoubles; a++) L.d[a] = reinterpret_cast<double*>(base) + (size_t)a * stride;
  unsigned char* fb = base + (size_t)kSmallDoubles * 8 * stride;
  for (int a = 0; a < kSmallFloats; a++) L.f[a] = reinterpret_cast<float*>(fb) + (size_t)a * stride;
  unsigned char* ub = fb + (size_t)kSmallFloats * 4 * stride;
  for (int a = 0; a < kSmallU32; a++) L.u[a] = reinterpret_cast<uint32_t*>(ub) + (size_t)a * stride;
  while (true) {
    unsigned q = 0;
    if (lane == 0) q = atomicAdd(W.queue_head, 32u);
    q = __shfl_sync(0xffffffffu, q, 0);
    if (q >= (unsigned)W.nqueue) break;
    const unsigned my = q + (unsigned)lane;
    if (my < (unsigned)W.nqueue) {
      const int h = W.queue[my];
      const uint64_t n = B.off[h + 1] - B.off[h];
      if (n <= nmax) small_halo(h, P, B, W, L);
      else atomicExch(W.err, kErrWorklist);   // a list above the work space: refused, reported
    }
  }
}

void launch_fp32c_small(const DevParams& P, const DevBatch& B, const Work& W, unsigned char* scratch, uint32_t nmax,
                        int grid, cudaStream_t st) {
  fp32c_small_kernel<<<grid, kSmallT, 0, st>>>(P, B, W, scratch, nmax);
}

int fp32c_small_occupancy() {
  int nb = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fp32c_small_kernel, kSmallT, 0);
  return nb;
}

}  // namespace ahfgpu
