// halo_fp64.cu -- FP64 form of AHF's per-halo unbinding + property stage.
//
// One CTA owns one halo at a time (a persistent grid takes haloes from a
// largest-first queue; the plain form launches it once per halo in batch
// order).  Compiled with --fmad=false so each FP64 operation rounds exactly
// as the reference's ISO-C build (-std=c99, no contraction) does.
//
// Per halo (src/libahf/ahf_halos_sfc.c:140-156):
//   keys      dR^2 per particle, signed periodic wrap   ahf_halos.c:5816-5843
//   sort      (key, list slot) ascending                ahf_halos.c:5846
//   rvir0     walk while ovdens >= ovlim                ahf_halos.c:3687-3889
//   unbind    Phi0 pass + bound pass, iterated          ahf_halos.c:3292-3607
//   rvir1     as rvir0
//   profiles  per-particle and per-bin properties       ahf_halos.c:3961-5261
//
// Sums whose rounding depends on order (the potential integral, the running
// bulk velocity) are block scans here.  Each particle's bound test carries a
// rigorous bound on how far the reference's sequential sums can be from the
// scan; if any particle of a halo falls inside that band, the halo's
// unbinding is replayed by one thread in exactly the reference's order
// (serial_unbind), so the kept sets equal the reference's bit for bit.
// Mass prefixes are exact (the host checks that the weights make them so).
#include <cstdint>
#include <cmath>

#include "common.cuh"
#include "sort.cuh"
#include "finish.cuh"

namespace ahfgpu {

constexpr int kT = 256;                 // threads per CTA
constexpr double kEps = 1.1102230246251565e-16;  // 2^-53


struct HaloSmem {
  SortSmem sort;
  double scan[32 * 16];
  int iscan[64];
  double lastd[32];
  int lasti[32];
  double edge[kMaxBins];
  Bin bins[kMaxBins];
  // broadcast slots
  double bd[16];
  long long bl[8];
  int bi[8];
};

// ---------------------------------------------------------------------------
// small helpers
__device__ __forceinline__ double dmin_pos(double a, double b) { return a < b ? a : b; }

struct HaloCtx {
  int h;
  uint64_t o, n;
  double cx, cy, cz;
};

// ---------------------------------------------------------------------------
// keys + slots of the input list
__device__ void compute_keys(const HaloCtx& c, const DevBatch& B, const Work& W) {
  for (uint64_t i = threadIdx.x; i < c.n; i += blockDim.x) {
    uint64_t e = c.o + i;
    double dX = wrap_s((double)B.x[e] - c.cx);
    double dY = wrap_s((double)B.y[e] - c.cy);
    double dZ = wrap_s((double)B.z[e] - c.cz);
    double k = (dX * dX + dY * dY) + dZ * dZ;
    W.keyA[e] = (uint64_t)__double_as_longlong(k);
    W.idxA[e] = (uint32_t)i;
  }
  __syncthreads();
}

// sorted particle arrays; returns (via smem) max |v| component and tie count
__device__ void gather_sorted(const HaloCtx& c, const DevBatch& B, const Work& W, HaloSmem& S,
                              float* vmax_out, unsigned long long* ties_out) {
  float vm = 0.f;
  unsigned long long ties = 0;
  for (uint64_t i = threadIdx.x; i < c.n; i += blockDim.x) {
    uint64_t s = c.o + i;
    uint32_t j = W.idxA[s];
    uint64_t e = c.o + j;
    double dX = wrap_s((double)B.x[e] - c.cx);
    double dY = wrap_s((double)B.y[e] - c.cy);
    double dZ = wrap_s((double)B.z[e] - c.cz);
    uint64_t kb = W.keyA[s];
    double k = __longlong_as_double((long long)kb);
    W.sdx[s] = dX;
    W.sdy[s] = dY;
    W.sdz[s] = dZ;
    W.sd[s] = sqrt(k);
    float vx = B.vx[e], vy = B.vy[e], vz = B.vz[e];
    W.svx[s] = vx;
    W.svy[s] = vy;
    W.svz[s] = vz;
    W.sw[s] = B.w ? B.w[e] : 1.0f;
    W.seid[s] = j;
    W.flag[s] = 1;
    vm = fmaxf(vm, fmaxf(fabsf(vx), fmaxf(fabsf(vy), fabsf(vz))));
    if (i > 0 && W.keyA[s - 1] == kb) ties++;
  }
  // reductions
  for (int off = 16; off > 0; off >>= 1) {
    vm = fmaxf(vm, __shfl_xor_sync(0xffffffffu, vm, off));
    ties += __shfl_xor_sync(0xffffffffu, ties, off);
  }
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (lane == 0) { S.scan[wid] = vm; S.scan[32 + wid] = (double)ties; }
  __syncthreads();
  float m = 0.f;
  double t = 0;
  for (int w = 0; w < nw; w++) { m = fmaxf(m, (float)S.scan[w]); t += S.scan[32 + w]; }
  *vmax_out = m;
  *ties_out = (unsigned long long)t;
  __syncthreads();
}

// ---------------------------------------------------------------------------
// rem_outsideRvir on the members (flag bit0) of slots [0, nlist): keep the
// prefix up to and including the first member whose ovdens < ovlim.
// Returns the new member count; writes M, R, ovdens to out[0..2].
__device__ uint64_t rvir_cut(const HaloCtx& c, uint64_t nlist, const DevParams& P, const Work& W, HaloSmem& S,
                             double* out) {
  const double V43 = 4. * kPi / 3.;
  double carryM = 0.0;
  int carryN = 0;
  long long stop = -1;           // slot of the first failing member
  double lastM = 0, lastR = -1.0, lastOv = 2 * P.ovlim;
  int keepN = 0;
  for (uint64_t base = 0; base < nlist; base += blockDim.x) {
    uint64_t i = base + threadIdx.x;
    bool valid = i < nlist;
    bool mem = valid && (W.flag[c.o + i] & 1);
    double w = mem ? (double)W.sw[c.o + i] : 0.0;
    double v[1] = {w}, tot[1];
    block_scan<1>(v, tot, S.scan);
    int tn;
    int cnt = block_scan_int(mem ? 1 : 0, &tn, S.iscan);
    double M = carryM + v[0];
    double R = 0, ov = 0;
    bool fail = false;
    if (mem) {
      R = W.sd[c.o + i];
      double V = V43 * (R * R * R);
      ov = M / V * P.rho_fac / P.rho_vir;
      fail = !(ov >= P.ovlim);
    }
    // first failing slot of this tile
    unsigned fb = __ballot_sync(0xffffffffu, fail);
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (lane == 0) S.iscan[32 + wid] = fb ? (wid * 32 + __ffs(fb) - 1) : 0x7fffffff;
    // last member of this tile
    unsigned mb = __ballot_sync(0xffffffffu, mem);
    if (lane == 0) S.lasti[wid] = mb ? (wid * 32 + 31 - __clz(mb)) : -1;
    __syncthreads();
    int first = 0x7fffffff, lastm = -1;
    for (int w = 0; w < nw; w++) {
      first = min(first, S.iscan[32 + w]);
      lastm = max(lastm, S.lasti[w]);
    }
    __syncthreads();
    if (first != 0x7fffffff) {
      if ((int)threadIdx.x == first) {
        S.bd[0] = M; S.bd[1] = R; S.bd[2] = ov;
        S.bi[0] = carryN + cnt;
      }
      __syncthreads();
      lastM = S.bd[0]; lastR = S.bd[1]; lastOv = S.bd[2];
      keepN = S.bi[0];
      stop = (long long)(base + first);
      __syncthreads();
      break;
    }
    if (lastm >= 0) {
      if ((int)threadIdx.x == lastm) { S.bd[0] = M; S.bd[1] = R; S.bd[2] = ov; }
      __syncthreads();
      lastM = S.bd[0]; lastR = S.bd[1]; lastOv = S.bd[2];
      __syncthreads();
    }
    carryM += tot[0];
    carryN += tn;
    keepN = carryN;
  }
  if (stop >= 0) {
    for (uint64_t i = (uint64_t)stop + 1 + threadIdx.x; i < nlist; i += blockDim.x) W.flag[c.o + i] &= ~1u;
    __syncthreads();
  }
  out[0] = lastM; out[1] = lastR; out[2] = lastOv;
  return (uint64_t)keepN;
}

// ---------------------------------------------------------------------------
// Potential pass over members of [0, nlist): phi[slot] = running integral
// (inclusive), returns Phi0 (ahf_halos.c:3343-3426).
__device__ double phi_pass(const HaloCtx& c, uint64_t nlist, const Work& W, HaloSmem& S) {
  double carryM = 0.0, carryPhi = 0.0, carryD = 0.0;
  for (uint64_t base = 0; base < nlist; base += blockDim.x) {
    uint64_t i = base + threadIdx.x;
    bool valid = i < nlist;
    bool mem = valid && (W.flag[c.o + i] & 1);
    double w = mem ? (double)W.sw[c.o + i] : 0.0;
    double d = mem ? W.sd[c.o + i] : 0.0;
    bool any;
    double lastd;
    double dprev = block_last_excl(mem, d, carryD, &any, &lastd, S.lastd, S.lasti);
    double v[1] = {w}, tot[1];
    block_scan<1>(v, tot, S.scan);
    double M = carryM + v[0];
    double term = 0.0;
    if (mem && d > kMachineZero) {
      double Mprev = M - w;
      double Iprev = dprev > kMachineZero ? Mprev / (dprev * dprev) : 0.0;
      double Inow = M / (d * d);
      term = ((Inow + Iprev) / 2.) * (d - dprev);
    }
    double t[1] = {term}, tt[1];
    block_scan<1>(t, tt, S.scan);
    if (mem) W.phi[c.o + i] = carryPhi + t[0];
    carryM += tot[0];
    carryPhi += tt[0];
    carryD = lastd;
  }
  return carryPhi + carryM / carryD;
}

// ---------------------------------------------------------------------------
// Exact sequential replay of rem_unbound (ahf_halos.c:3292-3607) by one
// thread, over the sorted slots [0, n1) (all members at entry).  Leaves the
// final members in flag bit0.  out: M_vir, R_vir, Phi0, niter, nobound.
__device__ void serial_unbind(const HaloCtx& c, uint64_t n1, const DevParams& P, const Work& W, double* out,
                              int* niter_out, int* nobound_out) {
  const uint64_t o = c.o;
  uint64_t no_vbulk = (uint64_t)(P.MINPART / 2);
  uint64_t nremove = 4;
  int niter = 0, nobound = 0;
  double R_vir = 0.0, M_vir_out = 0.0, Phi0 = 0.0;
  uint64_t npart = n1;
  for (uint64_t i = 0; i < n1; i++) W.flag[o + i] = 1;
  while (nremove > 3) {
    niter++;
    double I_now = 0.0, I_prev = 0.0, d_prev = 0.0, M_r = 0.0, dist = 0.0;
    Phi0 = 0.0;
    for (uint64_t i = 0; i < n1; i++) {
      if (!(W.flag[o + i] & 1)) continue;
      M_r += (double)W.sw[o + i];
      dist = W.sd[o + i];
      if (dist > kMachineZero) {
        I_now = M_r / (dist * dist);
        double I_mid = (I_now + I_prev) / 2.;
        double dr = dist - d_prev;
        Phi0 += I_mid * dr;
      }
      d_prev = dist;
      I_prev = I_now;
    }
    Phi0 += M_r / dist;
    // seed
    uint64_t js = 0;
    if (niter == 1) {
      float m2[64];
      uint32_t pos[64];
      uint64_t nv = no_vbulk < 64 ? no_vbulk : 64;
      for (uint64_t j = 0; j < nv; j++) {
        float mx = W.svx[o + j], my = W.svy[o + j], mz = W.svz[o + j];
        float t = __fadd_rn(__fadd_rn(__fmul_rn(mx, mx), __fmul_rn(my, my)), __fmul_rn(mz, mz));
        m2[j] = t;
        pos[j] = (uint32_t)j;
      }
      for (uint64_t i = 1; i < nv; i++) {
        float kv = m2[i];
        uint32_t kp = pos[i];
        uint64_t k = i;
        while (k > 0 && m2[k - 1] > kv) { m2[k] = m2[k - 1]; pos[k] = pos[k - 1]; k--; }
        m2[k] = kv;
        pos[k] = kp;
      }
      js = pos[no_vbulk / 2 - 1];
    } else {
      js = 0;
      while (js < n1 && !(W.flag[o + js] & 1)) js++;
    }
    double w0 = (double)W.sw[o + js];
    double M_vel = w0;
    double VXc = w0 * (double)W.svx[o + js], VYc = w0 * (double)W.svy[o + js], VZc = w0 * (double)W.svz[o + js];
    nremove = 0;
    I_now = 0.0; I_prev = 0.0; d_prev = 0.0; M_r = 0.0;
    double M_vir = 0.0, Phi = 0.0;
    uint64_t nb = 0;
    for (uint64_t i = 0; i < n1; i++) {
      uint8_t f = W.flag[o + i];
      if (!(f & 1)) continue;
      double weight = (double)W.sw[o + i];
      M_r += weight;
      double dX = W.sdx[o + i], dY = W.sdy[o + i], dZ = W.sdz[o + i];
      dist = W.sd[o + i];
      double v_esc2;
      if (dist > kMachineZero) {
        I_now = M_r / (dist * dist);
        double I_mid = (I_now + I_prev) / 2.;
        double dr = dist - d_prev;
        Phi += I_mid * dr;
        v_esc2 = (2 * fabs(Phi - Phi0) * P.phi_fac);
      } else {
        v_esc2 = 1e30;
      }
      double VXp = (double)W.svx[o + i], VYp = (double)W.svy[o + i], VZp = (double)W.svz[o + i];
      double dVX = (VXp - VXc / M_vel) * P.v_fac + P.Hubble * (dX) * P.r_fac;
      double dVY = (VYp - VYc / M_vel) * P.v_fac + P.Hubble * (dY) * P.r_fac;
      double dVZ = (VZp - VZc / M_vel) * P.v_fac + P.Hubble * (dZ) * P.r_fac;
      double vel2 = (dVX * dVX + dVY * dVY) + dVZ * dVZ;
      if (vel2 > P.v2_tune * v_esc2) {
        nremove++;
        W.flag[o + i] = 2;  // removed this pass (bit0 cleared after the pass)
      } else {
        M_vel += weight;
        VXc += weight * VXp;
        VYc += weight * VYp;
        VZc += weight * VZp;
        nb++;
        M_vir += weight;
        R_vir = dist;
      }
      I_prev = I_now;
      d_prev = dist;
    }
    for (uint64_t i = 0; i < n1; i++)
      if (W.flag[o + i] == 2) W.flag[o + i] = 0;
    if (nb == 0) nobound = 1;
    npart = nb;
    M_vir_out = M_vir;
    if (((double)npart) < ((double)P.MINPART)) break;
  }
  out[0] = M_vir_out;
  out[1] = R_vir;
  out[2] = Phi0;
  out[3] = (double)npart;
  *niter_out = niter;
  *nobound_out = nobound;
}

// ---------------------------------------------------------------------------
// Warp-sequential prefix sums in exactly the order of a C loop: one FP64
// rounding per addition, left to right, starting from s0.  The 32 lanes load
// 32 addends at a time and every lane performs the same chain of additions
// on the broadcast values, so the prefix costs one dependent DADD per
// element.  incl=1: out[i] = s0 + a[0] + ... + a[i];  incl=0: out[i] = the
// sum before a[i].  Returns the total.  `a` and `out` may alias.
__device__ double warp_chain(const double* a, double* out, uint64_t n, double s0, int incl) {
  const unsigned FULL = 0xffffffffu;
  int lane = threadIdx.x & 31;
  double s = s0;
  for (uint64_t base = 0; base < n; base += 32) {
    uint64_t i = base + lane;
    double t = i < n ? a[i] : 0.0;
    double mine = s;
#pragma unroll
    for (int k = 0; k < 32; k++) {
      double tk = __shfl_sync(FULL, t, k);
      if (!incl && k == lane) mine = s;
      s += tk;
      if (incl && k == lane) mine = s;
    }
    if (i < n) out[i] = mine;
  }
  return s;
}

// One rem_unbound iteration (ahf_halos.c:3343-3583) in exactly the
// reference's summation order, for a halo whose parallel evaluation left a
// particle inside the rounding band.  Members: flag bit0 of slots [0, n1);
// bit1 holds the speculated bound flags on entry and the exact ones on exit.
// The order-dependent sums (potential integral, running bulk velocity) are
// warp chains; the bound tests are re-evaluated in parallel until no flag
// changes (the recurrence is triangular, so the fixpoint is the sequential
// result).  Returns Phi0; *mb/*nb/*rlast: kept mass, count, last distance.
__device__ double exact_iteration(const HaloCtx& c, uint64_t n1, const DevParams& P, const Work& W, HaloSmem& S,
                                  uint64_t js, double* mb, long long* nbo, double* rlast, bool* any_b,
                                  int* rounds_out) {
  const uint64_t o = c.o;
  double* term = W.phi + o;
  double* ax = W.prof_b + o;
  double* ay = W.prof_c + o;
  double* az = W.prof_d + o;
  // potential terms of the members (0 elsewhere)
  double carryM = 0.0, carryD = 0.0;
  for (uint64_t base = 0; base < n1; base += blockDim.x) {
    uint64_t i = base + threadIdx.x;
    bool mem = i < n1 && (W.flag[o + i] & 1);
    double w = mem ? (double)W.sw[o + i] : 0.0;
    double d = mem ? W.sd[o + i] : 0.0;
    bool any;
    double lastd;
    double dprev = block_last_excl(mem, d, carryD, &any, &lastd, S.lastd, S.lasti);
    double v[1] = {w}, tot[1];
    block_scan<1>(v, tot, S.scan);
    double M = carryM + v[0];
    double t = 0.0;
    if (mem && d > kMachineZero) {
      double Mprev = M - w;
      double Iprev = dprev > kMachineZero ? Mprev / (dprev * dprev) : 0.0;
      double Inow = M / (d * d);
      t = ((Inow + Iprev) / 2.) * (d - dprev);
    }
    if (i < n1) term[i] = t;
    carryM += tot[0];
    carryD = lastd;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    double s = warp_chain(term, term, n1, 0.0, 1);
    if (threadIdx.x == 0) S.bd[12] = s;
  }
  __syncthreads();
  const double Phi0 = S.bd[12] + carryM / carryD;
  const double w0 = (double)W.sw[o + js];
  const double sVX = w0 * (double)W.svx[o + js], sVY = w0 * (double)W.svy[o + js], sVZ = w0 * (double)W.svz[o + js];
  int rounds = 0;
  double Mb = 0, Rl = 0;
  long long nb = 0;
  bool anyb = false;
  while (true) {
    rounds++;
    // addends of the running bulk velocity under the current flags
    for (uint64_t i = threadIdx.x; i < n1; i += blockDim.x) {
      uint8_t f = W.flag[o + i];
      bool b = (f & 1) && ((f >> 1) & 1);
      double w = b ? (double)W.sw[o + i] : 0.0;
      ax[i] = b ? w * (double)W.svx[o + i] : 0.0;
      ay[i] = b ? w * (double)W.svy[o + i] : 0.0;
      az[i] = b ? w * (double)W.svz[o + i] : 0.0;
    }
    __syncthreads();
    int warp = threadIdx.x >> 5;
    if (warp == 0) warp_chain(ax, ax, n1, sVX, 0);
    else if (warp == 1) warp_chain(ay, ay, n1, sVY, 0);
    else if (warp == 2) warp_chain(az, az, n1, sVZ, 0);
    __syncthreads();
    int changed = 0;
    double cMV = w0, carryMb = 0.0, carryR = 0.0;
    long long carryNb = 0;
    bool anyR = false;
    for (uint64_t base = 0; base < n1; base += blockDim.x) {
      uint64_t i = base + threadIdx.x;
      bool valid = i < n1;
      uint8_t f = valid ? W.flag[o + i] : 0;
      bool mem = f & 1;
      bool b = mem && ((f >> 1) & 1);
      double w = mem ? (double)W.sw[o + i] : 0.0;
      double cw = b ? w : 0.0;
      double v[1] = {cw}, ex[1], tot[1];
      block_scan_excl<1>(v, ex, tot, S.scan);
      bool nbv = false;
      double d = 0.0;
      if (mem) {
        double M_vel = cMV + ex[0];
        d = W.sd[o + i];
        double dX = W.sdx[o + i], dY = W.sdy[o + i], dZ = W.sdz[o + i];
        double v_esc2;
        if (d > kMachineZero) v_esc2 = (2 * fabs(term[i] - Phi0) * P.phi_fac);
        else v_esc2 = 1e30;
        double VXp = (double)W.svx[o + i], VYp = (double)W.svy[o + i], VZp = (double)W.svz[o + i];
        double dVX = (VXp - ax[i] / M_vel) * P.v_fac + P.Hubble * (dX) * P.r_fac;
        double dVY = (VYp - ay[i] / M_vel) * P.v_fac + P.Hubble * (dY) * P.r_fac;
        double dVZ = (VZp - az[i] / M_vel) * P.v_fac + P.Hubble * (dZ) * P.r_fac;
        double vel2 = (dVX * dVX + dVY * dVY) + dVZ * dVZ;
        nbv = !(vel2 > P.v2_tune * v_esc2);
        if (nbv != b) changed = 1;
        W.flag[o + i] = (uint8_t)(1 | (nbv ? 2 : 0));
      }
      int tcnt;
      block_scan_int(b ? 1 : 0, &tcnt, S.iscan);
      bool any;
      double lastR;
      block_last_excl(b, d, carryR, &any, &lastR, S.lastd, S.lasti);
      carryR = lastR;
      anyR |= any;
      carryMb += tot[0];
      carryNb += tcnt;
      cMV += tot[0];
    }
    if (!__syncthreads_or(changed)) {
      Mb = carryMb;
      nb = carryNb;
      Rl = carryR;
      anyb = anyR;
      break;
    }
  }
  *mb = Mb;
  *nbo = nb;
  *rlast = Rl;
  *any_b = anyb;
  *rounds_out = rounds;
  return Phi0;
}

// ---------------------------------------------------------------------------
// Parallel rem_unbound.  An iteration whose bound decisions include one
// inside the rounding band is redone by exact_iteration (*replayed set).
__device__ bool parallel_unbind(const HaloCtx& c, uint64_t n1, const DevParams& P, const Work& W, HaloSmem& S,
                                float vmax, double* out, int* niter_out, int* nobound_out, int* rounds_out,
                                int* replayed) {
  const uint64_t o = c.o;
  uint64_t no_vbulk = (uint64_t)(P.MINPART / 2);
  uint64_t nremove = 4;
  int niter = 0, nobound = 0, maxrounds = 0;
  double R_vir = 0.0, M_vir_out = 0.0, Phi0 = 0.0;
  uint64_t npart = n1;
  const float fe = (float)kEps;
  while (nremove > 3) {
    niter++;
    Phi0 = phi_pass(c, n1, W, S);
    // seed slot
    if (threadIdx.x == 0) {
      uint64_t js = 0;
      if (niter == 1) {
        float m2[64];
        uint32_t pos[64];
        uint64_t nv = no_vbulk < 64 ? no_vbulk : 64;
        for (uint64_t j = 0; j < nv; j++) {
          float mx = W.svx[o + j], my = W.svy[o + j], mz = W.svz[o + j];
          m2[j] = __fadd_rn(__fadd_rn(__fmul_rn(mx, mx), __fmul_rn(my, my)), __fmul_rn(mz, mz));
          pos[j] = (uint32_t)j;
        }
        for (uint64_t i = 1; i < nv; i++) {
          float kv = m2[i];
          uint32_t kp = pos[i];
          uint64_t k = i;
          while (k > 0 && m2[k - 1] > kv) { m2[k] = m2[k - 1]; pos[k] = pos[k - 1]; k--; }
          m2[k] = kv;
          pos[k] = kp;
        }
        js = pos[no_vbulk / 2 - 1];
      } else {
        while (js < n1 && !(W.flag[o + js] & 1)) js++;
      }
      S.bl[0] = (long long)js;
    }
    __syncthreads();
    uint64_t js = (uint64_t)S.bl[0];
    double w0 = (double)W.sw[o + js];
    double sVX = w0 * (double)W.svx[o + js], sVY = w0 * (double)W.svy[o + js], sVZ = w0 * (double)W.svz[o + js];
    __syncthreads();
    // speculation: every member bound (bit1 = bit0)
    for (uint64_t i = threadIdx.x; i < n1; i += blockDim.x) {
      uint8_t f = W.flag[o + i] & 1;
      W.flag[o + i] = f | (f << 1);
    }
    __syncthreads();
    const float gam_n = 2.0f * (float)(n1 + 64) * fe;
    int rounds = 0;
    bool amb_any = false;
    double Mb = 0, Rlast = 0;
    long long nb = 0;
    while (true) {
      rounds++;
      double cVX = sVX, cVY = sVY, cVZ = sVZ, cMV = w0;
      int changed = 0, amb = 0;
      double carryMb = 0.0;
      long long carryNb = 0;
      double carryR = R_vir;
      bool anyR = false;
      for (uint64_t base = 0; base < n1; base += blockDim.x) {
        uint64_t i = base + threadIdx.x;
        bool valid = i < n1;
        uint8_t f = valid ? W.flag[o + i] : 0;
        bool mem = f & 1;
        bool b = (f >> 1) & 1;
        double w = 0, vx = 0, vy = 0, vz = 0;
        if (mem) {
          w = (double)W.sw[o + i];
          vx = (double)W.svx[o + i];
          vy = (double)W.svy[o + i];
          vz = (double)W.svz[o + i];
        }
        double cw = b ? w : 0.0;
        double v[4] = {cw * vx, cw * vy, cw * vz, cw}, ex[4], tot[4];
        block_scan_excl<4>(v, ex, tot, S.scan);
        bool nbv = false;
        if (mem) {
          double VXc = cVX + ex[0], VYc = cVY + ex[1], VZc = cVZ + ex[2], Mv = cMV + ex[3];
          double d = W.sd[o + i];
          double dX = W.sdx[o + i], dY = W.sdy[o + i], dZ = W.sdz[o + i];
          double phi = W.phi[o + i];
          double v_esc2;
          if (d > kMachineZero) v_esc2 = (2 * fabs(phi - Phi0) * P.phi_fac);
          else v_esc2 = 1e30;
          double bx = vx - VXc / Mv, by = vy - VYc / Mv, bz = vz - VZc / Mv;
          double hx = P.Hubble * (dX) * P.r_fac, hy = P.Hubble * (dY) * P.r_fac, hz = P.Hubble * (dZ) * P.r_fac;
          double dVX = bx * P.v_fac + hx, dVY = by * P.v_fac + hy, dVZ = bz * P.v_fac + hz;
          double vel2 = (dVX * dVX + dVY * dVY) + dVZ * dVZ;
          double thr = P.v2_tune * v_esc2;
          nbv = !(vel2 > thr);
          // rounding band (float arithmetic on magnitudes, factor 2 slack)
          float A = (float)fabs(phi - Phi0);
          float fthr = (float)thr, fv2 = (float)vel2;
          float dthr = (d > kMachineZero)
                           ? fthr * (gam_n * (float)Phi0 * 2.0f / fmaxf(A, 1e-30f) + 8.0f * fe)
                           : fthr * 8.0f * fe;
          float gj = 2.0f * (float)(i + 64) * fe;
          float vf = (float)P.v_fac;
          float sb = vmax * vf;
          float ddv = gj * sb + 6.0f * fe * (2.0f * sb + fabsf((float)hx) + fabsf((float)hy) + fabsf((float)hz));
          float dvel2 = 2.0f * 1.7320508f * sqrtf(fv2) * ddv + 3.0f * ddv * ddv + 8.0f * fe * fv2;
          float margin = (float)fabs(vel2 - thr);
          if (margin <= 2.0f * (dthr + dvel2) * 1.25f) amb = 1;
        }
        bool nbm = mem && nbv;
        if (mem && (nbm != b)) changed = 1;
        if (valid) W.flag[o + i] = (uint8_t)((mem ? 1 : 0) | (nbm ? 2 : 0));
        // totals over the flags used in this round (== final at convergence)
        carryMb += tot[3];
        int tcnt;
        block_scan_int(b ? 1 : 0, &tcnt, S.iscan);
        carryNb += tcnt;
        bool any;
        double lastR;
        block_last_excl(b, mem ? W.sd[o + i] : 0.0, carryR, &any, &lastR, S.lastd, S.lasti);
        carryR = lastR;
        anyR |= any;
        cVX += tot[0]; cVY += tot[1]; cVZ += tot[2]; cMV += tot[3];
      }
      int ch = __syncthreads_or(changed);
      int am = __syncthreads_or(amb);
      if (!ch) {
        amb_any = am != 0;
        Mb = carryMb;
        nb = carryNb;
        Rlast = carryR;
        break;
      }
      if (rounds >= kMaxFixRounds) { amb_any = true; break; }
    }
    if (rounds > maxrounds) maxrounds = rounds;
    if (amb_any || P.force_exact) {
      // a decision lies inside the rounding band: redo this iteration in
      // the reference's exact summation order
      long long nbx;
      double mbx, rlx;
      bool anyb;
      int rr;
      Phi0 = exact_iteration(c, n1, P, W, S, js, &mbx, &nbx, &rlx, &anyb, &rr);
      Mb = mbx;
      nb = nbx;
      Rlast = anyb ? rlx : R_vir;
      *replayed = 1;
      if (rr > maxrounds) maxrounds = rr;
    }
    // members <- bound
    for (uint64_t i = threadIdx.x; i < n1; i += blockDim.x) {
      uint8_t f = W.flag[o + i];
      W.flag[o + i] = (f >> 1) & 1;
    }
    __syncthreads();
    nremove = npart - (uint64_t)nb;
    npart = (uint64_t)nb;
    if (nb == 0) nobound = 1;
    M_vir_out = Mb;
    R_vir = Rlast;
    if (((double)npart) < ((double)P.MINPART)) break;
  }
  out[0] = M_vir_out;
  out[1] = R_vir;
  out[2] = Phi0;
  out[3] = (double)npart;
  *niter_out = niter;
  *nobound_out = nobound;
  *rounds_out = maxrounds;
  return true;
}

// smooth3 (src/libutility/general.c:548-573), `ns` passes over y[0..m),
// ping-ponging with t; returns the buffer that holds the result.
__device__ double* block_smooth3(double* y, double* t, uint64_t m, int ns) {
  if (ns == 0 || m < 3) return y;
  for (int p = 0; p < ns; p++) {
    for (uint64_t i = threadIdx.x; i < m; i += blockDim.x) {
      double r;
      if (i == 0) r = (y[0] + y[1]) / 2.;
      else if (i == m - 1) r = (y[m - 1] + y[m - 2]) / 2.;
      else r = (y[i - 1] + y[i] + y[i + 1]) / 3.;
      t[i] = r;
    }
    __syncthreads();
    double* s = y; y = t; t = s;
  }
  return y;
}

// find_max (src/libutility/general.c:608-650): first strict maximum of the
// smoothed array over [0, m-2] (m-1 if none exceeds -10).
__device__ uint64_t block_argmax_first(const double* y, uint64_t m, HaloSmem& S) {
  double best = -10.0;
  long long bi = -1;
  for (uint64_t i = threadIdx.x; i + 1 < m; i += blockDim.x) {
    double v = y[i];
    if (v > best) { best = v; bi = (long long)i; }   // per-thread first (increasing i)
  }
  // reduce: larger value wins; equal -> smaller index
  for (int off = 16; off > 0; off >>= 1) {
    double ob = __shfl_xor_sync(0xffffffffu, best, off);
    long long oi = __shfl_xor_sync(0xffffffffu, bi, off);
    bool take = (oi >= 0) && (bi < 0 || ob > best || (ob == best && oi < bi));
    if (take) { best = ob; bi = oi; }
  }
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (lane == 0) { S.scan[wid] = best; S.bl[0] = 0; ((long long*)S.scan)[32 + wid] = bi; }
  __syncthreads();
  double B = -10.0;
  long long I = -1;
  for (int w = 0; w < nw; w++) {
    double ob = S.scan[w];
    long long oi = ((long long*)S.scan)[32 + w];
    bool take = (oi >= 0) && (I < 0 || ob > B || (ob == B && oi < I));
    if (take) { B = ob; I = oi; }
  }
  __syncthreads();
  return I < 0 ? m - 1 : (uint64_t)I;
}

// ---------------------------------------------------------------------------
// HaloProfiles over the members of [0, n1) (n2 of them).
__device__ void profiles(const HaloCtx& c, uint64_t n1, uint64_t n2, const DevParams& P, const DevBatch& B,
                         const Work& W, HaloSmem& S, ahfgpu_halo& hout) {
  const uint64_t o = c.o;
  const double FPT = 4. * kPi / 3.;
  double* radius = W.prof_c + o;
  double* ovd = W.prof_d + o;
  double* vc2 = W.prof_b + o;
  double* dr2 = W.prof_a + o;
  // compact member distances first (needed by binning_parameter)
  {
    int carry = 0;
    for (uint64_t base = 0; base < n1; base += blockDim.x) {
      uint64_t i = base + threadIdx.x;
      bool mem = i < n1 && (W.flag[o + i] & 1);
      int tot;
      int r = block_scan_int(mem ? 1 : 0, &tot, S.iscan) - 1 + carry;
      if (mem) radius[r] = W.sd[o + i];
      carry += tot;
    }
    __syncthreads();
  }
  // binning_parameter, src/libutility/specific.c:259-322
  if (threadIdx.x == 0) {
    int nb = (int)(6.2 * (log10((double)n2)) - 3.5);
    if (nb < 2) nb = 2;
    if (nb > kMaxBins) nb = kMaxBins;
    long np = (long)floor(((double)P.MINPART / 10.) + 0.5);
    double dmin = -1.0;
    while (np < (long)n2 - 1 && dmin < kMachineZero) { dmin = radius[np]; np++; }
    double dmax = radius[n2 - 1];
    if (dmin < kMachineZero) dmin = dmax / 2.;
    double ld0 = log10(dmin), ld1 = log10(dmax);
    S.bd[2] = ld0;
    S.bd[3] = (ld1 - ld0) / (double)nb;
    S.bi[0] = nb;
    S.bd[0] = dmin;
    S.bd[1] = dmax;
  }
  __syncthreads();
  for (int b = threadIdx.x; b < S.bi[0]; b += blockDim.x)
    S.edge[b] = b == S.bi[0] - 1 ? S.bd[1] + kZero : pow(10., S.bd[2] + ((double)b + 1) * S.bd[3]);
  __syncthreads();
  const int nbins = S.bi[0];
  const double Phi0 = hout.Phi0;
  // main pass
  double cM = 0, cVX = 0, cVY = 0, cVZ = 0, cD = 0.0;
  double cs[16] = {0};   // phi, Lx, Ly, Lz, T, CoMx, CoMy, CoMz, a11, a22, a33, a12, a13, a23, Mhi, Mlo
  double cU = 0.0;
  double Emin = 1e30;
  long long mbslot = -1;
  int cr = 0;
  for (uint64_t base = 0; base < n1; base += blockDim.x) {
    uint64_t i = base + threadIdx.x;
    bool mem = i < n1 && (W.flag[o + i] & 1);
    double w = 0, vx = 0, vy = 0, vz = 0, dX = 0, dY = 0, dZ = 0, d = 0;
    if (mem) {
      w = (double)W.sw[o + i];
      vx = (double)W.svx[o + i]; vy = (double)W.svy[o + i]; vz = (double)W.svz[o + i];
      dX = W.sdx[o + i]; dY = W.sdy[o + i]; dZ = W.sdz[o + i];
      d = W.sd[o + i];
    }
    bool any;
    double lastd;
    double dp = block_last_excl(mem, d, cD, &any, &lastd, S.lastd, S.lasti);
    int tn;
    int rank = block_scan_int(mem ? 1 : 0, &tn, S.iscan) - 1 + cr;
    double s1[4] = {w, w * vx, w * vy, w * vz}, t1[4];
    block_scan<4>(s1, t1, S.scan);
    double M = cM + s1[0];
    double VXc = cVX + s1[1], VYc = cVY + s1[2], VZc = cVZ + s1[3];
    double s2[16] = {0};
    if (mem) {
      double dVX = (vx - VXc / M), dVY = (vy - VYc / M), dVZ = (vz - VZc / M);
      s2[1] = w * (dY * dVZ - dZ * dVY);
      s2[2] = w * (dZ * dVX - dX * dVZ);
      s2[3] = w * (dX * dVY - dY * dVX);
      dVX += P.Hubble * dX * P.r_fac / P.v_fac;
      dVY += P.Hubble * dY * P.r_fac / P.v_fac;
      dVZ += P.Hubble * dZ * P.r_fac / P.v_fac;
      s2[4] = w * ((dVX * dVX + dVY * dVY) + dVZ * dVZ);
      if (d > kMachineZero) {
        double Mp = M - w;
        double Ip = dp > kMachineZero ? Mp / (dp * dp) : 0.0;
        double In = M / (d * d);
        s2[0] = ((In + Ip) / 2.) * (d - dp);
      }
      s2[5] = w * (c.cx + dX);
      s2[6] = w * (c.cy + dY);
      s2[7] = w * (c.cz + dZ);
      s2[8] = w * dX * dX;
      s2[9] = w * dY * dY;
      s2[10] = w * dZ * dZ;
      s2[11] = w * dX * dY;
      s2[12] = w * dX * dZ;
      s2[13] = w * dY * dZ;
      if (P.has_w) {
        if (fabs(w - 1.0) < kZero) s2[14] = w;
        else if (w > 1.0) s2[15] = w;
      } else {
        s2[14] = w;
      }
      // per-member arrays (ahf_halos.c:4598-4616)
      double dV = FPT * ((d * d * d) - (dp * dp * dp));
      double dM = M - (M - w);
      double rm = (d + dp) / 2.;
      ovd[rank] = M / (FPT * (d * d * d));
      vc2[rank] = M / d;
      dr2[rank] = dM / dV * (rm * rm);
    }
    double myT = s2[4];
    double t2[16];
    block_scan<16>(s2, t2, S.scan);
    double phi = cs[0] + s2[0];
    double U = mem ? (phi - Phi0) * w : 0.0;
    double Tpart = myT;
    double su[1] = {U}, tu[1];
    block_scan<1>(su, tu, S.scan);
    // most bound particle: first strict minimum of 0.5 T + U
    double E = mem ? (0.5 * Tpart + U) : 1e300;
    long long es = mem ? (long long)i : -1;
    for (int off = 16; off > 0; off >>= 1) {
      double oE = __shfl_xor_sync(0xffffffffu, E, off);
      long long oi = __shfl_xor_sync(0xffffffffu, es, off);
      bool take = oi >= 0 && (es < 0 || oE < E || (oE == E && oi < es));
      if (take) { E = oE; es = oi; }
    }
    {
      int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
      if (lane == 0) { S.scan[wid] = E; ((long long*)S.scan)[32 + wid] = es; }
      __syncthreads();
      double bE = 1e300;
      long long bs = -1;
      for (int w2 = 0; w2 < nw; w2++) {
        double oE = S.scan[w2];
        long long oi = ((long long*)S.scan)[32 + w2];
        bool take = oi >= 0 && (bs < 0 || oE < bE || (oE == bE && oi < bs));
        if (take) { bE = oE; bs = oi; }
      }
      __syncthreads();
      if (bs >= 0 && bE < Emin) { Emin = bE; mbslot = bs; }
    }
    // bin records at bin ends
    if (mem) {
      int bcur = 0;
      if (rank > 0) { while (bcur < nbins && !(dp < S.edge[bcur])) bcur++; }
      int bnext = 0;
      while (bnext < nbins && !(d < S.edge[bnext])) bnext++;
      bool last = (uint64_t)(rank + 1) == n2;
      int bend = last ? nbins : bnext;
      for (int b = bcur; b < bend; b++) {
        Bin& R = S.bins[b];
        R.npart = (double)(rank + 1);
        R.M = M;
        R.Lx = cs[1] + s2[1]; R.Ly = cs[2] + s2[2]; R.Lz = cs[3] + s2[3];
        R.T = cs[4] + s2[4];
        R.U = cU + su[0];
        R.a11 = cs[8] + s2[8]; R.a22 = cs[9] + s2[9]; R.a33 = cs[10] + s2[10];
        R.a12 = cs[11] + s2[11]; R.a13 = cs[12] + s2[12]; R.a23 = cs[13] + s2[13];
        R.vesc2 = 2 * fabs(U) / w;
      }
    }
    cM += t1[0]; cVX += t1[1]; cVY += t1[2]; cVZ += t1[3];
#pragma unroll
    for (int k = 0; k < 16; k++) cs[k] += t2[k];
    cU += tu[0];
    cD = lastd;
    cr += tn;
    __syncthreads();
  }
  double* rows = W.prof_stage + W.prof_cap_off[c.h] * AHFGPU_PROF_NFIELDS;
  write_bin_rows(S.bins, S.edge, nbins, rows);
  __syncthreads();
  // find_max on dens_r2 (3 smoothings) and Vcirc2 (1), both from slot nignore
  uint64_t m = n2 - kNignore;
  double* tmpbuf = W.phi + o;   // phi is free now
  double* ys;
  // copy (find_max smooths a copy)
  for (uint64_t i = threadIdx.x; i < m; i += blockDim.x) tmpbuf[i] = dr2[kNignore + i];
  __syncthreads();
  double* tmp2 = (double*)(W.keyB + o);
  ys = block_smooth3(tmpbuf, tmp2, m, 3);
  uint64_t i_r2 = block_argmax_first(ys, m, S);
  for (uint64_t i = threadIdx.x; i < m; i += blockDim.x) tmpbuf[i] = vc2[kNignore + i];
  __syncthreads();
  ys = block_smooth3(tmpbuf, tmp2, m, 1);
  uint64_t i_rm = block_argmax_first(ys, m, S);
  __syncthreads();
  if (threadIdx.x == 0) {
    double r2 = (radius[kNignore + i_r2] + radius[kNignore + i_r2]) / 2;
    double x_max = (radius[kNignore + i_rm] + radius[kNignore + i_rm]) / 2;
    double R_max = x_max;
    // first slot with radius >= x_max (linear rule of ahf_halos.c:4897-4899)
    uint64_t lo = 0, hi = n2 - 1;
    while (lo < hi) {
      uint64_t mid = (lo + hi) / 2;
      if (radius[mid] < x_max) lo = mid + 1; else hi = mid;
    }
    uint64_t ib = lo;
    double M_max = ovd[ib] * FPT * (radius[ib] * radius[ib] * radius[ib]);
    double V_max = M_max / R_max;
    long long mbe = mbslot >= 0 ? (long long)(o + W.seid[o + mbslot]) : -1;
    finish_scalars(rows, nbins, cM, cVX, cVY, cVZ, cs[5], cs[6], cs[7], cs[14], cs[15], mbe, r2, R_max, V_max,
                   P, B, c.cx, c.cy, c.cz, hout);
    hout.nbins = nbins;
    hout.flags |= AHFGPU_HALO_RAN_PROFILE;
  }
  __syncthreads();
}

// kept list in radial order -> staging (gidx or entry index)
__device__ void write_members(const HaloCtx& c, uint64_t nlist, const DevBatch& B, const Work& W, HaloSmem& S) {
  int carry = 0;
  for (uint64_t base = 0; base < nlist; base += blockDim.x) {
    uint64_t i = base + threadIdx.x;
    bool mem = i < nlist && (W.flag[c.o + i] & 1);
    int tot;
    int r = block_scan_int(mem ? 1 : 0, &tot, S.iscan) - 1 + carry;
    if (mem) {
      uint64_t e = c.o + W.seid[c.o + i];
      W.mem_stage[c.o + r] = B.gidx ? B.gidx[e] : e;
    }
    carry += tot;
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
__device__ void process_halo(int h, const DevParams& P, const DevBatch& B, const Work& W, HaloSmem& S,
                             uint4* stack) {
  HaloCtx c;
  c.h = h;
  c.o = B.off[h];
  c.n = B.off[h + 1] - c.o;
  c.cx = B.cx[h]; c.cy = B.cy[h]; c.cz = B.cz[h];
  __shared__ ahfgpu_halo hout;
  if (threadIdx.x == 0) {
    char* p = (char*)&hout;
    for (unsigned k = 0; k < sizeof(ahfgpu_halo); k++) p[k] = 0;
  }
  __syncthreads();
  if (c.n == 0) {
    if (threadIdx.x == 0) { hout.flags = AHFGPU_HALO_EMPTY; W.halo[h] = hout; }
    __syncthreads();
    return;
  }
  if (c.n < (uint64_t)P.MINPART) {
    // nothing runs; the gathered list passes through unchanged
    for (uint64_t i = threadIdx.x; i < c.n; i += blockDim.x) {
      uint64_t e = c.o + i;
      W.mem_stage[e] = B.gidx ? B.gidx[e] : e;
    }
    if (threadIdx.x == 0) { hout.npart = c.n; W.halo[h] = hout; }
    __syncthreads();
    return;
  }
  compute_keys(c, B, W);
  const int src = radial_sort(W.keyA, W.idxA, W.keyB, W.idxB, c.o, c.n, stack, W.stack_cap, S.sort);
  if (src != kErrNone) {
    if (threadIdx.x == 0) {
      atomicExch(W.err, src);
      W.halo[h] = hout;   // npart 0: nothing is packed for this halo
    }
    __syncthreads();
    return;
  }
  float vmax;
  unsigned long long ties;
  gather_sorted(c, B, W, S, &vmax, &ties);
  if (threadIdx.x == 0) {
    hout.flags |= AHFGPU_HALO_RAN_SORT | AHFGPU_HALO_RAN_RVIR0;
    if (ties) atomicAdd(&W.counters[2], ties);
  }
  double r0[3];
  uint64_t n1 = rvir_cut(c, c.n, P, W, S, r0);
  if (threadIdx.x == 0) {
    hout.M_vir = r0[0]; hout.R_vir = r0[1]; hout.ovdens = r0[2]; hout.Phi0 = 0.0;
  }
  uint64_t nlist = c.n;
  uint64_t ncur = n1;
  if (n1 >= (uint64_t)P.MINPART) {
    double uo[4];
    int niter = 0, nob = 0, rounds = 0, replayed = 0;
    bool pok = P.force_serial ? false
                              : parallel_unbind(c, n1, P, W, S, vmax, uo, &niter, &nob, &rounds, &replayed);
    if (replayed && threadIdx.x == 0) {
      atomicAdd(&W.counters[1], 1ull);
      hout.flags |= AHFGPU_HALO_REPLAYED;
    }
    if (!pok) {
      // weights whose FP64 sums are not exact: one thread, reference order
      if (threadIdx.x == 0) {
        serial_unbind(c, n1, P, W, uo, &niter, &nob);
        S.bd[8] = uo[0]; S.bd[9] = uo[1]; S.bd[10] = uo[2]; S.bd[11] = uo[3];
        S.bi[4] = niter; S.bi[5] = nob;
        atomicAdd(&W.counters[1], 1ull);
        hout.flags |= AHFGPU_HALO_REPLAYED;
      }
      __syncthreads();
      uo[0] = S.bd[8]; uo[1] = S.bd[9]; uo[2] = S.bd[10]; uo[3] = S.bd[11];
      niter = S.bi[4]; nob = S.bi[5];
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      hout.flags |= AHFGPU_HALO_RAN_UNBIND;
      if (nob) hout.flags |= AHFGPU_HALO_NOBOUND;
      hout.M_vir = uo[0];
      hout.R_vir = uo[1];
      hout.Phi0 = uo[2];
      hout.niter = niter;
      hout.fix_rounds = rounds;
    }
    ncur = (uint64_t)uo[3];
    nlist = n1;
    if (ncur >= (uint64_t)P.MINPART) {
      double r1[3];
      ncur = rvir_cut(c, n1, P, W, S, r1);
      if (threadIdx.x == 0) {
        hout.flags |= AHFGPU_HALO_RAN_RVIR1;
        hout.M_vir = r1[0]; hout.R_vir = r1[1]; hout.ovdens = r1[2];
      }
      __syncthreads();
      if (ncur >= (uint64_t)P.MINPART) profiles(c, n1, ncur, P, B, W, S, hout);
    }
  } else {
    nlist = c.n;
  }
  write_members(c, nlist, B, W, S);
  if (threadIdx.x == 0) {
    hout.npart = ncur;
    W.halo[h] = hout;
  }
  __syncthreads();
}

__global__ void __launch_bounds__(kT, 1) halo_fp64_kernel(DevParams P, DevBatch B, Work W, int single) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  HaloSmem& S = *reinterpret_cast<HaloSmem*>(smem_raw);
  uint4* stack = W.sort_stack + (uint64_t)blockIdx.x * W.stack_cap;
  if (single >= 0) {
    process_halo(single, P, B, W, S, stack);
    return;
  }
  while (true) {
    if (threadIdx.x == 0) S.bi[7] = (int)atomicAdd(W.queue_head, 1u);
    __syncthreads();
    int q = S.bi[7];
    __syncthreads();
    if (q >= W.nqueue) break;
    process_halo(W.queue[q], P, B, W, S, stack);
  }
}

// cNFW (src/libutility/specific.c:2041-2072) and cR1 (:1993-2018) of every
// halo whose profile pass ran: one thread per halo, after the halo kernels.
__global__ void concentration_kernel(ahfgpu_halo* halo, int64_t nh) {
  for (int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; h < nh; h += (int64_t)gridDim.x * blockDim.x) {
    ahfgpu_halo& o = halo[h];
    if (!(o.flags & AHFGPU_HALO_RAN_PROFILE)) continue;
    o.cNFW = calc_cNFW(o.V2_max, o.M_vir / o.R_vir);
    o.cR1 = calc_cR1(o.R1);
  }
}

void launch_concentration(ahfgpu_halo* halo, int64_t nh, int grid, cudaStream_t st) {
  concentration_kernel<<<grid, 128, 0, st>>>(halo, nh);
}

size_t fp64_smem_bytes() { return sizeof(HaloSmem); }

void launch_fp64(const DevParams& P, const DevBatch& B, const Work& W, int grid, int single, cudaStream_t st) {
  halo_fp64_kernel<<<grid, kT, sizeof(HaloSmem), st>>>(P, B, W, single);
}

int fp64_max_blocks_per_sm() {
  int nb = 0;
  cudaFuncSetAttribute(halo_fp64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(HaloSmem));
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, halo_fp64_kernel, kT, sizeof(HaloSmem));
  return nb;
}

}  // namespace ahfgpu
