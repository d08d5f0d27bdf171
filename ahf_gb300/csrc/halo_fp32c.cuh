// halo_fp32c.cuh -- FP32-compensated batched form of AHF's per-halo
// unbinding + property stage.
//
// One persistent grid; each CTA takes haloes from a largest-first queue and
// runs the whole per-halo sequence (src/libahf/ahf_halos_sfc.c:140-156):
//
//   keys     exact squared distances from 62-bit fixed-point offsets
//            (integer arithmetic only), normalised to a 64-bit monotone key
//            with a 56-bit mantissa; adjacent keys closer than 2^-47 relative
//            are re-ordered by the reference's own FP64 key
//            (ahf_halos.c:5816-5843) so the order equals the FP64 sort's.
//   sort     the shared bucket + shared-memory bitonic sort (sort.cuh)
//   rvir0    mass prefix, overdensity test, fused with the potential
//            integral of the first unbinding iteration
//   unbind   ONE pass per iteration: the potential prefix is a float-float
//            scan, the running bulk velocity is resolved tile by tile (the
//            recurrence is triangular, so each tile iterates its flags to a
//            fixpoint with the exact carry of the tiles before it), and the
//            same pass accumulates the next iteration's Phi0 and the rvir1
//            candidate.
//   profiles one pass of float-float scans; the per-bin rows and integral
//            properties use the FP64 finishing shared with the FP64 form.
//
// Every FP32 decision (overdensity cut, bound test, most-bound particle,
// rotation-curve and density maxima) carries a relative band; a particle
// inside it is re-tested in FP64 from its own input values and the
// float-float prefixes (n_retest).  If the FP64 re-test is itself inside the
// reference-rounding band, the halo is queued for the FP64 form, which
// resolves it in the reference's exact summation order.
#pragma once
#include <cstdint>
#include <cmath>

#include "common.cuh"
#include "ffloat.cuh"
#include "finish.cuh"
#include "sort.cuh"

namespace ahfgpu {

constexpr int kItems = 4;                 // consecutive slots per thread
constexpr double kEps64 = 1.1102230246251565e-16;
constexpr float kBand1 = 2e-5f;      // relative band of the FP32 decisions

template <class SS>
struct F32Smem {
  SS sort;
  float scan[32 * 2 * 16];
  int iscan[96];
  float lasth[32], lastl[32];
  double lastd[32];
  int lasti[32];
  double edge[kMaxBins];
  Bin bins[kMaxBins];
  double bd[32];
  long long bl[16];
  int bi[16];
  float bf[16];
};

struct Ctx32 {
  int h;
  uint64_t o, n;
  double cx, cy, cz;
  long long fx, fy, fz;    // centre in 2^-62 box units
};

// ---------------------------------------------------------------------------
// block-level primitives over thread totals (kT32 threads)

// exclusive scan of NC float-float channels; ex = sum over lower threads,
// tot = block total
template <int NC>
__device__ __noinline__ void bscan_ff(const ff (&v)[NC], ff (&ex)[NC], ff (&tot)[NC], float* sm) {
  const unsigned FULL = 0xffffffffu;
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  ff inc[NC];
#pragma unroll (NC <= 4 ? NC : 1)
  for (int c = 0; c < NC; c++) inc[c] = v[c];
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
#pragma unroll (NC <= 4 ? NC : 1)
    for (int c = 0; c < NC; c++) {
      ff y = {__shfl_up_sync(FULL, inc[c].hi, off), __shfl_up_sync(FULL, inc[c].lo, off)};
      if (lane >= off) inc[c] = ff_add(y, inc[c]);
    }
  }
  if (lane == 31) {
#pragma unroll (NC <= 4 ? NC : 1)
    for (int c = 0; c < NC; c++) { sm[(wid * NC + c) * 2] = inc[c].hi; sm[(wid * NC + c) * 2 + 1] = inc[c].lo; }
  }
  __syncthreads();
  if (wid == 0) {
#pragma unroll (NC <= 4 ? NC : 1)
    for (int c = 0; c < NC; c++) {
      ff t = lane < nw ? ff{sm[(lane * NC + c) * 2], sm[(lane * NC + c) * 2 + 1]} : ffz();
#pragma unroll
      for (int off = 1; off < 32; off <<= 1) {
        ff y = {__shfl_up_sync(FULL, t.hi, off), __shfl_up_sync(FULL, t.lo, off)};
        if (lane >= off) t = ff_add(y, t);
      }
      if (lane < nw) { sm[(lane * NC + c) * 2] = t.hi; sm[(lane * NC + c) * 2 + 1] = t.lo; }
    }
  }
  __syncthreads();
#pragma unroll (NC <= 4 ? NC : 1)
  for (int c = 0; c < NC; c++) {
    ff wp = wid > 0 ? ff{sm[((wid - 1) * NC + c) * 2], sm[((wid - 1) * NC + c) * 2 + 1]} : ffz();
    ff prev = {__shfl_up_sync(FULL, inc[c].hi, 1), __shfl_up_sync(FULL, inc[c].lo, 1)};
    ex[c] = lane > 0 ? ff_add(wp, prev) : wp;
    tot[c] = ff{sm[((nw - 1) * NC + c) * 2], sm[((nw - 1) * NC + c) * 2 + 1]};
  }
  __syncthreads();
}

// exclusive "last value" over threads: value of the nearest lower thread with
// has=true, else carry; any/last describe the whole block (last = carry when
// no thread has one)
template <class SM>
__device__ __forceinline__ ff blast_ff(bool has, ff val, ff carry, ff* last, SM& S) {
  const unsigned FULL = 0xffffffffu;
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  unsigned m = __ballot_sync(FULL, has);
  int lastlane = m ? (31 - __clz(m)) : 0;
  float wh = __shfl_sync(FULL, val.hi, lastlane), wl = __shfl_sync(FULL, val.lo, lastlane);
  if (lane == 0) { S.lasti[wid] = m ? 1 : 0; S.lasth[wid] = wh; S.lastl[wid] = wl; }
  __syncthreads();
  ff from_lower = carry;
  for (int w = wid - 1; w >= 0; w--)
    if (S.lasti[w]) { from_lower = ff{S.lasth[w], S.lastl[w]}; break; }
  unsigned below = m & ((1u << lane) - 1u);
  int src = below ? (31 - __clz(below)) : 0;
  ff mine = {__shfl_sync(FULL, val.hi, src), __shfl_sync(FULL, val.lo, src)};
  ff res = below ? mine : from_lower;
  ff l = carry;
  for (int w = nw - 1; w >= 0; w--)
    if (S.lasti[w]) { l = ff{S.lasth[w], S.lastl[w]}; break; }
  *last = l;
  __syncthreads();
  return res;
}

template <class SM>
__device__ __forceinline__ int bscan_int_ex(int v, int* tot, SM& S) {
  int t;
  int inc = block_scan_int(v, &t, S.iscan);
  *tot = t;
  return inc - v;
}

template <class SM>
__device__ __forceinline__ long long bmin_ll(long long v, SM& S) {
  for (int off = 16; off > 0; off >>= 1) {
    long long o = __shfl_xor_sync(0xffffffffu, v, off);
    v = o < v ? o : v;
  }
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (lane == 0) S.bl[wid & 7] = v;   // kT32/32 = 8 warps
  __syncthreads();
  long long r = S.bl[0];
  for (int w = 1; w < nw; w++) r = S.bl[w] < r ? S.bl[w] : r;
  __syncthreads();
  return r;
}

// ---------------------------------------------------------------------------
// fixed-point geometry

// float in [0,1) -> 2^-62 fixed point (exact for x >= 2^-38)
__device__ __forceinline__ long long fixp(float x) {
  unsigned b = __float_as_uint(x);
  int e = (int)((b >> 23) & 0xff);
  unsigned long long m = (b & 0x7fffffu) | (e ? 0x800000u : 0u);
  if (e == 0) e = 1;
  int sh = e - 88;
  return (long long)(sh >= 0 ? (m << sh) : (sh > -64 ? (m >> -sh) : 0ull));
}

__device__ __forceinline__ long long wrapfix(long long d) {
  const long long half = 1ll << 61, one = 1ll << 62;
  if (d > half) d -= one;
  if (d < -half) d += one;
  return d;
}

// 128-bit sum of squares -> monotone 64-bit key (exponent + 56-bit mantissa)
__device__ __forceinline__ uint64_t sqkey(long long dx, long long dy, long long dz) {
  unsigned long long a = (unsigned long long)(dx < 0 ? -dx : dx);
  unsigned long long b = (unsigned long long)(dy < 0 ? -dy : dy);
  unsigned long long c = (unsigned long long)(dz < 0 ? -dz : dz);
  unsigned long long lo = a * a, hi = __umul64hi(a, a);
  unsigned long long l2 = b * b, h2 = __umul64hi(b, b);
  unsigned long long t = lo + l2;
  hi += h2 + (t < lo);
  lo = t;
  l2 = c * c; h2 = __umul64hi(c, c);
  t = lo + l2;
  hi += h2 + (t < lo);
  lo = t;
  if (hi == 0 && lo == 0) return 0;
  int lz;
  unsigned long long m;
  int E;
  if (hi) {
    lz = __clzll(hi);
    m = lz ? ((hi << lz) | (lo >> (64 - lz))) : hi;
    E = 127 - lz;
  } else {
    lz = __clzll(lo);
    m = lo << lz;
    E = 63 - lz;
  }
  return ((unsigned long long)(E + 1) << 56) | ((m << 1) >> 8);
}

__device__ __forceinline__ float pow2f(int k) { return __int_as_float((k + 127) << 23); }

// key -> squared distance (box units^2) as float-float
__device__ __forceinline__ ff key_d2(uint64_t key) {
  if (key == 0) return ffz();
  int E = (int)(key >> 56) - 1;
  unsigned long long mant = (1ull << 56) | (key & ((1ull << 56) - 1));
  unsigned long long h24 = mant >> 33, l24 = (mant >> 9) & 0xffffffull;
  // value = mant * 2^(E-56) * 2^-124
  int eh = E - 56 - 124 + 33, el = E - 56 - 124 + 9;
  float hi = __fmul_rn((float)h24, pow2f(eh));
  float lo = el >= -126 ? __fmul_rn((float)l24, pow2f(el)) : 0.f;
  return ff_quick(hi, lo);
}

// the reference's FP64 squared distance of an entry (ahf_halos.c:5816-5843)
static __device__ __noinline__ double ref_key(const DevBatch& B, uint64_t e, double cx, double cy, double cz) {
  double dX = wrap_s((double)B.x[e] - cx);
  double dY = wrap_s((double)B.y[e] - cy);
  double dZ = wrap_s((double)B.z[e] - cz);
  return (dX * dX + dY * dY) + dZ * dZ;
}

// ---------------------------------------------------------------------------
static __device__ void keys32(const Ctx32& c, const DevBatch& B, const Work& W) {
  for (uint64_t i = threadIdx.x; i < c.n; i += blockDim.x) {
    uint64_t e = c.o + i;
    long long dx = wrapfix(fixp(B.x[e]) - c.fx);
    long long dy = wrapfix(fixp(B.y[e]) - c.fy);
    long long dz = wrapfix(fixp(B.z[e]) - c.fz);
    W.keyA[e] = sqkey(dx, dy, dz);
    W.idxA[e] = (uint32_t)i;
  }
  __syncthreads();
}

// Runs of adjacent keys closer than the reference's rounding are put in the
// order of the reference's FP64 keys (ties by slot).  Returns exact ties.
static __device__ __noinline__ unsigned long long fix_near_ties(const Ctx32& c, const DevBatch& B, const Work& W) {
  unsigned long long ties = 0;
  const uint64_t o = c.o;
  // mark ambiguous adjacent pairs first (flag is free until gather32)
  for (uint64_t i = threadIdx.x; i < c.n; i += blockDim.x)
    W.flag[o + i] = (i + 1 < c.n && W.keyA[o + i + 1] - W.keyA[o + i] <= 512ull) ? 1 : 0;
  __syncthreads();
  for (uint64_t i = threadIdx.x; i + 1 < c.n; i += blockDim.x) {
    if (!W.flag[o + i] || (i > 0 && W.flag[o + i - 1])) continue;
    // run [i, j] of mutually ambiguous neighbours, owned by this thread
    uint64_t j = i + 1;
    while (j + 1 < c.n && W.flag[o + j]) j++;
    // insertion sort of the run by (reference key, slot)
    for (uint64_t a = i + 1; a <= j; a++) {
      uint32_t sa = W.idxA[o + a];
      uint64_t ka = W.keyA[o + a];
      double ra = ref_key(B, o + sa, c.cx, c.cy, c.cz);
      uint64_t b = a;
      while (b > i) {
        uint32_t sb = W.idxA[o + b - 1];
        double rb = ref_key(B, o + sb, c.cx, c.cy, c.cz);
        if (rb < ra || (rb == ra && sb < sa)) break;
        W.idxA[o + b] = sb;
        W.keyA[o + b] = W.keyA[o + b - 1];
        b--;
      }
      W.idxA[o + b] = sa;
      W.keyA[o + b] = ka;
    }
    for (uint64_t a = i; a < j; a++) {
      double r0 = ref_key(B, o + W.idxA[o + a], c.cx, c.cy, c.cz);
      double r1 = ref_key(B, o + W.idxA[o + a + 1], c.cx, c.cy, c.cz);
      if (r0 == r1) ties++;
    }
  }
  __syncthreads();
  return ties;
}

static __device__ void gather32(const Ctx32& c, const DevBatch& B, const Work& W) {
  const float s62 = pow2f(-62);
  for (uint64_t i = threadIdx.x; i < c.n; i += blockDim.x) {
    uint64_t s = c.o + i;
    uint32_t j = W.idxA[s];
    uint64_t e = c.o + j;
    long long dx = wrapfix(fixp(B.x[e]) - c.fx);
    long long dy = wrapfix(fixp(B.y[e]) - c.fy);
    long long dz = wrapfix(fixp(B.z[e]) - c.fz);
    ff d = ff_sqrt(key_d2(sqkey(dx, dy, dz)));
    W.fdh[s] = d.hi;
    W.fdl[s] = d.lo;
    // offsets as float-float (hi kept for the FP32 arithmetic, lo for the
    // centre-of-mass sums)
    float hx = __ll2float_rn(dx), hy = __ll2float_rn(dy), hz = __ll2float_rn(dz);
    W.fdx[s] = __fmul_rn(hx, s62);
    W.fdy[s] = __fmul_rn(hy, s62);
    W.fdz[s] = __fmul_rn(hz, s62);
    W.fdxl[s] = __fmul_rn(__ll2float_rn(dx - __float2ll_rn(hx)), s62);
    W.fdyl[s] = __fmul_rn(__ll2float_rn(dy - __float2ll_rn(hy)), s62);
    W.fdzl[s] = __fmul_rn(__ll2float_rn(dz - __float2ll_rn(hz)), s62);
    W.svx[s] = B.vx[e];
    W.svy[s] = B.vy[e];
    W.svz[s] = B.vz[e];
    W.sw[s] = B.w ? B.w[e] : 1.0f;
    W.seid[s] = j;
    W.flag[s] = 1;
  }
  __syncthreads();
}

// exact reference distance of the entry in slot s (fabs form, ahf_halos.c:3381-3389)
static __device__ __noinline__ double ref_dist(const Ctx32& c, const DevBatch& B, const Work& W, uint64_t s) {
  uint64_t e = c.o + W.seid[s];
  return sqrt(ref_key(B, e, c.cx, c.cy, c.cz));
}

// d > MACHINE_ZERO in float-float (5e-16 = MZH + MZL exactly to ~2^-48)
__device__ __forceinline__ bool dpos(ff d) {
  const float MZH = 4.99999997e-16f;              // float nearest 5e-16
  const float MZL = 2.9753098e-24f;               // 5e-16 - MZH
  return d.hi > MZH || (d.hi == MZH && d.lo > MZL);
}

// potential-integral term of a member (ahf_halos.c:3398-3418)
static __device__ __noinline__ ff phi_term(ff M, float w, ff d, ff dp) {
  if (!dpos(d)) return ffz();
  ff Mp = ff_sub(M, fff(w));
  ff In = ff_div(M, ff_mul(d, d));
  ff Ip = dpos(dp) ? ff_div(Mp, ff_mul(dp, dp)) : ffz();
  ff Im = ff_mulf(ff_add(In, Ip), 0.5f);
  return ff_mul(Im, ff_sub(d, dp));
}

// FP32 overdensity test with band; FP64 re-test inside the band.  Returns
// fail (ovdens < ovlim).  M: mass prefix, d: distance (float-float).
static __device__ __noinline__ bool ov_fail(const Ctx32& c, const DevBatch& B, const Work& W, const DevParams& P,
                                        uint64_t s, ff M, ff d, unsigned* nret) {
  const float V43f = (float)(4. * kPi / 3.);
  float df = ff_f(d);
  float ov = __fdiv_rn(__fdiv_rn(ff_f(M), __fmul_rn(V43f, __fmul_rn(__fmul_rn(df, df), df))), P.f_rvrf);
  float lim = P.f_ovlim;
  if (isfinite(ov) && fabsf(ov - lim) <= kBand1 * lim) {
    (*nret)++;
    double R = ref_dist(c, B, W, s);
    double V = 4. * kPi / 3. * (R * R * R);
    double o64 = ff_d(M) / V * P.rho_fac / P.rho_vir;
    return !(o64 >= P.ovlim);
  }
  return !(ov >= lim);
}

// ---------------------------------------------------------------------------
// rem_outsideRvir(.,0) over all slots, fused with the potential prefix of
// the first unbinding iteration.  Returns n1; sets *Phi0 (float-float).
template <class SM>
static __device__ uint64_t rvir0_phi(const Ctx32& c, const DevBatch& B, const Work& W, const DevParams& P, SM& S,
                              ff* Phi0, double* mo, unsigned* nret) {
  ff cM = ffz(), cPhi = ffz();
  long long stop = -1;
  ff stopM = ffz(), stopD = ffz(), stopPhi = ffz();
  for (uint64_t base = 0; base < c.n; base += (uint64_t)blockDim.x * kItems) {
    uint64_t i0 = base + (uint64_t)threadIdx.x * kItems;
    float w[kItems];
    ff d[kItems], dp;
    ff locM[kItems];
    ff accM = ffz();
#pragma unroll
    for (int k = 0; k < kItems; k++) {
      uint64_t i = i0 + k;
      bool v = i < c.n;
      w[k] = v ? W.sw[c.o + i] : 0.f;
      d[k] = v ? ff{W.fdh[c.o + i], W.fdl[c.o + i]} : ffz();
      accM = ff_add(accM, fff(w[k]));
      locM[k] = accM;
    }
    dp = (i0 > 0 && i0 < c.n) ? ff{W.fdh[c.o + i0 - 1], W.fdl[c.o + i0 - 1]} : ffz();
    ff ex[1], tot[1];
    ff vv[1] = {accM};
    bscan_ff<1>(vv, ex, tot, S.scan);
    ff base_M = ff_add(cM, ex[0]);
    ff term[kItems], accT = ffz();
    ff Mk[kItems];
#pragma unroll
    for (int k = 0; k < kItems; k++) {
      uint64_t i = i0 + k;
      Mk[k] = ff_add(base_M, locM[k]);
      ff prevd = k == 0 ? dp : d[k - 1];
      term[k] = i < c.n ? phi_term(Mk[k], w[k], d[k], prevd) : ffz();
      accT = ff_add(accT, term[k]);
      term[k] = accT;     // thread-local inclusive
    }
    ff exT[1], totT[1];
    ff vt[1] = {accT};
    bscan_ff<1>(vt, exT, totT, S.scan);
    ff basePhi = ff_add(cPhi, exT[0]);
    long long myfail = 0x7fffffffffffffffll;
#pragma unroll
    for (int k = 0; k < kItems; k++) {
      uint64_t i = i0 + k;
      if (i < c.n && myfail == 0x7fffffffffffffffll) {
        if (ov_fail(c, B, W, P, c.o + i, Mk[k], d[k], nret)) myfail = (long long)i;
      }
    }
    long long f = bmin_ll(myfail, S);
    if (f != 0x7fffffffffffffffll) {
      if ((long long)i0 <= f && f < (long long)(i0 + kItems)) {
        int k = (int)(f - (long long)i0);
        ff phi = ff_add(basePhi, term[k]);
        S.bd[0] = ff_d(Mk[k]); S.bd[1] = ff_d(phi);
        S.bf[0] = Mk[k].hi; S.bf[1] = Mk[k].lo; S.bf[2] = d[k].hi; S.bf[3] = d[k].lo;
        S.bf[4] = phi.hi; S.bf[5] = phi.lo;
      }
      __syncthreads();
      stop = f;
      stopM = ff{S.bf[0], S.bf[1]}; stopD = ff{S.bf[2], S.bf[3]}; stopPhi = ff{S.bf[4], S.bf[5]};
      __syncthreads();
      break;
    }
    cM = ff_add(cM, tot[0]);
    cPhi = ff_add(cPhi, totT[0]);
  }
  uint64_t n1;
  if (stop < 0) {
    n1 = c.n;
    stopM = cM;
    stopPhi = cPhi;
    stopD = ff{W.fdh[c.o + c.n - 1], W.fdl[c.o + c.n - 1]};
  } else {
    n1 = (uint64_t)stop + 1;
  }
  // outputs in FP64 for the cut particle (as rem_outsideRvir computes them)
  double R = ref_dist(c, B, W, c.o + n1 - 1);
  double M = ff_d(stopM);
  double V = 4. * kPi / 3. * (R * R * R);
  mo[0] = M;
  mo[1] = R;
  mo[2] = M / V * P.rho_fac / P.rho_vir;
  *Phi0 = ff_add(stopPhi, ff_div(stopM, stopD));
  for (uint64_t i = n1 + threadIdx.x; i < c.n; i += blockDim.x) W.flag[c.o + i] = 0;
  __syncthreads();
  return n1;
}

// ---------------------------------------------------------------------------
// FP64 re-test of a bound decision (reference operation order, own inputs,
// prefixes from the float-float scans).  Sets *amb when the result is inside
// the reference's rounding band.
static __device__ __noinline__ bool retest_bound(const Ctx32& c, const DevBatch& B, const Work& W, const DevParams& P,
                                             uint64_t s, uint64_t pos, uint64_t n1, ff Phi, ff Phi0, ff VX,
                                             ff VY, ff VZ, ff Mv, float vmax, bool* amb) {
  uint64_t e = c.o + W.seid[s];
  double dX = wrap_s((double)B.x[e] - c.cx);
  double dY = wrap_s((double)B.y[e] - c.cy);
  double dZ = wrap_s((double)B.z[e] - c.cz);
  double d = sqrt((dX * dX + dY * dY) + dZ * dZ);
  double phi = ff_d(Phi), phi0 = ff_d(Phi0);
  double v_esc2 = d > kMachineZero ? (2 * fabs(phi - phi0) * P.phi_fac) : 1e30;
  double M_vel = ff_d(Mv);
  double VXp = (double)B.vx[e], VYp = (double)B.vy[e], VZp = (double)B.vz[e];
  double hx = P.Hubble * (dX) * P.r_fac, hy = P.Hubble * (dY) * P.r_fac, hz = P.Hubble * (dZ) * P.r_fac;
  double dVX = (VXp - ff_d(VX) / M_vel) * P.v_fac + hx;
  double dVY = (VYp - ff_d(VY) / M_vel) * P.v_fac + hy;
  double dVZ = (VZp - ff_d(VZ) / M_vel) * P.v_fac + hz;
  double vel2 = (dVX * dVX + dVY * dVY) + dVZ * dVZ;
  double thr = P.v2_tune * v_esc2;
  // band: the reference's sequential sums differ from exact ones by at most
  // ~(j+1)u of their absolute sums; the float-float prefixes by ~2^-40
  double g = 2.0 * ((double)pos + 64.0) * kEps64 + 9.1e-13;
  double gn = 2.0 * ((double)n1 + 64.0) * kEps64 + 9.1e-13;
  double A = fabs(phi - phi0);
  double dthr = d > kMachineZero ? thr * ((gn * fabs(phi0) * 2.0) / fmax(A, 1e-300) + 8 * kEps64) : thr * 8 * kEps64;
  double sb = (double)vmax * P.v_fac;
  double ddv = g * sb + 6.0 * kEps64 * (2.0 * sb + fabs(hx) + fabs(hy) + fabs(hz));
  double dvel2 = 2.0 * 1.7320508075688772 * sqrt(vel2) * ddv + 3.0 * ddv * ddv + 8 * kEps64 * vel2;
  if (fabs(vel2 - thr) <= 2.5 * (dthr + dvel2)) *amb = true;
  return !(vel2 > thr);
}

// ---------------------------------------------------------------------------
// One rem_unbound iteration (ahf_halos.c:3336-3601) in one pass over slots
// [0, n1) with members in flag bit0.  In: Phi0 of this iteration, seed slot.
// Out: flags bit0 <- bound; next-iteration Phi0; kept count/mass; last kept
// slot; the rvir1 candidate (first kept slot failing the overdensity test).
struct IterOut {
  long long nb;
  ff Mb, Phi0n;
  long long last_slot;
  long long rv_slot;   // first failing kept slot or -1
  ff rv_M, rv_d;
  int amb;             // needs the FP64 form
  int rounds;
};

template <class SM>
static __device__ void unbind_pass(const Ctx32& c, const DevBatch& B, const Work& W, const DevParams& P, SM& S,
                            uint64_t n1, ff Phi0, uint64_t js, float vmax, IterOut& out, unsigned* nret) {
  const uint64_t o = c.o;
  const float vf = (float)P.v_fac, Hr = (float)(P.Hubble * P.r_fac), v2t = (float)P.v2_tune;
  const float pf2 = (float)(2.0 * P.phi_fac);
  const float w0 = W.sw[o + js];
  // carries
  ff cM = ffz(), cPhi = ffz(), cD = ffz();
  ff cVX = two_prod(w0, W.svx[o + js]), cVY = two_prod(w0, W.svy[o + js]), cVZ = two_prod(w0, W.svz[o + js]);
  ff cMv = fff(w0);
  ff cMb = ffz(), cPhiN = ffz(), cDb = ffz();
  long long cNb = 0, last_slot = -1, rv = -1;
  ff rvM = ffz(), rvD = ffz();
  int amb_any = 0, maxr = 0;
  for (uint64_t base = 0; base < n1; base += (uint64_t)blockDim.x * kItems) {
    uint64_t i0 = base + (uint64_t)threadIdx.x * kItems;
    bool m[kItems];
    float w[kItems], vx[kItems], vy[kItems], vz[kItems], dx[kItems], dy[kItems], dz[kItems];
    ff d[kItems];
    bool any_m = false;
    ff lastm = ffz();
#pragma unroll
    for (int k = 0; k < kItems; k++) {
      uint64_t i = i0 + k;
      m[k] = i < n1 && (W.flag[o + i] & 1);
      w[k] = vx[k] = vy[k] = vz[k] = dx[k] = dy[k] = dz[k] = 0.f;
      d[k] = ffz();
      if (m[k]) {
        w[k] = W.sw[o + i];
        vx[k] = W.svx[o + i]; vy[k] = W.svy[o + i]; vz[k] = W.svz[o + i];
        dx[k] = W.fdx[o + i]; dy[k] = W.fdy[o + i]; dz[k] = W.fdz[o + i];
        d[k] = ff{W.fdh[o + i], W.fdl[o + i]};
        any_m = true;
        lastm = d[k];
      }
    }
    // member mass prefix, previous member distance, potential prefix
    ff accM = ffz(), locM[kItems];
#pragma unroll
    for (int k = 0; k < kItems; k++) { if (m[k]) accM = ff_add(accM, fff(w[k])); locM[k] = accM; }
    ff exM[1], totM[1], vM[1] = {accM};
    bscan_ff<1>(vM, exM, totM, S.scan);
    ff blockLast;
    ff dprev0 = blast_ff(any_m, lastm, cD, &blockLast, S);
    ff Mk[kItems], phi[kItems], accP = ffz();
    ff dp = dprev0;
#pragma unroll
    for (int k = 0; k < kItems; k++) {
      Mk[k] = ff_add(ff_add(cM, exM[0]), locM[k]);
      if (m[k]) {
        accP = ff_add(accP, phi_term(Mk[k], w[k], d[k], dp));
        dp = d[k];
      }
      phi[k] = accP;
    }
    ff exP[1], totP[1], vP[1] = {accP};
    bscan_ff<1>(vP, exP, totP, S.scan);
    float thr[kItems];
#pragma unroll
    for (int k = 0; k < kItems; k++) {
      phi[k] = ff_add(ff_add(cPhi, exP[0]), phi[k]);
      float A = fabsf(ff_f(ff_sub(phi[k], Phi0)));
      thr[k] = dpos(d[k]) ? __fmul_rn(v2t, __fmul_rn(pf2, A)) : __fmul_rn(v2t, 1e30f);
    }
    // tile fixpoint of the bound flags
    bool b[kItems];
#pragma unroll
    for (int k = 0; k < kItems; k++) b[k] = m[k];
    int rounds = 0;
    ff tVX, tVY, tVZ, tMv;
    bool amb_tile = false;
    while (true) {
      rounds++;
      ff ax = ffz(), ay = ffz(), az = ffz(), am = ffz();
      ff lx[kItems], ly[kItems], lz[kItems], lm[kItems];
#pragma unroll
      for (int k = 0; k < kItems; k++) {
        lx[k] = ax; ly[k] = ay; lz[k] = az; lm[k] = am;     // exclusive within thread
        if (b[k]) {
          ax = ff_add(ax, two_prod(w[k], vx[k]));
          ay = ff_add(ay, two_prod(w[k], vy[k]));
          az = ff_add(az, two_prod(w[k], vz[k]));
          am = ff_add(am, fff(w[k]));
        }
      }
      ff ex4[4], tot4[4], v4[4] = {ax, ay, az, am};
      bscan_ff<4>(v4, ex4, tot4, S.scan);
      tVX = tot4[0]; tVY = tot4[1]; tVZ = tot4[2]; tMv = tot4[3];
      int changed = 0;
#pragma unroll
      for (int k = 0; k < kItems; k++) {
        if (!m[k]) continue;
        ff VX = ff_add(ff_add(cVX, ex4[0]), lx[k]);
        ff VY = ff_add(ff_add(cVY, ex4[1]), ly[k]);
        ff VZ = ff_add(ff_add(cVZ, ex4[2]), lz[k]);
        ff Mv = ff_add(ff_add(cMv, ex4[3]), lm[k]);
        float mvf = ff_f(Mv);
        float bx = __fsub_rn(vx[k], __fdiv_rn(ff_f(VX), mvf));
        float by = __fsub_rn(vy[k], __fdiv_rn(ff_f(VY), mvf));
        float bz = __fsub_rn(vz[k], __fdiv_rn(ff_f(VZ), mvf));
        float dVX = __fadd_rn(__fmul_rn(bx, vf), __fmul_rn(Hr, dx[k]));
        float dVY = __fadd_rn(__fmul_rn(by, vf), __fmul_rn(Hr, dy[k]));
        float dVZ = __fadd_rn(__fmul_rn(bz, vf), __fmul_rn(Hr, dz[k]));
        float vel2 = __fadd_rn(__fadd_rn(__fmul_rn(dVX, dVX), __fmul_rn(dVY, dVY)), __fmul_rn(dVZ, dVZ));
        float margin = __fsub_rn(thr[k], vel2);
        bool nb;
        if (fabsf(margin) > kBand1 * fmaxf(thr[k], vel2) && isfinite(margin)) {
          nb = margin >= 0.f;
        } else {
          (*nret)++;
          bool amb = false;
          nb = retest_bound(c, B, W, P, o + i0 + k, i0 + k, n1, phi[k], Phi0, VX, VY, VZ, Mv, vmax, &amb);
          if (amb) amb_tile = true;
        }
        if (nb != b[k]) { b[k] = nb; changed = 1; }
      }
      if (!__syncthreads_or(changed)) break;
      if (rounds >= kMaxFixRounds) { amb_tile = true; break; }
    }
    if (rounds > maxr) maxr = rounds;
    amb_any |= __syncthreads_or(amb_tile ? 1 : 0);
    // next-iteration channels over the kept particles
    ff accB = ffz(), locB[kItems];
    bool any_b = false;
    ff lastb = ffz();
    int nbl = 0;
    long long lslot = -1;
#pragma unroll
    for (int k = 0; k < kItems; k++) {
      if (b[k]) { accB = ff_add(accB, fff(w[k])); any_b = true; lastb = d[k]; nbl++; lslot = (long long)(i0 + k); }
      locB[k] = accB;
    }
    ff exB[1], totB[1], vB[1] = {accB};
    bscan_ff<1>(vB, exB, totB, S.scan);
    ff blastB;
    ff dpb = blast_ff(any_b, lastb, cDb, &blastB, S);
    int tnb;
    bscan_int_ex(nbl, &tnb, S);
    ff accN = ffz();
    long long myfail = 0x7fffffffffffffffll;
    ff fM = ffz(), fD = ffz();
#pragma unroll
    for (int k = 0; k < kItems; k++) {
      if (!b[k]) continue;
      ff Mb = ff_add(ff_add(cMb, exB[0]), locB[k]);
      accN = ff_add(accN, phi_term(Mb, w[k], d[k], dpb));
      dpb = d[k];
      if (rv < 0 && myfail == 0x7fffffffffffffffll) {
        if (ov_fail(c, B, W, P, o + i0 + k, Mb, d[k], nret)) { myfail = (long long)(i0 + k); fM = Mb; fD = d[k]; }
      }
    }
    ff exN[1], totN[1], vN[1] = {accN};
    bscan_ff<1>(vN, exN, totN, S.scan);
    if (rv < 0) {
      long long f = bmin_ll(myfail, S);
      if (f != 0x7fffffffffffffffll) {
        if (myfail == f) { S.bf[0] = fM.hi; S.bf[1] = fM.lo; S.bf[2] = fD.hi; S.bf[3] = fD.lo; }
        __syncthreads();
        rv = f;
        rvM = ff{S.bf[0], S.bf[1]};
        rvD = ff{S.bf[2], S.bf[3]};
        __syncthreads();
      }
    }
    long long ls = -bmin_ll(-lslot, S);
    if (ls >= 0) last_slot = ls;
    // write flags
#pragma unroll
    for (int k = 0; k < kItems; k++) {
      uint64_t i = i0 + k;
      if (i < n1) W.flag[o + i] = (uint8_t)((m[k] ? 1 : 0) | (b[k] ? 2 : 0));
    }
    cM = ff_add(cM, totM[0]);
    cPhi = ff_add(cPhi, totP[0]);
    cD = blockLast;
    cVX = ff_add(cVX, tVX); cVY = ff_add(cVY, tVY); cVZ = ff_add(cVZ, tVZ); cMv = ff_add(cMv, tMv);
    cMb = ff_add(cMb, totB[0]);
    cPhiN = ff_add(cPhiN, totN[0]);
    cDb = blastB;
    cNb += tnb;
  }
  out.nb = cNb;
  out.Mb = cMb;
  out.Phi0n = cNb > 0 ? ff_add(cPhiN, ff_div(cMb, cDb)) : ffz();
  out.last_slot = last_slot;
  out.rv_slot = rv;
  out.rv_M = rvM;
  out.rv_d = rvD;
  out.amb = amb_any;
  out.rounds = maxr;
  __syncthreads();
}

// ---------------------------------------------------------------------------
// Warp-sequential prefix in exactly a C loop's order (one FP64 rounding per
// addition); see halo_fp64.cu.  incl: out[i] includes a[i].
static __device__ double chain64(const double* a, double* out, uint64_t n, double s0, int incl) {
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

// One rem_unbound iteration in the reference's exact summation order, for a
// pass whose FP64 re-test stayed inside the rounding band.  Members: flag
// bit0 of [0, n1); bit1 = speculated bound flags on entry, exact on exit.
// Per-member distances and offsets are recomputed in FP64 from the inputs
// exactly as the reference computes them; the order-dependent sums are warp
// chains.  Returns kept count/mass, last kept slot.
template <class SM>
static __device__ void exact_iter32(const Ctx32& c, const DevBatch& B, const Work& W, const DevParams& P, SM& S,
                             uint64_t n1, uint64_t js, long long* nb_out, double* mb_out, long long* last_out) {
  const uint64_t o = c.o;
  double* term = W.phi + o;
  double* d64 = W.prof_a + o;
  double* ax = W.prof_b + o;
  double* ay = W.prof_c + o;
  double* az = W.prof_d + o;
  double* dsm = reinterpret_cast<double*>(S.scan);
  double carryM = 0.0, carryD = 0.0;
  for (uint64_t base = 0; base < n1; base += blockDim.x) {
    uint64_t i = base + threadIdx.x;
    bool mem = i < n1 && (W.flag[o + i] & 1);
    double w = mem ? (double)W.sw[o + i] : 0.0;
    double d = mem ? ref_dist(c, B, W, o + i) : 0.0;
    if (i < n1) d64[i] = d;
    bool any;
    double lastd;
    double dprev = block_last_excl(mem, d, carryD, &any, &lastd, S.lastd, S.lasti);
    double v[1] = {w}, tot[1];
    block_scan<1>(v, tot, dsm);
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
    double s = chain64(term, term, n1, 0.0, 1);
    if (threadIdx.x == 0) S.bd[20] = s;
  }
  __syncthreads();
  const double Phi0 = S.bd[20] + carryM / carryD;
  const double w0 = (double)W.sw[o + js];
  const double sVX = w0 * (double)W.svx[o + js], sVY = w0 * (double)W.svy[o + js], sVZ = w0 * (double)W.svz[o + js];
  long long nb = 0, last = -1;
  double Mb = 0.0;
  int nwarps = blockDim.x >> 5;
  while (true) {
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
    if (nwarps >= 3) {
      if (warp == 0) chain64(ax, ax, n1, sVX, 0);
      else if (warp == 1) chain64(ay, ay, n1, sVY, 0);
      else if (warp == 2) chain64(az, az, n1, sVZ, 0);
    } else if (warp == 0) {
      chain64(ax, ax, n1, sVX, 0);
      chain64(ay, ay, n1, sVY, 0);
      chain64(az, az, n1, sVZ, 0);
    }
    __syncthreads();
    int changed = 0;
    double cMV = w0, cMb = 0.0;
    long long cNb = 0, cLast = -1;
    for (uint64_t base = 0; base < n1; base += blockDim.x) {
      uint64_t i = base + threadIdx.x;
      uint8_t f = i < n1 ? W.flag[o + i] : 0;
      bool mem = f & 1;
      bool b = mem && ((f >> 1) & 1);
      double w = mem ? (double)W.sw[o + i] : 0.0;
      double cw = b ? w : 0.0;
      double v[1] = {cw}, ex[1], tot[1];
      block_scan_excl<1>(v, ex, tot, dsm);
      if (mem) {
        double M_vel = cMV + ex[0];
        uint64_t e = o + W.seid[o + i];
        double dX = wrap_s((double)B.x[e] - c.cx), dY = wrap_s((double)B.y[e] - c.cy), dZ = wrap_s((double)B.z[e] - c.cz);
        double d = d64[i];
        double v_esc2 = d > kMachineZero ? (2 * fabs(term[i] - Phi0) * P.phi_fac) : 1e30;
        double VXp = (double)W.svx[o + i], VYp = (double)W.svy[o + i], VZp = (double)W.svz[o + i];
        double dVX = (VXp - ax[i] / M_vel) * P.v_fac + P.Hubble * (dX) * P.r_fac;
        double dVY = (VYp - ay[i] / M_vel) * P.v_fac + P.Hubble * (dY) * P.r_fac;
        double dVZ = (VZp - az[i] / M_vel) * P.v_fac + P.Hubble * (dZ) * P.r_fac;
        double vel2 = (dVX * dVX + dVY * dVY) + dVZ * dVZ;
        bool nbv = !(vel2 > P.v2_tune * v_esc2);
        if (nbv != b) changed = 1;
        W.flag[o + i] = (uint8_t)(1 | (nbv ? 2 : 0));
      }
      int tcnt;
      block_scan_int(b ? 1 : 0, &tcnt, S.iscan);
      unsigned bb = __ballot_sync(0xffffffffu, b);
      int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
      if (lane == 0) S.iscan[64 + wid] = bb ? (wid * 32 + 31 - __clz(bb)) : -1;
      __syncthreads();
      int lt = -1;
      for (int q = 0; q < nwarps; q++) lt = max(lt, S.iscan[64 + q]);
      __syncthreads();
      if (lt >= 0) cLast = (long long)(base + lt);
      cMb += tot[0];
      cMV += tot[0];
      cNb += tcnt;
    }
    if (!__syncthreads_or(changed)) {
      nb = cNb;
      Mb = cMb;
      last = cLast;
      break;
    }
  }
  if (threadIdx.x == 0) S.bd[21] = Phi0;
  __syncthreads();
  *nb_out = nb;
  *mb_out = Mb;
  *last_out = last;
}

// potential zero point Phi0 of the members in [0, n1) (the Phi0 pass,
// ahf_halos.c:3343-3426), float-float
template <class SM>
static __device__ ff phi0_pass32(const Ctx32& c, const Work& W, SM& S, uint64_t n1) {
  const uint64_t o = c.o;
  ff cM = ffz(), cPhi = ffz(), cD = ffz();
  for (uint64_t base = 0; base < n1; base += (uint64_t)blockDim.x * kItems) {
    uint64_t i0 = base + (uint64_t)threadIdx.x * kItems;
    bool m[kItems];
    float w[kItems];
    ff d[kItems];
    bool any = false;
    ff lastm = ffz();
    ff accM = ffz(), locM[kItems];
#pragma unroll
    for (int k = 0; k < kItems; k++) {
      uint64_t i = i0 + k;
      m[k] = i < n1 && (W.flag[o + i] & 1);
      w[k] = m[k] ? W.sw[o + i] : 0.f;
      d[k] = m[k] ? ff{W.fdh[o + i], W.fdl[o + i]} : ffz();
      if (m[k]) { accM = ff_add(accM, fff(w[k])); any = true; lastm = d[k]; }
      locM[k] = accM;
    }
    ff exM[1], totM[1], vM[1] = {accM};
    bscan_ff<1>(vM, exM, totM, S.scan);
    ff blockLast;
    ff dp = blast_ff(any, lastm, cD, &blockLast, S);
    ff accP = ffz();
#pragma unroll
    for (int k = 0; k < kItems; k++) {
      if (!m[k]) continue;
      accP = ff_add(accP, phi_term(ff_add(ff_add(cM, exM[0]), locM[k]), w[k], d[k], dp));
      dp = d[k];
    }
    ff exP[1], totP[1], vP[1] = {accP};
    bscan_ff<1>(vP, exP, totP, S.scan);
    cM = ff_add(cM, totM[0]);
    cPhi = ff_add(cPhi, totP[0]);
    cD = blockLast;
  }
  return ff_add(cPhi, ff_div(cM, cD));
}

// rem_outsideRvir(.,1) over the members of [0, n1): slot of the first member
// failing the overdensity test (-1: none) and the mass prefix there
template <class SM>
static __device__ long long rvir_pass32(const Ctx32& c, const DevBatch& B, const Work& W, const DevParams& P, SM& S,
                                 uint64_t n1, ff* Mfail, unsigned* nret) {
  const uint64_t o = c.o;
  ff cM = ffz();
  for (uint64_t base = 0; base < n1; base += (uint64_t)blockDim.x * kItems) {
    uint64_t i0 = base + (uint64_t)threadIdx.x * kItems;
    bool m[kItems];
    float w[kItems];
    ff accM = ffz(), locM[kItems];
#pragma unroll
    for (int k = 0; k < kItems; k++) {
      uint64_t i = i0 + k;
      m[k] = i < n1 && (W.flag[o + i] & 1);
      w[k] = m[k] ? W.sw[o + i] : 0.f;
      if (m[k]) accM = ff_add(accM, fff(w[k]));
      locM[k] = accM;
    }
    ff exM[1], totM[1], vM[1] = {accM};
    bscan_ff<1>(vM, exM, totM, S.scan);
    long long myfail = 0x7fffffffffffffffll;
    ff fM = ffz();
#pragma unroll
    for (int k = 0; k < kItems; k++) {
      if (!m[k] || myfail != 0x7fffffffffffffffll) continue;
      ff M = ff_add(ff_add(cM, exM[0]), locM[k]);
      if (ov_fail(c, B, W, P, o + i0 + k, M, ff{W.fdh[o + i0 + k], W.fdl[o + i0 + k]}, nret)) {
        myfail = (long long)(i0 + k);
        fM = M;
      }
    }
    long long f = bmin_ll(myfail, S);
    if (f != 0x7fffffffffffffffll) {
      if (myfail == f) { S.bf[0] = fM.hi; S.bf[1] = fM.lo; }
      __syncthreads();
      *Mfail = ff{S.bf[0], S.bf[1]};
      __syncthreads();
      return f;
    }
    cM = ff_add(cM, totM[0]);
  }
  *Mfail = cM;
  return -1;
}

// ---------------------------------------------------------------------------
// seed slot of the bulk velocity (ahf_halos.c:3441-3470)
template <class SM>
static __device__ uint64_t seed_slot(const Ctx32& c, const Work& W, const DevParams& P, int niter, uint64_t n1,
                              SM& S) {
  if (threadIdx.x == 0) {
    uint64_t js = 0;
    if (niter == 1) {
      uint64_t no_vbulk = (uint64_t)(P.MINPART / 2);
      float m2[64];
      uint32_t pos[64];
      uint64_t nv = no_vbulk < 64 ? no_vbulk : 64;
      for (uint64_t j = 0; j < nv; j++) {
        float mx = W.svx[c.o + j], my = W.svy[c.o + j], mz = W.svz[c.o + j];
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
      while (js < n1 && !(W.flag[c.o + js] & 1)) js++;
    }
    S.bl[8] = (long long)js;
  }
  __syncthreads();
  uint64_t r = (uint64_t)S.bl[8];
  __syncthreads();
  return r;
}

// ---------------------------------------------------------------------------
// smoothed maximum with an FP64 re-check of every FP32 candidate
// (find_max, src/libutility/general.c:608-650, on ranks nignore..n2-1)
static __device__ __noinline__ double raw64(const Ctx32& c, const DevBatch& B, const Work& W, const double* d64c, int which,
                        uint64_t r) {
  // which 0: dens_r2 (ahf_halos.c:4610-4616), 1: Vcirc2 (:4612)
  const float2* Mff = reinterpret_cast<const float2*>(W.prof_b + c.o);
  float2 mr = Mff[r];
  double M = (double)mr.x + (double)mr.y;
  double d = d64c[1];
  if (which == 1) return M / d;
  double dp = d64c[0];
  double Mp;
  if (r > 0) { float2 mp = Mff[r - 1]; Mp = (double)mp.x + (double)mp.y; } else Mp = 0.0;
  const double FPT = 4. * kPi / 3.;
  double dV = FPT * ((d * d * d) - (dp * dp * dp));
  double dM = M - Mp;
  double rm = (d + dp) / 2.;
  return dM / dV * (rm * rm);
}

static __device__ __noinline__ double rank_dist64(const Ctx32& c, const DevBatch& B, const Work& W, uint64_t r) {
  const uint32_t* ent = reinterpret_cast<const uint32_t*>(W.prof_d + c.o);
  return sqrt(ref_key(B, c.o + ent[r], c.cx, c.cy, c.cz));
}

// FP64 smoothed value at index i of the array y[j] = raw(j + kNignore),
// j in [0, m), after ns passes of smooth3
static __device__ __noinline__ double smooth_at64(const Ctx32& c, const DevBatch& B, const Work& W, int which, uint64_t m, int ns,
                              uint64_t i) {
  double lvl[8][8];
  long long lo = (long long)i - ns, hi = (long long)i + ns;
  if (lo < 0) lo = 0;
  if (hi > (long long)m - 1) hi = (long long)m - 1;
  int w = (int)(hi - lo + 1);
  for (int t = 0; t < w; t++) {
    uint64_t r = (uint64_t)(lo + t) + kNignore;
    double dd[2];
    dd[1] = rank_dist64(c, B, W, r);
    dd[0] = r > 0 ? rank_dist64(c, B, W, r - 1) : 0.0;
    lvl[0][t] = raw64(c, B, W, dd, which, r);
  }
  if (ns == 0 || m < 3) return lvl[0][i - lo];
  for (int p = 1; p <= ns; p++) {
    for (int t = 0; t < w; t++) {
      long long j = lo + t;
      double v;
      if (j == 0) v = (lvl[p - 1][t] + lvl[p - 1][t + 1]) / 2.;
      else if (j == (long long)m - 1) v = (lvl[p - 1][t] + lvl[p - 1][t - 1]) / 2.;
      else if (t == 0 || t == w - 1) v = 0.0;   // outside the window of i
      else v = (lvl[p - 1][t - 1] + lvl[p - 1][t] + lvl[p - 1][t + 1]) / 3.;
      lvl[p][t] = v;
    }
    // the window shrinks by one per pass except at array ends
  }
  return lvl[ns][i - lo];
}

template <class SM>
static __device__ uint64_t find_max32(const Ctx32& c, const DevBatch& B, const Work& W, SM& S, int which, int ns,
                               uint64_t n2, unsigned* nret) {
  uint64_t m = n2 - kNignore;
  float* y = reinterpret_cast<float*>(W.prof_c + c.o) + (which ? 0 : n2);
  float* t0 = reinterpret_cast<float*>(W.phi + c.o);
  float* t1 = t0 + n2;
  // y holds raw FP32 values at ranks; smooth a copy of [nignore, n2)
  for (uint64_t i = threadIdx.x; i < m; i += blockDim.x) t0[i] = y[kNignore + i];
  __syncthreads();
  float* cur = t0;
  float* nxt = t1;
  if (ns > 0 && m >= 3) {
    for (int p = 0; p < ns; p++) {
      for (uint64_t i = threadIdx.x; i < m; i += blockDim.x) {
        float r;
        if (i == 0) r = __fdiv_rn(__fadd_rn(cur[0], cur[1]), 2.f);
        else if (i == m - 1) r = __fdiv_rn(__fadd_rn(cur[m - 1], cur[m - 2]), 2.f);
        else r = __fdiv_rn(__fadd_rn(__fadd_rn(cur[i - 1], cur[i]), cur[i + 1]), 3.f);
        nxt[i] = r;
      }
      __syncthreads();
      float* sw = cur; cur = nxt; nxt = sw;
    }
  }
  // FP32 maximum over [0, m-2]
  float best = -10.f;
  for (uint64_t i = threadIdx.x; i + 1 < m; i += blockDim.x) best = fmaxf(best, isnan(cur[i]) ? -10.f : cur[i]);
  for (int off = 16; off > 0; off >>= 1) best = fmaxf(best, __shfl_xor_sync(0xffffffffu, best, off));
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (lane == 0) S.bf[wid] = best;
  __syncthreads();
  float B32 = -10.f;
  for (int w = 0; w < nw; w++) B32 = fmaxf(B32, S.bf[w]);
  __syncthreads();
  // candidates: within 1e-4 of the FP32 maximum -> FP64 smoothed value
  float thr = isinf(B32) ? B32 : B32 - 1e-4f * fabsf(B32) - 1e-30f;
  double bv = -10.0;
  long long bi = -1;
  for (uint64_t i = threadIdx.x; i + 1 < m; i += blockDim.x) {
    float v = cur[i];
    if (!(v >= thr)) continue;
    (*nret)++;
    double v64 = smooth_at64(c, B, W, which, m, ns, i);
    if (bi < 0 || v64 > bv) { bv = v64; bi = (long long)i; }
  }
  for (int off = 16; off > 0; off >>= 1) {
    double ov = __shfl_xor_sync(0xffffffffu, bv, off);
    long long oi = __shfl_xor_sync(0xffffffffu, bi, off);
    bool take = oi >= 0 && (bi < 0 || ov > bv || (ov == bv && oi < bi));
    if (take) { bv = ov; bi = oi; }
  }
  if (lane == 0) { S.bd[wid] = bv; S.bl[wid & 7] = bi; }
  __syncthreads();
  double BV = -10.0;
  long long BI = -1;
  for (int w = 0; w < nw; w++) {
    double ov = S.bd[w];
    long long oi = S.bl[w];
    bool take = oi >= 0 && (BI < 0 || ov > BV || (ov == BV && oi < BI));
    if (take) { BV = ov; BI = oi; }
  }
  __syncthreads();
  return BI < 0 || !(BV > -10.0) ? m - 1 : (uint64_t)BI;
}

// HaloProfiles per-particle terms (ahf_halos.c:4320-4420): 0 potential
// integral, 1-3 angular momentum, 4 kinetic T, 5-7 centre of mass, 8-13
// inertia tensor, 14/15 high/low resolution mass.  VX.. are the momentum
// prefixes INCLUDING the particle (the reference updates VXc first).
static __device__ __noinline__ void prof_terms(const DevParams& P, float w, float vx, float vy, float vz, float dx,
                                           float dy, float dz, float dxl, float dyl, float dzl, ff d, ff dp, ff M,
                                           ff VX, ff VY, ff VZ, ff cxf, ff cyf, ff czf, float Hrv, ff (&tm)[16],
                                           float* Tout) {
  // velocity relative to the running bulk velocity, float-float
  ff gX = ff_sub(fff(vx), ff_div(VX, M));
  ff gY = ff_sub(fff(vy), ff_div(VY, M));
  ff gZ = ff_sub(fff(vz), ff_div(VZ, M));
  float dVX = ff_f(gX), dVY = ff_f(gY), dVZ = ff_f(gZ);
  tm[0] = phi_term(M, w, d, dp);
  tm[1] = two_prod(w, __fsub_rn(__fmul_rn(dy, dVZ), __fmul_rn(dz, dVY)));
  tm[2] = two_prod(w, __fsub_rn(__fmul_rn(dz, dVX), __fmul_rn(dx, dVZ)));
  tm[3] = two_prod(w, __fsub_rn(__fmul_rn(dx, dVY), __fmul_rn(dy, dVX)));
  // Hubble drag, then the kinetic term (float-float: Ekin + Epot cancels in
  // lambdaE)
  gX = ff_add(gX, ff_mulf(two_sum(dx, dxl), Hrv));
  gY = ff_add(gY, ff_mulf(two_sum(dy, dyl), Hrv));
  gZ = ff_add(gZ, ff_mulf(two_sum(dz, dzl), Hrv));
  ff T = ff_mulf(ff_add(ff_add(ff_mul(gX, gX), ff_mul(gY, gY)), ff_mul(gZ, gZ)), w);
  *Tout = ff_f(T);
  tm[4] = T;
  tm[5] = ff_mulf(ff_add(cxf, two_sum(dx, dxl)), w);
  tm[6] = ff_mulf(ff_add(cyf, two_sum(dy, dyl)), w);
  tm[7] = ff_mulf(ff_add(czf, two_sum(dz, dzl)), w);
  tm[8] = two_prod(__fmul_rn(w, dx), dx);
  tm[9] = two_prod(__fmul_rn(w, dy), dy);
  tm[10] = two_prod(__fmul_rn(w, dz), dz);
  tm[11] = two_prod(__fmul_rn(w, dx), dy);
  tm[12] = two_prod(__fmul_rn(w, dx), dz);
  tm[13] = two_prod(__fmul_rn(w, dy), dz);
  tm[14] = ffz();
  tm[15] = ffz();
  if (P.has_w) {
    if (fabsf(w - 1.0f) < (float)kZero) tm[14] = fff(w);
    else if (w > 1.0f) tm[15] = fff(w);
  } else {
    tm[14] = fff(w);
  }
}

// ---------------------------------------------------------------------------
// HaloProfiles (ahf_halos.c:3961-5261) over the n2 members of [0, n1)
template <class SM>
static __device__ void profiles32(const Ctx32& c, const DevBatch& B, const Work& W, const DevParams& P, SM& S,
                           uint64_t n1, uint64_t n2, ff Phi0, ahfgpu_halo& hout, unsigned* nret) {
  const uint64_t o = c.o;
  const double FPT = 4. * kPi / 3.;
  float2* Rff = reinterpret_cast<float2*>(W.prof_a + o);   // radius (float-float) per rank
  float2* Mff = reinterpret_cast<float2*>(W.prof_b + o);   // mass prefix per rank
  float* vc2 = reinterpret_cast<float*>(W.prof_c + o);     // Vcirc2 per rank
  float* dr2 = vc2 + n2;                                   // dens_r2 per rank
  uint32_t* ent = reinterpret_cast<uint32_t*>(W.prof_d + o);
  // ranks -> distances (binning_parameter needs them)
  {
    int carry = 0;
    for (uint64_t base = 0; base < n1; base += blockDim.x) {
      uint64_t i = base + threadIdx.x;
      bool mem = i < n1 && (W.flag[o + i] & 1);
      int tot;
      int r = block_scan_int(mem ? 1 : 0, &tot, S.iscan) - 1 + carry;
      if (mem) {
        Rff[r] = make_float2(W.fdh[o + i], W.fdl[o + i]);
        ent[r] = W.seid[o + i];
      }
      carry += tot;
    }
    __syncthreads();
  }
  // binning_parameter, src/libutility/specific.c:259-322 (exact distances)
  if (threadIdx.x == 0) {
    int nb = (int)(6.2 * (log10((double)n2)) - 3.5);
    if (nb < 2) nb = 2;
    if (nb > kMaxBins) nb = kMaxBins;
    long np = (long)floor(((double)P.MINPART / 10.) + 0.5);
    double dmin = -1.0;
    while (np < (long)n2 - 1 && dmin < kMachineZero) { dmin = rank_dist64(c, B, W, (uint64_t)np); np++; }
    double dmax = rank_dist64(c, B, W, n2 - 1);
    if (dmin < kMachineZero) dmin = dmax / 2.;
    double ld0 = log10(dmin), ld1 = log10(dmax);
    S.bd[2] = ld0;
    S.bd[3] = (ld1 - ld0) / (double)nb;
    S.bd[1] = dmax;
    S.bi[0] = nb;
  }
  __syncthreads();
  for (int b = threadIdx.x; b < S.bi[0]; b += blockDim.x)
    S.edge[b] = b == S.bi[0] - 1 ? S.bd[1] + kZero : pow(10., S.bd[2] + ((double)b + 1) * S.bd[3]);
  __syncthreads();
  const int nbins = S.bi[0];
  const float vf = (float)P.v_fac;
  const float Hrv = (float)(P.Hubble * P.r_fac / P.v_fac);
  const double cxd = c.cx, cyd = c.cy, czd = c.cz;
  const ff cxf = ff_from_d(cxd), cyf = ff_from_d(cyd), czf = ff_from_d(czd);
  ff c1[4] = {ffz(), ffz(), ffz(), ffz()};          // M, VX, VY, VZ
  ff c2[16];
#pragma unroll
  for (int k = 0; k < 16; k++) c2[k] = ffz();        // phi, Lx,Ly,Lz, T, CoMx..z, a11..a23, Mhi, Mlo
  ff cU = ffz(), cD = ffz();
  int cr = 0;
  double Ebest = 1e30;
  long long Eslot = -1;
  for (uint64_t base = 0; base < n1; base += (uint64_t)blockDim.x * kItems) {
    uint64_t i0 = base + (uint64_t)threadIdx.x * kItems;
    bool m[kItems];
    float w[kItems], vx[kItems], vy[kItems], vz[kItems], dx[kItems], dy[kItems], dz[kItems];
    float dxl[kItems], dyl[kItems], dzl[kItems];
    ff d[kItems];
    int nm = 0;
    bool any = false;
    ff lastm = ffz();
#pragma unroll
    for (int k = 0; k < kItems; k++) {
      uint64_t i = i0 + k;
      m[k] = i < n1 && (W.flag[o + i] & 1);
      w[k] = vx[k] = vy[k] = vz[k] = dx[k] = dy[k] = dz[k] = 0.f;
      dxl[k] = dyl[k] = dzl[k] = 0.f;
      d[k] = ffz();
      if (m[k]) {
        w[k] = W.sw[o + i];
        vx[k] = W.svx[o + i]; vy[k] = W.svy[o + i]; vz[k] = W.svz[o + i];
        dx[k] = W.fdx[o + i]; dy[k] = W.fdy[o + i]; dz[k] = W.fdz[o + i];
        dxl[k] = W.fdxl[o + i]; dyl[k] = W.fdyl[o + i]; dzl[k] = W.fdzl[o + i];
        d[k] = ff{W.fdh[o + i], W.fdl[o + i]};
        nm++; any = true; lastm = d[k];
      }
    }
    int tn;
    int rank0 = bscan_int_ex(nm, &tn, S) + cr;
    ff blockLast;
    ff dp0 = blast_ff(any, lastm, cD, &blockLast, S);
    // scan 1: mass and momentum prefixes (inclusive, include the particle)
    ff a1[4] = {ffz(), ffz(), ffz(), ffz()}, l1[kItems][4];
#pragma unroll
    for (int k = 0; k < kItems; k++) {
      if (m[k]) {
        a1[0] = ff_add(a1[0], fff(w[k]));
        a1[1] = ff_add(a1[1], two_prod(w[k], vx[k]));
        a1[2] = ff_add(a1[2], two_prod(w[k], vy[k]));
        a1[3] = ff_add(a1[3], two_prod(w[k], vz[k]));
      }
#pragma unroll
      for (int q = 0; q < 4; q++) l1[k][q] = a1[q];
    }
    ff e1[4], t1[4];
    bscan_ff<4>(a1, e1, t1, S.scan);
    // per-particle terms (thread totals); per-item phi terms kept for U
    ff a2[16];
#pragma unroll
    for (int q = 0; q < 16; q++) a2[q] = ffz();
    float Tp[kItems];
    ff pt[kItems];
    ff Mr[kItems];
    {
      ff dp = dp0;
      int r = rank0;
#pragma unroll
      for (int k = 0; k < kItems; k++) {
        Tp[k] = 0.f;
        pt[k] = ffz();
        ff M = ff_add(ff_add(c1[0], e1[0]), l1[k][0]);
        Mr[k] = M;
        if (!m[k]) continue;
        ff tm[16];
        prof_terms(P, w[k], vx[k], vy[k], vz[k], dx[k], dy[k], dz[k], dxl[k], dyl[k], dzl[k], d[k], dp, M,
                   ff_add(ff_add(c1[1], e1[1]), l1[k][1]), ff_add(ff_add(c1[2], e1[2]), l1[k][2]),
                   ff_add(ff_add(c1[3], e1[3]), l1[k][3]), cxf, cyf, czf, Hrv, tm, &Tp[k]);
#pragma unroll
        for (int q = 0; q < 16; q++) a2[q] = ff_add(a2[q], tm[q]);
        pt[k] = tm[0];
        // per-rank arrays (ahf_halos.c:4598-4616)
        Mff[r] = make_float2(M.hi, M.lo);
        float df = ff_f(d[k]);
        vc2[r] = __fdiv_rn(ff_f(M), df);
        ff d3 = ff_mul(ff_mul(d[k], d[k]), d[k]);
        ff p3 = ff_mul(ff_mul(dp, dp), dp);
        float dV = __fmul_rn((float)FPT, ff_f(ff_sub(d3, p3)));
        float rm = __fmul_rn(__fadd_rn(df, ff_f(dp)), 0.5f);
        dr2[r] = __fmul_rn(__fdiv_rn(w[k], dV), __fmul_rn(rm, rm));
        dp = d[k];
        r++;
      }
    }
    ff e2[16], t2[16];
    bscan_ff<16>(a2, e2, t2, S.scan);
    // potential energy and most-bound candidates
    ff phi[kItems], aU = ffz(), lU[kItems];
    float Ef[kItems];
    ff runp = ffz();
#pragma unroll
    for (int k = 0; k < kItems; k++) {
      runp = ff_add(runp, pt[k]);
      phi[k] = ff_add(ff_add(c2[0], e2[0]), runp);
      Ef[k] = 3.0e38f;
      if (m[k]) {
        ff U = ff_mulf(ff_sub(phi[k], Phi0), w[k]);
        aU = ff_add(aU, U);
        Ef[k] = __fadd_rn(__fmul_rn(0.5f, Tp[k]), ff_f(U));
      }
      lU[k] = aU;
    }
    ff eU[1], tU[1], vU[1] = {aU};
    bscan_ff<1>(vU, eU, tU, S.scan);
    // most bound particle: FP32 screen, FP64 decision
    float emin = 3.0e38f;
#pragma unroll
    for (int k = 0; k < kItems; k++) emin = fminf(emin, Ef[k]);
    for (int off = 16; off > 0; off >>= 1) emin = fminf(emin, __shfl_xor_sync(0xffffffffu, emin, off));
    {
      int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
      if (lane == 0) S.bf[wid] = emin;
      __syncthreads();
      float tmin = 3.0e38f;
      for (int q = 0; q < nw; q++) tmin = fminf(tmin, S.bf[q]);
      __syncthreads();
      float ref = fminf(tmin, (float)Ebest);
      float cut = ref + 1e-4f * fabsf(ref) + 1e-30f;
      double bE = 1e300;
      long long bs = -1;
#pragma unroll
      for (int k = 0; k < kItems; k++) {
        if (!m[k] || !(Ef[k] <= cut)) continue;
        (*nret)++;
        uint64_t e = o + W.seid[o + i0 + k];
        double dX = wrap_s((double)B.x[e] - cxd), dY = wrap_s((double)B.y[e] - cyd), dZ = wrap_s((double)B.z[e] - czd);
        ff M = Mr[k];
        double Md = ff_d(M);
        ff VX = ff_add(ff_add(c1[1], e1[1]), l1[k][1]);
        ff VY = ff_add(ff_add(c1[2], e1[2]), l1[k][2]);
        ff VZ = ff_add(ff_add(c1[3], e1[3]), l1[k][3]);
        double dVX = ((double)B.vx[e] - ff_d(VX) / Md), dVY = ((double)B.vy[e] - ff_d(VY) / Md),
               dVZ = ((double)B.vz[e] - ff_d(VZ) / Md);
        dVX += P.Hubble * dX * P.r_fac / P.v_fac;
        dVY += P.Hubble * dY * P.r_fac / P.v_fac;
        dVZ += P.Hubble * dZ * P.r_fac / P.v_fac;
        double wk = (double)w[k];
        double Tpart = wk * ((dVX * dVX + dVY * dVY) + dVZ * dVZ);
        double Upart = (ff_d(phi[k]) - ff_d(Phi0)) * wk;
        double E = 0.5 * Tpart + Upart;
        if (E < bE) { bE = E; bs = (long long)(i0 + k); }
      }
      for (int off = 16; off > 0; off >>= 1) {
        double oE = __shfl_xor_sync(0xffffffffu, bE, off);
        long long oi = __shfl_xor_sync(0xffffffffu, bs, off);
        bool take = oi >= 0 && (bs < 0 || oE < bE || (oE == bE && oi < bs));
        if (take) { bE = oE; bs = oi; }
      }
      if (lane == 0) { S.bd[wid] = bE; S.bl[wid & 7] = bs; }
      __syncthreads();
      double TE = 1e300;
      long long TS = -1;
      for (int q = 0; q < nw; q++) {
        double oE = S.bd[q];
        long long oi = S.bl[q];
        bool take = oi >= 0 && (TS < 0 || oE < TE || (oE == TE && oi < TS));
        if (take) { TE = oE; TS = oi; }
      }
      __syncthreads();
      if (TS >= 0 && TE < Ebest) { Ebest = TE; Eslot = TS; }
    }
    // bin records at bin ends
    {
      ff dpk = dp0;
      int r = rank0;
#pragma unroll
      for (int k = 0; k < kItems; k++) {
        if (!m[k]) continue;
        double dpd = ff_d(dpk), dd = ff_d(d[k]);
        int bcur = 0;
        if (r > 0) { while (bcur < nbins && !(dpd < S.edge[bcur])) bcur++; }
        int bnext = 0;
        while (bnext < nbins && !(dd < S.edge[bnext])) bnext++;
        bool last = (uint64_t)(r + 1) == n2;
        int bend = last ? nbins : bnext;
        if (bend > bcur) {
          ff Mk = ff_add(ff_add(c1[0], e1[0]), l1[k][0]);
          // cumulative channels at this item: recompute the terms of items <= k
          ff run[16];
#pragma unroll
          for (int q = 0; q < 16; q++) run[q] = ff_add(c2[q], e2[q]);
          {
            ff dq = dp0;
            for (int kk = 0; kk <= k; kk++) {
              if (!m[kk]) continue;
              ff tm[16];
              float tdummy;
              prof_terms(P, w[kk], vx[kk], vy[kk], vz[kk], dx[kk], dy[kk], dz[kk], dxl[kk], dyl[kk], dzl[kk], d[kk],
                         dq, Mr[kk],
                         ff_add(ff_add(c1[1], e1[1]), l1[kk][1]), ff_add(ff_add(c1[2], e1[2]), l1[kk][2]),
                         ff_add(ff_add(c1[3], e1[3]), l1[kk][3]), cxf, cyf, czf, Hrv, tm, &tdummy);
              for (int q = 0; q < 16; q++) run[q] = ff_add(run[q], tm[q]);
              dq = d[kk];
            }
          }
          double Phid = ff_d(phi[k]);
          double Upart = (Phid - ff_d(Phi0)) * (double)w[k];
          ff Uc = ff_add(ff_add(cU, eU[0]), lU[k]);
          for (int b = bcur; b < bend; b++) {
            Bin& R = S.bins[b];
            R.npart = (double)(r + 1);
            R.M = ff_d(Mk);
            R.Lx = ff_d(run[1]);
            R.Ly = ff_d(run[2]);
            R.Lz = ff_d(run[3]);
            R.T = ff_d(run[4]);
            R.U = ff_d(Uc);
            R.a11 = ff_d(run[8]);
            R.a22 = ff_d(run[9]);
            R.a33 = ff_d(run[10]);
            R.a12 = ff_d(run[11]);
            R.a13 = ff_d(run[12]);
            R.a23 = ff_d(run[13]);
            R.vesc2 = 2 * fabs(Upart) / (double)w[k];
          }
        }
        dpk = d[k];
        r++;
      }
    }
#pragma unroll
    for (int q = 0; q < 4; q++) c1[q] = ff_add(c1[q], t1[q]);
#pragma unroll
    for (int q = 0; q < 16; q++) c2[q] = ff_add(c2[q], t2[q]);
    cU = ff_add(cU, tU[0]);
    cD = blockLast;
    cr += tn;
    __syncthreads();
  }
  double* rows = W.prof_stage + W.prof_cap_off[c.h] * AHFGPU_PROF_NFIELDS;
  write_bin_rows(S.bins, S.edge, nbins, rows);
  __syncthreads();
  uint64_t i_r2 = find_max32(c, B, W, S, 0, 3, n2, nret);
  uint64_t i_rm = find_max32(c, B, W, S, 1, 1, n2, nret);
  if (threadIdx.x == 0) {
    double r2 = rank_dist64(c, B, W, kNignore + i_r2);
    double x_max = rank_dist64(c, B, W, kNignore + i_rm);
    double R_max = x_max;
    uint64_t lo = 0, hi = n2 - 1;
    while (lo < hi) {
      uint64_t mid = (lo + hi) / 2;
      if (rank_dist64(c, B, W, mid) < x_max) lo = mid + 1; else hi = mid;
    }
    uint64_t ib = lo;
    double rb = rank_dist64(c, B, W, ib);
    float2 mb = Mff[ib];
    double Mb = (double)mb.x + (double)mb.y;
    double ovd = Mb / (FPT * (rb * rb * rb));
    double M_max = ovd * FPT * (rb * rb * rb);
    double V_max = M_max / R_max;
    long long mbe = Eslot >= 0 ? (long long)(o + W.seid[o + Eslot]) : -1;
    finish_scalars(rows, nbins, ff_d(c1[0]), ff_d(c1[1]), ff_d(c1[2]), ff_d(c1[3]), ff_d(c2[5]), ff_d(c2[6]),
                   ff_d(c2[7]), ff_d(c2[14]), ff_d(c2[15]), mbe, r2, R_max, V_max, P, B, c.cx, c.cy, c.cz, hout);
    hout.nbins = nbins;
    hout.flags |= AHFGPU_HALO_RAN_PROFILE;
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
static __device__ void write_members32(const Ctx32& c, uint64_t nlist, const DevBatch& B, const Work& W) {
  int carry = 0;
  __shared__ int isc[64];
  for (uint64_t base = 0; base < nlist; base += blockDim.x) {
    uint64_t i = base + threadIdx.x;
    bool mem = i < nlist && (W.flag[c.o + i] & 1);
    int tot;
    int r = block_scan_int(mem ? 1 : 0, &tot, isc) - 1 + carry;
    if (mem) {
      uint64_t e = c.o + W.seid[c.o + i];
      W.mem_stage[c.o + r] = B.gidx ? B.gidx[e] : e;
    }
    carry += tot;
  }
  __syncthreads();
}

template <class SM>
static __device__ void process_halo32(int h, const DevParams& P, const DevBatch& B, const Work& W, SM& S,
                               uint4* stack) {
  Ctx32 c;
  c.h = h;
  c.o = B.off[h];
  c.n = B.off[h + 1] - c.o;
  c.cx = B.cx[h]; c.cy = B.cy[h]; c.cz = B.cz[h];
  c.fx = llrint(c.cx * 4611686018427387904.0);   // 2^62
  c.fy = llrint(c.cy * 4611686018427387904.0);
  c.fz = llrint(c.cz * 4611686018427387904.0);
  __shared__ ahfgpu_halo hout;
  __shared__ unsigned nret_s;
  if (threadIdx.x == 0) {
    char* p = (char*)&hout;
    for (unsigned k = 0; k < sizeof(ahfgpu_halo); k++) p[k] = 0;
    nret_s = 0;
  }
  __syncthreads();
  unsigned nret = 0;
  if (c.n == 0) {
    if (threadIdx.x == 0) { hout.flags = AHFGPU_HALO_EMPTY; W.halo[h] = hout; }
    __syncthreads();
    return;
  }
  if (c.n < (uint64_t)P.MINPART) {
    for (uint64_t i = threadIdx.x; i < c.n; i += blockDim.x) {
      uint64_t e = c.o + i;
      W.mem_stage[e] = B.gidx ? B.gidx[e] : e;
    }
    if (threadIdx.x == 0) { hout.npart = c.n; W.halo[h] = hout; }
    __syncthreads();
    return;
  }
  keys32(c, B, W);
  bool ok = radial_sort(W.keyA, W.idxA, W.keyB, W.idxB, c.o, c.n, stack, W.stack_cap, S.sort);
  if (!ok) {
    if (threadIdx.x == 0) { atomicExch(W.err, kErrWorklist); W.halo[h] = hout; }
    __syncthreads();
    return;
  }
  unsigned long long ties = fix_near_ties(c, B, W);
  gather32(c, B, W);
  // max |v| component (FP64 band of the re-test)
  float vm = 0.f;
  for (uint64_t i = threadIdx.x; i < c.n; i += blockDim.x)
    vm = fmaxf(vm, fmaxf(fabsf(W.svx[c.o + i]), fmaxf(fabsf(W.svy[c.o + i]), fabsf(W.svz[c.o + i]))));
  for (int off = 16; off > 0; off >>= 1) vm = fmaxf(vm, __shfl_xor_sync(0xffffffffu, vm, off));
  if ((threadIdx.x & 31) == 0) S.bf[8 + (threadIdx.x >> 5)] = vm;
  __syncthreads();
  float vmax = 0.f;
  for (int w = 0; w < (int)(blockDim.x >> 5); w++) vmax = fmaxf(vmax, S.bf[8 + w]);
  __syncthreads();
  if (threadIdx.x == 0) {
    hout.flags |= AHFGPU_HALO_RAN_SORT | AHFGPU_HALO_RAN_RVIR0;
    if (ties) atomicAdd(&W.counters[2], ties);
  }
  double mo[3];
  ff Phi0;
  uint64_t n1 = rvir0_phi(c, B, W, P, S, &Phi0, mo, &nret);
  if (threadIdx.x == 0) { hout.M_vir = mo[0]; hout.R_vir = mo[1]; hout.ovdens = mo[2]; hout.Phi0 = 0.0; }
  uint64_t nlist = c.n, ncur = n1;
  bool to_fp64 = false;
  if (n1 >= (uint64_t)P.MINPART) {
    uint64_t npart = n1;
    uint64_t nremove = 4;
    int niter = 0, maxr = 0, nob = 0;
    double R_vir = 0.0, M_vir = 0.0, Phi0_exact = 0.0;
    ff Phi0_used = Phi0;
    IterOut it;
    bool last_exact = false;
    int nexact = 0;
    while (nremove > 3) {
      niter++;
      uint64_t js = seed_slot(c, W, P, niter, n1, S);
      Phi0_used = Phi0;
      unbind_pass(c, B, W, P, S, n1, Phi0, js, vmax, it, &nret);
      last_exact = it.amb != 0;
      if (last_exact) {
        // a bound decision inside the reference's rounding band: redo this
        // iteration in the reference's exact summation order
        long long nbx, lsx;
        double mbx;
        exact_iter32(c, B, W, P, S, n1, js, &nbx, &mbx, &lsx);
        Phi0_used = ff_from_d(S.bd[21]);
        Phi0_exact = S.bd[21];
        it.nb = nbx;
        it.Mb = ff_from_d(mbx);
        it.last_slot = lsx;
        nexact++;
      }
      // members <- bound
      for (uint64_t i = threadIdx.x; i < n1; i += blockDim.x) W.flag[c.o + i] = (W.flag[c.o + i] >> 1) & 1;
      __syncthreads();
      if (it.rounds > maxr) maxr = it.rounds;
      nremove = npart - (uint64_t)it.nb;
      npart = (uint64_t)it.nb;
      if (it.nb == 0) nob = 1;
      M_vir = ff_d(it.Mb);
      if (it.last_slot >= 0) R_vir = ref_dist(c, B, W, c.o + it.last_slot);
      Phi0 = last_exact ? (npart > 0 ? phi0_pass32(c, W, S, n1) : ffz()) : it.Phi0n;
      if (((double)npart) < ((double)P.MINPART)) break;
    }
    if (nexact && threadIdx.x == 0) {
      atomicAdd(&W.counters[1], 1ull);
      hout.flags |= AHFGPU_HALO_REPLAYED;
    }
    if (last_exact && npart >= (uint64_t)P.MINPART) {
      ff Mf;
      it.rv_slot = rvir_pass32(c, B, W, P, S, n1, &Mf, &nret);
      it.rv_M = Mf;
    }
    if (!to_fp64) {
      if (threadIdx.x == 0) {
        hout.flags |= AHFGPU_HALO_RAN_UNBIND;
        if (nob) hout.flags |= AHFGPU_HALO_NOBOUND;
        hout.M_vir = M_vir;
        hout.R_vir = R_vir;
        hout.Phi0 = last_exact ? Phi0_exact : ff_d(Phi0_used);
        hout.niter = niter;
        hout.fix_rounds = maxr;
      }
      ncur = npart;
      nlist = n1;
      if (npart >= (uint64_t)P.MINPART) {
        // rem_outsideRvir(.,1): the candidate of the last pass
        if (it.rv_slot >= 0) {
          for (uint64_t i = (uint64_t)it.rv_slot + 1 + threadIdx.x; i < n1; i += blockDim.x) W.flag[c.o + i] = 0;
          __syncthreads();
        }
        int tot = 0, carry = 0;
        for (uint64_t base = 0; base < n1; base += blockDim.x) {
          uint64_t i = base + threadIdx.x;
          bool mem = i < n1 && (W.flag[c.o + i] & 1);
          block_scan_int(mem ? 1 : 0, &tot, S.iscan);
          carry += tot;
        }
        ncur = (uint64_t)carry;
        if (threadIdx.x == 0) {
          long long ls = it.rv_slot;
          if (ls < 0) ls = it.last_slot;
          double R = ref_dist(c, B, W, c.o + ls);
          double M = it.rv_slot >= 0 ? ff_d(it.rv_M) : M_vir;
          double V = 4. * kPi / 3. * (R * R * R);
          hout.flags |= AHFGPU_HALO_RAN_RVIR1;
          hout.M_vir = M;
          hout.R_vir = R;
          hout.ovdens = M / V * P.rho_fac / P.rho_vir;
        }
        __syncthreads();
        if (ncur >= (uint64_t)P.MINPART) profiles32(c, B, W, P, S, n1, ncur, Phi0_used, hout, &nret);
      }
    }
  }
  atomicAdd(&nret_s, nret);
  __syncthreads();
  if (to_fp64) {
    // the FP64 form resolves this halo in the reference's summation order
    if (threadIdx.x == 0) {
      unsigned k = atomicAdd(W.exact_count, 1u);
      W.exact_list[k] = h;
      W.halo[h] = hout;
      atomicAdd(&W.counters[0], (unsigned long long)nret_s);
    }
    __syncthreads();
    return;
  }
  write_members32(c, nlist, B, W);
  if (threadIdx.x == 0) {
    hout.npart = ncur;
    W.halo[h] = hout;
    atomicAdd(&W.counters[0], (unsigned long long)nret_s);
  }
  __syncthreads();
}

template <int T, class SS>
__global__ void __launch_bounds__(T) halo_fp32c_kernel(DevParams P, DevBatch B, Work W) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  using SM = F32Smem<SS>;
  SM& S = *reinterpret_cast<SM*>(smem_raw);
  uint4* stack = W.sort_stack + (uint64_t)blockIdx.x * W.stack_cap;
  while (true) {
    if (threadIdx.x == 0) S.bi[15] = (int)atomicAdd(W.queue_head, 1u);
    __syncthreads();
    int q = S.bi[15];
    __syncthreads();
    if (q >= W.nqueue) break;
    process_halo32(W.queue[q], P, B, W, S, stack);
  }
}

}  // namespace ahfgpu
