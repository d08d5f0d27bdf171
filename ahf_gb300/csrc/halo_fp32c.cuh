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
  float lastv[32 * 4];
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

// exclusive FP32 scan of NC channels over thread totals (fixed tree)
template <int NC>
__device__ __forceinline__ void bscan_f(const float (&v)[NC], float (&ex)[NC], float (&tot)[NC], float* sm) {
  const unsigned FULL = 0xffffffffu;
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  float inc[NC];
#pragma unroll
  for (int c = 0; c < NC; c++) inc[c] = v[c];
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
#pragma unroll
    for (int c = 0; c < NC; c++) {
      float y = __shfl_up_sync(FULL, inc[c], off);
      if (lane >= off) inc[c] = __fadd_rn(y, inc[c]);
    }
  }
  if (lane == 31) {
#pragma unroll
    for (int c = 0; c < NC; c++) sm[wid * NC + c] = inc[c];
  }
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int c = 0; c < NC; c++) {
      float t = lane < nw ? sm[lane * NC + c] : 0.f;
#pragma unroll
      for (int off = 1; off < 32; off <<= 1) {
        float y = __shfl_up_sync(FULL, t, off);
        if (lane >= off) t = __fadd_rn(y, t);
      }
      if (lane < nw) sm[lane * NC + c] = t;
    }
  }
  __syncthreads();
#pragma unroll
  for (int c = 0; c < NC; c++) {
    float wp = wid > 0 ? sm[(wid - 1) * NC + c] : 0.f;
    float prev = __shfl_up_sync(FULL, inc[c], 1);
    ex[c] = lane > 0 ? __fadd_rn(wp, prev) : wp;
    tot[c] = sm[(nw - 1) * NC + c];
  }
  __syncthreads();
}

// block total of NC float-float channels (the same in every thread)
template <int NC>
__device__ __noinline__ void breduce_ff(const ff (&v)[NC], ff (&tot)[NC], float* sm) {
  const unsigned FULL = 0xffffffffu;
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll (NC <= 4 ? NC : 1)
  for (int c = 0; c < NC; c++) {
    ff x = v[c];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      ff y = {__shfl_xor_sync(FULL, x.hi, off), __shfl_xor_sync(FULL, x.lo, off)};
      x = lane < (lane ^ off) ? ff_add(x, y) : ff_add(y, x);
    }
    if (lane == 0) { sm[(wid * NC + c) * 2] = x.hi; sm[(wid * NC + c) * 2 + 1] = x.lo; }
  }
  __syncthreads();
#pragma unroll (NC <= 4 ? NC : 1)
  for (int c = 0; c < NC; c++) {
    ff t = ffz();
    for (int w = 0; w < nw; w++) t = ff_add(t, ff{sm[(w * NC + c) * 2], sm[(w * NC + c) * 2 + 1]});
    tot[c] = t;
  }
  __syncthreads();
}

// block total of NC float channels
template <int NC>
__device__ __noinline__ void breduce_f(const float (&v)[NC], float (&tot)[NC], float* sm) {
  const unsigned FULL = 0xffffffffu;
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll (NC <= 4 ? NC : 1)
  for (int c = 0; c < NC; c++) {
    float x = v[c];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      float y = __shfl_xor_sync(FULL, x, off);
      x = lane < (lane ^ off) ? __fadd_rn(x, y) : __fadd_rn(y, x);
    }
    if (lane == 0) sm[wid * NC + c] = x;
  }
  __syncthreads();
#pragma unroll (NC <= 4 ? NC : 1)
  for (int c = 0; c < NC; c++) {
    float t = 0.f;
    for (int w = 0; w < nw; w++) t = __fadd_rn(t, sm[w * NC + c]);
    tot[c] = t;
  }
  __syncthreads();
}

// exclusive "last value" over threads with a 4-float payload (distance and
// inverse squared distance of the last member, both float-float)
template <class SM>
__device__ __forceinline__ void blast4(bool has, const float (&val)[4], const float (&carry)[4], float (&res)[4],
                                       float (&last)[4], SM& S) {
  const unsigned FULL = 0xffffffffu;
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  unsigned m = __ballot_sync(FULL, has);
  int lastlane = m ? (31 - __clz(m)) : 0;
  float wv[4];
#pragma unroll
  for (int j = 0; j < 4; j++) wv[j] = __shfl_sync(FULL, val[j], lastlane);
  if (lane == 0) {
    S.lasti[wid] = m ? 1 : 0;
#pragma unroll
    for (int j = 0; j < 4; j++) S.lastv[wid * 4 + j] = wv[j];
  }
  __syncthreads();
  float fl[4] = {carry[0], carry[1], carry[2], carry[3]};
  for (int w = wid - 1; w >= 0; w--)
    if (S.lasti[w]) {
#pragma unroll
      for (int j = 0; j < 4; j++) fl[j] = S.lastv[w * 4 + j];
      break;
    }
  unsigned below = m & ((1u << lane) - 1u);
  int src = below ? (31 - __clz(below)) : 0;
#pragma unroll
  for (int j = 0; j < 4; j++) {
    float mine = __shfl_sync(FULL, val[j], src);
    res[j] = below ? mine : fl[j];
  }
#pragma unroll
  for (int j = 0; j < 4; j++) last[j] = carry[j];
  for (int w = nw - 1; w >= 0; w--)
    if (S.lasti[w]) {
#pragma unroll
      for (int j = 0; j < 4; j++) last[j] = S.lastv[w * 4 + j];
      break;
    }
  __syncthreads();
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
    ff d2 = key_d2(sqkey(dx, dy, dz));
    ff d = ff_sqrt(d2);
    ff q = d2.hi > 0.f ? ff_div(fff(1.f), d2) : ffz();
    W.fdh[s] = d.hi;
    W.fdl[s] = d.lo;
    W.fqh[s] = q.hi;
    W.fql[s] = q.lo;
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

// potential-integral term with the stored 1/d^2 of this and the previous
// member (no division): ((M/d^2 + Mp/dp^2)/2) (d - dp)
__device__ __forceinline__ ff phi_termq(ff M, float w, ff d, ff q, ff dp, ff qp) {
  if (!dpos(d)) return ffz();
  ff Mp = ff_sub(M, fff(w));
  ff In = ff_mul(M, q);
  ff Ip = dpos(dp) ? ff_mul(Mp, qp) : ffz();
  ff Im = ff_add(In, Ip);
  Im.hi = __fmul_rn(Im.hi, 0.5f);
  Im.lo = __fmul_rn(Im.lo, 0.5f);
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
    ff d[kItems], q[kItems], dp, qp;
    ff locM[kItems];
    ff accM = ffz();
#pragma unroll
    for (int k = 0; k < kItems; k++) {
      uint64_t i = i0 + k;
      bool v = i < c.n;
      w[k] = v ? W.sw[c.o + i] : 0.f;
      d[k] = v ? ff{W.fdh[c.o + i], W.fdl[c.o + i]} : ffz();
      q[k] = v ? ff{W.fqh[c.o + i], W.fql[c.o + i]} : ffz();
      accM = ff_add(accM, fff(w[k]));
      locM[k] = accM;
    }
    bool hasp = i0 > 0 && i0 < c.n;
    dp = hasp ? ff{W.fdh[c.o + i0 - 1], W.fdl[c.o + i0 - 1]} : ffz();
    qp = hasp ? ff{W.fqh[c.o + i0 - 1], W.fql[c.o + i0 - 1]} : ffz();
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
      ff prevq = k == 0 ? qp : q[k - 1];
      term[k] = i < c.n ? phi_termq(Mk[k], w[k], d[k], q[k], prevd, prevq) : ffz();
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
// Out: flag bit1 = bound (bit0 kept); next-iteration Phi0; kept count/mass;
// last kept slot; the rvir1 candidate (first kept slot failing the
// overdensity test).  amb: some decision stayed inside the reference-rounding
// band (the caller redoes the iteration exactly).
struct IterOut {
  long long nb;
  ff Mb, Phi0n;
  long long last_slot;
  long long rv_slot;   // first failing kept slot or -1
  ff rv_M, rv_d;
  int amb;
  int rounds;
};

template <class SM>
static __device__ void unbind_pass(const Ctx32& c, const DevBatch& B, const Work& W, const DevParams& P, SM& S,
                                   uint64_t n1, ff Phi0, uint64_t js, float vmax, IterOut& out, unsigned* nret) {
  const uint64_t o = c.o;
  const float vf = (float)P.v_fac, Hr = (float)(P.Hubble * P.r_fac), v2t = (float)P.v2_tune;
  const float pf2 = (float)(2.0 * P.phi_fac);
  const float V43f = (float)(4. * kPi / 3.);
  const float w0 = W.sw[o + js];
  ff cM = ffz(), cPhi = ffz();
  float cD[4] = {0.f, 0.f, 0.f, 0.f};
  ff cVX = two_prod(w0, W.svx[o + js]), cVY = two_prod(w0, W.svy[o + js]), cVZ = two_prod(w0, W.svz[o + js]);
  ff cMv = fff(w0);
  ff cMb = ffz(), cPhiN = ffz();
  float cDb[4] = {0.f, 0.f, 0.f, 0.f};
  long long cNb = 0, last_slot = -1, rv = -1;
  ff rvM = ffz(), rvD = ffz();
  int amb_any = 0, maxr = 0;
  for (uint64_t base = 0; base < n1; base += (uint64_t)blockDim.x * kItems) {
    const uint64_t i0 = base + (uint64_t)threadIdx.x * kItems;
    bool m[kItems];
    float w[kItems], vx[kItems], vy[kItems], vz[kItems], dx[kItems], dy[kItems], dz[kItems];
    ff d[kItems], q[kItems];
    bool any_m = false;
    float lastm[4] = {0.f, 0.f, 0.f, 0.f};
    ff accM = ffz(), locM[kItems];
#pragma unroll
    for (int k = 0; k < kItems; k++) {
      uint64_t i = i0 + k;
      m[k] = i < n1 && (W.flag[o + i] & 1);
      w[k] = vx[k] = vy[k] = vz[k] = dx[k] = dy[k] = dz[k] = 0.f;
      d[k] = q[k] = ffz();
      if (m[k]) {
        w[k] = W.sw[o + i];
        vx[k] = W.svx[o + i]; vy[k] = W.svy[o + i]; vz[k] = W.svz[o + i];
        dx[k] = W.fdx[o + i]; dy[k] = W.fdy[o + i]; dz[k] = W.fdz[o + i];
        d[k] = ff{W.fdh[o + i], W.fdl[o + i]};
        q[k] = ff{W.fqh[o + i], W.fql[o + i]};
        any_m = true;
        lastm[0] = d[k].hi; lastm[1] = d[k].lo; lastm[2] = q[k].hi; lastm[3] = q[k].lo;
        accM = ff_add(accM, fff(w[k]));
      }
      locM[k] = accM;
    }
    // member mass prefix, previous member, potential prefix
    ff exM[1], totM[1], vM[1] = {accM};
    bscan_ff<1>(vM, exM, totM, S.scan);
    float dprev[4], blockLast[4];
    blast4(any_m, lastm, cD, dprev, blockLast, S);
    ff Mk[kItems], phi[kItems], accP = ffz();
    {
      ff dp = {dprev[0], dprev[1]}, qp = {dprev[2], dprev[3]};
      ff baseM = ff_add(cM, exM[0]);
#pragma unroll
      for (int k = 0; k < kItems; k++) {
        Mk[k] = ff_add(baseM, locM[k]);
        if (m[k]) {
          accP = ff_add(accP, phi_termq(Mk[k], w[k], d[k], q[k], dp, qp));
          dp = d[k];
          qp = q[k];
        }
        phi[k] = accP;
      }
    }
    ff exP[1], totP[1], vP[1] = {accP};
    bscan_ff<1>(vP, exP, totP, S.scan);
    float thr[kItems];
    {
      ff basePhi = ff_add(cPhi, exP[0]);
#pragma unroll
      for (int k = 0; k < kItems; k++) {
        phi[k] = ff_add(basePhi, phi[k]);
        float A = fabsf(ff_f(ff_sub(phi[k], Phi0)));
        thr[k] = dpos(d[k]) ? __fmul_rn(v2t, __fmul_rn(pf2, A)) : __fmul_rn(v2t, 1e30f);
      }
    }
    // tile fixpoint of the bound flags.  FP32 decisions use momenta relative
    // to the tile's reference bulk velocity Vr = cV/cMv (small, random
    // deviations u = v - Vr), so V = Vr + (R + sum w u)/Mv with R = cV - Vr cMv
    // kept in float-float; each decision carries a first-order bound on its
    // FP32 error.  Float-float prefixes (for the FP64 re-test) are built only
    // in rounds where some decision falls inside its bound.
    const float fe = 5.9604645e-08f;   // 2^-24
    const float Vrx = ff_f(ff_div(cVX, cMv)), Vry = ff_f(ff_div(cVY, cMv)), Vrz = ff_f(ff_div(cVZ, cMv));
    const float Rx = ff_f(ff_sub(cVX, ff_mul(fff(Vrx), cMv)));
    const float Ry = ff_f(ff_sub(cVY, ff_mul(fff(Vry), cMv)));
    const float Rz = ff_f(ff_sub(cVZ, ff_mul(fff(Vrz), cMv)));
    float ux[kItems], uy[kItems], uz[kItems];
#pragma unroll
    for (int k = 0; k < kItems; k++) {
      ux[k] = __fsub_rn(vx[k], Vrx);
      uy[k] = __fsub_rn(vy[k], Vry);
      uz[k] = __fsub_rn(vz[k], Vrz);
    }
    bool b[kItems];
#pragma unroll
    for (int k = 0; k < kItems; k++) b[k] = m[k];
    int rounds = 0;
    bool amb_tile = false;
    while (true) {
      rounds++;
      float fx[kItems], fy[kItems], fz[kItems], fm[kItems], fa[kItems];
      float sx = 0.f, sy = 0.f, sz = 0.f, sm = 0.f, sa = 0.f;
#pragma unroll
      for (int k = 0; k < kItems; k++) {
        fx[k] = sx; fy[k] = sy; fz[k] = sz; fm[k] = sm; fa[k] = sa;
        if (b[k]) {
          float wx = __fmul_rn(w[k], ux[k]), wy = __fmul_rn(w[k], uy[k]), wz = __fmul_rn(w[k], uz[k]);
          sx = __fadd_rn(sx, wx);
          sy = __fadd_rn(sy, wy);
          sz = __fadd_rn(sz, wz);
          sm = __fadd_rn(sm, w[k]);
          sa = __fadd_rn(sa, __fadd_rn(__fadd_rn(fabsf(wx), fabsf(wy)), fabsf(wz)));
        }
      }
      float ex5[5], tot5[5], v5[5] = {sx, sy, sz, sm, sa};
      bscan_f<5>(v5, ex5, tot5, S.scan);
      int changed = 0;
      bool need[kItems];
      bool any_need = false;
#pragma unroll
      for (int k = 0; k < kItems; k++) {
        need[k] = false;
        if (!m[k]) continue;
        float Ux = __fadd_rn(ex5[0], fx[k]), Uy = __fadd_rn(ex5[1], fy[k]), Uz = __fadd_rn(ex5[2], fz[k]);
        float Mv = __fadd_rn(cMv.hi, __fadd_rn(ex5[3], fm[k]));
        float Asum = __fadd_rn(ex5[4], fa[k]);
        float rmv = __fdiv_rn(1.f, Mv);
        float Dx = __fmul_rn(__fadd_rn(Rx, Ux), rmv), Dy = __fmul_rn(__fadd_rn(Ry, Uy), rmv),
              Dz = __fmul_rn(__fadd_rn(Rz, Uz), rmv);
        float hx = __fmul_rn(Hr, dx[k]), hy = __fmul_rn(Hr, dy[k]), hz = __fmul_rn(Hr, dz[k]);
        float dVX = __fadd_rn(__fmul_rn(__fsub_rn(ux[k], Dx), vf), hx);
        float dVY = __fadd_rn(__fmul_rn(__fsub_rn(uy[k], Dy), vf), hy);
        float dVZ = __fadd_rn(__fmul_rn(__fsub_rn(uz[k], Dz), vf), hz);
        float vel2 = __fadd_rn(__fadd_rn(__fmul_rn(dVX, dVX), __fmul_rn(dVY, dVY)), __fmul_rn(dVZ, dVZ));
        // error bound: tile-sum error (depth <= 16 per component), the rest
        // a few roundings of each magnitude involved; x2 slack
        float eD = __fmul_rn(__fadd_rn(__fmul_rn(16.f * fe, Asum), __fmul_rn(fe, __fadd_rn(fabsf(Rx) + fabsf(Ry),
                                                                                            fabsf(Rz)))), rmv);
        float mag = __fadd_rn(__fmul_rn(__fadd_rn(fabsf(ux[k]) + fabsf(uy[k]) + fabsf(uz[k]),
                                                  fabsf(Dx) + fabsf(Dy) + fabsf(Dz)), vf),
                              fabsf(hx) + fabsf(hy) + fabsf(hz));
        float edv = __fadd_rn(__fmul_rn(eD, vf), __fmul_rn(4.f * fe, mag));
        float sdv = fabsf(dVX) + fabsf(dVY) + fabsf(dVZ);
        float err = __fmul_rn(2.f, __fadd_rn(__fadd_rn(__fmul_rn(2.f * sdv, edv), __fmul_rn(3.f, __fmul_rn(edv, edv))),
                                             __fmul_rn(8.f * fe, __fadd_rn(vel2, thr[k]))));
        float margin = __fsub_rn(thr[k], vel2);
        if (fabsf(margin) > err && isfinite(margin) && isfinite(err)) {
          bool nb = margin >= 0.f;
          if (nb != b[k]) { b[k] = nb; changed = 1; }
        } else {
          need[k] = true;
          any_need = true;
        }
      }
      if (__syncthreads_or(any_need ? 1 : 0)) {
        // exact float-float prefixes of this round's flags
        ff ax = ffz(), ay = ffz(), az = ffz(), am = ffz(), lx[kItems], ly[kItems], lz[kItems], lm[kItems];
#pragma unroll
        for (int k = 0; k < kItems; k++) {
          lx[k] = ax; ly[k] = ay; lz[k] = az; lm[k] = am;
          if (b[k]) {
            ax = ff_add(ax, two_prod(w[k], vx[k]));
            ay = ff_add(ay, two_prod(w[k], vy[k]));
            az = ff_add(az, two_prod(w[k], vz[k]));
            am = ff_add(am, fff(w[k]));
          }
        }
        ff e4[4], t4[4], a4[4] = {ax, ay, az, am};
        bscan_ff<4>(a4, e4, t4, S.scan);
#pragma unroll
        for (int k = 0; k < kItems; k++) {
          if (!need[k]) continue;
          (*nret)++;
          bool amb = false;
          bool nb = retest_bound(c, B, W, P, o + i0 + k, i0 + k, n1, phi[k], Phi0,
                                 ff_add(ff_add(cVX, e4[0]), lx[k]), ff_add(ff_add(cVY, e4[1]), ly[k]),
                                 ff_add(ff_add(cVZ, e4[2]), lz[k]), ff_add(ff_add(cMv, e4[3]), lm[k]), vmax, &amb);
          if (amb) amb_tile = true;
          if (nb != b[k]) { b[k] = nb; changed = 1; }
        }
      }
      if (!__syncthreads_or(changed)) break;
      if (rounds >= kMaxFixRounds) { amb_tile = true; break; }
    }
    if (rounds > maxr) maxr = rounds;
    amb_any |= __syncthreads_or(amb_tile ? 1 : 0);
    // carries of the running bulk velocity: float-float tile totals
    {
      ff ax = ffz(), ay = ffz(), az = ffz(), am = ffz();
#pragma unroll
      for (int k = 0; k < kItems; k++) {
        if (b[k]) {
          ax = ff_add(ax, two_prod(w[k], vx[k]));
          ay = ff_add(ay, two_prod(w[k], vy[k]));
          az = ff_add(az, two_prod(w[k], vz[k]));
          am = ff_add(am, fff(w[k]));
        }
      }
      ff t4[4], a4[4] = {ax, ay, az, am};
      breduce_ff<4>(a4, t4, S.scan);
      cVX = ff_add(cVX, t4[0]); cVY = ff_add(cVY, t4[1]); cVZ = ff_add(cVZ, t4[2]); cMv = ff_add(cMv, t4[3]);
    }
    // next-iteration channels over the kept particles
    ff accB = ffz(), locB[kItems];
    bool any_b = false;
    float lastb[4] = {0.f, 0.f, 0.f, 0.f};
    int nbl = 0;
    long long lslot = -1;
#pragma unroll
    for (int k = 0; k < kItems; k++) {
      if (b[k]) {
        accB = ff_add(accB, fff(w[k]));
        any_b = true;
        lastb[0] = d[k].hi; lastb[1] = d[k].lo; lastb[2] = q[k].hi; lastb[3] = q[k].lo;
        nbl++;
        lslot = (long long)(i0 + k);
      }
      locB[k] = accB;
    }
    ff exB[1], totB[1], vB[1] = {accB};
    bscan_ff<1>(vB, exB, totB, S.scan);
    float dpb4[4], blastB[4];
    blast4(any_b, lastb, cDb, dpb4, blastB, S);
    int tnb;
    bscan_int_ex(nbl, &tnb, S);
    ff accN = ffz();
    long long myfail = 0x7fffffffffffffffll;
    ff fM = ffz(), fD = ffz();
    {
      ff dpb = {dpb4[0], dpb4[1]}, qpb = {dpb4[2], dpb4[3]};
      ff baseB = ff_add(cMb, exB[0]);
      const float lim = P.f_ovlim, rvrf = P.f_rvrf;
#pragma unroll
      for (int k = 0; k < kItems; k++) {
        if (!b[k]) continue;
        ff Mb = ff_add(baseB, locB[k]);
        accN = ff_add(accN, phi_termq(Mb, w[k], d[k], q[k], dpb, qpb));
        dpb = d[k];
        qpb = q[k];
        if (rv < 0 && myfail == 0x7fffffffffffffffll) {
          // cheap FP32 screen; the banded test (with FP64 re-test) only near ovlim
          float df = d[k].hi;
          float ov = __fdiv_rn(__fdiv_rn(Mb.hi, __fmul_rn(V43f, __fmul_rn(__fmul_rn(df, df), df))), rvrf);
          if (!(ov > lim * (1.f + 4.f * kBand1)) &&
              ov_fail(c, B, W, P, o + i0 + k, Mb, d[k], nret)) {
            myfail = (long long)(i0 + k);
            fM = Mb;
            fD = d[k];
          }
        }
      }
    }
    ff totN[1], vN[1] = {accN};
    breduce_ff<1>(vN, totN, S.scan);
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
#pragma unroll
    for (int k = 0; k < kItems; k++) {
      uint64_t i = i0 + k;
      if (i < n1) W.flag[o + i] = (uint8_t)((m[k] ? 1 : 0) | (b[k] ? 2 : 0));
    }
    cM = ff_add(cM, totM[0]);
    cPhi = ff_add(cPhi, totP[0]);
#pragma unroll
    for (int j = 0; j < 4; j++) { cD[j] = blockLast[j]; cDb[j] = blastB[j]; }
    cMb = ff_add(cMb, totB[0]);
    cPhiN = ff_add(cPhiN, totN[0]);
    cNb += tnb;
  }
  out.nb = cNb;
  out.Mb = cMb;
  out.Phi0n = cNb > 0 ? ff_add(cPhiN, ff_div(cMb, ff{cDb[0], cDb[1]})) : ffz();
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
  ff cM = ffz(), cPhi = ffz();
  float cD[4] = {0.f, 0.f, 0.f, 0.f};
  for (uint64_t base = 0; base < n1; base += (uint64_t)blockDim.x * kItems) {
    uint64_t i0 = base + (uint64_t)threadIdx.x * kItems;
    bool m[kItems];
    float w[kItems];
    ff d[kItems], q[kItems];
    bool any = false;
    float lastm[4] = {0.f, 0.f, 0.f, 0.f};
    ff accM = ffz(), locM[kItems];
#pragma unroll
    for (int k = 0; k < kItems; k++) {
      uint64_t i = i0 + k;
      m[k] = i < n1 && (W.flag[o + i] & 1);
      w[k] = m[k] ? W.sw[o + i] : 0.f;
      d[k] = m[k] ? ff{W.fdh[o + i], W.fdl[o + i]} : ffz();
      q[k] = m[k] ? ff{W.fqh[o + i], W.fql[o + i]} : ffz();
      if (m[k]) {
        accM = ff_add(accM, fff(w[k]));
        any = true;
        lastm[0] = d[k].hi; lastm[1] = d[k].lo; lastm[2] = q[k].hi; lastm[3] = q[k].lo;
      }
      locM[k] = accM;
    }
    ff exM[1], totM[1], vM[1] = {accM};
    bscan_ff<1>(vM, exM, totM, S.scan);
    float dp4[4], blockLast[4];
    blast4(any, lastm, cD, dp4, blockLast, S);
    ff dp = {dp4[0], dp4[1]}, qp = {dp4[2], dp4[3]};
    ff accP = ffz();
#pragma unroll
    for (int k = 0; k < kItems; k++) {
      if (!m[k]) continue;
      accP = ff_add(accP, phi_termq(ff_add(ff_add(cM, exM[0]), locM[k]), w[k], d[k], q[k], dp, qp));
      dp = d[k];
      qp = q[k];
    }
    ff totP[1], vP[1] = {accP};
    breduce_ff<1>(vP, totP, S.scan);
    cM = ff_add(cM, totM[0]);
    cPhi = ff_add(cPhi, totP[0]);
#pragma unroll
    for (int j = 0; j < 4; j++) cD[j] = blockLast[j];
  }
  return ff_add(cPhi, ff_div(cM, ff{cD[0], cD[1]}));
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

// HaloProfiles per-particle terms (ahf_halos.c:4320-4420).  VX.. are the
// momentum prefixes INCLUDING the particle (the reference updates VXc
// first).  The velocity relative to the running bulk velocity is
// float-float (one float division plus its residual), so the kinetic term
// T stays accurate where Ekin + Epot cancels (lambdaE).
struct PTerms {
  ff phi, T, cx, cy, cz;   // potential term, kinetic term, w dX, w dY, w dZ
  float g[11];             // Lx, Ly, Lz, a11, a22, a33, a12, a13, a23, Mhi, Mlo
};

__device__ __forceinline__ ff rel_vel(float v, ff V, ff M) {
  float b = __fdiv_rn(V.hi, M.hi);
  ff r = ff_sub(V, ff_mulf(M, b));
  ff Vb = ff_quick(b, __fdiv_rn(r.hi, M.hi));
  return ff_sub(fff(v), Vb);
}

__device__ __forceinline__ void pterms(float w, float vx, float vy, float vz, float dx, float dy, float dz,
                                       float dxl, float dyl, float dzl, ff d, ff q, ff dp, ff qp, ff M, ff VX,
                                       ff VY, ff VZ, float Hrv, int has_w, PTerms& t) {
  ff gx = rel_vel(vx, VX, M), gy = rel_vel(vy, VY, M), gz = rel_vel(vz, VZ, M);
  float gxf = ff_f(gx), gyf = ff_f(gy), gzf = ff_f(gz);
  t.phi = phi_termq(M, w, d, q, dp, qp);
  t.g[0] = __fmul_rn(w, __fsub_rn(__fmul_rn(dy, gzf), __fmul_rn(dz, gyf)));
  t.g[1] = __fmul_rn(w, __fsub_rn(__fmul_rn(dz, gxf), __fmul_rn(dx, gzf)));
  t.g[2] = __fmul_rn(w, __fsub_rn(__fmul_rn(dx, gyf), __fmul_rn(dy, gxf)));
  gx = ff_add(gx, ff_mulf(two_sum(dx, dxl), Hrv));
  gy = ff_add(gy, ff_mulf(two_sum(dy, dyl), Hrv));
  gz = ff_add(gz, ff_mulf(two_sum(dz, dzl), Hrv));
  t.T = ff_mulf(ff_add(ff_add(ff_mul(gx, gx), ff_mul(gy, gy)), ff_mul(gz, gz)), w);
  t.cx = ff_add(two_prod(w, dx), fff(__fmul_rn(w, dxl)));
  t.cy = ff_add(two_prod(w, dy), fff(__fmul_rn(w, dyl)));
  t.cz = ff_add(two_prod(w, dz), fff(__fmul_rn(w, dzl)));
  float wx = __fmul_rn(w, dx), wy = __fmul_rn(w, dy), wz = __fmul_rn(w, dz);
  t.g[3] = __fmul_rn(wx, dx);
  t.g[4] = __fmul_rn(wy, dy);
  t.g[5] = __fmul_rn(wz, dz);
  t.g[6] = __fmul_rn(wx, dy);
  t.g[7] = __fmul_rn(wx, dz);
  t.g[8] = __fmul_rn(wy, dz);
  t.g[9] = 0.f;
  t.g[10] = 0.f;
  if (has_w) {
    if (fabsf(w - 1.0f) < (float)kZero) t.g[9] = w;
    else if (w > 1.0f) t.g[10] = w;
  } else {
    t.g[9] = w;
  }
}

// out-of-line copy for the (rare) bin-end recomputation
static __device__ __noinline__ void pterms_ool(float w, float vx, float vy, float vz, float dx, float dy, float dz,
                                               float dxl, float dyl, float dzl, ff d, ff q, ff dp, ff qp, ff M,
                                               ff VX, ff VY, ff VZ, float Hrv, int has_w, PTerms& t) {
  pterms(w, vx, vy, vz, dx, dy, dz, dxl, dyl, dzl, d, q, dp, qp, M, VX, VY, VZ, Hrv, has_w, t);
}

// FP64 energy 0.5 T + U of a most-bound candidate (ahf_halos.c:4380-4420)
static __device__ __noinline__ double mbp_energy64(const Ctx32& c, const DevBatch& B, const Work& W,
                                                   const DevParams& P, uint64_t s, ff M, ff VX, ff VY, ff VZ,
                                                   ff phi, ff Phi0, float w) {
  uint64_t e = c.o + W.seid[s];
  double dX = wrap_s((double)B.x[e] - c.cx), dY = wrap_s((double)B.y[e] - c.cy), dZ = wrap_s((double)B.z[e] - c.cz);
  double Md = ff_d(M);
  double dVX = ((double)B.vx[e] - ff_d(VX) / Md), dVY = ((double)B.vy[e] - ff_d(VY) / Md),
         dVZ = ((double)B.vz[e] - ff_d(VZ) / Md);
  dVX += P.Hubble * dX * P.r_fac / P.v_fac;
  dVY += P.Hubble * dY * P.r_fac / P.v_fac;
  dVZ += P.Hubble * dZ * P.r_fac / P.v_fac;
  double wk = (double)w;
  double Tpart = wk * ((dVX * dVX + dVY * dVY) + dVZ * dVZ);
  double Upart = (ff_d(phi) - ff_d(Phi0)) * wk;
  return 0.5 * Tpart + Upart;
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
  ff c1[4] = {ffz(), ffz(), ffz(), ffz()};   // M, VX, VY, VZ (inclusive prefixes)
  ff cPhi = ffz(), cU = ffz();
  ff cf[4] = {ffz(), ffz(), ffz(), ffz()};   // T, sum w dX, sum w dY, sum w dZ
  float cg[11];                              // Lx, Ly, Lz, a11, a22, a33, a12, a13, a23, Mhi, Mlo
#pragma unroll
  for (int j = 0; j < 11; j++) cg[j] = 0.f;
  ff cgc[11];                                // float-float carries of the float channels
#pragma unroll
  for (int j = 0; j < 11; j++) cgc[j] = ffz();
  float cD[4] = {0.f, 0.f, 0.f, 0.f};
  int cr = 0;
  double Ebest = 1e30;
  long long Eslot = -1;
  for (uint64_t base = 0; base < n1; base += (uint64_t)blockDim.x * kItems) {
    const uint64_t i0 = base + (uint64_t)threadIdx.x * kItems;
    bool m[kItems];
    float w[kItems], vx[kItems], vy[kItems], vz[kItems], dx[kItems], dy[kItems], dz[kItems];
    float dxl[kItems], dyl[kItems], dzl[kItems];
    ff d[kItems], q[kItems];
    int nm = 0;
    bool any = false;
    float lastm[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int k = 0; k < kItems; k++) {
      uint64_t i = i0 + k;
      m[k] = i < n1 && (W.flag[o + i] & 1);
      w[k] = vx[k] = vy[k] = vz[k] = dx[k] = dy[k] = dz[k] = 0.f;
      dxl[k] = dyl[k] = dzl[k] = 0.f;
      d[k] = q[k] = ffz();
      if (m[k]) {
        w[k] = W.sw[o + i];
        vx[k] = W.svx[o + i]; vy[k] = W.svy[o + i]; vz[k] = W.svz[o + i];
        dx[k] = W.fdx[o + i]; dy[k] = W.fdy[o + i]; dz[k] = W.fdz[o + i];
        dxl[k] = W.fdxl[o + i]; dyl[k] = W.fdyl[o + i]; dzl[k] = W.fdzl[o + i];
        d[k] = ff{W.fdh[o + i], W.fdl[o + i]};
        q[k] = ff{W.fqh[o + i], W.fql[o + i]};
        nm++; any = true;
        lastm[0] = d[k].hi; lastm[1] = d[k].lo; lastm[2] = q[k].hi; lastm[3] = q[k].lo;
      }
    }
    int tn;
    int rank0 = bscan_int_ex(nm, &tn, S) + cr;
    float dp4[4], blockLast[4];
    blast4(any, lastm, cD, dp4, blockLast, S);
    // scan 1: mass and momentum prefixes (inclusive: the reference adds the
    // particle before using them)
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
      for (int j = 0; j < 4; j++) l1[k][j] = a1[j];
    }
    ff e1[4], t1[4];
    bscan_ff<4>(a1, e1, t1, S.scan);
    ff b1[4];
#pragma unroll
    for (int j = 0; j < 4; j++) b1[j] = ff_add(c1[j], e1[j]);
    // per-particle terms, thread totals; bin ends of this tile
    ff tf[4] = {ffz(), ffz(), ffz(), ffz()}, tphi = ffz();
    float tg[11];
#pragma unroll
    for (int j = 0; j < 11; j++) tg[j] = 0.f;
    float Tp[kItems];
    ff pt[kItems];
    bool has_end = false;
    {
      ff dp = {dp4[0], dp4[1]}, qp = {dp4[2], dp4[3]};
      int r = rank0;
#pragma unroll
      for (int k = 0; k < kItems; k++) {
        Tp[k] = 0.f;
        pt[k] = ffz();
        if (!m[k]) continue;
        ff M = ff_add(b1[0], l1[k][0]);
        PTerms t;
        pterms(w[k], vx[k], vy[k], vz[k], dx[k], dy[k], dz[k], dxl[k], dyl[k], dzl[k], d[k], q[k], dp, qp, M,
               ff_add(b1[1], l1[k][1]), ff_add(b1[2], l1[k][2]), ff_add(b1[3], l1[k][3]), Hrv, P.has_w, t);
        pt[k] = t.phi;
        tphi = ff_add(tphi, t.phi);
        Tp[k] = ff_f(t.T);
        tf[0] = ff_add(tf[0], t.T);
        tf[1] = ff_add(tf[1], t.cx);
        tf[2] = ff_add(tf[2], t.cy);
        tf[3] = ff_add(tf[3], t.cz);
#pragma unroll
        for (int j = 0; j < 11; j++) tg[j] = __fadd_rn(tg[j], t.g[j]);
        // per-rank arrays (ahf_halos.c:4598-4616)
        Mff[r] = make_float2(M.hi, M.lo);
        float df = ff_f(d[k]);
        vc2[r] = __fdiv_rn(ff_f(M), df);
        ff d3 = ff_mul(ff_mul(d[k], d[k]), d[k]);
        ff p3 = ff_mul(ff_mul(dp, dp), dp);
        float dV = __fmul_rn((float)FPT, ff_f(ff_sub(d3, p3)));
        float rm = __fmul_rn(__fadd_rn(df, ff_f(dp)), 0.5f);
        dr2[r] = __fmul_rn(__fdiv_rn(w[k], dV), __fmul_rn(rm, rm));
        // bin boundary after this particle?
        double dd = ff_d(d[k]);
        int bnext = 0;
        while (bnext < nbins && !(dd < S.edge[bnext])) bnext++;
        double dpd = ff_d(dp);
        int bcur = 0;
        if (r > 0) { while (bcur < nbins && !(dpd < S.edge[bcur])) bcur++; }
        if (bnext > bcur || (uint64_t)(r + 1) == n2) has_end = true;
        dp = d[k];
        qp = q[k];
        r++;
      }
    }
    // potential: per-particle prefix (needed for U of every particle)
    ff ePh[1], tPh[1], vPh[1] = {tphi};
    bscan_ff<1>(vPh, ePh, tPh, S.scan);
    ff phi[kItems], tU = ffz();
    float Ef[kItems];
    {
      ff run = ff_add(cPhi, ePh[0]);
#pragma unroll
      for (int k = 0; k < kItems; k++) {
        run = ff_add(run, pt[k]);
        phi[k] = run;
        Ef[k] = 3.0e38f;
        if (m[k]) {
          ff U = ff_mulf(ff_sub(run, Phi0), w[k]);
          tU = ff_add(tU, U);
          Ef[k] = __fadd_rn(__fmul_rn(0.5f, Tp[k]), ff_f(U));
        }
      }
    }
    // channels needed only at bin ends: full scans in tiles with a bin end,
    // block totals otherwise
    const bool tile_end = __syncthreads_or(has_end ? 1 : 0) != 0;
    ff ef5[5], tf5[5], af5[5] = {tf[0], tf[1], tf[2], tf[3], tU};
    float eg[11], tgt[11];
    if (tile_end) {
      bscan_ff<5>(af5, ef5, tf5, S.scan);
      bscan_f<11>(tg, eg, tgt, S.scan);
    } else {
      breduce_ff<5>(af5, tf5, S.scan);
      breduce_f<11>(tg, tgt, S.scan);
#pragma unroll
      for (int j = 0; j < 5; j++) ef5[j] = ffz();
#pragma unroll
      for (int j = 0; j < 11; j++) eg[j] = 0.f;
    }
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
      for (int qq = 0; qq < nw; qq++) tmin = fminf(tmin, S.bf[qq]);
      __syncthreads();
      float ref = fminf(tmin, (float)Ebest);
      float cut = ref + 1e-4f * fabsf(ref) + 1e-30f;
      double bE = 1e300;
      long long bs = -1;
#pragma unroll
      for (int k = 0; k < kItems; k++) {
        if (!m[k] || !(Ef[k] <= cut)) continue;
        (*nret)++;
        double E = mbp_energy64(c, B, W, P, o + i0 + k, ff_add(b1[0], l1[k][0]), ff_add(b1[1], l1[k][1]),
                                ff_add(b1[2], l1[k][2]), ff_add(b1[3], l1[k][3]), phi[k], Phi0, w[k]);
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
      for (int qq = 0; qq < nw; qq++) {
        double oE = S.bd[qq];
        long long oi = S.bl[qq];
        bool take = oi >= 0 && (TS < 0 || oE < TE || (oE == TE && oi < TS));
        if (take) { TE = oE; TS = oi; }
      }
      __syncthreads();
      if (TS >= 0 && TE < Ebest) { Ebest = TE; Eslot = TS; }
    }
    // bin records at bin ends (cumulative values over the members so far)
    if (tile_end && has_end) {
      ff dp = {dp4[0], dp4[1]}, qp = {dp4[2], dp4[3]};
      int r = rank0;
      ff runf[5];
      float rung[11];
#pragma unroll
      for (int j = 0; j < 5; j++) runf[j] = ff_add(j < 4 ? cf[j] : cU, ef5[j]);
#pragma unroll
      for (int j = 0; j < 11; j++) rung[j] = __fadd_rn(cg[j], eg[j]);
      ff runU = ff_add(cU, ef5[4]);
      for (int k = 0; k < kItems; k++) {
        if (!m[k]) continue;
        ff M = ff_add(b1[0], l1[k][0]);
        PTerms t;
        pterms_ool(w[k], vx[k], vy[k], vz[k], dx[k], dy[k], dz[k], dxl[k], dyl[k], dzl[k], d[k], q[k], dp, qp, M,
                   ff_add(b1[1], l1[k][1]), ff_add(b1[2], l1[k][2]), ff_add(b1[3], l1[k][3]), Hrv, P.has_w, t);
        runf[0] = ff_add(runf[0], t.T);
        for (int j = 0; j < 11; j++) rung[j] = __fadd_rn(rung[j], t.g[j]);
        ff U = ff_mulf(ff_sub(phi[k], Phi0), w[k]);
        runU = ff_add(runU, U);
        double dd = ff_d(d[k]), dpd = ff_d(dp);
        int bcur = 0;
        if (r > 0) { while (bcur < nbins && !(dpd < S.edge[bcur])) bcur++; }
        int bnext = 0;
        while (bnext < nbins && !(dd < S.edge[bnext])) bnext++;
        bool last = (uint64_t)(r + 1) == n2;
        int bend = last ? nbins : bnext;
        for (int bb = bcur; bb < bend; bb++) {
          Bin& R = S.bins[bb];
          R.npart = (double)(r + 1);
          R.M = ff_d(M);
          R.Lx = ff_d(ff_add(cgc[0], fff(rung[0])));
          R.Ly = ff_d(ff_add(cgc[1], fff(rung[1])));
          R.Lz = ff_d(ff_add(cgc[2], fff(rung[2])));
          R.T = ff_d(runf[0]);
          R.U = ff_d(runU);
          R.a11 = ff_d(ff_add(cgc[3], fff(rung[3])));
          R.a22 = ff_d(ff_add(cgc[4], fff(rung[4])));
          R.a33 = ff_d(ff_add(cgc[5], fff(rung[5])));
          R.a12 = ff_d(ff_add(cgc[6], fff(rung[6])));
          R.a13 = ff_d(ff_add(cgc[7], fff(rung[7])));
          R.a23 = ff_d(ff_add(cgc[8], fff(rung[8])));
          R.vesc2 = 2 * fabs((ff_d(phi[k]) - ff_d(Phi0)) * (double)w[k]) / (double)w[k];
        }
        dp = d[k];
        qp = q[k];
        r++;
      }
    }
    // carries
#pragma unroll
    for (int j = 0; j < 4; j++) c1[j] = ff_add(c1[j], t1[j]);
    cPhi = ff_add(cPhi, tPh[0]);
#pragma unroll
    for (int j = 0; j < 4; j++) cf[j] = ff_add(cf[j], tf5[j]);
    cU = ff_add(cU, tf5[4]);
#pragma unroll
    for (int j = 0; j < 11; j++) { cgc[j] = ff_add(cgc[j], fff(tgt[j])); cg[j] = 0.f; }
#pragma unroll
    for (int j = 0; j < 4; j++) cD[j] = blockLast[j];
    cr += tn;
    __syncthreads();
  }
  double* rows = W.prof_stage + W.prof_cap_off[c.h] * AHFGPU_PROF_NFIELDS;
#ifdef AHFGPU_PHASE_TIMERS
  long long _pp = clock64();
#endif
  write_bin_rows(S.bins, S.edge, nbins, rows);
  __syncthreads();
#ifdef AHFGPU_PHASE_TIMERS
  if (threadIdx.x == 0 && W.phase) { long long t = clock64(); atomicAdd(&W.phase[8], (unsigned long long)(t - _pp)); _pp = t; }
#endif
  uint64_t i_r2 = find_max32(c, B, W, S, 0, 3, n2, nret);
  uint64_t i_rm = find_max32(c, B, W, S, 1, 1, n2, nret);
#ifdef AHFGPU_PHASE_TIMERS
  __syncthreads();
  if (threadIdx.x == 0 && W.phase) { long long t = clock64(); atomicAdd(&W.phase[9], (unsigned long long)(t - _pp)); }
#endif
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
    double Mt = ff_d(c1[0]);
    finish_scalars(rows, nbins, Mt, ff_d(c1[1]), ff_d(c1[2]), ff_d(c1[3]), Mt * c.cx + ff_d(cf[1]),
                   Mt * c.cy + ff_d(cf[2]), Mt * c.cz + ff_d(cf[3]), ff_d(cgc[9]), ff_d(cgc[10]), mbe, r2, R_max,
                   V_max, P, B, c.cx, c.cy, c.cz, hout);
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
  PT_BEGIN;
  keys32(c, B, W);
  PT_MARK(W, 0);
  bool ok = radial_sort(W.keyA, W.idxA, W.keyB, W.idxB, c.o, c.n, stack, W.stack_cap, S.sort);
  PT_MARK(W, 1);
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
  PT_MARK(W, 2);
  double mo[3];
  ff Phi0;
  uint64_t n1 = rvir0_phi(c, B, W, P, S, &Phi0, mo, &nret);
  PT_MARK(W, 3);
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
    PT_MARK(W, 4);
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
        PT_MARK(W, 5);
        if (ncur >= (uint64_t)P.MINPART) profiles32(c, B, W, P, S, n1, ncur, Phi0_used, hout, &nret);
        PT_MARK(W, 6);
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
  PT_MARK(W, 7);
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
