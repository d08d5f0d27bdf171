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

constexpr int kItems = 4;                 // consecutive slots per thread (default; per class: F32Smem::kItems)
constexpr double kEps64 = 1.1102230246251565e-16;
constexpr float kBand1 = 2e-5f;      // relative band of the FP32 decisions

// Per-thread staging of a tile's per-slot inputs (classes with >= 128
// threads): each thread copies its own four slots of every array with
// cp.async one tile ahead, into one of two buffers, and reads them back after
// cp.async.wait_group -- no other thread touches its bytes, so no barrier is
// needed.  Layout of a buffer: the flags (4 B per thread), eleven 16-byte
// arrays (w, vx, vy, vz, dx, dy, dz, d hi, d lo, q hi, q lo) and five 32-byte
// arrays (potential prefix, fixed-point w, vx, vy, vz), each thread-major.
template <int T>
struct StageGeo {
  static constexpr int k16 = T * 4;
  static constexpr int k32 = k16 + 11 * T * 16;
  static constexpr int kBuf = k32 + 5 * T * 32;
};

template <class SS, int T = 256>
struct F32Smem {
  static constexpr int kT = T;
  static constexpr int kItems = T >= 128 ? 4 : 2;   // consecutive slots per thread
  static constexpr int kStage = T >= 128 ? 2 * StageGeo<T>::kBuf : 0;
  union {
    SS sort;
    __align__(16) unsigned char stage[kStage > 0 ? kStage : 16];
  };
  float scan[32 * 2 * 16];
  uint4 rec[16 * 4];       // two halves of 8 warp records (WRec, 64 bytes each)
  float eup[kMaxBins], edn[kMaxBins];   // float neighbours of the bin edges
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
  // slots whose FP64 re-test stayed inside the reference-rounding band in the
  // last unbinding pass, with the flag the pass settled on
  int amb_n, amb_ovf;
  long long amb_slot[32];
  int amb_b[32];
  double amb_m[32];
};

struct Ctx32 {
  int h;
  uint64_t o, n;
  uint64_t s;              // first slot of the halo's work arrays (a multiple of 4)
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
// Exact running sums of masses and momenta: 64-bit fixed point with a
// per-halo scale 2^s chosen so that the whole list sums below 2^61.  Integer
// addition is associative, so every block-level prefix equals the sequential
// sum of the same (rounded) terms; a term loses only bits below 2^-s.

struct Fix {
  int sm, sv;          // mass and momentum scale exponents
  float fm, fv;        // 2^sm, 2^sv
  float im, iv;        // 2^-sm, 2^-sv
  double dm, dv;       // 2^-sm, 2^-sv
  double vq;           // bound of the quantisation error of a bulk-velocity component
  float vqf;           // 3 vq v_fac (FP32 test)
  long long w1;        // weight 1 in fixed point
};

__device__ __forceinline__ float pow2f(int k) { return __int_as_float((k + 127) << 23); }

// A float rounded to the nearest 64-bit integer (ties to even), |x| < 2^62,
// by integer arithmetic: the 64-bit conversion instructions issue on the
// FP64 pipe, which this GPU runs at a small fraction of the FP32 rate, and
// this runs once per list entry and array.
__device__ __forceinline__ long long f2ll_rn(float x) {
  const unsigned u = __float_as_uint(x);
  const int e = (int)((u >> 23) & 0xffu);
  if (e < 126) return 0;   // |x| < 1/2 (zero and subnormals included)
  const unsigned long long m = (u & 0x7fffffu) | 0x800000u;
  unsigned long long r;
  if (e >= 150) {
    r = m << (e - 150);   // an integer already
  } else {
    const int k = 150 - e;   // 1 .. 24 fraction bits
    const unsigned long long q = m >> k, rem = m & ((1ull << k) - 1ull), half = 1ull << (k - 1);
    r = q + ((rem > half || (rem == half && (q & 1ull))) ? 1ull : 0ull);
  }
  return (u >> 31) ? -(long long)r : (long long)r;
}

// round(x 2^s) for |x 2^s| < 2^62 (the scaling by 2^s is exact)
__device__ __forceinline__ long long f2fix(float x, float scale) { return f2ll_rn(__fmul_rn(x, scale)); }

// w v in fixed point: the exact product (two floats) rounded to the grid
__device__ __forceinline__ long long wv2fix(float w, float v, float scale, int has_w) {
  if (!has_w) return f2fix(v, scale);
  float p = __fmul_rn(w, v);
  float e = __fmaf_rn(w, v, -p);
  return f2fix(p, scale) + f2fix(e, scale);
}

// 64-bit integer -> float without 64-bit conversion instructions (those
// run at the FP64 rate): two 32-bit conversions, one rounding each, and an
// FMA (within 1.5 ulp)
__device__ __forceinline__ float l2f(long long v) {
  float hi = __int2float_rn((int)(v >> 32));
  float lo = __uint2float_rn((unsigned)(v & 0xffffffffll));
  return __fmaf_rn(hi, 4294967296.f, lo);
}

// fixed point -> float-float: three exact 24-bit pieces (relative error
// <= 2^-47)
__device__ __forceinline__ ff i2ff(long long v, float iscale) {
  float f2 = __fmul_rn(__int2float_rn((int)(v >> 48)), 281474976710656.f);                // 2^48
  float f1 = __fmul_rn(__uint2float_rn((unsigned)(v >> 24) & 0xffffffu), 16777216.f);   // 2^24
  float f0 = __uint2float_rn((unsigned)v & 0xffffffu);
  ff r = ff_add(two_sum(f2, f1), fff(f0));
  return ff{__fmul_rn(r.hi, iscale), __fmul_rn(r.lo, iscale)};
}

__device__ __forceinline__ float i2f(long long v, float iscale) { return __fmul_rn(l2f(v), iscale); }

// mass prefix as float-float: with unit weights it is the particle count
// (exact in one float below 2^24), else the fixed-point sum
__device__ __forceinline__ ff mass_ff(long long fixsum, long long count, int has_w, float iscale) {
  if (!has_w && count < (1ll << 24)) return ff{__int2float_rn((int)count), 0.f};   // exact: a 32-bit conversion
  return i2ff(fixsum, iscale);
}

// Four consecutive slots of a per-slot array.  Halo slot ranges start at a
// multiple of 4 (slot_base) and tiles at multiples of 4 slots, so every group
// is 16-byte aligned (8-byte arrays: 32-byte); a group may run up to 3 slots
// past the halo's last slot, into its own alignment gap (never another
// halo's slots).
__device__ __forceinline__ void ld4f(const float* p, float (&v)[4]) {
  float4 t = *reinterpret_cast<const float4*>(p);
  v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
}
__device__ __forceinline__ void ld4f(const float* p, float (&v)[2]) {
  float2 t = *reinterpret_cast<const float2*>(p);
  v[0] = t.x; v[1] = t.y;
}
__device__ __forceinline__ void ld4ff(const double* p, ff (&v)[4]) {
  const float4* q = reinterpret_cast<const float4*>(p);
  float4 a = q[0], b = q[1];
  v[0] = ff{a.x, a.y}; v[1] = ff{a.z, a.w}; v[2] = ff{b.x, b.y}; v[3] = ff{b.z, b.w};
}
__device__ __forceinline__ void ld4ff(const double* p, ff (&v)[2]) {
  float4 a = *reinterpret_cast<const float4*>(p);
  v[0] = ff{a.x, a.y}; v[1] = ff{a.z, a.w};
}
__device__ __forceinline__ unsigned ld4u8(const uint8_t* p) { return *reinterpret_cast<const unsigned*>(p); }
// N consecutive flags (N = 4 or 2) as the low bytes of an unsigned, and back
template <int N>
__device__ __forceinline__ unsigned ldnu8(const uint8_t* p) {
  if (N == 4) return *reinterpret_cast<const unsigned*>(p);
  return *reinterpret_cast<const unsigned short*>(p);
}
template <int N>
__device__ __forceinline__ void stnu8(uint8_t* p, unsigned v) {
  if (N == 4) *reinterpret_cast<unsigned*>(p) = v;
  else *reinterpret_cast<unsigned short*>(p) = (unsigned short)v;
}
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
  unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

__device__ __forceinline__ void ld4ll(const long long* p, long long (&v)[4]) {
  const longlong2* q = reinterpret_cast<const longlong2*>(p);
  longlong2 a = q[0], b = q[1];
  v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
}
__device__ __forceinline__ void ld4ll(const long long* p, long long (&v)[2]) {
  longlong2 a = *reinterpret_cast<const longlong2*>(p);
  v[0] = a.x; v[1] = a.y;
}

// fixed-point weights and momenta of the sorted slots (FP32C), written once
// by the gather into the FP64 form's offset arrays
__device__ __forceinline__ long long* fix_w(const Work& W) { return reinterpret_cast<long long*>(W.sd); }
__device__ __forceinline__ long long* fix_x(const Work& W) { return reinterpret_cast<long long*>(W.sdx); }
__device__ __forceinline__ long long* fix_y(const Work& W) { return reinterpret_cast<long long*>(W.sdy); }
__device__ __forceinline__ long long* fix_z(const Work& W) { return reinterpret_cast<long long*>(W.sdz); }

// issue the copies of this thread's four slots (i0..i0+3) of a tile into
// stage buffer `buf`; always commits one group (empty past the list end)
template <class SM>
__device__ __forceinline__ void stage_issue(SM& S, int buf, const Work& W, uint64_t o, uint64_t i0, uint64_t n1,
                                            int has_w) {
  using G = StageGeo<SM::kT>;
  constexpr int T = SM::kT;
  unsigned char* b = S.stage + buf * G::kBuf;
  const int t = threadIdx.x;
  if (i0 < n1) {
    const uint64_t s = o + i0;
    cp_async4(b + t * 4, W.flag + s);
    const float* a16[11] = {W.sw, W.svx, W.svy, W.svz, W.fdx, W.fdy, W.fdz, W.fdh, W.fdl, W.fqh, W.fql};
#pragma unroll
    for (int a = 0; a < 11; a++) {
      if (a == 0 && !has_w) continue;
      cp_async16(b + G::k16 + a * T * 16 + t * 16, a16[a] + s);
    }
    const unsigned char* a32[5] = {reinterpret_cast<const unsigned char*>(W.phi + s),
                                   reinterpret_cast<const unsigned char*>(fix_w(W) + s),
                                   reinterpret_cast<const unsigned char*>(fix_x(W) + s),
                                   reinterpret_cast<const unsigned char*>(fix_y(W) + s),
                                   reinterpret_cast<const unsigned char*>(fix_z(W) + s)};
#pragma unroll
    for (int a = 0; a < 5; a++) {
      if (a == 1 && !has_w) continue;
      cp_async16(b + G::k32 + a * T * 32 + t * 32, a32[a]);
      cp_async16(b + G::k32 + a * T * 32 + t * 32 + 16, a32[a] + 16);
    }
  }
  cp_async_commit();
}

template <class SM>
__device__ __forceinline__ const unsigned char* stage_buf(SM& S, int buf) {
  return S.stage + buf * StageGeo<SM::kT>::kBuf;
}
template <class SM>
__device__ __forceinline__ void st_f(const unsigned char* b, int a, float (&v)[4]) {
  ld4f(reinterpret_cast<const float*>(b + StageGeo<SM::kT>::k16 + a * SM::kT * 16 + threadIdx.x * 16), v);
}
template <class SM>
__device__ __forceinline__ void st_ll(const unsigned char* b, int a, long long (&v)[4]) {
  ld4ll(reinterpret_cast<const long long*>(b + StageGeo<SM::kT>::k32 + a * SM::kT * 32 + threadIdx.x * 32), v);
}
template <class SM>
__device__ __forceinline__ void st_ff(const unsigned char* b, int a, ff (&v)[4]) {
  ld4ff(reinterpret_cast<const double*>(b + StageGeo<SM::kT>::k32 + a * SM::kT * 32 + threadIdx.x * 32), v);
}
template <class SM>
__device__ __forceinline__ unsigned st_flag(const unsigned char* b) {
  return *reinterpret_cast<const unsigned*>(b + threadIdx.x * 4);
}

// per-halo scales from the list length and the largest weight / velocity
__device__ __forceinline__ Fix make_fix(uint64_t n, float wmax, float wmin, float vmax, double v_fac) {
  Fix F;
  double nb = (double)n + 2.0;
  int e;
  frexp(nb * (double)wmax, &e);
  F.sm = min(max(61 - e, -100), 100);
  double bv = nb * (double)wmax * (double)vmax;
  if (!(bv > 1e-30)) bv = 1e-30;
  frexp(bv, &e);
  F.sv = min(max(61 - e, -100), 100);
  F.fm = pow2f(F.sm); F.im = pow2f(-F.sm);
  F.fv = pow2f(F.sv); F.iv = pow2f(-F.sv);
  F.dm = ldexp(1.0, -F.sm); F.dv = ldexp(1.0, -F.sv);
  // |V_j - exact| <= (j lsb_v / 2 + |V_j| j lsb_m / 2) / (j wmin); x2 slack
  double wl = wmin > 0.f ? (double)wmin : 1e-30;
  F.vq = (F.dv + (double)vmax * F.dm) / wl;
  F.vqf = (float)(3.0 * F.vq * v_fac);
  F.w1 = f2fix(1.f, F.fm);
  return F;
}

// ---------------------------------------------------------------------------
// One-barrier block scans.  Each warp scans its lanes with shuffles and
// leaves its total in a 64-byte record; after one barrier every thread folds
// the records of the lower warps in warp order (a fixed order, so results
// are deterministic).  Successive calls alternate between the two halves of
// the record buffer (`par`, uniform over the block), so a record is never
// rewritten while a slower warp may still be reading it.

struct __align__(16) WRec {
  long long a[4];      // int64 sums
  long long slot;      // payload slot of the warp's last valid lane
  int cnt, valid;
  float p[4];          // payload of the warp's last valid lane
};

template <class SM>
__device__ __forceinline__ WRec* wrec(SM& S, int& par) {
  WRec* r = reinterpret_cast<WRec*>(&S.rec[(par & 1) * 32]);
  par++;
  return r;
}

// 4 int64 sums + a count + the "last valid" payload (4 floats and a slot).
// ex/excnt: sums over lower threads; pe/pslot: payload of the nearest lower
// valid thread (carry cp/cslot if none); tot/pb: block totals / last.
template <class SM>
__device__ __forceinline__ void scan_bound(const long long (&a)[4], int cnt, bool has, const float (&p)[4],
                                           long long slot, const float (&cp)[4], long long cslot,
                                           long long (&ex)[4], long long (&tot)[4], int& excnt, int& totcnt,
                                           float (&pe)[4], long long& pslot, float (&pb)[4], long long& pbslot,
                                           SM& S, int& par) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  long long inc[4];
  int ic = cnt;
#pragma unroll
  for (int c = 0; c < 4; c++) inc[c] = a[c];
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
#pragma unroll
    for (int c = 0; c < 4; c++) {
      long long y = __shfl_up_sync(FULL, inc[c], off);
      if (lane >= off) inc[c] += y;
    }
    int yc = __shfl_up_sync(FULL, ic, off);
    if (lane >= off) ic += yc;
  }
  const unsigned m = __ballot_sync(FULL, has);
  const unsigned below = m & ((1u << lane) - 1u);
  const int src = below ? (31 - __clz(below)) : 0;
  const int ll = m ? (31 - __clz(m)) : 0;
  float mp[4], wp[4];
#pragma unroll
  for (int j = 0; j < 4; j++) {
    mp[j] = __shfl_sync(FULL, p[j], src);
    wp[j] = __shfl_sync(FULL, p[j], ll);
  }
  long long ms = __shfl_sync(FULL, slot, src);
  long long wsl = __shfl_sync(FULL, slot, ll);
  WRec* R = wrec(S, par);
  if (lane == 31) {
    WRec& r = R[wid];
#pragma unroll
    for (int c = 0; c < 4; c++) r.a[c] = inc[c];
    r.cnt = ic;
    r.valid = m != 0u;
#pragma unroll
    for (int j = 0; j < 4; j++) r.p[j] = wp[j];
    r.slot = wsl;
  }
  __syncthreads();
  long long e[4] = {0, 0, 0, 0};
  int ec = 0;
  float lp[4] = {cp[0], cp[1], cp[2], cp[3]};
  long long ls = cslot;
  for (int w = 0; w < wid; w++) {
    const WRec& r = R[w];
#pragma unroll
    for (int c = 0; c < 4; c++) e[c] += r.a[c];
    ec += r.cnt;
    if (r.valid) {
#pragma unroll
      for (int j = 0; j < 4; j++) lp[j] = r.p[j];
      ls = r.slot;
    }
  }
  long long t[4] = {e[0], e[1], e[2], e[3]};
  int tc = ec;
  float bp[4] = {lp[0], lp[1], lp[2], lp[3]};
  long long bs = ls;
  for (int w = wid; w < nw; w++) {
    const WRec& r = R[w];
#pragma unroll
    for (int c = 0; c < 4; c++) t[c] += r.a[c];
    tc += r.cnt;
    if (r.valid) {
#pragma unroll
      for (int j = 0; j < 4; j++) bp[j] = r.p[j];
      bs = r.slot;
    }
  }
#pragma unroll
  for (int c = 0; c < 4; c++) {
    ex[c] = e[c] + (inc[c] - a[c]);
    tot[c] = t[c];
  }
  excnt = ec + (ic - cnt);
  totcnt = tc;
#pragma unroll
  for (int j = 0; j < 4; j++) {
    pe[j] = below ? mp[j] : lp[j];
    pb[j] = bp[j];
  }
  pslot = below ? ms : ls;
  pbslot = bs;
}

// one float-float sum (exclusive prefix and block total) and one int64
// minimum (block minimum)
template <class SM>
__device__ __forceinline__ void scan_ff_min(ff v, long long mn, ff& ex, ff& tot, long long& bmin, SM& S, int& par) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  ff inc = v;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    ff y = {__shfl_up_sync(FULL, inc.hi, off), __shfl_up_sync(FULL, inc.lo, off)};
    if (lane >= off) inc = ff_add(y, inc);
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    long long o = __shfl_xor_sync(FULL, mn, off);
    mn = o < mn ? o : mn;
  }
  ff prev = {__shfl_up_sync(FULL, inc.hi, 1), __shfl_up_sync(FULL, inc.lo, 1)};
  WRec* R = wrec(S, par);
  if (lane == 31) {
    R[wid].p[0] = inc.hi;
    R[wid].p[1] = inc.lo;
    R[wid].a[0] = mn;
  }
  __syncthreads();
  ff e = ffz();
  long long bm = 0x7fffffffffffffffll;
  for (int w = 0; w < wid; w++) {
    e = ff_add(e, ff{R[w].p[0], R[w].p[1]});
    bm = R[w].a[0] < bm ? R[w].a[0] : bm;
  }
  ff t = e;
  for (int w = wid; w < nw; w++) {
    t = ff_add(t, ff{R[w].p[0], R[w].p[1]});
    bm = R[w].a[0] < bm ? R[w].a[0] : bm;
  }
  ex = lane > 0 ? ff_add(e, prev) : e;
  tot = t;
  bmin = bm;
}

// one int64 sum: exclusive prefix and block total
template <class SM>
__device__ __forceinline__ void scan_i64(long long v, long long& ex, long long& tot, SM& S, int& par) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  long long inc = v;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    long long y = __shfl_up_sync(FULL, inc, off);
    if (lane >= off) inc += y;
  }
  WRec* R = wrec(S, par);
  if (lane == 31) R[wid].a[0] = inc;
  __syncthreads();
  long long e = 0;
  for (int w = 0; w < wid; w++) e += R[w].a[0];
  long long t = e;
  for (int w = wid; w < nw; w++) t += R[w].a[0];
  ex = e + (inc - v);
  tot = t;
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

// key -> squared distance (box units^2) as float-float
__device__ __forceinline__ ff key_d2(uint64_t key) {
  if (key == 0) return ffz();
  int E = (int)(key >> 56) - 1;
  unsigned long long mant = (1ull << 56) | (key & ((1ull << 56) - 1));
  unsigned long long h24 = mant >> 33, l24 = (mant >> 9) & 0xffffffull;
  // value = mant * 2^(E-56) * 2^-124
  int eh = E - 56 - 124 + 33, el = E - 56 - 124 + 9;
  // two power-of-two factors keep each in the normal range (eh >= -147)
  float hi = __fmul_rn(__fmul_rn(__uint2float_rn((unsigned)h24), pow2f(eh + 64)), pow2f(-64));
  float lo = __fmul_rn(__fmul_rn(__uint2float_rn((unsigned)l24), pow2f(el + 64)), pow2f(-64));
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
// squared-distance keys of the list; lim = {max |v| component, max w, min w}
template <class SM>
static __device__ void keys32(const Ctx32& c, const DevBatch& B, const Work& W, const DevParams& P, SM& S,
                              float (&lim)[3]) {
  constexpr int G = 8;   // entries in flight per thread
  float vm = 0.f, wx = 0.f, wn = 3.0e38f;
  for (uint64_t base = 0; base < c.n; base += (uint64_t)blockDim.x * G) {
    float px[G], py[G], pz[G], pvx[G], pvy[G], pvz[G], pw[G];
    unsigned long long pg[G];
#pragma unroll
    for (int k = 0; k < G; k++) {
      uint64_t i = base + threadIdx.x + (uint64_t)k * blockDim.x;
      px[k] = py[k] = pz[k] = pvx[k] = pvy[k] = pvz[k] = 0.f;
      pw[k] = 1.f;
      pg[k] = 0;
      if (i < c.n) {
        const uint64_t e = c.o + i;
        px[k] = __ldg(B.x + e); py[k] = __ldg(B.y + e); pz[k] = __ldg(B.z + e);
        pvx[k] = __ldg(B.vx + e); pvy[k] = __ldg(B.vy + e); pvz[k] = __ldg(B.vz + e);
        pg[k] = B.gidx ? __ldg(reinterpret_cast<const unsigned long long*>(B.gidx) + e) : e;
        if (B.w) pw[k] = __ldg(B.w + e);
      }
    }
#pragma unroll
    for (int k = 0; k < G; k++) {
      uint64_t i = base + threadIdx.x + (uint64_t)k * blockDim.x;
      if (i >= c.n) continue;
      long long dx = wrapfix(fixp(px[k]) - c.fx);
      long long dy = wrapfix(fixp(py[k]) - c.fy);
      long long dz = wrapfix(fixp(pz[k]) - c.fz);
      W.keyA[c.s + i] = sqkey(dx, dy, dz);
      W.idxA[c.s + i] = (uint32_t)i;
      // the entry as one 32-byte record: the gather reads one sector per entry
      W.rec[2 * (c.s + i)] = make_float4(px[k], py[k], pz[k], pvx[k]);
      W.rec[2 * (c.s + i) + 1] = make_float4(pvy[k], pvz[k], __uint_as_float((unsigned)pg[k]),
                                             __uint_as_float((unsigned)(pg[k] >> 32)));
      vm = fmaxf(vm, fmaxf(fabsf(pvx[k]), fmaxf(fabsf(pvy[k]), fabsf(pvz[k]))));
      wx = fmaxf(wx, pw[k]);
      wn = fminf(wn, pw[k]);
    }
  }
  for (int off = 16; off > 0; off >>= 1) {
    vm = fmaxf(vm, __shfl_xor_sync(0xffffffffu, vm, off));
    wx = fmaxf(wx, __shfl_xor_sync(0xffffffffu, wx, off));
    wn = fminf(wn, __shfl_xor_sync(0xffffffffu, wn, off));
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (lane == 0) { S.scan[3 * wid] = vm; S.scan[3 * wid + 1] = wx; S.scan[3 * wid + 2] = wn; }
  __syncthreads();
  lim[0] = 0.f; lim[1] = 0.f; lim[2] = 3.0e38f;
  for (int w = 0; w < nw; w++) {
    lim[0] = fmaxf(lim[0], S.scan[3 * w]);
    lim[1] = fmaxf(lim[1], S.scan[3 * w + 1]);
    lim[2] = fminf(lim[2], S.scan[3 * w + 2]);
  }
  if (!P.has_w) { lim[1] = 1.f; lim[2] = 1.f; }
  __syncthreads();
}

// Runs of adjacent keys closer than the reference's rounding are put in the
// order of the reference's FP64 keys (ties by slot).  Returns exact ties.
static __device__ __noinline__ unsigned long long fix_near_ties(const Ctx32& c, const DevBatch& B, const Work& W) {
  unsigned long long ties = 0;
  const uint64_t o = c.s;
  constexpr int G = 8;   // slots in flight per thread
  // mark ambiguous adjacent pairs first (flag is free until gather32)
  for (uint64_t base = 0; base < c.n; base += (uint64_t)blockDim.x * G) {
    uint64_t k0[G], k1[G];
#pragma unroll
    for (int k = 0; k < G; k++) {
      const uint64_t i = base + threadIdx.x + (uint64_t)k * blockDim.x;
      k0[k] = i + 1 < c.n ? W.keyA[o + i] : 0ull;
      k1[k] = i + 1 < c.n ? W.keyA[o + i + 1] : ~0ull;
    }
#pragma unroll
    for (int k = 0; k < G; k++) {
      const uint64_t i = base + threadIdx.x + (uint64_t)k * blockDim.x;
      if (i < c.n) W.flag[o + i] = (i + 1 < c.n && k1[k] - k0[k] <= 512ull) ? 1 : 0;
    }
  }
  __syncthreads();
  // runs of flagged pairs, each sorted by the thread that holds its start
  for (uint64_t base = 0; base + 1 < c.n; base += (uint64_t)blockDim.x * G) {
    unsigned st = 0u;   // bit k: slot base + thread + k blocks starts a run
#pragma unroll
    for (int k = 0; k < G; k++) {
      const uint64_t i = base + threadIdx.x + (uint64_t)k * blockDim.x;
      const bool f = i + 1 < c.n && W.flag[o + i];
      const bool fp = i + 1 < c.n && i > 0 && W.flag[o + i - 1];
      if (f && !fp) st |= 1u << k;
    }
    if (st == 0u) continue;
#pragma unroll 1
    for (int k = 0; k < G; k++) {
      if (!((st >> k) & 1u)) continue;
      const uint64_t i = base + threadIdx.x + (uint64_t)k * blockDim.x;
      // run [i, j] of mutually ambiguous neighbours, owned by this thread
      uint64_t j = i + 1;
      while (j + 1 < c.n && W.flag[o + j]) j++;
      // insertion sort of the run by (reference key, slot)
      for (uint64_t a = i + 1; a <= j; a++) {
        uint32_t sa = W.idxA[o + a];
        uint64_t ka = W.keyA[o + a];
        double ra = ref_key(B, c.o + sa, c.cx, c.cy, c.cz);
        uint64_t b = a;
        while (b > i) {
          uint32_t sb = W.idxA[o + b - 1];
          double rb = ref_key(B, c.o + sb, c.cx, c.cy, c.cz);
          if (rb < ra || (rb == ra && sb < sa)) break;
          W.idxA[o + b] = sb;
          W.keyA[o + b] = W.keyA[o + b - 1];
          b--;
        }
        W.idxA[o + b] = sa;
        W.keyA[o + b] = ka;
      }
      for (uint64_t a = i; a < j; a++) {
        double r0 = ref_key(B, c.o + W.idxA[o + a], c.cx, c.cy, c.cz);
        double r1 = ref_key(B, c.o + W.idxA[o + a + 1], c.cx, c.cy, c.cz);
        if (r0 == r1) ties++;
      }
    }
  }
  __syncthreads();
  return ties;
}

// gathers the sorted slots, with the fixed-point weights and momenta
static __device__ void gather32(const Ctx32& c, const DevBatch& B, const Work& W, const DevParams& P, const Fix& F) {
  const float s62 = pow2f(-62);
  constexpr int G = 8;   // entries in flight per thread (the reads are random)
  for (uint64_t base = 0; base < c.n; base += (uint64_t)blockDim.x * G) {
    uint32_t jj[G];
    float px[G], py[G], pz[G], pvx[G], pvy[G], pvz[G], pw[G];
    unsigned pgl[G], pgh[G];
#pragma unroll
    for (int k = 0; k < G; k++) {
      uint64_t i = base + threadIdx.x + (uint64_t)k * blockDim.x;
      jj[k] = i < c.n ? W.idxA[c.s + i] : 0u;
    }
#pragma unroll
    for (int k = 0; k < G; k++) {
      uint64_t i = base + threadIdx.x + (uint64_t)k * blockDim.x;
      px[k] = py[k] = pz[k] = pvx[k] = pvy[k] = pvz[k] = 0.f;
      pw[k] = 1.f;
      if (i < c.n) {
        float4 r0 = W.rec[2 * (c.s + jj[k])], r1 = W.rec[2 * (c.s + jj[k]) + 1];
        px[k] = r0.x; py[k] = r0.y; pz[k] = r0.z; pvx[k] = r0.w; pvy[k] = r1.x; pvz[k] = r1.y;
        pgl[k] = __float_as_uint(r1.z);
        pgh[k] = __float_as_uint(r1.w);
        if (B.w) pw[k] = __ldg(B.w + c.o + jj[k]);
      }
    }
#pragma unroll
    for (int k = 0; k < G; k++) {
      uint64_t i = base + threadIdx.x + (uint64_t)k * blockDim.x;
      if (i >= c.n) continue;
      uint64_t s = c.s + i;
      long long dx = wrapfix(fixp(px[k]) - c.fx);
      long long dy = wrapfix(fixp(py[k]) - c.fy);
      long long dz = wrapfix(fixp(pz[k]) - c.fz);
      ff d2 = key_d2(sqkey(dx, dy, dz));
      ff d = ff_sqrt(d2);
      ff q = d2.hi > 0.f ? ff_div(fff(1.f), d2) : ffz();
      W.fdh[s] = d.hi;
      W.fdl[s] = d.lo;
      W.fqh[s] = q.hi;
      W.fql[s] = q.lo;
      // offsets as float-float (hi kept for the FP32 arithmetic, lo for the
      // centre-of-mass sums)
      ff ox = i2ff(dx, s62), oy = i2ff(dy, s62), oz = i2ff(dz, s62);
      W.fdx[s] = ox.hi;
      W.fdy[s] = oy.hi;
      W.fdz[s] = oz.hi;
      W.fdxl[s] = ox.lo;
      W.fdyl[s] = oy.lo;
      W.fdzl[s] = oz.lo;
      W.svx[s] = pvx[k];
      W.svy[s] = pvy[k];
      W.svz[s] = pvz[k];
      W.sw[s] = pw[k];
      W.seid[s] = jj[k];
      W.keyB[s] = ((unsigned long long)pgh[k] << 32) | pgl[k];   // output id of the slot
      W.flag[s] = 1;
      fix_w(W)[s] = f2fix(pw[k], F.fm);
      fix_x(W)[s] = wv2fix(pw[k], pvx[k], F.fv, P.has_w);
      fix_y(W)[s] = wv2fix(pw[k], pvy[k], F.fv, P.has_w);
      fix_z(W)[s] = wv2fix(pw[k], pvz[k], F.fv, P.has_w);
    }
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

// the same with the mass prefixes exact floats (unit weights: particle
// counts M and M - 1)
__device__ __forceinline__ ff phi_termq_c(float M, float Mp, ff d, ff q, ff dp, ff qp) {
  if (!dpos(d)) return ffz();
  ff In = ff_mulf(q, M);
  ff Ip = dpos(dp) ? ff_mulf(qp, Mp) : ffz();
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
// the first unbinding iteration (stored, float-float inclusive, in phi for
// the slots that stay).  Returns n1; sets *Phi0 (float-float).
template <class SM>
static __device__ uint64_t rvir0_phi(const Ctx32& c, const DevBatch& B, const Work& W, const DevParams& P, SM& S,
                                     const Fix& F, ff* Phi0, double* mo, unsigned* nret, int& par) {
  constexpr int kItems = SM::kItems;
  const float V43f = (float)(4. * kPi / 3.);
  const float ovk = __fmul_rn(__fmul_rn(P.f_ovlim, P.f_rvrf), V43f);
  float2* phs = reinterpret_cast<float2*>(W.phi + c.s);
  long long cM = 0;
  ff cPhi = ffz();
  long long stop = -1;
  ff stopM = ffz(), stopD = ffz(), stopPhi = ffz();
  const uint64_t tile = (uint64_t)blockDim.x * kItems;
  for (uint64_t base = 0; base < c.n; base += tile) {
    uint64_t i0 = base + (uint64_t)threadIdx.x * kItems;
    float w[kItems];
    ff d[kItems], q[kItems], dp, qp;
    long long fw[kItems], acc = 0;
    {
      float dh[kItems], dl[kItems], qh[kItems], ql[kItems];
#pragma unroll
      for (int k = 0; k < kItems; k++) { w[k] = 1.f; fw[k] = F.w1; dh[k] = dl[k] = qh[k] = ql[k] = 0.f; }
      if (i0 < c.n) {
        if (P.has_w) { ld4f(W.sw + c.s + i0, w); ld4ll(fix_w(W) + c.s + i0, fw); }
        ld4f(W.fdh + c.s + i0, dh); ld4f(W.fdl + c.s + i0, dl);
        ld4f(W.fqh + c.s + i0, qh); ld4f(W.fql + c.s + i0, ql);
      }
#pragma unroll
      for (int k = 0; k < kItems; k++) {
        bool v = i0 + k < c.n;
        if (!v) { w[k] = 0.f; fw[k] = 0; }
        d[k] = v ? ff{dh[k], dl[k]} : ffz();
        q[k] = v ? ff{qh[k], ql[k]} : ffz();
        acc += fw[k];
      }
    }
    bool hasp = i0 > 0 && i0 < c.n;
    dp = hasp ? ff{W.fdh[c.s + i0 - 1], W.fdl[c.s + i0 - 1]} : ffz();
    qp = hasp ? ff{W.fqh[c.s + i0 - 1], W.fql[c.s + i0 - 1]} : ffz();
    long long exM, totM;
    scan_i64(acc, exM, totM, S, par);
    long long rM = cM + exM;
    ff term[kItems], accT = ffz(), Mk[kItems];
    long long myfail = 0x7fffffffffffffffll;
#pragma unroll
    for (int k = 0; k < kItems; k++) {
      uint64_t i = i0 + k;
      rM += fw[k];
      Mk[k] = mass_ff(rM, (long long)(i + 1), P.has_w, F.im);
      ff prevd = k == 0 ? dp : d[k - 1];
      ff prevq = k == 0 ? qp : q[k - 1];
      if (i < c.n) {
        const bool cnt_mass = !P.has_w && i + 1 < (1ull << 24);
        accT = ff_add(accT, cnt_mass ? phi_termq_c(__uint2float_rn((unsigned)(i + 1)), __uint2float_rn((unsigned)i),
                                                   d[k], q[k], prevd, prevq)
                                     : phi_termq(Mk[k], w[k], d[k], q[k], prevd, prevq));
      }
      term[k] = accT;     // thread-local inclusive
      if (i < c.n && myfail == 0x7fffffffffffffffll) {
        float rhs = __fmul_rn(ovk, __fmul_rn(__fmul_rn(d[k].hi, d[k].hi), d[k].hi));
        if (!(Mk[k].hi > __fmul_rn(rhs, 1.f + 4.f * kBand1)) && ov_fail(c, B, W, P, c.s + i, Mk[k], d[k], nret))
          myfail = (long long)i;
      }
    }
    ff exT, totT;
    long long f;
    scan_ff_min(accT, myfail, exT, totT, f, S, par);
    ff basePhi = ff_add(cPhi, exT);
#pragma unroll
    for (int k = 0; k < kItems; k++) {
      long long i = (long long)(i0 + k);
      if (i < (long long)c.n && i <= f) {
        ff v = ff_add(basePhi, term[k]);
        phs[i] = make_float2(v.hi, v.lo);
      }
    }
    if (f != 0x7fffffffffffffffll) {
      if ((long long)i0 <= f && f < (long long)(i0 + kItems)) {
        int k = (int)(f - (long long)i0);
        ff phi = ff_add(basePhi, term[k]);
        S.bf[0] = Mk[k].hi; S.bf[1] = Mk[k].lo; S.bf[2] = d[k].hi; S.bf[3] = d[k].lo;
        S.bf[4] = phi.hi; S.bf[5] = phi.lo;
      }
      __syncthreads();
      stop = f;
      stopM = ff{S.bf[0], S.bf[1]}; stopD = ff{S.bf[2], S.bf[3]}; stopPhi = ff{S.bf[4], S.bf[5]};
      __syncthreads();
      break;
    }
    cM += totM;
    cPhi = ff_add(cPhi, totT);
  }
  uint64_t n1;
  if (stop < 0) {
    n1 = c.n;
    stopM = i2ff(cM, F.im);
    stopPhi = cPhi;
    stopD = ff{W.fdh[c.s + c.n - 1], W.fdl[c.s + c.n - 1]};
  } else {
    n1 = (uint64_t)stop + 1;
  }
  // outputs in FP64 for the cut particle (as rem_outsideRvir computes them)
  double R = ref_dist(c, B, W, c.s + n1 - 1);
  double M = ff_d(stopM);
  double V = 4. * kPi / 3. * (R * R * R);
  mo[0] = M;
  mo[1] = R;
  mo[2] = M / V * P.rho_fac / P.rho_vir;
  *Phi0 = ff_add(stopPhi, ff_div(stopM, stopD));
  for (uint64_t i = n1 + threadIdx.x; i < c.n; i += blockDim.x) W.flag[c.s + i] = 0;
  __syncthreads();
  return n1;
}

// ---------------------------------------------------------------------------
// FP64 re-test of a bound decision (reference operation order, own inputs,
// exact fixed-point running sums, float-float potential).  Sets *amb when the
// result is inside the reference's rounding band.
static __device__ __noinline__ bool retest_bound(const Ctx32& c, const DevBatch& B, const Work& W, const DevParams& P,
                                             uint64_t s, uint64_t pos, uint64_t n1, double phi, double phi0,
                                             double VXc, double VYc, double VZc, double M_vel, float vmax, double vq,
                                             bool* amb) {
  uint64_t e = c.o + W.seid[s];
  double dX = wrap_s((double)B.x[e] - c.cx);
  double dY = wrap_s((double)B.y[e] - c.cy);
  double dZ = wrap_s((double)B.z[e] - c.cz);
  double d = sqrt((dX * dX + dY * dY) + dZ * dZ);
  double v_esc2 = d > kMachineZero ? (2 * fabs(phi - phi0) * P.phi_fac) : 1e30;
  double VXp = (double)B.vx[e], VYp = (double)B.vy[e], VZp = (double)B.vz[e];
  double hx = P.Hubble * (dX) * P.r_fac, hy = P.Hubble * (dY) * P.r_fac, hz = P.Hubble * (dZ) * P.r_fac;
  double dVX = (VXp - VXc / M_vel) * P.v_fac + hx;
  double dVY = (VYp - VYc / M_vel) * P.v_fac + hy;
  double dVZ = (VZp - VZc / M_vel) * P.v_fac + hz;
  double vel2 = (dVX * dVX + dVY * dVY) + dVZ * dVZ;
  double thr = P.v2_tune * v_esc2;
  // band: the reference's sequential sums differ from exact ones by at most
  // ~(j+1)u of their absolute sums; the float-float potential by ~2^-40, the
  // fixed-point bulk velocity by vq
  double g = 2.0 * ((double)pos + 64.0) * kEps64 + 9.1e-13;
  double gn = 2.0 * ((double)n1 + 64.0) * kEps64 + 9.1e-13;
  double A = fabs(phi - phi0);
  double dthr = d > kMachineZero ? thr * ((gn * fabs(phi0) * 2.0) / fmax(A, 1e-300) + 8 * kEps64) : thr * 8 * kEps64;
  double sb = (double)vmax * P.v_fac;
  double ddv = g * sb + 6.0 * kEps64 * (2.0 * sb + fabs(hx) + fabs(hy) + fabs(hz)) + vq * P.v_fac;
  double dvel2 = 2.0 * 1.7320508075688772 * sqrt(vel2) * ddv + 3.0 * ddv * ddv + 8 * kEps64 * vel2;
  if (fabs(vel2 - thr) <= 2.5 * (dthr + dvel2)) *amb = true;
  return !(vel2 > thr);
}

// FP32 bound test of a member against exact running sums (fixed point):
// 1 bound, 0 unbound, -1 inside the bound of its own rounding errors
__device__ __forceinline__ int bound32(float vx, float vy, float vz, float dx, float dy, float dz, float thr,
                                       float ethr, long long Mi, long long Xi, long long Yi, long long Zi,
                                       const Fix& F, float vf, float Hr) {
  const float fe = 5.9604645e-08f;   // 2^-24
  float rM = __frcp_rn(i2f(Mi, F.im));
  float Vx = __fmul_rn(i2f(Xi, F.iv), rM), Vy = __fmul_rn(i2f(Yi, F.iv), rM), Vz = __fmul_rn(i2f(Zi, F.iv), rM);
  float hx = __fmul_rn(Hr, dx), hy = __fmul_rn(Hr, dy), hz = __fmul_rn(Hr, dz);
  float dVX = __fadd_rn(__fmul_rn(__fsub_rn(vx, Vx), vf), hx);
  float dVY = __fadd_rn(__fmul_rn(__fsub_rn(vy, Vy), vf), hy);
  float dVZ = __fadd_rn(__fmul_rn(__fsub_rn(vz, Vz), vf), hz);
  float vel2 = __fadd_rn(__fadd_rn(__fmul_rn(dVX, dVX), __fmul_rn(dVY, dVY)), __fmul_rn(dVZ, dVZ));
  // error bound: each component a few roundings of the magnitudes involved
  // (the bulk velocity carries four), the squares and sums a few more; x2
  float mag = __fadd_rn(__fmul_rn(__fadd_rn(fabsf(vx) + fabsf(vy) + fabsf(vz), fabsf(Vx) + fabsf(Vy) + fabsf(Vz)), vf),
                        fabsf(hx) + fabsf(hy) + fabsf(hz));
  float edv = __fadd_rn(__fmul_rn(8.f * fe, mag), F.vqf);
  float sdv = fabsf(dVX) + fabsf(dVY) + fabsf(dVZ);
  float err = __fadd_rn(__fmul_rn(2.f, __fadd_rn(__fadd_rn(__fmul_rn(2.f * sdv, edv), __fmul_rn(3.f, __fmul_rn(edv, edv))),
                                                 __fmul_rn(8.f * fe, __fadd_rn(vel2, thr)))), ethr);
  float margin = __fsub_rn(thr, vel2);
  if (isfinite(margin) && isfinite(err) && fabsf(margin) > err) return margin >= 0.f ? 1 : 0;
  return -1;
}

// ---------------------------------------------------------------------------
// One rem_unbound iteration (ahf_halos.c:3336-3601) in one pass over slots
// [0, n1) with members in flag bit0 and their potential prefix (float-float,
// inclusive) in phi.  In: Phi0 of this iteration, seed slot.  Out: flag bit1
// = bound (bit0 kept); the potential prefix of the kept particles (the next
// iteration's members) written over phi; next-iteration Phi0; kept
// count/mass; last kept slot; the rvir1 candidate (first kept slot failing
// the overdensity test).  amb: some decision stayed inside the reference-
// rounding band (the caller redoes the iteration exactly).
struct IterOut {
  long long nb;
  ff Mb, Phi0n;
  long long last_slot;
  long long rv_slot;   // first failing kept slot or -1
  long long rv_cnt;    // kept particles up to and including rv_slot
  ff rv_M, rv_d;
  int amb;
  int rounds;
};

template <class SM>
static __device__ void unbind_pass(const Ctx32& c, const DevBatch& B, const Work& W, const DevParams& P, SM& S,
                                   const Fix& F, uint64_t n1, ff Phi0, uint64_t js, float vmax, IterOut& out,
                                   unsigned* nret, int& par) {
  constexpr int kItems = SM::kItems;
  const uint64_t o = c.s;
  const float vf = (float)P.v_fac, Hr = (float)(P.Hubble * P.r_fac), v2t = (float)P.v2_tune;
  const float pf2 = (float)(2.0 * P.phi_fac);
  const float V43f = (float)(4. * kPi / 3.);
  const float ovk = __fmul_rn(__fmul_rn(P.f_ovlim, P.f_rvrf), V43f);
  const double phi0d = ff_d(Phi0);
  // absolute error of the float-float potential prefixes (chained carries)
  const float ethr = (float)(((double)n1 * 3e-17 + 1e-10) * fabs(phi0d) * (double)v2t * (double)pf2);
  float2* phs = reinterpret_cast<float2*>(W.phi + o);
  const int has_w = P.has_w;
  // running sums of the bound particles; the bulk velocity starts from the
  // seed particle (ahf_halos.c:3441-3470)
  const long long sM = fix_w(W)[o + js];
  const long long sX = fix_x(W)[o + js], sY = fix_y(W)[o + js], sZ = fix_z(W)[o + js];
  long long cM = 0, cX = 0, cY = 0, cZ = 0, cNb = 0;
  float cDb[4] = {0.f, 0.f, 0.f, 0.f};
  long long cLs = -1;
  ff cPhiN = ffz();
  long long rv = -1, rvC = 0;
  ff rvM = ffz(), rvD = ffz();
  int amb_any = 0, maxr = 0;
  const uint64_t tile = (uint64_t)blockDim.x * kItems;
  if (threadIdx.x == 0) { S.amb_n = 0; S.amb_ovf = P.force_exact == 1 ? 1 : 0; }
  __syncthreads();
  if constexpr (SM::kStage > 0) stage_issue(S, 0, W, o, (uint64_t)threadIdx.x * kItems, n1, has_w);
  int tix = 0;
  for (uint64_t base = 0; base < n1; base += tile, tix++) {
    PT_T0;
    const uint64_t i0 = base + (uint64_t)threadIdx.x * kItems;
    bool m[kItems], b[kItems], ambk[kItems];
    float w[kItems], vx[kItems], vy[kItems], vz[kItems], dx[kItems], dy[kItems], dz[kItems], thr[kItems];
    ff d[kItems], q[kItems];
    long long fw[kItems], fx[kItems], fy[kItems], fz[kItems];
    unsigned f4 = 0u;
    {
      float dh[kItems], dl[kItems], qh[kItems], ql[kItems];
      ff ph[kItems];
#pragma unroll
      for (int k = 0; k < kItems; k++) {
        w[k] = 1.f;
        vx[k] = vy[k] = vz[k] = dx[k] = dy[k] = dz[k] = dh[k] = dl[k] = qh[k] = ql[k] = 0.f;
        ph[k] = ffz();
      }
#pragma unroll
      for (int k = 0; k < kItems; k++) { fw[k] = F.w1; fx[k] = fy[k] = fz[k] = 0; }
      if constexpr (SM::kStage > 0) {
        // this tile's inputs were copied one tile ago; start the next tile's
        stage_issue(S, (tix & 1) ^ 1, W, o, i0 + tile, n1, has_w);
        cp_async_wait<1>();
        if (i0 < n1) {
          const unsigned char* sb = stage_buf(S, tix & 1);
          f4 = st_flag<SM>(sb);
          if (has_w) { st_f<SM>(sb, 0, w); st_ll<SM>(sb, 1, fw); }
          st_f<SM>(sb, 1, vx); st_f<SM>(sb, 2, vy); st_f<SM>(sb, 3, vz);
          st_f<SM>(sb, 4, dx); st_f<SM>(sb, 5, dy); st_f<SM>(sb, 6, dz);
          st_f<SM>(sb, 7, dh); st_f<SM>(sb, 8, dl); st_f<SM>(sb, 9, qh); st_f<SM>(sb, 10, ql);
          st_ff<SM>(sb, 0, ph);
          st_ll<SM>(sb, 2, fx); st_ll<SM>(sb, 3, fy); st_ll<SM>(sb, 4, fz);
        }
      } else if (i0 < n1) {
        f4 = ldnu8<kItems>(W.flag + o + i0);
        if (has_w) { ld4f(W.sw + o + i0, w); ld4ll(fix_w(W) + o + i0, fw); }
        ld4f(W.svx + o + i0, vx); ld4f(W.svy + o + i0, vy); ld4f(W.svz + o + i0, vz);
        ld4f(W.fdx + o + i0, dx); ld4f(W.fdy + o + i0, dy); ld4f(W.fdz + o + i0, dz);
        ld4f(W.fdh + o + i0, dh); ld4f(W.fdl + o + i0, dl);
        ld4f(W.fqh + o + i0, qh); ld4f(W.fql + o + i0, ql);
        ld4ff(W.phi + o + i0, ph);
        ld4ll(fix_x(W) + o + i0, fx); ld4ll(fix_y(W) + o + i0, fy); ld4ll(fix_z(W) + o + i0, fz);
      }
#pragma unroll
      for (int k = 0; k < kItems; k++) {
        m[k] = i0 + k < n1 && ((f4 >> (8 * k)) & 1u);
        d[k] = ff{dh[k], dl[k]};
        q[k] = ff{qh[k], ql[k]};
        thr[k] = 0.f;
        if (m[k]) {
          float A = fabsf(ff_f(ff_sub(ph[k], Phi0)));
          thr[k] = dpos(d[k]) ? __fmul_rn(v2t, __fmul_rn(pf2, A)) : __fmul_rn(v2t, 1e30f);
        }
      }
    }
    PT_T(W, 10);
    // first guess of the flags: the bulk velocity at the start of the tile
    {
      const float rM = __frcp_rn(i2f(sM + cM, F.im));
      const float Vx = __fmul_rn(i2f(sX + cX, F.iv), rM), Vy = __fmul_rn(i2f(sY + cY, F.iv), rM),
                  Vz = __fmul_rn(i2f(sZ + cZ, F.iv), rM);
#pragma unroll
      for (int k = 0; k < kItems; k++) {
        float dVX = __fadd_rn(__fmul_rn(__fsub_rn(vx[k], Vx), vf), __fmul_rn(Hr, dx[k]));
        float dVY = __fadd_rn(__fmul_rn(__fsub_rn(vy[k], Vy), vf), __fmul_rn(Hr, dy[k]));
        float dVZ = __fadd_rn(__fmul_rn(__fsub_rn(vz[k], Vz), vf), __fmul_rn(Hr, dz[k]));
        float vel2 = __fadd_rn(__fadd_rn(__fmul_rn(dVX, dVX), __fmul_rn(dVY, dVY)), __fmul_rn(dVZ, dVZ));
        b[k] = m[k] && !(vel2 > thr[k]);
      }
    }
    // fixpoint of the bound flags: each round scans the flags of the previous
    // round exactly and re-decides every member (the recurrence is
    // triangular, so the flags settle from the front of the tile)
    long long ex[4], tot[4];
    int excnt, totcnt;
    float pe[4], pb[4];
    long long pslot, pbslot;
    int rounds = 0;
    bool amb_tile = false;
#pragma unroll
    for (int k = 0; k < kItems; k++) ambk[k] = false;
    while (true) {
      rounds++;
      long long a[4] = {0, 0, 0, 0};
      int cnt = 0;
      bool has = false;
      float p[4] = {0.f, 0.f, 0.f, 0.f};
      long long ps = -1;
#pragma unroll
      for (int k = 0; k < kItems; k++) {
        if (b[k]) {
          a[0] += fw[k]; a[1] += fx[k]; a[2] += fy[k]; a[3] += fz[k];
          cnt++;
          has = true;
          p[0] = d[k].hi; p[1] = d[k].lo; p[2] = q[k].hi; p[3] = q[k].lo;
          ps = (long long)(i0 + k);
        }
      }
      scan_bound(a, cnt, has, p, ps, cDb, cLs, ex, tot, excnt, totcnt, pe, pslot, pb, pbslot, S, par);
      long long rM = sM + cM + ex[0], rX = sX + cX + ex[1], rY = sY + cY + ex[2], rZ = sZ + cZ + ex[3];
      int changed = 0;
      bool nb[kItems];
#pragma unroll
      for (int k = 0; k < kItems; k++) {
        nb[k] = b[k];
        if (m[k]) {
          int r = bound32(vx[k], vy[k], vz[k], dx[k], dy[k], dz[k], thr[k], ethr, rM, rX, rY, rZ, F, vf, Hr);
          ambk[k] = false;
          if (r < 0) {
            (*nret)++;
            bool amb = false;
            float2 ph = phs[i0 + k];
            r = retest_bound(c, B, W, P, o + i0 + k, i0 + k, n1, ff_d(ff{ph.x, ph.y}), phi0d, (double)rX * F.dv,
                             (double)rY * F.dv, (double)rZ * F.dv, (double)rM * F.dm, vmax, F.vq, &amb) ? 1 : 0;
            ambk[k] = amb;
          }
          nb[k] = r != 0;
          if (nb[k] != b[k]) changed = 1;
        }
        if (b[k]) { rM += fw[k]; rX += fx[k]; rY += fy[k]; rZ += fz[k]; }
      }
#pragma unroll
      for (int k = 0; k < kItems; k++) b[k] = nb[k];
      if (!__syncthreads_or(changed)) break;
      if (rounds >= kMaxFixRounds) { amb_tile = true; break; }
    }
    PT_T(W, 11);
    PT_ADD(W, 14, rounds);
    PT_ADD(W, 15, 1);
    if (rounds > maxr) maxr = rounds;
    if (amb_tile) S.amb_ovf = 1;   // fixpoint cap reached
    // test hook 2: the first member of each of the first 16 tiles is treated
    // as ambiguous
    if (P.force_exact == 2 && i0 == base && tix < 16) {
#pragma unroll
      for (int k = 0; k < kItems; k++)
        if (m[k]) { ambk[k] = true; break; }
    }
#pragma unroll
    for (int k = 0; k < kItems; k++) {
      if (!ambk[k]) continue;
      amb_tile = true;
      int q = atomicAdd(&S.amb_n, 1);
      if (q < 32) { S.amb_slot[q] = (long long)(i0 + k); S.amb_b[q] = b[k] ? 1 : 0; }
      else S.amb_ovf = 1;
    }
    if (P.force_exact == 1) amb_tile = true;
    amb_any |= amb_tile ? 1 : 0;
    // next iteration: potential prefix of the kept particles, rvir1 candidate
    ff accN = ffz(), pn[kItems];
    long long myfail = 0x7fffffffffffffffll, fC = 0;
    ff fM = ffz(), fD = ffz();
    {
      long long rMb = cM + ex[0], rC = cNb + excnt;
      ff dp = {pe[0], pe[1]}, qp = {pe[2], pe[3]};
#pragma unroll
      for (int k = 0; k < kItems; k++) {
        pn[k] = accN;
        if (!b[k]) continue;
        rMb += fw[k];
        rC++;
        ff Mb = mass_ff(rMb, rC, has_w, F.im);
        const bool cnt_mass = !has_w && rC < (1ll << 24);
        accN = ff_add(accN, cnt_mass ? phi_termq_c(__int2float_rn((int)rC), __int2float_rn((int)(rC - 1)), d[k], q[k],
                                                   dp, qp)
                                     : phi_termq(Mb, w[k], d[k], q[k], dp, qp));
        pn[k] = accN;
        dp = d[k];
        qp = q[k];
        if (rv < 0 && myfail == 0x7fffffffffffffffll) {
          // FP32 screen; the banded test (with FP64 re-test) only near ovlim
          float rhs = __fmul_rn(ovk, __fmul_rn(__fmul_rn(d[k].hi, d[k].hi), d[k].hi));
          if (!(Mb.hi > __fmul_rn(rhs, 1.f + 4.f * kBand1)) && ov_fail(c, B, W, P, o + i0 + k, Mb, d[k], nret)) {
            myfail = (long long)(i0 + k);
            fM = Mb;
            fD = d[k];
            fC = rC;
          }
        }
      }
    }
    ff exN, totN;
    long long fmin;
    scan_ff_min(accN, myfail, exN, totN, fmin, S, par);
    {
      ff baseN = ff_add(cPhiN, exN);
#pragma unroll
      for (int k = 0; k < kItems; k++) {
        if (!b[k]) continue;
        ff v = ff_add(baseN, pn[k]);
        phs[i0 + k] = make_float2(v.hi, v.lo);
      }
    }
    if (rv < 0 && fmin != 0x7fffffffffffffffll) {
      if (myfail == fmin) { S.bf[0] = fM.hi; S.bf[1] = fM.lo; S.bf[2] = fD.hi; S.bf[3] = fD.lo; S.bl[10] = fC; }
      __syncthreads();
      rv = fmin;
      rvM = ff{S.bf[0], S.bf[1]};
      rvD = ff{S.bf[2], S.bf[3]};
      rvC = S.bl[10];
      __syncthreads();
    }
    if (i0 < n1) {
      unsigned nf = f4;
#pragma unroll
      for (int k = 0; k < kItems; k++)
        if (i0 + k < n1) nf = (nf & ~(0xffu << (8 * k))) | ((unsigned)((m[k] ? 1 : 0) | (b[k] ? 2 : 0)) << (8 * k));
      stnu8<kItems>(W.flag + o + i0, nf);
    }
    PT_T(W, 12);
    cM += tot[0]; cX += tot[1]; cY += tot[2]; cZ += tot[3];
    cNb += totcnt;
    cPhiN = ff_add(cPhiN, totN);
#pragma unroll
    for (int j = 0; j < 4; j++) cDb[j] = pb[j];
    cLs = pbslot;
  }
  if constexpr (SM::kStage > 0) cp_async_wait<0>();
  out.nb = cNb;
  out.Mb = i2ff(cM, F.im);
  out.Phi0n = cNb > 0 ? ff_add(cPhiN, ff_div(out.Mb, ff{cDb[0], cDb[1]})) : ffz();
  out.last_slot = cLs;
  out.rv_slot = rv;
  out.rv_cnt = rvC;
  out.rv_M = rvM;
  out.rv_d = rvD;
  out.amb = __syncthreads_or(amb_any);
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

// FP64 potential prefix of the exact paths: the sort-key array, free after
// the gather (the stored float-float prefix in phi stays intact)
__device__ __forceinline__ double* exact_term(const Work& W, uint64_t o) {
  return reinterpret_cast<double*>(W.keyA) + o;
}

// The Phi0 pass of rem_unbound (ahf_halos.c:3343-3426) over the members of
// [0, n1) in the reference's exact order: per-member FP64 distances d64 and
// the potential prefix (inclusive, sequential FP64 sums) in term; returns
// Phi0.
template <class SM>
static __device__ double exact_potential(const Ctx32& c, const DevBatch& B, const Work& W, SM& S, uint64_t n1) {
  const uint64_t o = c.s;
  double* term = exact_term(W, o);
  double* d64 = W.prof_a + o;
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
  __syncthreads();
  return Phi0;
}

// The bound test of one member in the reference's operation order
// (ahf_halos.c:3528-3561) from exact potential and running sums.
static __device__ __noinline__ bool exact_bound(const Ctx32& c, const DevBatch& B, const Work& W, const DevParams& P,
                                                uint64_t j, double phi, double Phi0, double d, double VXc, double VYc,
                                                double VZc, double M_vel) {
  const uint64_t o = c.s;
  uint64_t e = c.o + W.seid[o + j];
  double dX = wrap_s((double)B.x[e] - c.cx), dY = wrap_s((double)B.y[e] - c.cy), dZ = wrap_s((double)B.z[e] - c.cz);
  double v_esc2 = d > kMachineZero ? (2 * fabs(phi - Phi0) * P.phi_fac) : 1e30;
  double VXp = (double)W.svx[o + j], VYp = (double)W.svy[o + j], VZp = (double)W.svz[o + j];
  double dVX = (VXp - VXc / M_vel) * P.v_fac + P.Hubble * (dX) * P.r_fac;
  double dVY = (VYp - VYc / M_vel) * P.v_fac + P.Hubble * (dY) * P.r_fac;
  double dVZ = (VZp - VZc / M_vel) * P.v_fac + P.Hubble * (dZ) * P.r_fac;
  double vel2 = (dVX * dVX + dVY * dVY) + dVZ * dVZ;
  return !(vel2 > P.v2_tune * v_esc2);
}

// Exact resolution of the decisions an unbinding pass left inside the
// reference-rounding band (recorded in S.amb_*): the potential in the
// reference's order over all members, the bound-only momentum chains up to
// the last recorded slot, the bound mass before each.  Every other decision
// of the pass already equals the reference's (its band is rigorous), so when
// each recorded decision stands the pass's flags are the reference's: returns
// true.  false: some decision differs, the iteration goes through
// exact_iter32.
template <class SM>
static __device__ bool exact_resolve(const Ctx32& c, const DevBatch& B, const Work& W, const DevParams& P, SM& S,
                                     uint64_t n1, uint64_t js) {
  __syncthreads();
  if (S.amb_ovf || S.amb_n <= 0) return false;
  const int na = S.amb_n < 32 ? S.amb_n : 32;
  const uint64_t o = c.s;
  const double Phi0 = exact_potential(c, B, W, S, n1);
  // recorded slots in ascending order (thread 0; at most 32)
  if (threadIdx.x == 0) {
    for (int a = 1; a < na; a++) {
      long long ks = S.amb_slot[a];
      int kb = S.amb_b[a], q = a;
      while (q > 0 && S.amb_slot[q - 1] > ks) { S.amb_slot[q] = S.amb_slot[q - 1]; S.amb_b[q] = S.amb_b[q - 1]; q--; }
      S.amb_slot[q] = ks;
      S.amb_b[q] = kb;
    }
  }
  __syncthreads();
  const uint64_t nl = (uint64_t)S.amb_slot[na - 1] + 1;
  double* ax = W.prof_b + o;
  double* ay = W.prof_c + o;
  double* az = W.prof_d + o;
  double* dsm = reinterpret_cast<double*>(S.scan);
  const double w0 = (double)W.sw[o + js];
  const double sVX = w0 * (double)W.svx[o + js], sVY = w0 * (double)W.svy[o + js], sVZ = w0 * (double)W.svz[o + js];
  for (uint64_t i = threadIdx.x; i < nl; i += blockDim.x) {
    uint8_t f = W.flag[o + i];
    bool b = (f & 1) && ((f >> 1) & 1);
    double w = b ? (double)W.sw[o + i] : 0.0;
    ax[i] = b ? w * (double)W.svx[o + i] : 0.0;
    ay[i] = b ? w * (double)W.svy[o + i] : 0.0;
    az[i] = b ? w * (double)W.svz[o + i] : 0.0;
  }
  __syncthreads();
  {
    const int warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    if (nwarps >= 3) {
      if (warp == 0) chain64(ax, ax, nl, sVX, 0);
      else if (warp == 1) chain64(ay, ay, nl, sVY, 0);
      else if (warp == 2) chain64(az, az, nl, sVZ, 0);
    } else if (warp == 0) {
      chain64(ax, ax, nl, sVX, 0);
      chain64(ay, ay, nl, sVY, 0);
      chain64(az, az, nl, sVZ, 0);
    }
  }
  __syncthreads();
  // bound mass before each recorded slot: FP64 sums of the weights are exact
  // (checked on the host), so block sums over the segments between slots
  double Mrun = w0;
  uint64_t lo = 0;
  for (int a = 0; a < na; a++) {
    const uint64_t hi = (uint64_t)S.amb_slot[a];
    double part = 0.0;
    for (uint64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
      uint8_t f = W.flag[o + i];
      if ((f & 1) && ((f >> 1) & 1)) part += (double)W.sw[o + i];
    }
    double v[1] = {part}, tot[1];
    block_scan<1>(v, tot, dsm);
    Mrun += tot[0];
    if (threadIdx.x == 0) S.amb_m[a] = Mrun;
    lo = hi;
  }
  __syncthreads();
  int bad = 0;
  if ((int)threadIdx.x < na) {
    const int a = threadIdx.x;
    const uint64_t j = (uint64_t)S.amb_slot[a];
    const double* term = exact_term(W, o);
    const double* d64 = W.prof_a + o;
    bool nbv = exact_bound(c, B, W, P, j, term[j], Phi0, d64[j], ax[j], ay[j], az[j], S.amb_m[a]);
    if ((nbv ? 1 : 0) != S.amb_b[a]) bad = 1;
#ifdef AHFGPU_DEBUG_RESOLVE
    if ((nbv ? 1 : 0) != S.amb_b[a])
      printf("resolve mismatch h %d slot %lld of n1 %llu: exact %d pass %d phi %.17g Phi0 %.17g d %.17g V %.17g M %.17g\n", c.h,
             (long long)j, (unsigned long long)n1, (int)nbv, S.amb_b[a], term[j], Phi0, d64[j], ax[j], S.amb_m[a]);
#endif
  }
  return !__syncthreads_or(bad);
}

// One rem_unbound iteration in the reference's exact summation order, for a
// pass whose FP64 re-test stayed inside the rounding band and whose
// ambiguous decision changed.  Members: flag bit0 of [0, n1); bit1 =
// speculated bound flags on entry, exact on exit.  Per-member distances and
// offsets are recomputed in FP64 from the inputs exactly as the reference
// computes them; the order-dependent sums are warp chains.  Returns kept
// count/mass, last kept slot.
template <class SM>
static __device__ void exact_iter32(const Ctx32& c, const DevBatch& B, const Work& W, const DevParams& P, SM& S,
                             uint64_t n1, uint64_t js, long long* nb_out, double* mb_out, long long* last_out) {
  const uint64_t o = c.s;
  double* term = exact_term(W, o);
  double* d64 = W.prof_a + o;
  double* ax = W.prof_b + o;
  double* ay = W.prof_c + o;
  double* az = W.prof_d + o;
  double* dsm = reinterpret_cast<double*>(S.scan);
  const double Phi0 = exact_potential(c, B, W, S, n1);
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
        uint64_t e = c.o + W.seid[o + i];
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
// ahf_halos.c:3343-3426), float-float; stores the members' potential prefix
// (inclusive) in phi
template <class SM>
static __device__ ff phi0_pass32(const Ctx32& c, const Work& W, const DevParams& P, SM& S, const Fix& F, uint64_t n1,
                                 int& par) {
  constexpr int kItems = SM::kItems;
  const uint64_t o = c.s;
  float2* phs = reinterpret_cast<float2*>(W.phi + o);
  long long cM = 0, cs = -1;
  ff cPhi = ffz();
  float cD[4] = {0.f, 0.f, 0.f, 0.f};
  for (uint64_t base = 0; base < n1; base += (uint64_t)blockDim.x * kItems) {
    uint64_t i0 = base + (uint64_t)threadIdx.x * kItems;
    bool m[kItems];
    float w[kItems];
    ff d[kItems], q[kItems];
    long long fw[kItems];
    long long a[4] = {0, 0, 0, 0};
    int cnt = 0;
    bool any = false;
    float lastm[4] = {0.f, 0.f, 0.f, 0.f};
    unsigned f4 = 0u;
    float dh[kItems], dl[kItems], qh[kItems], ql[kItems];
#pragma unroll
    for (int k = 0; k < kItems; k++) { w[k] = 1.f; fw[k] = F.w1; dh[k] = dl[k] = qh[k] = ql[k] = 0.f; }
    if (i0 < n1) {
      f4 = ldnu8<kItems>(W.flag + o + i0);
      if (P.has_w) { ld4f(W.sw + o + i0, w); ld4ll(fix_w(W) + o + i0, fw); }
      ld4f(W.fdh + o + i0, dh); ld4f(W.fdl + o + i0, dl);
      ld4f(W.fqh + o + i0, qh); ld4f(W.fql + o + i0, ql);
    }
#pragma unroll
    for (int k = 0; k < kItems; k++) {
      m[k] = i0 + k < n1 && ((f4 >> (8 * k)) & 1u);
      if (!m[k]) { w[k] = 0.f; fw[k] = 0; }
      d[k] = m[k] ? ff{dh[k], dl[k]} : ffz();
      q[k] = m[k] ? ff{qh[k], ql[k]} : ffz();
      if (m[k]) {
        a[0] += fw[k];
        cnt++;
        any = true;
        lastm[0] = d[k].hi; lastm[1] = d[k].lo; lastm[2] = q[k].hi; lastm[3] = q[k].lo;
      }
    }
    long long ex[4], tot[4], ps, pbs;
    int excnt, totcnt;
    float pe[4], pb[4];
    scan_bound(a, cnt, any, lastm, -1, cD, cs, ex, tot, excnt, totcnt, pe, ps, pb, pbs, S, par);
    ff dp = {pe[0], pe[1]}, qp = {pe[2], pe[3]};
    long long rM = cM + ex[0];
    ff accP = ffz(), pt[kItems];
#pragma unroll
    for (int k = 0; k < kItems; k++) {
      pt[k] = accP;
      if (!m[k]) continue;
      rM += fw[k];
      accP = ff_add(accP, phi_termq(i2ff(rM, F.im), w[k], d[k], q[k], dp, qp));
      pt[k] = accP;
      dp = d[k];
      qp = q[k];
    }
    ff exP, totP;
    long long dummy;
    scan_ff_min(accP, 0, exP, totP, dummy, S, par);
    ff baseP = ff_add(cPhi, exP);
#pragma unroll
    for (int k = 0; k < kItems; k++) {
      if (!m[k]) continue;
      ff v = ff_add(baseP, pt[k]);
      phs[i0 + k] = make_float2(v.hi, v.lo);
    }
    cM += tot[0];
    cPhi = ff_add(cPhi, totP);
#pragma unroll
    for (int j = 0; j < 4; j++) cD[j] = pb[j];
  }
  __syncthreads();
  return ff_add(cPhi, ff_div(i2ff(cM, F.im), ff{cD[0], cD[1]}));
}

// rem_outsideRvir(.,1) over the members of [0, n1): slot of the first member
// failing the overdensity test (-1: none) and the mass prefix there
template <class SM>
static __device__ long long rvir_pass32(const Ctx32& c, const DevBatch& B, const Work& W, const DevParams& P, SM& S,
                                 uint64_t n1, ff* Mfail, unsigned* nret) {
  constexpr int kItems = SM::kItems;
  const uint64_t o = c.s;
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
        float mx = W.svx[c.s + j], my = W.svy[c.s + j], mz = W.svz[c.s + j];
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
      while (js < n1 && !(W.flag[c.s + js] & 1)) js++;
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
  const float2* Mff = reinterpret_cast<const float2*>(W.prof_b + c.s);
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
  const uint32_t* ent = reinterpret_cast<const uint32_t*>(W.prof_d + c.s);
  return sqrt(ref_key(B, c.o + ent[r], c.cx, c.cy, c.cz));
}

// FP64 smoothed value at index i of the array y[j] = raw(j + kNignore),
// j in [0, m), after ns passes of smooth3
static __device__ __noinline__ double smooth_at64(const Ctx32& c, const DevBatch& B, const Work& W, int which, uint64_t m, int ns,
                              uint64_t i) {
  double lvl[8][8], dd[9];
  long long lo = (long long)i - ns, hi = (long long)i + ns;
  if (lo < 0) lo = 0;
  if (hi > (long long)m - 1) hi = (long long)m - 1;
  int w = (int)(hi - lo + 1);
  // reference distances of ranks lo-1 .. hi (each once)
  for (int t = 0; t <= w; t++) {
    long long r = lo + t - 1 + kNignore;
    dd[t] = r >= 0 ? rank_dist64(c, B, W, (uint64_t)r) : 0.0;
  }
  for (int t = 0; t < w; t++) lvl[0][t] = raw64(c, B, W, &dd[t], which, (uint64_t)(lo + t) + kNignore);
  if (ns == 0 || m < 3) return lvl[0][i - lo];
  // pass p is needed only within ns - p of i
  for (int p = 1; p <= ns; p++) {
    for (int t = 0; t < w; t++) {
      long long j = lo + t;
      long long dist = j > (long long)i ? j - (long long)i : (long long)i - j;
      if (dist > ns - p) continue;
      double v;
      if (j == 0) v = (lvl[p - 1][t] + lvl[p - 1][t + 1]) / 2.;
      else if (j == (long long)m - 1) v = (lvl[p - 1][t] + lvl[p - 1][t - 1]) / 2.;
      else v = (lvl[p - 1][t - 1] + lvl[p - 1][t] + lvl[p - 1][t + 1]) / 3.;
      lvl[p][t] = v;
    }
  }
  return lvl[ns][i - lo];
}

// FP32 value at index i of y after ns passes of smooth3 (general.c:548-573),
// for an index within ns of either end: the passes are run on the window
// [i-ns, i+ns] (values that would need data outside it are never used)
static __device__ __noinline__ float smooth_edge32(const float* y, uint64_t m, int ns, uint64_t i) {
  float lvl[8][8];
  long long lo = (long long)i - ns, hi = (long long)i + ns;
  if (lo < 0) lo = 0;
  if (hi > (long long)m - 1) hi = (long long)m - 1;
  int w = (int)(hi - lo + 1);
  for (int t = 0; t < w; t++) lvl[0][t] = y[lo + t];
  for (int p = 1; p <= ns; p++) {
    for (int t = 0; t < w; t++) {
      long long j = lo + t;
      float v;
      if (j == 0) v = __fdiv_rn(__fadd_rn(lvl[p - 1][t], lvl[p - 1][t + 1]), 2.f);
      else if (j == (long long)m - 1) v = __fdiv_rn(__fadd_rn(lvl[p - 1][t], lvl[p - 1][t - 1]), 2.f);
      else if (t == 0 || t == w - 1) v = 0.f;   // outside the window of i
      else v = __fdiv_rn(__fadd_rn(__fadd_rn(lvl[p - 1][t - 1], lvl[p - 1][t]), lvl[p - 1][t + 1]), 3.f);
      lvl[p][t] = v;
    }
  }
  return lvl[ns][i - lo];
}

// Smoothed maximum (find_max, src/libutility/general.c:608-650, on ranks
// nignore..n2-1).  FP32 screen: away from the ends ns passes of smooth3 are
// one stencil ((1,1,1)/3 for one pass, (1,3,6,7,6,3,1)/27 for three); every
// value within 1e-4 of the FP32 maximum is re-evaluated exactly in FP64.
template <class SM>
static __device__ uint64_t find_max32(const Ctx32& c, const DevBatch& B, const Work& W, SM& S, int which, int ns,
                                      uint64_t n2, unsigned* nret) {
  const uint64_t m = n2 - kNignore;
  const float* y = reinterpret_cast<const float*>(W.prof_c + c.s) + (which ? 0 : n2) + kNignore;
  float* sv = reinterpret_cast<float*>(W.phi + c.s);
#ifdef AHFGPU_PHASE_TIMERS
  // slots 27..31: FP64 path cycles, FP64 candidates, calls taking it, FP32 screen cycles, candidate scan cycles
  long long _f0 = clock64();
#endif
  // smoothed FP32 values (kept in sv) and, per thread, the two largest valid
  // values over [0, m-2] with their indices: the block's maximum is the
  // largest of them, and the candidates are counted from them without a
  // second pass.  The ends (within ns of either end) go through
  // smooth_edge32 first; the interior is one stencil with its loads batched.
  float b1 = -10.f, b2 = -10.f;
  long long i1 = -1, i2 = -1;
  const bool direct = ns == 0 || m < 3;
  const uint64_t ilo = direct ? 0 : (uint64_t)ns;
  const uint64_t ihi = direct ? m : (m > 2 * (uint64_t)ns ? m - (uint64_t)ns : (uint64_t)ns);
  if (!direct)
    for (int e = threadIdx.x; e < 2 * ns; e += blockDim.x) {
      const long long i = e < ns ? (long long)e : (long long)m - 2 * ns + e;
      if (i < 0 || i >= (long long)m || (e >= ns && i < ns)) continue;
      const float v = smooth_edge32(y, m, ns, (uint64_t)i);
      sv[i] = v;
      if ((uint64_t)i + 1 < m && !isnan(v)) {
        if (i1 < 0 || v > b1) { b2 = b1; i2 = i1; b1 = v; i1 = i; }
        else if (i2 < 0 || v > b2) { b2 = v; i2 = i; }
      }
    }
  for (uint64_t base = ilo; base < ihi; base += (uint64_t)blockDim.x * 4) {
    float v[4];
    if (direct) {
#pragma unroll
      for (int k = 0; k < 4; k++) {
        const uint64_t i = base + threadIdx.x + (uint64_t)k * blockDim.x;
        v[k] = i < ihi ? y[i] : 0.f;
      }
    } else if (ns == 1) {
      float t[4][3];
#pragma unroll
      for (int k = 0; k < 4; k++) {
        const uint64_t i = base + threadIdx.x + (uint64_t)k * blockDim.x;
#pragma unroll
        for (int q = 0; q < 3; q++) t[k][q] = i < ihi ? y[i - 1 + q] : 0.f;
      }
#pragma unroll
      for (int k = 0; k < 4; k++) v[k] = __fmul_rn(__fadd_rn(__fadd_rn(t[k][0], t[k][1]), t[k][2]), 0.33333334f);
    } else {
      // ns == 3 (the only other smoothing the profiles ask for)
      float t[4][7];
#pragma unroll
      for (int k = 0; k < 4; k++) {
        const uint64_t i = base + threadIdx.x + (uint64_t)k * blockDim.x;
#pragma unroll
        for (int q = 0; q < 7; q++) t[k][q] = i < ihi ? y[i - 3 + q] : 0.f;
      }
#pragma unroll
      for (int k = 0; k < 4; k++) {
        float a = __fadd_rn(t[k][0], t[k][6]);
        float b3 = __fadd_rn(t[k][1], t[k][5]);
        float c6 = __fadd_rn(t[k][2], t[k][4]);
        v[k] = __fmul_rn(__fadd_rn(__fadd_rn(a, __fmul_rn(3.f, b3)), __fadd_rn(__fmul_rn(6.f, c6), __fmul_rn(7.f, t[k][3]))),
                         0.037037037f);
      }
    }
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const uint64_t i = base + threadIdx.x + (uint64_t)k * blockDim.x;
      if (i >= ihi) continue;
      sv[i] = v[k];
      if (i + 1 < m && !isnan(v[k])) {
        if (i1 < 0 || v[k] > b1) { b2 = b1; i2 = i1; b1 = v[k]; i1 = (long long)i; }
        else if (i2 < 0 || v[k] > b2) { b2 = v[k]; i2 = (long long)i; }
      }
    }
  }
  float best = i1 >= 0 ? fmaxf(-10.f, b1) : -10.f;
  for (int off = 16; off > 0; off >>= 1) best = fmaxf(best, __shfl_xor_sync(0xffffffffu, best, off));
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (lane == 0) S.bf[wid] = best;
  __syncthreads();
  float B32 = -10.f;
  for (int w = 0; w < nw; w++) B32 = fmaxf(B32, S.bf[w]);
  __syncthreads();
#ifdef AHFGPU_PHASE_TIMERS
  if (threadIdx.x == 0 && W.phase) { long long _t = clock64(); atomicAdd(&W.phase[30], (unsigned long long)(_t - _f0)); _f0 = _t; }
#endif
  // candidates: within 2e-5 of the FP32 maximum (the FP32 values are within
  // ~1e-6 of the FP64 ones).  A single candidate is the maximum; several
  // are decided on their FP64 smoothed values.
  float thr = isinf(B32) ? B32 : B32 - 2e-5f * fabsf(B32) - 1e-30f;
  const bool c1 = i1 >= 0 && b1 >= thr, c2 = i2 >= 0 && b2 >= thr;
  const int multi = __syncthreads_or(c2 ? 1 : 0);
  const int nthr = __syncthreads_count(c1 ? 1 : 0);
#ifdef AHFGPU_PHASE_TIMERS
  if (threadIdx.x == 0 && W.phase) { long long _t = clock64(); atomicAdd(&W.phase[31], (unsigned long long)(_t - _f0)); _f0 = _t; }
  if (W.phase && (multi || nthr > 1)) {
    if (c1) atomicAdd(&W.phase[28], c2 ? 2ull : 1ull);
    if (threadIdx.x == 0) atomicAdd(&W.phase[29], 1ull);
  }
#endif
  if (!multi && nthr <= 1) {
    long long f = -bmin_ll(-(c1 ? i1 : -1ll), S);
    return f < 0 ? m - 1 : (uint64_t)f;
  }
  double bv = -10.0;
  long long bi = -1;
  // each thread's indices in ascending order, eight loads at a time
  for (uint64_t base = 0; base + 1 < m; base += (uint64_t)blockDim.x * 8) {
    float v[8];
#pragma unroll
    for (int k = 0; k < 8; k++) {
      const uint64_t i = base + threadIdx.x + (uint64_t)k * blockDim.x;
      v[k] = i + 1 < m ? sv[i] : 0.f;
    }
#pragma unroll 1
    for (int k = 0; k < 8; k++) {
      const uint64_t i = base + threadIdx.x + (uint64_t)k * blockDim.x;
      if (!(i + 1 < m) || !(v[k] >= thr)) continue;
      (*nret)++;
      double v64 = smooth_at64(c, B, W, which, m, ns, i);
      if (bi < 0 || v64 > bv) { bv = v64; bi = (long long)i; }
    }
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
#ifdef AHFGPU_PHASE_TIMERS
  if (threadIdx.x == 0 && W.phase) atomicAdd(&W.phase[27], (unsigned long long)(clock64() - _f0));
#endif
  return BI < 0 || !(BV > -10.0) ? m - 1 : (uint64_t)BI;
}

// HaloProfiles per-particle terms (ahf_halos.c:4320-4420).  VX.. are the
// momentum prefixes INCLUDING the particle (the reference updates VXc
// first).  The velocity relative to the running bulk velocity is
// float-float (one float division plus its residual), so the kinetic term
// T stays accurate where Ekin + Epot cancels (lambdaE).
struct PTerms {
  ff T, cx, cy, cz;        // kinetic term, w dX, w dY, w dZ
  ff L[3];                 // w (dX x dV): Lx, Ly, Lz
  float g[11];             // 3..10: a11, a22, a33, a12, a13, a23, Mhi, Mlo (0..2 unused)
};

// (a + al) gb - (b + bl) ga in float-float.  The angular-momentum terms of
// a slowly rotating halo cancel to |L| ~ 1e-4 of sum |w dX x dV|, so FP32
// products would leave L (and lambda) a relative error ~1e-3 / sqrt(N).
__device__ __forceinline__ ff cross_term(float a, float al, ff gb, float b, float bl, ff ga) {
  ff p = two_prod(a, gb.hi);
  p = ff_quick(p.hi, __fmaf_rn(a, gb.lo, __fmaf_rn(al, gb.hi, p.lo)));
  ff q = two_prod(b, ga.hi);
  q = ff_quick(q.hi, __fmaf_rn(b, ga.lo, __fmaf_rn(bl, ga.hi, q.lo)));
  return ff_sub(p, q);
}

__device__ __forceinline__ ff rel_vel(float v, ff V, ff M, float rM) {
  float b = __fmul_rn(V.hi, rM);
  ff r = ff_sub(V, ff_mulf(M, b));
  ff Vb = ff_quick(b, __fmul_rn(r.hi, rM));
  return ff_sub(fff(v), Vb);
}

__device__ __forceinline__ void pterms(float w, float vx, float vy, float vz, float dx, float dy, float dz,
                                       float dxl, float dyl, float dzl, ff M, ff VX, ff VY, ff VZ, float Hrv,
                                       int has_w, PTerms& t) {
  const float rM = __frcp_rn(M.hi);
  ff gx = rel_vel(vx, VX, M, rM), gy = rel_vel(vy, VY, M, rM), gz = rel_vel(vz, VZ, M, rM);
  t.L[0] = ff_mulf(cross_term(dy, dyl, gz, dz, dzl, gy), w);
  t.L[1] = ff_mulf(cross_term(dz, dzl, gx, dx, dxl, gz), w);
  t.L[2] = ff_mulf(cross_term(dx, dxl, gy, dy, dyl, gx), w);
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
                                               float dxl, float dyl, float dzl, ff M, ff VX, ff VY, ff VZ,
                                               float Hrv, int has_w, PTerms& t) {
  pterms(w, vx, vy, vz, dx, dy, dz, dxl, dyl, dzl, M, VX, VY, VZ, Hrv, has_w, t);
}

// edge_b <= x, exact: a float comparison against the float neighbours of
// the FP64 edge, FP64 only when x.hi lies between them
template <class SM>
__device__ __forceinline__ bool edge_le(const SM& S, int b, ff x) {
  if (x.hi > S.eup[b]) return true;
  if (x.hi < S.edn[b]) return false;
  return S.edge[b] <= ff_d(x);
}

// number of bin edges <= x, counting on from `from` (edges ascend)
template <class SM>
__device__ __forceinline__ int edges_le(const SM& S, int nbins, ff x, int from) {
  int b = from;
  while (b < nbins && edge_le(S, b, x)) b++;
  return b;
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
                                  const Fix& F, uint64_t n1, uint64_t n2, ff Phi0, ahfgpu_halo& hout, unsigned* nret,
                                  int& par) {
  constexpr int kItems = SM::kItems;
  const uint64_t o = c.s;
  const double FPT = 4. * kPi / 3.;
  float2* Rff = reinterpret_cast<float2*>(W.prof_a + o);   // radius (float-float) per rank
  float2* Mff = reinterpret_cast<float2*>(W.prof_b + o);   // mass prefix per rank
  float* vc2 = reinterpret_cast<float*>(W.prof_c + o);     // Vcirc2 per rank
  float* dr2 = vc2 + n2;                                   // dens_r2 per rank
  uint32_t* ent = reinterpret_cast<uint32_t*>(W.prof_d + o);
  PT_T0;
  // ranks -> distances (binning_parameter needs them)
  {
    int carry = 0;
    for (uint64_t base = 0; base < n1; base += (uint64_t)blockDim.x * 4) {
      const uint64_t i0 = base + (uint64_t)threadIdx.x * 4;
      unsigned f4 = i0 < n1 ? ld4u8(W.flag + o + i0) : 0u;
      // the four slots' distances and entries, loaded before the scan
      float dh[4], dl[4];
      uint32_t se[4];
#pragma unroll
      for (int k = 0; k < 4; k++) {
        const bool in = i0 + k < n1;
        dh[k] = in ? W.fdh[o + i0 + k] : 0.f;
        dl[k] = in ? W.fdl[o + i0 + k] : 0.f;
        se[k] = in ? W.seid[o + i0 + k] : 0u;
      }
      int cnt = 0;
#pragma unroll
      for (int k = 0; k < 4; k++) cnt += (i0 + k < n1 && ((f4 >> (8 * k)) & 1u)) ? 1 : 0;
      int tot;
      int r = block_scan_int(cnt, &tot, S.iscan) - cnt + carry;
#pragma unroll
      for (int k = 0; k < 4; k++) {
        if (i0 + k < n1 && ((f4 >> (8 * k)) & 1u)) {
          Rff[r] = make_float2(dh[k], dl[k]);
          ent[r] = se[k];
          r++;
        }
      }
      carry += tot;
    }
    __syncthreads();
  }
  PT_T(W, 16);
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
  for (int b = threadIdx.x; b < S.bi[0]; b += blockDim.x) {
    double e = b == S.bi[0] - 1 ? S.bd[1] + kZero : pow(10., S.bd[2] + ((double)b + 1) * S.bd[3]);
    S.edge[b] = e;
    float f = __double2float_rn(e);
    float up = f, dn = f;
    if ((double)f < e) up = nextafterf(f, 3.0e38f);
    if ((double)f > e) dn = nextafterf(f, -3.0e38f);
    S.eup[b] = up;
    S.edn[b] = dn;
  }
  __syncthreads();
  PT_T(W, 17);
  const int nbins = S.bi[0];
  const float Hrv = (float)(P.Hubble * P.r_fac / P.v_fac);
  const int has_w = P.has_w;
  const float2* phs = reinterpret_cast<const float2*>(W.phi + o);
  long long cM = 0, cX = 0, cY = 0, cZ = 0;   // fixed-point running sums (inclusive prefixes)
  ff cU = ffz();
  ff cf[4] = {ffz(), ffz(), ffz(), ffz()};   // T, sum w dX, sum w dY, sum w dZ
  float cg[11];                              // Lx, Ly, Lz, a11, a22, a33, a12, a13, a23, Mhi, Mlo
#pragma unroll
  for (int j = 0; j < 11; j++) cg[j] = 0.f;
  ff cgc[11];                                // float-float carries of the float channels
#pragma unroll
  for (int j = 0; j < 11; j++) cgc[j] = ffz();
  float cD[4] = {0.f, 0.f, 0.f, 0.f};
  int cr = 0;
  // per-thread sums of the channels needed only at bin ends, folded into the
  // uniform carries (cf, cU, cgc) at the next tile with a bin end: tiles
  // without one need no block reduction
  ff pacc[16];
#pragma unroll
  for (int j = 0; j < 16; j++) pacc[j] = ffz();
  bool pend = false;   // pacc holds tiles not folded yet (uniform)
  // most bound particle, per thread: the warp's running FP32 minimum as the
  // screen, FP64 energies of the candidates; one block reduction at the end
  float pEmin = 3.0e38f;
  double pEbest = 1e300;
  long long pEslot = -1;
  const uint64_t tile = (uint64_t)blockDim.x * kItems;
  if constexpr (SM::kStage > 0) stage_issue(S, 0, W, o, (uint64_t)threadIdx.x * kItems, n1, has_w);
  int tix = 0;
  for (uint64_t base = 0; base < n1; base += tile, tix++) {
    const uint64_t i0 = base + (uint64_t)threadIdx.x * kItems;
    bool m[kItems];
    float w[kItems], vx[kItems], vy[kItems], vz[kItems], dx[kItems], dy[kItems], dz[kItems];
    float dxl[kItems], dyl[kItems], dzl[kItems];
    ff d[kItems], q[kItems], phi[kItems];
    long long fw[kItems], fx[kItems], fy[kItems], fz[kItems];
    long long a[4] = {0, 0, 0, 0};
    int nm = 0;
    bool any = false;
    float lastm[4] = {0.f, 0.f, 0.f, 0.f};
    {
      unsigned f4 = 0u;
      float dh[kItems], dl[kItems], qh[kItems], ql[kItems];
#pragma unroll
      for (int k = 0; k < kItems; k++) {
        w[k] = 1.f;
        vx[k] = vy[k] = vz[k] = dx[k] = dy[k] = dz[k] = dxl[k] = dyl[k] = dzl[k] = 0.f;
        dh[k] = dl[k] = qh[k] = ql[k] = 0.f;
        phi[k] = ffz();
      }
#pragma unroll
      for (int k = 0; k < kItems; k++) { fw[k] = F.w1; fx[k] = fy[k] = fz[k] = 0; }
      if constexpr (SM::kStage > 0) {
        stage_issue(S, (tix & 1) ^ 1, W, o, i0 + tile, n1, has_w);
        if (i0 < n1) { ld4f(W.fdxl + o + i0, dxl); ld4f(W.fdyl + o + i0, dyl); ld4f(W.fdzl + o + i0, dzl); }
        cp_async_wait<1>();
        if (i0 < n1) {
          const unsigned char* sb = stage_buf(S, tix & 1);
          f4 = st_flag<SM>(sb);
          if (has_w) { st_f<SM>(sb, 0, w); st_ll<SM>(sb, 1, fw); }
          st_f<SM>(sb, 1, vx); st_f<SM>(sb, 2, vy); st_f<SM>(sb, 3, vz);
          st_f<SM>(sb, 4, dx); st_f<SM>(sb, 5, dy); st_f<SM>(sb, 6, dz);
          st_f<SM>(sb, 7, dh); st_f<SM>(sb, 8, dl); st_f<SM>(sb, 9, qh); st_f<SM>(sb, 10, ql);
          st_ff<SM>(sb, 0, phi);
          st_ll<SM>(sb, 2, fx); st_ll<SM>(sb, 3, fy); st_ll<SM>(sb, 4, fz);
        }
      } else if (i0 < n1) {
        f4 = ldnu8<kItems>(W.flag + o + i0);
        if (has_w) { ld4f(W.sw + o + i0, w); ld4ll(fix_w(W) + o + i0, fw); }
        ld4f(W.svx + o + i0, vx); ld4f(W.svy + o + i0, vy); ld4f(W.svz + o + i0, vz);
        ld4f(W.fdx + o + i0, dx); ld4f(W.fdy + o + i0, dy); ld4f(W.fdz + o + i0, dz);
        ld4f(W.fdxl + o + i0, dxl); ld4f(W.fdyl + o + i0, dyl); ld4f(W.fdzl + o + i0, dzl);
        ld4f(W.fdh + o + i0, dh); ld4f(W.fdl + o + i0, dl);
        ld4f(W.fqh + o + i0, qh); ld4f(W.fql + o + i0, ql);
        ld4ff(W.phi + o + i0, phi);
        ld4ll(fix_x(W) + o + i0, fx); ld4ll(fix_y(W) + o + i0, fy); ld4ll(fix_z(W) + o + i0, fz);
      }
#pragma unroll
      for (int k = 0; k < kItems; k++) {
        m[k] = i0 + k < n1 && ((f4 >> (8 * k)) & 1u);
        d[k] = ff{dh[k], dl[k]};
        q[k] = ff{qh[k], ql[k]};
      }
    }
#pragma unroll
    for (int k = 0; k < kItems; k++) {
      if (!m[k]) { fw[k] = fx[k] = fy[k] = fz[k] = 0; }
      if (m[k]) {
        a[0] += fw[k]; a[1] += fx[k]; a[2] += fy[k]; a[3] += fz[k];
        nm++; any = true;
        lastm[0] = d[k].hi; lastm[1] = d[k].lo; lastm[2] = q[k].hi; lastm[3] = q[k].lo;
      }
    }
    // mass and momentum prefixes (inclusive: the reference adds the
    // particle before using them), ranks, the previous member
    long long ex[4], tot[4], ps, pbs;
    int excnt, tn;
    float dp4[4], blockLast[4];
    PT_T(W, 18);
    scan_bound(a, nm, any, lastm, -1, cD, -1, ex, tot, excnt, tn, dp4, ps, blockLast, pbs, S, par);
    const int rank0 = cr + excnt;
    // per-particle terms, thread totals; bin ends of this tile
    ff tf[4] = {ffz(), ffz(), ffz(), ffz()}, tU = ffz();
    float tg[11];                 // channels 3..10 (0..2 stay zero: tL)
#pragma unroll
    for (int j = 0; j < 11; j++) tg[j] = 0.f;
    ff tL[3] = {ffz(), ffz(), ffz()};   // Lx, Ly, Lz in float-float (lambda cancels them)
    float Ef[kItems];
    ff Mk[kItems];
    bool has_end = false;
    {
      ff dp = {dp4[0], dp4[1]}, qp = {dp4[2], dp4[3]};
      int r = rank0;
      long long rM = cM + ex[0], rX = cX + ex[1], rY = cY + ex[2], rZ = cZ + ex[3];
      int bcur = r > 0 ? edges_le(S, nbins, dp, 0) : 0;
#pragma unroll
      for (int k = 0; k < kItems; k++) {
        Ef[k] = 3.0e38f;
        Mk[k] = ffz();
        if (!m[k]) continue;
        rM += fw[k]; rX += fx[k]; rY += fy[k]; rZ += fz[k];
        ff M = mass_ff(rM, (long long)r + 1, has_w, F.im);
        Mk[k] = M;
        PTerms t;
        pterms(w[k], vx[k], vy[k], vz[k], dx[k], dy[k], dz[k], dxl[k], dyl[k], dzl[k], M, i2ff(rX, F.iv),
               i2ff(rY, F.iv), i2ff(rZ, F.iv), Hrv, has_w, t);
        float Tp = ff_f(t.T);
        tf[0] = ff_add(tf[0], t.T);
        tf[1] = ff_add(tf[1], t.cx);
        tf[2] = ff_add(tf[2], t.cy);
        tf[3] = ff_add(tf[3], t.cz);
#pragma unroll
        for (int j = 0; j < 3; j++) tL[j] = ff_add(tL[j], t.L[j]);
#pragma unroll
        for (int j = 3; j < 11; j++) tg[j] = __fadd_rn(tg[j], t.g[j]);
        ff U = ff_mulf(ff_sub(phi[k], Phi0), w[k]);
        tU = ff_add(tU, U);
        Ef[k] = __fadd_rn(__fmul_rn(0.5f, Tp), ff_f(U));
        // per-rank arrays (ahf_halos.c:4598-4616): FP32 screens of find_max
        Mff[r] = make_float2(M.hi, M.lo);
        float df = ff_f(d[k]);
        vc2[r] = __fdividef(ff_f(M), df);
        ff d3 = ff_mul(ff_mul(d[k], d[k]), d[k]);
        ff p3 = ff_mul(ff_mul(dp, dp), dp);
        float dV = __fmul_rn((float)FPT, ff_f(ff_sub(d3, p3)));
        float rm = __fmul_rn(__fadd_rn(df, ff_f(dp)), 0.5f);
        dr2[r] = __fmul_rn(__fdividef(w[k], dV), __fmul_rn(rm, rm));
        // bin boundary after this particle?
        int bnext = edges_le(S, nbins, d[k], bcur);
        if (bnext > bcur || (uint64_t)(r + 1) == n2) has_end = true;
        bcur = bnext;
        dp = d[k];
        qp = q[k];
        r++;
      }
    }
    PT_T(W, 19);
    // channels needed only at bin ends: full scans in tiles with a bin end,
    // block totals otherwise
    const bool tile_end = __syncthreads_or(has_end ? 1 : 0) != 0;
    ff ef5[5], tf5[5], af5[5] = {tf[0], tf[1], tf[2], tf[3], tU};
    float eg[11], tgt[11];
    ff eL[3], tLt[3];
    if (tile_end) {
      // everything before this tile into the carries, then this tile's scans
      if (pend) {
        ff ptot[16];
        breduce_ff<16>(pacc, ptot, S.scan);
#pragma unroll
        for (int j = 0; j < 4; j++) cf[j] = ff_add(cf[j], ptot[j]);
        cU = ff_add(cU, ptot[4]);
#pragma unroll
        for (int j = 0; j < 11; j++) cgc[j] = ff_add(cgc[j], ptot[5 + j]);
#pragma unroll
        for (int j = 0; j < 16; j++) pacc[j] = ffz();
        pend = false;
      }
      bscan_ff<5>(af5, ef5, tf5, S.scan);
      bscan_ff<3>(tL, eL, tLt, S.scan);
      bscan_f<11>(tg, eg, tgt, S.scan);
    } else {
#pragma unroll
      for (int j = 0; j < 5; j++) { pacc[j] = ff_add(pacc[j], af5[j]); tf5[j] = ffz(); ef5[j] = ffz(); }
#pragma unroll
      for (int j = 0; j < 3; j++) { pacc[5 + j] = ff_add(pacc[5 + j], tL[j]); tLt[j] = ffz(); eL[j] = ffz(); }
#pragma unroll
      for (int j = 3; j < 11; j++) { pacc[5 + j] = ff_add(pacc[5 + j], fff(tg[j])); tgt[j] = 0.f; eg[j] = 0.f; }
      pend = true;
    }
    PT_T(W, 20);
    // most bound particle: FP32 screen against the warp's running minimum
    // (this tile included), FP64 energy of each candidate; the best per
    // thread is reduced over the block once, after the last tile
    {
      float tmin = 3.0e38f;
#pragma unroll
      for (int k = 0; k < kItems; k++) tmin = fminf(tmin, Ef[k]);
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) tmin = fminf(tmin, __shfl_xor_sync(0xffffffffu, tmin, off));
      pEmin = fminf(pEmin, tmin);
      const float cut = pEmin + 1e-4f * fabsf(pEmin) + 1e-30f;
      long long rX = cX + ex[1], rY = cY + ex[2], rZ = cZ + ex[3];
#pragma unroll
      for (int k = 0; k < kItems; k++) {
        if (!m[k]) continue;
        rX += fx[k]; rY += fy[k]; rZ += fz[k];
        if (Ef[k] <= cut) {
          (*nret)++;
          double E = mbp_energy64(c, B, W, P, o + i0 + k, Mk[k], i2ff(rX, F.iv), i2ff(rY, F.iv), i2ff(rZ, F.iv),
                                  phi[k], Phi0, w[k]);
          if (E < pEbest) { pEbest = E; pEslot = (long long)(i0 + k); }
        }
      }
    }
    PT_T(W, 21);
    // bin records at bin ends (cumulative values over the members so far)
    if (tile_end && has_end) {
      ff dp = {dp4[0], dp4[1]};
      int r = rank0;
      ff runf[5];
      float rung[11];
      ff runL[3] = {eL[0], eL[1], eL[2]};
#pragma unroll
      for (int j = 0; j < 5; j++) runf[j] = ff_add(j < 4 ? cf[j] : cU, ef5[j]);
#pragma unroll
      for (int j = 0; j < 11; j++) rung[j] = __fadd_rn(cg[j], eg[j]);
      ff runU = ff_add(cU, ef5[4]);
      long long rX = cX + ex[1], rY = cY + ex[2], rZ = cZ + ex[3];
      int bcur = r > 0 ? edges_le(S, nbins, dp, 0) : 0;
      for (int k = 0; k < kItems; k++) {
        if (!m[k]) continue;
        rX += fx[k]; rY += fy[k]; rZ += fz[k];
        ff M = Mk[k];
        PTerms t;
        pterms_ool(w[k], vx[k], vy[k], vz[k], dx[k], dy[k], dz[k], dxl[k], dyl[k], dzl[k], M, i2ff(rX, F.iv),
                   i2ff(rY, F.iv), i2ff(rZ, F.iv), Hrv, has_w, t);
        runf[0] = ff_add(runf[0], t.T);
        for (int j = 0; j < 3; j++) runL[j] = ff_add(runL[j], t.L[j]);
        for (int j = 3; j < 11; j++) rung[j] = __fadd_rn(rung[j], t.g[j]);
        ff U = ff_mulf(ff_sub(phi[k], Phi0), w[k]);
        runU = ff_add(runU, U);
        int bnext = edges_le(S, nbins, d[k], bcur);
        bool last = (uint64_t)(r + 1) == n2;
        int bend = last ? nbins : bnext;
        for (int bb = bcur; bb < bend; bb++) {
          Bin& R = S.bins[bb];
          R.npart = (double)(r + 1);
          R.M = ff_d(M);
          R.Lx = ff_d(ff_add(cgc[0], runL[0]));
          R.Ly = ff_d(ff_add(cgc[1], runL[1]));
          R.Lz = ff_d(ff_add(cgc[2], runL[2]));
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
        bcur = bnext;
        r++;
      }
    }
    // carries
    cM += tot[0]; cX += tot[1]; cY += tot[2]; cZ += tot[3];
#pragma unroll
    for (int j = 0; j < 4; j++) cf[j] = ff_add(cf[j], tf5[j]);
    cU = ff_add(cU, tf5[4]);
#pragma unroll
    for (int j = 0; j < 3; j++) cgc[j] = ff_add(cgc[j], tLt[j]);
#pragma unroll
    for (int j = 3; j < 11; j++) { cgc[j] = ff_add(cgc[j], fff(tgt[j])); cg[j] = 0.f; }
#pragma unroll
    for (int j = 0; j < 4; j++) cD[j] = blockLast[j];
    cr += tn;
    __syncthreads();
    PT_T(W, 22);
  }
  if constexpr (SM::kStage > 0) cp_async_wait<0>();
  if (pend) {
    ff ptot[16];
    breduce_ff<16>(pacc, ptot, S.scan);
#pragma unroll
    for (int j = 0; j < 4; j++) cf[j] = ff_add(cf[j], ptot[j]);
    cU = ff_add(cU, ptot[4]);
#pragma unroll
    for (int j = 0; j < 11; j++) cgc[j] = ff_add(cgc[j], ptot[5 + j]);
  }
  long long Eslot = -1;
  {
    double bE = pEbest;
    long long bs = pEslot;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int off = 16; off > 0; off >>= 1) {
      double oE = __shfl_xor_sync(0xffffffffu, bE, off);
      long long oi = __shfl_xor_sync(0xffffffffu, bs, off);
      bool take = oi >= 0 && (bs < 0 || oE < bE || (oE == bE && oi < bs));
      if (take) { bE = oE; bs = oi; }
    }
    if (lane == 0) { S.bd[wid] = bE; S.bl[wid & 7] = bs; }
    __syncthreads();
    double TE = 1e300;
    for (int qq = 0; qq < nw; qq++) {
      double oE = S.bd[qq];
      long long oi = S.bl[qq];
      bool take = oi >= 0 && (Eslot < 0 || oE < TE || (oE == TE && oi < Eslot));
      if (take) { TE = oE; Eslot = oi; }
    }
    __syncthreads();
  }
  double* rows = W.prof_stage + W.prof_cap_off[c.h] * AHFGPU_PROF_NFIELDS;
  PT_T(W, 23);
  // the bin records (rows and integral properties: fp32c_finish_kernel)
  for (int b = threadIdx.x; b < nbins; b += blockDim.x)
    stash_bin(rows + (uint64_t)b * AHFGPU_PROF_NFIELDS, S.bins[b], S.edge[b]);
  __syncthreads();
  PT_T(W, 24);
  uint64_t i_r2 = find_max32(c, B, W, S, 0, 3, n2, nret);
  uint64_t i_rm = find_max32(c, B, W, S, 1, 1, n2, nret);
  PT_T(W, 25);
  if (threadIdx.x == 0) {
    double r2 = rank_dist64(c, B, W, kNignore + i_r2);
    double x_max = rank_dist64(c, B, W, kNignore + i_rm);
    double R_max = x_max;
    uint64_t lo = 0, hi = n2 - 1;
    while (lo < hi) {
      uint64_t mid = (lo + hi) / 2;
      // float-float radius of the rank (48 bits of the exact distance);
      // the reference's FP64 distance only when the two are that close
      const float2* Rr = reinterpret_cast<const float2*>(W.prof_a + c.s);
      double rf = (double)Rr[mid].x + (double)Rr[mid].y;
      bool below = fabs(rf - x_max) > 1e-13 * x_max ? rf < x_max : rank_dist64(c, B, W, mid) < x_max;
      if (below) lo = mid + 1; else hi = mid;
    }
    uint64_t ib = lo;
    double rb = rank_dist64(c, B, W, ib);
    float2 mb = Mff[ib];
    double Mb = (double)mb.x + (double)mb.y;
    double ovd = Mb / (FPT * (rb * rb * rb));
    double M_max = ovd * FPT * (rb * rb * rb);
    double V_max = M_max / R_max;
    long long mbe = Eslot >= 0 ? (long long)(c.o + W.seid[o + Eslot]) : -1;
    double Mt = (double)cM * F.dm;
    double* fin = W.fin + (uint64_t)c.h * kFinStride;
    fin[kFinM] = Mt;
    fin[kFinVX] = (double)cX * F.dv; fin[kFinVY] = (double)cY * F.dv; fin[kFinVZ] = (double)cZ * F.dv;
    fin[kFinCX] = Mt * c.cx + ff_d(cf[1]); fin[kFinCY] = Mt * c.cy + ff_d(cf[2]); fin[kFinCZ] = Mt * c.cz + ff_d(cf[3]);
    fin[kFinMhi] = ff_d(cgc[9]); fin[kFinMlo] = ff_d(cgc[10]);
    fin[kFinMbe] = __longlong_as_double(mbe);
    fin[kFinR2] = r2; fin[kFinRmax] = R_max; fin[kFinVmax] = V_max;
    hout.nbins = nbins;
    hout.flags |= AHFGPU_HALO_RAN_PROFILE;
  }
  PT_T(W, 26);
  __syncthreads();
}

// ---------------------------------------------------------------------------
static __device__ void write_members32(const Ctx32& c, uint64_t nlist, const DevBatch& B, const Work& W) {
  __shared__ int isc[64];
  int carry = 0;
  for (uint64_t base = 0; base < nlist; base += (uint64_t)blockDim.x * 4) {
    const uint64_t i0 = base + (uint64_t)threadIdx.x * 4;
    unsigned f4 = i0 < nlist ? ld4u8(W.flag + c.s + i0) : 0u;
    int cnt = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) cnt += (i0 + k < nlist && ((f4 >> (8 * k)) & 1u)) ? 1 : 0;
    int tot;
    int r = block_scan_int(cnt, &tot, isc) - cnt + carry;
#pragma unroll
    for (int k = 0; k < 4; k++) {
      if (i0 + k < nlist && ((f4 >> (8 * k)) & 1u)) W.mem_stage[c.o + r++] = W.keyB[c.s + i0 + k];
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
  c.s = slot_base(c.o, h);
  c.cx = B.cx[h]; c.cy = B.cy[h]; c.cz = B.cz[h];
  c.fx = llrint(c.cx * 4611686018427387904.0);   // 2^62
  c.fy = llrint(c.cy * 4611686018427387904.0);
  c.fz = llrint(c.cz * 4611686018427387904.0);
  __shared__ ahfgpu_halo hout;
  __shared__ unsigned nret_s;
  if (threadIdx.x == 0) {
    nret_s = 0;
  }
  for (unsigned k = threadIdx.x; k < sizeof(ahfgpu_halo) / 8; k += blockDim.x) reinterpret_cast<uint64_t*>(&hout)[k] = 0;
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
#ifdef AHFGPU_PHASE_TIMERS
  unsigned long long _g0;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(_g0));
  const long long _c0 = clock64();
#endif
  float lim[3];
  keys32(c, B, W, P, S, lim);
  PT_MARK(W, 0);
  const int src = radial_sort(W.keyA, W.idxA, W.keyB, W.idxB, c.s, c.n, stack, W.stack_cap, S.sort);
  PT_MARK(W, 1);
  if (src != kErrNone) {
    if (threadIdx.x == 0) { atomicExch(W.err, src); W.halo[h] = hout; }
    __syncthreads();
    return;
  }
  unsigned long long ties = fix_near_ties(c, B, W);
  const float vmax = lim[0];
  const Fix F = make_fix(c.n, lim[1], lim[2], vmax, P.v_fac);
  gather32(c, B, W, P, F);
  int par = 0;
  if (threadIdx.x == 0) {
    hout.flags |= AHFGPU_HALO_RAN_SORT | AHFGPU_HALO_RAN_RVIR0;
    if (ties) atomicAdd(&W.counters[2], ties);
  }
  PT_MARK(W, 2);
  double mo[3];
  ff Phi0;
  uint64_t n1 = rvir0_phi(c, B, W, P, S, F, &Phi0, mo, &nret, par);
  PT_MARK(W, 3);
  if (threadIdx.x == 0) { hout.M_vir = mo[0]; hout.R_vir = mo[1]; hout.ovdens = mo[2]; hout.Phi0 = 0.0; }
  uint64_t nlist = c.n, ncur = n1;
  if (n1 >= (uint64_t)P.MINPART) {
    uint64_t npart = n1;
    uint64_t nremove = 4;
    int niter = 0, maxr = 0, nob = 0, nfull = 0;
    double R_vir = 0.0, M_vir = 0.0, Phi0_exact = 0.0;
    ff Phi0_used = Phi0;
    IterOut it;
    bool last_exact = false;
    int nexact = 0;
    while (nremove > 3) {
      niter++;
      uint64_t js = seed_slot(c, W, P, niter, n1, S);
      Phi0_used = Phi0;
      unbind_pass(c, B, W, P, S, F, n1, Phi0, js, vmax, it, &nret, par);
      last_exact = false;
      if (it.amb != 0) {
        // a bound decision inside the reference's rounding band: decide it in
        // the reference's exact summation order; if it differs from the
        // pass's, redo the whole iteration in that order
        nexact++;
        last_exact = !exact_resolve(c, B, W, P, S, n1, js);
      }
      if (last_exact) {
        nfull++;
        long long nbx, lsx;
        double mbx;
        exact_iter32(c, B, W, P, S, n1, js, &nbx, &mbx, &lsx);
        Phi0_used = ff_from_d(S.bd[21]);
        Phi0_exact = S.bd[21];
        it.nb = nbx;
        it.Mb = ff_from_d(mbx);
        it.last_slot = lsx;
      }
      // members <- bound: four flags per word (the slot range starts at a
      // multiple of 4), eight words in flight per thread, then the last
      // n1 mod 4 flags one by one
      {
        uint32_t* fw = reinterpret_cast<uint32_t*>(W.flag + c.s);
        const uint64_t nw4 = n1 >> 2;
        for (uint64_t base = 0; base < nw4; base += (uint64_t)blockDim.x * 8) {
          uint32_t v[8];
#pragma unroll
          for (int k = 0; k < 8; k++) {
            const uint64_t j = base + threadIdx.x + (uint64_t)k * blockDim.x;
            v[k] = j < nw4 ? fw[j] : 0u;
          }
#pragma unroll
          for (int k = 0; k < 8; k++) {
            const uint64_t j = base + threadIdx.x + (uint64_t)k * blockDim.x;
            if (j < nw4) fw[j] = (v[k] >> 1) & 0x01010101u;
          }
        }
        for (uint64_t i = (nw4 << 2) + threadIdx.x; i < n1; i += blockDim.x) W.flag[c.s + i] = (W.flag[c.s + i] >> 1) & 1;
      }
      __syncthreads();
      if (it.rounds > maxr) maxr = it.rounds;
      nremove = npart - (uint64_t)it.nb;
      npart = (uint64_t)it.nb;
      if (it.nb == 0) nob = 1;
      M_vir = ff_d(it.Mb);
      if (it.last_slot >= 0) R_vir = ref_dist(c, B, W, c.s + it.last_slot);
      Phi0 = last_exact ? (npart > 0 ? phi0_pass32(c, W, P, S, F, n1, par) : ffz()) : it.Phi0n;
      if (((double)npart) < ((double)P.MINPART)) break;
    }
    if (nfull && threadIdx.x == 0) atomicAdd(&W.counters[3], 1ull);
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
        for (uint64_t i = (uint64_t)it.rv_slot + 1 + threadIdx.x; i < n1; i += blockDim.x) W.flag[c.s + i] = 0;
        __syncthreads();
      }
      if (last_exact) {
        int tot = 0, carry = 0;
        for (uint64_t base = 0; base < n1; base += blockDim.x) {
          uint64_t i = base + threadIdx.x;
          bool mem = i < n1 && (W.flag[c.s + i] & 1);
          block_scan_int(mem ? 1 : 0, &tot, S.iscan);
          carry += tot;
        }
        ncur = (uint64_t)carry;
      } else {
        ncur = it.rv_slot >= 0 ? (uint64_t)it.rv_cnt : npart;
      }
      if (threadIdx.x == 0) {
        long long ls = it.rv_slot;
        if (ls < 0) ls = it.last_slot;
        double R = ref_dist(c, B, W, c.s + ls);
        double M = it.rv_slot >= 0 ? ff_d(it.rv_M) : M_vir;
        double V = 4. * kPi / 3. * (R * R * R);
        hout.flags |= AHFGPU_HALO_RAN_RVIR1;
        hout.M_vir = M;
        hout.R_vir = R;
        hout.ovdens = M / V * P.rho_fac / P.rho_vir;
      }
      __syncthreads();
      PT_MARK(W, 5);
      if (ncur >= (uint64_t)P.MINPART) profiles32(c, B, W, P, S, F, n1, ncur, Phi0_used, hout, &nret, par);
      PT_MARK(W, 6);
    }
  }
  atomicAdd(&nret_s, nret);
  __syncthreads();
  write_members32(c, nlist, B, W);
  PT_MARK(W, 7);
#ifdef AHFGPU_PHASE_TIMERS
  if (threadIdx.x == 0 && W.phase) {
    unsigned long long g1;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(g1));
    unsigned smid;
    asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
    W.phase[kPhaseSlots + 4 * h] = _g0;
    W.phase[kPhaseSlots + 4 * h + 1] = g1;
    W.phase[kPhaseSlots + 4 * h + 2] = (unsigned long long)(clock64() - _c0);
    W.phase[kPhaseSlots + 4 * h + 3] = smid;
  }
#endif
  if (threadIdx.x == 0) {
    hout.npart = ncur;
    W.halo[h] = hout;
    atomicAdd(&W.counters[0], (unsigned long long)nret_s);
  }
  __syncthreads();
}

static_assert(sizeof(ahfgpu_halo) % 8 == 0, "the halo record is cleared in 8-byte words");

template <int T, class SS, int MinB = 1>
__global__ void __launch_bounds__(T, MinB) halo_fp32c_kernel(DevParams P, DevBatch B, Work W) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  using SM = F32Smem<SS, T>;
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

