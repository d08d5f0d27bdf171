// amr_sum.cuh -- one node's TSC density (assign_npart, density.c:238) summed
// by one warp, bit for bit as the reference's sequential float sum.
//
// The reference adds, node after node and particle after particle, double
// terms to a float: acc <- (float)((double)acc + t).  For one node that is
// one dependent chain, up to ~1e6 terms long next to a large halo; at the
// FP64 latency of this GPU it would take tens of milliseconds on one thread.
//
// Within a binade of acc (float exponent e, ulp u = 2^(e-23), |acc| = A u
// with A in [2^23, 2^24)) a step is exact integer arithmetic: the double sum
// lies on the grid u 2^-29 (acc is on it), so it rounds the term alone to
// that grid, Q = round(t / (u 2^-29)) (ties to even: acc / (u 2^-29) is
// even); the float rounding then adds r = round(Q / 2^29) units of u, a tie
// going to the even acc / u: r depends on the term and on the parity of A
// only.  So every term is a two-state map, (parity in) -> (r, parity out),
// and maps compose: a window of 32 terms is one inclusive scan across the
// lanes.  Any term whose result would leave the binade -- reach the next
// power of two upward, or the binade's lower edge for a negative acc moving
// to zero -- ends the window; that term takes the exact step
// ((float)((double)acc + t), through amr_round_f32) and the next window
// starts after it.  Zero, subnormal and top-binade accumulators take exact
// steps.  Terms are the reference's m2d w_z w_y w_x: the first two products
// per particle are kept (b[9]), the third formed here; all are >= 0.
#pragma once
#include <cstdint>

#include "amr_tree.cuh"

namespace ahfgpu {

// a source node's part of a node's sum: its list slots s0 .. s0 + cnt - 1,
// the node's stencil slot in it (9 (dz+1) + 3 (dy+1) + (dx+1), target minus
// source), and the terms of the sources before it
struct AmrSrc {
  uint32_t s0, cnt, slot, cum;
};

// the two-state map of a run of terms: r[p] units of u for parity p in, the
// parity out in bit p of pb (r saturates at 2^25: any such run leaves the
// binade)
struct AmrTr {
  int r0, r1;
  unsigned pb;
};

constexpr int kAmrSat = 1 << 25;

__host__ __device__ __forceinline__ AmrTr amr_compose(const AmrTr& L, const AmrTr& R) {
  const unsigned q0 = L.pb & 1u, q1 = (L.pb >> 1) & 1u;
  AmrTr o;
  const int a0 = L.r0 + (q0 ? R.r1 : R.r0), a1 = L.r1 + (q1 ? R.r1 : R.r0);
  o.r0 = a0 < kAmrSat ? a0 : kAmrSat;
  o.r1 = a1 < kAmrSat ? a1 : kAmrSat;
  o.pb = ((R.pb >> q0) & 1u) | (((R.pb >> q1) & 1u) << 1);
  return o;
}

// the map of one term t >= 0 in the binade of float exponent ef
__host__ __device__ __forceinline__ AmrTr amr_term_map(double t, int ef) {
  const unsigned long long b = amr_bits(t);
  unsigned long long Q = 0;
  bool big = false;
  if (b != 0ull) {
    const int E = (int)((b >> 52) & 0x7ffu);
    if (E == 0 || E == 0x7ff || (b >> 63)) {
      big = true;   // subnormal, inf, NaN or negative: the exact step decides
    } else {
      const unsigned long long M = (b & 0x000fffffffffffffull) | 0x0010000000000000ull;
      const int d = (E - 1023) - ef;   // t = M 2^(E-1023-52), the grid 2^(ef-52)
      if (d > 8) {
        big = true;
      } else if (d >= 0) {
        Q = M << d;
      } else if (d > -64) {
        const int s = -d;
        const unsigned long long q = M >> s, rem = M & ((1ull << s) - 1ull), half = 1ull << (s - 1);
        Q = q + ((rem > half || (rem == half && (q & 1ull))) ? 1ull : 0ull);
      }
    }
  }
  AmrTr T;
  if (big) {
    T.r0 = T.r1 = kAmrSat;
    T.pb = 2u;
    return T;
  }
  const unsigned long long fl = Q >> 29, fr = Q & 0x1fffffffull;
  const unsigned long long half = 1ull << 28;
  const unsigned up0 = (fr > half || (fr == half && (fl & 1ull))) ? 1u : 0u;          // parity in 0
  const unsigned up1 = (fr > half || (fr == half && !(fl & 1ull))) ? 1u : 0u;         // parity in 1
  const int f = fl < (unsigned long long)kAmrSat ? (int)fl : kAmrSat;
  T.r0 = f + (int)up0 < kAmrSat ? f + (int)up0 : kAmrSat;
  T.r1 = f + (int)up1 < kAmrSat ? f + (int)up1 : kAmrSat;
  T.pb = ((unsigned)(T.r0 & 1)) | ((1u ^ (unsigned)(T.r1 & 1)) << 1);
  return T;
}

// the term of global index g of the node's concatenated source lists
template <bool DESC>
__device__ __forceinline__ double amr_term(const AmrSrc* __restrict__ src, int nsrc, uint32_t g,
                                           const double* __restrict__ w, uint64_t np) {
  int lo = 0, hi = nsrc - 1;   // the last source with cum <= g
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (src[mid].cum <= g) lo = mid;
    else hi = mid - 1;
  }
  const AmrSrc S = src[lo];
  const uint32_t j = g - S.cum;
  const uint64_t k = DESC ? (uint64_t)S.s0 + S.cnt - 1u - j : (uint64_t)S.s0 + j;
  return __ldg(w + (uint64_t)(S.slot / 3u) * np + k) * __ldg(w + (uint64_t)(9u + S.slot % 3u) * np + k);
}

// -1 plus the node's terms in order, as the reference's float sum; every
// lane of the warp calls it and gets the same value.  The accumulator is kept
// as a double holding a float; its float fields are read from, and written
// back into, the double's bits with integer arithmetic (the FP64 pipe of
// this GPU is the bottleneck: it keeps only the terms' products and the
// exact steps' additions).  A window's terms stay in the lanes: after an
// exit at lane j the next window shifts them down by j + 1 lanes and forms
// only the new ones.
template <bool DESC>
__device__ float amr_warp_sum(const AmrSrc* __restrict__ src, int nsrc, uint32_t nterm,
                              const double* __restrict__ w, uint64_t np) {
  const unsigned FULL = 0xffffffffu, lane = threadIdx.x & 31u;
  double acc = -1.0;
  uint32_t i = 0;
  double t = 0.0;          // this lane's term, index i + lane, when have > lane
  unsigned have = 0;       // terms of the window already formed
  while (i < nterm) {
    const unsigned m = nterm - i < 32u ? nterm - i : 32u;
    if (lane < m && lane >= have) t = amr_term<DESC>(src, nsrc, i + lane, w, np);
    have = m;
    // the float fields of acc (exactly a float): exponent, magnitude in units of its ulp
    const unsigned long long db = amr_bits(acc);
    const int de = (int)((db >> 52) & 0x7ffu);
    const int E = de == 0 ? 0 : de - 896;   // the float's biased exponent
    if (E <= 0 || E >= 254) {
      const double t0 = __shfl_sync(FULL, t, 0);
      acc = amr_round_f32(acc + t0);
      i++;
      t = __shfl_down_sync(FULL, t, 1);
      have = have > 0u ? have - 1u : 0u;
      continue;
    }
    const int ef = E - 127;
    const bool neg = (db >> 63) != 0ull;
    const int A = (int)(((db >> 29) & 0x7fffffull) | 0x800000ull);
    AmrTr T;
    T.r0 = 0; T.r1 = 0; T.pb = 2u;   // identity
    if (lane < m) T = amr_term_map(t, ef);
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      AmrTr P;
      P.r0 = __shfl_up_sync(FULL, T.r0, off);
      P.r1 = __shfl_up_sync(FULL, T.r1, off);
      P.pb = __shfl_up_sync(FULL, T.pb, off);
      if ((int)lane >= off) T = amr_compose(P, T);
    }
    const int R = (A & 1) ? T.r1 : T.r0;
    const int Ak = neg ? A - R : A + R;
    const bool leave = lane < m && (neg ? Ak <= (1 << 23) : Ak >= (1 << 24));
    const unsigned ex = __ballot_sync(FULL, leave);
    // the float of magnitude An ulps in this binade, as the bits of a double
    const unsigned long long hi = (db & 0x8000000000000000ull) | ((unsigned long long)(ef + 1023) << 52);
    if (ex == 0u) {
      const int An = __shfl_sync(FULL, Ak, (int)m - 1);
      acc = amr_from_bits(hi | ((unsigned long long)(An & 0x7fffff) << 29));
      i += m;
      have = 0;
    } else {
      const int j = __ffs((int)ex) - 1;
      const int Ap = __shfl_sync(FULL, Ak, j > 0 ? j - 1 : 0);
      const double tj = __shfl_sync(FULL, t, j);
      const int Ab = j > 0 ? Ap : A;
      acc = amr_from_bits(hi | ((unsigned long long)(Ab & 0x7fffff) << 29));
      acc = amr_round_f32(acc + tj);
      i += (uint32_t)j + 1u;
      // the window's later terms move down to their new lanes
      t = __shfl_down_sync(FULL, t, (unsigned)j + 1u);
      have = m - (unsigned)j - 1u;
    }
  }
  return (float)acc;
}

}  // namespace ahfgpu
