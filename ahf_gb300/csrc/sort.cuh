// sort.cuh -- block-level segmented radial sort of one halo's (key, slot)
// pairs.  Replaces the index sort of sort_halo_particles
// (src/libahf/ahf_halos.c:5846, an NR quicksort) with a deterministic total
// order: ascending key, ties by list position -- the order a stable sort
// gives.
//
// Lists up to kChunk pairs are sorted in shared memory: one counting pass by
// the leading bits of (key - chunk minimum) into about one bin per pair, then
// each thread insertion-sorts its bins on the composite (key, slot); a chunk
// whose keys crowd into a few bins takes a bitonic network on the composite
// instead.  Longer lists take an MSD bucket pass: keys are
// offset by the list minimum and split into up to kSortBuckets buckets by
// their high bits (histogram in shared memory, scatter with atomics into the
// B buffers), after which runs of consecutive buckets that fit a chunk are
// sorted in shared memory straight into the A buffers.  A bucket that is
// still larger than half a chunk is pushed on a per-CTA worklist and split
// again over its own (narrower) key range; a range whose keys are all equal
// is split by slot instead.  Scatter order inside a bucket is irrelevant
// because every chunk is finally sorted on the full composite key.
#pragma once

#include "common.cuh"

namespace ahfgpu {

constexpr int kChunk = 2048;          // pairs sorted in shared memory at once
constexpr int kSortBuckets = 4096;

// CH: pairs sorted in shared memory at once; NB: most buckets of one pass
template <int CH, int NB>
struct SortSmemT {
  static constexpr int kCh = CH;
  static constexpr int kNb = NB;
  uint64_t key[CH];
  uint32_t idx[CH];
  uint64_t key2[CH];      // chunk pairs in bin order
  uint32_t idx2[CH];
  uint32_t hist[NB];      // MSD pass
  uint32_t h2[CH];        // chunk counting pass
  uint64_t red_u64[64];
  int sp;                 // worklist depth
  int seg_lo, seg_hi;     // current run of buckets
  uint32_t run_lo, run_hi;  // its slot range (written by thread 0 only)
  int flag;               // 0, or the kErr* code that ended the sort
  int crowd;              // chunk: some bin too full for an insertion sort
};
using SortSmem = SortSmemT<kChunk, kSortBuckets>;

__device__ __forceinline__ bool pair_less(uint64_t ka, uint32_t ia, uint64_t kb, uint32_t ib) {
  return ka < kb || (ka == kb && ia < ib);
}

// Block min/max over a u64 sequence.
template <class SS>
__device__ __forceinline__ void block_minmax_u64(uint64_t& mn, uint64_t& mx, SS& S) {
  const unsigned FULL = 0xffffffffu;
  for (int off = 16; off > 0; off >>= 1) {
    uint64_t a = __shfl_xor_sync(FULL, mn, off);
    uint64_t b = __shfl_xor_sync(FULL, mx, off);
    mn = a < mn ? a : mn;
    mx = b > mx ? b : mx;
  }
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (lane == 0) { S.red_u64[wid] = mn; S.red_u64[32 + wid] = mx; }
  __syncthreads();
  mn = ~0ull; mx = 0;
  for (int w = 0; w < nw; w++) {
    mn = S.red_u64[w] < mn ? S.red_u64[w] : mn;
    mx = S.red_u64[32 + w] > mx ? S.red_u64[32 + w] : mx;
  }
  __syncthreads();
}

// Bitonic network on S.key/S.idx[0, cnt) (padded to a power of two), in place.
template <class SS>
static __device__ void bitonic_smem(int cnt, SS& S) {
  int P = 1;
  while (P < cnt) P <<= 1;
  for (int i = cnt + threadIdx.x; i < P; i += blockDim.x) {
    S.key[i] = ~0ull;
    S.idx[i] = 0xffffffffu;
  }
  __syncthreads();
  for (int k = 2; k <= P; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < P; i += blockDim.x) {
        int ixj = i ^ j;
        if (ixj > i) {
          uint64_t a = S.key[i], b = S.key[ixj];
          uint32_t ia = S.idx[i], ib = S.idx[ixj];
          bool up = (i & k) == 0;
          bool gt = pair_less(b, ib, a, ia);
          if (gt == up) {
            S.key[i] = b; S.key[ixj] = a;
            S.idx[i] = ib; S.idx[ixj] = ia;
          }
        }
      }
      __syncthreads();
    }
  }
}

// Sort `cnt` (<= kChunk) pairs from (ks, is)[lo..] into (kd, id)[lo..].
// In-place (ks == kd) is allowed: the data goes through shared memory.
template <class SS>
static __device__ void smem_sort_chunk(const uint64_t* ks, const uint32_t* is, uint64_t* kd, uint32_t* id,
                                       uint64_t lo, int cnt, SS& S) {
  constexpr int kCrowd = 48;    // largest bin sorted by insertion
  uint64_t mn = ~0ull, mx = 0;
  for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
    uint64_t k = ks[lo + i];
    S.key[i] = k;
    S.idx[i] = is[lo + i];
    mn = k < mn ? k : mn;
    mx = k > mx ? k : mx;
  }
  block_minmax_u64(mn, mx, S);   // includes the barriers
  int nb = 1;
  while (nb < cnt) nb <<= 1;
  if (nb > SS::kCh) nb = SS::kCh;
  const uint64_t range = mx - mn;
  int shift = 0;
  while ((range >> shift) >= (uint64_t)nb) shift++;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) S.h2[b] = 0;
  if (threadIdx.x == 0) S.crowd = 0;
  __syncthreads();
  for (int i = threadIdx.x; i < cnt; i += blockDim.x) atomicAdd(&S.h2[(int)((S.key[i] - mn) >> shift)], 1u);
  __syncthreads();
  // exclusive scan of the bin counts: contiguous runs of bins per thread
  {
    const int T = blockDim.x;
    const int per = (nb + T - 1) / T;
    const int b0 = threadIdx.x * per;
    const int b1 = min(b0 + per, nb);
    uint32_t run = 0;
    for (int b = b0; b < b1; b++) run += S.h2[b];
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    uint32_t inc = run;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      uint32_t y = __shfl_up_sync(FULL, inc, off);
      if (lane >= off) inc += y;
    }
    uint32_t* wt = reinterpret_cast<uint32_t*>(S.red_u64);
    if (lane == 31) wt[wid] = inc;
    __syncthreads();
    uint32_t base = inc - run;
    for (int w = 0; w < wid; w++) base += wt[w];
    (void)nw;
    for (int b = b0; b < b1; b++) {
      uint32_t c = S.h2[b];
      S.h2[b] = base;
      base += c;
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
    uint64_t k = S.key[i];
    uint32_t pos = atomicAdd(&S.h2[(int)((k - mn) >> shift)], 1u);
    S.key2[pos] = k;
    S.idx2[pos] = S.idx[i];
  }
  __syncthreads();
  // h2[b] is now the end of bin b: insertion sort of each bin by one thread
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    int s0 = b ? (int)S.h2[b - 1] : 0, s1 = (int)S.h2[b];
    if (s1 - s0 < 2) continue;
    if (s1 - s0 > kCrowd) { S.crowd = 1; continue; }
    for (int a = s0 + 1; a < s1; a++) {
      uint64_t ka = S.key2[a];
      uint32_t ia = S.idx2[a];
      int c = a;
      while (c > s0 && pair_less(ka, ia, S.key2[c - 1], S.idx2[c - 1])) {
        S.key2[c] = S.key2[c - 1];
        S.idx2[c] = S.idx2[c - 1];
        c--;
      }
      S.key2[c] = ka;
      S.idx2[c] = ia;
    }
  }
  __syncthreads();
  if (S.crowd) {
    bitonic_smem(cnt, S);
    for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
      kd[lo + i] = S.key[i];
      id[lo + i] = S.idx[i];
    }
  } else {
    for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
      kd[lo + i] = S.key2[i];
      id[lo + i] = S.idx2[i];
    }
  }
  __syncthreads();
}

// Sort (keyA, idxA)[o, o+n) in place by (key, slot).  Uses (keyB, idxB) and
// the CTA's worklist `stack` (capacity cap) as scratch.  Returns kErrNone, or
// kErrWorklist when the worklist overflows, or kErrSortState when a bucket
// run is inconsistent with its pass (the run is then skipped, not sorted).
template <class SS>
static __device__ int radial_sort(uint64_t* keyA, uint32_t* idxA, uint64_t* keyB, uint32_t* idxB, uint64_t o,
                                   uint64_t n, uint4* stack, int cap, SS& S) {
  constexpr int kChunk = SS::kCh;
  constexpr int kHalfChunk = SS::kCh / 2;
  constexpr int kSortBuckets = SS::kNb;
  if (n <= 1) return kErrNone;
  if (n <= (uint64_t)kChunk) {
    smem_sort_chunk(keyA, idxA, keyA, idxA, o, (int)n, S);
    return kErrNone;
  }
  // worklist entry: x = lo(low 32), y = lo(high 32), z = count, w = src(bit0) | by_slot(bit1)
  if (threadIdx.x == 0) {
    stack[0] = make_uint4((uint32_t)o, (uint32_t)(o >> 32), (uint32_t)n, 0u);
    S.sp = 1;
    S.flag = 0;
  }
  __syncthreads();
  while (true) {
    int sp = S.sp;
    if (sp == 0 || S.flag) break;
    uint4 e = stack[sp - 1];
    __syncthreads();
    if (threadIdx.x == 0) S.sp = sp - 1;
    uint64_t lo = (uint64_t)e.x | ((uint64_t)e.y << 32);
    uint32_t cnt = e.z;
    int src = e.w & 1;
    int by_slot = (e.w >> 1) & 1;
    uint64_t* ks = src ? keyB : keyA;
    uint32_t* is = src ? idxB : idxA;
    uint64_t* kd = src ? keyA : keyB;
    uint32_t* id = src ? idxA : idxB;
    if (cnt <= (uint32_t)kChunk) {
      __syncthreads();
      smem_sort_chunk(ks, is, keyA, idxA, lo, (int)cnt, S);
      continue;
    }
    // range of the bucketing key
    constexpr int U = 8;   // elements in flight per thread in the streaming loops
    uint64_t mn = ~0ull, mx = 0;
    for (uint32_t base = 0; base < cnt; base += blockDim.x * U) {
      uint64_t kk[U];
#pragma unroll
      for (int u = 0; u < U; u++) {
        uint32_t i = base + threadIdx.x + u * blockDim.x;
        kk[u] = i < cnt ? (by_slot ? (uint64_t)is[lo + i] : ks[lo + i]) : ~0ull;
      }
#pragma unroll
      for (int u = 0; u < U; u++) {
        uint32_t i = base + threadIdx.x + u * blockDim.x;
        if (i >= cnt) continue;
        mn = kk[u] < mn ? kk[u] : mn;
        mx = kk[u] > mx ? kk[u] : mx;
      }
    }
    block_minmax_u64(mn, mx, S);
    if (!by_slot && mn == mx) {
      // all keys equal: order by slot
      by_slot = 1;
      mn = ~0ull; mx = 0;
      for (uint32_t i = threadIdx.x; i < cnt; i += blockDim.x) {
        uint64_t k = (uint64_t)is[lo + i];
        mn = k < mn ? k : mn;
        mx = k > mx ? k : mx;
      }
      block_minmax_u64(mn, mx, S);
    }
    uint64_t range = mx - mn;
    int nb = 16;
    while (nb < kSortBuckets && (uint64_t)nb * 128 < cnt) nb <<= 1;
    int shift = 0;
    while ((range >> shift) >= (uint64_t)nb) shift++;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) S.hist[b] = 0;
    __syncthreads();
    for (uint32_t base = 0; base < cnt; base += blockDim.x * U) {
      uint64_t kk[U];
#pragma unroll
      for (int u = 0; u < U; u++) {
        uint32_t i = base + threadIdx.x + u * blockDim.x;
        kk[u] = i < cnt ? (by_slot ? (uint64_t)is[lo + i] : ks[lo + i]) : 0;
      }
#pragma unroll
      for (int u = 0; u < U; u++) {
        uint32_t i = base + threadIdx.x + u * blockDim.x;
        if (i < cnt) atomicAdd(&S.hist[(int)((kk[u] - mn) >> shift)], 1u);
      }
    }
    __syncthreads();
    // exclusive scan of the histogram: contiguous runs of buckets per thread
    {
      const int per = (nb + (int)blockDim.x - 1) / (int)blockDim.x;
      const int b0 = threadIdx.x * per, b1 = min(b0 + per, nb);
      uint32_t run = 0;
      for (int b = b0; b < b1; b++) run += S.hist[b];
      const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
      uint32_t inc = run;
#pragma unroll
      for (int off = 1; off < 32; off <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, inc, off);
        if (lane >= off) inc += y;
      }
      uint32_t* wt = reinterpret_cast<uint32_t*>(S.red_u64);
      if (lane == 31) wt[wid] = inc;
      __syncthreads();
      uint32_t b = inc - run;
      for (int w = 0; w < wid; w++) b += wt[w];
      for (int q = b0; q < b1; q++) {
        uint32_t c = S.hist[q];
        S.hist[q] = b;
        b += c;
      }
    }
    __syncthreads();
    for (uint32_t base = 0; base < cnt; base += blockDim.x * U) {
      uint64_t kk[U];
      uint32_t ss[U];
#pragma unroll
      for (int u = 0; u < U; u++) {
        uint32_t i = base + threadIdx.x + u * blockDim.x;
        kk[u] = i < cnt ? ks[lo + i] : 0;
        ss[u] = i < cnt ? is[lo + i] : 0;
      }
#pragma unroll
      for (int u = 0; u < U; u++) {
        uint32_t i = base + threadIdx.x + u * blockDim.x;
        if (i >= cnt) continue;
        uint64_t bk = by_slot ? (uint64_t)ss[u] : kk[u];
        uint32_t pos = atomicAdd(&S.hist[(int)((bk - mn) >> shift)], 1u);
        kd[lo + pos] = kk[u];
        id[lo + pos] = ss[u];
      }
    }
    __syncthreads();
    // hist[b] is now the END of bucket b; walk runs of buckets
    if (threadIdx.x == 0) { S.seg_lo = 0; }
    __syncthreads();
    while (true) {
      int b0 = S.seg_lo;
      if (b0 >= nb) break;
      __syncthreads();
      if (threadIdx.x == 0) {
        uint32_t start = b0 == 0 ? 0u : S.hist[b0 - 1];
        uint32_t size0 = S.hist[b0] - start;
        int b1 = b0 + 1;
        if (size0 > (uint32_t)kHalfChunk) {
          // big bucket: push (data now in the other buffer)
          if (S.sp >= cap) {
            S.flag = kErrWorklist;
          } else {
            uint64_t blo = lo + start;
            stack[S.sp] = make_uint4((uint32_t)blo, (uint32_t)(blo >> 32), size0,
                                     (uint32_t)((1 - src) | (by_slot << 1)));
            S.sp = S.sp + 1;
          }
          S.seg_hi = -1;  // nothing to sort here
        } else {
          // extend the run while it stays within a chunk and meets no big bucket
          while (b1 < nb) {
            uint32_t sb = S.hist[b1 - 1];
            uint32_t szb = S.hist[b1] - sb;
            if (szb > (uint32_t)kHalfChunk) break;
            if (S.hist[b1] - start > (uint32_t)kChunk) break;
            b1++;
          }
          S.seg_hi = b1;
        }
        S.seg_lo = b1;
        // the run's slots; fields of their own: the chunk sort below reuses
        // every scratch array before all warps have read its bounds
        const uint32_t end = S.hist[b1 - 1];
        S.run_lo = start;
        S.run_hi = end;
        if (S.seg_hi >= 0 && (end < start || end > cnt || end - start > (uint32_t)kChunk))
          S.flag = kErrSortState;
      }
      __syncthreads();
      if (S.flag) break;
      if (S.seg_hi >= 0) {
        const uint32_t s0 = S.run_lo, s1 = S.run_hi;
        const int c = (int)(s1 - s0);
        if (c > 0) smem_sort_chunk(kd, id, keyA, idxA, lo + s0, c, S);
      }
      __syncthreads();
    }
    __syncthreads();
  }
  const int rc = S.flag;
  __syncthreads();
  return rc;
}

}  // namespace ahfgpu
