// common.cuh -- shared device definitions of the GB300 unbinding + halo
// property stage: parameters, work-space layout, block-level scans, the
// radial-key bucket sort and the small helpers every halo kernel uses.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/ahfgpu.h"

namespace ahfgpu {

// src/param.h:125, :124 (single-precision build), :45
constexpr double kMachineZero = 5e-16;
constexpr double kZero = 1e-6;
constexpr double kGrav = 4.3006485e-9;
constexpr double kPi = 3.14159265358979323846264338;
constexpr int kNignore = 5;          // AHF_Rmax_r2_NIGNORE, src/param.h:26
constexpr int kMaxBins = 64;         // nbins = 6.2 log10(n) - 3.5 < 64 for n < 2^32
constexpr int kMaxFixRounds = 4096;  // cap of the bulk-velocity fixpoint

// device-side error codes (written to Work::err, read by the host)
// doubles per halo of the FP32C post-pass inputs (Work::fin)
constexpr int kFinStride = 16;

enum : int { kErrNone = 0, kErrFixpoint = 1, kErrSortDepth = 2, kErrWorklist = 3, kErrSortState = 4, kErrGatherDup = 5 };

struct DevParams {
  double VescTune;
  double v2_tune;
  int64_t MINPART;
  double ovlim, rho_vir;
  double r_fac, x_fac, v_fac, m_fac, rho_fac, phi_fac, Hubble;
  int has_w;
  int force_serial;   // weight sums not exact in FP64: replay every halo
  int force_exact;    // test hook: every unbinding iteration in exact order
  float f_ovlim;      // ovlim as float
  float f_rvrf;       // rho_vir / rho_fac as float
};

// Input batch, device pointers (entries of halo h: [off[h], off[h+1])).
struct DevBatch {
  int64_t nhalo;
  const uint64_t* off;
  const float *x, *y, *z, *vx, *vy, *vz, *w;
  const uint64_t* gidx;
  const double *cx, *cy, *cz;
};

// Per-entry scratch (all arrays sized to the batch's entry count N).
struct Work {
  // radial sort buffers (A = result, B = bucket scatter target)
  uint64_t *keyA, *keyB;
  uint32_t *idxA, *idxB;
  // sorted particle arrays (FP64 form): offsets from the centre, distance
  double *sdx, *sdy, *sdz, *sd;
  float *svx, *svy, *svz, *sw;
  uint32_t* seid;         // entry index (within the halo) of sorted slot i
  double* phi;            // potential prefix of the current pass
  float *fdh, *fdl;       // FP32C: distance as float-float
  float *fdx, *fdy, *fdz; // FP32C: offsets from the centre
  float *fdxl, *fdyl, *fdzl;  // FP32C: low parts of the offsets
  float *fqh, *fql;       // FP32C: 1/d^2 as float-float
  float4* rec;            // FP32C: per entry {x, y, z, vx} {vy, vz, id lo, id hi} (two float4)
  uint8_t* flag;          // member (1) / removed (0) per sorted slot
  uint8_t* nflag;         // fixpoint flags of the next round
  double *prof_a, *prof_b, *prof_c, *prof_d;  // per-member profile arrays
  // per-CTA worklists of the bucket sort (ranges still larger than a chunk)
  uint4* sort_stack;      // [nblocks * stack_cap]
  int stack_cap;
  // per-halo outputs (staging, packed afterwards)
  ahfgpu_halo* halo;      // [nhalo]
  uint64_t* mem_stage;    // [N] kept ids (gidx[e], or e where gidx is NULL), at the halo's input offset
  double* prof_stage;     // [nbins_cap_total * NFIELDS]
  double* fin;            // FP32C: [nhalo * kFinStride] inputs of the integral properties (post-pass)
  const uint64_t* prof_cap_off;  // [nhalo+1] staging row offsets
  // work queue / diagnostics
  unsigned int* queue_head;
  const int32_t* queue;   // halo indices, largest first
  int nqueue;
  unsigned long long* counters;  // [0] retest, [1] exact-order haloes, [2] key ties, [3] whole replays
  unsigned long long* phase;     // per-phase SM cycles (instrumented builds only)
  int* err;
};


// First slot of halo h in the FP32C per-slot work arrays: a multiple of 4
// (16-byte aligned float arrays), at least off[h] + n_h before the next
// halo's; the arrays hold N + 3 nhalo + 16 slots.
__host__ __device__ __forceinline__ uint64_t slot_base(uint64_t off, int64_t h) {
  return (off + 3ull * (uint64_t)h + 3ull) & ~3ull;
}

// Optional per-phase cycle counters (build with -DAHFGPU_PHASE_TIMERS):
// kPhaseSlots counters, then per halo {start ns, end ns, SM cycles, SM id}.
constexpr int kPhaseSlots = 32;
#ifdef AHFGPU_PHASE_TIMERS
#define PT_BEGIN long long _pt = clock64();
#define PT_MARK(W, k)                                              \
  do {                                                             \
    __syncthreads();                                               \
    if (threadIdx.x == 0 && (W).phase) {                           \
      long long _t = clock64();                                    \
      atomicAdd(&(W).phase[k], (unsigned long long)(_t - _pt));    \
      _pt = _t;                                                    \
    }                                                              \
  } while (0)
// sub-phase marks without a barrier (thread 0's clock) and event counts
#define PT_T0 long long _q = clock64();
#define PT_T(W, k)                                                 \
  do {                                                             \
    if (threadIdx.x == 0 && (W).phase) {                           \
      long long _t = clock64();                                    \
      atomicAdd(&(W).phase[k], (unsigned long long)(_t - _q));     \
      _q = _t;                                                     \
    }                                                              \
  } while (0)
#define PT_ADD(W, k, v)                                                              \
  do {                                                                               \
    if (threadIdx.x == 0 && (W).phase) atomicAdd(&(W).phase[k], (unsigned long long)(v)); \
  } while (0)
#else
#define PT_BEGIN
#define PT_MARK(W, k) do { } while (0)
#define PT_T0
#define PT_T(W, k) do { } while (0)
#define PT_ADD(W, k, v) do { } while (0)
#endif

// ---------------------------------------------------------------------------
// periodic wraps (src/libahf/ahf_halos.c:3505-3516 signed, :3381-3389 fabs)
__device__ __forceinline__ double wrap_s(double d) {
  if (d > 0.5) d -= 1.0;
  if (d < -0.5) d += 1.0;
  return d;
}

// ---------------------------------------------------------------------------
// Block-wide inclusive scan of NC double channels (one element per thread).
// Fixed reduction tree: deterministic for a given block size.
// smem: 32*NC doubles.  Returns the block total in `tot`.
template <int NC>
__device__ __forceinline__ void block_scan(double (&v)[NC], double (&tot)[NC], double* smem) {
  const unsigned FULL = 0xffffffffu;
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
#pragma unroll
    for (int c = 0; c < NC; c++) {
      double y = __shfl_up_sync(FULL, v[c], off);
      if (lane >= off) v[c] += y;
    }
  }
  if (lane == 31) {
#pragma unroll
    for (int c = 0; c < NC; c++) smem[wid * NC + c] = v[c];
  }
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int c = 0; c < NC; c++) {
      double t = lane < nw ? smem[lane * NC + c] : 0.0;
#pragma unroll
      for (int off = 1; off < 32; off <<= 1) {
        double y = __shfl_up_sync(FULL, t, off);
        if (lane >= off) t += y;
      }
      if (lane < nw) smem[lane * NC + c] = t;
    }
  }
  __syncthreads();
#pragma unroll
  for (int c = 0; c < NC; c++) {
    if (wid > 0) v[c] += smem[(wid - 1) * NC + c];
    tot[c] = smem[(nw - 1) * NC + c];
  }
  __syncthreads();
}

// Block-wide exclusive scan of NC double channels: ex = sum of lower
// threads (0 for thread 0), tot = block total.  Same tree as block_scan.
template <int NC>
__device__ __forceinline__ void block_scan_excl(const double (&v)[NC], double (&ex)[NC], double (&tot)[NC],
                                                double* smem) {
  const unsigned FULL = 0xffffffffu;
  double inc[NC];
#pragma unroll
  for (int c = 0; c < NC; c++) inc[c] = v[c];
  block_scan<NC>(inc, tot, smem);
  int lane = threadIdx.x & 31;
  // exclusive = inclusive of the previous thread; thread 0 of each warp
  // takes the previous warp's total, which block_scan folded into inc of
  // lane 31 of that warp.  Recompute through smem to keep one tree.
  int wid = threadIdx.x >> 5;
#pragma unroll
  for (int c = 0; c < NC; c++) {
    double prev = __shfl_up_sync(FULL, inc[c], 1);
    if (lane == 31) smem[wid * NC + c] = inc[c];
    ex[c] = prev;
  }
  __syncthreads();
  if (lane == 0) {
#pragma unroll
    for (int c = 0; c < NC; c++) ex[c] = wid > 0 ? smem[(wid - 1) * NC + c] : 0.0;
  }
  __syncthreads();
}

// Block-wide inclusive scan of an int (count) channel.
__device__ __forceinline__ int block_scan_int(int v, int* tot, int* smem) {
  const unsigned FULL = 0xffffffffu;
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    int y = __shfl_up_sync(FULL, v, off);
    if (lane >= off) v += y;
  }
  if (lane == 31) smem[wid] = v;
  __syncthreads();
  if (wid == 0) {
    int t = lane < nw ? smem[lane] : 0;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      int y = __shfl_up_sync(FULL, t, off);
      if (lane >= off) t += y;
    }
    if (lane < nw) smem[lane] = t;
  }
  __syncthreads();
  if (wid > 0) v += smem[wid - 1];
  *tot = smem[nw - 1];
  __syncthreads();
  return v;
}

// "last value" exclusive carry: for each thread, the value of the nearest
// lower-ranked thread with has=true (or the incoming carry).
__device__ __forceinline__ double block_last_excl(bool has, double val, double carry_in, bool* any_out,
                                                  double* last_out, double* smem_d, int* smem_i) {
  const unsigned FULL = 0xffffffffu;
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  unsigned m = __ballot_sync(FULL, has);
  // exclusive: lanes strictly below
  unsigned below_ex = m & ((1u << lane) - 1u);
  if (lane == 31) {
    smem_i[wid] = m ? (31 - __clz(m)) : -1;
  }
  // value of the last has-lane in the warp (for the warp total)
  int lastlane = m ? (31 - __clz(m)) : 0;
  double wlast = __shfl_sync(FULL, val, lastlane);
  if (lane == 0) smem_d[wid] = wlast;
  __syncthreads();
  // exclusive carry from lower warps
  double from_lower = carry_in;
  bool have_lower = false;
  for (int w = wid - 1; w >= 0; w--) {
    if (smem_i[w] >= 0) { from_lower = smem_d[w]; have_lower = true; break; }
  }
  (void)have_lower;
  int src = below_ex ? (31 - __clz(below_ex)) : -1;
  double mine = __shfl_sync(FULL, val, src < 0 ? 0 : src);
  double res = src >= 0 ? mine : from_lower;
  // block-wide last
  bool any = false;
  double last = carry_in;
  for (int w = nw - 1; w >= 0; w--) {
    if (smem_i[w] >= 0) { last = smem_d[w]; any = true; break; }
  }
  *any_out = any;
  *last_out = last;
  __syncthreads();
  return res;
}

}  // namespace ahfgpu
