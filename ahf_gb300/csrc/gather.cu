// gather.cu -- the particle gather on the GPU.  Replaces
// ahf_halos_sfc_gatherParts (src/libahf/ahf_halos_sfc.c:171-412) for every
// halo of a snapshot at once: the list of halo h is every particle i with
// dist2(i, h) <= gatherRad_h^2, dist2 computed as the reference's
// LOCAL_CAL_DXYZ (:69-78) on the float position promoted to double, the sum
// and the comparison as local_checkAndAddParticles (:329-332) makes them.
// The reference finds candidates through its Hilbert-key sorted particle
// array and the 3x3x3 cells around the centre; here the particles are
// bucketed once into a uniform G^3 grid (counting sort) and each halo scans
// the grid cells its sphere can touch.  Lists come out in ascending particle
// index (a bitmap of the matches, or a per-halo sort of them), a deterministic order; the
// reference's order follows its SFC cells.
#include <cstdint>

#include "common.cuh"
#include "sort.cuh"

namespace ahfgpu {

using GatherSS = SortSmemT<2048, 4096>;

__device__ __forceinline__ int cell_of(float x, int G) {
  int c = (int)(x * (float)G);
  return c < 0 ? 0 : (c >= G ? G - 1 : c);
}

// periodic squared distance of a float position from a double centre, in
// the reference's operation order (no contraction)
__device__ __forceinline__ double gather_d2(float px, float py, float pz, double cx, double cy, double cz) {
  double dx = fabs(__dsub_rn((double)px, cx)), dy = fabs(__dsub_rn((double)py, cy)),
         dz = fabs(__dsub_rn((double)pz, cz));
  if (dx > 0.5) dx = __dsub_rn(1.0, dx);
  if (dy > 0.5) dy = __dsub_rn(1.0, dy);
  if (dz > 0.5) dz = __dsub_rn(1.0, dz);
  return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
}

__global__ void k_gather_cells(uint64_t n, const float* __restrict__ x, const float* __restrict__ y,
                               const float* __restrict__ z, int G, uint32_t* __restrict__ cell,
                               uint32_t* __restrict__ count) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t c = ((uint32_t)cell_of(x[i], G) * (uint32_t)G + (uint32_t)cell_of(y[i], G)) * (uint32_t)G +
                       (uint32_t)cell_of(z[i], G);
    cell[i] = c;
    // one atomic per cell among the warp's active lanes (consecutive
    // particles of a snapshot often share cells)
    const unsigned act = __activemask(), grp = __match_any_sync(act, c);
    if ((int)(threadIdx.x & 31) == __ffs((int)grp) - 1) atomicAdd(&count[c], (unsigned)__popc(grp));
  }
}

// exclusive scan of m u32 counts in tiles of 2048 (block sums to `sums`)
__global__ void k_scan_tiles(const uint32_t* __restrict__ in, uint32_t* __restrict__ out, uint64_t m,
                             uint32_t* __restrict__ sums) {
  __shared__ uint32_t wsum[32];
  const uint64_t base = (uint64_t)blockIdx.x * 2048;
  const uint64_t i0 = base + 2 * (uint64_t)threadIdx.x;
  const uint32_t a = i0 < m ? in[i0] : 0u, b = i0 + 1 < m ? in[i0 + 1] : 0u;
  uint32_t v = a + b, inc = v;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) wsum[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    uint32_t w = lane < nw ? wsum[lane] : 0u;
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t t = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += t;
    }
    wsum[lane] = w;
  }
  __syncthreads();
  const uint32_t ex = (wid ? wsum[wid - 1] : 0u) + inc - v;
  if (i0 < m) out[i0] = ex;
  if (i0 + 1 < m) out[i0 + 1] = ex + a;
  if (threadIdx.x == blockDim.x - 1) sums[blockIdx.x] = wsum[nw - 1];
}

// exclusive scan of the tile sums in place (one block), total to *total
__global__ void k_scan_sums(uint32_t* __restrict__ sums, uint64_t ns, uint32_t* __restrict__ total) {
  __shared__ uint32_t wsum[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  uint32_t carry = 0;
  for (uint64_t base = 0; base < ns; base += blockDim.x) {
    const uint64_t i = base + threadIdx.x;
    const uint32_t v = i < ns ? sums[i] : 0u;
    uint32_t inc = v;
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += t;
    }
    if (lane == 31) wsum[wid] = inc;
    __syncthreads();
    if (wid == 0) {
      uint32_t w = lane < nw ? wsum[lane] : 0u;
      for (int o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += t;
      }
      wsum[lane] = w;
    }
    __syncthreads();
    if (i < ns) sums[i] = carry + (wid ? wsum[wid - 1] : 0u) + inc - v;
    carry += wsum[nw - 1];
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry;
}

__global__ void k_scan_add(uint32_t* __restrict__ out, uint64_t m, const uint32_t* __restrict__ sums) {
  const uint64_t i0 = (uint64_t)blockIdx.x * 2048;
  const uint32_t s = sums[blockIdx.x];
  for (uint64_t i = i0 + threadIdx.x; i < i0 + 2048 && i < m; i += blockDim.x) out[i] += s;
}

// particles in cell order: {x, y, z, index bits}
__global__ void k_gather_scatter(uint64_t n, const float* __restrict__ x, const float* __restrict__ y,
                                 const float* __restrict__ z, const uint32_t* __restrict__ cell,
                                 const uint32_t* __restrict__ start, uint32_t* __restrict__ fill,
                                 float4* __restrict__ sorted) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t c = cell[i];
    // one reservation per cell among the warp's active lanes, in lane order
    const unsigned act = __activemask(), grp = __match_any_sync(act, c);
    const int lane = (int)(threadIdx.x & 31), lead = __ffs((int)grp) - 1;
    uint32_t b = 0;
    if (lane == lead) b = atomicAdd(&fill[c], (unsigned)__popc(grp));
    b = __shfl_sync(act, b, lead);
    const uint32_t p = start[c] + b + (uint32_t)__popc(grp & ((1u << lane) - 1u));
    sorted[p] = make_float4(x[i], y[i], z[i], __uint_as_float((uint32_t)i));
  }
}

// FP32 screen of the sphere test: 1 = surely inside, 0 = surely outside,
// -1 = too close to the surface to tell.  Per axis |dxf - dx| <= 4e-7
// (positions < 1: the centre's rounding to float and the subtraction lose
// 6e-8 each, and where float and double fold differently near 0.5 the two
// values differ by twice that plus the fold's rounding), so
// |d2f - d2| <= 8e-7 (dxf + dyf + dzf) + 1.8e-7 d2f, below the margin
// 1e-6 (dxf + dyf + dzf + d2f) + 1e-12; lo and hi bracket r2 even after
// r2's rounding to float.
__device__ __forceinline__ int gather_screen(float px, float py, float pz, float fx, float fy, float fz, float r2f) {
  float dx = fabsf(__fsub_rn(px, fx)), dy = fabsf(__fsub_rn(py, fy)), dz = fabsf(__fsub_rn(pz, fz));
  if (dx > 0.5f) dx = __fsub_rn(1.0f, dx);
  if (dy > 0.5f) dy = __fsub_rn(1.0f, dy);
  if (dz > 0.5f) dz = __fsub_rn(1.0f, dz);
  const float d2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
  const float err = __fmaf_rn(1e-6f, __fadd_rn(__fadd_rn(dx, dy), __fadd_rn(dz, d2)), 1e-12f);
  const float lo = __fmaf_rn(-4e-7f, r2f, r2f), hi = __fmaf_rn(4e-7f, r2f, r2f);
  if (__fadd_rn(d2, err) < lo) return 1;
  if (__fsub_rn(d2, err) > hi) return 0;
  return -1;
}

// One CTA per halo (persistent, queue largest radius first).  The CTA's
// warps walk the grid cells the halo's sphere can touch together, cutting
// the particles of each batch of cell runs into chunks of 32 x 8 and taking
// every eighth chunk of the walk, so a halo of millions of particles is
// spread over all warps.
// Pass 0 adds each warp's matches to cnt[h] (zeroed before); pass 1 writes
// the particle indices at off[h] + a per-chunk reservation (k_gather_prep
// and the kernels after it order them).  The FP32 screen decides all but the particles near the
// surface, which take the reference's FP64 test.
__global__ void __launch_bounds__(256) k_gather_halos(int pass, int G, const uint32_t* __restrict__ start,
                                                      const float4* __restrict__ sorted, int64_t nhalo,
                                                      const int32_t* __restrict__ queue,
                                                      unsigned int* __restrict__ qhead,
                                                      const double* __restrict__ cx, const double* __restrict__ cy,
                                                      const double* __restrict__ cz, const double* __restrict__ rad,
                                                      uint64_t* __restrict__ cnt, const uint64_t* __restrict__ off,
                                                      unsigned long long* __restrict__ hfill,
                                                      uint64_t* __restrict__ out_idx) {
  constexpr int U = 8;                 // particles in flight per lane
  constexpr uint32_t CH = 32 * U;      // particles per chunk
  __shared__ int s_h;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const unsigned FULL = 0xffffffffu;
  while (true) {
    if (threadIdx.x == 0) {
      const unsigned q = atomicAdd(qhead, 1u);
      s_h = q < (unsigned)nhalo ? queue[q] : -1;
    }
    __syncthreads();
    const int h = s_h;
    __syncthreads();
    if (h < 0) break;
    const double ccx = cx[h], ccy = cy[h], ccz = cz[h], r = rad[h];
    const double r2 = __dmul_rn(r, r);
    const float fx = (float)ccx, fy = (float)ccy, fz = (float)ccz, r2f = (float)r2;
    // cells the sphere can touch, one cell of margin for the float cell
    // assignment; a span of G or more covers the whole periodic axis once
    int lo[3], nd[3];
    const double cc[3] = {ccx, ccy, ccz};
#pragma unroll
    for (int d = 0; d < 3; d++) {
      const long long a = (long long)floor((cc[d] - r) * (double)G) - 1;
      const long long b = (long long)floor((cc[d] + r) * (double)G) + 1;
      if (!(r >= 0.0) || b - a + 1 >= G) { lo[d] = 0; nd[d] = G; }
      else { lo[d] = (int)(((a % G) + G) % G); nd[d] = (int)(b - a + 1); }
    }
    unsigned long long found = 0;
    uint64_t chunk = 0;                // chunks of the walk so far
    // The sphere's cells as runs along z: cells (ix, iy, z) of consecutive z
    // are consecutive in `sorted`, so each (x, y) column of the walk is one
    // run of particles, or two where it wraps the periodic boundary.  Runs
    // are taken 32 at a time (lane j loads the range of run t0 + j), their
    // particles form one stream, and the warps take its chunks of CH
    // particles in turn; a particle's run is found by a binary search over
    // the lanes' inclusive run lengths.
    const bool wrap = lo[2] + nd[2] > G;
    const uint32_t nrun = (uint32_t)nd[0] * (uint32_t)nd[1] * (wrap ? 2u : 1u);
    for (uint32_t t0 = 0; t0 < nrun; t0 += 32) {
      uint32_t rs0 = 0, rlen = 0;
      const uint32_t t = t0 + (uint32_t)lane;
      if (t < nrun) {
        const uint32_t col = wrap ? t >> 1 : t, part = wrap ? (t & 1u) : 0u;
        const uint32_t ky = col % (uint32_t)nd[1], kx = col / (uint32_t)nd[1];
        const uint32_t ix = ((uint32_t)lo[0] + kx) % (uint32_t)G, iy = ((uint32_t)lo[1] + ky) % (uint32_t)G;
        const uint32_t za = part ? 0u : (uint32_t)lo[2];
        const uint32_t zb = wrap ? (part ? (uint32_t)(lo[2] + nd[2] - G) : (uint32_t)G) : (uint32_t)(lo[2] + nd[2]);
        const uint32_t cb = (ix * (uint32_t)G + iy) * (uint32_t)G;
        rs0 = start[cb + za];
        rlen = start[cb + zb] - rs0;
      }
      uint32_t incl = rlen;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const uint32_t x = __shfl_up_sync(FULL, incl, d);
        if (lane >= d) incl += x;
      }
      const uint32_t total = __shfl_sync(FULL, incl, 31);
      const uint64_t nch = (total + CH - 1) / CH;
      // this warp's chunks of the stream: global chunk numbers = wid mod nw
      const uint64_t first = (uint64_t)((wid - (int)(chunk % (uint64_t)nw) + nw) % nw);
      for (uint64_t k = first; k < nch; k += (uint64_t)nw) {
        const uint32_t v0 = (uint32_t)(k * CH);
        float4 p[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
          const uint32_t vi = v0 + (uint32_t)(u * 32 + lane);
          int r = 0;   // runs whose inclusive length is <= vi
#pragma unroll
          for (int step = 16; step > 0; step >>= 1) {
            const uint32_t x = __shfl_sync(FULL, incl, r + step - 1);
            if (x <= vi) r += step;
          }
          const uint32_t rs = __shfl_sync(FULL, rs0, r & 31), ri = __shfl_sync(FULL, incl, r & 31),
                         rl = __shfl_sync(FULL, rlen, r & 31);
          p[u] = vi < total ? sorted[rs + vi - (ri - rl)] : make_float4(0.f, 0.f, 0.f, 0.f);
        }
        unsigned m[U];
        unsigned tot = 0;
#pragma unroll
        for (int u = 0; u < U; u++) {
          const uint32_t vi = v0 + (uint32_t)(u * 32 + lane);
          bool in = false;
          if (vi < total) {
            const int sc = gather_screen(p[u].x, p[u].y, p[u].z, fx, fy, fz, r2f);
            in = sc > 0 || (sc < 0 && gather_d2(p[u].x, p[u].y, p[u].z, ccx, ccy, ccz) <= r2);
          }
          m[u] = __ballot_sync(FULL, in);
          tot += (unsigned)__popc(m[u]);
        }
        if (pass == 0) {
          found += tot;
        } else if (tot) {
          unsigned long long b = 0;
          if (lane == 0) b = atomicAdd(&hfill[h], (unsigned long long)tot);
          b = __shfl_sync(FULL, b, 0);
          const uint64_t at = off[h] + b;
          unsigned run = 0;
#pragma unroll
          for (int u = 0; u < U; u++) {
            if ((m[u] >> lane) & 1u)
              out_idx[at + run + (unsigned)__popc(m[u] & ((1u << lane) - 1u))] = (uint64_t)__float_as_uint(p[u].w);
            run += (unsigned)__popc(m[u]);
          }
        }
      }
      chunk += nch;
    }
    if (pass == 0 && lane == 0 && found) atomicAdd(reinterpret_cast<unsigned long long*>(&cnt[h]), found);
  }
}

// exclusive scan of nhalo u64 counts into off[0..nhalo] (one block)
__global__ void k_gather_offsets(const uint64_t* __restrict__ cnt, int64_t nhalo, uint64_t* __restrict__ off) {
  __shared__ unsigned long long wsum[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  unsigned long long carry = 0;
  for (int64_t base = 0; base < nhalo; base += blockDim.x) {
    const int64_t i = base + threadIdx.x;
    const unsigned long long v = i < nhalo ? cnt[i] : 0ull;
    unsigned long long inc = v;
    for (int o = 1; o < 32; o <<= 1) {
      unsigned long long t = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += t;
    }
    if (lane == 31) wsum[wid] = inc;
    __syncthreads();
    if (wid == 0) {
      unsigned long long w = lane < nw ? wsum[lane] : 0ull;
      for (int o = 1; o < 32; o <<= 1) {
        unsigned long long t = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += t;
      }
      wsum[lane] = w;
    }
    __syncthreads();
    if (i < nhalo) off[i + 1] = carry + (wid ? wsum[wid - 1] : 0ull) + inc;
    carry += wsum[nw - 1];
    __syncthreads();
  }
  if (threadIdx.x == 0) off[0] = 0;
}

// The lists in ascending particle index.  A halo's matches are distinct
// particle indices.  Each list's index range [mn, mx] is cut into windows of
// 2^wshift indices, and a window's keys are ordered in shared memory: marked
// in a bitmap and read back in ascending order where they are dense enough
// (span / 32 <= 4 cnt + 1024 words), else by a bitonic network (a sparse
// window holds fewer than kGbSortMax keys).  k_gather_prep takes the lists
// from the largest-first queue: a list of one window is ordered at once; a
// list of several is counted per window, scattered by window into keyB and
// queued as one work item per non-empty window for k_gather_windows, so that
// the windows of a long list run on many CTAs.  The bitmap read-back: each
// warp owns a contiguous run of the window's words (counted first, so that
// every warp knows where its output starts), and per group of 32 words a
// warp scan of the popcounts gives each word's first output position; output
// element e of the group is found by a binary search over the lanes'
// inclusive counts and a select of the bit inside its word, so consecutive
// lanes write consecutive positions.  Lists of more windows than the count
// table holds (only with a narrowed window), lists whose items do not fit the
// item table and, under the test hook, every list take the block radial sort
// instead (k_gather_sort).  mode: 1 = as above, 0 = every list to the radial
// sort, 2 = every window through the bitmap, 3 = every window of at most
// kGbSortMax keys through the bitonic network.
constexpr int kGbT = 256;
constexpr uint32_t kGbWords = 16384;           // shared words: a window's bitmap or a list's window counts
constexpr uint32_t kGbSortMax = kGbWords / 2;  // u64 keys of the bitonic network
constexpr int kGbU = 8;                        // keys in flight per thread
constexpr unsigned long long kGbNone = ~0ull;  // no key (indices are below 2^32)

struct GbItem {
  unsigned long long kb;    // the window's first index
  unsigned long long at;    // its first output position (in keyB and in the output)
  unsigned long long cnt;   // its keys
  unsigned long long pad;
};

struct GbShared {
  long long q;
  unsigned long long mn[kGbT / 32], mx[kGbT / 32];
  unsigned wa[kGbT / 32], wb[kGbT / 32];
  unsigned long long ibase;
  int ok;
};

// position of the set bit of rank r (0-based) in w (r < popc(w))
__device__ __forceinline__ unsigned select_bit(unsigned w, unsigned r) {
  unsigned pos = 0;
#pragma unroll
  for (int half = 16; half > 0; half >>= 1) {
    const unsigned lo = (unsigned)__popc(w & ((1u << half) - 1u));
    if (r >= lo) { r -= lo; w >>= half; pos += (unsigned)half; }
  }
  return pos;
}

// kGbU keys of src[0, n) per thread: i0 + u kGbT + thread (kGbNone past n)
__device__ __forceinline__ void gb_load(const uint64_t* __restrict__ src, uint64_t n, uint64_t i0,
                                        unsigned long long (&k)[kGbU]) {
#pragma unroll
  for (int u = 0; u < kGbU; u++) {
    const uint64_t i = i0 + (uint64_t)u * kGbT + threadIdx.x;
    k[u] = i < n ? src[i] : kGbNone;
  }
}

// block minimum and maximum of src[0, n) (n > 0)
__device__ void gb_minmax(const uint64_t* __restrict__ src, uint64_t n, unsigned long long& mn,
                          unsigned long long& mx, GbShared& S) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  mn = kGbNone;
  mx = 0ull;
  for (uint64_t i0 = 0; i0 < n; i0 += (uint64_t)kGbT * kGbU) {
    unsigned long long k[kGbU];
    gb_load(src, n, i0, k);
#pragma unroll
    for (int u = 0; u < kGbU; u++)
      if (k[u] != kGbNone) {
        mn = k[u] < mn ? k[u] : mn;
        mx = k[u] > mx ? k[u] : mx;
      }
  }
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) {
    const unsigned long long a = __shfl_xor_sync(FULL, mn, d), b = __shfl_xor_sync(FULL, mx, d);
    mn = a < mn ? a : mn;
    mx = b > mx ? b : mx;
  }
  if (lane == 0) { S.mn[wid] = mn; S.mx[wid] = mx; }
  __syncthreads();
#pragma unroll
  for (int v = 0; v < kGbT / 32; v++) {
    mn = S.mn[v] < mn ? S.mn[v] : mn;
    mx = S.mx[v] > mx ? S.mx[v] : mx;
  }
  __syncthreads();
}

// block exclusive scan of two u32 values (ea, eb) and the totals (ta, tb)
__device__ void gb_scan2(unsigned a, unsigned b, unsigned& ea, unsigned& eb, unsigned& ta, unsigned& tb, GbShared& S) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  unsigned ia = a, ib = b;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const unsigned x = __shfl_up_sync(FULL, ia, d), y = __shfl_up_sync(FULL, ib, d);
    if (lane >= d) { ia += x; ib += y; }
  }
  if (lane == 31) { S.wa[wid] = ia; S.wb[wid] = ib; }
  __syncthreads();
  ea = ia - a;
  eb = ib - b;
  ta = 0;
  tb = 0;
#pragma unroll
  for (int v = 0; v < kGbT / 32; v++) {
    if (v < wid) { ea += S.wa[v]; eb += S.wb[v]; }
    ta += S.wa[v];
    tb += S.wb[v];
  }
  __syncthreads();
}

// Orders the distinct keys src[0, cnt), all in [lo, hi] (hi - lo < 32
// kGbWords), into dst[0, cnt); every thread of the CTA calls it.  Returns the
// keys written: cnt unless a key repeats.
__device__ uint64_t gb_order(const uint64_t* __restrict__ src, uint64_t cnt, unsigned long long lo,
                             unsigned long long hi, uint64_t* __restrict__ dst, int mode, unsigned* bm,
                             GbShared& S) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  constexpr int NW = kGbT / 32;
  const uint64_t span = hi - lo + 1;
  const uint32_t nwd = (uint32_t)((span + 31u) / 32u);
  const bool net = cnt <= kGbSortMax && (mode == 3 || (mode != 2 && (uint64_t)nwd > 4u * cnt + 1024u));
  if (net) {
    unsigned long long* sk = reinterpret_cast<unsigned long long*>(bm);
    uint32_t P = 1;
    while (P < cnt) P <<= 1;
    for (uint32_t i = threadIdx.x; i < P; i += kGbT) sk[i] = i < cnt ? src[i] : kGbNone;
    __syncthreads();
    for (uint32_t k = 2; k <= P; k <<= 1)
      for (uint32_t j = k >> 1; j > 0; j >>= 1) {
        for (uint32_t i = threadIdx.x; i < P; i += kGbT) {
          const uint32_t l = i ^ j;
          if (l > i) {
            const unsigned long long a = sk[i], b = sk[l];
            if ((a > b) == ((i & k) == 0u)) { sk[i] = b; sk[l] = a; }
          }
        }
        __syncthreads();
      }
    int rep = 0;
    for (uint32_t i = threadIdx.x; i < cnt; i += kGbT) {
      dst[i] = sk[i];
      if (i + 1u < cnt && sk[i + 1u] == sk[i]) rep = 1;
    }
    return __syncthreads_or(rep) ? cnt - 1u : cnt;
  }
  for (uint32_t j = threadIdx.x; j < nwd; j += kGbT) bm[j] = 0u;
  __syncthreads();
  for (uint64_t i0 = 0; i0 < cnt; i0 += (uint64_t)kGbT * kGbU) {
    unsigned long long k[kGbU];
    gb_load(src, cnt, i0, k);
#pragma unroll
    for (int u = 0; u < kGbU; u++) {
      const uint64_t d = k[u] - lo;
      if (k[u] != kGbNone && d < span) atomicOr(&bm[d >> 5], 1u << (d & 31u));
    }
  }
  __syncthreads();
  // this warp's words [w0, w1)
  const uint32_t per = ((nwd + NW - 1) / NW + 31u) & ~31u;
  const uint32_t w0 = min((uint32_t)wid * per, nwd), w1 = min(w0 + per, nwd);
  unsigned c0 = 0;
  for (uint32_t j = w0 + lane; j < w1; j += 32) c0 += (unsigned)__popc(bm[j]);
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) c0 += __shfl_xor_sync(FULL, c0, d);
  if (lane == 0) S.wa[wid] = c0;
  __syncthreads();
  uint64_t base = 0, tot = 0;
#pragma unroll
  for (int v = 0; v < NW; v++) {
    if (v < wid) base += S.wa[v];
    tot += S.wa[v];
  }
  for (uint32_t g = w0; g < w1; g += 32) {
    const uint32_t j = g + (uint32_t)lane;
    const unsigned word = j < w1 ? bm[j] : 0u;
    const unsigned c = (unsigned)__popc(word);
    unsigned incl = c;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const unsigned t = __shfl_up_sync(FULL, incl, d);
      if (lane >= d) incl += t;
    }
    const unsigned total = __shfl_sync(FULL, incl, 31);
    for (unsigned e0 = 0; e0 < total; e0 += 32) {
      const unsigned e = e0 + (unsigned)lane;
      // s = the number of lanes whose inclusive count is <= e
      int s = 0;
#pragma unroll
      for (int step = 16; step > 0; step >>= 1) {
        const unsigned v = __shfl_sync(FULL, incl, s + step - 1);
        if (v <= e) s += step;
      }
      const unsigned ws = __shfl_sync(FULL, word, s & 31), cs = __shfl_sync(FULL, c, s & 31),
                     is = __shfl_sync(FULL, incl, s & 31);
      if (e < total) dst[base + e] = lo + ((uint64_t)(g + (uint32_t)s) << 5) + select_bit(ws, e - (is - cs));
    }
    base += total;
  }
  __syncthreads();   // the bitmap is rewritten by the caller's next window
  return tot;
}

__global__ void __launch_bounds__(kGbT) k_gather_prep(int64_t nhalo, const int32_t* __restrict__ queue,
                                                      unsigned int* __restrict__ qhead,
                                                      const uint64_t* __restrict__ off,
                                                      const uint64_t* __restrict__ idx, uint64_t* __restrict__ keyB,
                                                      uint64_t* __restrict__ dst, int wshift, int mode,
                                                      GbItem* __restrict__ items,
                                                      unsigned long long* __restrict__ nitems,
                                                      unsigned long long icap, int32_t* __restrict__ fbq,
                                                      unsigned int* __restrict__ fbn, int* __restrict__ err) {
  extern __shared__ unsigned bm[];
  __shared__ GbShared S;
  while (true) {
    if (threadIdx.x == 0) {
      const unsigned q = atomicAdd(qhead, 1u);
      S.q = q < (unsigned)nhalo ? queue[q] : -1;
    }
    __syncthreads();
    const int h = (int)S.q;
    __syncthreads();
    if (h < 0) break;
    const uint64_t o = off[h], n = off[h + 1] - o;
    if (n == 0) continue;
    if (mode == 0) {
      if (threadIdx.x == 0) fbq[atomicAdd(fbn, 1u)] = h;
      continue;
    }
    unsigned long long mn, mx;
    gb_minmax(idx + o, n, mn, mx, S);
    const uint64_t nwin = ((mx - mn) >> wshift) + 1;
    if (nwin == 1) {
      const uint64_t got = gb_order(idx + o, n, mn, mx, dst + o, mode, bm, S);
      if (threadIdx.x == 0 && got != n) atomicExch(err, kErrGatherDup);
      continue;
    }
    if (nwin > kGbWords) {
      if (threadIdx.x == 0) fbq[atomicAdd(fbn, 1u)] = h;
      continue;
    }
    // keys per window
    for (uint32_t j = threadIdx.x; j < (uint32_t)nwin; j += kGbT) bm[j] = 0u;
    __syncthreads();
    for (uint64_t i0 = 0; i0 < n; i0 += (uint64_t)kGbT * kGbU) {
      unsigned long long k[kGbU];
      gb_load(idx + o, n, i0, k);
#pragma unroll
      for (int u = 0; u < kGbU; u++)
        if (k[u] != kGbNone) atomicAdd(&bm[(k[u] - mn) >> wshift], 1u);
    }
    __syncthreads();
    // each thread's run of windows [c0, c1): keys and non-empty windows, scanned
    const uint32_t per = (uint32_t)((nwin + kGbT - 1) / kGbT);
    const uint32_t c0 = min((uint32_t)threadIdx.x * per, (uint32_t)nwin), c1 = min(c0 + per, (uint32_t)nwin);
    unsigned sk = 0, sn = 0;
    for (uint32_t j = c0; j < c1; j++) { sk += bm[j]; sn += bm[j] ? 1u : 0u; }
    unsigned ek, en, tk, tn;
    gb_scan2(sk, sn, ek, en, tk, tn, S);
    if (threadIdx.x == 0) {
      // reserve tn items if they fit the table
      unsigned long long cur = *nitems;
      S.ok = 0;
      while (cur + tn <= icap) {
        const unsigned long long prev = atomicCAS(nitems, cur, cur + tn);
        if (prev == cur) { S.ok = 1; S.ibase = cur; break; }
        cur = prev;
      }
      if (!S.ok) fbq[atomicAdd(fbn, 1u)] = h;
    }
    __syncthreads();
    if (!S.ok) continue;
    unsigned run = ek;
    unsigned long long it = S.ibase + en;
    for (uint32_t j = c0; j < c1; j++) {
      const unsigned c = bm[j];
      if (c) {
        GbItem I;
        I.kb = mn + ((unsigned long long)j << wshift);
        I.at = o + run;
        I.cnt = c;
        I.pad = 0;
        items[it++] = I;
      }
      bm[j] = run;   // the window's cursor
      run += c;
    }
    __syncthreads();
    for (uint64_t i0 = 0; i0 < n; i0 += (uint64_t)kGbT * kGbU) {
      unsigned long long k[kGbU];
      gb_load(idx + o, n, i0, k);
#pragma unroll
      for (int u = 0; u < kGbU; u++)
        if (k[u] != kGbNone) keyB[o + atomicAdd(&bm[(k[u] - mn) >> wshift], 1u)] = k[u];
    }
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kGbT) k_gather_windows(const GbItem* __restrict__ items,
                                                         const unsigned long long* __restrict__ nitems,
                                                         unsigned int* __restrict__ qhead,
                                                         const uint64_t* __restrict__ keyB,
                                                         uint64_t* __restrict__ dst, int mode, int* __restrict__ err) {
  extern __shared__ unsigned bm[];
  __shared__ GbShared S;
  const unsigned long long ni = *nitems;
  while (true) {
    if (threadIdx.x == 0) {
      const unsigned long long q = atomicAdd(qhead, 1u);
      S.q = q < ni ? (long long)q : -1;
    }
    __syncthreads();
    const long long q = S.q;
    __syncthreads();
    if (q < 0) break;
    const GbItem I = items[q];
    unsigned long long lo, hi;
    gb_minmax(keyB + I.at, I.cnt, lo, hi, S);
    const uint64_t got = gb_order(keyB + I.at, I.cnt, lo, hi, dst + I.at, mode, bm, S);
    if (threadIdx.x == 0 && got != I.cnt) atomicExch(err, kErrGatherDup);
  }
}

// The radial-sort path: each queued halo's list in ascending particle index
// by the block radial sort on (index, slot) over [off[h], off[h+1]) of keyA
// (indices) / idxA (scratch), copied to dst.  The queue length is read on
// the device (*nq).
__global__ void __launch_bounds__(256) k_gather_sort(const unsigned int* __restrict__ nq,
                                                     const int32_t* __restrict__ queue,
                                                     unsigned int* __restrict__ qhead, const uint64_t* __restrict__ off,
                                                     uint64_t* keyA, uint32_t* idxA, uint64_t* keyB, uint32_t* idxB,
                                                     uint4* stack, int stack_cap, uint64_t* __restrict__ dst, int* err) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  GatherSS& S = *reinterpret_cast<GatherSS*>(smem_raw);
  __shared__ int s_h;
  uint4* my_stack = stack + (uint64_t)blockIdx.x * stack_cap;
  const unsigned nhalo = *nq;
  while (true) {
    if (threadIdx.x == 0) {
      const unsigned q = atomicAdd(qhead, 1u);
      s_h = q < nhalo ? queue[q] : -1;
    }
    __syncthreads();
    const int h = s_h;
    if (h < 0) break;
    const uint64_t o = off[h], n = off[h + 1] - o;
    for (uint64_t i = threadIdx.x; i < n; i += blockDim.x) idxA[o + i] = (uint32_t)i;
    __syncthreads();
    const int rc = radial_sort(keyA, idxA, keyB, idxB, o, n, my_stack, stack_cap, S);
    if (rc != kErrNone && threadIdx.x == 0) atomicExch(err, rc);
    __syncthreads();
    for (uint64_t i = threadIdx.x; i < n; i += blockDim.x) dst[o + i] = keyA[o + i];
    __syncthreads();
  }
}

// the gathered lists as a stage batch: SoA particle data per entry (the
// entry's particle index already in idx)
__global__ void k_gather_pack(uint64_t ng, const uint64_t* __restrict__ idx, const float* __restrict__ x,
                              const float* __restrict__ y, const float* __restrict__ z, const float* __restrict__ vx,
                              const float* __restrict__ vy, const float* __restrict__ vz, const float* __restrict__ w,
                              float* __restrict__ ox, float* __restrict__ oy, float* __restrict__ oz,
                              float* __restrict__ ovx, float* __restrict__ ovy, float* __restrict__ ovz,
                              float* __restrict__ ow) {
  for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < ng; k += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t i = idx[k];
    ox[k] = x[i]; oy[k] = y[i]; oz[k] = z[i];
    ovx[k] = vx[i]; ovy[k] = vy[i]; ovz[k] = vz[i];
    if (w) ow[k] = w[i];
  }
}

// ---------------------------------------------------------------------------
// Gather radii: the loop of spatialRef2halos (src/libahf/ahf_halos.c:2987-3051).
// Haloes come sorted by particle count, largest first (s = sorted position);
// lim[s] = how many haloes have strictly more particles than halo s, i.e.
// the candidates are sorted positions [0, lim[s]).  For each halo the
// reference takes the smallest periodic squared distance (double, its
// operation order) to a candidate; here pass A finds, in FP32, the smallest
// upper bound m of any candidate's distance, and pass B evaluates in FP64 the
// candidates whose lower bound is within m (they include every exact
// minimiser).  Per-pair float error as in gather_screen: |d2f - d2| below
// 1e-6 (dxf + dyf + dzf + d2f) + 1e-12.
__device__ __forceinline__ float pair_d2f(float ax, float ay, float az, float bx, float by, float bz, float* err) {
  float dx = fabsf(__fsub_rn(ax, bx)), dy = fabsf(__fsub_rn(ay, by)), dz = fabsf(__fsub_rn(az, bz));
  if (dx > 0.5f) dx = __fsub_rn(1.0f, dx);
  if (dy > 0.5f) dy = __fsub_rn(1.0f, dy);
  if (dz > 0.5f) dz = __fsub_rn(1.0f, dz);
  const float d2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
  *err = __fmaf_rn(1e-6f, __fadd_rn(__fadd_rn(dx, dy), __fadd_rn(dz, d2)), 1e-12f);
  return d2;
}

__device__ __forceinline__ double pair_d2(double ax, double ay, double az, double bx, double by, double bz) {
  double dx = fabs(__dsub_rn(ax, bx)), dy = fabs(__dsub_rn(ay, by)), dz = fabs(__dsub_rn(az, bz));
  if (dx > 0.5) dx = __dsub_rn(1.0, dx);
  if (dy > 0.5) dy = __dsub_rn(1.0, dy);
  if (dz > 0.5) dz = __dsub_rn(1.0, dz);
  return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
}

__global__ void __launch_bounds__(256) k_gather_radii(int64_t nh, const double* __restrict__ px,
                                                      const double* __restrict__ py, const double* __restrict__ pz,
                                                      const int64_t* __restrict__ lim, const double* __restrict__ rv,
                                                      const int32_t* __restrict__ orig, double maxr,
                                                      double* __restrict__ out) {
  __shared__ double tx[256], ty[256], tz[256];
  __shared__ float fx[256], fy[256], fz[256];
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool live = s < nh;
  const int64_t my_lim = live ? lim[s] : 0;
  const int64_t last = min((int64_t)(blockIdx.x + 1) * blockDim.x, nh) - 1;
  const int64_t blim = lim[last];   // the block's largest candidate range (lim grows with s)
  const double ax = live ? px[s] : 0.0, ay = live ? py[s] : 0.0, az = live ? pz[s] : 0.0;
  const float afx = (float)ax, afy = (float)ay, afz = (float)az;
  float m = 3.0e38f;
  for (int pass = 0; pass < 2; pass++) {
    double best = 100000000000.0;    // the reference's initial gatherRad
    for (int64_t t0 = 0; t0 < blim; t0 += blockDim.x) {
      const int64_t j = t0 + threadIdx.x;
      if (j < blim) {
        tx[threadIdx.x] = px[j]; ty[threadIdx.x] = py[j]; tz[threadIdx.x] = pz[j];
        fx[threadIdx.x] = (float)px[j]; fy[threadIdx.x] = (float)py[j]; fz[threadIdx.x] = (float)pz[j];
      }
      __syncthreads();
      const int64_t n = min((int64_t)blockDim.x, my_lim - t0);
      for (int64_t k = 0; k < n; k++) {
        float err;
        const float d2f = pair_d2f(afx, afy, afz, fx[k], fy[k], fz[k], &err);
        if (pass == 0) {
          m = fminf(m, __fadd_rn(d2f, err));
        } else if (__fsub_rn(d2f, err) <= m) {
          const double d2 = pair_d2(ax, ay, az, tx[k], ty[k], tz[k]);
          if (d2 < best) best = d2;
        }
      }
      __syncthreads();
    }
    if (pass == 1 && live) {
      double r = my_lim > 0 ? sqrt(best) * 0.5 : maxr;
      r = fmax(r, rv[s]);
      r = fmin(r, maxr);
      out[orig[s]] = r;
    }
  }
}

// ---------------------------------------------------------------------------
// launchers (host)

void gather_cells(uint64_t n, const float* x, const float* y, const float* z, int G, uint32_t* cell,
                  uint32_t* count, int grid, cudaStream_t st) {
  k_gather_cells<<<grid, 256, 0, st>>>(n, x, y, z, G, cell, count);
}

// exclusive scan of m counts into out[0..m) with out[m] = total (out has m+1)
void gather_scan_u32(const uint32_t* in, uint32_t* out, uint64_t m, uint32_t* sums, cudaStream_t st) {
  const uint64_t nt = (m + 2047) / 2048;
  k_scan_tiles<<<(unsigned)nt, 1024, 0, st>>>(in, out, m, sums);
  k_scan_sums<<<1, 1024, 0, st>>>(sums, nt, out + m);
  k_scan_add<<<(unsigned)nt, 256, 0, st>>>(out, m, sums);
}

void gather_scatter(uint64_t n, const float* x, const float* y, const float* z, const uint32_t* cell,
                    const uint32_t* start, uint32_t* fill, float4* sorted, int grid, cudaStream_t st) {
  k_gather_scatter<<<grid, 256, 0, st>>>(n, x, y, z, cell, start, fill, sorted);
}

void gather_halos(int pass, int G, const uint32_t* start, const float4* sorted, int64_t nhalo, const int32_t* queue,
                  unsigned int* qhead, const double* cx, const double* cy, const double* cz, const double* rad,
                  uint64_t* cnt, const uint64_t* off, unsigned long long* hfill, uint64_t* out_idx, int grid,
                  cudaStream_t st) {
  k_gather_halos<<<grid, 256, 0, st>>>(pass, G, start, sorted, nhalo, queue, qhead, cx, cy, cz, rad, cnt, off, hfill,
                                       out_idx);
}

void gather_offsets(const uint64_t* cnt, int64_t nhalo, uint64_t* off, cudaStream_t st) {
  k_gather_offsets<<<1, 1024, 0, st>>>(cnt, nhalo, off);
}

size_t gather_sort_smem() { return sizeof(GatherSS); }

int gather_sort_setup() {
  cudaError_t e = cudaFuncSetAttribute(k_gather_sort, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(GatherSS));
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_gather_prep, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(kGbWords * 4));
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_gather_windows, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(kGbWords * 4));
  return (int)e;
}

int gather_window_shift_max() { return 19; }   // 2^19 = 32 kGbWords indices
size_t gather_item_bytes() { return sizeof(GbItem); }

// The lists in ascending index (into oid), then packed: the per-list pass,
// the windows it queued, the radial sort of the lists it left, the pack.
// qhead: 3 queue heads; fbn: the radial-sort queue length (u32 at byte 0) and
// the item count (u64 at byte 8).
void gather_order_pack(int64_t nhalo, const int32_t* queue, unsigned int* qhead, const uint64_t* off, uint64_t* keyA,
                       uint32_t* idxA, uint64_t* keyB, uint32_t* idxB, uint4* stack, int stack_cap, int wshift,
                       int mode, void* items, uint64_t icap, int32_t* fbq, unsigned int* fbn, uint64_t ng,
                       const float* x, const float* y, const float* z, const float* vx, const float* vy,
                       const float* vz, const float* w, float* ox, float* oy, float* oz, float* ovx, float* ovy,
                       float* ovz, float* ow, uint64_t* oid, int* err, int grid, int grid_p, cudaStream_t st) {
  unsigned long long* nitems = reinterpret_cast<unsigned long long*>(reinterpret_cast<unsigned char*>(fbn) + 8);
  cudaMemsetAsync(qhead, 0, 16, st);
  cudaMemsetAsync(fbn, 0, 16, st);
  GbItem* it = reinterpret_cast<GbItem*>(items);
  k_gather_prep<<<grid, kGbT, kGbWords * 4, st>>>(nhalo, queue, qhead, off, keyA, keyB, oid, wshift, mode, it, nitems,
                                                   (unsigned long long)icap, fbq, fbn, err);
  k_gather_windows<<<grid, kGbT, kGbWords * 4, st>>>(it, nitems, qhead + 2, keyB, oid, mode, err);
  k_gather_sort<<<grid, 256, sizeof(GatherSS), st>>>(fbn, fbq, qhead + 1, off, keyA, idxA, keyB, idxB, stack,
                                                      stack_cap, oid, err);
  k_gather_pack<<<grid_p, 256, 0, st>>>(ng, oid, x, y, z, vx, vy, vz, w, ox, oy, oz, ovx, ovy, ovz, w ? ow : nullptr);
}

}  // namespace ahfgpu

namespace ahfgpu {
void gather_radii(int64_t nh, const double* px, const double* py, const double* pz, const int64_t* lim,
                  const double* rv, const int32_t* orig, double maxr, double* out, cudaStream_t st) {
  const unsigned nb = (unsigned)((nh + 255) / 256);
  if (nb) k_gather_radii<<<nb, 256, 0, st>>>(nh, px, py, pz, lim, rv, orig, maxr, out);
}
}  // namespace ahfgpu
