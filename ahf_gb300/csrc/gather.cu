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
// index (a per-halo sort of the matches), a deterministic order; the
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
    atomicAdd(&count[c], 1u);
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
    const uint32_t p = start[c] + atomicAdd(&fill[c], 1u);
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
// each cell's particles into chunks of 32 x 8 and taking every eighth chunk
// of the walk, so a halo of millions of particles is spread over all warps.
// Pass 0 adds each warp's matches to cnt[h] (zeroed before); pass 1 writes
// the particle indices at off[h] + a per-chunk reservation (k_gather_sort
// orders them).  The FP32 screen decides all but the particles near the
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
    for (int kx = 0; kx < nd[0]; kx++) {
      const uint32_t ix = (uint32_t)((lo[0] + kx) % G);
      for (int ky = 0; ky < nd[1]; ky++) {
        const uint32_t iy = (uint32_t)((lo[1] + ky) % G);
        for (int kz = 0; kz < nd[2]; kz++) {
          const uint32_t c = (ix * (uint32_t)G + iy) * (uint32_t)G + (uint32_t)((lo[2] + kz) % G);
          const uint32_t s0 = start[c], s1 = start[c + 1];
          const uint64_t nch = (s1 - s0 + CH - 1) / CH;
          // this warp's chunks of the cell: global chunk numbers = wid mod nw
          uint64_t first = (uint64_t)((wid - (int)(chunk % (uint64_t)nw) + nw) % nw);
          for (uint64_t k = first; k < nch; k += (uint64_t)nw) {
            const uint32_t j0 = s0 + (uint32_t)(k * CH);
            float4 p[U];
#pragma unroll
            for (int u = 0; u < U; u++) {
              const uint32_t j = j0 + (uint32_t)(u * 32 + lane);
              p[u] = j < s1 ? sorted[j] : make_float4(0.f, 0.f, 0.f, 0.f);
            }
            unsigned m[U];
            unsigned tot = 0;
#pragma unroll
            for (int u = 0; u < U; u++) {
              const uint32_t j = j0 + (uint32_t)(u * 32 + lane);
              bool in = false;
              if (j < s1) {
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
      }
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

// each halo's list in ascending particle index: the block radial sort on
// (index, slot) over [off[h], off[h+1]) of keyA (indices) / idxA (scratch)
__global__ void __launch_bounds__(256) k_gather_sort(int64_t nhalo, const int32_t* __restrict__ queue,
                                                     unsigned int* __restrict__ qhead, const uint64_t* __restrict__ off,
                                                     uint64_t* keyA, uint32_t* idxA, uint64_t* keyB, uint32_t* idxB,
                                                     uint4* stack, int stack_cap, int* err) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  GatherSS& S = *reinterpret_cast<GatherSS*>(smem_raw);
  __shared__ int s_h;
  uint4* my_stack = stack + (uint64_t)blockIdx.x * stack_cap;
  while (true) {
    if (threadIdx.x == 0) {
      const unsigned q = atomicAdd(qhead, 1u);
      s_h = q < (unsigned)nhalo ? queue[q] : -1;
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
  }
}

// the gathered lists as a stage batch: SoA particle data per entry, the
// particle index as the entry's id
__global__ void k_gather_pack(uint64_t ng, const uint64_t* __restrict__ idx, const float* __restrict__ x,
                              const float* __restrict__ y, const float* __restrict__ z, const float* __restrict__ vx,
                              const float* __restrict__ vy, const float* __restrict__ vz, const float* __restrict__ w,
                              float* __restrict__ ox, float* __restrict__ oy, float* __restrict__ oz,
                              float* __restrict__ ovx, float* __restrict__ ovy, float* __restrict__ ovz,
                              float* __restrict__ ow, uint64_t* __restrict__ oid) {
  for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < ng; k += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t i = idx[k];
    ox[k] = x[i]; oy[k] = y[i]; oz[k] = z[i];
    ovx[k] = vx[i]; ovy[k] = vy[i]; ovz[k] = vz[i];
    if (w) ow[k] = w[i];
    oid[k] = i;
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
  return (int)cudaFuncSetAttribute(k_gather_sort, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)sizeof(GatherSS));
}

void gather_sort(int64_t nhalo, const int32_t* queue, unsigned int* qhead, const uint64_t* off, uint64_t* keyA,
                 uint32_t* idxA, uint64_t* keyB, uint32_t* idxB, uint4* stack, int stack_cap, int* err, int grid,
                 cudaStream_t st) {
  k_gather_sort<<<grid, 256, sizeof(GatherSS), st>>>(nhalo, queue, qhead, off, keyA, idxA, keyB, idxB, stack, stack_cap,
                                                      err);
}

void gather_pack(uint64_t ng, const uint64_t* idx, const float* x, const float* y, const float* z, const float* vx,
                 const float* vy, const float* vz, const float* w, float* ox, float* oy, float* oz, float* ovx,
                 float* ovy, float* ovz, float* ow, uint64_t* oid, int grid, cudaStream_t st) {
  k_gather_pack<<<grid, 256, 0, st>>>(ng, idx, x, y, z, vx, vy, vz, w, ox, oy, oz, ovx, ovy, ovz, ow, oid);
}

}  // namespace ahfgpu

namespace ahfgpu {
void gather_radii(int64_t nh, const double* px, const double* py, const double* pz, const int64_t* lim,
                  const double* rv, const int32_t* orig, double maxr, double* out, cudaStream_t st) {
  const unsigned nb = (unsigned)((nh + 255) / 256);
  if (nb) k_gather_radii<<<nb, 256, 0, st>>>(nh, px, py, pz, lim, rv, orig, maxr, out);
}
}  // namespace ahfgpu
