// amr.cu -- the first two levels of AHF's AMR hierarchy (libamr_serial):
// the domain grid's TSC particle density and its first refinement.
//
// Domain grid (gen_domgrids, src/libamr_serial/generate_grids.c:24; ll();
// assign_npart, density.c:238): l1^3 nodes in ascending (z, y, x); every
// particle sits in the node floor(l1 x) per axis (an index past l1 - 1, a
// coordinate of exactly 1.0, folded into node 0), in its node's list in
// descending input index (ll prepends).  The reference visits the nodes in
// order and, per particle in list order, adds m2d w_z w_y w_x (double) to the
// float density of the 27 nodes around (periodic), starting from -1 (minus
// the mean density); m2d = l1^3 / n, separations from the node centre
// ((x / l1 + 1/(2 l1)) + 1, folded into [0, 1)) in cells, through the fold
// again when |d| > l1 / 2; weights 0.75 - d^2, (1/2 - d)^2 / 2,
// (1/2 + d)^2 / 2.
//
// Here the same sums run as a gather: one thread per target node walks its
// 27 source nodes in ascending node index (the reference's visiting order;
// with l1 >= 3 they are distinct) and each source's particles in list order,
// adding the same double term to a float in the same order -- the floats
// equal the reference's bit for bit.  The particles are grouped by node by a
// stable radix sort of their node index (ascending index within a node; the
// list order is that read backwards), and each particle's TSC factors are
// formed once, in that order: the nine (m2d w_z) w_y and the three w_x, so a
// target's loop reads two of them per particle, forms the last product and
// the sum.  The sums are FP64-pipe bound on this GPU, so the rounding of
// each sum to float is done by integer arithmetic (amr_round_f32), leaving
// two FP64 operations per term.
//
// First refinement (refine_grid, refine_grid.c:899, test_node :113-137 on the
// domain grid): a node is flagged when any node at dz, dy in {-1,0,1} and
// dx in {0,1} has density >= critdens - mean_dens, critdens = NperDomCell
// l1^3 / n; along x a run also covers the node after a flagged one (wrapping
// at x = 0, not at x = l1 - 1); every covered node becomes 2 x 2 x 2 fine
// nodes; the fine grid is kept only with at least MIN_NNODES = 125 nodes.
// The fine nodes come out in ascending (z, y, x): per coarse row a count of
// covered nodes, a scan over the rows, then each row writes its fine nodes.
#include <cstdint>

#include "common.cuh"
#include "amr_tree.cuh"
#include "amr_sum.cuh"

namespace ahfgpu {

constexpr int kAmrT = 256;

__device__ __forceinline__ double amr_fold(double v) { return v >= 2.0 ? v - 2.0 : (v >= 1.0 ? v - 1.0 : v); }

// the node of every particle as a sort key (and the identity index)
__global__ void __launch_bounds__(kAmrT) k_amr_cells(uint32_t n, const float* __restrict__ x,
                                                     const float* __restrict__ y, const float* __restrict__ z,
                                                     int l1, uint64_t* __restrict__ key, uint32_t* __restrict__ idx,
                                                     uint32_t* __restrict__ count) {
  const double dl1 = (double)l1;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    unsigned long c[3];
    const float p[3] = {x[i], y[i], z[i]};
    for (int d = 0; d < 3; d++) {
      c[d] = (unsigned long)(dl1 * (double)p[d]);
      if (c[d] > (unsigned long)(l1 - 1)) c[d] = 0;
    }
    const uint64_t node = ((uint64_t)c[2] * (uint64_t)l1 + c[1]) * (uint64_t)l1 + c[0];
    key[i] = node;
    idx[i] = i;
    atomicAdd(&count[node], 1u);
  }
}

// the three source coordinates around t along one axis, ascending
__device__ __forceinline__ void amr_three(int t, int l1, int (&s)[3]) {
  int a = t == 0 ? l1 - 1 : t - 1, b = t, c = t == l1 - 1 ? 0 : t + 1;
  // sort a, b, c (l1 >= 3: distinct)
  int lo = min(a, min(b, c)), hi = max(a, max(b, c));
  s[0] = lo;
  s[1] = a + b + c - lo - hi;
  s[2] = hi;
}

// TSC weight of the target at offset o in {-1, 0, 1} from the source node,
// for separation `sep` (cells) of the particle from the source's centre
__device__ __forceinline__ double amr_w(double sep, int o) {
  if (o == 0) return 0.75 - sep * sep;
  if (o < 0) return ((0.5 - sep) * (0.5 - sep)) / 2;
  return ((0.5 + sep) * (0.5 + sep)) / 2;
}

__device__ __forceinline__ double amr_sep(float p, double centre, double dl1) {
  double sep = ((double)p - centre) * dl1;
  if (fabs(sep) > 0.5 * dl1) {
    const double a = amr_fold(((double)p + 0.5) + 1.0);
    const double b = amr_fold((centre + 0.5) + 1.0);
    sep = (a - b) * dl1;
  }
  return sep;
}

// each particle's TSC factors, in node order (the order of the sorted node
// keys), computed once and read by the 27 targets around the node: the
// reference forms m2d * w_z * w_y * w_x left to right, so the first two
// products are kept, b[3 oz + oy] = (m2d * w_z(oz - 1)) * w_y(oy - 1), and
// x[ox] = w_x(ox - 1); o = offset + 1 of the target from the source
struct AmrW {
  double* b[9];
  double* x[3];
};

// a node's folded centre coordinate per grid index c, as the reference forms
// it: fold((c / l1 + 1 / (2 l1)) + 1) -- one FP64 division per index here
// instead of three per particle in the weights (FP64 is slow on this GPU)
__global__ void __launch_bounds__(kAmrT) k_amr_cfold(int l1, double* __restrict__ cfold) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= l1) return;
  const double dl1 = (double)l1, shift = 0.5 / dl1;
  cfold[c] = amr_fold(((double)c / dl1 + shift) + 1.0);
}

__global__ void __launch_bounds__(kAmrT) k_amr_weights(int l1, uint32_t n, const uint64_t* __restrict__ skey,
                                                       const uint32_t* __restrict__ ord, const float* __restrict__ x,
                                                       const float* __restrict__ y, const float* __restrict__ z,
                                                       const double* __restrict__ cfold, AmrW W) {
  const double dl1 = (double)l1;
  const double m2d = (dl1 * dl1 * dl1) / (double)n;
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const uint64_t node = skey[k];
    const uint32_t i = ord[k];
    const int cx = (int)(node % (uint64_t)l1), cy = (int)((node / (uint64_t)l1) % (uint64_t)l1),
              cz = (int)(node / ((uint64_t)l1 * l1));
    const double sx = amr_sep(x[i], cfold[cx], dl1);
    const double sy = amr_sep(y[i], cfold[cy], dl1);
    const double sz = amr_sep(z[i], cfold[cz], dl1);
#pragma unroll
    for (int oz = 0; oz < 3; oz++) {
      const double az = m2d * amr_w(sz, oz - 1);
#pragma unroll
      for (int oy = 0; oy < 3; oy++) W.b[3 * oz + oy][k] = az * amr_w(sy, oy - 1);
    }
#pragma unroll
    for (int o = 0; o < 3; o++) W.x[o][k] = amr_w(sx, o - 1);
  }
}

// one warp per target node: its 27 source nodes (ascending node index, the
// reference's visiting order; with l1 >= 3 distinct), those with particles
// compacted with their stencil slots and term offsets into shared memory,
// then the float sum over their particles in list order (amr_warp_sum)
__global__ void __launch_bounds__(kAmrT) k_amr_dens(int l1, const uint32_t* __restrict__ start,
                                                    const double* __restrict__ wts, uint64_t n,
                                                    float* __restrict__ dens) {
  __shared__ AmrSrc sh[kAmrT / 32][32];
  const unsigned FULL = 0xffffffffu, lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
  const uint64_t nn = (uint64_t)l1 * l1 * l1;
  const uint64_t t = (uint64_t)blockIdx.x * (kAmrT / 32) + wid;
  if (t >= nn) return;   // uniform over the warp
  const int tx = (int)(t % (uint64_t)l1), ty = (int)((t / (uint64_t)l1) % (uint64_t)l1),
            tz = (int)(t / ((uint64_t)l1 * l1));
  int sz3[3], sy3[3], sx3[3];
  amr_three(tz, l1, sz3);
  amr_three(ty, l1, sy3);
  amr_three(tx, l1, sx3);
  uint32_t s0 = 0, cnt = 0, slot = 0;
  if (lane < 27u) {
    const int a = (int)lane / 9, b = ((int)lane / 3) % 3, c = (int)lane % 3;
    // offset of the target from the source per axis, in {-1, 0, 1}
    const int oz = ((tz - sz3[a] + l1 + 1) % l1) - 1;
    const int oy = ((ty - sy3[b] + l1 + 1) % l1) - 1;
    const int ox = ((tx - sx3[c] + l1 + 1) % l1) - 1;
    const uint64_t s = ((uint64_t)sz3[a] * l1 + (uint64_t)sy3[b]) * l1 + (uint64_t)sx3[c];
    s0 = start[s];
    cnt = start[s + 1] - s0;
    slot = (uint32_t)(9 * (oz + 1) + 3 * (oy + 1) + (ox + 1));
  }
  uint32_t inc = cnt;   // inclusive scan of the counts
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const uint32_t v = __shfl_up_sync(FULL, inc, off);
    if ((int)lane >= off) inc += v;
  }
  const unsigned nz = __ballot_sync(FULL, cnt > 0u);
  if (cnt > 0u) sh[wid][__popc(nz & ((1u << lane) - 1u))] = AmrSrc{s0, cnt, slot, inc - cnt};
  __syncwarp();
  const uint32_t nterm = __shfl_sync(FULL, inc, 31);
  const float d = nterm ? amr_warp_sum<true>(sh[wid], __popc(nz), nterm, wts, n) : (float)(-1.0);
  if (lane == 0u) dens[t] = d;
}

// refinement flag of every coarse node: any of its 18 nodes at dz, dy in
// {-1, 0, 1}, dx in {0, 1} at or above the threshold
__global__ void __launch_bounds__(kAmrT) k_amr_flags(int l1, const float* __restrict__ dens, double thr,
                                                     uint8_t* __restrict__ flag) {
  const uint64_t nn = (uint64_t)l1 * l1 * l1;
  const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nn) return;
  const int tx = (int)(t % (uint64_t)l1), ty = (int)((t / (uint64_t)l1) % (uint64_t)l1),
            tz = (int)(t / ((uint64_t)l1 * l1));
  uint8_t f = 0;
  for (int dz = -1; dz <= 1 && !f; dz++)
    for (int dy = -1; dy <= 1 && !f; dy++)
      for (int dx = 0; dx <= 1 && !f; dx++) {
        const uint64_t s = ((uint64_t)((tz + dz + l1) % l1) * l1 + (uint64_t)((ty + dy + l1) % l1)) * l1 +
                           (uint64_t)((tx + dx + l1) % l1);
        f = (double)dens[s] >= thr;
      }
  flag[t] = f;
}

__device__ __forceinline__ bool amr_cov(const uint8_t* row, int x, int l1) {
  return row[x] || (x != l1 - 1 && row[x == 0 ? l1 - 1 : x - 1]);
}

// covered coarse nodes per coarse row
__global__ void __launch_bounds__(kAmrT) k_amr_rowcount(int l1, const uint8_t* __restrict__ flag,
                                                        uint32_t* __restrict__ rowcnt) {
  const uint64_t nr = (uint64_t)l1 * l1;
  const uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nr) return;
  const uint8_t* row = flag + r * (uint64_t)l1;
  uint32_t c = 0;
  for (int x = 0; x < l1; x++) c += amr_cov(row, x, l1);
  rowcnt[r] = c;
}

// fine nodes of every coarse row at their place in ascending (z, y, x);
// rowoff is the exclusive scan of rowcnt over the rows (rowoff[l1^2] = total)
__global__ void __launch_bounds__(kAmrT) k_amr_emit(int l1, const uint8_t* __restrict__ flag,
                                                    const uint32_t* __restrict__ rowcnt,
                                                    const uint32_t* __restrict__ rowoff, int64_t cap,
                                                    int32_t* __restrict__ zyx, int* __restrict__ err) {
  const uint64_t nr = (uint64_t)l1 * l1;
  const uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nr) return;
  const int zz = (int)(r / (uint64_t)l1), yy = (int)(r % (uint64_t)l1);
  const uint64_t plane = rowoff[(uint64_t)zz * l1];                 // covered nodes before plane zz
  const uint64_t P = rowoff[(uint64_t)(zz + 1) * l1] - plane;       // covered nodes in plane zz
  const uint64_t rip = rowoff[r] - plane;                           // ... before this row in the plane
  const uint64_t C = rowcnt[r];
  const uint8_t* row = flag + r * (uint64_t)l1;
  uint64_t rank = 0;
  for (int xx = 0; xx < l1; xx++) {
    if (!amr_cov(row, xx, l1)) continue;
    for (int a = 0; a < 2; a++)
      for (int b = 0; b < 2; b++)
        for (int c = 0; c < 2; c++) {
          const uint64_t k = 8 * plane + (uint64_t)a * 4 * P + 4 * rip + (uint64_t)b * 2 * C + 2 * rank + c;
          if ((int64_t)k >= cap) {
            atomicExch(err, 1);
            continue;
          }
          zyx[3 * k + 0] = 2 * zz + a;
          zyx[3 * k + 1] = 2 * yy + b;
          zyx[3 * k + 2] = 2 * xx + c;
        }
    rank++;
  }
}

void amr_cells(uint32_t n, const float* x, const float* y, const float* z, int l1, uint64_t* key, uint32_t* idx,
               uint32_t* count, int grid, cudaStream_t st) {
  k_amr_cells<<<grid, kAmrT, 0, st>>>(n, x, y, z, l1, key, idx, count);
}

void amr_dens(int l1, uint64_t n, const float* x, const float* y, const float* z, const uint32_t* start,
              const uint64_t* skey, const uint32_t* ord, double* wts, double* cfold, float* dens, int grid,
              cudaStream_t st) {
  const uint64_t nn = (uint64_t)l1 * l1 * l1;
  AmrW W;
  for (int o = 0; o < 9; o++) W.b[o] = wts + (uint64_t)o * n;
  for (int o = 0; o < 3; o++) W.x[o] = wts + (uint64_t)(9 + o) * n;
  k_amr_cfold<<<(unsigned)((l1 + kAmrT - 1) / kAmrT), kAmrT, 0, st>>>(l1, cfold);
  k_amr_weights<<<grid, kAmrT, 0, st>>>(l1, (uint32_t)n, skey, ord, x, y, z, cfold, W);
  k_amr_dens<<<(unsigned)((nn + kAmrT / 32 - 1) / (kAmrT / 32)), kAmrT, 0, st>>>(l1, start, wts, n, dens);
}

void amr_flags(int l1, const float* dens, double thr, uint8_t* flag, uint32_t* rowcnt, cudaStream_t st) {
  const uint64_t nn = (uint64_t)l1 * l1 * l1, nr = (uint64_t)l1 * l1;
  k_amr_flags<<<(unsigned)((nn + kAmrT - 1) / kAmrT), kAmrT, 0, st>>>(l1, dens, thr, flag);
  k_amr_rowcount<<<(unsigned)((nr + kAmrT - 1) / kAmrT), kAmrT, 0, st>>>(l1, flag, rowcnt);
}

void amr_emit(int l1, const uint8_t* flag, const uint32_t* rowcnt, const uint32_t* rowoff, int64_t cap, int32_t* zyx,
              int* err, cudaStream_t st) {
  const uint64_t nr = (uint64_t)l1 * l1;
  k_amr_emit<<<(unsigned)((nr + kAmrT - 1) / kAmrT), kAmrT, 0, st>>>(l1, flag, rowcnt, rowoff, cap, zyx, err);
}

}  // namespace ahfgpu
