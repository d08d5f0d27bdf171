// sfc.cu -- Hilbert keys of every particle and the particle order by key,
// replacing the keying loop and the qsort of src/main.c:342-356 (libsfc's
// sfc_curve_calcKey with SFC_CURVE_HILBERT at BITS_PER_DIMENSION, then
// qsort with cmp_sfckey_part).
//
// Key: grid coordinates c_d = trunc(x_d 2^bits) capped at 2^bits - 1
// (libsfc/hilbert_util.c:69-92), then the index of that cell on libsfc's
// Hilbert curve (libsfc/hilbert.c:197-240), level by level from the top:
// g_b the 3-bit group of bit b of (c_0, c_1, c_2), G_b = g_b ^ g_{b+1};
// emit rotr3(G_b ^ flip, rot); flip = 1 << rot; rot += 1 (+1 or +2 when the
// lowest set bit of the emitted group is bit 0 or 1), mod 3.  Bit 2 of every
// level but the top one is inverted and the index Gray-decoded.  For a
// float position in [0, 1] the scaling by 2^bits is exact in float, so the
// truncation equals the reference's double one.
//
// Sort: least-significant-digit radix sort with 8-bit digits over the 3 bits
// key bits (8 passes at 21 bits), stable, so equal keys keep their original
// index order.  Per pass: a digit histogram of every 4096-key tile (one
// block per tile), an exclusive scan of the digit-major histogram (three
// kernels), and a stable scatter per tile: each warp ranks its 512 keys 32
// at a time with __match_any_sync, the tile is reordered by digit in shared
// memory, and the keys are written out in that order, so each digit's run
// of the tile (16 keys on average) lands as one contiguous, coalesced piece.
// Every store index is checked against n; a violation sets the error flag
// instead of writing.
#include <cstdint>

#include "common.cuh"
#include "sfc_key.cuh"

namespace ahfgpu {

constexpr int kSfcTile = 4096;          // keys per tile (one block)
constexpr int kSfcT = 256;              // threads per tile block
constexpr int kSfcWarps = kSfcT / 32;   // 8 warps, 512 keys each
constexpr int kSfcPer = kSfcTile / kSfcT;
constexpr int kScanChunk = 4096;        // values per block of the generic scan

struct SfcTileSmem {
  uint64_t key[kSfcTile];               // the tile, reordered by digit
  uint32_t idx[kSfcTile];
  uint32_t wcnt[kSfcWarps][256];        // per-warp digit counts, then offsets
  uint32_t dstart[256];                 // tile-local start of each digit
  uint32_t gbase[256];                  // where the tile's digit-d keys go
  uint32_t wsum[kSfcWarps];
};

__global__ void __launch_bounds__(256) k_sfc_keys(uint32_t n, const float* __restrict__ x,
                                                  const float* __restrict__ y, const float* __restrict__ z, int bits,
                                                  uint64_t* __restrict__ keys, uint32_t* __restrict__ idx) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    keys[i] = hilbert_key(x[i], y[i], z[i], bits);
    idx[i] = i;
  }
}

// digit counts of every tile, digit-major: gh[d * ntiles + t]
__global__ void __launch_bounds__(kSfcT) k_sfc_hist(uint32_t n, uint32_t ntiles, const uint64_t* __restrict__ keys,
                                                    int shift, uint32_t* __restrict__ gh) {
  __shared__ uint32_t cnt[256];
  const uint32_t tile = blockIdx.x;
  cnt[threadIdx.x] = 0;
  __syncthreads();
  const uint64_t base = (uint64_t)tile * kSfcTile;
  for (int r = 0; r < kSfcPer; r++) {
    const uint64_t i = base + (uint64_t)r * kSfcT + threadIdx.x;
    if (i < n) atomicAdd(&cnt[(uint32_t)(keys[i] >> shift) & 255u], 1u);
  }
  __syncthreads();
  gh[(uint64_t)threadIdx.x * ntiles + tile] = cnt[threadIdx.x];
}

// stable scatter of one tile per block; goff[d * ntiles + t] is where tile
// t's first key of digit d goes
__global__ void __launch_bounds__(kSfcT) k_sfc_scatter(uint32_t n, uint32_t ntiles, const uint64_t* __restrict__ kin,
                                                       const uint32_t* __restrict__ iin, int shift,
                                                       const uint32_t* __restrict__ goff,
                                                       uint64_t* __restrict__ kout, uint32_t* __restrict__ iout,
                                                       int* __restrict__ err) {
  extern __shared__ __align__(16) unsigned char sfc_smem[];
  SfcTileSmem& S = *reinterpret_cast<SfcTileSmem*>(sfc_smem);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const uint32_t tile = blockIdx.x;
  const uint64_t base = (uint64_t)tile * kSfcTile;
  for (int d = lane; d < 256; d += 32) S.wcnt[w][d] = 0;
  S.gbase[threadIdx.x] = goff[(uint64_t)threadIdx.x * ntiles + tile];
  __syncwarp();
  // 1. ranks within each warp's 512 consecutive keys, in order
  const uint32_t lt = (1u << lane) - 1u;
  uint64_t k[kSfcPer];
  uint32_t v[kSfcPer], rank[kSfcPer], dig[kSfcPer];
#pragma unroll
  for (int r = 0; r < kSfcPer; r++) {
    const uint64_t i = base + (uint64_t)w * (kSfcTile / kSfcWarps) + (uint64_t)r * 32 + lane;
    const bool valid = i < n;
    k[r] = valid ? kin[i] : 0ull;
    v[r] = valid ? iin[i] : 0u;
    dig[r] = valid ? ((uint32_t)(k[r] >> shift) & 255u) : 256u + (uint32_t)lane;
    const uint32_t peers = __match_any_sync(0xffffffffu, dig[r]);
    rank[r] = valid ? S.wcnt[w][dig[r]] + __popc(peers & lt) : 0u;
    __syncwarp();
    if (valid && lane == __ffs(peers) - 1) S.wcnt[w][dig[r]] += __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  // 2. per digit (thread = digit): the warps' offsets within the digit, the
  //    digit's total; then the digits' starts in the tile (a block scan)
  uint32_t tot = 0;
#pragma unroll
  for (int q = 0; q < kSfcWarps; q++) {
    const uint32_t c = S.wcnt[q][threadIdx.x];
    S.wcnt[q][threadIdx.x] = tot;
    tot += c;
  }
  uint32_t inc = tot;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) S.wsum[w] = inc;
  __syncthreads();
  uint32_t before = 0;
  for (int q = 0; q < w; q++) before += S.wsum[q];
  S.dstart[threadIdx.x] = before + inc - tot;
  __syncthreads();
  // 3. the tile reordered by digit in shared memory
#pragma unroll
  for (int r = 0; r < kSfcPer; r++) {
    if (dig[r] < 256u) {
      const uint32_t p = S.dstart[dig[r]] + S.wcnt[w][dig[r]] + rank[r];
      S.key[p] = k[r];
      S.idx[p] = v[r];
    }
  }
  __syncthreads();
  // 4. out in that order: each digit's run contiguous in the output
  const uint64_t left = (uint64_t)n - base;
  const uint32_t valid_n = left < (uint64_t)kSfcTile ? (uint32_t)left : (uint32_t)kSfcTile;
  for (uint32_t p = threadIdx.x; p < valid_n; p += kSfcT) {
    const uint64_t key = S.key[p];
    const uint32_t d = (uint32_t)(key >> shift) & 255u;
    const uint64_t pos = (uint64_t)S.gbase[d] + (p - S.dstart[d]);
    if (pos < n) {
      kout[pos] = key;
      iout[pos] = S.idx[p];
    } else {
      atomicExch(err, 1);
    }
  }
}

// generic exclusive scan of m uint32 values (totals below 2^32), three steps
__global__ void __launch_bounds__(256) k_scan_sums(const uint32_t* __restrict__ in, uint32_t m,
                                                   uint32_t* __restrict__ part) {
  __shared__ uint32_t ws[8];
  const uint64_t b0 = (uint64_t)blockIdx.x * kScanChunk;
  uint32_t s = 0;
  for (int k = threadIdx.x; k < kScanChunk; k += 256) {
    const uint64_t i = b0 + k;
    if (i < m) s += in[i];
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (int k = 0; k < 8; k++) t += ws[k];
    part[blockIdx.x] = t;
  }
}

// in-place exclusive scan of np values (one block of 1024)
__global__ void __launch_bounds__(1024) k_scan_parts(uint32_t* __restrict__ part, uint32_t np) {
  __shared__ uint32_t ws[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint32_t carry = 0;
  for (uint32_t base = 0; base < np; base += 1024) {
    const uint32_t i = base + threadIdx.x;
    const uint32_t v = i < np ? part[i] : 0u;
    uint32_t inc = v;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += t;
    }
    if (lane == 31) ws[wid] = inc;
    __syncthreads();
    if (wid == 0) {
      uint32_t x = ws[lane];
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += t;
      }
      ws[lane] = x;
    }
    __syncthreads();
    if (i < np) part[i] = carry + (wid ? ws[wid - 1] : 0u) + inc - v;
    carry += ws[31];
    __syncthreads();
  }
}

__global__ void __launch_bounds__(256) k_scan_apply(const uint32_t* __restrict__ in, uint32_t m,
                                                    const uint32_t* __restrict__ part, uint32_t* __restrict__ out) {
  __shared__ uint32_t ws[8];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const uint64_t b0 = (uint64_t)blockIdx.x * kScanChunk;
  uint32_t carry = part[blockIdx.x];
  for (int base = 0; base < kScanChunk; base += 256) {
    const uint64_t i = b0 + base + threadIdx.x;
    const uint32_t v = i < m ? in[i] : 0u;
    uint32_t inc = v;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += t;
    }
    if (lane == 31) ws[wid] = inc;
    __syncthreads();
    uint32_t before = 0, total = 0;
    for (int k = 0; k < 8; k++) {
      if (k < wid) before += ws[k];
      total += ws[k];
    }
    if (i < m) out[i] = carry + before + inc - v;
    carry += total;
    __syncthreads();
  }
}

__global__ void __launch_bounds__(256) k_sfc_order(uint32_t n, const uint32_t* __restrict__ idx,
                                                   uint64_t* __restrict__ order) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) order[i] = idx[i];
}

uint32_t sfc_ntiles(uint32_t n) { return (n + kSfcTile - 1) / kSfcTile; }
uint32_t sfc_scan_blocks(uint32_t m) { return (m + kScanChunk - 1) / kScanChunk; }

void sfc_keys(uint32_t n, const float* x, const float* y, const float* z, int bits, uint64_t* keys, uint32_t* idx,
              int grid, cudaStream_t st) {
  k_sfc_keys<<<grid, 256, 0, st>>>(n, x, y, z, bits, keys, idx);
}

// one radix pass: (kin, iin) -> (kout, iout) by the digit at `shift`;
// gh and goff hold 256 * ntiles values, part sfc_scan_blocks(256 * ntiles)
void sfc_pass(uint32_t n, const uint64_t* kin, const uint32_t* iin, int shift, uint32_t* gh, uint32_t* goff,
              uint32_t* part, uint64_t* kout, uint32_t* iout, int* err, cudaStream_t st) {
  const uint32_t nt = sfc_ntiles(n);
  const uint32_t m = 256u * nt;
  const uint32_t nb = sfc_scan_blocks(m);
  cudaFuncSetAttribute(k_sfc_scatter, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SfcTileSmem));
  k_sfc_hist<<<nt, kSfcT, 0, st>>>(n, nt, kin, shift, gh);
  k_scan_sums<<<nb, 256, 0, st>>>(gh, m, part);
  k_scan_parts<<<1, 1024, 0, st>>>(part, nb);
  k_scan_apply<<<nb, 256, 0, st>>>(gh, m, part, goff);
  k_sfc_scatter<<<nt, kSfcT, sizeof(SfcTileSmem), st>>>(n, nt, kin, iin, shift, goff, kout, iout, err);
}

void sfc_order(uint32_t n, const uint32_t* idx, uint64_t* order, int grid, cudaStream_t st) {
  k_sfc_order<<<grid, 256, 0, st>>>(n, idx, order);
}

}  // namespace ahfgpu
