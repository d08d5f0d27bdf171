// writer.cu -- the AHF_particles files on the GPU, for a device-resident
// stage result.
//
// ASCII: WriteParticlesLegacy (src/libahf/ahf_io.c:1095-1175, default
// build): the exact bytes the reference's fprintf calls produce ("%15lu\n"
// good-halo count; per halo of at least MINPART particles, in the caller's
// order j, "%lu %10ld\n" (npart, j); per kept particle "%" PRIu64 "\t%d\n"
// (id, (int)weight, or (int)(-PDM) = 1 without weights)).  Integer
// formatting only: the bytes are exact by construction.
//
// Binary: ahf_binwrite_particles (src/libahf/ahf_io.c:1733-1855, AHFbinary
// build without GAS_PARTICLES or AHFnewHaloIDs): int32 1, uint64 haloes
// written, uint32 2 (columns); per halo j with at least MINPART particles,
// uint64 npart and uint64 j, then per kept particle uint64 id and int32 1
// (the type is (int32)(-u) only with GAS_PARTICLES).  Native byte order, no
// padding: a halo block is 16 + 12 n bytes, so every block and every field
// starts on a 4-byte boundary and the file is written as 32-bit words.
//
// Both cut every written halo block into chunks of kChunk particles (chunk 0
// also carries the block header) taken from one queue, so the largest lists
// (~2e6 lines) spread over many CTAs instead of setting the tail.
#include <cstdint>

#include "common.cuh"

namespace ahfgpu {

constexpr int kChunk = 4096;
constexpr int kUnroll = 4;

__device__ __forceinline__ int ndig_u64(uint64_t v) {
  int n = 1;
  while (v >= 10) { v /= 10; n++; }
  return n;
}

__device__ __forceinline__ int len_int(int v) { return v < 0 ? 1 + ndig_u64((uint64_t)(-(long long)v)) : ndig_u64((uint64_t)v); }

// digits of v right-aligned ending just before `end`
__device__ __forceinline__ void put_u64(unsigned char* end, uint64_t v) {
  do { *--end = (unsigned char)('0' + (int)(v % 10)); v /= 10; } while (v);
}

__device__ __forceinline__ int particle_type(const float* w, uint64_t e) {
  return w ? __float2int_rz(w[e]) : 1;   // (int)weight, or (int)(-PDM) with PDM = -1
}

__device__ __forceinline__ int header_len(uint64_t npart, long long j) {   // j >= 0
  const int dj = ndig_u64((uint64_t)j);
  return ndig_u64(npart) + 1 + (dj > 10 ? dj : 10) + 1;
}

// per output position j: chunks of the block (0 below MINPART), the binary
// block's bytes, and the number of blocks written
__global__ void __launch_bounds__(256) k_w_sizes(int64_t nh, const int64_t* __restrict__ order,
                                                 const ahfgpu_halo* __restrict__ halo, int64_t minpart,
                                                 uint64_t* __restrict__ blk, uint64_t* __restrict__ nchunk,
                                                 unsigned long long* __restrict__ good) {
  unsigned long long mine = 0;
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < nh; j += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t np = halo[order[j]].npart;
    const bool ok = (int64_t)np >= minpart;
    if (blk) blk[j] = ok ? 16 + 12 * np : 0;
    nchunk[j] = ok ? (np > 0 ? (np + kChunk - 1) / kChunk : 1) : 0;   // chunk 0 writes the block header
    mine += ok;
  }
  for (int o = 16; o > 0; o >>= 1) mine += __shfl_xor_sync(0xffffffffu, mine, o);
  if ((threadIdx.x & 31) == 0 && mine) atomicAdd(good, mine);
}

// exclusive scan of n u64 values into out[0..n] (one block)
__global__ void k_wp_offsets(const uint64_t* __restrict__ blk, int64_t nh, uint64_t* __restrict__ boff) {
  __shared__ unsigned long long wsum[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  unsigned long long carry = 0;
  for (int64_t base = 0; base < nh; base += blockDim.x) {
    const int64_t i = base + threadIdx.x;
    const unsigned long long v = i < nh ? blk[i] : 0ull;
    unsigned long long inc = v;
    for (int o = 1; o < 32; o <<= 1) {
      unsigned long long t = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += t;
    }
    if (lane == 31) wsum[wid] = inc;
    __syncthreads();
    if (wid == 0) {
      unsigned long long x = lane < nw ? wsum[lane] : 0ull;
      for (int o = 1; o < 32; o <<= 1) {
        unsigned long long t = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += t;
      }
      wsum[lane] = x;
    }
    __syncthreads();
    if (i < nh) boff[i] = carry + (wid ? wsum[wid - 1] : 0ull) + inc - v;
    carry += wsum[nw - 1];
    __syncthreads();
  }
  if (threadIdx.x == 0) boff[nh] = carry;
}

// thread 0: the next chunk of the queue as (block j, chunk c of the block);
// j = -1 when the queue is empty.  coff is the exclusive scan of the chunk
// counts, coff[nh] the total.
__device__ __forceinline__ void claim_chunk(unsigned int* qhead, const uint64_t* __restrict__ coff, int64_t nh,
                                            long long& s_j, unsigned long long& s_c) {
  const unsigned q = atomicAdd(qhead, 1u);
  if ((uint64_t)q >= coff[nh]) {
    s_j = -1;
    return;
  }
  int64_t lo = 0, hi = nh;   // coff[lo] <= q < coff[hi]
  while (hi - lo > 1) {
    const int64_t mid = (lo + hi) >> 1;
    if (coff[mid] <= q) lo = mid; else hi = mid;
  }
  s_j = lo;
  s_c = q - coff[lo];
}

// ---------------------------------------------------------------------------
// ASCII, pass 1: bytes of every chunk (its lines, plus the block header in
// chunk 0) into cbytes[coff[j] + c]
__global__ void __launch_bounds__(256) k_wp_count(int64_t nh, const int64_t* __restrict__ order,
                                                  const ahfgpu_halo* __restrict__ halo,
                                                  const uint64_t* __restrict__ moff, const uint64_t* __restrict__ member,
                                                  const uint64_t* __restrict__ ids, const float* __restrict__ w,
                                                  const uint64_t* __restrict__ coff, unsigned int* __restrict__ qhead,
                                                  uint64_t* __restrict__ cbytes) {
  __shared__ long long s_j;
  __shared__ unsigned long long s_c, s_sum;
  while (true) {
    if (threadIdx.x == 0) {
      claim_chunk(qhead, coff, nh, s_j, s_c);
      s_sum = 0;
    }
    __syncthreads();
    const long long j = s_j;
    const uint64_t c = s_c;
    if (j < 0) break;
    const int64_t i = order[j];
    const uint64_t np = halo[i].npart;
    const uint64_t k0 = c * kChunk, k1 = np < k0 + kChunk ? np : k0 + kChunk;
    const uint64_t* mem = member + moff[i];
    unsigned long long mine = 0;
    for (uint64_t base = k0 + threadIdx.x; base < k1; base += (uint64_t)blockDim.x * kUnroll) {
      uint64_t e[kUnroll];
#pragma unroll
      for (int u = 0; u < kUnroll; u++) {
        const uint64_t k = base + (uint64_t)u * blockDim.x;
        e[u] = k < k1 ? mem[k] : 0;
      }
#pragma unroll
      for (int u = 0; u < kUnroll; u++) {
        const uint64_t k = base + (uint64_t)u * blockDim.x;
        if (k < k1) mine += (unsigned long long)(ndig_u64(ids[e[u]]) + 1 + len_int(particle_type(w, e[u])) + 1);
      }
    }
    for (int o = 16; o > 0; o >>= 1) mine += __shfl_xor_sync(0xffffffffu, mine, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(&s_sum, mine);
    __syncthreads();
    if (threadIdx.x == 0) cbytes[coff[j] + c] = s_sum + (c == 0 ? (unsigned long long)header_len(np, j) : 0ull);
    __syncthreads();
  }
}

// ASCII, pass 2: the file.  Bytes [0, 16) the count line; chunk q at
// 16 + cboff[q], its lines placed by a block scan of their lengths.
__global__ void __launch_bounds__(256) k_wp_write(int64_t nh, const int64_t* __restrict__ order,
                                                  const ahfgpu_halo* __restrict__ halo,
                                                  const uint64_t* __restrict__ moff, const uint64_t* __restrict__ member,
                                                  const uint64_t* __restrict__ ids, const float* __restrict__ w,
                                                  const uint64_t* __restrict__ coff, unsigned int* __restrict__ qhead,
                                                  const uint64_t* __restrict__ cboff,
                                                  const unsigned long long* __restrict__ good,
                                                  unsigned char* __restrict__ out) {
  __shared__ long long s_j;
  __shared__ unsigned long long s_c;
  __shared__ unsigned long long wsum[8];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    // "%15lu\n"
    const unsigned long long gcount = *good;
    for (int k = 0; k < 15; k++) out[k] = ' ';
    put_u64(out + 15, gcount);
    out[15] = '\n';
  }
  while (true) {
    if (threadIdx.x == 0) claim_chunk(qhead, coff, nh, s_j, s_c);
    __syncthreads();
    const long long j = s_j;
    const uint64_t c = s_c;
    __syncthreads();
    if (j < 0) break;
    const int64_t i = order[j];
    const uint64_t np = halo[i].npart;
    unsigned char* p = out + 16 + cboff[coff[j] + c];
    unsigned long long carry = 0;
    if (c == 0) {
      const int hl = header_len(np, j);
      if (threadIdx.x == 0) {
        // "%lu %10ld\n"
        const int dn = ndig_u64(np);
        put_u64(p + dn, np);
        p[dn] = ' ';
        unsigned char* e = p + hl - 1;
        *e = '\n';
        for (unsigned char* q = p + dn + 1; q < e; q++) *q = ' ';
        put_u64(e, (uint64_t)j);
      }
      carry = (unsigned long long)hl;
    }
    const uint64_t k0 = c * kChunk, k1 = np < k0 + kChunk ? np : k0 + kChunk;
    const uint64_t* mem = member + moff[i];
    for (uint64_t base = k0; base < k1; base += blockDim.x) {
      const uint64_t k = base + threadIdx.x;
      uint64_t e = 0, id = 0;
      int t = 0, len = 0;
      if (k < k1) {
        e = mem[k];
        id = ids[e];
        t = particle_type(w, e);
        len = ndig_u64(id) + 1 + len_int(t) + 1;
      }
      unsigned long long inc = (unsigned long long)len;
      for (int o = 1; o < 32; o <<= 1) {
        unsigned long long v = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += v;
      }
      if (lane == 31) wsum[wid] = inc;
      __syncthreads();
      unsigned long long before = 0, total = 0;
      for (int x = 0; x < nw; x++) {
        if (x < wid) before += wsum[x];
        total += wsum[x];
      }
      if (k < k1) {
        // "%" PRIu64 "\t%d\n"
        unsigned char* q = p + carry + before + inc - (unsigned long long)len;
        const int di = ndig_u64(id);
        put_u64(q + di, id);
        q[di] = '\t';
        unsigned char* te = q + len - 1;
        *te = '\n';
        if (t < 0) {
          put_u64(te, (uint64_t)(-(long long)t));
          q[di + 1] = '-';
        } else {
          put_u64(te, (uint64_t)t);
        }
      }
      carry += total;
      __syncthreads();
    }
  }
}

// ---------------------------------------------------------------------------
// Binary: one 32-particle group of a warp is 96 words; lane l stores words
// l, l+32, l+64 (word w is field w % 3 of particle w / 3: id low, id high,
// type 1), so each store instruction covers 128 contiguous bytes.
__device__ __forceinline__ void wb_group(uint32_t* __restrict__ rec, uint64_t id, int cnt, int lane) {
  const uint32_t lo = (uint32_t)id, hi = (uint32_t)(id >> 32);
#pragma unroll
  for (int r = 0; r < 3; r++) {
    const int w = lane + 32 * r;
    const int src = w / 3, f = w - 3 * src;
    const uint32_t a = __shfl_sync(0xffffffffu, lo, src), b = __shfl_sync(0xffffffffu, hi, src);
    if (src < cnt) rec[w] = f == 0 ? a : (f == 1 ? b : 1u);
  }
}

__global__ void __launch_bounds__(256) k_wb_write(int64_t nh, const int64_t* __restrict__ order,
                                                  const ahfgpu_halo* __restrict__ halo,
                                                  const uint64_t* __restrict__ moff, const uint64_t* __restrict__ member,
                                                  const uint64_t* __restrict__ ids, const uint64_t* __restrict__ boff,
                                                  const uint64_t* __restrict__ coff,
                                                  const unsigned long long* __restrict__ good,
                                                  unsigned int* __restrict__ qhead, uint32_t* __restrict__ out) {
  __shared__ long long s_j;
  __shared__ unsigned long long s_c;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const unsigned long long gc = *good;
    out[0] = 1u;
    out[1] = (uint32_t)gc;
    out[2] = (uint32_t)(gc >> 32);
    out[3] = 2u;
  }
  while (true) {
    if (threadIdx.x == 0) claim_chunk(qhead, coff, nh, s_j, s_c);
    __syncthreads();
    const long long j = s_j;
    const uint64_t c = s_c;
    __syncthreads();
    if (j < 0) break;
    const int64_t i = order[j];
    const uint64_t np = halo[i].npart;
    uint32_t* blkw = out + (16 + boff[j]) / 4;
    if (c == 0 && threadIdx.x < 4) {
      const uint64_t v = threadIdx.x < 2 ? np : (uint64_t)j;
      blkw[threadIdx.x] = (threadIdx.x & 1) ? (uint32_t)(v >> 32) : (uint32_t)v;
    }
    const uint64_t k0 = c * kChunk, k1 = np < k0 + kChunk ? np : k0 + kChunk;
    const uint64_t* mem = member + moff[i];
    uint32_t* rec = blkw + 4;
    for (uint64_t base = k0 + (uint64_t)wid * 32 * kUnroll; base < k1; base += (uint64_t)blockDim.x * kUnroll) {
      uint64_t e[kUnroll], id[kUnroll];
#pragma unroll
      for (int u = 0; u < kUnroll; u++) {
        const uint64_t k = base + 32 * u + lane;
        e[u] = k < k1 ? mem[k] : 0;
      }
#pragma unroll
      for (int u = 0; u < kUnroll; u++) {
        const uint64_t k = base + 32 * u + lane;
        id[u] = k < k1 ? ids[e[u]] : 0;
      }
#pragma unroll
      for (int u = 0; u < kUnroll; u++) {
        const uint64_t g0 = base + 32 * u;
        if (g0 < k1) {
          const int cnt = k1 - g0 < 32 ? (int)(k1 - g0) : 32;
          wb_group(rec + 3 * g0, id[u], cnt, lane);
        }
      }
    }
  }
}

void writer_sizes(int64_t nh, const int64_t* order, const ahfgpu_halo* halo, int64_t minpart, uint64_t* blk,
                  uint64_t* nchunk, unsigned long long* good, int grid, cudaStream_t st) {
  k_w_sizes<<<grid, 256, 0, st>>>(nh, order, halo, minpart, blk, nchunk, good);
}

void writer_offsets(const uint64_t* blk, int64_t nh, uint64_t* boff, cudaStream_t st) {
  k_wp_offsets<<<1, 1024, 0, st>>>(blk, nh, boff);
}

void writer_count(int64_t nh, const int64_t* order, const ahfgpu_halo* halo, const uint64_t* moff,
                  const uint64_t* member, const uint64_t* ids, const float* w, const uint64_t* coff,
                  unsigned int* qhead, uint64_t* cbytes, int grid, cudaStream_t st) {
  k_wp_count<<<grid, 256, 0, st>>>(nh, order, halo, moff, member, ids, w, coff, qhead, cbytes);
}

void writer_write(int64_t nh, const int64_t* order, const ahfgpu_halo* halo, const uint64_t* moff,
                  const uint64_t* member, const uint64_t* ids, const float* w, const uint64_t* coff,
                  unsigned int* qhead, const uint64_t* cboff, const unsigned long long* good, unsigned char* out,
                  int grid, cudaStream_t st) {
  k_wp_write<<<grid, 256, 0, st>>>(nh, order, halo, moff, member, ids, w, coff, qhead, cboff, good, out);
}

void writer_bin_write(int64_t nh, const int64_t* order, const ahfgpu_halo* halo, const uint64_t* moff,
                      const uint64_t* member, const uint64_t* ids, const uint64_t* boff, const uint64_t* coff,
                      const unsigned long long* good, unsigned int* qhead, uint32_t* out, int grid, cudaStream_t st) {
  k_wb_write<<<grid, 256, 0, st>>>(nh, order, halo, moff, member, ids, boff, coff, good, qhead, out);
}

}  // namespace ahfgpu
