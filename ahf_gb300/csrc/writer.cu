// writer.cu -- the AHF_particles file on the GPU.  Replaces
// WriteParticlesLegacy (src/libahf/ahf_io.c:1095-1175, default build) for a
// device-resident stage result: the exact bytes the reference's fprintf
// calls produce, formatted by the GPU ("%15lu\n" good-halo count; per halo
// of at least MINPART particles, in the caller's order j, "%lu %10ld\n"
// (npart, j); per kept particle "%" PRIu64 "\t%d\n" (id, (int)weight, or
// (int)(-PDM) = 1 without weights)).  Integer formatting only: the bytes are
// exact by construction.  Two passes: every halo block's byte count, a scan,
// then each block written by one CTA with a block scan of its line lengths.
#include <cstdint>

#include "common.cuh"

namespace ahfgpu {

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

__device__ __forceinline__ int line_len(const uint64_t* ids, const float* w, uint64_t e) {
  return ndig_u64(ids[e]) + 1 + len_int(particle_type(w, e)) + 1;
}

__device__ __forceinline__ int header_len(uint64_t npart, long long j) {   // j >= 0
  const int dj = ndig_u64((uint64_t)j);
  return ndig_u64(npart) + 1 + (dj > 10 ? dj : 10) + 1;
}

// pass 1: bytes of halo block j (0 below MINPART) into blk[j]; good-halo count
__global__ void __launch_bounds__(256) k_wp_count(int64_t nh, const int64_t* __restrict__ order,
                                                  const ahfgpu_halo* __restrict__ halo,
                                                  const uint64_t* __restrict__ moff, const uint64_t* __restrict__ member,
                                                  const uint64_t* __restrict__ ids, const float* __restrict__ w,
                                                  int64_t minpart, unsigned int* __restrict__ qhead,
                                                  uint64_t* __restrict__ blk, unsigned long long* __restrict__ good) {
  __shared__ int s_j;
  __shared__ unsigned long long s_sum;
  while (true) {
    if (threadIdx.x == 0) {
      const unsigned q = atomicAdd(qhead, 1u);
      s_j = q < (unsigned)nh ? (int)q : -1;
      s_sum = 0;
    }
    __syncthreads();
    const int j = s_j;
    if (j < 0) break;
    const int64_t i = order[j];
    const uint64_t np = halo[i].npart;
    if ((int64_t)np >= minpart) {
      unsigned long long mine = 0;
      for (uint64_t k = threadIdx.x; k < np; k += blockDim.x) mine += (unsigned long long)line_len(ids, w, member[moff[i] + k]);
      for (int o = 16; o > 0; o >>= 1) mine += __shfl_xor_sync(0xffffffffu, mine, o);
      if ((threadIdx.x & 31) == 0) atomicAdd(&s_sum, mine);
      __syncthreads();
      if (threadIdx.x == 0) {
        blk[j] = s_sum + (unsigned long long)header_len(np, j);
        atomicAdd(good, 1ull);
      }
    } else if (threadIdx.x == 0) {
      blk[j] = 0;
    }
    __syncthreads();
  }
}

// exclusive scan of nh u64 block sizes into boff[0..nh] (one block)
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

// pass 2: the file.  Bytes [0, 16) the count line; block j at 16 + boff[j].
__global__ void __launch_bounds__(256) k_wp_write(int64_t nh, const int64_t* __restrict__ order,
                                                  const ahfgpu_halo* __restrict__ halo,
                                                  const uint64_t* __restrict__ moff, const uint64_t* __restrict__ member,
                                                  const uint64_t* __restrict__ ids, const float* __restrict__ w,
                                                  int64_t minpart, unsigned int* __restrict__ qhead,
                                                  const uint64_t* __restrict__ boff,
                                                  const unsigned long long* __restrict__ good,
                                                  unsigned char* __restrict__ out) {
  __shared__ int s_j;
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
    if (threadIdx.x == 0) {
      const unsigned q = atomicAdd(qhead, 1u);
      s_j = q < (unsigned)nh ? (int)q : -1;
    }
    __syncthreads();
    const int j = s_j;
    __syncthreads();
    if (j < 0) break;
    const int64_t i = order[j];
    const uint64_t np = halo[i].npart;
    if ((int64_t)np < minpart) continue;
    unsigned char* p = out + 16 + boff[j];
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
    unsigned long long carry = (unsigned long long)hl;
    for (uint64_t base = 0; base < np; base += blockDim.x) {
      const uint64_t k = base + threadIdx.x;
      uint64_t e = 0, id = 0;
      int t = 0, len = 0;
      if (k < np) {
        e = member[moff[i] + k];
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
      if (k < np) {
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

void writer_count(int64_t nh, const int64_t* order, const ahfgpu_halo* halo, const uint64_t* moff,
                  const uint64_t* member, const uint64_t* ids, const float* w, int64_t minpart, unsigned int* qhead,
                  uint64_t* blk, unsigned long long* good, int grid, cudaStream_t st) {
  k_wp_count<<<grid, 256, 0, st>>>(nh, order, halo, moff, member, ids, w, minpart, qhead, blk, good);
}

void writer_offsets(const uint64_t* blk, int64_t nh, uint64_t* boff, cudaStream_t st) {
  k_wp_offsets<<<1, 1024, 0, st>>>(blk, nh, boff);
}

void writer_write(int64_t nh, const int64_t* order, const ahfgpu_halo* halo, const uint64_t* moff,
                  const uint64_t* member, const uint64_t* ids, const float* w, int64_t minpart, unsigned int* qhead,
                  const uint64_t* boff, const unsigned long long* good, unsigned char* out, int grid,
                  cudaStream_t st) {
  k_wp_write<<<grid, 256, 0, st>>>(nh, order, halo, moff, member, ids, w, minpart, qhead, boff, good, out);
}

}  // namespace ahfgpu
