// sfc_key.cuh -- the Hilbert key of one position (libsfc's
// sfc_curve_calcKey with SFC_CURVE_HILBERT: libsfc/hilbert_util.c:69-92 and
// hilbert_c2i, libsfc/hilbert.c:197-240), restated level by level from the
// most significant bit.  Host and device code: the same level loop runs in
// the sort kernel and in the host-compiled check of it.
#pragma once

#include <cstdint>

#ifdef __CUDACC__
#define AHFGPU_HD __host__ __device__ __forceinline__
#else
#define AHFGPU_HD inline
#endif

namespace ahfgpu {

// grid coordinate trunc(x 2^bits), capped at 2^bits - 1; x in [0, 1]: the
// scaling by a power of two is exact in float, as in the reference's double
AHFGPU_HD uint32_t sfc_coord(float x, int bits) {
  const float scale = (float)(1u << bits);
  const uint32_t top = (1u << bits) - 1u;
#ifdef __CUDA_ARCH__
  // a 32-bit conversion (saturating: negative and NaN give 0, past 2^32 - 1
  // the maximum, then the cap); the 64-bit one would issue on the FP64 pipe
  const uint32_t q = __float2uint_rz(__fmul_rn(x, scale));
#else
  const float p = x * scale;
  const uint32_t q = p > 0.f ? (p < 4194304.f ? (uint32_t)p : top) : 0u;
#endif
  return q > top ? top : q;
}

// g_b the 3-bit group of bit b of (c0, c1, c2), G_b = g_b ^ g_{b+1}; each
// level emits rotr3(G_b ^ flip, rot), then flip = 1 << rot and rot advances
// by 1, plus 1 or 2 when the lowest set bit of the emitted group is bit 0 or
// bit 1 (mod 3).  Bit 2 of every level but the top one is inverted and the
// index Gray-decoded.
AHFGPU_HD uint64_t hilbert_key_cells(uint32_t c0, uint32_t c1, uint32_t c2, int bits) {
  uint64_t key = 0;
  uint32_t rot = 0, flip = 0, gup = 0;
  for (int b = bits - 1; b >= 0; b--) {
    const uint32_t g = ((c0 >> b) & 1u) | (((c1 >> b) & 1u) << 1) | (((c2 >> b) & 1u) << 2);
    const uint32_t t = (g ^ gup ^ flip) & 7u;
    const uint32_t r = ((t >> rot) | (t << (3u - rot))) & 7u;
    key = (key << 3) | r;
    flip = 1u << rot;
    rot += 1u + (r & (0u - r) & 3u);   // the lowest set bit, if bit 0 or 1, is the extra advance
    if (rot >= 3u) rot -= 3u;
    gup = g;
  }
  for (int b = 0; b + 1 < bits; b++) key ^= 4ull << (3 * b);
  for (int s = 1; s < 3 * bits; s *= 2) key ^= key >> s;
  return key;
}

AHFGPU_HD uint64_t hilbert_key(float x, float y, float z, int bits) {
  return hilbert_key_cells(sfc_coord(x, bits), sfc_coord(y, bits), sfc_coord(z, bits), bits);
}

}  // namespace ahfgpu
