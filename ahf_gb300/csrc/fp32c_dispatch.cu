// fp32c_dispatch.cu -- size classes of the FP32-compensated form: class 0
// takes lists of up to 512 particles with two-warp CTAs (4 haloes in flight
// per SM), class 1 lists up to 16384 with four-warp CTAs, class 2 the rest
// with eight-warp CTAs.
#include <cstdint>
#include <cstdio>
#include <cstdlib>

#include "common.cuh"

namespace ahfgpu {

void launch_fp32c_class0(const DevParams&, const DevBatch&, const Work&, int, cudaStream_t);
void launch_fp32c_class1(const DevParams&, const DevBatch&, const Work&, int, cudaStream_t);
void launch_fp32c_class2(const DevParams&, const DevBatch&, const Work&, int, cudaStream_t);
int fp32c_occupancy_class0();
int fp32c_occupancy_class1();
int fp32c_occupancy_class2();

// Largest list of classes 0 and 1.  AHFGPU_CLASS_MAX="a,b" overrides them
// (tuning runs); read once.
uint64_t fp32c_class_max(int cls) {
  static uint64_t lim[2] = {0, 0};
  if (lim[0] == 0) {
    uint64_t a = 512, b = 16384;
    if (const char* e = getenv("AHFGPU_CLASS_MAX")) {
      unsigned long long x = 0, y = 0;
      if (sscanf(e, "%llu,%llu", &x, &y) == 2 && x >= 1 && x <= 512 && y >= x) { a = x; b = y; }
    }
    lim[1] = b;
    lim[0] = a;
  }
  return cls == 0 ? lim[0] : cls == 1 ? lim[1] : ~0ull;
}

void launch_fp32c(int cls, const DevParams& P, const DevBatch& B, const Work& W, int grid, cudaStream_t st) {
  if (cls == 0) launch_fp32c_class0(P, B, W, grid, st);
  else if (cls == 1) launch_fp32c_class1(P, B, W, grid, st);
  else launch_fp32c_class2(P, B, W, grid, st);
}

int fp32c_max_blocks_per_sm(int cls) {
  if (cls == 0) return fp32c_occupancy_class0();
  if (cls == 1) return fp32c_occupancy_class1();
  return fp32c_occupancy_class2();
}

}  // namespace ahfgpu
