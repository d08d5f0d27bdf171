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

// Largest list of classes 0 and 1.  Set once per device by the tuning at
// ahfgpu_init.
static uint64_t g_class_max[2] = {512, 16384};

// cap0: the largest class-0 list the class-0 kernel takes (512 for the
// 64-thread CTAs, whose shared-memory sort holds 512 pairs; more for the
// one-list-per-thread kernel, whose work space is sized per call)
void fp32c_set_class_max(uint64_t a, uint64_t b, uint64_t cap0) {
  a = a < 1 ? 1 : (a > cap0 ? cap0 : a);
  g_class_max[0] = a;
  g_class_max[1] = b < a ? a : b;
}

uint64_t fp32c_class_max(int cls) { return cls == 0 ? g_class_max[0] : cls == 1 ? g_class_max[1] : ~0ull; }

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
