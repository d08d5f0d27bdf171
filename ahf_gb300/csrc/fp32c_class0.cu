// fp32c_class0.cu -- instantiation of the FP32-compensated halo kernel for
// size class 0 (64 threads per CTA, shared-memory sort SortSmemT<512, 16>).  One
// translation unit per class so the classes compile in parallel.
#include "halo_fp32c.cuh"

namespace ahfgpu {

// the only CTA shape built for class 0: 64 threads, no register cap
constexpr int kT0 = 64;
constexpr int kMinB0 = 1;
using SS0 = SortSmemT<512, 16>;

void launch_fp32c_class0(const DevParams& P, const DevBatch& B, const Work& W, int grid, cudaStream_t st) {
  halo_fp32c_kernel<kT0, SS0, kMinB0><<<grid, kT0, sizeof(F32Smem<SS0, kT0>), st>>>(P, B, W);
}

int fp32c_occupancy_class0() {
  int nb = 0;
  cudaFuncSetAttribute(halo_fp32c_kernel<kT0, SS0, kMinB0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)sizeof(F32Smem<SS0, kT0>));
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, halo_fp32c_kernel<kT0, SS0, kMinB0>, kT0, sizeof(F32Smem<SS0, kT0>));
  return nb;
}

}  // namespace ahfgpu
