// fp32c_class1.cu -- instantiation of the FP32-compensated halo kernel for
// size class 1 (128 threads per CTA, shared-memory sort SortSmemT<2048, 1024>).  One
// translation unit per class so the classes compile in parallel.
#include "halo_fp32c.cuh"

namespace ahfgpu {

void launch_fp32c_class1(const DevParams& P, const DevBatch& B, const Work& W, int grid, cudaStream_t st) {
  halo_fp32c_kernel<128, SortSmemT<2048, 1024>><<<grid, 128, sizeof(F32Smem<SortSmemT<2048, 1024>, 128>), st>>>(P, B, W);
}

int fp32c_occupancy_class1() {
  int nb = 0;
  cudaFuncSetAttribute(halo_fp32c_kernel<128, SortSmemT<2048, 1024>>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)sizeof(F32Smem<SortSmemT<2048, 1024>, 128>));
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, halo_fp32c_kernel<128, SortSmemT<2048, 1024>>, 128, sizeof(F32Smem<SortSmemT<2048, 1024>, 128>));
  return nb;
}

}  // namespace ahfgpu
