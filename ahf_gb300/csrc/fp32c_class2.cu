// fp32c_class2.cu -- instantiation of the FP32-compensated halo kernel for
// size class 2 (256 threads per CTA, shared-memory sort SortSmemT<2048, 4096>).  One
// translation unit per class so the classes compile in parallel.
#include "halo_fp32c.cuh"

namespace ahfgpu {

void launch_fp32c_class2(const DevParams& P, const DevBatch& B, const Work& W, int grid, cudaStream_t st) {
  halo_fp32c_kernel<256, SortSmemT<2048, 4096>><<<grid, 256, sizeof(F32Smem<SortSmemT<2048, 4096>, 256>), st>>>(P, B, W);
}

int fp32c_occupancy_class2() {
  int nb = 0;
  cudaFuncSetAttribute(halo_fp32c_kernel<256, SortSmemT<2048, 4096>>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)sizeof(F32Smem<SortSmemT<2048, 4096>, 256>));
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, halo_fp32c_kernel<256, SortSmemT<2048, 4096>>, 256, sizeof(F32Smem<SortSmemT<2048, 4096>, 256>));
  return nb;
}

}  // namespace ahfgpu
