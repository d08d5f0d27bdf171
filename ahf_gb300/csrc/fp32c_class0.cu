// fp32c_class0.cu -- instantiation of the FP32-compensated halo kernel for
// size class 0 (32 threads per CTA, shared-memory sort SortSmemT<512, 16>).  One
// translation unit per class so the classes compile in parallel.
#include "halo_fp32c.cuh"

namespace ahfgpu {

void launch_fp32c_class0(const DevParams& P, const DevBatch& B, const Work& W, int grid, cudaStream_t st) {
  halo_fp32c_kernel<32, SortSmemT<512, 16>><<<grid, 32, sizeof(F32Smem<SortSmemT<512, 16>, 32>), st>>>(P, B, W);
}

int fp32c_occupancy_class0() {
  int nb = 0;
  cudaFuncSetAttribute(halo_fp32c_kernel<32, SortSmemT<512, 16>>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)sizeof(F32Smem<SortSmemT<512, 16>, 32>));
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, halo_fp32c_kernel<32, SortSmemT<512, 16>>, 32, sizeof(F32Smem<SortSmemT<512, 16>, 32>));
  return nb;
}

}  // namespace ahfgpu
