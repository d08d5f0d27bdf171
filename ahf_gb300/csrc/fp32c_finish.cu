// fp32c_finish.cu -- the FP32-compensated form's post-pass over all haloes:
// profile rows and integral properties from the records the class kernels
// stash (finish.cuh).  Compiled like the class kernels (no FMA contraction:
// the FP64 finishing arithmetic follows the reference's operation order).
#include "halo_fp32c.cuh"

namespace ahfgpu {

// The FP32C post-pass, one thread per halo that ran HaloProfiles: its
// profile rows from the stashed bin records (in place, bin by bin), then the
// integral properties (finish_scalars) into its record -- the FP64 work of
// every halo's tail with full warps, instead of one thread per CTA.
__global__ void fp32c_finish_kernel(DevParams P, DevBatch B, ahfgpu_halo* halo, const uint64_t* prof_cap_off,
                                    double* prof_stage, const double* fin, int64_t nh) {
  for (int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; h < nh; h += (int64_t)gridDim.x * blockDim.x) {
    ahfgpu_halo& H = halo[h];
    if (!(H.flags & AHFGPU_HALO_RAN_PROFILE)) continue;
    const int nb = H.nbins;
    double* rows = prof_stage + prof_cap_off[h] * AHFGPU_PROF_NFIELDS;
    double Mprev = 0.0, eprev = 0.0;
    for (int b = 0; b < nb; b++) {
      Bin R;
      double e;
      double* row = rows + (uint64_t)b * AHFGPU_PROF_NFIELDS;
      load_bin(row, R, e);
      bin_row(R, e, b > 0, Mprev, eprev, row, true);
      Mprev = R.M;
      eprev = e;
    }
    const double* f = fin + (uint64_t)h * kFinStride;
    finish_scalars(rows, nb, f[kFinM], f[kFinVX], f[kFinVY], f[kFinVZ], f[kFinCX], f[kFinCY], f[kFinCZ], f[kFinMhi],
                   f[kFinMlo], __double_as_longlong(f[kFinMbe]), f[kFinR2], f[kFinRmax], f[kFinVmax], P, B, B.cx[h],
                   B.cy[h], B.cz[h], H);
  }
}

void launch_fp32c_finish(const DevParams& P, const DevBatch& B, ahfgpu_halo* halo, const uint64_t* prof_cap_off,
                         double* prof_stage, const double* fin, int64_t nh, int grid, cudaStream_t st) {
  fp32c_finish_kernel<<<grid, 128, 0, st>>>(P, B, halo, prof_cap_off, prof_stage, fin, nh);
}

}  // namespace ahfgpu
