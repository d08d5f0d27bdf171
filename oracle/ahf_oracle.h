/*
 * ahf_oracle.h -- CPU restatement of AHF's unbinding + halo-property stage.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker the GPU library is compared
 * against (and the timed CPU baseline when the reference itself cannot be
 * built).  Nothing in the product links or calls it.
 *
 * It takes the same ahfgpu_params / ahfgpu_batch as include/ahfgpu.h and
 * fills an ahfgpu_result with malloc()ed arrays, processing each halo
 * sequentially in the reference's exact operation order (FP64, no fused
 * multiply-add).  See ahf_oracle.c for the per-function citations.
 */
#ifndef AHF_ORACLE_H
#define AHF_ORACLE_H

#include "../include/ahfgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* nthreads <= 0: all OpenMP threads (halos in dynamic order, as the
 * reference's own loop at src/libahf/ahf_halos.c:504-506).                 */
int  ahforacle_construct_halos(const ahfgpu_params *params,
                               const ahfgpu_batch *batch,
                               ahfgpu_result *result, int nthreads);
void ahforacle_result_free(ahfgpu_result *result);
int  ahforacle_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
