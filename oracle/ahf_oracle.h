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

/* The particle gather (src/libahf/ahf_halos_sfc.c:171-412): the list of halo
 * h is every particle i with dist2 <= rad[h]^2, dist2 computed as the
 * reference's LOCAL_CAL_DXYZ (:69-78) and local_checkAndAddParticles
 * (:329-332) do, in ascending particle index.  CSR out: out_off[nhalo+1],
 * *out_idx malloc()ed (free with ahforacle_gather_free).                  */
int  ahforacle_gather(uint64_t n, const float *x, const float *y, const float *z, int64_t nhalo,
                      const double *cx, const double *cy, const double *cz, const double *rad,
                      uint64_t *out_off, uint64_t **out_idx);
void ahforacle_gather_free(uint64_t *idx);

/* The AHF_particles file (WriteParticlesLegacy, src/libahf/ahf_io.c:1095-1175,
 * default build): "%15lu\n" with the number of haloes of at least minpart
 * particles, then per such halo in `order`: "%lu %10ld\n" (npart, its
 * position j in `order`) and per kept particle "%" PRIu64 "\t%d\n" (id,
 * (int)weight with weights, else (int)(-PDM) = 1).  *out malloc()ed.      */
int  ahforacle_write_particles(const uint64_t *ids, const float *w, int64_t nhalo, const uint64_t *member_off,
                               const uint64_t *member, const uint64_t *halo_npart, const int64_t *order,
                               int64_t minpart, unsigned char **out, uint64_t *nbytes);
int  ahforacle_write_particles_bin(const uint64_t *ids, int64_t nhalo, const uint64_t *member_off,
                                   const uint64_t *member, const uint64_t *halo_npart, const int64_t *order,
                                   int64_t minpart, unsigned char **out, uint64_t *nbytes);

/* The gather radii, the loop of spatialRef2halos (src/libahf/ahf_halos.c:
 * 2987-3051): half the distance to the closest halo with strictly more
 * particles (or max_rad without one), raised to rvir, capped at max_rad =
 * min(max_gather_rad_box, 1/4).                                            */
void ahforacle_gather_radii(int64_t nhalo, const uint64_t *npart, const double *cx, const double *cy,
                            const double *cz, const double *rvir, double max_gather_rad_box, double *rad);

/* Hilbert keys (sfc_curve_calcKey, SFC_CURVE_HILBERT) and the particle sort
 * by key (src/main.c:342-356; equal keys by original index).              */
uint64_t ahforacle_sfc_key(double x, double y, double z, unsigned bits);
int  ahforacle_sfc_sort(uint64_t n, const float *x, const float *y, const float *z, unsigned bits, uint64_t *keys,
                        uint64_t *order);

/* The domain grid's TSC number density (assign_npart), l1^3 nodes. */
int  ahforacle_domain_dens(uint64_t n, const float *x, const float *y, const float *z, int l1, double *dens_out);

/* The first refinement of the l1^3 domain grid: its fine nodes (z, y, x). */
int64_t ahforacle_first_refinement(uint64_t n, const float *x, const float *y, const float *z, int l1,
                                   double nth_dom, int64_t *zyx, int64_t max_nodes);

/* The AMR hierarchy (oracle_amr.c): per grid (l1, nodes, particles). */
int  ahforacle_amr_levels(uint64_t n, const float *x, const float *y, const float *z, int ngrid_dom,
                          int ngrid_max, double nth_dom, double nth_ref, int64_t *levels, int max_levels);
int64_t ahforacle_amr_list_order_violations(uint64_t n, const float *x, const float *y, const float *z,
                                            int ngrid_dom, int ngrid_max, double nth_dom, double nth_ref);
int64_t ahforacle_amr_gather_mismatches(uint64_t n, const float *x, const float *y, const float *z, int ngrid_dom,
                                        int ngrid_max, double nth_dom, double nth_ref);
int64_t ahforacle_amr_nodes(uint64_t n, const float *x, const float *y, const float *z, int ngrid_dom,
                            int ngrid_max, double nth_dom, double nth_ref, int level, int64_t *zyx, double *dens,
                            int64_t max_nodes);

#ifdef __cplusplus
}
#endif
#endif
