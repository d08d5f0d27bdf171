/*
 * ahfgpu.h -- C ABI of the GB300 unbinding + halo-property stage of AHF.
 *
 * The stage replaced is the per-halo sequence that AHF runs after gathering
 * a halo's particles (src/libahf/ahf_halos_sfc.c:140-156):
 *
 *     sort_halo_particles(halo);      src/libahf/ahf_halos.c:5786-5894
 *     rem_outsideRvir(halo, 0);       src/libahf/ahf_halos.c:3687-3889
 *     rem_unbound(halo);              src/libahf/ahf_halos.c:3292-3607
 *     rem_outsideRvir(halo, 1);
 *     HaloProfiles(halo);             src/libahf/ahf_halos.c:3961-5261
 *
 * In AHF that sequence runs once per halo inside the OpenMP loop at
 * src/libahf/ahf_halos.c:504-510 (one call of
 * ahf_halos_sfc_constructHalo(HALO*), declared in
 * src/libahf/ahf_halos_sfc.h:15-16).  Here the caller gathers every halo on
 * the host, packs the lists into one CSR batch and makes ONE call; the
 * library returns, per halo, the fields that the five functions above write
 * into HALO, the profile arrays that c_profile() would hold, and the kept
 * particle list in radial order.
 *
 * Conventions: all pointers are plain host pointers unless the function name
 * ends in _device; sizes are 64-bit; nothing here uses C++ or CUDA types.
 * Every function returns AHFGPU_OK (0) or a negative AHFGPU_ERR_* code and
 * never calls exit(); ahfgpu_last_error() gives the message of the last
 * failure on the calling thread.
 */
#ifndef AHFGPU_H
#define AHFGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AHFGPU_ABI_VERSION 1

#if defined(__GNUC__)
#define AHFGPU_API __attribute__((visibility("default")))
#else
#define AHFGPU_API
#endif

/* ---- status codes ------------------------------------------------------ */
#define AHFGPU_OK              0
#define AHFGPU_ERR_INVALID    -1   /* malformed batch or parameters          */
#define AHFGPU_ERR_OOM        -2   /* host or device allocation failed       */
#define AHFGPU_ERR_CUDA       -3   /* a CUDA runtime call failed             */
#define AHFGPU_ERR_TIMEOUT    -4   /* a bounded device wait ran out          */
#define AHFGPU_ERR_NO_DEVICE  -5   /* no usable sm_103 device                */
#define AHFGPU_ERR_CAPACITY   -6   /* a size exceeds a documented maximum    */
#define AHFGPU_ERR_STATE      -7   /* call sequence error (e.g. no init)     */

/* ---- execution forms --------------------------------------------------- */
typedef enum {
  /* Halos one at a time, in batch order, FP64 arithmetic; bound sets are
   * bit-exact with the reference (exact sequential replay on device for any
   * halo with a particle inside the rounding band). */
  AHFGPU_PLAIN_FP64    = 0,
  /* Every halo of the batch in one persistent launch (size-sorted work
   * queue), FP64 arithmetic, same exactness rule as the plain form. */
  AHFGPU_BATCHED_FP64  = 1,
  /* Batched, FP32 positions/velocities/keys with compensated (two-sum) FP32
   * scans, FP64 edge normalisation and an FP64 re-test of near-threshold
   * particles; membership equals the FP64 reference. */
  AHFGPU_BATCHED_FP32C = 2
} ahfgpu_mode;

/* ---- parameters (AHF.input keys and the ahf_halos() unit factors) -------
 * Fill exactly as src/libahf/ahf_halos.c:199-221 computes them:
 *   r_fac = simu.boxsize*global.a;       x_fac = simu.boxsize;
 *   v_fac = simu.boxsize/simu.t_unit/global.a;  m_fac = simu.pmass;
 *   rho_fac = simu.pmass/pow3(simu.boxsize);
 *   phi_fac = Grav*simu.pmass/(simu.boxsize*global.a);
 *   Hubble = calc_Hubble(a); ovlim = global.ovlim; rho_vir = global.rho_vir.
 * VescTune = simu.AHF_VTUNE (AHF.input VescTune), MINPART =
 * simu.AHF_MINPART (AHF.input NminPerHalo, >= 4).                           */
typedef struct {
  double  VescTune;
  int64_t MINPART;
  double  ovlim;
  double  rho_vir;
  double  r_fac, x_fac, v_fac, m_fac, rho_fac, phi_fac, Hubble;
} ahfgpu_params;

/* ---- input batch ---------------------------------------------------------
 * Halo h owns entries [off[h], off[h+1]) of the particle arrays, in the
 * order ahf_halos_sfc_gatherParts() produced them.  Positions are box units
 * in [0,1), velocities are AHF internal momenta (struct particle .pos/.mom,
 * src/tdef.h:36-77).  w is the MULTIMASS weight (NULL = all 1.0, the default
 * build).  gidx is the particle's index in global.fst_part and is what the
 * kept list returns (NULL = return the entry index inside the batch); the
 * particle ids stay with the caller, who maps the returned indices to them
 * (AHF writes fst_part[ipart].id).  cx/cy/cz are HALO.pos.                 */
typedef struct {
  int64_t         nhalo;
  const uint64_t *off;                    /* [nhalo+1], off[0] == 0        */
  const float    *x, *y, *z;              /* [off[nhalo]]                  */
  const float    *vx, *vy, *vz;           /* [off[nhalo]]                  */
  const float    *w;                      /* [off[nhalo]] or NULL          */
  const uint64_t *gidx;                   /* [off[nhalo]] or NULL          */
  const double   *cx, *cy, *cz;           /* [nhalo]                       */
} ahfgpu_batch;

/* ---- per-halo result ---------------------------------------------------- */
#define AHFGPU_HALO_EMPTY        0x001u  /* n == 0: nothing ran (ahf_halos_sfc.c:122)   */
#define AHFGPU_HALO_RAN_SORT     0x002u  /* sort_halo_particles ran                     */
#define AHFGPU_HALO_RAN_RVIR0    0x004u  /* rem_outsideRvir(.,0) ran                    */
#define AHFGPU_HALO_RAN_UNBIND   0x008u  /* rem_unbound ran                             */
#define AHFGPU_HALO_RAN_RVIR1    0x010u  /* rem_outsideRvir(.,1) ran                    */
#define AHFGPU_HALO_RAN_PROFILE  0x020u  /* HaloProfiles ran                            */
#define AHFGPU_HALO_NO_MBP       0x040u  /* no most-bound particle (mbp_offset = -1)    */
#define AHFGPU_HALO_REPLAYED     0x100u  /* exact sequential replay was used            */
#define AHFGPU_HALO_NOBOUND      0x200u  /* an unbinding pass kept no particle          */

typedef struct {
  uint64_t npart;          /* HALO.npart after the stage                       */
  int32_t  nbins;          /* HALO.prof.nbins, 0 when HaloProfiles did not run */
  uint32_t flags;          /* AHFGPU_HALO_* bits                               */
  int32_t  niter;          /* rem_unbound iterations (0 if it did not run)     */
  int32_t  fix_rounds;     /* max bulk-velocity fixpoint rounds (diagnostic)   */
  double   M_vir, R_vir, ovdens, Phi0;
  double   vel[3];
  double   sigV, v_esc2, V2_max, R_max, r2;
  double   lambda, lambdaE, Ekin, Epot, SurfP;
  double   pos_com[3], com_offset;
  double   pos_mbp[3], vel_mbp[3], mbp_offset;
  double   AngMom[3], axis[3], E1[3], E2[3], E3[3];
  double   fMhires, cNFW, R1, cR1;
} ahfgpu_halo;

/* Profile arrays, one row of AHFGPU_PROF_NFIELDS doubles per bin, fields in
 * the order of HALOPROFILE (src/tdef.h:591-688).                            */
enum {
  AHFGPU_PROF_R = 0, AHFGPU_PROF_NPART, AHFGPU_PROF_NVPART, AHFGPU_PROF_OVDENS,
  AHFGPU_PROF_DENS, AHFGPU_PROF_V2_CIRC, AHFGPU_PROF_V_ESC2, AHFGPU_PROF_SIG_V,
  AHFGPU_PROF_EKIN, AHFGPU_PROF_EPOT, AHFGPU_PROF_LX, AHFGPU_PROF_LY,
  AHFGPU_PROF_LZ, AHFGPU_PROF_AXIS1, AHFGPU_PROF_E1X, AHFGPU_PROF_E1Y,
  AHFGPU_PROF_E1Z, AHFGPU_PROF_AXIS2, AHFGPU_PROF_E2X, AHFGPU_PROF_E2Y,
  AHFGPU_PROF_E2Z, AHFGPU_PROF_AXIS3, AHFGPU_PROF_E3X, AHFGPU_PROF_E3Y,
  AHFGPU_PROF_E3Z, AHFGPU_PROF_NFIELDS
};

typedef struct {
  uint64_t n_particles_in;   /* off[nhalo]                                    */
  uint64_t n_kept;           /* member_off[nhalo]                             */
  uint64_t n_retest;         /* particles routed to the FP64 re-test          */
  uint64_t n_replay_halos;   /* halos finished by the exact sequential replay */
  uint64_t n_key_ties;       /* equal radial keys met by the sort             */
  uint64_t n_fp64_halos;     /* FP32C: haloes with an unbinding iteration
                                replayed whole in the reference's FP64 order */
  uint64_t n_launches;       /* kernels launched by the call                  */
  double   ms_device;        /* device time of the compute kernels (ms)       */
  double   ms_total;         /* wall time of the whole call (ms)              */
  double   ms_plan;          /* host: checks, halo queue and size classes     */
  double   ms_h2d;           /* host calls: input copies, first to last byte  */
  double   ms_h2d_first;     /* host calls: until the largest lists are in    */
  double   ms_pack;          /* device: result packing after the compute      */
  double   ms_d2h;           /* host calls: result copies to the host         */
} ahfgpu_stats;

/* Library-owned result; release with ahfgpu_result_free().                  */
typedef struct {
  int64_t      nhalo;
  ahfgpu_halo *halo;         /* [nhalo]                                        */
  uint64_t    *member_off;   /* [nhalo+1]                                      */
  uint64_t    *member;       /* kept gidx (or entry index), radial order       */
  uint64_t    *prof_off;     /* [nhalo+1], in bins                             */
  double      *prof;         /* [prof_off[nhalo]][AHFGPU_PROF_NFIELDS]         */
  ahfgpu_stats stats;
  void        *priv;         /* library bookkeeping, do not touch              */
} ahfgpu_result;

/* ---- entry points -------------------------------------------------------- */

/* Select and initialise a CUDA device (AHF's startrun-time set-up).  Safe to
 * call more than once; a later call with another device re-initialises.     */
AHFGPU_API int ahfgpu_init(int device);

/* Release every device and host resource the library holds.                 */
AHFGPU_API int ahfgpu_shutdown(void);

/* Replaces the per-halo loop body of src/libahf/ahf_halos.c:504-510
 * (ahf_halos_sfc_constructHalo, src/libahf/ahf_halos_sfc.c:118-169, minus its
 * gather at :137).  Host batch in, host result out (copies are inside).     */
AHFGPU_API int ahfgpu_construct_halos(const ahfgpu_params *params,
                           const ahfgpu_batch  *batch,
                           ahfgpu_result       *result,
                           ahfgpu_mode          mode);

/* ---- the particle gather (the stage's input) ------------------------------ */

/* A snapshot's particles in device memory: positions in box units [0,1)
 * (float), momenta (float), weights (float, NULL = 1).  n < 2^32.          */
typedef struct {
  uint64_t     n;
  const float *x, *y, *z, *vx, *vy, *vz, *w;
} ahfgpu_particles;

/* Halo centres (box units) and gather radii (HALO.gatherRad), device memory */
typedef struct {
  int64_t       nhalo;
  const double *cx, *cy, *cz, *rad;
} ahfgpu_centres;

/* Replaces ahf_halos_sfc_gatherParts (src/libahf/ahf_halos_sfc.c:171-412) for
 * every halo at once: the list of halo h is every particle i whose periodic
 * squared distance from the centre, computed as the reference computes it
 * (LOCAL_CAL_DXYZ :69-78 on the float position promoted to double, compared
 * by islessequal with gatherRad^2, :329-332), is within the radius; each
 * list in ascending particle index (the reference lists its SFC cells in
 * turn).  `gathered` is filled with device pointers to library-owned
 * buffers (valid until the next gather or ahfgpu_shutdown) in the layout
 * ahfgpu_construct_halos_device takes: off, the particles' x..vz (w when
 * given), gidx = particle index, and the caller's centres.                 */
AHFGPU_API int ahfgpu_gather_device(const ahfgpu_particles *parts,
                                    const ahfgpu_centres   *centres,
                                    ahfgpu_batch           *gathered,
                                    void                   *stream);

/* Replaces the keying loop and the particle sort of src/main.c:342-356
 * (sfc_curve_calcKey(SFC_CURVE_HILBERT, pos, BITS_PER_DIMENSION) for every
 * particle, then qsort by cmp_sfckey_part, src/libutility/specific.c:1117):
 * keys[k] the k-th smallest Hilbert key at `bits` levels (1..21; AHF uses
 * 21), order[k] the input index of that particle; equal keys keep their
 * input order.  Device pointers; positions in [0, 1]; n < 2^31.           */
AHFGPU_API int ahfgpu_sfc_sort_device(uint64_t n, const float *x, const float *y, const float *z, int bits,
                                      uint64_t *keys, uint64_t *order, void *stream);

/* Replaces the gather-radius loop of spatialRef2halos
 * (src/libahf/ahf_halos.c:2987-3051): for each halo, half the periodic
 * distance (double, the reference's operation order) to the closest halo
 * with strictly more particles, or max_rad without one; then raised to
 * rvir[h] (the halo's R_vir at that stage) and capped at max_rad, where
 * max_rad = min(MaxGatherRad / boxsize, 1/4) (:2987).  Device pointers:
 * npart[nhalo], centres, rvir in; rad[nhalo] out.                          */
AHFGPU_API int ahfgpu_gather_radii_device(int64_t nhalo, const uint64_t *npart,
                                          const double *cx, const double *cy, const double *cz,
                                          const double *rvir, double max_gather_rad_box,
                                          double *rad, void *stream);

/* Replaces WriteParticlesLegacy (src/libahf/ahf_io.c:1095-1175, default
 * build; the AHF_particles file) for the last device-resident result: the
 * file's exact bytes in a library-owned device buffer (*out, *nbytes; valid
 * until the next call or ahfgpu_shutdown).  The kept entries of the result
 * index ids[] (and w[], NULL without weights) -- the particle index when the
 * batch's gidx held HALO.ipart; order[nhalo] (device) is the reference's idx
 * (the output order); haloes below minpart are left out as the reference
 * does.                                                                    */
AHFGPU_API int ahfgpu_write_particles_device(const uint64_t *ids, const float *w, const int64_t *order,
                                             int64_t minpart, const unsigned char **out, uint64_t *nbytes,
                                             void *stream);

/* Replaces ahf_binwrite_particles (src/libahf/ahf_io.c:1733-1855, the
 * AHFbinary build; the AHF_particles_bin file) for the last device-resident
 * result, arguments as ahfgpu_write_particles_device (the binary file has no
 * weight column: every particle's type is 1).  Bytes: int32 1, uint64
 * haloes written, uint32 2; per halo uint64 npart, uint64 j, then per kept
 * particle uint64 id, int32 1 -- native byte order, no padding.  The text
 * companion <prefix>.AHF_particles_info (ahf_io.c:1766-1774, constant) stays
 * with the caller.                                                          */
AHFGPU_API int ahfgpu_write_particles_bin_device(const uint64_t *ids, const int64_t *order, int64_t minpart,
                                                 const unsigned char **out, uint64_t *nbytes, void *stream);

/* Same stage with every pointer of `batch` already in device memory; the
 * results stay on the device in library-owned buffers (valid until the next
 * call or ahfgpu_shutdown) and are described by `dres` (device pointers,
 * member_off/prof_off included).  `stream` is a cudaStream_t or NULL for the
 * library's own stream.  Used when the caller keeps a snapshot resident.    */
AHFGPU_API int ahfgpu_construct_halos_device(const ahfgpu_params *params,
                                  const ahfgpu_batch  *batch,
                                  ahfgpu_result       *dres,
                                  ahfgpu_mode          mode,
                                  void                *stream);

/* Copy the device-resident result of the last _device call into a host
 * result (library-owned host arrays; free with ahfgpu_result_free).          */
AHFGPU_API int ahfgpu_fetch_result(ahfgpu_result *result);

AHFGPU_API void ahfgpu_result_free(ahfgpu_result *result);

/* Message of the last failure on this thread (empty when none); returns the
 * untruncated length.                                                       */
AHFGPU_API int ahfgpu_last_error(char *buf, size_t len);

AHFGPU_API const char *ahfgpu_version(void);

/* The FP32C size-class tuning in effect on the initialised device, as JSON:
 * {"key": "<name>|<SMs>|<cc>", "source": <cache path|"default"|"environment">,
 *  "class_max": [a, b], "class_bps": [c0, c1, c2]}.  Tuning comes from the
 * per-GPU cache written by `python -m ahf_gb300.autotune` (tune_cache.json
 * beside the library, or AHFGPU_TUNE_CACHE).  Returns AHFGPU_OK.           */
AHFGPU_API int ahfgpu_tuning(char *buf, size_t len);

/* ---- the AMR hierarchy, first levels ---------------------------------------
 * Replaces, for the domain grid, gen_domgrids + ll + assign_npart
 * (src/libamr_serial/generate_grids.c:24, lltools.c, density.c:238; default
 * TSC build, periodic): dens[(z*l1 + y)*l1 + x] (device, float, l1^3) is the
 * node's TSC number density minus the mean, the float the reference's
 * assign_npart leaves there bit for bit (each node's sum in its visiting
 * order: source nodes ascending, each node's particles by descending input
 * index).  Positions in [0, 1] (device floats; a coordinate of exactly 1.0
 * falls in node 0 as ll() folds it); 3 <= l1 <= 1024; n < 2^31.            */
AHFGPU_API int ahfgpu_amr_domain_density_device(uint64_t n, const float *x, const float *y, const float *z,
                                                int l1, float *dens, void *stream);

/* Replaces the first refine_grid call on the domain grid (gen_refgrid ->
 * refine_grid, src/libamr_serial/generate_grids.c:126, refine_grid.c:899):
 * the fine grid's nodes, 2 per dimension inside each coarse node that
 * test_node (refine_grid.c:113-137) flags -- a node any of whose 18 nodes at
 * dz, dy in {-1,0,1}, dx in {0,1} has dens >= NperDomCell l1^3 / n - 1 --
 * or that follows a flagged node along x (wrapping at x = 0, not at
 * x = l1 - 1).  zyx[3k .. 3k+2] (device int32) = (z, y, x) of fine node k on
 * the 2 l1 grid, ascending; *nnodes their number, 0 when below MIN_NNODES
 * (125, no fine grid).  A buffer of fewer than *nnodes nodes returns
 * AHFGPU_ERR_CAPACITY with *nnodes set.  dens as returned by
 * ahfgpu_amr_domain_density_device for the same n particles.               */
AHFGPU_API int ahfgpu_amr_first_refinement_device(int l1, const float *dens, uint64_t n, double nth_dom,
                                                  int32_t *zyx, int64_t max_nodes, int64_t *nnodes,
                                                  void *stream);

/* ---- the AMR hierarchy, every level ---------------------------------------
 * Replaces the grid generation of src/main.c:614-648 (gen_domgrids + ll +
 * assign_npart on the ngrid_dom^3 domain grid, then gen_AMRhierarchy,
 * src/libamr_serial/generate_grids.c:278: refine_grid, relink, assign_npart
 * per level; default TSC build, periodic, no NP_LIMIT, non-MULTIMASS).
 * While the finest grid has fewer than ngrid_max nodes per dimension it is
 * refined with threshold critdens - mean_dens (critdens = nth_dom m2d on the
 * domain grid, nth_ref m2d below, i.e. NperDomCell and NperRefCell; m2d =
 * ngrid_dom^3 / n, times 8 per level); a refined grid of fewer than
 * MIN_NNODES = 125 nodes is dropped and ends the hierarchy.  Every grid keeps
 * the reference's run structure, node order, particle lists and float
 * densities bit for bit.  levels[3g .. 3g+2] (host, max_levels entries) =
 * nodes per dimension, nodes, particles in the lists of grid g; *ngrids the
 * number of grids.  The grids stay in the library (until the next call or
 * ahfgpu_shutdown) for ahfgpu_amr_grid_device.  Positions in [0, 1]
 * (device floats); 3 <= ngrid_dom <= 1024; ngrid_dom <= ngrid_max <= 2^20;
 * n < 2^31.                                                                */
AHFGPU_API int ahfgpu_amr_hierarchy_device(uint64_t n, const float *x, const float *y, const float *z,
                                           int ngrid_dom, int ngrid_max, double nth_dom, double nth_ref,
                                           int64_t *levels, int max_levels, int *ngrids, void *stream);

/* Grid `level` of the last ahfgpu_amr_hierarchy_device call: *nnodes its
 * node count; with max_nodes > 0, zyx[3k .. 3k+2] (device int32, may be
 * NULL) = (z, y, x) of node k in the reference's node order (ascending) and
 * dens[k] (device float, may be NULL) its density.  max_nodes = 0 only
 * reports *nnodes; fewer than *nnodes returns AHFGPU_ERR_CAPACITY.          */
AHFGPU_API int ahfgpu_amr_grid_device(int level, int32_t *zyx, float *dens, int64_t max_nodes, int64_t *nnodes,
                                      void *stream);

/* ---- the split across GPUs ------------------------------------------------
 * Replaces nothing in one process: AHF's haloes are independent
 * (src/libahf/ahf_halos.c:504-510 runs them in any order), so a caller with
 * several GPUs splits one snapshot's batch by halo and makes one
 * ahfgpu_construct_halos call per GPU on its share -- no data exchange.
 * rank_of_halo[h] (out, [nhalo]) is the rank of halo h: longest processing
 * time first on the cost n log2(n + 2), n = off[h+1] - off[h], haloes by
 * decreasing cost (ties: lower index), each to the least-loaded rank so far
 * (ties: lower rank).  Host pointers; needs no device.                    */
AHFGPU_API int ahfgpu_shard_halos(int64_t nhalo, const uint64_t *off, int32_t nranks,
                                  int32_t *rank_of_halo);

/* ---- no-allocation variant ----------------------------------------------
 * No counterpart in the reference (AHF has no GPU path).  For callers that
 * cannot allocate device memory: an application that gives AHF's analysis a
 * fixed device budget and partitions the GPU's memory itself, or a plugin
 * inside a running simulation that may not call cudaMalloc/cudaFree.  The
 * batched FP64 stage with every byte of work space taken from one static
 * device array of about 16 MB that each GPU loading the library holds until
 * exit.  All pointers are device pointers; the batch is as for
 * ahfgpu_construct_halos_device; nothing is allocated.
 * Outputs (caller-owned): out_halo[nhalo]; halo h's kept list in radial order
 * at out_member[off[h] .. off[h] + out_halo[h].npart) (out_member has
 * off[nhalo] entries); profile rows of halo h at
 * out_prof[(h * AHFGPU_NOALLOC_MAX_BINS + b) * AHFGPU_PROF_NFIELDS + f].
 * Larger batches return AHFGPU_ERR_CAPACITY.  The first call on a device
 * sets the array up (cudaGetSymbolAddress, with that device current) and
 * should come before any stream capture.  Each call waits for `stream` (it
 * reads the entry count, the batch checks and the error word back).  Calls
 * that overlap on the GPU share the array and race: serialise them.
 * stream: cudaStream_t or NULL. */
#define AHFGPU_NOALLOC_MAX_PARTICLES 131072
#define AHFGPU_NOALLOC_MAX_HALOS     8192
#define AHFGPU_NOALLOC_MAX_BINS      64
AHFGPU_API int ahfgpu_construct_halos_noalloc(const ahfgpu_params *params,
                                              const ahfgpu_batch  *batch,
                                              ahfgpu_halo         *out_halo,
                                              uint64_t            *out_member,
                                              double              *out_prof,
                                              void                *stream);
/* Message of the last failure of ahfgpu_construct_halos_noalloc on this
 * thread; returns the untruncated length. */
AHFGPU_API int ahfgpu_noalloc_last_error(char *buf, size_t len);

#ifdef __cplusplus
}
#endif
#endif /* AHFGPU_H */
