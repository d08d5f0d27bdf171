// api.cu -- the extern "C" boundary (include/ahfgpu.h) of the GB300
// unbinding + halo-property stage: device set-up, batch validation and
// planning, work-space management, kernel launches, result packing and the
// copies to and from the host.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <new>
#include <stdexcept>
#include <numeric>
#include <string>
#include <vector>

#include <cuda_runtime.h>
#include <dlfcn.h>

#include "common.cuh"
#include "amr_tree.cuh"

namespace ahfgpu {
size_t fp64_smem_bytes();
void launch_fp64(const DevParams& P, const DevBatch& B, const Work& W, int grid, int single, cudaStream_t st);
int fp64_max_blocks_per_sm();
void launch_fp32c(int cls, const DevParams& P, const DevBatch& B, const Work& W, int grid, cudaStream_t st);
int fp32c_max_blocks_per_sm(int cls);
// the small lists of the FP32C form, one per thread (fp32c_small.cu)
void launch_fp32c_small(const DevParams& P, const DevBatch& B, const Work& W, unsigned char* scratch, uint32_t nmax,
                        int grid, cudaStream_t st);
size_t fp32c_small_bytes_per_warp(uint64_t nmax);
int fp32c_small_occupancy();
uint64_t fp32c_class_max(int cls);
void fp32c_set_class_max(uint64_t a, uint64_t b, uint64_t cap0);
void launch_concentration(ahfgpu_halo* halo, int64_t nh, int grid, cudaStream_t st);
void launch_fp32c_finish(const DevParams& P, const DevBatch& B, ahfgpu_halo* halo, const uint64_t* prof_cap_off,
                         double* prof_stage, const double* fin, int64_t nh, int grid, cudaStream_t st);
// the particle gather (gather.cu)
void gather_cells(uint64_t n, const float* x, const float* y, const float* z, int G, uint32_t* cell,
                  uint32_t* count, int grid, cudaStream_t st);
void gather_scan_u32(const uint32_t* in, uint32_t* out, uint64_t m, uint32_t* sums, cudaStream_t st);
void gather_scatter(uint64_t n, const float* x, const float* y, const float* z, const uint32_t* cell,
                    const uint32_t* start, uint32_t* fill, float4* sorted, int grid, cudaStream_t st);
void gather_halos(int pass, int G, const uint32_t* start, const float4* sorted, int64_t nhalo, const int32_t* queue,
                  unsigned int* qhead, const double* cx, const double* cy, const double* cz, const double* rad,
                  uint64_t* cnt, const uint64_t* off, unsigned long long* hfill, uint64_t* out_idx, int grid,
                  cudaStream_t st);
void gather_offsets(const uint64_t* cnt, int64_t nhalo, uint64_t* off, cudaStream_t st);
int gather_sort_setup();
int gather_window_shift_max();
size_t gather_item_bytes();
void gather_order_pack(int64_t nhalo, const int32_t* queue, unsigned int* qhead, const uint64_t* off, uint64_t* keyA,
                       uint32_t* idxA, uint64_t* keyB, uint32_t* idxB, uint4* stack, int stack_cap, int wshift,
                       int mode, void* items, uint64_t icap, int32_t* fbq, unsigned int* fbn, uint64_t ng,
                       const float* x, const float* y, const float* z, const float* vx, const float* vy,
                       const float* vz, const float* w, float* ox, float* oy, float* oz, float* ovx, float* ovy,
                       float* ovz, float* ow, uint64_t* oid, int* err, int grid, int grid_p, cudaStream_t st);
void gather_radii(int64_t nh, const double* px, const double* py, const double* pz, const int64_t* lim,
                  const double* rv, const int32_t* orig, double maxr, double* out, cudaStream_t st);
uint32_t sfc_ntiles(uint32_t n);
uint32_t sfc_scan_blocks(uint32_t m);
void sfc_keys(uint32_t n, const float* x, const float* y, const float* z, int bits, uint64_t* keys, uint32_t* idx,
              int grid, cudaStream_t st);
void sfc_pass(uint32_t n, const uint64_t* kin, const uint32_t* iin, int shift, uint32_t* gh, uint32_t* goff,
              uint32_t* part, uint64_t* kout, uint32_t* iout, int* err, cudaStream_t st);
void sfc_order(uint32_t n, const uint32_t* idx, uint64_t* order, int grid, cudaStream_t st);
// the AMR hierarchy's first levels (amr.cu)
void amr_cells(uint32_t n, const float* x, const float* y, const float* z, int l1, uint64_t* key, uint32_t* idx,
               uint32_t* count, int grid, cudaStream_t st);
void amr_dens(int l1, uint64_t n, const float* x, const float* y, const float* z, const uint32_t* start,
              const uint64_t* skey, const uint32_t* ord, double* wts, double* cfold, float* dens, int grid,
              cudaStream_t st);
void amr_flags(int l1, const float* dens, double thr, uint8_t* flag, uint32_t* rowcnt, cudaStream_t st);
void amr_emit(int l1, const uint8_t* flag, const uint32_t* rowcnt, const uint32_t* rowoff, int64_t cap, int32_t* zyx,
              int* err, cudaStream_t st);
void writer_sizes(int64_t nh, const int64_t* order, const ahfgpu_halo* halo, int64_t minpart, uint64_t* blk,
                  uint64_t* nchunk, unsigned long long* good, int grid, cudaStream_t st);
void writer_offsets(const uint64_t* blk, int64_t nh, uint64_t* boff, cudaStream_t st);
void writer_count(int64_t nh, const int64_t* order, const ahfgpu_halo* halo, const uint64_t* moff,
                  const uint64_t* member, const uint64_t* ids, const float* w, const uint64_t* coff,
                  unsigned int* qhead, uint64_t* cbytes, int grid, cudaStream_t st);
void writer_write(int64_t nh, const int64_t* order, const ahfgpu_halo* halo, const uint64_t* moff,
                  const uint64_t* member, const uint64_t* ids, const float* w, const uint64_t* coff,
                  unsigned int* qhead, const uint64_t* cboff, const unsigned long long* good, unsigned char* out,
                  int grid, cudaStream_t st);
void writer_bin_write(int64_t nh, const int64_t* order, const ahfgpu_halo* halo, const uint64_t* moff,
                      const uint64_t* member, const uint64_t* ids, const uint64_t* boff, const uint64_t* coff,
                      const unsigned long long* good, unsigned int* qhead, uint32_t* out, int grid, cudaStream_t st);
}  // namespace ahfgpu

using namespace ahfgpu;

namespace {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

// Host-side fault injection for tests: AHFGPU_INJECT_OOM names one
// allocation site whose next allocation fails as a real one would --
// "device_work" (a cudaMalloc of the work space), "host_result" (the result's
// page-locked block and its malloc fallback), "host_plan" (a host container
// of the call's plan: std::bad_alloc).  Unset in normal use.
static bool inject_oom(const char* site) {
  const char* e = getenv("AHFGPU_INJECT_OOM");
  return e && strcmp(e, site) == 0;
}

// Every exported call runs inside this guard: a C++ exception (a failed host
// allocation in a std::vector, for one) must not cross the C ABI.
template <class F>
static int guarded(F&& f) {
  try {
    return f();
  } catch (const std::bad_alloc&) {
    return fail(AHFGPU_ERR_OOM, "host allocation failed (std::bad_alloc)");
  } catch (const std::exception& ex) {
    return fail(AHFGPU_ERR_STATE, "unexpected C++ exception: %s", ex.what());
  } catch (...) {
    return fail(AHFGPU_ERR_STATE, "unexpected C++ exception");
  }
}

#define CK(call)                                                                         \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess)                                                               \
      return fail(e_ == cudaErrorMemoryAllocation ? AHFGPU_ERR_OOM : AHFGPU_ERR_CUDA,    \
                  "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
  } while (0)

// growable device buffer
struct DBuf {
  void* p = nullptr;
  size_t cap = 0;
  int ensure(size_t bytes) {
    if (bytes <= cap) return AHFGPU_OK;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    size_t want = std::max<size_t>(bytes + bytes / 8, 256);
    cudaError_t e = inject_oom("device_work") ? cudaErrorMemoryAllocation : cudaMalloc(&p, want);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return fail(AHFGPU_ERR_OOM, "cudaMalloc(%zu) failed: %s", want, cudaGetErrorString(e));
    }
    cap = want;
    return AHFGPU_OK;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
  template <class T> T* as() const { return reinterpret_cast<T*>(p); }
};

constexpr int kMaxParts = 16;  // queue parts of a staged host call
// queue heads: [0] the FP64 forms, [2 + s] FP32C launch segment s
constexpr int kQueueHeads = 2 + 3 * kMaxParts;

struct Ctx {
  bool init = false;
  int device = -1;
  int nsm = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev2 = nullptr, ev_cp0 = nullptr;
  int fp64_bps = 1, fp32c_bps[3] = {1, 1, 1};
  // FP32C size-class tuning of this device (defaults, the per-GPU tuning
  // cache written by ahf_gb300.autotune, then environment overrides)
  std::string tune_key, tune_source = "default";
  // device-resident calls: the launch sequence as a CUDA graph, re-launched
  // while the launches (kernels, grids, arguments) stay the same
  bool use_graph = true;
  bool small_on = true;        // FP32C class 0 by the one-list-per-thread kernel
  int small_bps = 1;           // its blocks (128 threads) per SM
  DBuf small_scr;              // its work space
  cudaGraphExec_t graph_exec = nullptr;
  std::vector<unsigned char> graph_sig;
  uint64_t graph_launches = 0, graph_replays = 0;
  uint64_t tune_class_max[2] = {512, 16384};
  int tune_bps_cap[3] = {0, 0, 0};
  // FP32C launches: one stream per (queue part, size class); the host path
  // copies the inputs part by part, the largest lists first
  cudaStream_t seg_stream[kMaxParts][3] = {};
  cudaEvent_t ev_fork = nullptr, ev_join[kMaxParts][3] = {};
  cudaStream_t copy_stream = nullptr;       // host-to-device input copies
  cudaEvent_t ev_part[kMaxParts] = {};      // inputs of queue part p are in
  cudaEvent_t ev_ids = nullptr;             // the ids (gidx) are in
  // inputs copied from the host (host API)
  DBuf in_off, in_x, in_y, in_z, in_vx, in_vy, in_vz, in_w, in_gidx, in_cx, in_cy, in_cz;
  // work space
  DBuf keyA, keyB, idxA, idxB, sdx, sdy, sdz, sd, svx, svy, svz, sw, seid, phi, flag, nflag;
  DBuf fdh, fdl, fdx, fdy, fdz, fdxl, fdyl, fdzl, fqh, fql, rec;
  DBuf pa, pb, pc, pd, stack, halo, mem_stage, prof_stage, prof_cap_off, queue, qhead, counters, err, wred, fin;
  // packed results (device)
  DBuf member_off, member, prof_off, prof, phase;
  // the particle gather: grid buckets, per-halo counts and lists, the
  // gathered batch
  DBuf ga_cell, ga_count, ga_start, ga_fill, ga_sums, ga_sorted, ga_queue, ga_qhead, ga_cnt, ga_off, ga_hfill;
  DBuf ga_idx, ga_idxA, ga_keyB, ga_idxB, ga_stack, ga_err, ga_x, ga_y, ga_z, ga_vx, ga_vy, ga_vz, ga_w, ga_id,
       ga_fbq, ga_fbn, ga_items;
  DBuf gr_pos, gr_lim, gr_orig;   // gather radii: sorted centres and R_vir, candidate counts, order
  DBuf wp_blk, wp_boff, wp_good, wp_qhead, wp_out;   // the AHF_particles bytes
  DBuf wb_chunk, wb_coff;                            // both writers: chunks per block, their scan
  DBuf wp_cbytes, wp_cboff;                          // ASCII: bytes per chunk, their scan
  DBuf sfc_kb, sfc_ia, sfc_ib, sfc_gh, sfc_goff, sfc_part, sfc_err;   // the SFC key sort
  DBuf am_key, am_keyb, am_idx, am_idxb, am_cnt, am_start, am_sums;    // AMR: particles by domain node
  DBuf am_gh, am_goff, am_part, am_err, am_flag, am_rowcnt, am_rowoff, am_rsums, am_seps;
  // the AMR hierarchy: every kept grid's run tables, nodes, TSC table,
  // flags, densities and particle lists (slot k: particle ord[k] of node
  // node[k]; node s's slots start[s] .. start[s + 1] - 1)
  struct AmrLevel {
    int l1 = 0, nP = 0, npl = 0, nC = 0, nR = 0, nN = 0, nn = 0;
    uint32_t np = 0;
    DBuf P, pl, C, R, N, key, nseg, tsc, flag, dens, start, ord, node;
  };
  static constexpr int kAmrMaxGrids = 40;
  AmrLevel amr_lv[kAmrMaxGrids + 1];
  int amr_nlev = 0;
  // ... and its scratch: row and plane state machines, fine planes, relink,
  // the radix passes, the density pairs
  DBuf at_rrun, at_rnode, at_rref, at_runoff, at_runs, at_pref, at_po, at_pnc, at_pnsel, at_rroff, at_seloff;
  DBuf at_rr, at_sel, at_fpl, at_tot, at_dest, at_moved, at_moff, at_cnt, at_kA, at_kB, at_iA, at_iB;
  DBuf at_gh, at_goff, at_part, at_err, at_sums, at_w, at_ne, at_srcoff, at_tcnt, at_child, at_cen, at_cfold;
  DBuf am_cfold;   // the domain grid's folded node centres
  // last device result description
  int64_t last_nhalo = -1;
  uint64_t last_nkept = 0, last_nbins = 0;
  ahfgpu_stats last_stats{};
};

Ctx g;

// ---------------------------------------------------------------------------
// small packing kernels

// exclusive scans of the kept counts (block 0, into moff) and of the bin
// counts (block 1, into poff); four consecutive haloes per thread
__global__ void k_scan_counts(const ahfgpu_halo* halo, int64_t nh, uint64_t* moff, uint64_t* poff) {
  const int which = blockIdx.x;
  uint64_t* out = which ? poff : moff;
  __shared__ unsigned long long wsum[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  unsigned long long carry = 0;
  for (int64_t base = 0; base < nh; base += 4 * (int64_t)blockDim.x) {
    const int64_t i0 = base + 4 * (int64_t)threadIdx.x;
    unsigned long long v[4], t = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
      int64_t i = i0 + k;
      v[k] = i < nh ? (which == 0 ? halo[i].npart : (unsigned long long)halo[i].nbins) : 0ull;
    }
#pragma unroll
    for (int k = 0; k < 4; k++) t += v[k];
    unsigned long long inc = t;            // inclusive scan over the warp
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      unsigned long long u = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += u;
    }
    if (lane == 31) wsum[wid] = inc;
    __syncthreads();
    if (wid == 0) {
      unsigned long long w = lane < nw ? wsum[lane] : 0ull;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        unsigned long long u = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += u;
      }
      wsum[lane] = w;
    }
    __syncthreads();
    unsigned long long run = carry + (wid ? wsum[wid - 1] : 0ull) + inc - t;
#pragma unroll
    for (int k = 0; k < 4; k++) {
      run += v[k];
      if (i0 + k < nh) out[i0 + k + 1] = run;
    }
    carry += wsum[nw - 1];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = 0;
}

// kept entries into the packed CSR list of ids (gidx[e], or e without gidx).
// A block copies one chunk of kPackChunk
// output slots: two binary searches over moff bound the haloes it touches;
// when there are at most kPackHaloes of them their offsets are staged in
// shared memory and each slot's halo (the last h with moff[h] <= j) is
// searched there, else in global memory within the same bounds.
constexpr int kPackChunk = 4096, kPackHaloes = 1024;

__device__ __forceinline__ int64_t last_le(const uint64_t* a, int64_t lo, int64_t hi, uint64_t j) {
  while (lo < hi) {
    int64_t mid = (lo + hi + 1) >> 1;
    if (a[mid] <= j) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__global__ void k_pack_members(const uint64_t* off, const uint64_t* stage, const uint64_t* moff,
                               const uint64_t* gidx, uint64_t* member, int64_t nh) {
  __shared__ uint64_t s_moff[kPackHaloes], s_off[kPackHaloes];
  __shared__ int64_t s_h[2];
  const uint64_t total = moff[nh];
  for (uint64_t c0 = (uint64_t)blockIdx.x * kPackChunk; c0 < total; c0 += (uint64_t)gridDim.x * kPackChunk) {
    const uint64_t c1 = c0 + kPackChunk < total ? c0 + kPackChunk : total;
    if (threadIdx.x < 2) s_h[threadIdx.x] = last_le(moff, 0, nh - 1, threadIdx.x ? c1 - 1 : c0);
    __syncthreads();
    const int64_t h0 = s_h[0], nc = s_h[1] - h0 + 1;
    if (nc <= kPackHaloes) {
      for (int64_t i = threadIdx.x; i < nc; i += blockDim.x) {
        s_moff[i] = moff[h0 + i];
        s_off[i] = off[h0 + i];
      }
      __syncthreads();
      for (uint64_t j = c0 + threadIdx.x; j < c1; j += blockDim.x) {
        int64_t i = last_le(s_moff, 0, nc - 1, j);
        uint64_t e = stage[s_off[i] + (j - s_moff[i])];
        member[j] = gidx ? gidx[e] : e;
      }
    } else {
      for (uint64_t j = c0 + threadIdx.x; j < c1; j += blockDim.x) {
        int64_t h = last_le(moff, h0, h0 + nc - 1, j);
        uint64_t e = stage[off[h] + (j - moff[h])];
        member[j] = gidx ? gidx[e] : e;
      }
    }
    __syncthreads();
  }
}

__global__ void k_pack_prof(const ahfgpu_halo* halo, const uint64_t* cap_off, const double* stage,
                            const uint64_t* poff, double* prof, int64_t nh) {
  int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t h = warp; h < nh; h += nw) {
    uint64_t nb = (uint64_t)halo[h].nbins;
    uint64_t cnt = nb * AHFGPU_PROF_NFIELDS;
    const double* s = stage + cap_off[h] * AHFGPU_PROF_NFIELDS;
    double* d = prof + poff[h] * AHFGPU_PROF_NFIELDS;
    for (uint64_t i = lane; i < cnt; i += 32) d[i] = s[i];
  }
}

// min / max of the weights (exactness check of FP64 mass prefixes)
__global__ void k_weight_range(const float* w, uint64_t n, float* out) {
  float mn = INFINITY, mx = 0.f;
  int bad = 0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    float v = w[i];
    if (!(v > 0.f) || !isfinite(v)) bad = 1;
    else { mn = fminf(mn, v); mx = fmaxf(mx, v); }
  }
  for (int o = 16; o > 0; o >>= 1) {
    mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
    mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    bad |= __shfl_xor_sync(0xffffffffu, bad, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin((int*)&out[0], __float_as_int(mn));   // positive floats order as ints
    atomicMax((int*)&out[1], __float_as_int(mx));
    if (bad) atomicMax((int*)&out[2], 1);
  }
}

__global__ void k_init_wred(float* out) {
  out[0] = INFINITY;
  out[1] = 0.f;
  ((int*)out)[2] = 0;
}

int ensure_init() {
  if (!g.init) return fail(AHFGPU_ERR_STATE, "ahfgpu_init() has not been called");
  CK(cudaSetDevice(g.device));
  return AHFGPU_OK;
}

int nbins_cap(uint64_t n, int64_t minpart) {
  if (n < (uint64_t)minpart || n == 0) return 0;
  int nb = (int)(6.2 * log10((double)n) - 3.5);
  nb = std::max(2, nb) + 1;            // +1: device log10 may differ by an ulp
  return std::min(nb, kMaxBins);
}

// the longest list the one-list-per-thread kernel may be given (class 0)
constexpr uint64_t kSmallMaxList = 1024;

// batches below this many particles are copied in one piece
constexpr uint64_t kSplitMinParticles = 1u << 22;

struct Plan {
  int64_t nhalo = 0;
  uint64_t N = 0, maxn = 0, nbins_total = 0;
  std::vector<int32_t> queue;
  int cls_begin[4] = {0, 0, 0, 0};   // queue positions of the FP32C size classes (largest class first)
  // FP32C: queue positions ending parts 0..P-2 (increasing); part p is
  // launched as soon as its inputs are in.  Empty: one part.
  std::vector<int> cuts;
  std::vector<uint64_t> prof_cap_off;
};

int validate_and_plan(const ahfgpu_params* p, const uint64_t* off, int64_t nh, Plan& pl) {
  if (inject_oom("host_plan")) throw std::bad_alloc();
  if (!p) return fail(AHFGPU_ERR_INVALID, "params is NULL");
  if (p->MINPART < 4) return fail(AHFGPU_ERR_INVALID, "MINPART must be >= 4 (got %lld)", (long long)p->MINPART);
  if (p->MINPART > 128)
    return fail(AHFGPU_ERR_CAPACITY, "MINPART %lld exceeds the supported maximum of 128", (long long)p->MINPART);
  if (!(p->VescTune > 0) || !(p->rho_vir > 0) || !(p->v_fac > 0))
    return fail(AHFGPU_ERR_INVALID, "non-positive VescTune, rho_vir or v_fac");
  if (nh < 0) return fail(AHFGPU_ERR_INVALID, "nhalo < 0");
  if (nh > 0x7fffffff) return fail(AHFGPU_ERR_CAPACITY, "nhalo %lld exceeds 2^31-1", (long long)nh);
  pl.nhalo = nh;
  if (nh == 0) return AHFGPU_OK;
  if (!off) return fail(AHFGPU_ERR_INVALID, "off is NULL");
  if (off[0] != 0) return fail(AHFGPU_ERR_INVALID, "off[0] != 0");
  pl.prof_cap_off.assign(nh + 1, 0);
  for (int64_t h = 0; h < nh; h++) {
    if (off[h + 1] < off[h]) return fail(AHFGPU_ERR_INVALID, "off not monotone at halo %lld", (long long)h);
    uint64_t n = off[h + 1] - off[h];
    if (n > 0xffffffffull) return fail(AHFGPU_ERR_CAPACITY, "halo %lld has %llu > 2^32-1 particles", (long long)h,
                                       (unsigned long long)n);
    pl.maxn = std::max(pl.maxn, n);
    pl.prof_cap_off[h + 1] = pl.prof_cap_off[h] + (uint64_t)nbins_cap(n, p->MINPART);
  }
  pl.N = off[nh];
  pl.nbins_total = pl.prof_cap_off[nh];
  // largest first, ties by index: a stable radix sort (two 16-bit digits)
  // of the complemented sizes, starting from the ascending indices
  pl.queue.resize(nh);
  {
    std::vector<int32_t> tmp(nh);
    std::vector<uint32_t> cnt(65537);
    std::iota(tmp.begin(), tmp.end(), 0);
    int32_t* src = tmp.data();
    int32_t* dst = pl.queue.data();
    for (int shift = 0; shift < 32; shift += 16) {
      std::fill(cnt.begin(), cnt.end(), 0u);
      auto digit = [&](int32_t h) { return (~(uint32_t)(off[h + 1] - off[h]) >> shift) & 0xffffu; };
      for (int64_t i = 0; i < nh; i++) cnt[digit(src[i]) + 1]++;
      for (int d = 0; d < 65536; d++) cnt[d + 1] += cnt[d];
      for (int64_t i = 0; i < nh; i++) dst[cnt[digit(src[i])]++] = src[i];
      std::swap(src, dst);
    }
    // two passes: the sorted order is back in tmp
    std::copy(tmp.begin(), tmp.end(), pl.queue.begin());
  }
  // the queue is largest first: class 2 (largest) occupies the front
  int64_t qp = 0;
  pl.cls_begin[0] = 0;
  while (qp < nh && off[pl.queue[qp] + 1] - off[pl.queue[qp]] > fp32c_class_max(1)) qp++;
  pl.cls_begin[1] = (int)qp;
  while (qp < nh && off[pl.queue[qp] + 1] - off[pl.queue[qp]] > fp32c_class_max(0)) qp++;
  pl.cls_begin[2] = (int)qp;
  pl.cls_begin[3] = (int)nh;
  return AHFGPU_OK;
}

int ensure_work(const Plan& pl, int nblocks, int stack_cap) {
  // per-slot arrays also hold the FP32C alignment gaps (slot_base)
  const uint64_t N = std::max<uint64_t>(pl.N, 1) + 3 * (uint64_t)pl.nhalo + 16;
  int rc;
#define EN(buf, bytes) if ((rc = (buf).ensure(bytes)) != AHFGPU_OK) return rc
  EN(g.keyA, N * 8); EN(g.keyB, N * 8); EN(g.idxA, N * 4); EN(g.idxB, N * 4);
  EN(g.sdx, N * 8); EN(g.sdy, N * 8); EN(g.sdz, N * 8); EN(g.sd, N * 8);
  EN(g.svx, N * 4); EN(g.svy, N * 4); EN(g.svz, N * 4); EN(g.sw, N * 4);
  EN(g.seid, N * 4); EN(g.phi, N * 8); EN(g.flag, N); EN(g.nflag, N);
  EN(g.pa, N * 8); EN(g.pb, N * 8); EN(g.pc, N * 8); EN(g.pd, N * 8);
  EN(g.fdh, N * 4); EN(g.fdl, N * 4); EN(g.fdx, N * 4); EN(g.fdy, N * 4); EN(g.fdz, N * 4);
  EN(g.fdxl, N * 4); EN(g.fdyl, N * 4); EN(g.fdzl, N * 4); EN(g.fqh, N * 4); EN(g.fql, N * 4);
  EN(g.rec, N * 32);
  EN(g.stack, (size_t)nblocks * stack_cap * sizeof(uint4));
  EN(g.halo, std::max<int64_t>(pl.nhalo, 1) * sizeof(ahfgpu_halo));
  EN(g.mem_stage, N * 8);
  EN(g.prof_stage, std::max<uint64_t>(pl.nbins_total, 1) * AHFGPU_PROF_NFIELDS * 8);
  EN(g.prof_cap_off, (pl.nhalo + 1) * 8);
  EN(g.fin, std::max<int64_t>(pl.nhalo, 1) * kFinStride * 8);
  EN(g.queue, std::max<int64_t>(pl.nhalo, 1) * 4);
  EN(g.qhead, kQueueHeads * 4);
  EN(g.counters, 64);
  EN(g.err, 64);
  EN(g.wred, 64);
  EN(g.member_off, (pl.nhalo + 1) * 8);
  EN(g.member, N * 8);
  EN(g.prof_off, (pl.nhalo + 1) * 8);
  EN(g.prof, std::max<uint64_t>(pl.nbins_total, 1) * AHFGPU_PROF_NFIELDS * 8);
#undef EN
  return AHFGPU_OK;
}

// One FP32C launch: the queue range [q0, q1) of one size class within one
// queue part, with its grid.
struct Seg {
  int part, cls, q0, q1, grid;
};

int part_begin(const Plan& pl, int p) { return p == 0 ? 0 : pl.cuts[p - 1]; }
int part_end(const Plan& pl, int p) { return p < (int)pl.cuts.size() ? pl.cuts[p] : (int)pl.nhalo; }

std::vector<Seg> fp32c_segments(const Plan& pl) {
  std::vector<Seg> v;
  for (int p = 0; p <= (int)pl.cuts.size(); p++)
    for (int k = 0; k < 3; k++) {                 // queue segment k holds class 2-k
      int q0 = std::max(pl.cls_begin[k], part_begin(pl, p));
      int q1 = std::min(pl.cls_begin[k + 1], part_end(pl, p));
      if (q1 <= q0) continue;
      int cls = 2 - k;
      if (cls == 0 && g.small_on)   // blocks of 128 threads, one list per thread
        v.push_back({p, cls, q0, q1, std::min(g.nsm * g.small_bps, (q1 - q0 + 127) / 128)});
      else
        v.push_back({p, cls, q0, q1, std::min(g.nsm * g.fp32c_bps[cls], q1 - q0)});
    }
  return v;
}

// Runs the stage on a device batch.  Results stay in g.* buffers.  With a
// staging hook (host path), stage(p) issues the input copies of queue part
// p on g.copy_stream and records g.ev_part[p] (stage(P): the ids, g.ev_ids);
// it is called after the small set-up copies for part 0 and right before
// the first launch of each later part, and each part's launches wait for
// its own event only.
int run_device(const ahfgpu_params* prm, const ahfgpu_batch* db, const Plan& pl, ahfgpu_mode mode,
               cudaStream_t st, ahfgpu_stats* stats, const std::function<int(int)>* stage = nullptr) {
  int rc;
  if (mode != AHFGPU_PLAIN_FP64 && mode != AHFGPU_BATCHED_FP64 && mode != AHFGPU_BATCHED_FP32C)
    return fail(AHFGPU_ERR_INVALID, "unknown mode %d", (int)mode);
  if (!pl.cuts.empty() && mode != AHFGPU_BATCHED_FP32C) return fail(AHFGPU_ERR_STATE, "split queue outside FP32C");
  if ((int)pl.cuts.size() >= kMaxParts) return fail(AHFGPU_ERR_STATE, "too many queue parts");
  const std::vector<Seg> segs = fp32c_segments(pl);
  int grid = g.nsm * g.fp64_bps;
  {
    int sum = 0;
    for (const Seg& sg : segs) sum += sg.grid;
    grid = std::max(1, std::max(grid, sum));
  }
  const int stack_cap = (int)std::min<uint64_t>(std::max<uint64_t>(pl.maxn / 512 + 64, 64), 1u << 20);
  if ((rc = ensure_work(pl, grid, stack_cap))) return rc;
  // the small-list kernel's work space: per class-0 segment, per warp
  const uint32_t small_nmax = (uint32_t)std::min<uint64_t>(fp32c_class_max(0), std::max<uint64_t>(pl.maxn, 1));
  std::vector<size_t> small_off;
  if (mode == AHFGPU_BATCHED_FP32C && g.small_on) {
    size_t tot = 0;
    for (const Seg& sg : segs) {
      small_off.push_back(tot);
      if (sg.cls == 0) tot += (size_t)sg.grid * 4 * fp32c_small_bytes_per_warp(small_nmax);
    }
    if (tot && (rc = g.small_scr.ensure(tot))) return rc;
  }
  const int64_t nh = pl.nhalo;
  stats->n_particles_in = pl.N;
  if (nh == 0) {
    CK(cudaMemsetAsync(g.member_off.p, 0, 8, st));
    CK(cudaMemsetAsync(g.prof_off.p, 0, 8, st));
    g.last_nhalo = 0; g.last_nkept = 0; g.last_nbins = 0;
    return AHFGPU_OK;
  }
  CK(cudaMemcpyAsync(g.prof_cap_off.p, pl.prof_cap_off.data(), (nh + 1) * 8, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(g.queue.p, pl.queue.data(), nh * 4, cudaMemcpyHostToDevice, st));
  CK(cudaMemsetAsync(g.qhead.p, 0, kQueueHeads * 4, st));
  CK(cudaMemsetAsync(g.counters.p, 0, 64, st));
  CK(cudaMemsetAsync(g.err.p, 0, 64, st));
  CK(cudaMemsetAsync(g.halo.p, 0, nh * sizeof(ahfgpu_halo), st));
  int staged = 0;   // parts whose copies are issued
  const int nparts = (int)pl.cuts.size() + 1;
  if (stage) {
    if ((rc = (*stage)(staged++))) return rc;
    // the set-up work on this stream (weight check, device timer) waits for
    // the inputs of the first part (all of them without a split)
    CK(cudaStreamWaitEvent(st, g.ev_part[0], 0));
  }

  DevParams P;
  memset(&P, 0, sizeof P);   // padding too: the struct is part of the graph signature
  P.VescTune = prm->VescTune;
  P.v2_tune = prm->VescTune * prm->VescTune;
  P.MINPART = prm->MINPART;
  P.ovlim = prm->ovlim;
  P.rho_vir = prm->rho_vir;
  P.r_fac = prm->r_fac; P.x_fac = prm->x_fac; P.v_fac = prm->v_fac; P.m_fac = prm->m_fac;
  P.rho_fac = prm->rho_fac; P.phi_fac = prm->phi_fac; P.Hubble = prm->Hubble;
  P.has_w = db->w != nullptr;
  P.f_ovlim = (float)prm->ovlim;
  P.f_rvrf = (float)(prm->rho_vir / prm->rho_fac);
  P.force_serial = 0;
  {
    const char* fe = getenv("AHFGPU_FORCE_EXACT");   // test hook
    // 1: every unbinding iteration in the reference's exact order;
    // 2 (FP32C): one decision per tile through the exact resolution
    P.force_exact = (fe && fe[0] == '1') ? 1 : (fe && fe[0] == '2') ? 2 : 0;
  }
  uint64_t launches = 0;
  if (db->w) {
    // FP64 mass prefixes are exact when every partial sum is a multiple of
    // the smallest weight's quantum below 2^53 of them.
    k_init_wred<<<1, 1, 0, st>>>(g.wred.as<float>());
    k_weight_range<<<g.nsm * 4, 256, 0, st>>>(db->w, pl.N, g.wred.as<float>());
    launches += 2;
    float wr[3];
    CK(cudaMemcpyAsync(wr, g.wred.p, 12, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    int bad = 0;
    memcpy(&bad, &wr[2], 4);
    if (bad) return fail(AHFGPU_ERR_INVALID, "weights must be positive and finite");
    double q = std::ldexp(1.0, std::ilogb((double)wr[0]) - 23);
    double bound = (double)pl.maxn * (double)wr[1] / q;
    if (!(bound < 4503599627370496.0)) P.force_serial = 1;   // 2^52
  }

  DevBatch B;
  memset(&B, 0, sizeof B);
  B.nhalo = nh;
  B.off = db->off;
  B.x = db->x; B.y = db->y; B.z = db->z;
  B.vx = db->vx; B.vy = db->vy; B.vz = db->vz;
  B.w = db->w;
  B.gidx = nullptr;   // the kernels stage entry indices; the pack maps them to ids
  B.cx = db->cx; B.cy = db->cy; B.cz = db->cz;

  Work W;
  memset(&W, 0, sizeof W);
  W.keyA = g.keyA.as<uint64_t>(); W.keyB = g.keyB.as<uint64_t>();
  W.rec = g.rec.as<float4>();
  W.idxA = g.idxA.as<uint32_t>(); W.idxB = g.idxB.as<uint32_t>();
  W.sdx = g.sdx.as<double>(); W.sdy = g.sdy.as<double>(); W.sdz = g.sdz.as<double>(); W.sd = g.sd.as<double>();
  W.svx = g.svx.as<float>(); W.svy = g.svy.as<float>(); W.svz = g.svz.as<float>(); W.sw = g.sw.as<float>();
  W.seid = g.seid.as<uint32_t>();
  W.phi = g.phi.as<double>();
  W.flag = g.flag.as<uint8_t>();
  W.nflag = g.nflag.as<uint8_t>();
  W.prof_a = g.pa.as<double>(); W.prof_b = g.pb.as<double>(); W.prof_c = g.pc.as<double>(); W.prof_d = g.pd.as<double>();
  W.sort_stack = g.stack.as<uint4>();
  W.stack_cap = stack_cap;
  W.halo = g.halo.as<ahfgpu_halo>();
  W.mem_stage = g.mem_stage.as<uint64_t>();
  W.prof_stage = g.prof_stage.as<double>();
  W.fin = g.fin.as<double>();
  W.prof_cap_off = g.prof_cap_off.as<uint64_t>();
  W.queue_head = g.qhead.as<unsigned int>();
  W.queue = g.queue.as<int32_t>();
  W.nqueue = (int)nh;
  W.counters = g.counters.as<unsigned long long>();
  W.err = g.err.as<int>();
  W.fdh = g.fdh.as<float>(); W.fdl = g.fdl.as<float>();
  W.fdx = g.fdx.as<float>(); W.fdy = g.fdy.as<float>(); W.fdz = g.fdz.as<float>();
  W.fdxl = g.fdxl.as<float>(); W.fdyl = g.fdyl.as<float>(); W.fdzl = g.fdzl.as<float>();
  W.fqh = g.fqh.as<float>(); W.fql = g.fql.as<float>();
#ifdef AHFGPU_PHASE_TIMERS
  // kPhaseSlots phase counters, then per halo {start ns, end ns, SM cycles, SM id}
  if ((rc = g.phase.ensure((kPhaseSlots + 4 * (size_t)nh) * 8))) return rc;
  W.phase = g.phase.as<unsigned long long>();
#endif

  // the launch sequence, from the device timer's start to the end of the
  // pack; issued directly, or captured once as a CUDA graph and re-launched
  bool capturing = false;
  auto rec_time = [&](cudaEvent_t ev, cudaStream_t s) {
    return cudaEventRecordWithFlags(ev, s, capturing ? cudaEventRecordExternal : cudaEventRecordDefault);
  };
  auto issue = [&]() -> int {
    CK(rec_time(g.ev0, st));
    if (mode == AHFGPU_PLAIN_FP64) {
      // one halo at a time, in batch order
      for (int64_t h = 0; h < nh; h++) {
        launch_fp64(P, B, W, 1, (int)h, st);
        launches++;
      }
    } else if (mode == AHFGPU_BATCHED_FP64) {
      launch_fp64(P, B, W, g.nsm * g.fp64_bps, -1, st);
      launches++;
    } else {
      // size classes on streams of their own (larger classes at higher
      // priority), queue parts in order; each segment has its own queue
      // range, queue head and worklist region.  A later part's launch takes
      // SMs as the CTAs of the earlier parts run out of work and exit.
      CK(cudaEventRecord(g.ev_fork, st));
      int stack_base = 0, slot = 2;
      for (const Seg& sg : segs) {
        while (stage && staged <= sg.part)
          if ((rc = (*stage)(staged++))) return rc;
        Work Wc = W;
        Wc.queue = g.queue.as<int32_t>() + sg.q0;
        Wc.nqueue = sg.q1 - sg.q0;
        Wc.queue_head = g.qhead.as<unsigned int>() + slot++;
        Wc.sort_stack = g.stack.as<uint4>() + (size_t)stack_base * stack_cap;
        stack_base += sg.grid;
        cudaStream_t cs = g.seg_stream[sg.part][sg.cls];
        CK(cudaStreamWaitEvent(cs, g.ev_fork, 0));
        if (stage) CK(cudaStreamWaitEvent(cs, g.ev_part[sg.part], 0));
        if (sg.cls == 0 && g.small_on)
          launch_fp32c_small(P, B, Wc, g.small_scr.as<unsigned char>() + small_off[&sg - segs.data()], small_nmax,
                             sg.grid, cs);
        else
          launch_fp32c(sg.cls, P, B, Wc, sg.grid, cs);
        CK(cudaEventRecord(g.ev_join[sg.part][sg.cls], cs));
        CK(cudaStreamWaitEvent(st, g.ev_join[sg.part][sg.cls], 0));
        launches++;
      }
    }
    if (mode == AHFGPU_BATCHED_FP32C) {
      launch_fp32c_finish(P, B, W.halo, W.prof_cap_off, W.prof_stage, W.fin, nh,
                          std::max(1, std::min<int>(g.nsm * 4, (int)((nh + 127) / 128))), st);
      launches++;
    }
    launch_concentration(W.halo, nh, std::max(1, std::min<int>(g.nsm * 4, (int)((nh + 127) / 128))), st);
    launches++;
    CK(cudaGetLastError());
    CK(rec_time(g.ev1, st));
    // pack
    k_scan_counts<<<2, 1024, 0, st>>>(W.halo, nh, g.member_off.as<uint64_t>(), g.prof_off.as<uint64_t>());
    int pg = (int)std::min<int64_t>((nh * 32 + 255) / 256, (int64_t)g.nsm * 16);
    int mg = (int)std::max<uint64_t>(1, std::min<uint64_t>((pl.N + kPackChunk - 1) / kPackChunk, (uint64_t)g.nsm * 8));
    if (stage) {
      while (staged <= nparts)   // the parts without launches, then the ids
        if ((rc = (*stage)(staged++))) return rc;
      CK(cudaStreamWaitEvent(st, g.ev_ids, 0));   // the ids come last
    }
    k_pack_members<<<mg, 256, 0, st>>>(db->off, W.mem_stage, g.member_off.as<uint64_t>(), db->gidx,
                                        g.member.as<uint64_t>(), nh);
    k_pack_prof<<<pg, 256, 0, st>>>(W.halo, W.prof_cap_off, W.prof_stage, g.prof_off.as<uint64_t>(),
                                     g.prof.as<double>(), nh);
    launches += 3;
    CK(cudaGetLastError());
    CK(rec_time(g.ev2, st));
    return AHFGPU_OK;
  };
  const bool graphable = g.use_graph && !stage && mode != AHFGPU_PLAIN_FP64;
  bool done = false;
  if (graphable) {
    // everything the sequence depends on: the kernels' arguments (params,
    // batch, work-space pointers), the queue segments and grids, the outputs
    std::vector<unsigned char> sig;
    auto put = [&](const void* p, size_t n) {
      const unsigned char* c = (const unsigned char*)p;
      sig.insert(sig.end(), c, c + n);
    };
    put(&mode, sizeof mode);
    put(&P, sizeof P);
    put(&B, sizeof B);
    put(&W, sizeof W);
    put(&nh, sizeof nh);
    put(&pl.N, sizeof pl.N);
    put(&stack_cap, sizeof stack_cap);
    put(&st, sizeof st);
    for (const Seg& sg : segs) put(&sg, sizeof sg);
    put(&g.small_on, sizeof g.small_on);
    put(&g.small_scr.p, sizeof g.small_scr.p);
    put(&small_nmax, sizeof small_nmax);
    const void* outs[6] = {db->off, db->gidx, g.member_off.p, g.prof_off.p, g.member.p, g.prof.p};
    put(outs, sizeof outs);
    if (g.graph_exec && sig == g.graph_sig) {
      CK(cudaGraphLaunch(g.graph_exec, st));
      launches = g.graph_launches;
      g.graph_replays++;
      done = true;
    } else if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      capturing = true;
      const uint64_t l0 = launches;
      rc = issue();
      cudaGraph_t graph = nullptr;
      cudaError_t e = cudaStreamEndCapture(st, &graph);
      capturing = false;
      if (rc) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
      }
      cudaGraphExec_t ex = nullptr;
      if (e == cudaSuccess && cudaGraphInstantiate(&ex, graph, 0) == cudaSuccess) {
        if (g.graph_exec) cudaGraphExecDestroy(g.graph_exec);
        g.graph_exec = ex;
        g.graph_sig.swap(sig);
        g.graph_launches = launches;
        CK(cudaGraphLaunch(ex, st));
        done = true;
      } else {
        launches = l0;   // capture refused: issue the launches directly
      }
      if (graph) cudaGraphDestroy(graph);
      cudaGetLastError();
    } else {
      cudaGetLastError();
    }
  }
  if (!done && (rc = issue())) return rc;
  uint64_t tails[2];
  unsigned long long cnt[4];
  int derr = 0;
  CK(cudaMemcpyAsync(&tails[0], g.member_off.as<uint64_t>() + nh, 8, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(&tails[1], g.prof_off.as<uint64_t>() + nh, 8, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(cnt, g.counters.p, 32, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(&derr, g.err.p, 4, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (derr == kErrWorklist) return fail(AHFGPU_ERR_CAPACITY, "radial sort worklist overflow");
  if (derr == kErrSortState) return fail(AHFGPU_ERR_CUDA, "radial sort: inconsistent bucket run (self-check)");
  if (derr) return fail(AHFGPU_ERR_CUDA, "device error code %d", derr);
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, g.ev0, g.ev1));
  stats->ms_device = ms;
  CK(cudaEventElapsedTime(&ms, g.ev1, g.ev2));
  stats->ms_pack = ms;
  if (stage) {
    CK(cudaEventElapsedTime(&ms, g.ev_cp0, g.ev_ids));
    stats->ms_h2d = ms;
    CK(cudaEventElapsedTime(&ms, g.ev_cp0, g.ev_part[0]));
    stats->ms_h2d_first = ms;
  }
  stats->n_kept = tails[0];
  stats->n_retest = cnt[0];
  stats->n_replay_halos = cnt[1];
  stats->n_key_ties = cnt[2];
  stats->n_fp64_halos = mode == AHFGPU_BATCHED_FP32C ? cnt[3] : 0;
  stats->n_launches = launches;
  g.last_nhalo = nh;
  g.last_nkept = tails[0];
  g.last_nbins = tails[1];
  return AHFGPU_OK;
}

void library_anchor() {}

// The tuning cache: a JSON object keyed by "<device name>|<SMs>|<cc>", each
// value {"class_max": [a, b], "class_bps": [c0, c1, c2]} (written by
// python -m ahf_gb300.autotune).  Path: AHFGPU_TUNE_CACHE, else
// tune_cache.json beside this library.
std::string tune_cache_path() {
  if (const char* e = getenv("AHFGPU_TUNE_CACHE")) return e;
  Dl_info info;
  if (dladdr((void*)&library_anchor, &info) && info.dli_fname) {
    std::string f = info.dli_fname;
    size_t k = f.find_last_of('/');
    return (k == std::string::npos ? std::string(".") : f.substr(0, k)) + "/tune_cache.json";
  }
  return "tune_cache.json";
}

void load_tuning(const cudaDeviceProp& prop) {
  char key[320];
  snprintf(key, sizeof key, "%s|%d|%d.%d", prop.name, prop.multiProcessorCount, prop.major, prop.minor);
  g.tune_key = key;
  g.tune_source = "default";
  g.tune_class_max[0] = 512; g.tune_class_max[1] = 16384;
  for (int k = 0; k < 3; k++) g.tune_bps_cap[k] = 0;
  const std::string path = tune_cache_path();
  if (FILE* f = fopen(path.c_str(), "rb")) {
    std::string js;
    char buf[4096];
    size_t r;
    while ((r = fread(buf, 1, sizeof buf, f)) > 0 && js.size() < (1u << 20)) js.append(buf, r);
    fclose(f);
    size_t at = js.find(std::string("\"") + key + "\"");
    if (at != std::string::npos) {
      size_t end = js.find('}', at);
      std::string obj = js.substr(at, end == std::string::npos ? std::string::npos : end - at);
      unsigned long long a = 0, b = 0;
      int c0 = 0, c1 = 0, c2 = 0;
      size_t m = obj.find("\"class_max\"");
      size_t q = m == std::string::npos ? m : obj.find('[', m);
      if (q != std::string::npos && sscanf(obj.c_str() + q, "[ %llu , %llu", &a, &b) == 2 && a >= 1 && b >= a) {
        g.tune_class_max[0] = a; g.tune_class_max[1] = b;
        g.tune_source = path;
      }
      m = obj.find("\"class_bps\"");
      q = m == std::string::npos ? m : obj.find('[', m);
      if (q != std::string::npos && sscanf(obj.c_str() + q, "[ %d , %d , %d", &c0, &c1, &c2) == 3) {
        g.tune_bps_cap[0] = c0; g.tune_bps_cap[1] = c1; g.tune_bps_cap[2] = c2;
        g.tune_source = path;
      }
    }
  }
  // environment overrides (tuning runs)
  if (const char* e = getenv("AHFGPU_CLASS_MAX")) {
    unsigned long long a = 0, b = 0;
    if (sscanf(e, "%llu,%llu", &a, &b) == 2 && a >= 1 && b >= a) {
      g.tune_class_max[0] = a; g.tune_class_max[1] = b;
      g.tune_source = "environment";
    }
  }
  if (const char* e = getenv("AHFGPU_CLASS_BPS")) {
    int c[3] = {0, 0, 0};
    if (sscanf(e, "%d,%d,%d", &c[0], &c[1], &c[2]) == 3) {
      for (int k = 0; k < 3; k++) g.tune_bps_cap[k] = c[k];
      g.tune_source = "environment";
    }
  }
  fp32c_set_class_max(g.tune_class_max[0], g.tune_class_max[1], g.small_on ? kSmallMaxList : 512);
  g.tune_class_max[0] = fp32c_class_max(0);
  g.tune_class_max[1] = fp32c_class_max(1);
}

void fill_dres(ahfgpu_result* r) {
  memset(r, 0, sizeof(*r));
  r->nhalo = g.last_nhalo;
  r->halo = g.halo.as<ahfgpu_halo>();
  r->member_off = g.member_off.as<uint64_t>();
  r->member = g.member.as<uint64_t>();
  r->prof_off = g.prof_off.as<uint64_t>();
  r->prof = g.prof.as<double>();
  r->stats = g.last_stats;
}

}  // namespace

extern "C" {

static int init_impl(int device) {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    cudaGetLastError();
    return fail(AHFGPU_ERR_NO_DEVICE, "no CUDA device: %s", cudaGetErrorString(e));
  }
  if (device < 0 || device >= n) return fail(AHFGPU_ERR_NO_DEVICE, "device %d out of range [0,%d)", device, n);
  if (g.init && g.device == device) return AHFGPU_OK;
  if (g.init) ahfgpu_shutdown();
  CK(cudaSetDevice(device));
  cudaDeviceProp prop;
  CK(cudaGetDeviceProperties(&prop, device));
  if (prop.major != 10 || prop.minor != 3)
    return fail(AHFGPU_ERR_NO_DEVICE, "device %d is sm_%d%d; this build targets sm_103a", device, prop.major,
                prop.minor);
  g.device = device;
  g.nsm = prop.multiProcessorCount;
  CK(cudaStreamCreateWithFlags(&g.stream, cudaStreamNonBlocking));
  CK(cudaEventCreate(&g.ev0));
  CK(cudaEventCreate(&g.ev1));
  g.fp64_bps = std::max(1, fp64_max_blocks_per_sm());
  {
    const char* e = getenv("AHFGPU_GRAPH");   // "0": device-resident calls launch directly
    g.use_graph = !(e && e[0] == '0');
    const char* sm = getenv("AHFGPU_SMALL");  // "0": the small lists on 64-thread CTAs instead
    g.small_on = !(sm && sm[0] == '0');
    g.small_bps = std::max(1, fp32c_small_occupancy());
  }
  load_tuning(prop);
  // the class-0 cap also bounds the one-list-per-thread kernel's CTAs per SM
  if (g.tune_bps_cap[0] >= 1) g.small_bps = std::min(g.small_bps, g.tune_bps_cap[0]);
  CK((cudaError_t)gather_sort_setup());
  for (int k = 0; k < 3; k++) {
    g.fp32c_bps[k] = std::max(1, fp32c_max_blocks_per_sm(k));
    if (g.tune_bps_cap[k] >= 1) g.fp32c_bps[k] = std::min(g.fp32c_bps[k], g.tune_bps_cap[k]);
    // larger classes get higher priority: their CTAs are scheduled first and
    // the small-halo classes fill SMs as they free up
    int lo = 0, hi = 0;
    CK(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    int pr = k == 2 ? hi : (k == 1 ? (lo + hi) / 2 : lo);
    for (int p = 0; p < kMaxParts; p++) {
      CK(cudaStreamCreateWithPriority(&g.seg_stream[p][k], cudaStreamNonBlocking, pr));
      CK(cudaEventCreateWithFlags(&g.ev_join[p][k], cudaEventDisableTiming));
    }
  }
  CK(cudaEventCreateWithFlags(&g.ev_fork, cudaEventDisableTiming));
  CK(cudaStreamCreateWithFlags(&g.copy_stream, cudaStreamNonBlocking));
  for (int p = 0; p < kMaxParts; p++) CK(cudaEventCreate(&g.ev_part[p]));
  CK(cudaEventCreate(&g.ev_ids));
  CK(cudaEventCreate(&g.ev2));
  CK(cudaEventCreate(&g.ev_cp0));
  CK(cudaGetLastError());
  g.init = true;
  g_err.clear();
  return AHFGPU_OK;
}

static void host_spare_release();

int ahfgpu_shutdown(void) {
  host_spare_release();
  if (!g.init) return AHFGPU_OK;
  cudaSetDevice(g.device);
  cudaDeviceSynchronize();
  DBuf* bufs[] = {&g.in_off, &g.in_x, &g.in_y, &g.in_z, &g.in_vx, &g.in_vy, &g.in_vz, &g.in_w, &g.in_gidx,
                  &g.in_cx, &g.in_cy, &g.in_cz, &g.keyA, &g.keyB, &g.idxA, &g.idxB, &g.sdx, &g.sdy, &g.sdz,
                  &g.sd, &g.svx, &g.svy, &g.svz, &g.sw, &g.seid, &g.phi, &g.flag, &g.nflag, &g.pa, &g.pb,
                  &g.pc, &g.pd, &g.fdh, &g.fdl, &g.fdx, &g.fdy, &g.fdz, &g.fdxl, &g.fdyl, &g.fdzl, &g.fqh, &g.fql, &g.rec, &g.stack, &g.halo, &g.mem_stage, &g.prof_stage, &g.prof_cap_off, &g.queue,
                  &g.qhead, &g.counters, &g.err, &g.wred, &g.fin, &g.member_off, &g.member, &g.prof_off, &g.prof,
                  &g.ga_cell, &g.ga_count, &g.ga_start, &g.ga_fill, &g.ga_sums, &g.ga_sorted, &g.ga_queue,
                  &g.ga_qhead, &g.ga_cnt, &g.ga_off, &g.ga_hfill, &g.ga_idx, &g.ga_idxA, &g.ga_keyB, &g.ga_idxB,
                  &g.ga_stack, &g.ga_err, &g.ga_x, &g.ga_y, &g.ga_z, &g.ga_vx, &g.ga_vy, &g.ga_vz, &g.ga_w,
                  &g.ga_id, &g.ga_fbq, &g.ga_fbn, &g.ga_items, &g.gr_pos, &g.gr_lim, &g.gr_orig, &g.wp_blk, &g.wp_boff, &g.wp_good, &g.wp_qhead,
                  &g.wp_out, &g.wb_chunk, &g.wb_coff, &g.wp_cbytes,
                  &g.wp_cboff, &g.sfc_kb, &g.sfc_ia, &g.sfc_ib, &g.sfc_gh, &g.sfc_goff, &g.sfc_part,
                  &g.sfc_err, &g.phase, &g.am_key, &g.am_keyb, &g.am_idx, &g.am_idxb, &g.am_cnt,
                  &g.am_start, &g.am_sums, &g.am_gh, &g.am_goff, &g.am_part, &g.am_err, &g.am_flag,
                  &g.am_rowcnt, &g.am_rowoff, &g.am_rsums, &g.am_seps, &g.small_scr, &g.at_rrun, &g.at_rnode,
                  &g.at_rref, &g.at_runoff, &g.at_runs, &g.at_pref, &g.at_po, &g.at_pnc, &g.at_pnsel, &g.at_rroff,
                  &g.at_seloff, &g.at_rr, &g.at_sel, &g.at_fpl, &g.at_tot, &g.at_dest, &g.at_moved, &g.at_moff,
                  &g.at_cnt, &g.at_kA, &g.at_kB, &g.at_iA, &g.at_iB, &g.at_gh, &g.at_goff, &g.at_part, &g.at_err,
                  &g.at_sums, &g.at_w, &g.at_ne, &g.at_srcoff, &g.at_tcnt, &g.at_child,
                  &g.at_cen, &g.at_cfold, &g.am_cfold};
  for (DBuf* b : bufs) b->release();
  for (Ctx::AmrLevel& L : g.amr_lv)
    for (DBuf* b : {&L.P, &L.pl, &L.C, &L.R, &L.N, &L.key, &L.nseg, &L.tsc, &L.flag, &L.dens, &L.start, &L.ord, &L.node})
      b->release();
  g.amr_nlev = 0;
  for (int p = 0; p < kMaxParts; p++)
    for (int k = 0; k < 3; k++) {
      if (g.seg_stream[p][k]) cudaStreamDestroy(g.seg_stream[p][k]);
      if (g.ev_join[p][k]) cudaEventDestroy(g.ev_join[p][k]);
    }
  if (g.copy_stream) cudaStreamDestroy(g.copy_stream);
  for (int p = 0; p < kMaxParts; p++)
    if (g.ev_part[p]) cudaEventDestroy(g.ev_part[p]);
  if (g.ev_ids) cudaEventDestroy(g.ev_ids);
  if (g.ev_fork) cudaEventDestroy(g.ev_fork);
  if (g.graph_exec) cudaGraphExecDestroy(g.graph_exec);
  if (g.ev0) cudaEventDestroy(g.ev0);
  if (g.ev1) cudaEventDestroy(g.ev1);
  if (g.ev2) cudaEventDestroy(g.ev2);
  if (g.ev_cp0) cudaEventDestroy(g.ev_cp0);
  if (g.stream) cudaStreamDestroy(g.stream);
  g = Ctx();
  return AHFGPU_OK;
}

static int construct_halos_device_impl(const ahfgpu_params* params, const ahfgpu_batch* batch, ahfgpu_result* dres,
                                  ahfgpu_mode mode, void* stream) {
  int rc = ensure_init();
  if (rc) return rc;
  if (!batch || !dres) return fail(AHFGPU_ERR_INVALID, "batch/result is NULL");
  auto t0 = std::chrono::steady_clock::now();
  cudaStream_t st = stream ? (cudaStream_t)stream : g.stream;
  int64_t nh = batch->nhalo;
  std::vector<uint64_t> off(nh > 0 ? nh + 1 : 1, 0);
  if (nh > 0) {
    if (!batch->off) return fail(AHFGPU_ERR_INVALID, "off is NULL");
    CK(cudaMemcpyAsync(off.data(), batch->off, (nh + 1) * 8, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
  }
  ahfgpu_stats s{};
  Plan pl;
  if ((rc = validate_and_plan(params, off.data(), nh, pl))) return rc;
  s.ms_plan = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  rc = run_device(params, batch, pl, mode, st, &s);
  if (rc) return rc;
  s.ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  g.last_stats = s;
  fill_dres(dres);
  return AHFGPU_OK;
}

// Host inputs -> device on stream cs, part by part, issued by run_device
// between its launches (issue(p) right before the first launch of queue part
// p), so a part's kernels are queued as soon as its copies are.
// g.ev_part[p] is recorded once the particles of part p are in; issue(P)
// copies the ids (gidx), which only the final pack reads, and records
// g.ev_ids.  The particle ranges of parts 0..P-2 (merged where adjacent) go
// first; the last part is the gaps between them, so every particle crosses
// the link once.
struct Stager {
  using Range = std::pair<uint64_t, uint64_t>;
  struct Arr {
    DBuf* buf;
    const void* src;
    size_t esize, count;
    const void** dst;
  };
  const ahfgpu_batch* hb;
  ahfgpu_batch* db;
  const Plan& pl;
  cudaStream_t cs;
  uint64_t N = 0;
  int P = 1;
  Arr arr[12];
  std::vector<Range> taken;   // ranges of parts 0..P-2, sorted

  Stager(const ahfgpu_batch* hb_, ahfgpu_batch* db_, const Plan& pl_, cudaStream_t cs_)
      : hb(hb_), db(db_), pl(pl_), cs(cs_) {}

  int put(const Arr& a, uint64_t lo, uint64_t hi) {
    if (!a.src || hi <= lo) return AHFGPU_OK;
    cudaError_t e = cudaMemcpyAsync((char*)a.buf->p + lo * a.esize, (const char*)a.src + lo * a.esize,
                                    (hi - lo) * a.esize, cudaMemcpyHostToDevice, cs);
    if (e != cudaSuccess) return fail(AHFGPU_ERR_CUDA, "H2D copy failed: %s", cudaGetErrorString(e));
    return AHFGPU_OK;
  }

  int issue(int p) {
    const int64_t nh = hb->nhalo;
    int rc;
    if (p == 0) {
      *db = *hb;
      P = (int)pl.cuts.size() + 1;
      CK(cudaEventRecord(g.ev_cp0, cs));
      if (nh > 0 &&
          (!hb->x || !hb->y || !hb->z || !hb->vx || !hb->vy || !hb->vz || !hb->cx || !hb->cy || !hb->cz))
        return fail(AHFGPU_ERR_INVALID, "a required batch array is NULL");
      N = nh > 0 ? hb->off[nh] : 0;
      const Arr init[12] = {{&g.in_off, hb->off, 8, (size_t)nh + 1, (const void**)&db->off},
                            {&g.in_cx, hb->cx, 8, (size_t)nh, (const void**)&db->cx},
                            {&g.in_cy, hb->cy, 8, (size_t)nh, (const void**)&db->cy},
                            {&g.in_cz, hb->cz, 8, (size_t)nh, (const void**)&db->cz},
                            {&g.in_x, hb->x, 4, N, (const void**)&db->x},
                            {&g.in_y, hb->y, 4, N, (const void**)&db->y},
                            {&g.in_z, hb->z, 4, N, (const void**)&db->z},
                            {&g.in_vx, hb->vx, 4, N, (const void**)&db->vx},
                            {&g.in_vy, hb->vy, 4, N, (const void**)&db->vy},
                            {&g.in_vz, hb->vz, 4, N, (const void**)&db->vz},
                            {&g.in_w, hb->w, 4, N, (const void**)&db->w},
                            {&g.in_gidx, hb->gidx, 8, N, (const void**)&db->gidx}};
      for (int i = 0; i < 12; i++) {
        arr[i] = init[i];
        if (nh == 0 || !arr[i].src) { *arr[i].dst = nullptr; continue; }
        if ((rc = arr[i].buf->ensure(std::max<size_t>(arr[i].esize * arr[i].count, 8)))) return rc;
        *arr[i].dst = arr[i].buf->p;
      }
      if (nh > 0)
        for (int i = 0; i < 4; i++)
          if ((rc = put(arr[i], 0, arr[i].count))) return rc;
    }
    if (nh == 0) {
      CK(cudaEventRecord(p < P ? g.ev_part[p] : g.ev_ids, cs));
      return AHFGPU_OK;
    }
    if (p + 1 < P) {
      std::vector<Range> head;
      for (int q = part_begin(pl, p); q < part_end(pl, p); q++) {
        int32_t h = pl.queue[q];
        if (hb->off[h + 1] > hb->off[h]) head.push_back({hb->off[h], hb->off[h + 1]});
      }
      std::sort(head.begin(), head.end());
      std::vector<Range> merged;
      for (const Range& r : head) {
        if (!merged.empty() && merged.back().second == r.first) merged.back().second = r.second;
        else merged.push_back(r);
      }
      for (int i = 4; i < 11; i++)
        for (const Range& r : merged)
          if ((rc = put(arr[i], r.first, r.second))) return rc;
      CK(cudaEventRecord(g.ev_part[p], cs));
      taken.insert(taken.end(), merged.begin(), merged.end());
    } else if (p + 1 == P) {
      std::sort(taken.begin(), taken.end());
      for (int i = 4; i < 11; i++) {
        uint64_t at = 0;
        for (const Range& r : taken) {
          if ((rc = put(arr[i], at, r.first))) return rc;
          at = r.second;
        }
        if ((rc = put(arr[i], at, N))) return rc;
      }
      CK(cudaEventRecord(g.ev_part[p], cs));
    } else {
      if ((rc = put(arr[11], 0, N))) return rc;
      CK(cudaEventRecord(g.ev_ids, cs));
    }
    return AHFGPU_OK;
  }
};

// Result arrays live in page-locked host blocks (device-to-host copies run
// at link speed instead of through a bounce buffer).  A block handed out in
// a result comes back on ahfgpu_result_free and is kept for the next fetch.
struct HostBlock {
  void* p = nullptr;
  size_t cap = 0;
};
static HostBlock g_spare;                    // one cached block
static std::vector<HostBlock> g_lent;        // blocks held by results

static void* host_block_get(size_t bytes) {
  if (inject_oom("host_result")) return nullptr;
  if (g_spare.p && g_spare.cap >= bytes) {
    g_lent.push_back(g_spare);
    void* p = g_spare.p;
    g_spare = HostBlock{};
    return p;
  }
  if (g_spare.p) { cudaFreeHost(g_spare.p); g_spare = HostBlock{}; }
  void* p = nullptr;
  size_t cap = bytes + bytes / 8 + 4096;
  cudaError_t e = cudaMallocHost(&p, cap);
  if (getenv("AHFGPU_LOG"))
    fprintf(stderr, "ahfgpu: page-locked result block of %zu bytes: %s\n", cap, cudaGetErrorString(e));
  if (e != cudaSuccess) { cudaGetLastError(); return nullptr; }
  g_lent.push_back(HostBlock{p, cap});
  return p;
}

static void host_spare_release() {
  if (g_spare.p) cudaFreeHost(g_spare.p);
  g_spare = HostBlock{};
}

static bool host_block_put(void* p) {
  for (size_t i = 0; i < g_lent.size(); i++) {
    if (g_lent[i].p != p) continue;
    HostBlock b = g_lent[i];
    g_lent.erase(g_lent.begin() + (long)i);
    if (!g_spare.p) g_spare = b;
    else if (b.cap > g_spare.cap) { cudaFreeHost(g_spare.p); g_spare = b; }
    else cudaFreeHost(b.p);
    return true;
  }
  return false;
}

static int fetch_result_impl(ahfgpu_result* r) {
  int rc = ensure_init();
  if (rc) return rc;
  if (!r) return fail(AHFGPU_ERR_INVALID, "result is NULL");
  if (g.last_nhalo < 0) return fail(AHFGPU_ERR_STATE, "no device result to fetch");
  memset(r, 0, sizeof(*r));
  int64_t nh = g.last_nhalo;
  r->nhalo = nh;
  const size_t b_halo = ((size_t)std::max<int64_t>(nh, 1) * sizeof(ahfgpu_halo) + 255) & ~(size_t)255;
  const size_t b_off = ((size_t)(nh + 1) * 8 + 255) & ~(size_t)255;
  const size_t b_mem = ((size_t)std::max<uint64_t>(g.last_nkept, 1) * 8 + 255) & ~(size_t)255;
  const size_t b_prof = (size_t)std::max<uint64_t>(g.last_nbins, 1) * AHFGPU_PROF_NFIELDS * 8;
  char* blk = (char*)host_block_get(b_halo + 2 * b_off + b_mem + b_prof);
  if (blk) {
    r->halo = (ahfgpu_halo*)blk;
    r->member_off = (uint64_t*)(blk + b_halo);
    r->prof_off = (uint64_t*)(blk + b_halo + b_off);
    r->member = (uint64_t*)(blk + b_halo + 2 * b_off);
    r->prof = (double*)(blk + b_halo + 2 * b_off + b_mem);
  } else {
    const bool fail_all = inject_oom("host_result");
    r->halo = fail_all ? nullptr : (ahfgpu_halo*)malloc(b_halo);
    r->member_off = (uint64_t*)malloc(b_off);
    r->member = (uint64_t*)malloc(b_mem);
    r->prof_off = (uint64_t*)malloc(b_off);
    r->prof = (double*)malloc(b_prof);
    if (!r->halo || !r->member_off || !r->member || !r->prof_off || !r->prof) {
      ahfgpu_result_free(r);
      return fail(AHFGPU_ERR_OOM, "host allocation of the result failed");
    }
  }
  cudaStream_t st = g.stream;
  CK(cudaStreamSynchronize(0));
  auto t0 = std::chrono::steady_clock::now();
  if (nh > 0) CK(cudaMemcpyAsync(r->halo, g.halo.p, nh * sizeof(ahfgpu_halo), cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(r->member_off, g.member_off.p, (nh + 1) * 8, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(r->prof_off, g.prof_off.p, (nh + 1) * 8, cudaMemcpyDeviceToHost, st));
  if (g.last_nkept) CK(cudaMemcpyAsync(r->member, g.member.p, g.last_nkept * 8, cudaMemcpyDeviceToHost, st));
  if (g.last_nbins)
    CK(cudaMemcpyAsync(r->prof, g.prof.p, g.last_nbins * AHFGPU_PROF_NFIELDS * 8, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  g.last_stats.ms_d2h = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  r->stats = g.last_stats;
  return AHFGPU_OK;
}

// The gather's work queue: haloes by descending radius rounded to float,
// ties in index order (two stable counting passes over 16-bit digits of the
// float's bits, which order like the values for radii >= 0).  The order only
// balances the work (largest first); the lists do not depend on it.
static void gather_queue(const std::vector<double>& rad, int64_t nh, std::vector<int32_t>& queue) {
  std::vector<uint32_t> key((size_t)std::max<int64_t>(nh, 1));
  std::vector<int32_t> tmp((size_t)std::max<int64_t>(nh, 1));
  for (int64_t h = 0; h < nh; h++) {
    const float f = (float)rad[h];
    uint32_t b;
    memcpy(&b, &f, 4);
    key[h] = ~b;
    queue[h] = (int32_t)h;
  }
  std::vector<uint32_t> pos(65536);
  for (int shift = 0; shift < 32; shift += 16) {
    std::fill(pos.begin(), pos.end(), 0u);
    for (int64_t i = 0; i < nh; i++) pos[(key[queue[i]] >> shift) & 0xffffu]++;
    uint32_t run = 0;
    for (auto& p : pos) { const uint32_t c = p; p = run; run += c; }
    for (int64_t i = 0; i < nh; i++) tmp[pos[(key[queue[i]] >> shift) & 0xffffu]++] = queue[i];
    std::copy(tmp.begin(), tmp.begin() + nh, queue.begin());
  }
}

static int gather_device_impl(const ahfgpu_particles* parts, const ahfgpu_centres* cen, ahfgpu_batch* out,
                         void* stream) {
  int rc = ensure_init();
  if (rc) return rc;
  if (!parts || !cen || !out) return fail(AHFGPU_ERR_INVALID, "particles/centres/out is NULL");
  const uint64_t n = parts->n;
  const int64_t nh = cen->nhalo;
  if (nh < 0 || nh > 0x7fffffff) return fail(AHFGPU_ERR_INVALID, "nhalo %lld out of range", (long long)nh);
  if (n >= (1ull << 32)) return fail(AHFGPU_ERR_CAPACITY, "the gather takes fewer than 2^32 particles");
  if (n > 0 && (!parts->x || !parts->y || !parts->z || !parts->vx || !parts->vy || !parts->vz))
    return fail(AHFGPU_ERR_INVALID, "a particle array is NULL");
  if (nh > 0 && (!cen->cx || !cen->cy || !cen->cz || !cen->rad)) return fail(AHFGPU_ERR_INVALID, "a centre array is NULL");
  cudaStream_t st = stream ? (cudaStream_t)stream : g.stream;
  memset(out, 0, sizeof(*out));
  out->nhalo = nh;
  // radii on the host: the grid resolution and the queue (largest first)
  std::vector<double> rad((size_t)std::max<int64_t>(nh, 1));
  if (nh > 0) {
    CK(cudaMemcpyAsync(rad.data(), cen->rad, nh * 8, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
  }
  for (int64_t h = 0; h < nh; h++)
    if (!(rad[h] >= 0.0) || !(rad[h] <= 1.0)) return fail(AHFGPU_ERR_INVALID, "gather radius of halo %lld not in [0, 1]", (long long)h);
  std::vector<int32_t> queue((size_t)std::max<int64_t>(nh, 1));
  gather_queue(rad, nh, queue);
  double rmed = nh > 0 ? rad[queue[nh / 2]] : 0.5;
  // cells of about half the median radius, 8..256 per axis
  int G = rmed > 0 ? (int)std::min(256.0, std::max(8.0, std::floor(2.0 / rmed))) : 8;
  const uint64_t m = (uint64_t)G * G * G;
#define EN(buf, bytes) if ((rc = (buf).ensure(std::max<size_t>((size_t)(bytes), 8))) != AHFGPU_OK) return rc
  EN(g.ga_cell, n * 4);
  EN(g.ga_count, m * 4);
  EN(g.ga_fill, m * 4);
  EN(g.ga_start, (m + 1) * 4);
  EN(g.ga_sums, ((m + 2047) / 2048) * 4);
  EN(g.ga_sorted, n * 16);
  EN(g.ga_queue, nh * 4);
  EN(g.ga_qhead, 64);
  EN(g.ga_cnt, nh * 8);
  EN(g.ga_off, (nh + 1) * 8);
  EN(g.ga_hfill, nh * 8);
  EN(g.ga_err, 64);
  const int grid_p = std::max(1, std::min<int>(g.nsm * 8, (int)((n + 255) / 256)));
  const int grid_h = std::max(1, std::min<int>(g.nsm * 4, (int)std::max<int64_t>(nh, 1)));
  CK(cudaMemsetAsync(g.ga_count.p, 0, m * 4, st));
  CK(cudaMemsetAsync(g.ga_fill.p, 0, m * 4, st));
  CK(cudaMemsetAsync(g.ga_qhead.p, 0, 64, st));
  CK(cudaMemsetAsync(g.ga_err.p, 0, 64, st));
  if (nh > 0) {
    CK(cudaMemcpyAsync(g.ga_queue.p, queue.data(), nh * 4, cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(g.ga_hfill.p, 0, nh * 8, st));
    CK(cudaMemsetAsync(g.ga_cnt.p, 0, nh * 8, st));
  }
  if (n > 0) gather_cells(n, parts->x, parts->y, parts->z, G, g.ga_cell.as<uint32_t>(), g.ga_count.as<uint32_t>(), grid_p, st);
  gather_scan_u32(g.ga_count.as<uint32_t>(), g.ga_start.as<uint32_t>(), m, g.ga_sums.as<uint32_t>(), st);
  if (n > 0)
    gather_scatter(n, parts->x, parts->y, parts->z, g.ga_cell.as<uint32_t>(), g.ga_start.as<uint32_t>(),
                   g.ga_fill.as<uint32_t>(), g.ga_sorted.as<float4>(), grid_p, st);
  if (nh > 0)
    gather_halos(0, G, g.ga_start.as<uint32_t>(), g.ga_sorted.as<float4>(), nh, g.ga_queue.as<int32_t>(),
                 g.ga_qhead.as<unsigned int>(), cen->cx, cen->cy, cen->cz, cen->rad, g.ga_cnt.as<uint64_t>(), nullptr,
                 nullptr, nullptr, grid_h, st);
  gather_offsets(g.ga_cnt.as<uint64_t>(), nh, g.ga_off.as<uint64_t>(), st);
  CK(cudaGetLastError());
  std::vector<uint64_t> cnt((size_t)std::max<int64_t>(nh, 1), 0);
  if (nh > 0) CK(cudaMemcpyAsync(cnt.data(), g.ga_cnt.p, nh * 8, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  uint64_t ng = 0, maxn = 0;
  for (int64_t h = 0; h < nh; h++) { ng += cnt[h]; maxn = std::max(maxn, cnt[h]); }
  if (maxn >= (1ull << 32)) return fail(AHFGPU_ERR_CAPACITY, "a gathered list exceeds 2^32-1 particles");
  const int stack_cap = (int)std::min<uint64_t>(std::max<uint64_t>(maxn / 512 + 64, 64), 1u << 20);
  EN(g.ga_idx, ng * 8);
  EN(g.ga_idxA, ng * 4);
  EN(g.ga_keyB, ng * 8);
  EN(g.ga_idxB, ng * 4);
  EN(g.ga_stack, (size_t)grid_h * stack_cap * sizeof(uint4));
  EN(g.ga_x, ng * 4); EN(g.ga_y, ng * 4); EN(g.ga_z, ng * 4);
  EN(g.ga_vx, ng * 4); EN(g.ga_vy, ng * 4); EN(g.ga_vz, ng * 4);
  if (parts->w) EN(g.ga_w, ng * 4);
  EN(g.ga_id, ng * 8);
  EN(g.ga_fbq, nh * 4);
  EN(g.ga_fbn, 64);
  // window items of the lists that span several windows (lists whose items
  // do not fit take the radial sort)
  const uint64_t icap = (uint64_t)nh * 16 + 65536;
  EN(g.ga_items, icap * gather_item_bytes());
#undef EN
  if (nh > 0 && ng > 0) {
    CK(cudaMemsetAsync(g.ga_qhead.p, 0, 64, st));
    gather_halos(1, G, g.ga_start.as<uint32_t>(), g.ga_sorted.as<float4>(), nh, g.ga_queue.as<int32_t>(),
                 g.ga_qhead.as<unsigned int>(), cen->cx, cen->cy, cen->cz, cen->rad, g.ga_cnt.as<uint64_t>(),
                 g.ga_off.as<uint64_t>(), g.ga_hfill.as<unsigned long long>(), g.ga_idx.as<uint64_t>(), grid_h, st);
    // the lists in ascending index and packed.  Test hooks: AHFGPU_GATHER_BITMAP
    // "0" every list through the radial sort, "2" every window through the
    // bitmap, "3" every window that fits through the bitonic network;
    // AHFGPU_GATHER_WBITS a narrower window (a power of two, >= 32).
    int mode = 1, wshift = gather_window_shift_max();
    if (const char* e = getenv("AHFGPU_GATHER_BITMAP")) {
      const int v = atoi(e);
      mode = (v >= 0 && v <= 3) ? v : 1;
    }
    if (const char* e = getenv("AHFGPU_GATHER_WBITS")) {
      const long v = atol(e);
      int sh = 5;
      while (sh < wshift && (2l << sh) <= v) sh++;
      if (v >= 32) wshift = sh;
    }
    gather_order_pack(nh, g.ga_queue.as<int32_t>(), g.ga_qhead.as<unsigned int>(), g.ga_off.as<uint64_t>(),
                      g.ga_idx.as<uint64_t>(), g.ga_idxA.as<uint32_t>(), g.ga_keyB.as<uint64_t>(),
                      g.ga_idxB.as<uint32_t>(), g.ga_stack.as<uint4>(), stack_cap, wshift, mode, g.ga_items.p, icap,
                      g.ga_fbq.as<int32_t>(), g.ga_fbn.as<unsigned int>(), ng, parts->x, parts->y, parts->z,
                      parts->vx, parts->vy, parts->vz, parts->w, g.ga_x.as<float>(), g.ga_y.as<float>(),
                      g.ga_z.as<float>(), g.ga_vx.as<float>(), g.ga_vy.as<float>(), g.ga_vz.as<float>(),
                      parts->w ? g.ga_w.as<float>() : nullptr, g.ga_id.as<uint64_t>(), g.ga_err.as<int>(), grid_h,
                      std::max(1, std::min<int>(g.nsm * 8, (int)((ng + 255) / 256))), st);
  }
  CK(cudaGetLastError());
  int derr = 0;
  CK(cudaMemcpyAsync(&derr, g.ga_err.p, 4, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (derr == kErrWorklist) return fail(AHFGPU_ERR_CAPACITY, "gather sort worklist overflow");
  if (derr == kErrGatherDup) return fail(AHFGPU_ERR_CUDA, "gather: a list holds a particle twice (self-check)");
  if (derr) return fail(AHFGPU_ERR_CUDA, "gather: device error code %d", derr);
  out->off = g.ga_off.as<uint64_t>();
  out->x = g.ga_x.as<float>(); out->y = g.ga_y.as<float>(); out->z = g.ga_z.as<float>();
  out->vx = g.ga_vx.as<float>(); out->vy = g.ga_vy.as<float>(); out->vz = g.ga_vz.as<float>();
  out->w = parts->w ? g.ga_w.as<float>() : nullptr;
  out->gidx = g.ga_id.as<uint64_t>();
  out->cx = cen->cx; out->cy = cen->cy; out->cz = cen->cz;
  return AHFGPU_OK;
}

// The chunk plan shared by both writers: per output position j the chunks
// of its block (wb_chunk) and their exclusive scan (wb_coff), the written
// block count (wp_good), optionally the binary block bytes (wp_blk) and
// their scan (wp_boff).  Returns the chunk total in *nchunks.
static int writer_plan(const int64_t* order, int64_t minpart, bool bin_blocks, cudaStream_t st, uint64_t* nchunks,
                       uint64_t* bin_total) {
  const int64_t nh = g.last_nhalo;
  int rc;
  if ((rc = g.wp_blk.ensure(std::max<size_t>(nh * 8, 8)))) return rc;
  if ((rc = g.wp_boff.ensure((nh + 1) * 8))) return rc;
  if ((rc = g.wb_chunk.ensure(std::max<size_t>(nh * 8, 8)))) return rc;
  if ((rc = g.wb_coff.ensure((nh + 1) * 8))) return rc;
  if ((rc = g.wp_good.ensure(64))) return rc;
  if ((rc = g.wp_qhead.ensure(64))) return rc;
  CK(cudaMemsetAsync(g.wp_good.p, 0, 64, st));
  if (nh > 0)
    writer_sizes(nh, order, g.halo.as<ahfgpu_halo>(), minpart, bin_blocks ? g.wp_blk.as<uint64_t>() : nullptr,
                 g.wb_chunk.as<uint64_t>(), g.wp_good.as<unsigned long long>(),
                 std::max(1, std::min<int>(g.nsm * 4, (int)((nh + 255) / 256))), st);
  if (bin_blocks) writer_offsets(g.wp_blk.as<uint64_t>(), nh, g.wp_boff.as<uint64_t>(), st);
  writer_offsets(g.wb_chunk.as<uint64_t>(), nh, g.wb_coff.as<uint64_t>(), st);
  CK(cudaGetLastError());
  uint64_t tail[2] = {0, 0};
  CK(cudaMemcpyAsync(&tail[0], g.wb_coff.as<uint64_t>() + nh, 8, cudaMemcpyDeviceToHost, st));
  if (bin_blocks) CK(cudaMemcpyAsync(&tail[1], g.wp_boff.as<uint64_t>() + nh, 8, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (tail[0] >= (1ull << 31)) return fail(AHFGPU_ERR_CAPACITY, "writer: %llu chunks", (unsigned long long)tail[0]);
  *nchunks = tail[0];
  if (bin_total) *bin_total = tail[1];
  return AHFGPU_OK;
}

static int write_particles_device_impl(const uint64_t* ids, const float* w, const int64_t* order, int64_t minpart,
                                  const unsigned char** out, uint64_t* nbytes, void* stream) {
  int rc = ensure_init();
  if (rc) return rc;
  if (!out || !nbytes) return fail(AHFGPU_ERR_INVALID, "out/nbytes is NULL");
  if (g.last_nhalo < 0) return fail(AHFGPU_ERR_STATE, "no device result to write");
  const int64_t nh = g.last_nhalo;
  if (nh > 0 && (!ids || !order)) return fail(AHFGPU_ERR_INVALID, "ids/order is NULL");
  cudaStream_t st = stream ? (cudaStream_t)stream : g.stream;
  uint64_t nch = 0;
  if ((rc = writer_plan(order, minpart, false, st, &nch, nullptr))) return rc;
  if ((rc = g.wp_cbytes.ensure(std::max<uint64_t>(nch * 8, 8)))) return rc;
  if ((rc = g.wp_cboff.ensure((nch + 1) * 8))) return rc;
  const int grid = (int)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)g.nsm * 8, nch));
  CK(cudaMemsetAsync(g.wp_qhead.p, 0, 64, st));
  if (nch > 0)
    writer_count(nh, order, g.halo.as<ahfgpu_halo>(), g.member_off.as<uint64_t>(), g.member.as<uint64_t>(), ids, w,
                 g.wb_coff.as<uint64_t>(), g.wp_qhead.as<unsigned int>(), g.wp_cbytes.as<uint64_t>(), grid, st);
  writer_offsets(g.wp_cbytes.as<uint64_t>(), (int64_t)nch, g.wp_cboff.as<uint64_t>(), st);
  CK(cudaGetLastError());
  uint64_t body = 0;
  CK(cudaMemcpyAsync(&body, g.wp_cboff.as<uint64_t>() + nch, 8, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  const uint64_t total = 16 + body;
  if ((rc = g.wp_out.ensure(total))) return rc;
  CK(cudaMemsetAsync(g.wp_qhead.p, 0, 64, st));
  writer_write(nh, order, g.halo.as<ahfgpu_halo>(), g.member_off.as<uint64_t>(), g.member.as<uint64_t>(), ids, w,
               g.wb_coff.as<uint64_t>(), g.wp_qhead.as<unsigned int>(), g.wp_cboff.as<uint64_t>(),
               g.wp_good.as<unsigned long long>(), g.wp_out.as<unsigned char>(), grid, st);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(st));
  *out = g.wp_out.as<unsigned char>();
  *nbytes = total;
  return AHFGPU_OK;
}

static int write_particles_bin_device_impl(const uint64_t* ids, const int64_t* order, int64_t minpart,
                                      const unsigned char** out, uint64_t* nbytes, void* stream) {
  int rc = ensure_init();
  if (rc) return rc;
  if (!out || !nbytes) return fail(AHFGPU_ERR_INVALID, "out/nbytes is NULL");
  if (g.last_nhalo < 0) return fail(AHFGPU_ERR_STATE, "no device result to write");
  const int64_t nh = g.last_nhalo;
  if (nh > 0 && (!ids || !order)) return fail(AHFGPU_ERR_INVALID, "ids/order is NULL");
  cudaStream_t st = stream ? (cudaStream_t)stream : g.stream;
  uint64_t nch = 0, body = 0;
  if ((rc = writer_plan(order, minpart, true, st, &nch, &body))) return rc;
  const uint64_t total = 16 + body;
  if ((rc = g.wp_out.ensure(total))) return rc;
  const int grid = (int)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)g.nsm * 8, nch));
  CK(cudaMemsetAsync(g.wp_qhead.p, 0, 64, st));
  writer_bin_write(nh, order, g.halo.as<ahfgpu_halo>(), g.member_off.as<uint64_t>(), g.member.as<uint64_t>(), ids,
                   g.wp_boff.as<uint64_t>(), g.wb_coff.as<uint64_t>(), g.wp_good.as<unsigned long long>(),
                   g.wp_qhead.as<unsigned int>(), g.wp_out.as<uint32_t>(), grid, st);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(st));
  *out = g.wp_out.as<unsigned char>();
  *nbytes = total;
  return AHFGPU_OK;
}

static int sfc_sort_device_impl(uint64_t n, const float* x, const float* y, const float* z, int bits, uint64_t* keys,
                           uint64_t* order, void* stream) {
  int rc = ensure_init();
  if (rc) return rc;
  if (n == 0) return AHFGPU_OK;
  if (n >= (1ull << 31)) return fail(AHFGPU_ERR_CAPACITY, "sfc sort: %llu particles (limit 2^31 - 1)",
                                     (unsigned long long)n);
  if (bits < 1 || bits > 21) return fail(AHFGPU_ERR_INVALID, "sfc sort: bits %d outside 1..21", bits);
  if (!x || !y || !z || !keys || !order) return fail(AHFGPU_ERR_INVALID, "sfc sort: a pointer is NULL");
  cudaStream_t st = stream ? (cudaStream_t)stream : g.stream;
  const uint32_t nn = (uint32_t)n, nt = sfc_ntiles(nn), m = 256u * nt, nb = sfc_scan_blocks(m);
  if ((rc = g.sfc_kb.ensure(n * 8))) return rc;
  if ((rc = g.sfc_ia.ensure(n * 4))) return rc;
  if ((rc = g.sfc_ib.ensure(n * 4))) return rc;
  if ((rc = g.sfc_gh.ensure((size_t)m * 4))) return rc;
  if ((rc = g.sfc_goff.ensure((size_t)m * 4))) return rc;
  if ((rc = g.sfc_part.ensure((size_t)nb * 4))) return rc;
  if ((rc = g.sfc_err.ensure(64))) return rc;
  CK(cudaMemsetAsync(g.sfc_err.p, 0, 64, st));
  const int grid = (int)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)g.nsm * 8, (n + 255) / 256));
  sfc_keys(nn, x, y, z, bits, keys, g.sfc_ia.as<uint32_t>(), grid, st);
  uint64_t *kin = keys, *kout = g.sfc_kb.as<uint64_t>();
  uint32_t *iin = g.sfc_ia.as<uint32_t>(), *iout = g.sfc_ib.as<uint32_t>();
  for (int shift = 0; shift < 3 * bits; shift += 8) {
    sfc_pass(nn, kin, iin, shift, g.sfc_gh.as<uint32_t>(), g.sfc_goff.as<uint32_t>(), g.sfc_part.as<uint32_t>(),
             kout, iout, g.sfc_err.as<int>(), st);
    std::swap(kin, kout);
    std::swap(iin, iout);
  }
  if (kin != keys) CK(cudaMemcpyAsync(keys, kin, n * 8, cudaMemcpyDeviceToDevice, st));
  sfc_order(nn, iin, order, grid, st);
  CK(cudaGetLastError());
  int derr = 0;
  CK(cudaMemcpyAsync(&derr, g.sfc_err.p, 4, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (derr) return fail(AHFGPU_ERR_CUDA, "sfc sort: a scatter index left the array");
  return AHFGPU_OK;
}

// the particles of the domain grid's lists (ll, lltools.c): node of every
// particle (floor(l1 x) per axis, an index past l1 - 1 folded to node 0),
// list starts in g.am_start, and the particles by node with ascending index
// within a node (stable radix sort) in *key / *idx
static int amr_domain_lists(uint64_t n, const float* x, const float* y, const float* z, int l1, cudaStream_t st,
                            uint64_t** key, uint32_t** idx) {
  int rc;
  const uint64_t nn = (uint64_t)l1 * l1 * l1;
  const uint32_t n32 = (uint32_t)n, nt = sfc_ntiles(n32), m = 256u * nt, nb = sfc_scan_blocks(m);
  if ((rc = g.am_key.ensure(n * 8)) || (rc = g.am_keyb.ensure(n * 8)) || (rc = g.am_idx.ensure(n * 4)) ||
      (rc = g.am_idxb.ensure(n * 4)) || (rc = g.am_cnt.ensure(nn * 4)) || (rc = g.am_start.ensure((nn + 1) * 4)) ||
      (rc = g.am_sums.ensure(((nn + 2047) / 2048) * 4)) || (rc = g.am_gh.ensure((size_t)m * 4)) ||
      (rc = g.am_goff.ensure((size_t)m * 4)) || (rc = g.am_part.ensure((size_t)nb * 4)) ||
      (rc = g.am_err.ensure(64)) || (rc = g.am_seps.ensure(n * 96)))
    return rc;
  CK(cudaMemsetAsync(g.am_cnt.p, 0, nn * 4, st));
  CK(cudaMemsetAsync(g.am_err.p, 0, 64, st));
  const int grid = (int)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)g.nsm * 8, (n + 255) / 256));
  amr_cells(n32, x, y, z, l1, g.am_key.as<uint64_t>(), g.am_idx.as<uint32_t>(), g.am_cnt.as<uint32_t>(), grid, st);
  gather_scan_u32(g.am_cnt.as<uint32_t>(), g.am_start.as<uint32_t>(), nn, g.am_sums.as<uint32_t>(), st);
  int bits = 1;
  while ((1ull << bits) < nn) bits++;
  uint64_t *kin = g.am_key.as<uint64_t>(), *kout = g.am_keyb.as<uint64_t>();
  uint32_t *iin = g.am_idx.as<uint32_t>(), *iout = g.am_idxb.as<uint32_t>();
  for (int shift = 0; shift < bits; shift += 8) {
    sfc_pass(n32, kin, iin, shift, g.am_gh.as<uint32_t>(), g.am_goff.as<uint32_t>(), g.am_part.as<uint32_t>(), kout,
             iout, g.am_err.as<int>(), st);
    std::swap(kin, kout);
    std::swap(iin, iout);
  }
  *key = kin;
  *idx = iin;
  return AHFGPU_OK;
}

static int amr_domain_check(uint64_t n, int l1) {
  if (n == 0) return fail(AHFGPU_ERR_INVALID, "amr: no particles");
  if (n >= (1ull << 31)) return fail(AHFGPU_ERR_CAPACITY, "amr: %llu particles (limit 2^31 - 1)",
                                     (unsigned long long)n);
  if (l1 < 3 || l1 > 1024) return fail(AHFGPU_ERR_INVALID, "amr: domain grid %d outside 3..1024", l1);
  return AHFGPU_OK;
}

static int amr_domain_density_device_impl(uint64_t n, const float* x, const float* y, const float* z, int l1,
                                          float* dens, void* stream) {
  int rc = ensure_init();
  if (rc) return rc;
  if ((rc = amr_domain_check(n, l1))) return rc;
  if (!x || !y || !z || !dens) return fail(AHFGPU_ERR_INVALID, "amr: a pointer is NULL");
  cudaStream_t st = stream ? (cudaStream_t)stream : g.stream;
  uint64_t* kin;
  uint32_t* iin;
  if ((rc = amr_domain_lists(n, x, y, z, l1, st, &kin, &iin))) return rc;
  const int grid = (int)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)g.nsm * 8, (n + 255) / 256));
  if ((rc = g.am_cfold.ensure((size_t)l1 * 8 + 8))) return rc;
  amr_dens(l1, n, x, y, z, g.am_start.as<uint32_t>(), kin, iin, g.am_seps.as<double>(), g.am_cfold.as<double>(), dens,
           grid, st);
  CK(cudaGetLastError());
  int derr = 0;
  CK(cudaMemcpyAsync(&derr, g.am_err.p, 4, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (derr) return fail(AHFGPU_ERR_CUDA, "amr: a scatter index left the array");
  return AHFGPU_OK;
}

static int amr_first_refinement_device_impl(int l1, const float* dens, uint64_t n, double nth_dom, int32_t* zyx,
                                            int64_t max_nodes, int64_t* nnodes, void* stream) {
  int rc = ensure_init();
  if (rc) return rc;
  if (!nnodes || !dens) return fail(AHFGPU_ERR_INVALID, "amr: a pointer is NULL");
  *nnodes = 0;
  if (n == 0) return fail(AHFGPU_ERR_INVALID, "amr: no particles");
  if (l1 < 3 || l1 > 1024) return fail(AHFGPU_ERR_INVALID, "amr: domain grid %d outside 3..1024", l1);
  if (max_nodes < 0 || (max_nodes > 0 && !zyx)) return fail(AHFGPU_ERR_INVALID, "amr: bad output buffer");
  cudaStream_t st = stream ? (cudaStream_t)stream : g.stream;
  const uint64_t nn = (uint64_t)l1 * l1 * l1, nr = (uint64_t)l1 * l1;
  if ((rc = g.am_flag.ensure(nn)) || (rc = g.am_rowcnt.ensure(nr * 4)) || (rc = g.am_rowoff.ensure((nr + 1) * 4)) ||
      (rc = g.am_rsums.ensure(((nr + 2047) / 2048) * 4)) || (rc = g.am_err.ensure(64)))
    return rc;
  // critdens - mean_dens, as refine_grid.c:120 and generate_grids.c:82 form it
  const double dl1 = (double)l1;
  const double thr = nth_dom * ((dl1 * dl1 * dl1) / (double)n) - 1.0;
  CK(cudaMemsetAsync(g.am_err.p, 0, 64, st));
  amr_flags(l1, dens, thr, g.am_flag.as<uint8_t>(), g.am_rowcnt.as<uint32_t>(), st);
  gather_scan_u32(g.am_rowcnt.as<uint32_t>(), g.am_rowoff.as<uint32_t>(), nr, g.am_rsums.as<uint32_t>(), st);
  uint32_t covered = 0;
  CK(cudaMemcpyAsync(&covered, g.am_rowoff.as<uint32_t>() + nr, 4, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  const int64_t count = 8 * (int64_t)covered;
  if (count < 125) return AHFGPU_OK;   // MIN_NNODES: no fine grid
  *nnodes = count;
  if (count > max_nodes)
    return fail(AHFGPU_ERR_CAPACITY, "amr: the first refinement has %lld nodes, the buffer %lld", (long long)count,
                (long long)max_nodes);
  amr_emit(l1, g.am_flag.as<uint8_t>(), g.am_rowcnt.as<uint32_t>(), g.am_rowoff.as<uint32_t>(), max_nodes, zyx,
           g.am_err.as<int>(), st);
  CK(cudaGetLastError());
  int derr = 0;
  CK(cudaMemcpyAsync(&derr, g.am_err.p, 4, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (derr) return fail(AHFGPU_ERR_CUDA, "amr: a fine node left the output buffer");
  return AHFGPU_OK;
}

// ---------------------------------------------------------------------------
// the AMR hierarchy (gen_AMRhierarchy, src/libamr_serial/generate_grids.c:278,
// called from src/main.c:614-648): the domain grid as above, then, while the
// finest grid is below ngrid_max, refine it (threshold critdens - mean_dens,
// critdens = NperDomCell m2d on the domain grid and NperRefCell m2d below,
// m2d = ngrid_dom^3 / n times 8 per level), relink the particles and assign
// the refined grid's densities; a refined grid of fewer than MIN_NNODES =
// 125 nodes is dropped and ends the hierarchy.  The run tables and the state
// machines are in amr_tree.cu.

static AGrid agrid_of(const Ctx::AmrLevel& L) {
  AGrid a;
  a.l1 = L.l1; a.nP = L.nP; a.npl = L.npl; a.nC = L.nC; a.nR = L.nR; a.nN = L.nN; a.nn = L.nn;
  a.P = L.P.as<APRun>(); a.pl = L.pl.as<APlane>(); a.C = L.C.as<ACRun>(); a.R = L.R.as<ARow>();
  a.N = L.N.as<ANRun>(); a.key = L.key.as<uint64_t>(); a.nseg = L.nseg.as<int>();
  return a;
}

// exclusive scan of m counts, the total at out[m]
static int amr_scan(const uint32_t* in, uint32_t* out, uint64_t m, cudaStream_t st) {
  int rc;
  if (m == 0) {
    CK(cudaMemsetAsync(out, 0, 4, st));
    return AHFGPU_OK;
  }
  if ((rc = g.at_sums.ensure(((m + 2047) / 2048) * 4))) return rc;
  gather_scan_u32(in, out, m, g.at_sums.as<uint32_t>(), st);
  return AHFGPU_OK;
}

// stable radix sort of n (key, value) pairs on the low `bits` bits of the
// keys; the result is in (*k, *v), the other pair of buffers is scratch
static int amr_radix(uint32_t n, int bits, uint64_t** k, uint32_t** v, uint64_t** kb, uint32_t** vb,
                     cudaStream_t st) {
  int rc;
  if (n == 0) return AHFGPU_OK;
  const uint32_t nt = sfc_ntiles(n), m = 256u * nt, nb = sfc_scan_blocks(m);
  if ((rc = g.at_gh.ensure((size_t)m * 4)) || (rc = g.at_goff.ensure((size_t)m * 4)) ||
      (rc = g.at_part.ensure((size_t)nb * 4)))
    return rc;
  for (int shift = 0; shift < bits; shift += 8) {
    sfc_pass(n, *k, *v, shift, g.at_gh.as<uint32_t>(), g.at_goff.as<uint32_t>(), g.at_part.as<uint32_t>(), *kb, *vb,
             g.at_err.as<int>(), st);
    std::swap(*k, *kb);
    std::swap(*v, *vb);
  }
  return AHFGPU_OK;
}

static int amr_bits(uint64_t m) {
  int b = 1;
  while ((1ull << b) < m) b++;
  return b;
}

static int amr_hierarchy_device_impl(uint64_t n, const float* x, const float* y, const float* z, int ngrid_dom,
                                     int ngrid_max, double nth_dom, double nth_ref, int64_t* levels, int max_levels,
                                     int* ngrids, void* stream) {
  int rc = ensure_init();
  if (rc) return rc;
  if (!ngrids) return fail(AHFGPU_ERR_INVALID, "amr: ngrids is NULL");
  *ngrids = 0;
  g.amr_nlev = 0;
  if ((rc = amr_domain_check(n, ngrid_dom))) return rc;
  if (ngrid_max < ngrid_dom || ngrid_max > (1 << 20))
    return fail(AHFGPU_ERR_INVALID, "amr: ngrid_max %d outside %d..2^20", ngrid_max, ngrid_dom);
  if (!x || !y || !z) return fail(AHFGPU_ERR_INVALID, "amr: a pointer is NULL");
  if (max_levels < 0 || (max_levels > 0 && !levels)) return fail(AHFGPU_ERR_INVALID, "amr: bad levels buffer");
  cudaStream_t st = stream ? (cudaStream_t)stream : g.stream;
  const int L = ngrid_dom;
  const uint64_t nn0 = (uint64_t)L * L * L;
  if ((rc = g.at_err.ensure(64)) || (rc = g.at_tot.ensure(sizeof(AFineTotals)))) return rc;
  CK(cudaMemsetAsync(g.at_err.p, 0, 64, st));

  // the domain grid: lists, densities, run tables, TSC table
  uint64_t* kin;
  uint32_t* iin;
  if ((rc = amr_domain_lists(n, x, y, z, L, st, &kin, &iin))) return rc;
  Ctx::AmrLevel& d = g.amr_lv[0];
  if ((rc = d.P.ensure(sizeof(APRun))) || (rc = d.pl.ensure(sizeof(APlane) * L)) ||
      (rc = d.C.ensure(sizeof(ACRun) * L)) || (rc = d.R.ensure(sizeof(ARow) * (size_t)L * L)) ||
      (rc = d.N.ensure(sizeof(ANRun) * (size_t)L * L)) || (rc = d.key.ensure(nn0 * 8)) ||
      (rc = d.nseg.ensure(nn0 * 4)) || (rc = d.tsc.ensure(nn0 * 108)) || (rc = d.flag.ensure(nn0)) ||
      (rc = d.dens.ensure(nn0 * 4)) || (rc = d.start.ensure((nn0 + 1) * 4)) || (rc = d.ord.ensure(n * 4)) ||
      (rc = d.node.ensure(n * 8)))
    return rc;
  d.l1 = L; d.nP = 1; d.npl = L; d.nC = L; d.nR = L * L; d.nN = L * L; d.nn = (int)nn0; d.np = (uint32_t)n;
  const int pgrid = (int)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)g.nsm * 8, (n + 255) / 256));
  if ((rc = g.am_cfold.ensure((size_t)L * 8 + 8))) return rc;
  amr_dens(L, n, x, y, z, g.am_start.as<uint32_t>(), kin, iin, g.am_seps.as<double>(), g.am_cfold.as<double>(),
           d.dens.as<float>(), pgrid, st);
  CK(cudaMemcpyAsync(d.ord.p, iin, n * 4, cudaMemcpyDeviceToDevice, st));
  CK(cudaMemcpyAsync(d.node.p, kin, n * 8, cudaMemcpyDeviceToDevice, st));
  CK(cudaMemcpyAsync(d.start.p, g.am_start.p, (nn0 + 1) * 4, cudaMemcpyDeviceToDevice, st));
  ag_domain(L, d.P.as<APRun>(), d.pl.as<APlane>(), d.C.as<ACRun>(), d.R.as<ARow>(), d.N.as<ANRun>(),
            d.key.as<uint64_t>(), d.nseg.as<int>(), st);
  ag_tsc(agrid_of(d), d.tsc.as<int>(), d.flag.as<uint8_t>(), st);
  CK(cudaGetLastError());
  if (max_levels > 0) { levels[0] = L; levels[1] = (int64_t)nn0; levels[2] = (int64_t)n; }
  int ng = 1;
  const double dl = (double)L;
  double m2d = (dl * dl * dl) / (double)n;
  double thr = nth_dom * m2d - 1.0;

  while (ng < Ctx::kAmrMaxGrids) {
    Ctx::AmrLevel& c = g.amr_lv[ng - 1];
    Ctx::AmrLevel& f = g.amr_lv[ng];
    if (c.l1 >= ngrid_max) break;
    const AGrid gc = agrid_of(c);
    // refine: test_node, rows, planes, plane runs
    ag_test(c.nn, c.tsc.as<int>(), c.dens.as<float>(), thr, c.flag.as<uint8_t>(), st);
    const uint64_t runs_cap = (uint64_t)c.nn + 2ull * c.nN + 1;
    if ((rc = g.at_rrun.ensure((size_t)c.nR * 4 + 4)) || (rc = g.at_rnode.ensure((size_t)c.nR * 4 + 4)) ||
        (rc = g.at_rref.ensure((size_t)c.nR + 1)) || (rc = g.at_runoff.ensure(((size_t)c.nR + 1) * 4)) ||
        (rc = g.at_runs.ensure(runs_cap * 8)) || (rc = g.at_pref.ensure((size_t)c.npl + 1)) ||
        (rc = g.at_po.ensure(sizeof(APlaneOut) * ((size_t)c.npl + 1))) ||
        (rc = g.at_pnc.ensure((size_t)c.npl * 4 + 4)) || (rc = g.at_pnsel.ensure((size_t)c.npl * 4 + 4)) ||
        (rc = g.at_rroff.ensure(((size_t)c.npl + 1) * 4)) || (rc = g.at_seloff.ensure(((size_t)c.npl + 1) * 4)) ||
        (rc = g.at_rr.ensure(((size_t)c.nR + 1) * 8)) || (rc = g.at_sel.ensure(((size_t)c.nR + 1) * 4)) ||
        (rc = g.at_fpl.ensure(sizeof(AFPlane) * (2 * (size_t)c.npl + 2))) ||
        (rc = f.P.ensure(sizeof(APRun) * ((size_t)c.npl + 1))))
      return rc;
    ag_rows(gc, c.flag.as<uint8_t>(), g.at_rrun.as<uint32_t>(), g.at_rnode.as<uint32_t>(), g.at_rref.as<uint8_t>(), st);
    if ((rc = amr_scan(g.at_rrun.as<uint32_t>(), g.at_runoff.as<uint32_t>(), c.nR, st))) return rc;
    ag_rows_emit(gc, c.flag.as<uint8_t>(), g.at_runoff.as<uint32_t>(), g.at_runs.as<int2>(), st);
    ag_planes(gc, g.at_rref.as<uint8_t>(), g.at_rrun.as<uint32_t>(), g.at_rnode.as<uint32_t>(),
              g.at_pref.as<uint8_t>(), g.at_po.as<APlaneOut>(), g.at_pnc.as<uint32_t>(), g.at_pnsel.as<uint32_t>(), st);
    if ((rc = amr_scan(g.at_pnc.as<uint32_t>(), g.at_rroff.as<uint32_t>(), c.npl, st)) ||
        (rc = amr_scan(g.at_pnsel.as<uint32_t>(), g.at_seloff.as<uint32_t>(), c.npl, st)))
      return rc;
    ag_planes_emit(gc, g.at_rref.as<uint8_t>(), g.at_rrun.as<uint32_t>(), g.at_rnode.as<uint32_t>(),
                   g.at_rroff.as<uint32_t>(), g.at_seloff.as<uint32_t>(), g.at_rr.as<int2>(), g.at_sel.as<int>(), st);
    ag_pquad(gc, g.at_pref.as<uint8_t>(), g.at_po.as<APlaneOut>(), f.P.as<APRun>(), g.at_fpl.as<AFPlane>(),
             g.at_tot.as<AFineTotals>(), st);
    CK(cudaGetLastError());
    AFineTotals T;
    uint32_t nruns = 0;
    CK(cudaMemcpyAsync(&T, g.at_tot.p, sizeof T, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&nruns, g.at_runoff.as<uint32_t>() + c.nR, 4, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if ((uint64_t)nruns > runs_cap) return fail(AHFGPU_ERR_STATE, "amr: %u fine node runs past the bound", nruns);
    if (!T.refined) break;
    if (T.err) return fail(AHFGPU_ERR_CAPACITY, "amr: the refined grid of %d^3 exceeds 2^31 - 1 entries", 2 * c.l1);
    f.l1 = 2 * c.l1; f.nP = T.nP; f.npl = T.npl; f.nC = T.nC; f.nR = T.nR; f.nN = T.nN; f.nn = T.nn;
    const size_t fnn = (size_t)f.nn;
    if ((rc = f.pl.ensure(sizeof(APlane) * ((size_t)f.npl + 1))) || (rc = f.C.ensure(sizeof(ACRun) * ((size_t)f.nC + 1))) ||
        (rc = f.R.ensure(sizeof(ARow) * ((size_t)f.nR + 1))) || (rc = f.N.ensure(sizeof(ANRun) * ((size_t)f.nN + 1))) ||
        (rc = f.key.ensure(fnn * 8 + 8)) || (rc = f.nseg.ensure(fnn * 4 + 4)) || (rc = f.tsc.ensure(fnn * 108 + 108)) ||
        (rc = f.flag.ensure(fnn + 1)) || (rc = f.dens.ensure(fnn * 4 + 4)) || (rc = f.start.ensure((fnn + 1) * 4)))
      return rc;
    ag_fplanes(f.npl, g.at_fpl.as<AFPlane>(), g.at_rroff.as<uint32_t>(), g.at_seloff.as<uint32_t>(),
               g.at_po.as<APlaneOut>(), g.at_rr.as<int2>(), g.at_sel.as<int>(), gc, g.at_runoff.as<uint32_t>(),
               g.at_runs.as<int2>(), f.pl.as<APlane>(), f.C.as<ACRun>(), f.R.as<ARow>(), f.N.as<ANRun>(), st);
    ag_fnodes(f.nN, f.l1, f.N.as<ANRun>(), f.R.as<ARow>(), f.pl.as<APlane>(), f.key.as<uint64_t>(), f.nseg.as<int>(),
              st);
    ag_tsc(agrid_of(f), f.tsc.as<int>(), f.flag.as<uint8_t>(), st);

    // relink: the coarse grid's listed particles to the fine nodes
    const uint32_t npc = c.np;
    if ((rc = g.at_dest.ensure((size_t)npc * 4 + 4)) || (rc = g.at_moved.ensure((size_t)npc * 4 + 4)) ||
        (rc = g.at_moff.ensure(((size_t)npc + 1) * 4)) || (rc = g.at_cnt.ensure((fnn + 1) * 4)) ||
        (rc = g.at_kA.ensure((size_t)npc * 8 + 8)) || (rc = g.at_kB.ensure((size_t)npc * 8 + 8)) ||
        (rc = g.at_iA.ensure((size_t)npc * 4 + 4)) || (rc = g.at_iB.ensure((size_t)npc * 4 + 4)))
      return rc;
    CK(cudaMemsetAsync(g.at_cnt.p, 0, (fnn + 1) * 4, st));
    if ((rc = g.at_child.ensure((size_t)c.nn * 16 + 16)) || (rc = g.at_cen.ensure((size_t)f.l1 * 8 + 8)) ||
        (rc = g.at_cfold.ensure((size_t)f.l1 * 8 + 8)))
      return rc;
    ag_centres(f.l1, g.at_cen.as<double>(), g.at_cfold.as<double>(), st);
    CK(cudaMemsetAsync(g.at_child.p, 0xff, (size_t)c.nn * 16, st));   // i0 = -1: not refined
    ag_child0(agrid_of(f), c.key.as<uint64_t>(), c.nn, g.at_child.as<int4>(), st);
    ag_relink(npc, c.ord.as<uint32_t>(), c.node.as<uint64_t>(), c.key.as<uint64_t>(), c.l1, agrid_of(f),
              g.at_child.as<int4>(), g.at_cen.as<double>(), f.flag.as<uint8_t>(), x, y, z, g.at_dest.as<int>(),
              g.at_moved.as<uint32_t>(), st);
    if ((rc = amr_scan(g.at_moved.as<uint32_t>(), g.at_moff.as<uint32_t>(), npc, st))) return rc;
    ag_compact(npc, g.at_dest.as<int>(), g.at_moff.as<uint32_t>(), c.ord.as<uint32_t>(), g.at_kA.as<uint64_t>(),
               g.at_iA.as<uint32_t>(), g.at_cnt.as<uint32_t>(), st);
    if ((rc = amr_scan(g.at_cnt.as<uint32_t>(), f.start.as<uint32_t>(), fnn, st))) return rc;
    uint32_t nm = 0;
    CK(cudaMemcpyAsync(&nm, g.at_moff.as<uint32_t>() + npc, 4, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    uint64_t *k = g.at_kA.as<uint64_t>(), *kb = g.at_kB.as<uint64_t>();
    uint32_t *v = g.at_iA.as<uint32_t>(), *vb = g.at_iB.as<uint32_t>();
    if ((rc = amr_radix(nm, amr_bits(fnn), &k, &v, &kb, &vb, st))) return rc;
    if ((rc = f.ord.ensure((size_t)nm * 4 + 4)) || (rc = f.node.ensure((size_t)nm * 8 + 8))) return rc;
    if (nm) {
      CK(cudaMemcpyAsync(f.ord.p, v, (size_t)nm * 4, cudaMemcpyDeviceToDevice, st));
      CK(cudaMemcpyAsync(f.node.p, k, (size_t)nm * 8, cudaMemcpyDeviceToDevice, st));
    }
    f.np = nm;

    // densities: the one-sided (source, target) pairs per target, then the
    // gather
    const double m2f = m2d * 8.0;
    if ((rc = g.at_w.ensure((size_t)nm * 96 + 96)) || (rc = g.at_ne.ensure(fnn * 4 + 4)) ||
        (rc = g.at_srcoff.ensure((fnn + 1) * 4)) || (rc = g.at_tcnt.ensure(fnn * 4 + 4)))
      return rc;
    ag_weights(f.l1, m2f, nm, f.node.as<uint64_t>(), f.key.as<uint64_t>(), f.ord.as<uint32_t>(), x, y, z,
               g.at_cfold.as<double>(), g.at_w.as<double>(), st);
    CK(cudaMemsetAsync(g.at_ne.p, 0, fnn * 4 + 4, st));
    ag_extras(f.nn, f.start.as<uint32_t>(), f.tsc.as<int>(), 0, g.at_ne.as<uint32_t>(), nullptr, nullptr, nullptr,
              st);
    if ((rc = amr_scan(g.at_ne.as<uint32_t>(), g.at_srcoff.as<uint32_t>(), fnn, st))) return rc;
    uint32_t nextra = 0;
    CK(cudaMemcpyAsync(&nextra, g.at_srcoff.as<uint32_t>() + fnn, 4, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if ((rc = g.at_kB.ensure((size_t)nextra * 8 + 8))) return rc;
    if (nextra) {
      CK(cudaMemsetAsync(g.at_tcnt.p, 0, fnn * 4 + 4, st));
      ag_extras(f.nn, f.start.as<uint32_t>(), f.tsc.as<int>(), 1, nullptr, g.at_srcoff.as<uint32_t>(),
                g.at_tcnt.as<uint32_t>(), g.at_kB.as<uint64_t>(), st);
    }
    ag_dens(f.nn, f.tsc.as<int>(), g.at_srcoff.as<uint32_t>(), g.at_kB.as<uint64_t>(), f.start.as<uint32_t>(),
            g.at_w.as<double>(), nm, ng % 2 == 0, f.dens.as<float>(), g.at_err.as<int>() + 1, st);
    CK(cudaGetLastError());
    if (f.nn < 125) break;   // MIN_NNODES: the refined grid is dropped
    if (ng < max_levels) {
      levels[3 * ng] = f.l1;
      levels[3 * ng + 1] = f.nn;
      levels[3 * ng + 2] = nm;
    }
    ng++;
    m2d = m2f;
    thr = nth_ref * m2d - 1.0;
  }
  int derr[2] = {0, 0};
  CK(cudaMemcpyAsync(&derr[0], g.am_err.p, 4, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(&derr[1], g.at_err.p, 4, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (derr[0] || derr[1]) return fail(AHFGPU_ERR_CUDA, "amr: a scatter index left the array");
  CK(cudaMemcpyAsync(&derr[1], g.at_err.as<int>() + 1, 4, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (derr[1]) return fail(AHFGPU_ERR_STATE, "amr: a node with more than 27 TSC sources");
  *ngrids = ng;
  g.amr_nlev = ng;
  return AHFGPU_OK;
}

// grid `level` of the last hierarchy: node (z, y, x) and density
static int amr_grid_device_impl(int level, int32_t* zyx, float* dens, int64_t max_nodes, int64_t* nnodes,
                                void* stream) {
  int rc = ensure_init();
  if (rc) return rc;
  if (!nnodes) return fail(AHFGPU_ERR_INVALID, "amr: nnodes is NULL");
  *nnodes = 0;
  if (level < 0 || level >= g.amr_nlev)
    return fail(AHFGPU_ERR_INVALID, "amr: no grid %d in the last hierarchy (%d grids)", level, g.amr_nlev);
  const Ctx::AmrLevel& L = g.amr_lv[level];
  *nnodes = L.nn;
  if (max_nodes == 0) return AHFGPU_OK;
  if (max_nodes < 0 || (!zyx && !dens)) return fail(AHFGPU_ERR_INVALID, "amr: bad output buffer");
  if (L.nn > max_nodes)
    return fail(AHFGPU_ERR_CAPACITY, "amr: grid %d has %d nodes, the buffer %lld", level, L.nn, (long long)max_nodes);
  cudaStream_t st = stream ? (cudaStream_t)stream : g.stream;
  if (zyx) ag_zyx(L.nn, L.l1, L.key.as<uint64_t>(), zyx, st);
  if (dens && L.nn) CK(cudaMemcpyAsync(dens, L.dens.p, (size_t)L.nn * 4, cudaMemcpyDeviceToDevice, st));
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(st));
  return AHFGPU_OK;
}

static int gather_radii_device_impl(int64_t nh, const uint64_t* npart, const double* cx, const double* cy,
                               const double* cz, const double* rvir, double max_gather_rad_box, double* rad,
                               void* stream) {
  int rc = ensure_init();
  if (rc) return rc;
  if (nh < 0 || nh > 0x7fffffff) return fail(AHFGPU_ERR_INVALID, "nhalo %lld out of range", (long long)nh);
  if (nh == 0) return AHFGPU_OK;
  if (!npart || !cx || !cy || !cz || !rvir || !rad) return fail(AHFGPU_ERR_INVALID, "a gather-radius array is NULL");
  cudaStream_t st = stream ? (cudaStream_t)stream : g.stream;
  // counts, centres and R_vir to the host: the order by particle count
  // (largest first) and each halo's number of strictly larger haloes
  std::vector<uint64_t> np(nh);
  std::vector<double> h4((size_t)nh * 4);
  CK(cudaMemcpyAsync(np.data(), npart, nh * 8, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(h4.data(), cx, nh * 8, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(h4.data() + nh, cy, nh * 8, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(h4.data() + 2 * nh, cz, nh * 8, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(h4.data() + 3 * nh, rvir, nh * 8, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  std::vector<int32_t> ord(nh);
  std::iota(ord.begin(), ord.end(), 0);
  std::sort(ord.begin(), ord.end(), [&](int32_t a, int32_t b) { return np[a] > np[b] || (np[a] == np[b] && a < b); });
  std::vector<int64_t> lim(nh);
  std::vector<double> sp((size_t)nh * 4);
  for (int64_t s2 = 0; s2 < nh; s2++) {
    lim[s2] = (s2 > 0 && np[ord[s2]] == np[ord[s2 - 1]]) ? lim[s2 - 1] : s2;
    for (int k = 0; k < 4; k++) sp[(size_t)k * nh + s2] = h4[(size_t)k * nh + ord[s2]];
  }
  const double maxr = std::min(max_gather_rad_box, 0.25);
  if ((rc = g.gr_pos.ensure(nh * 32))) return rc;
  if ((rc = g.gr_lim.ensure(nh * 8))) return rc;
  if ((rc = g.gr_orig.ensure(nh * 4))) return rc;
  CK(cudaMemcpyAsync(g.gr_pos.p, sp.data(), nh * 32, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(g.gr_lim.p, lim.data(), nh * 8, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(g.gr_orig.p, ord.data(), nh * 4, cudaMemcpyHostToDevice, st));
  const double* d = g.gr_pos.as<double>();
  gather_radii(nh, d, d + nh, d + 2 * nh, g.gr_lim.as<int64_t>(), d + 3 * nh, g.gr_orig.as<int32_t>(), maxr, rad, st);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(st));
  return AHFGPU_OK;
}

static int construct_halos_impl(const ahfgpu_params* params, const ahfgpu_batch* batch, ahfgpu_result* result,
                           ahfgpu_mode mode) {
  int rc = ensure_init();
  if (rc) return rc;
  if (!batch || !result) return fail(AHFGPU_ERR_INVALID, "batch/result is NULL");
  memset(result, 0, sizeof(*result));
  auto t0 = std::chrono::steady_clock::now();
  cudaStream_t st = g.stream;
  Plan pl;
  if ((rc = validate_and_plan(params, batch->off, batch->nhalo, pl))) return rc;
  // FP32C on unit weights: the largest lists (one per class-2 CTA) start as
  // soon as their particles are in, while the rest of the batch crosses the
  // link.  (A weighted batch is checked as a whole before any launch.)
  if (mode == AHFGPU_BATCHED_FP32C && !batch->w && pl.N >= kSplitMinParticles) {
    // the class-2 lists in parts that double in size (the first 1/8 of one
    // list per class-2 CTA), then the small classes as the gaps between
    // them: the particles cross the link in the order the SMs take them
    const int n2 = pl.cls_begin[1];
    const int K = g.nsm * g.fp32c_bps[2];
    for (int c = std::max(1, K / 8); ; c *= 2) {
      const int cut = std::min(c, n2);
      if (cut > 0 && (pl.cuts.empty() || cut > pl.cuts.back())) pl.cuts.push_back(cut);
      if (cut >= n2 || (int)pl.cuts.size() + 1 >= kMaxParts) break;
    }
    if (!pl.cuts.empty() && pl.cuts.back() < n2 && (int)pl.cuts.size() + 1 < kMaxParts) pl.cuts.push_back(n2);
  }
  ahfgpu_batch db;
  Stager stager(batch, &db, pl, g.copy_stream);
  std::function<int(int)> stage = [&](int p) { return stager.issue(p); };
  ahfgpu_stats s{};
  s.ms_plan = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  rc = run_device(params, &db, pl, mode, st, &s, &stage);
  if (rc) return rc;
  g.last_stats = s;
  if ((rc = ahfgpu_fetch_result(result))) return rc;
  s.ms_d2h = g.last_stats.ms_d2h;
  s.ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  result->stats = s;
  g.last_stats = s;
  return AHFGPU_OK;
}

// the exported calls: each body above, inside the exception guard
int ahfgpu_init(int device) {
  return guarded([&] { return init_impl(device); });
}

int ahfgpu_construct_halos_device(const ahfgpu_params* params, const ahfgpu_batch* batch, ahfgpu_result* dres,
                                  ahfgpu_mode mode, void* stream) {
  return guarded([&] { return construct_halos_device_impl(params, batch, dres, mode, stream); });
}

int ahfgpu_fetch_result(ahfgpu_result* r) {
  return guarded([&] { return fetch_result_impl(r); });
}

int ahfgpu_gather_device(const ahfgpu_particles* parts, const ahfgpu_centres* cen, ahfgpu_batch* out,
                         void* stream) {
  return guarded([&] { return gather_device_impl(parts, cen, out, stream); });
}

int ahfgpu_write_particles_device(const uint64_t* ids, const float* w, const int64_t* order, int64_t minpart,
                                  const unsigned char** out, uint64_t* nbytes, void* stream) {
  return guarded([&] { return write_particles_device_impl(ids, w, order, minpart, out, nbytes, stream); });
}

int ahfgpu_write_particles_bin_device(const uint64_t* ids, const int64_t* order, int64_t minpart,
                                      const unsigned char** out, uint64_t* nbytes, void* stream) {
  return guarded([&] { return write_particles_bin_device_impl(ids, order, minpart, out, nbytes, stream); });
}

int ahfgpu_sfc_sort_device(uint64_t n, const float* x, const float* y, const float* z, int bits, uint64_t* keys,
                           uint64_t* order, void* stream) {
  return guarded([&] { return sfc_sort_device_impl(n, x, y, z, bits, keys, order, stream); });
}

int ahfgpu_gather_radii_device(int64_t nh, const uint64_t* npart, const double* cx, const double* cy,
                               const double* cz, const double* rvir, double max_gather_rad_box, double* rad,
                               void* stream) {
  return guarded([&] { return gather_radii_device_impl(nh, npart, cx, cy, cz, rvir, max_gather_rad_box, rad, stream); });
}

int ahfgpu_amr_domain_density_device(uint64_t n, const float* x, const float* y, const float* z, int l1,
                                     float* dens, void* stream) {
  return guarded([&] { return amr_domain_density_device_impl(n, x, y, z, l1, dens, stream); });
}

int ahfgpu_amr_first_refinement_device(int l1, const float* dens, uint64_t n, double nth_dom, int32_t* zyx,
                                       int64_t max_nodes, int64_t* nnodes, void* stream) {
  return guarded([&] { return amr_first_refinement_device_impl(l1, dens, n, nth_dom, zyx, max_nodes, nnodes, stream); });
}

int ahfgpu_amr_hierarchy_device(uint64_t n, const float* x, const float* y, const float* z, int ngrid_dom,
                                int ngrid_max, double nth_dom, double nth_ref, int64_t* levels, int max_levels,
                                int* ngrids, void* stream) {
  return guarded([&] {
    return amr_hierarchy_device_impl(n, x, y, z, ngrid_dom, ngrid_max, nth_dom, nth_ref, levels, max_levels, ngrids,
                                     stream);
  });
}

int ahfgpu_amr_grid_device(int level, int32_t* zyx, float* dens, int64_t max_nodes, int64_t* nnodes, void* stream) {
  return guarded([&] { return amr_grid_device_impl(level, zyx, dens, max_nodes, nnodes, stream); });
}

int ahfgpu_construct_halos(const ahfgpu_params* params, const ahfgpu_batch* batch, ahfgpu_result* result,
                           ahfgpu_mode mode) {
  return guarded([&] { return construct_halos_impl(params, batch, result, mode); });
}

void ahfgpu_result_free(ahfgpu_result* r) {
  if (!r) return;
  if (!(r->halo && host_block_put(r->halo))) {
    free(r->halo);
    free(r->member_off);
    free(r->member);
    free(r->prof_off);
    free(r->prof);
  }
  memset(r, 0, sizeof(*r));
}

int ahfgpu_last_error(char* buf, size_t len) {
  if (buf && len) {
    size_t n = std::min(len - 1, g_err.size());
    memcpy(buf, g_err.data(), n);
    buf[n] = 0;
  }
  return (int)g_err.size();
}

const char* ahfgpu_version(void) { return "ahfgpu 1.0 (sm_103a)"; }

int ahfgpu_tuning(char* buf, size_t len) {
  int rc = ensure_init();
  if (rc) return rc;
  char tmp[1024];
  snprintf(tmp, sizeof tmp,
           "{\"key\": \"%s\", \"source\": \"%s\", \"class_max\": [%llu, %llu], \"class_bps\": [%d, %d, %d], "
           "\"graph\": %s, \"graph_replays\": %llu}",
           g.tune_key.c_str(), g.tune_source.c_str(), (unsigned long long)g.tune_class_max[0],
           (unsigned long long)g.tune_class_max[1], g.fp32c_bps[0], g.fp32c_bps[1], g.fp32c_bps[2],
           g.use_graph ? "true" : "false", (unsigned long long)g.graph_replays);
  if (buf && len) {
    size_t n = std::min(len - 1, strlen(tmp));
    memcpy(buf, tmp, n);
    buf[n] = 0;
  }
  return AHFGPU_OK;
}

#ifdef AHFGPU_PHASE_TIMERS
// instrumented builds: per-phase SM cycles summed over the last call's CTAs
AHFGPU_API int ahfgpu_debug_halo_times(unsigned long long* out, long long nh) {
  if (!g.phase.p) return AHFGPU_ERR_STATE;
  cudaDeviceSynchronize();
  cudaMemcpy(out, g.phase.as<unsigned long long>() + kPhaseSlots, (size_t)nh * 4 * 8, cudaMemcpyDeviceToHost);
  return AHFGPU_OK;
}

AHFGPU_API int ahfgpu_debug_phase(unsigned long long* out, int reset) {
  if (!g.phase.p) return AHFGPU_ERR_STATE;
  cudaDeviceSynchronize();
  cudaMemcpy(out, g.phase.p, kPhaseSlots * 8, cudaMemcpyDeviceToHost);
  if (reset) cudaMemset(g.phase.p, 0, kPhaseSlots * 8);
  return AHFGPU_OK;
}
#endif

}  // extern "C"
