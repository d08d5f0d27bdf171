// noalloc.cu -- ahfgpu_construct_halos_noalloc: the batched FP64 stage with
// every byte of work space taken from one file-scope device array, for
// callers that must not allocate device memory.
//
// Who cannot allocate: an application that hands AHF's analysis a fixed
// device-memory budget and partitions the GPU's memory itself up front (a
// memory pool that the host owns), or a plugin loaded into a running
// simulation that may not call cudaMalloc/cudaFree behind its host's back.
// They pass device pointers for the inputs and the outputs; this entry point
// allocates nothing (no cudaMalloc/cudaFree, no allocating library call).
//
// Limits (compile-time): at most AHFGPU_NOALLOC_MAX_PARTICLES list entries
// and AHFGPU_NOALLOC_MAX_HALOS haloes per call, profile rows at a fixed
// AHFGPU_NOALLOC_MAX_BINS per halo.  The scratch array is about 16 MB and is
// held by every GPU that loads the library until the process exits.
//
// Set-up: the first call on a device (with that device current) looks up the
// array's device address with cudaGetSymbolAddress and fills its constant
// parts (identity work queue, profile row offsets).  That first call should
// come before any stream capture.  Every later call on the device reuses the
// array, which keeps the previous call's contents; the per-call counters,
// queue head, weight range and error word are cleared at the start of each
// call.  Calls that overlap on the GPU (different streams or host threads)
// share the array and race: serialise them.  Each call waits for its stream
// three times: it reads the entry count off[nhalo], the batch checks and the
// device error word back to the host.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>

#include <cuda_runtime.h>

#include "common.cuh"

namespace ahfgpu {
void launch_fp64(const DevParams& P, const DevBatch& B, const Work& W, int grid, int single, cudaStream_t st);
int fp64_max_blocks_per_sm();
void launch_concentration(ahfgpu_halo* halo, int64_t nh, int grid, cudaStream_t st);
}  // namespace ahfgpu

using namespace ahfgpu;

namespace {

constexpr uint64_t kNaN = AHFGPU_NOALLOC_MAX_PARTICLES;
constexpr int kNaH = AHFGPU_NOALLOC_MAX_HALOS;
constexpr int kNaCtas = 512;                          // persistent CTAs at most
constexpr int kNaStack = (int)(kNaN / 512 + 64);      // sort worklist per CTA

// byte offsets of the sub-arrays inside the scratch array (256-aligned)
constexpr size_t al(size_t x) { return (x + 255) & ~size_t(255); }
constexpr size_t oKeyA = 0;
constexpr size_t oKeyB = al(oKeyA + kNaN * 8);
constexpr size_t oIdxA = al(oKeyB + kNaN * 8);
constexpr size_t oIdxB = al(oIdxA + kNaN * 4);
constexpr size_t oSdx = al(oIdxB + kNaN * 4);
constexpr size_t oSdy = al(oSdx + kNaN * 8);
constexpr size_t oSdz = al(oSdy + kNaN * 8);
constexpr size_t oSd = al(oSdz + kNaN * 8);
constexpr size_t oSvx = al(oSd + kNaN * 8);
constexpr size_t oSvy = al(oSvx + kNaN * 4);
constexpr size_t oSvz = al(oSvy + kNaN * 4);
constexpr size_t oSw = al(oSvz + kNaN * 4);
constexpr size_t oSeid = al(oSw + kNaN * 4);
constexpr size_t oPhi = al(oSeid + kNaN * 4);
constexpr size_t oFlag = al(oPhi + kNaN * 8);
constexpr size_t oPa = al(oFlag + kNaN);
constexpr size_t oPb = al(oPa + kNaN * 8);
constexpr size_t oPc = al(oPb + kNaN * 8);
constexpr size_t oPd = al(oPc + kNaN * 8);
constexpr size_t oStack = al(oPd + kNaN * 8);
constexpr size_t oProfOff = al(oStack + (size_t)kNaCtas * kNaStack * 16);
constexpr size_t oQueue = al(oProfOff + (size_t)(kNaH + 1) * 8);
constexpr size_t oQhead = al(oQueue + (size_t)kNaH * 4);
constexpr size_t oCounters = al(oQhead + 64);
constexpr size_t oErr = al(oCounters + 64);
constexpr size_t oWred = al(oErr + 64);
constexpr size_t kNaBytes = al(oWred + 64);

// The scratch: one file-scope array.  Host code must not use its name as an
// address (it is a host-side stand-in); set-up fetches the device address.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNaBytes];

struct DevState {
  unsigned char* base = nullptr;   // device address of g_noalloc_scratch
  int nsm = 0, bps = 0;
};

std::mutex g_mu;
DevState g_dev[64];
thread_local char g_na_err[256];

int na_fail(int code, const char* msg) {
  strncpy(g_na_err, msg, sizeof g_na_err - 1);
  g_na_err[sizeof g_na_err - 1] = 0;
  return code;
}

__global__ void na_init_constants(int32_t* queue, uint64_t* prof_off) {
  for (int h = blockIdx.x * blockDim.x + threadIdx.x; h <= kNaH; h += gridDim.x * blockDim.x) {
    if (h < kNaH) queue[h] = h;
    prof_off[h] = (uint64_t)h * AHFGPU_NOALLOC_MAX_BINS;
  }
}

// batch checks on the device: offsets monotone from 0, weights positive and
// finite, the weight range and the largest list (exactness of FP64 mass
// prefixes)
__global__ void na_check(const uint64_t* off, int64_t nh, const float* w, uint64_t n, int* err, float* wred,
                         unsigned long long* maxn) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  unsigned long long longest = 0;
  for (int64_t h = t; h < nh; h += stride) {
    if (off[h + 1] < off[h]) atomicExch(&err[1], 1);
    else if (off[h + 1] - off[h] > longest) longest = off[h + 1] - off[h];
  }
  if (longest) atomicMax(maxn, longest);
  if (t == 0 && off[0] != 0) atomicExch(&err[1], 1);
  if (!w) return;
  float mn = INFINITY, mx = 0.f;
  int bad = 0;
  for (uint64_t i = (uint64_t)t; i < n; i += (uint64_t)stride) {
    float v = w[i];
    if (!(v > 0.f) || !isfinite(v)) bad = 1;
    else { mn = fminf(mn, v); mx = fmaxf(mx, v); }
  }
  atomicMin((int*)&wred[0], __float_as_int(mn));
  atomicMax((int*)&wred[1], __float_as_int(mx));
  if (bad) atomicExch(&err[2], 1);
}

__global__ void na_clear(int* err, unsigned* qhead, unsigned long long* counters, float* wred,
                         unsigned long long* maxn) {
  int t = threadIdx.x;
  if (t < 16) { err[t] = 0; qhead[t] = 0; }
  if (t < 8) counters[t] = 0;
  if (t == 0) { wred[0] = INFINITY; wred[1] = 0.f; *maxn = 0; }
}

// set-up of the current device (once): symbol address + constant parts
int na_setup(int dev, DevState** out) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (dev < 0 || dev >= 64) return na_fail(AHFGPU_ERR_NO_DEVICE, "device index out of range");
  DevState& s = g_dev[dev];
  if (!s.base) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      return na_fail(AHFGPU_ERR_CUDA, "cudaGetSymbolAddress of the scratch array failed");
    }
    int nsm = 0;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || nsm <= 0)
      return na_fail(AHFGPU_ERR_CUDA, "cannot query the SM count");
    unsigned char* b = (unsigned char*)p;
    na_init_constants<<<64, 256>>>((int32_t*)(b + oQueue), (uint64_t*)(b + oProfOff));
    if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess)
      return na_fail(AHFGPU_ERR_CUDA, "initialising the scratch array failed");
    s.nsm = nsm;
    s.bps = fp64_max_blocks_per_sm();
    if (s.bps < 1) s.bps = 1;
    s.base = b;
  }
  *out = &s;
  return AHFGPU_OK;
}

}  // namespace

extern "C" AHFGPU_API int ahfgpu_construct_halos_noalloc(const ahfgpu_params* prm, const ahfgpu_batch* db,
                                                         ahfgpu_halo* out_halo, uint64_t* out_member,
                                                         double* out_prof, void* stream) {
  g_na_err[0] = 0;
  if (!prm || !db || !out_halo || !out_member || !out_prof)
    return na_fail(AHFGPU_ERR_INVALID, "a required pointer is NULL");
  if (prm->MINPART < 4 || prm->MINPART > 128) return na_fail(AHFGPU_ERR_INVALID, "MINPART must be in [4, 128]");
  if (!(prm->VescTune > 0) || !(prm->rho_vir > 0) || !(prm->v_fac > 0))
    return na_fail(AHFGPU_ERR_INVALID, "non-positive VescTune, rho_vir or v_fac");
  const int64_t nh = db->nhalo;
  if (nh < 0) return na_fail(AHFGPU_ERR_INVALID, "nhalo < 0");
  if (nh > kNaH) return na_fail(AHFGPU_ERR_CAPACITY, "nhalo exceeds AHFGPU_NOALLOC_MAX_HALOS");
  if (nh == 0) return AHFGPU_OK;
  if (!db->off || !db->x || !db->y || !db->z || !db->vx || !db->vy || !db->vz || !db->cx || !db->cy || !db->cz)
    return na_fail(AHFGPU_ERR_INVALID, "a required batch array is NULL");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return na_fail(AHFGPU_ERR_NO_DEVICE, "no current CUDA device");
  DevState* s = nullptr;
  int rc = na_setup(dev, &s);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  unsigned char* b = s->base;
  int* err = (int*)(b + oErr);
  float* wred = (float*)(b + oWred);
  unsigned* qhead = (unsigned*)(b + oQhead);
  unsigned long long* counters = (unsigned long long*)(b + oCounters);
  unsigned long long* maxn = (unsigned long long*)(b + oWred + 8);
  // entry count, then the batch checks
  uint64_t N = 0;
  if (cudaMemcpyAsync(&N, db->off + nh, 8, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return na_fail(AHFGPU_ERR_CUDA, "reading off[nhalo] failed");
  if (N > kNaN) return na_fail(AHFGPU_ERR_CAPACITY, "off[nhalo] exceeds AHFGPU_NOALLOC_MAX_PARTICLES");
  na_clear<<<1, 32, 0, st>>>(err, qhead, counters, wred, maxn);
  na_check<<<s->nsm, 256, 0, st>>>(db->off, nh, db->w, N, err, wred, maxn);
  int herr[3] = {0, 0, 0};
  float hw[2] = {0.f, 0.f};
  unsigned long long hmaxn = 0;
  if (cudaMemcpyAsync(herr, err, 12, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaMemcpyAsync(hw, wred, 8, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaMemcpyAsync(&hmaxn, maxn, 8, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return na_fail(AHFGPU_ERR_CUDA, "batch check failed");
  if (herr[1]) return na_fail(AHFGPU_ERR_INVALID, "off must start at 0 and be monotone");
  if (herr[2]) return na_fail(AHFGPU_ERR_INVALID, "weights must be positive and finite");

  DevParams P{};
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
  if (db->w) {
    // FP64 mass prefixes are exact when every partial sum of the longest
    // list stays below 2^52 quanta of the lightest weight; otherwise every
    // halo is replayed serially in the reference's order
    double q = ldexp(1.0, ilogb((double)hw[0]) - 23);
    if (!((double)hmaxn * (double)hw[1] / q < 4503599627370496.0)) P.force_serial = 1;
  }
  DevBatch B{};
  B.nhalo = nh;
  B.off = db->off;
  B.x = db->x; B.y = db->y; B.z = db->z;
  B.vx = db->vx; B.vy = db->vy; B.vz = db->vz;
  B.w = db->w;
  B.gidx = db->gidx;
  B.cx = db->cx; B.cy = db->cy; B.cz = db->cz;
  Work W{};
  W.keyA = (uint64_t*)(b + oKeyA); W.keyB = (uint64_t*)(b + oKeyB);
  W.idxA = (uint32_t*)(b + oIdxA); W.idxB = (uint32_t*)(b + oIdxB);
  W.sdx = (double*)(b + oSdx); W.sdy = (double*)(b + oSdy); W.sdz = (double*)(b + oSdz); W.sd = (double*)(b + oSd);
  W.svx = (float*)(b + oSvx); W.svy = (float*)(b + oSvy); W.svz = (float*)(b + oSvz); W.sw = (float*)(b + oSw);
  W.seid = (uint32_t*)(b + oSeid);
  W.phi = (double*)(b + oPhi);
  W.flag = (uint8_t*)(b + oFlag);
  W.prof_a = (double*)(b + oPa); W.prof_b = (double*)(b + oPb);
  W.prof_c = (double*)(b + oPc); W.prof_d = (double*)(b + oPd);
  W.sort_stack = (uint4*)(b + oStack);
  W.stack_cap = kNaStack;
  W.halo = out_halo;
  W.mem_stage = out_member;
  W.prof_stage = out_prof;
  W.prof_cap_off = (const uint64_t*)(b + oProfOff);
  W.queue_head = qhead;
  W.queue = (const int32_t*)(b + oQueue);
  W.nqueue = (int)nh;
  W.counters = counters;
  W.err = err;
  int grid = s->nsm * s->bps;
  if (grid > kNaCtas) grid = kNaCtas;
  if (grid > nh) grid = (int)nh;
  launch_fp64(P, B, W, grid, -1, st);
  launch_concentration(out_halo, nh, (int)((nh + 127) / 128), st);
  if (cudaGetLastError() != cudaSuccess) return na_fail(AHFGPU_ERR_CUDA, "kernel launch failed");
  int derr = 0;
  if (cudaMemcpyAsync(&derr, err, 4, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return na_fail(AHFGPU_ERR_CUDA, "device error after the halo kernel");
  if (derr == kErrWorklist) return na_fail(AHFGPU_ERR_CAPACITY, "radial sort worklist overflow");
  if (derr == kErrSortState) return na_fail(AHFGPU_ERR_CUDA, "radial sort: inconsistent bucket run (self-check)");
  if (derr) {
    char msg[64];
    snprintf(msg, sizeof msg, "device error code %d", derr);
    return na_fail(AHFGPU_ERR_CUDA, msg);
  }
  return AHFGPU_OK;
}

extern "C" AHFGPU_API int ahfgpu_noalloc_last_error(char* buf, size_t len) {
  size_t n = strlen(g_na_err);
  if (buf && len) {
    size_t k = n < len - 1 ? n : len - 1;
    memcpy(buf, g_na_err, k);
    buf[k] = 0;
  }
  return (int)n;
}
