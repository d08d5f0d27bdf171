// amr_tree.cuh -- the run tables of an AMR grid (as libamr_serial keeps a
// grid: plane runs, planes, row runs, rows, node runs, nodes) and the launch
// wrappers of amr_tree.cu.
#pragma once
#include <cstdint>
#include <cstring>

#include <cuda_runtime.h>

namespace ahfgpu {

// (double)(float)s: for s whose float rounding is a normal float below the
// largest binade, the double's significand rounded to 24 bits (to nearest,
// ties to even) by integer arithmetic -- the same value the conversion
// instructions give, without their FP64-pipe issue slots; every other s
// (zero, subnormal float results, the top binade, inf, NaN) through the
// conversions.  The TSC density sums round to float after every double
// addition, so this runs once per term.
// the bits of a double and back (host code too: the host checks of the
// summation rules compile these helpers)
__host__ __device__ __forceinline__ unsigned long long amr_bits(double d) {
#ifdef __CUDA_ARCH__
  return (unsigned long long)__double_as_longlong(d);
#else
  unsigned long long b;
  memcpy(&b, &d, 8);
  return b;
#endif
}

__host__ __device__ __forceinline__ double amr_from_bits(unsigned long long b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)b);
#else
  double d;
  memcpy(&d, &b, 8);
  return d;
#endif
}

__host__ __device__ __forceinline__ double amr_round_f32(double s) {
  const unsigned long long b = amr_bits(s);
  const unsigned e = (unsigned)(b >> 52) & 0x7ffu;
  if (e - 897u <= 252u) {   // biased exponent 897 .. 1149: float exponent 1 .. 253
    unsigned long long m = b & 0x7fffffffffffffffull;
    m += 0x0fffffffull + ((m >> 29) & 1ull);
    m &= ~0x1fffffffull;
    return amr_from_bits((b & 0x8000000000000000ull) | m);
  }
  return (double)(float)s;
}

struct APRun { int z0, len, pl0, pad; };
struct APlane { int z, pq, c0, nc; };
struct ACRun { int y0, len, r0, pl; };
struct __align__(16) ARow { int y, pl, cq, s0, ns, pad0, pad1, pad2; };
struct ANRun { int x0, len, n0, row; };

// a grid as the kernels read it (device pointers, host-side counts)
struct AGrid {
  int l1, nP, npl, nC, nR, nN, nn;
  const APRun* P;
  const APlane* pl;
  const ACRun* C;
  const ARow* R;
  const ANRun* N;
  const uint64_t* key;
  const int* nseg;
};

// per coarse plane, what its refined copy holds (the same for fine planes
// 2 z and 2 z + 1)
struct APlaneOut {
  uint32_t nc;     // fine row runs
  uint32_t nsel;   // coarse rows refined (two fine rows each)
  uint32_t nrun;   // fine node runs over one copy of the selected rows
  uint32_t nnode;  // fine nodes over one copy of the selected rows
};

// the fine grid's totals (written by k_ag_pquad, read by the host)
struct AFineTotals {
  int refined;           // ref_pquad's result: false, no fine grid
  int nP, npl, nC, nR, nN, nn;
  int err;               // a count overflowed int
};

// per fine plane: its coarse plane and where its rows, runs and nodes start
struct AFPlane {
  int z, cp, pq, c0, r0, s0, n0, pad;
};

void ag_domain(int l1, APRun* P, APlane* pl, ACRun* C, ARow* R, ANRun* N, uint64_t* key, int* nseg,
               cudaStream_t st);
void ag_tsc(const AGrid& g, int* tsc, uint8_t* flag, cudaStream_t st);
void ag_test(int nn, const int* tsc, const float* dens, double thr, uint8_t* flag, cudaStream_t st);
void ag_rows(const AGrid& g, const uint8_t* flag, uint32_t* nrun, uint32_t* nnode, uint8_t* rref, cudaStream_t st);
void ag_rows_emit(const AGrid& g, const uint8_t* flag, const uint32_t* run_off, int2* runs, cudaStream_t st);
void ag_planes(const AGrid& g, const uint8_t* rref, const uint32_t* rrun, const uint32_t* rnode, uint8_t* pref,
               APlaneOut* po, uint32_t* pnc, uint32_t* pnsel, cudaStream_t st);
void ag_planes_emit(const AGrid& g, const uint8_t* rref, const uint32_t* rrun, const uint32_t* rnode,
                    const uint32_t* rr_off, const uint32_t* sel_off, int2* rr, int* sel, cudaStream_t st);
void ag_pquad(const AGrid& g, const uint8_t* pref, const APlaneOut* po, APRun* fP, AFPlane* fpl, AFineTotals* tot,
              cudaStream_t st);
void ag_fplanes(int npl_f, const AFPlane* fpl, const uint32_t* rr_off, const uint32_t* sel_off, const APlaneOut* po,
                const int2* rr, const int* sel, const AGrid& gc, const uint32_t* run_off, const int2* runs,
                APlane* pl, ACRun* C, ARow* R, ANRun* N, cudaStream_t st);
void ag_fnodes(int nN, int l1, const ANRun* N, const ARow* R, const APlane* pl, uint64_t* key, int* nseg,
               cudaStream_t st);
void ag_child0(const AGrid& gf, const uint64_t* ckey, int nnc, int4* child, cudaStream_t st);
void ag_relink(uint32_t np, const uint32_t* ord, const uint64_t* cnode, const uint64_t* ckey, int l1c,
               const AGrid& gf, const int4* child, const double* cen, const uint8_t* fflag, const float* x,
               const float* y, const float* z, int* dest, uint32_t* moved, cudaStream_t st);
void ag_centres(int l1, double* cen, double* cfold, cudaStream_t st);
void ag_compact(uint32_t np, const int* dest, const uint32_t* off, const uint32_t* ord, uint64_t* fkey_out,
                uint32_t* fidx_out, uint32_t* count, cudaStream_t st);
void ag_weights(int l1, double m2d, uint32_t np, const uint64_t* node, const uint64_t* nkey, const uint32_t* ord,
                const float* x, const float* y, const float* z, const double* cfold, double* w, cudaStream_t st);
void ag_extras(int nn, const uint32_t* start, const int* tsc, int pass, uint32_t* ecount, const uint32_t* eoff,
               uint32_t* efill, uint64_t* extra, cudaStream_t st);
void ag_dens(int nn, const int* tsc, const uint32_t* eoff, const uint64_t* extra, const uint32_t* start,
             const double* w, uint32_t np, int desc, float* dens, int* err, cudaStream_t st);
void ag_zyx(int nn, int l1, const uint64_t* key, int32_t* zyx, cudaStream_t st);

}  // namespace ahfgpu
