// shard.cu -- the halo split across GPUs (host code only).
//
// Haloes are independent in the stage (src/libahf/ahf_halos.c:504-510 runs
// them in any order under OpenMP's dynamic schedule), so a snapshot's batch
// is split by halo with no data-path collective: longest-processing-time
// first on the estimated cost n log2(n + 2) -- haloes by decreasing cost
// (ties: lower halo index first), each to the rank with the smallest load so
// far (ties: lower rank).  Each rank then calls the stage on its haloes and
// the caller puts the per-halo results back in batch order.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <numeric>
#include <queue>
#include <vector>

#include "../../include/ahfgpu.h"

extern "C" AHFGPU_API int ahfgpu_shard_halos(int64_t nhalo, const uint64_t* off, int32_t nranks,
                                             int32_t* rank_of_halo) {
  if (nhalo < 0 || nranks < 1 || (nhalo > 0 && (!off || !rank_of_halo))) return AHFGPU_ERR_INVALID;
  if (nhalo == 0) return AHFGPU_OK;
  std::vector<double> cost((size_t)nhalo);
  for (int64_t h = 0; h < nhalo; ++h) {
    if (off[h + 1] < off[h]) return AHFGPU_ERR_INVALID;
    double n = (double)(off[h + 1] - off[h]);
    cost[(size_t)h] = n * std::log2(n + 2.0);
  }
  std::vector<int64_t> order((size_t)nhalo);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(),
                   [&](int64_t a, int64_t b) { return cost[(size_t)a] > cost[(size_t)b]; });
  using Load = std::pair<double, int32_t>;   // (load, rank): smallest load, then lowest rank
  std::priority_queue<Load, std::vector<Load>, std::greater<Load>> heap;
  for (int32_t r = 0; r < nranks; ++r) heap.push({0.0, r});
  for (int64_t h : order) {
    Load l = heap.top();
    heap.pop();
    rank_of_halo[h] = l.second;
    heap.push({l.first + cost[(size_t)h], l.second});
  }
  return AHFGPU_OK;
}
