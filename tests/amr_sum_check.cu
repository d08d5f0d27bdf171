// Host check of the summation rules of ahf_gb300/csrc/amr_sum.cuh: the
// windowed float sum (two-state maps per term, composed across a window, the
// exact step where a result would leave the accumulator's binade) against
// the reference's sequential acc <- (float)((double)acc + t), on seeded
// random term sequences with exact ties, zero terms, float-representable
// terms and binade crossings (from -1 through zero upward).  The window loop
// below is the warp loop of amr_warp_sum written for one host thread (the
// scan across lanes as a running composition); the per-term map, the
// composition and the exact step are the library's own functions.
// Prints "mismatches N terms T exact E".
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <random>
#include <vector>

#include "amr_sum.cuh"

using namespace ahfgpu;

static double chain(double acc, const double* t, int n) {
  for (int i = 0; i < n; i++) acc = (double)(float)(acc + t[i]);
  return acc;
}

static double windowed(double acc, const double* t, int n, int W, long* exact) {
  int i = 0;
  while (i < n) {
    float af = (float)acc;
    uint32_t fb;
    memcpy(&fb, &af, 4);
    const int E = (int)((fb >> 23) & 0xffu);
    if (E == 0 || E >= 254) {
      acc = amr_round_f32(acc + t[i]);
      i++;
      (*exact)++;
      continue;
    }
    const int ef = E - 127;
    const bool neg = (fb >> 31) != 0u;
    const int A = (int)((fb & 0x7fffffu) | 0x800000u);
    const int m = n - i < W ? n - i : W;
    AmrTr pre;
    int j = -1, Alast = A;
    for (int k = 0; k < m; k++) {
      const AmrTr T = amr_term_map(t[i + k], ef);
      pre = k == 0 ? T : amr_compose(pre, T);
      const int R = (A & 1) ? pre.r1 : pre.r0;
      const int Ak = neg ? A - R : A + R;
      if (neg ? Ak <= (1 << 23) : Ak >= (1 << 24)) {
        j = k;
        break;
      }
      Alast = Ak;
    }
    const double u = amr_from_bits((unsigned long long)(ef - 23 + 1023) << 52);
    acc = (neg ? -(double)Alast : (double)Alast) * u;
    if (j < 0) {
      i += m;
    } else {
      acc = amr_round_f32(acc + t[i + j]);
      (*exact)++;
      i += j + 1;
    }
  }
  return acc;
}

int main() {
  std::mt19937_64 rng(20261204);
  long bad = 0, terms = 0, exact = 0;
  for (int trial = 0; trial < 1500; trial++) {
    const int n = 1 + (int)(rng() % 2500);
    std::vector<double> t(n);
    const int sh = (int)(rng() % 30);
    for (int i = 0; i < n; i++) {
      const int kind = (int)(rng() % 10);
      double v = (double)(rng() >> 11) / 9007199254740992.0;
      for (int k = 0; k < sh; k++) v *= 0.5;
      if (kind == 0) v = 0.0;
      if (kind == 1) {   // a short mantissa: ties at the float and the double grid
        v = (double)(rng() % 64);
        for (int k = (int)(rng() % 60); k > 0; k--) v *= 0.5;
      }
      if (kind == 2) v = (double)(float)v;
      t[i] = v;
    }
    const double starts[3] = {-1.0, 0.0, (double)(float)(7.3e-3 * (1 + (int)(rng() % 5)))};
    const double a0 = starts[trial % 3];
    const double want = chain(a0, t.data(), n);
    for (int W : {1, 7, 32}) {
      const double got = windowed(a0, t.data(), n, W, &exact);
      terms += n;
      if (memcmp(&want, &got, 8) != 0) bad++;
    }
  }
  printf("mismatches %ld terms %ld exact %ld\n", bad, terms, exact);
  return bad != 0;
}
