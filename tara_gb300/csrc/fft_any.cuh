// Complex FFTs of lengths that are not powers of two (n = 2^a 3^b 5^c, even,
// up to kAnyMaxN), for the grids the reference accepts beyond the power-of-two
// kernels: a mixed-radix Stockham transform in shared memory, radix 4, 2, 3 and
// 5 stages, one CTA per transform, FP64.
//
// Stage with radix R over the current span Ns (the product of the radices
// already applied; Govindaraju et al., "High performance discrete Fourier
// transforms on graphics processors", SC 2008): for every j < n/R
//   v[r]   = src[j + r n/R] * W_n^(r (j mod Ns) n / (Ns R))        r < R
//   V      = DFT_R(v)
//   dst[(j / Ns) Ns R + (j mod Ns) + r Ns] = V[r]
// then Ns *= R; the result is in natural order after the last stage.  W_n^t is
// read from a table of the n roots exp(-2 pi i t / n) (conjugated for the
// inverse), so the small DFTs use the same table: W_R^m = W_n^(m n / R).
#pragma once
#include <cuda_runtime.h>

namespace tara {

constexpr int kAnyMaxN = 2048;  // longest transform (the row pass holds four of them)
constexpr int kAnyMaxStages = 16;

struct AnyPlan {
  int n;
  int stages;
  int radix[kAnyMaxStages];
};

// Factorisation n = 4^a 2^b 3^c 5^d (radix 4 first); false when n has another factor.
inline bool any_plan(int n, AnyPlan* p) {
  if (n < 2 || n > kAnyMaxN) return false;
  p->n = n;
  p->stages = 0;
  int m = n;
  const int order[4] = {4, 2, 3, 5};
  for (int r : order)
    while (m % r == 0 && p->stages < kAnyMaxStages) {
      p->radix[p->stages++] = r;
      m /= r;
    }
  return m == 1;
}

// Sizes the mixed-radix path takes: even, 8 to kAnyMaxN, factors 2, 3, 5 only.
inline bool any_size_ok(int n) {
  AnyPlan p;
  return n >= 8 && n % 2 == 0 && any_plan(n, &p);
}

__device__ __forceinline__ double2 cmul_any(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}

// In-place transform of buf[0, n) with scratch tmp[0, n) (both shared memory),
// by all `nthreads` threads of the CTA (tid < nthreads).  w: the n roots
// exp(-2 pi i t / n); inverse: their conjugates.  Ends with a barrier; the
// result is in buf.
__device__ inline void fft_any(double2* buf, double2* tmp, const AnyPlan& pl, const double2* __restrict__ w,
                               bool inverse, int tid, int nthreads) {
  const int n = pl.n;
  double2* src = buf;
  double2* dst = tmp;
  int ns = 1;
  for (int st = 0; st < pl.stages; ++st) {
    const int R = pl.radix[st], m = n / R;
    for (int j = tid; j < m; j += nthreads) {
      const int jm = j % ns, base = (j / ns) * ns * R + jm;
      const int tstep = jm * (n / (ns * R));  // twiddle index step per r
      double2 v[5];
      for (int r = 0; r < R; ++r) {
        double2 x = src[j + r * m];
        if (r > 0 && tstep > 0) {
          double2 t = w[(r * tstep) % n];
          if (inverse) t.y = -t.y;
          x = cmul_any(x, t);
        }
        v[r] = x;
      }
      // V[k] = sum_r v[r] W_R^(r k)
      const int q = n / R;
      for (int k = 0; k < R; ++k) {
        double2 acc = v[0];
        for (int r = 1; r < R; ++r) {
          double2 t = w[((r * k) % R) * q];
          if (inverse) t.y = -t.y;
          const double2 p = cmul_any(v[r], t);
          acc.x += p.x;
          acc.y += p.y;
        }
        dst[base + k * ns] = acc;
      }
    }
    __syncthreads();
    double2* s = src;
    src = dst;
    dst = s;
    ns *= R;
  }
  if (src != buf) {
    for (int i = tid; i < n; i += nthreads) buf[i] = src[i];
    __syncthreads();
  }
}

}  // namespace tara
