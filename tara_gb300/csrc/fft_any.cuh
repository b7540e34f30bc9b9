// Complex FFTs of lengths that are not powers of two (n = 2^a 3^b 5^c 7^d,
// even, up to kAnyMaxN), for the grids the reference accepts beyond the
// power-of-two kernels: a mixed-radix Stockham transform in shared memory,
// radix 4, 2, 3, 5 and 7 stages, one CTA per transform, FP64.
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

constexpr int kAnyMaxN = 3600;  // longest transform: the row pass holds four, 4 x 3600 x 16 B = 225 KB
constexpr int kAnyMaxStages = 16;

struct AnyPlan {
  int n;
  int stages;
  int radix[kAnyMaxStages];
};

// Factorisation n = 4^a 2^b 3^c 5^d 7^e (radix 4 first); false when n has another factor.
inline bool any_plan(int n, AnyPlan* p) {
  if (n < 2 || n > kAnyMaxN) return false;
  p->n = n;
  p->stages = 0;
  int m = n;
  const int order[5] = {4, 2, 3, 5, 7};
  for (int r : order)
    while (m % r == 0 && p->stages < kAnyMaxStages) {
      p->radix[p->stages++] = r;
      m /= r;
    }
  return m == 1;
}

// Sizes the mixed-radix path takes: even, 8 to kAnyMaxN, factors 2, 3, 5, 7 only.
inline bool any_size_ok(int n) {
  AnyPlan p;
  return n >= 8 && n % 2 == 0 && any_plan(n, &p);
}

__device__ __forceinline__ double2 cmul_any(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}

// One Stockham stage of radix R (compile-time: the R values stay in registers).
// The small DFTs are the standard butterflies; radix 3, 5 and 7 take their
// cosines and sines from the table roots W_R^m = W_n^(m n / R), read once per
// stage.  Radix 7 pairs the inputs m and R - m: with t_m = v_m + v_(R-m) and
// d_m = v_m - v_(R-m), V_k = a_k - i b_k and V_(R-k) = a_k + i b_k for
// a_k = v_0 + sum_m cos(2 pi m k / R) t_m and b_k = sum_m sin(2 pi m k / R) d_m.
template <int R>
__device__ __forceinline__ void any_stage(const double2* __restrict__ src, double2* __restrict__ dst, int n, int ns,
                                          const double2* __restrict__ w, bool inverse, int tid, int nthreads) {
  const int m = n / R;
  const int q = n / (ns * R);  // twiddle index step per unit of (j mod ns) and r
  double2 wr[R];
#pragma unroll
  for (int k = 0; k < R; ++k) {
    wr[k] = w[k * (n / R)];
    if (inverse) wr[k].y = -wr[k].y;
  }
  for (int j = tid; j < m; j += nthreads) {
    const int jm = j % ns, base = (j / ns) * ns * R + jm;
    const int tstep = jm * q;
    double2 v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      double2 x = src[j + r * m];
      if (r > 0 && tstep > 0) {
        double2 t = w[r * tstep];  // r * tstep < n
        if (inverse) t.y = -t.y;
        x = cmul_any(x, t);
      }
      v[r] = x;
    }
    double2 V[R];
    if constexpr (R == 2) {
      V[0] = make_double2(v[0].x + v[1].x, v[0].y + v[1].y);
      V[1] = make_double2(v[0].x - v[1].x, v[0].y - v[1].y);
    } else if constexpr (R == 4) {
      // W_4 = -i forward, +i inverse
      const double2 a = make_double2(v[0].x + v[2].x, v[0].y + v[2].y);
      const double2 b = make_double2(v[0].x - v[2].x, v[0].y - v[2].y);
      const double2 c = make_double2(v[1].x + v[3].x, v[1].y + v[3].y);
      const double2 d = make_double2(v[1].x - v[3].x, v[1].y - v[3].y);
      // -i d (forward) or +i d (inverse)
      const double2 e = inverse ? make_double2(-d.y, d.x) : make_double2(d.y, -d.x);
      V[0] = make_double2(a.x + c.x, a.y + c.y);
      V[1] = make_double2(b.x + e.x, b.y + e.y);
      V[2] = make_double2(a.x - c.x, a.y - c.y);
      V[3] = make_double2(b.x - e.x, b.y - e.y);
    } else if constexpr (R == 3) {
      // W_3 = c - i s (forward; the inverse table carries -s)
      const double c = wr[1].x, sn = -wr[1].y;
      const double2 t1 = make_double2(v[1].x + v[2].x, v[1].y + v[2].y);
      const double2 t2 = make_double2(v[1].x - v[2].x, v[1].y - v[2].y);
      const double2 a = make_double2(fma(c, t1.x, v[0].x), fma(c, t1.y, v[0].y));
      const double2 b = make_double2(sn * t2.x, sn * t2.y);  // V1 = a - i b, V2 = a + i b
      V[0] = make_double2(v[0].x + t1.x, v[0].y + t1.y);
      V[1] = make_double2(a.x + b.y, a.y - b.x);
      V[2] = make_double2(a.x - b.y, a.y + b.x);
    } else if constexpr (R == 7) {
      double2 t[3], d[3];
#pragma unroll
      for (int m = 1; m <= 3; ++m) {
        t[m - 1] = make_double2(v[m].x + v[7 - m].x, v[m].y + v[7 - m].y);
        d[m - 1] = make_double2(v[m].x - v[7 - m].x, v[m].y - v[7 - m].y);
      }
      V[0] = make_double2(v[0].x + t[0].x + t[1].x + t[2].x, v[0].y + t[0].y + t[1].y + t[2].y);
#pragma unroll
      for (int k = 1; k <= 3; ++k) {
        double2 a = v[0], b = make_double2(0.0, 0.0);
#pragma unroll
        for (int m = 1; m <= 3; ++m) {
          const double c = wr[(m * k) % 7].x, sn = -wr[(m * k) % 7].y;
          a = make_double2(fma(c, t[m - 1].x, a.x), fma(c, t[m - 1].y, a.y));
          b = make_double2(fma(sn, d[m - 1].x, b.x), fma(sn, d[m - 1].y, b.y));
        }
        V[k] = make_double2(a.x + b.y, a.y - b.x);      // a - i b
        V[7 - k] = make_double2(a.x - b.y, a.y + b.x);  // a + i b
      }
    } else {  // R == 5: W_5 = c1 - i s1, W_5^2 = c2 - i s2
      const double c1 = wr[1].x, s1 = -wr[1].y, c2 = wr[2].x, s2 = -wr[2].y;
      const double2 t1 = make_double2(v[1].x + v[4].x, v[1].y + v[4].y);
      const double2 t2 = make_double2(v[2].x + v[3].x, v[2].y + v[3].y);
      const double2 t3 = make_double2(v[1].x - v[4].x, v[1].y - v[4].y);
      const double2 t4 = make_double2(v[2].x - v[3].x, v[2].y - v[3].y);
      const double2 a1 = make_double2(fma(c2, t2.x, fma(c1, t1.x, v[0].x)), fma(c2, t2.y, fma(c1, t1.y, v[0].y)));
      const double2 a2 = make_double2(fma(c1, t2.x, fma(c2, t1.x, v[0].x)), fma(c1, t2.y, fma(c2, t1.y, v[0].y)));
      const double2 b1 = make_double2(fma(s2, t4.x, s1 * t3.x), fma(s2, t4.y, s1 * t3.y));
      const double2 b2 = make_double2(fma(-s1, t4.x, s2 * t3.x), fma(-s1, t4.y, s2 * t3.y));
      V[0] = make_double2(v[0].x + t1.x + t2.x, v[0].y + t1.y + t2.y);
      V[1] = make_double2(a1.x + b1.y, a1.y - b1.x);  // a1 - i b1
      V[4] = make_double2(a1.x - b1.y, a1.y + b1.x);  // a1 + i b1
      V[2] = make_double2(a2.x + b2.y, a2.y - b2.x);
      V[3] = make_double2(a2.x - b2.y, a2.y + b2.x);
    }
#pragma unroll
    for (int k = 0; k < R; ++k) dst[base + k * ns] = V[k];
  }
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
    const int R = pl.radix[st];
    switch (R) {
      case 4: any_stage<4>(src, dst, n, ns, w, inverse, tid, nthreads); break;
      case 2: any_stage<2>(src, dst, n, ns, w, inverse, tid, nthreads); break;
      case 3: any_stage<3>(src, dst, n, ns, w, inverse, tid, nthreads); break;
      case 5: any_stage<5>(src, dst, n, ns, w, inverse, tid, nthreads); break;
      default: any_stage<7>(src, dst, n, ns, w, inverse, tid, nthreads); break;
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
