// Shared-memory Stockham FFT building blocks for sm_103a.
//
// One "slot" is a length-N complex vector in shared memory, transformed by a
// group of G = N/16 threads (16 elements per thread: four radix-4 butterflies
// per stage, or, for odd log2 N, eight radix-2 butterflies in a final stage
// (FP32, double-float) or two 8-point DFTs in a first stage (FP64)).  Every
// thread of the CTA calls the same transform so that the stage barriers line
// up; `active` masks threads whose slot holds nothing.
//
// Stockham autosort form (Govindaraju et al., SC'08): at a stage with
// sub-transform length Ns and radix R, butterfly j reads in[j + r*N/R],
// multiplies input r by W^(r*k*N/(R*Ns)) with k = j mod Ns, and writes the R
// outputs to out[(j-k)*R + k + r*Ns].  Results come out in natural order, so no
// bit reversal is needed.  Reads and writes of a stage touch different slots,
// so each thread stages its inputs in registers between two barriers and the
// transform runs in place.
//
// Arithmetic: the twiddled radix-4 butterfly is written with the two-sided FMA
// form a = v0 + w*v2, b = 2*v0 - a, which costs 3 FMA-pipe instructions per
// output pair component instead of a separate multiply and two adds; a full
// twiddled radix-4 butterfly is 24 instructions for 4 points over 2 stages.
// The FP64 radix-4 path goes further with twiddles factored as w = c (1 + i tau)
// (Goedecker, "Fast radix 2, 3, 4, and 5 kernels for fast Fourier
// transformations on computers with overlapping multiply-add instructions",
// SIAM J. Sci. Comput. 18, 1997): 22 FMAs per butterfly (dft4_tw_ratio).  The
// first stage has unit twiddles and uses 16 adds.
#pragma once
#include <cuda_runtime.h>
#include <type_traits>

namespace tara {

template <typename T> struct cplx_of;
template <> struct cplx_of<double> { typedef double2 type; };
template <> struct cplx_of<float> { typedef float2 type; };
}  // namespace tara

#include "df64.cuh"

namespace tara {
template <> struct cplx_of<df64> { typedef df64c type; };

template <typename T>
__device__ __forceinline__ typename cplx_of<T>::type mkc(T x, T y) {
  typename cplx_of<T>::type c;
  c.x = x;
  c.y = y;
  return c;
}

__host__ __device__ constexpr int ilog2c(int n) { return n <= 1 ? 0 : 1 + ilog2c(n >> 1); }

// threads per transform of length N
__host__ __device__ constexpr int fft_group(int n) { return n >= 16 ? n / 16 : 1; }

// Twiddle table of a length-n transform (LG = log2 n, LG/2 radix-4 stages):
//   [0, n)           W^m = exp(-2 pi i m/n), with tw[n - m] = conj(tw[m]) exactly
//   [n, n + S)       forward stage tables
//   [n + S, n + 2S)  inverse stage tables (the same, conjugated), S = 4^(LG/2) - 4
// The twiddled radix-4 stage s (Ns = 4^s, 1 <= s < LG/2) owns entries
// [Ns - 4, 4 Ns - 4) of each direction's stage tables: W^(r k n/(4 Ns)) at
// [(r - 1) Ns + k] for r = 1, 2, 3 and k < Ns, so the lanes of a warp (consecutive
// k) read consecutive entries.  In the FP64 table these stage entries hold the
// ratio form of dft4_tw_ratio instead: (tau1, c1), (tau2, c2), (tau3, c3 / c1).
__host__ __device__ constexpr int tw_stage_span(int n) { return (1 << (2 * (ilog2c(n) / 2))) - 4; }

// Radix-8 path (the autotuner's alternative to the radix-4 one): radix-8
// stages first, then zero, one or two radix-4 stages -- 2048 = 8^3 * 4 runs
// four passes through shared memory instead of six.  The first stage has unit
// twiddles; a twiddled radix-8 stage at sub-transform length Ns owns 4 Ns
// entries, W^m, W^2m, W^4m and W^(m + n/8) (= W8 W^m) for m = k n/(8 Ns), each
// run consecutive in k; a twiddled radix-4 stage owns 3 Ns, as above.  The
// forward stage tables follow the radix-4 path's two copies, then the
// inverse copy (conjugated).
__host__ __device__ constexpr int r8_stages8(int n) {
  return (ilog2c(n) % 3 == 1 && ilog2c(n) >= 4) ? ilog2c(n) / 3 - 1 : ilog2c(n) / 3;
}
__host__ __device__ constexpr int r8_stages4(int n) {
  return ilog2c(n) % 3 == 1 ? 2 : ilog2c(n) % 3 == 2 ? 1 : 0;
}
// radix and sub-transform length of stage i of the radix-8 path
__host__ __device__ constexpr int r8_radix(int n, int i) { return i < r8_stages8(n) ? 8 : 4; }
__host__ __device__ constexpr int r8_ns(int n, int i) {
  return i <= r8_stages8(n) ? (1 << (3 * i)) : (1 << (3 * r8_stages8(n))) << (2 * (i - r8_stages8(n)));
}
__host__ __device__ constexpr int r8_stage_size(int n, int i) {
  return i == 0 ? 0 : (r8_radix(n, i) == 8 ? 4 : 3) * r8_ns(n, i);
}
__host__ __device__ constexpr int r8_stage_off(int n, int i) {
  return i <= 1 ? 0 : r8_stage_off(n, i - 1) + r8_stage_size(n, i - 1);
}
__host__ __device__ constexpr int r8_span(int n) {
  return r8_stage_off(n, r8_stages8(n) + r8_stages4(n) - 1) +
         r8_stage_size(n, r8_stages8(n) + r8_stages4(n) - 1);
}
__host__ __device__ constexpr int tw_r8_base(int n) { return n + 2 * tw_stage_span(n); }

// FP64 lengths with odd log2 n (fft_slot_m8): an untwiddled radix-8 first stage,
// then (log2 n - 3) / 2 twiddled radix-4 stages at Ns = 8, 32, 128, ...; stage
// Ns owns [Ns - 8, 4 Ns - 8) of each direction's tables, (r, k) at (Ns - 8) +
// (r - 1) Ns + k, in the ratio form of dft4_tw_ratio (the FP32 and double-float
// tables hold the plain twiddles there, unused).
__host__ __device__ constexpr int tw_m8_span(int n) {
  return (ilog2c(n) & 1) && n >= 32 ? 8 * ((1 << (ilog2c(n) - 3)) - 1) : 0;
}
__host__ __device__ constexpr int tw_m8_base(int n) { return tw_r8_base(n) + 2 * r8_span(n); }
__host__ __device__ constexpr int tw_count(int n) { return tw_m8_base(n) + 2 * tw_m8_span(n); }

// Untwiddled radix-4 DFT (first stage).  Forward: y1 = a1 - i a3, y3 = a1 + i a3.
template <bool INV, typename C>
__device__ __forceinline__ void dft4(C& v0, C& v1, C& v2, C& v3) {
  const auto a0r = v0.x + v2.x, a0i = v0.y + v2.y;
  const auto a1r = v0.x - v2.x, a1i = v0.y - v2.y;
  const auto a2r = v1.x + v3.x, a2i = v1.y + v3.y;
  const auto a3r = v1.x - v3.x, a3i = v1.y - v3.y;
  v0.x = a0r + a2r; v0.y = a0i + a2i;
  v2.x = a0r - a2r; v2.y = a0i - a2i;
  if (!INV) {
    v1.x = a1r + a3i; v1.y = a1i - a3r;
    v3.x = a1r - a3i; v3.y = a1i + a3r;
  } else {
    v1.x = a1r - a3i; v1.y = a1i + a3r;
    v3.x = a1r + a3i; v3.y = a1i - a3r;
  }
}

// Twiddled radix-4 butterfly; w1..w3 are already conjugated for the inverse.
template <bool INV, typename C>
__device__ __forceinline__ void dft4_tw(C& v0, C& v1, C& v2, C& v3, const C w1, const C w2,
                                        const C w3) {
  typedef decltype(v0.x) T;
  const T two = T(2);
  // a0 = v0 + w2 v2, a1 = v0 - w2 v2
  const T a0r = fma(v2.x, w2.x, fma(-v2.y, w2.y, v0.x));
  const T a0i = fma(v2.x, w2.y, fma(v2.y, w2.x, v0.y));
  const T a1r = fma(two, v0.x, -a0r);
  const T a1i = fma(two, v0.y, -a0i);
  // t1 = w1 v1; a2 = t1 + w3 v3, a3 = t1 - w3 v3
  const T t1r = fma(v1.x, w1.x, -v1.y * w1.y);
  const T t1i = fma(v1.x, w1.y, v1.y * w1.x);
  const T a2r = fma(v3.x, w3.x, fma(-v3.y, w3.y, t1r));
  const T a2i = fma(v3.x, w3.y, fma(v3.y, w3.x, t1i));
  const T a3r = fma(two, t1r, -a2r);
  const T a3i = fma(two, t1i, -a2i);
  v0.x = a0r + a2r; v0.y = a0i + a2i;
  v2.x = a0r - a2r; v2.y = a0i - a2i;
  if (!INV) {
    v1.x = a1r + a3i; v1.y = a1i - a3r;
    v3.x = a1r - a3i; v3.y = a1i + a3r;
  } else {
    v1.x = a1r - a3i; v1.y = a1i + a3r;
    v3.x = a1r + a3i; v3.y = a1i - a3r;
  }
}

// FP64 twiddled radix-4 butterfly on ratio-form twiddles.  With w_r = c_r + i s_r
// (already conjugated for the inverse) and tau_r = s_r / c_r, the table entries
// are e1 = (tau1, c1), e2 = (tau2, c2), e3 = (tau3, c3 / c1).  Then
//   z_r = v_r (1 + i tau_r)            so that w_r v_r = c_r z_r   (2 FMAs each)
//   a0, a1 = v0 +- c2 z2
//   b, d   = z1 +- (c3 / c1) z3        so that w1 v1 +- w3 v3 = c1 (b, d)
//   y0, y2 = a0 +- c1 b;  y1, y3 = a1 -+ i c1 d (forward; +- for the inverse)
// 22 FMAs against 24.  Every rounding is relative to |v| as in the plain form
// (|c_r z_r| = |v_r|); c2 = 0 at the quarter turn is stored as 2^-256 with
// tau2 = s2 2^256, both exact, so c2 z2 still rounds to w2 v2.
template <bool INV>
__device__ __forceinline__ void dft4_tw_ratio(double2& v0, double2& v1, double2& v2, double2& v3, const double2 e1,
                                              const double2 e2, const double2 e3) {
  const double z1r = fma(-e1.x, v1.y, v1.x), z1i = fma(e1.x, v1.x, v1.y);
  const double z2r = fma(-e2.x, v2.y, v2.x), z2i = fma(e2.x, v2.x, v2.y);
  const double z3r = fma(-e3.x, v3.y, v3.x), z3i = fma(e3.x, v3.x, v3.y);
  const double c1 = e1.y, c2 = e2.y, rho = e3.y;
  const double a0r = fma(c2, z2r, v0.x), a0i = fma(c2, z2i, v0.y);
  const double a1r = fma(-c2, z2r, v0.x), a1i = fma(-c2, z2i, v0.y);
  const double br = fma(rho, z3r, z1r), bi = fma(rho, z3i, z1i);
  const double dr = fma(-rho, z3r, z1r), di = fma(-rho, z3i, z1i);
  v0.x = fma(c1, br, a0r); v0.y = fma(c1, bi, a0i);
  v2.x = fma(-c1, br, a0r); v2.y = fma(-c1, bi, a0i);
  if (!INV) {  // y1 = a1 - i c1 d, y3 = a1 + i c1 d
    v1.x = fma(c1, di, a1r); v1.y = fma(-c1, dr, a1i);
    v3.x = fma(-c1, di, a1r); v3.y = fma(c1, dr, a1i);
  } else {
    v1.x = fma(-c1, di, a1r); v1.y = fma(c1, dr, a1i);
    v3.x = fma(c1, di, a1r); v3.y = fma(-c1, dr, a1i);
  }
}

// Radix-2 butterfly x = a + w c, y = a - w c (two-sided FMA form).
template <typename C>
__device__ __forceinline__ void bfly2_tw(const C a, const C c, const C w, C& x, C& y) {
  typedef decltype(a.x) T;
  x.x = fma(c.x, w.x, fma(-c.y, w.y, a.x));
  x.y = fma(c.x, w.y, fma(c.y, w.x, a.y));
  y.x = fma(T(2), a.x, -x.x);
  y.y = fma(T(2), a.y, -x.y);
}

// Double-float butterflies: the same dataflow with unnormalised intermediate
// sums and products (add_u, mul_u) and one renormalisation per output.
template <bool INV>
__device__ __forceinline__ void dft4(df64c& v0, df64c& v1, df64c& v2, df64c& v3) {
  const df64 a0r = add_u(v0.x, v2.x), a0i = add_u(v0.y, v2.y);
  const df64 a1r = sub_u(v0.x, v2.x), a1i = sub_u(v0.y, v2.y);
  const df64 a2r = add_u(v1.x, v3.x), a2i = add_u(v1.y, v3.y);
  const df64 a3r = sub_u(v1.x, v3.x), a3i = sub_u(v1.y, v3.y);
  v0.x = renorm(add_u(a0r, a2r)); v0.y = renorm(add_u(a0i, a2i));
  v2.x = renorm(sub_u(a0r, a2r)); v2.y = renorm(sub_u(a0i, a2i));
  if (!INV) {
    v1.x = renorm(add_u(a1r, a3i)); v1.y = renorm(sub_u(a1i, a3r));
    v3.x = renorm(sub_u(a1r, a3i)); v3.y = renorm(add_u(a1i, a3r));
  } else {
    v1.x = renorm(sub_u(a1r, a3i)); v1.y = renorm(add_u(a1i, a3r));
    v3.x = renorm(add_u(a1r, a3i)); v3.y = renorm(sub_u(a1i, a3r));
  }
}

__device__ __forceinline__ void cmul_u(const df64c v, const df64c w, df64& r, df64& i) {
  r = sub_u(mul_u(v.x, w.x), mul_u(v.y, w.y));
  i = add_u(mul_u(v.x, w.y), mul_u(v.y, w.x));
}

template <bool INV>
__device__ __forceinline__ void dft4_tw(df64c& v0, df64c& v1, df64c& v2, df64c& v3, const df64c w1,
                                        const df64c w2, const df64c w3) {
  df64 cr, ci, t1r, t1i, t3r, t3i;
  cmul_u(v2, w2, cr, ci);
  cmul_u(v1, w1, t1r, t1i);
  cmul_u(v3, w3, t3r, t3i);
  const df64 a0r = add_u(v0.x, cr), a0i = add_u(v0.y, ci);
  const df64 a1r = sub_u(v0.x, cr), a1i = sub_u(v0.y, ci);
  const df64 a2r = add_u(t1r, t3r), a2i = add_u(t1i, t3i);
  const df64 a3r = sub_u(t1r, t3r), a3i = sub_u(t1i, t3i);
  v0.x = renorm(add_u(a0r, a2r)); v0.y = renorm(add_u(a0i, a2i));
  v2.x = renorm(sub_u(a0r, a2r)); v2.y = renorm(sub_u(a0i, a2i));
  if (!INV) {
    v1.x = renorm(add_u(a1r, a3i)); v1.y = renorm(sub_u(a1i, a3r));
    v3.x = renorm(sub_u(a1r, a3i)); v3.y = renorm(add_u(a1i, a3r));
  } else {
    v1.x = renorm(sub_u(a1r, a3i)); v1.y = renorm(add_u(a1i, a3r));
    v3.x = renorm(add_u(a1r, a3i)); v3.y = renorm(sub_u(a1i, a3r));
  }
}

__device__ __forceinline__ void bfly2_tw(const df64c a, const df64c c, const df64c w, df64c& x, df64c& y) {
  df64 tr, ti;
  cmul_u(c, w, tr, ti);
  x.x = renorm(add_u(a.x, tr));
  x.y = renorm(add_u(a.y, ti));
  y.x = renorm(sub_u(a.x, tr));
  y.y = renorm(sub_u(a.y, ti));
}

// Twiddle W^m of a length-N table, conjugated for the inverse transform.  The
// tables hold tw[N - m] = conj(tw[m]) exactly, so for FP64 the conjugate is a
// load at the mirrored index (a negation would be one more FP64-pipe
// instruction); an FP32 negation is free and the FP32 form measured faster
// reading the plain index.
template <typename C>
__device__ __forceinline__ C load_tw_raw(const C* __restrict__ tw, int i) {
  return __ldg(tw + i);
}

__device__ __forceinline__ df64c load_tw_raw(const df64c* __restrict__ tw, int i) {
  const float4 v = __ldg(reinterpret_cast<const float4*>(tw) + i);
  df64c w;
  w.x = df64(v.x, v.y);
  w.y = df64(v.z, v.w);
  return w;
}

template <bool INV, int N, typename C>
__device__ __forceinline__ C load_tw(const C* __restrict__ tw, int m) {
  if constexpr (sizeof(C) == 8) {
    C w = __ldg(tw + m);
    if (INV) w.y = -w.y;
    return w;
  } else {
    return __ldg(tw + (INV ? ((N - m) & (N - 1)) : m));
  }
}

template <bool INV, int N>
__device__ __forceinline__ df64c load_tw(const df64c* __restrict__ tw, int m) {
  const float4 v = __ldg(reinterpret_cast<const float4*>(tw) + (INV ? ((N - m) & (N - 1)) : m));
  df64c w;
  w.x = df64(v.x, v.y);
  w.y = df64(v.z, v.w);
  return w;
}

template <int N, bool INV, int G>
__device__ __forceinline__ void fft_slot_m8(double2* buf, int lane, bool active, const double2* __restrict__ tw);

// In-place length-N transform of buf (unnormalised); tw is the length-N twiddle
// table described above (tw_count(N) entries).
// Forward: X[k] = sum x[n] e^{-2 pi i nk/N}; inverse uses e^{+...}.
// G threads share the transform (default N/16; up to N/4, one butterfly each).
template <typename T, int N, bool INV, int G = fft_group(N)>
__device__ __forceinline__ void fft_slot(typename cplx_of<T>::type* buf, int lane, bool active,
                                         const typename cplx_of<T>::type* __restrict__ tw) {
  typedef typename cplx_of<T>::type C;
  constexpr int Q = N / 4;
  constexpr int LG = ilog2c(N);
  constexpr int NR4 = LG / 2;
  static_assert((1 << LG) == N && N >= 16, "power-of-two length >= 16");
  static_assert(Q % G == 0, "group must divide the butterfly count");
  constexpr int BPT = Q / G;
  if constexpr (std::is_same<T, double>::value && (LG & 1) && N >= 32) {
    fft_slot_m8<N, INV, G>(buf, lane, active, tw);
  } else {
#pragma unroll
    for (int s = 0; s < NR4; ++s) {
      const int Ns = 1 << (2 * s);
      C v[BPT][4];
      if (active) {
#pragma unroll
        for (int b = 0; b < BPT; ++b) {
          const int j = lane + b * G;
#pragma unroll
          for (int r = 0; r < 4; ++r) v[b][r] = buf[j + r * Q];
        }
      }
      __syncthreads();
      if (active) {
#pragma unroll
        for (int b = 0; b < BPT; ++b) {
          const int j = lane + b * G;
          const int k = j & (Ns - 1);
          if (s == 0) {
            dft4<INV>(v[b][0], v[b][1], v[b][2], v[b][3]);
          } else {
            // this stage's table, already conjugated for the inverse
            const C* ts = tw + N + (INV ? tw_stage_span(N) : 0) + (Ns - 4);
            const C w1 = load_tw_raw(ts, k);
            const C w2 = load_tw_raw(ts, Ns + k);
            const C w3 = load_tw_raw(ts, 2 * Ns + k);
            if constexpr (std::is_same<T, double>::value)  // ratio-form table entries
              dft4_tw_ratio<INV>(v[b][0], v[b][1], v[b][2], v[b][3], w1, w2, w3);
            else
              dft4_tw<INV>(v[b][0], v[b][1], v[b][2], v[b][3], w1, w2, w3);
          }
          const int base = ((j - k) << 2) + k;
#pragma unroll
          for (int r = 0; r < 4; ++r) buf[base + r * Ns] = v[b][r];
        }
      }
      __syncthreads();
    }
    if (LG & 1) {
      // final radix-2 stage, Ns = N/2: out[j] = a + w^j b, out[j + N/2] = a - w^j b
      constexpr int H = N / 2;
      constexpr int B2 = H / G;
      if (active) {
#pragma unroll
        for (int b = 0; b < B2; ++b) {
          const int j = lane + b * G;
          const C a = buf[j], c = buf[j + H];
          const C w = load_tw<INV, N>(tw, j);
          C x, y;
          bfly2_tw(a, c, w, x, y);
          buf[j] = x;
          buf[j + H] = y;
        }
      }
      __syncthreads();
    }
  }
}

// ---------------------------------------------------------------------------
// Radix-8 (FP64 and FP32 only)
// ---------------------------------------------------------------------------
// a' = a + t b, b' = a - t b in the two-sided FMA form (6 FMA-pipe instructions).
template <typename C>
__device__ __forceinline__ void pair_t(C& a, C& b, const C t) {
  typedef decltype(a.x) T;
  const T xr = fma(b.x, t.x, fma(-b.y, t.y, a.x));
  const T xi = fma(b.x, t.y, fma(b.y, t.x, a.y));
  b.x = fma(T(2), a.x, -xr);
  b.y = fma(T(2), a.y, -xi);
  a.x = xr;
  a.y = xi;
}

// t times W4 (W4 = -i forward, +i inverse): a swap and a sign, no arithmetic.
template <bool INV, typename C>
__device__ __forceinline__ C mul_w4(const C t) {
  C r;
  if (!INV) {
    r.x = t.y;
    r.y = -t.x;
  } else {
    r.x = -t.y;
    r.y = t.x;
  }
  return r;
}

// a +- b, a +- W4 b (untwiddled pairs: 4 adds)
template <typename C>
__device__ __forceinline__ void pair_1(C& a, C& b) {
  const C s = mkc<decltype(a.x)>(a.x + b.x, a.y + b.y);
  b = mkc<decltype(a.x)>(a.x - b.x, a.y - b.y);
  a = s;
}
template <bool INV, typename C>
__device__ __forceinline__ void pair_w4(C& a, C& b) {
  const C q = mul_w4<INV>(b);
  const C s = mkc<decltype(a.x)>(a.x + q.x, a.y + q.y);
  b = mkc<decltype(a.x)>(a.x - q.x, a.y - q.y);
  a = s;
}
// a +- W8^e b for e = 1 or 3 (W8 = (1 -+ i)/sqrt(2)): two adds form the rotated
// pair up to the factor 1/sqrt(2), which four FMAs then apply (6 instructions).
template <bool INV, int E, typename C>
__device__ __forceinline__ void pair_w8(C& a, C& b) {
  typedef decltype(a.x) T;
  const T c = T(0.70710678118654752440);
  T p, q;  // W8^E b = c (p, q)
  if (!INV) {
    if (E == 1) { p = b.x + b.y; q = b.y - b.x; }    // (1 - i)(x + iy)
    else        { p = b.y - b.x; q = -(b.x + b.y); }  // (-1 - i)(x + iy)
  } else {
    if (E == 1) { p = b.x - b.y; q = b.x + b.y; }    // (1 + i)(x + iy)
    else        { p = -(b.x + b.y); q = b.x - b.y; }  // (-1 + i)(x + iy)
  }
  const C s = mkc<T>(fma(c, p, a.x), fma(c, q, a.y));
  b = mkc<T>(fma(-c, p, a.x), fma(-c, q, a.y));
  a = s;
}

// Untwiddled 8-point DFT (52 FP64-pipe instructions).  In: v[r] = x[r];
// out: v[] holds X in the order 0, 4, 2, 6, 1, 5, 3, 7.
template <bool INV, typename C>
__device__ __forceinline__ void dft8(C* v) {
  pair_1(v[0], v[4]); pair_1(v[1], v[5]); pair_1(v[2], v[6]); pair_1(v[3], v[7]);
  pair_1(v[0], v[2]); pair_1(v[1], v[3]);
  pair_w4<INV>(v[4], v[6]); pair_w4<INV>(v[5], v[7]);
  pair_1(v[0], v[1]);
  pair_w4<INV>(v[2], v[3]);
  pair_w8<INV, 1>(v[4], v[5]);
  pair_w8<INV, 3>(v[6], v[7]);
}

// Twiddled 8-point DFT of x[r] W^(r m): X_q = sum_r x_r W^(rm) W8^(rq), with the
// twiddles folded into the three pair levels (w = W^m, w2 = W^2m, w4 = W^4m,
// w8 = W8 W^m; 12 pairs, 72 FP64-pipe instructions).  Output order as dft8.
template <bool INV, typename C>
__device__ __forceinline__ void dft8_tw(C* v, const C w, const C w2, const C w4, const C w8) {
  pair_t(v[0], v[4], w4); pair_t(v[1], v[5], w4); pair_t(v[2], v[6], w4); pair_t(v[3], v[7], w4);
  pair_t(v[0], v[2], w2); pair_t(v[1], v[3], w2);
  const C w2q = mul_w4<INV>(w2);
  pair_t(v[4], v[6], w2q); pair_t(v[5], v[7], w2q);
  pair_t(v[0], v[1], w);
  pair_t(v[2], v[3], mul_w4<INV>(w));
  pair_t(v[4], v[5], w8);
  pair_t(v[6], v[7], mul_w4<INV>(w8));
}

// FP64 transform of odd log2 N >= 32 (called by fft_slot; same contract): the
// untwiddled 8-point DFT as the first stage (52 FMA-pipe instructions per 8
// points, against 16 per 4 points of the radix-4 stage plus 6 per 2 points of
// a final radix-2 stage), then ratio-form radix-4 stages at Ns = 8, 32, ...:
// 28.5 FP64 instructions per point at N = 2048 instead of 29, and one pass
// through shared memory fewer.
// x times W4 when `rot` (a swap and an exact sign flip on the integer pipe), else x.
template <bool INV>
__device__ __forceinline__ double2 rot_w4_if(const double2 x, bool rot) {
  const double nx = __longlong_as_double(__double_as_longlong(x.x) ^ (long long)0x8000000000000000ULL);
  const double ny = __longlong_as_double(__double_as_longlong(x.y) ^ (long long)0x8000000000000000ULL);
  return rot ? (INV ? make_double2(ny, x.x) : make_double2(x.y, nx)) : x;
}

template <int N, bool INV, int G>
__device__ __forceinline__ void fft_slot_m8(double2* buf, int lane, bool active, const double2* __restrict__ tw) {
  constexpr int LG = ilog2c(N), B8 = N / 8, Q = N / 4;
  constexpr int BPT8 = (B8 + G - 1) / G, BPT4 = Q / G;
  static_assert((LG & 1) && N >= 32 && Q % G == 0, "odd log2 length >= 32");
  static_assert(B8 % G == 0 || G == 2 * B8, "whole 8-point butterflies per thread, or one per lane pair");
  constexpr int OUTQ[8] = {0, 4, 2, 6, 1, 5, 3, 7};  // dft8 leaves X_OUTQ[i] in v[i]
  if constexpr (G == 2 * B8) {
    // One 8-point DFT per lane pair, with dft8's pairs and arithmetic: the even
    // lane holds x0, x2, x4, x6, the odd lane x1, x3, x5, x7; the first two pair
    // levels stay within a lane, then the lanes swap two values each.  The odd
    // lane's last level, (x2, x3) by W4 and (x6, x7) by W8^3 = W8 W4, is the even
    // lane's, (x0, x1) plain and (x4, x5) by W8, with its second values turned
    // by W4 first (exact), so both lanes run the same instructions.  Every
    // thread of the CTA reaches the shuffles (the whole CTA runs each stage), and
    // a lane's partner (lane ^ 1) belongs to the same slot since G is even.
    const int j = lane >> 1;
    const bool odd = lane & 1;
    double2 u[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) u[i] = active ? buf[j + (2 * i + (odd ? 1 : 0)) * B8] : make_double2(0.0, 0.0);
    __syncthreads();
    pair_1(u[0], u[2]);  // (x0, x4) | (x1, x5)
    pair_1(u[1], u[3]);  // (x2, x6) | (x3, x7)
    pair_1(u[0], u[1]);  // (x0, x2) | (x1, x3)
    pair_w4<INV>(u[2], u[3]);  // (x4, x6) | (x5, x7)
    const double2 s0 = odd ? u[0] : u[1], s1 = odd ? u[2] : u[3];
    const unsigned m = __activemask();  // the warp's lanes (converged after the barrier)
    const double2 r0 = make_double2(__shfl_xor_sync(m, s0.x, 1), __shfl_xor_sync(m, s0.y, 1));
    const double2 r1 = make_double2(__shfl_xor_sync(m, s1.x, 1), __shfl_xor_sync(m, s1.y, 1));
    double2 x0 = odd ? r0 : u[0];                  // v0 | v2
    double2 x1 = rot_w4_if<INV>(odd ? u[1] : r0, odd);  // v1 | W4 v3
    double2 x4 = odd ? r1 : u[2];                  // v4 | v6
    double2 x5 = rot_w4_if<INV>(odd ? u[3] : r1, odd);  // v5 | W4 v7
    pair_1(x0, x1);
    pair_w8<INV, 1>(x4, x5);
    if (active) {  // X0, X4, X1, X5 | X2, X6, X3, X7
      double2* o = buf + 8 * j + (odd ? 2 : 0);
      o[0] = x0;
      o[4] = x1;
      o[1] = x4;
      o[5] = x5;
    }
    __syncthreads();
  } else {
    double2 v[BPT8][8];
    if (active) {
#pragma unroll
      for (int b = 0; b < BPT8; ++b) {
        const int j = lane + b * G;
        if (j < B8) {
#pragma unroll
          for (int r = 0; r < 8; ++r) v[b][r] = buf[j + r * B8];
        }
      }
    }
    __syncthreads();
    if (active) {
#pragma unroll
      for (int b = 0; b < BPT8; ++b) {
        const int j = lane + b * G;
        if (j < B8) {
          dft8<INV>(v[b]);
#pragma unroll
          for (int i = 0; i < 8; ++i) buf[8 * j + OUTQ[i]] = v[b][i];
        }
      }
    }
    __syncthreads();
  }
  const double2* tb = tw + tw_m8_base(N) + (INV ? tw_m8_span(N) : 0);
#pragma unroll
  for (int s = 0; s < (LG - 3) / 2; ++s) {
    const int Ns = 8 << (2 * s);
    double2 v[BPT4][4];
    if (active) {
#pragma unroll
      for (int b = 0; b < BPT4; ++b) {
        const int j = lane + b * G;
#pragma unroll
        for (int r = 0; r < 4; ++r) v[b][r] = buf[j + r * Q];
      }
    }
    __syncthreads();
    if (active) {
#pragma unroll
      for (int b = 0; b < BPT4; ++b) {
        const int j = lane + b * G;
        const int k = j & (Ns - 1);
        const double2* ts = tb + (Ns - 8);
        dft4_tw_ratio<INV>(v[b][0], v[b][1], v[b][2], v[b][3], load_tw_raw(ts, k), load_tw_raw(ts, Ns + k),
                           load_tw_raw(ts, 2 * Ns + k));
        const int base = ((j - k) << 2) + k;
#pragma unroll
        for (int r = 0; r < 4; ++r) buf[base + r * Ns] = v[b][r];
      }
    }
    __syncthreads();
  }
}

// In-place length-N transform along the radix-8 path (same contract and result
// layout as fft_slot).  G threads share it; in radix-8 stages lanes beyond the
// N/8 butterflies idle.
template <typename T, int N, bool INV, int G = fft_group(N)>
__device__ __forceinline__ void fft_slot_r8(typename cplx_of<T>::type* buf, int lane, bool active,
                                            const typename cplx_of<T>::type* __restrict__ tw) {
  typedef typename cplx_of<T>::type C;
  constexpr int S8 = r8_stages8(N), S4 = r8_stages4(N);
  constexpr int B8 = N / 8, Q = N / 4;
  constexpr int BPT8 = (B8 + G - 1) / G, BPT4 = (Q + G - 1) / G;
  static_assert((1 << ilog2c(N)) == N && N >= 16, "power-of-two length >= 16");
  const C* tb = tw + tw_r8_base(N) + (INV ? r8_span(N) : 0);
  constexpr int OUTQ[8] = {0, 4, 2, 6, 1, 5, 3, 7};  // v[i] holds X_OUTQ[i]
#pragma unroll
  for (int s = 0; s < S8; ++s) {
    const int Ns = 1 << (3 * s);
    C v[BPT8][8];
    if (active) {
#pragma unroll
      for (int b = 0; b < BPT8; ++b) {
        const int j = lane + b * G;
        if (j < B8) {
#pragma unroll
          for (int r = 0; r < 8; ++r) v[b][r] = buf[j + r * B8];
        }
      }
    }
    __syncthreads();
    if (active) {
#pragma unroll
      for (int b = 0; b < BPT8; ++b) {
        const int j = lane + b * G;
        if (j < B8) {
          const int k = j & (Ns - 1);
          if (s == 0) {
            dft8<INV>(v[b]);
          } else {
            const C* ts = tb + r8_stage_off(N, s);
            dft8_tw<INV>(v[b], load_tw_raw(ts, k), load_tw_raw(ts, Ns + k), load_tw_raw(ts, 2 * Ns + k),
                         load_tw_raw(ts, 3 * Ns + k));
          }
          const int base = ((j - k) << 3) + k;
#pragma unroll
          for (int i = 0; i < 8; ++i) buf[base + OUTQ[i] * Ns] = v[b][i];
        }
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int s = 0; s < S4; ++s) {
    const int Ns = (1 << (3 * S8)) << (2 * s);
    C v[BPT4][4];
    if (active) {
#pragma unroll
      for (int b = 0; b < BPT4; ++b) {
        const int j = lane + b * G;
        if (j < Q) {
#pragma unroll
          for (int r = 0; r < 4; ++r) v[b][r] = buf[j + r * Q];
        }
      }
    }
    __syncthreads();
    if (active) {
#pragma unroll
      for (int b = 0; b < BPT4; ++b) {
        const int j = lane + b * G;
        if (j < Q) {
          const int k = j & (Ns - 1);
          if (S8 == 0 && s == 0) {
            dft4<INV>(v[b][0], v[b][1], v[b][2], v[b][3]);
          } else {
            const C* ts = tb + r8_stage_off(N, S8 + s);
            dft4_tw<INV>(v[b][0], v[b][1], v[b][2], v[b][3], load_tw_raw(ts, k), load_tw_raw(ts, Ns + k),
                         load_tw_raw(ts, 2 * Ns + k));
          }
          const int base = ((j - k) << 2) + k;
#pragma unroll
          for (int r = 0; r < 4; ++r) buf[base + r * Ns] = v[b][r];
        }
      }
    }
    __syncthreads();
  }
}

// The transform of a step kernel along the path R (4 or 8; the double-float
// form has only the radix-4 path).
template <typename T, int N, bool INV, int G, int R>
__device__ __forceinline__ void fft_path(typename cplx_of<T>::type* buf, int lane, bool active,
                                         const typename cplx_of<T>::type* __restrict__ tw) {
  if constexpr (R == 8 && !std::is_same<T, df64>::value)
    fft_slot_r8<T, N, INV, G>(buf, lane, active, tw);
  else
    fft_slot<T, N, INV, G>(buf, lane, active, tw);
}

}  // namespace tara
