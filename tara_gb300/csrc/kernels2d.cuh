// 2D pseudo-spectral kernels: the reference's derive2csh / derive2css RHS and the
// AB2 / RK4 updates, split into three passes over HBM per RHS evaluation.
//
// Layout in HBM: every spectral field is a half spectrum stored row by row,
// field[y * pitch + x] for ky row y in [0, Ny) and kx column x in [0, Nh),
// Nh = Nx/2 + 1, pitch = Nh rounded up to 8 elements (128 B rows for FP64).
// This is the reference's complex(8) a(Nh,Ny) layout with padded rows.
//
// Pass A  k_col_inverse   per tile of kx columns: read omega_hat, form
//         u_x = i ky psi, u_y = -i kx psi, i kx w, i ky w (w = omega_hat for the
//         plain RHS, w = k^2 psi for the screened one) and inverse-transform
//         each along y.  (src/derive2csh.f95:29-71, src/derive2css.f95:22-55)
// Pass B  k_row_nl        per pair of ky rows: the x-direction c2r of the four
//         fields as two complex transforms (u_x + i u_y, w_x + i w_y), the
//         product u.grad(w), and the x-direction r2c of the two rows' products
//         as one complex transform.  (src/derive2csh.f95:73-106)
// Pass C  k_col_forward   per tile of kx columns: forward transform along y,
//         2/3 truncation, scaling, nu k^2 term, and the stage update of the
//         chosen scheme.  (src/derive2csh.f95:108-145, src/ab2csh.f95:10-14)
//
// The c2r follows FFTW's rank-2 c2r semantics: complex DFTs along y for all
// Nh columns first, then a 1D c2r along x that reads only the real parts of the
// kx = 0 and kx = Nx/2 bins (lib/fftw/rdft/rank-geq2-rdft2.c).  The reference
// feeds it non-Hermitian spectra (e.g. i ky w on the ky = -Ny/2 row), so the
// order and the discard rule are kept exactly.
#pragma once
#include <type_traits>

#include "fft.cuh"

namespace tara {

// Element loop of a CTA over TOTAL items with THREADS threads (both
// compile-time): the trip count is a constant, so the loop unrolls and the
// independent global loads of different iterations issue together.  (With a
// thread-dependent start the compiler keeps the loop rolled and every element
// waits out one memory latency, which dominates on small grids.)
#define TARA_ELEM_LOOP(e, TOTAL, THREADS)                                                   \
  _Pragma("unroll 4") for (int e##_i = 0; e##_i < ((TOTAL) + (THREADS)-1) / (THREADS); ++e##_i) \
    if (const int e = tid + e##_i * (THREADS); (TOTAL) % (THREADS) == 0 || e < (TOTAL))

// A double is finite when its exponent field is not all ones (an integer test on
// the high word, kept off the FP64 pipe).
__device__ __forceinline__ bool finite_bits(double v) {
  return ((unsigned int)__double2hiint(v) & 0x7ff00000u) != 0x7ff00000u;
}

struct Grid2D {
  int nx, ny, nh, pitch;
  const double* __restrict__ kx;   // [nh]
  const double* __restrict__ ky;   // [ny]
  const int* __restrict__ i0;      // [ny]: first kx index removed by the 2/3 rule
  const double* __restrict__ inv;  // [ny][nh]: 1/(kx^2+ky^2) (+lambda when screened), 0 at k = 0
  int i0max;                       // columns x >= i0max lose the whole nonlinear term
  // FP32 copies of kx, ky, inv for the FP32-transform mode, whose spectral
  // products run in FP32 (only the state update stays FP64)
  const float* __restrict__ kxf;
  const float* __restrict__ kyf;
  const float* __restrict__ invf;
  // double-float copies of kx, ky, inv for the double-float mode, whose
  // spectral products run on the FP32 pipes
  const df64* __restrict__ kxd;
  const df64* __restrict__ kyd;
  const df64* __restrict__ invd;
};

enum StepMode {
  MODE_DERIVE = 0,  // write F = dt_omegak_new
  MODE_AB2 = 1,     // w0 += (3/2 F - 1/2 Fold) dt ; Fold = F
  MODE_RK1 = 2,     // S = F ; ws = w0 + F dt/2
  MODE_RK2 = 3,     // S += 2F ; ws = w0 + F dt/2
  MODE_RK3 = 4,     // S += 2F ; ws = w0 + F dt
  MODE_RK4 = 5      // w0 += dt/6 (S + F)
};

struct RhsParams {
  int rhs;          // 0 plain (derive2csh), 1 screened (derive2css)
  double nu, alpha, lambda;
  double nl_scale;  // 1/2 (pair split) * 1/(Nx Ny)^2 (two unnormalised c2r)
  double dt;
  float nu_f, alpha_f, nl_scale_f;  // the same in FP32 for the FP32-transform mode
  df64 nu_d, alpha_d, nl_scale_d;   // and in double-float for the double-float mode
};

template <typename T>
constexpr bool is_df64() { return std::is_same<T, df64>::value; }

// Dynamic shared memory one CTA may use on sm_103a (227 KB).
constexpr int kMaxSmem = 227 * 1024;

// Largest power-of-two column tile with tile smem <= budget and <= 512 threads.
__host__ __device__ constexpr int pick_tc(int bytes_per_col, int threads_per_col,
                                          int budget = 100 * 1024) {
  int tc = 32;
  while (tc > 1 && (tc * bytes_per_col > budget || tc * threads_per_col > 512)) tc >>= 1;
  return tc;
}

// Row pairs per CTA for the row pass: <= 512 threads, <= 64 KB (at least 1).
__host__ __device__ constexpr int pick_rp(int n, int csize) {
  int rp = 32;
  while (rp > 1 && (4 * rp * fft_group(n) > 512 || rp * 4 * n * csize > 64 * 1024)) rp >>= 1;
  return rp;
}

// V selects a tile variant for the autotuner: 0 the default tile, 1 half of it,
// 2 one column (one row pair) per CTA, for grids too small to fill the SMs
// with the larger tiles.  In the column passes variant 2 also gives each
// column 4x the threads (one radix-4 butterfly per thread per stage), so a
// 16-byte-element CTA at N = 2048 has 512 (1024 in pass A) threads instead of
// 128: more loads in flight per column where the default tile is already one
// column.  The butterflies are the same, so the results are too, bit for bit.
template <typename T, int N, int V = 0> struct ColCfg {
  typedef typename cplx_of<T>::type C;
  static constexpr int G0 = fft_group(N);
  static constexpr int G = V == 2 ? 4 * G0 : G0;  // threads per column slot
  static constexpr int S = N + 1;  // smem column stride (one element of padding)
  static constexpr int TCA0 = pick_tc(2 * S * (int)sizeof(C), 2 * G0);  // pass A: 2 slots/column
  // pass C: 1 slot/column; a small tile keeps the live (not fully truncated)
  // columns spread evenly over the SMs
  static constexpr int TCC0 = pick_tc(S * (int)sizeof(C), G0, 48 * 1024);
  static constexpr int TCA = V == 2 ? 1 : (V == 1 && TCA0 > 1) ? TCA0 / 2 : TCA0;
  static constexpr int TCC = V == 2 ? 1 : (V == 1 && TCC0 > 1) ? TCC0 / 2 : TCC0;
  static constexpr int THREADS_A = 2 * TCA * G;
  static constexpr int THREADS_C = TCC * G;
  static constexpr int SMEM_A = 2 * TCA * S * (int)sizeof(C);
  static constexpr int SMEM_C = TCC * S * (int)sizeof(C);
  // a tile exists when it fits one CTA (at 4096 points variant 2 of pass A
  // would need 2048 threads)
  static constexpr bool VALID_A = THREADS_A <= 1024 && SMEM_A <= kMaxSmem;
  static constexpr bool VALID_C = THREADS_C <= 1024 && SMEM_C <= kMaxSmem;
};

// Row pass tiles.  Variants 0-2 hold RP row pairs in four slots each (the two
// inverse transforms of both rows run together).  Variant 3 holds one row pair
// in three slots with half the threads: the two inverse transforms of row a,
// then of row b, each leaving its products in the third slot, then the forward
// transform of that slot.  Its 96 KB of shared memory (FP64, N = 2048) and
// 256 threads let two CTAs share an SM, so one CTA's loads, stores and stage
// barriers overlap the other's butterflies.  Same arithmetic, same results.
template <typename T, int N, int V = 0> struct RowCfg {
  typedef typename cplx_of<T>::type C;
  static constexpr int G = fft_group(N);
  static constexpr int RP0 = pick_rp(N, (int)sizeof(C));
  static constexpr int RP = V >= 2 ? 1 : (V == 1 && RP0 > 1) ? RP0 / 2 : RP0;
  static constexpr int THREADS = V == 3 ? 2 * G : 4 * RP * G;
  static constexpr int SL = N;  // smem stride between row slots
  static constexpr int SMEM = (V == 3 ? 3 : RP * 4) * SL * (int)sizeof(C);
  // four FP64 slots of 4096 points (256 KB) do not fit a CTA: variant 3 only
  static constexpr bool VALID = THREADS <= 1024 && SMEM <= kMaxSmem;
  // CTAs per SM the row kernel asks for: two for variant 3 and the 512-thread
  // FP32 tiles -- as far as shared memory allows.  (Asking three of the
  // 256-thread FP32 tiles held them to 80 registers but scheduled them worse:
  // the 512^2 row pass took 503 instead of 364 us.)
  static constexpr int MINB0 = (V == 3 || (sizeof(T) == 4 && THREADS >= 512)) ? 2 : 1;
  static constexpr int MINB = MINB0 * SMEM <= kMaxSmem ? MINB0 : 1;
};

// ---------------------------------------------------------------------------
// Pass A
// ---------------------------------------------------------------------------
// blockIdx.y = 0: (u_x, u_y); blockIdx.y = 1: (i kx w, i ky w).  Splitting the
// two field pairs over the grid halves the tail of the last wave.
// blockIdx.z = run of a batch (runs are ny*pitch apart in every field).
// The double-float form asks for three 256-thread CTAs per SM (80 registers,
// a little spill): its prologue waits on strided loads, which a third CTA hides
// (measured 255 -> 240 us at 2048^2); the FP64 form gains nothing from it.  The
// FP32 form keeps two 512-thread CTAs per SM (64 registers; at 80 registers one
// CTA per SM took 113 instead of 95 us at 2048^2).
// The CTA body (block coordinates given explicitly, so that the ensemble's
// persistent kernel can run it for any run and tile): tile bx, field pair
// `pair`, run `run`.
template <typename T, int N, int V, int R>
__device__ __forceinline__ void col_inverse_cta(unsigned bx, unsigned pair, unsigned run,
                                                const double2* __restrict__ win,
                                                typename cplx_of<T>::type* __restrict__ u, const Grid2D& g,
                                                const RhsParams& p,
                                                const typename cplx_of<T>::type* __restrict__ tw) {
  typedef typename cplx_of<T>::type C;
  typedef ColCfg<T, N, V> CF;
  constexpr int TC = CF::TCA, S = CF::S, G = CF::G;
  extern __shared__ __align__(16) unsigned char smraw[];
  C* sm = reinterpret_cast<C*>(smraw);  // [2][TC][S]
  const int x0 = bx * TC;
  const int tid = threadIdx.x;
  const size_t fsz = (size_t)g.ny * g.pitch;
  win += run * fsz;
  u += run * 4 * fsz;
  const int slot = tid / G, lane = tid % G;
  TARA_ELEM_LOOP(e, N * TC, CF::THREADS_A) {
    const int y = e / TC, c = e % TC, x = x0 + c;
    C fa = mkc<T>(T(0), T(0)), fb = fa;
    if constexpr (sizeof(T) == 4) {
      if (x < g.nh) {  // FP32 products from the FP64 state
        const double2 wd = win[(size_t)y * g.pitch + x];
        const float wx = (float)wd.x, wy = (float)wd.y;
        const float kx = g.kxf[x], ky = g.kyf[y], inv = g.invf[(size_t)y * g.nh + x];
        if (pair == 0) {
          const float pr = wx * inv, pim = wy * inv;
          fa = mkc<T>(-ky * pim, ky * pr);
          fb = mkc<T>(kx * pim, -(kx * pr));
        } else {
          float dr = wx, di = wy;
          if (p.rhs) {
            const float k2 = kx * kx + ky * ky;
            dr = k2 * (wx * inv);
            di = k2 * (wy * inv);
          }
          fa = mkc<T>(-kx * di, kx * dr);
          fb = mkc<T>(-ky * di, ky * dr);
        }
      }
    } else if constexpr (is_df64<T>()) {
      if (x < g.nh) {  // double-float products from the FP64 state (FP32 pipes only)
        const double2 wd = win[(size_t)y * g.pitch + x];
        const df64 wx = split_double(wd.x), wy = split_double(wd.y);
        const df64 kx = g.kxd[x], ky = g.kyd[y], inv = g.invd[(size_t)y * g.nh + x];
        if (pair == 0) {
          const df64 pr = wx * inv, pim = wy * inv;
          fa = mkc<T>(-(ky * pim), ky * pr);
          fb = mkc<T>(kx * pim, -(kx * pr));
        } else {
          df64 dr = wx, di = wy;
          if (p.rhs) {
            const df64 k2 = kx * kx + ky * ky;
            dr = k2 * (wx * inv);
            di = k2 * (wy * inv);
          }
          fa = mkc<T>(-(kx * di), kx * dr);
          fb = mkc<T>(-(ky * di), ky * dr);
        }
      }
    } else if (x < g.nh) {
      const double2 w = win[(size_t)y * g.pitch + x];
      const double kx = g.kx[x], ky = g.ky[y];
      const double inv = g.inv[(size_t)y * g.nh + x];  // 1/k^2 or 1/(k^2+lambda); 0 at k = 0
      if (pair == 0) {
        // psi = omega/(k^2 [+lambda]); u_x = (0,1) ky psi, u_y = -(0,1) kx psi
        const double pr = w.x * inv, pim = w.y * inv;
        fa = mkc<T>(T(-ky * pim), T(ky * pr));
        fb = mkc<T>(T(kx * pim), T(-(kx * pr)));
      } else {
        // i kx w, i ky w with w = omega_hat (plain) or k^2 psi (screened)
        double dr = w.x, di = w.y;
        if (p.rhs) {
          const double k2 = kx * kx + ky * ky;
          dr = k2 * (w.x * inv);
          di = k2 * (w.y * inv);
        }
        fa = mkc<T>(T(-kx * di), T(kx * dr));
        fb = mkc<T>(T(-ky * di), T(ky * dr));
      }
    }
    sm[c * S + y] = fa;
    sm[(TC + c) * S + y] = fb;
  }
  __syncthreads();
  fft_path<T, N, true, G, R>(sm + slot * S, lane, true, tw);
  TARA_ELEM_LOOP(e, N * TC, CF::THREADS_A) {
    const int y = e / TC, c = e % TC, x = x0 + c;
    if (x < g.nh) {
      const size_t q = (size_t)y * g.pitch + x;
      u[(size_t)(2 * pair) * fsz + q] = sm[c * S + y];
      u[(size_t)(2 * pair + 1) * fsz + q] = sm[(TC + c) * S + y];
    }
  }
}

template <typename T, int N, int V, int R = 4>
__global__ void __launch_bounds__(ColCfg<T, N, V>::THREADS_A,
                                  (is_df64<T>() && ColCfg<T, N, V>::THREADS_A == 256)       ? 3
                                  : (sizeof(T) == 4 && ColCfg<T, N, V>::THREADS_A == 512) ? 2
                                                                                          : 1)
    k_col_inverse(const double2* __restrict__ win, typename cplx_of<T>::type* __restrict__ u,
                  Grid2D g, RhsParams p, const typename cplx_of<T>::type* __restrict__ tw) {
  col_inverse_cta<T, N, V, R>(blockIdx.x, blockIdx.y, blockIdx.z, win, u, g, p, tw);
}

// ---------------------------------------------------------------------------
// Pass B
// ---------------------------------------------------------------------------
// Slot s of row pair p: s = 0 (u_x + i u_y, row a), 1 (w_x + i w_y, row a),
// 2 and 3 the same for row b = a + 1.  Hermitian extension of a half row A:
// Z[k] = A[k] + i B[k] (k <= N/2), Z[N-k] = conj(A[k]) + i conj(B[k]), with the
// imaginary parts of the k = 0 and k = N/2 bins dropped first.
// blockIdx.y = run of a batch.
// Load of a spectral value through the non-coherent (read-only) path, for data
// that no thread of the running kernel writes.
template <typename C>
__device__ __forceinline__ C ldg_c(const C* p) {
  return __ldg(p);
}
__device__ __forceinline__ df64c ldg_c(const df64c* p) {
  const float4 v = __ldg(reinterpret_cast<const float4*>(p));
  df64c w;
  w.x = df64(v.x, v.y);
  w.y = df64(v.z, v.w);
  return w;
}

// Hermitian extension of the half rows A, B (two spectra of one ky row) into
// slot entry k of Z = A + i B (see above).  NC: read through the non-coherent
// path -- the per-pass row kernel does (a plain load there, once the body sat
// in a device function, cost the FP32 512^2 row pass 40 %); the persistent
// ensemble kernel must not, since it wrote the rows itself earlier in the launch.
template <typename T, int N, bool NC, typename C>
__device__ __forceinline__ C row_pair_entry(const C* __restrict__ fa, const C* __restrict__ fb, int k) {
  constexpr int H = N / 2;
  const int kk = k <= H ? k : N - k;
  C A, B;
  if constexpr (NC) {
    A = ldg_c(fa + kk);
    B = ldg_c(fb + kk);
  } else {
    A = fa[kk];
    B = fb[kk];
  }
  if (kk == 0 || kk == H) {
    A.y = T(0);
    B.y = T(0);
  }
  return (k <= H) ? mkc<T>(A.x - B.y, A.y + B.x) : mkc<T>(A.x + B.y, -A.y + B.x);
}

// The CTA body: row-pair tile bx of run `run` (NC: see row_pair_entry).  The
// block coordinates are unsigned, as blockIdx is: with int coordinates the
// 64-bit address arithmetic took 84 instead of 80 registers in the FP32 row
// tile, which then fitted two CTAs per SM instead of three.
template <typename T, int N, int V, int R, bool NC = true>
__device__ __forceinline__ void row_nl_cta(unsigned bx, unsigned run, const typename cplx_of<T>::type* __restrict__ u,
                                           typename cplx_of<T>::type* __restrict__ nl, const Grid2D& g,
                                           const typename cplx_of<T>::type* __restrict__ tw) {
  typedef typename cplx_of<T>::type C;
  typedef RowCfg<T, N, V> RC;
  constexpr int G = RC::G, H = N / 2, RP = RC::RP, SL = RC::SL;
  extern __shared__ __align__(16) unsigned char smraw[];
  C* sm = reinterpret_cast<C*>(smraw);  // [RP][4][N], or [3][N] in variant 3
  const int tid = threadIdx.x;
  const int slot = tid / G, lane = tid % G;
  const int y_base = bx * (2 * RP);
  const size_t fsz = (size_t)g.ny * g.pitch;
  u += run * 4 * fsz;
  nl += run * fsz;
  if constexpr (V == 3) {
    C* pk = sm + 2 * SL;  // products of rows a (real part) and b (imaginary part)
#pragma unroll 1
    for (int r = 0; r < 2; ++r) {
      const int y = y_base + r;
      TARA_ELEM_LOOP(e, 2 * N, RC::THREADS) {
        const int k = e % N, s = e / N;  // s = 0: u_x + i u_y, 1: w_x + i w_y
        C z = mkc<T>(T(0), T(0));
        if (y < g.ny) {
          const C* fa = u + (size_t)(2 * s) * fsz + (size_t)y * g.pitch;
          z = row_pair_entry<T, N, NC>(fa, fa + fsz, k);
        }
        sm[s * SL + k] = z;
      }
      __syncthreads();
      fft_path<T, N, true, G, R>(sm + slot * SL, lane, true, tw);
      TARA_ELEM_LOOP(e, N, RC::THREADS) {
        const C c1 = sm[e], c2 = sm[SL + e];
        const T v = fma(c1.x, c2.x, c1.y * c2.y);
        if (r == 0)
          pk[e].x = v;
        else
          pk[e].y = v;
      }
      __syncthreads();
    }
    fft_path<T, N, false, 2 * G, R>(pk, tid, true, tw);
    TARA_ELEM_LOOP(e, H + 1, RC::THREADS) {
      const int k = e;
      if (y_base < g.ny) {
        const C z = pk[k], m = pk[(N - k) & (N - 1)];
        nl[(size_t)y_base * g.pitch + k] = mkc<T>(z.x + m.x, z.y - m.y);
        nl[(size_t)(y_base + 1) * g.pitch + k] = mkc<T>(z.y + m.y, -(z.x - m.x));
      }
    }
  } else {
    TARA_ELEM_LOOP(e, RP * 4 * N, RC::THREADS) {
      const int k = e % N, sl = e / N;
      const int pp = sl >> 2, s = sl & 3;
      const int y = y_base + 2 * pp + (s >> 1);
      C z = mkc<T>(T(0), T(0));
      if (y < g.ny) {
        const C* fa = u + (size_t)(2 * (s & 1)) * fsz + (size_t)y * g.pitch;
        z = row_pair_entry<T, N, NC>(fa, fa + fsz, k);
      }
      sm[sl * SL + k] = z;
    }
    __syncthreads();
    fft_path<T, N, true, G, R>(sm + slot * SL, lane, true, tw);
    // products u_x w_x + u_y w_y for rows a and b, packed as a + i b
    TARA_ELEM_LOOP(e, RP * N, RC::THREADS) {
      const int x = e % N, pp = e / N;
      C* b = sm + (size_t)pp * 4 * SL;
      const C c1a = b[x], c2a = b[SL + x], c1b = b[2 * SL + x], c2b = b[3 * SL + x];
      const T na = fma(c1a.x, c2a.x, c1a.y * c2a.y);
      const T nb = fma(c1b.x, c2b.x, c1b.y * c2b.y);
      b[x] = mkc<T>(na, nb);
    }
    __syncthreads();
    // forward transform of each pair's packed products (its first slot), shared
    // by all 4 G threads of the pair so that no thread idles through it
    fft_path<T, N, false, 4 * G, R>(sm + (tid / (4 * G)) * 4 * SL, tid % (4 * G), true, tw);
    // split: 2 X_a[k] = Z[k] + conj Z[N-k], 2 X_b[k] = -i (Z[k] - conj Z[N-k])
    TARA_ELEM_LOOP(e, RP * (H + 1), RC::THREADS) {
      const int k = e % (H + 1), pp = e / (H + 1);
      const int ya = y_base + 2 * pp;
      if (ya < g.ny) {
        const C* b = sm + (size_t)pp * 4 * SL;
        const C z = b[k], m = b[(N - k) & (N - 1)];
        nl[(size_t)ya * g.pitch + k] = mkc<T>(z.x + m.x, z.y - m.y);
        nl[(size_t)(ya + 1) * g.pitch + k] = mkc<T>(z.y + m.y, -(z.x - m.x));
      }
    }
  }
}

// The per-pass row kernel.  Variant 3 runs the CTA body above; variants 0-2
// spell the same body out in the kernel itself: compiled through the device
// function, the FP32 256-thread tile at 512 points ran 500 instead of 364 us
// (same arithmetic and register count, a different schedule).
template <typename T, int N, int V, int R = 4>
__global__ void __launch_bounds__(RowCfg<T, N, V>::THREADS, RowCfg<T, N, V>::MINB)
    k_row_nl(const typename cplx_of<T>::type* __restrict__ u,
             typename cplx_of<T>::type* __restrict__ nl, Grid2D g,
             const typename cplx_of<T>::type* __restrict__ tw) {
  if constexpr (V == 3) {
    row_nl_cta<T, N, V, R>(blockIdx.x, blockIdx.y, u, nl, g, tw);
  } else {
    typedef typename cplx_of<T>::type C;
    typedef RowCfg<T, N, V> RC;
    constexpr int G = RC::G, H = N / 2, RP = RC::RP, SL = RC::SL;
    extern __shared__ __align__(16) unsigned char smraw[];
    C* sm = reinterpret_cast<C*>(smraw);  // [RP][4][N]
    const int tid = threadIdx.x;
    const int slot = tid / G, lane = tid % G;
    const int y_base = blockIdx.x * (2 * RP);
    const size_t fsz = (size_t)g.ny * g.pitch;
    u += blockIdx.y * 4 * fsz;
    nl += blockIdx.y * fsz;
    TARA_ELEM_LOOP(e, RP * 4 * N, RC::THREADS) {
      const int k = e % N, sl = e / N;
      const int pp = sl >> 2, s = sl & 3;
      const int y = y_base + 2 * pp + (s >> 1);
      C z = mkc<T>(T(0), T(0));
      if (y < g.ny) {
        const C* fa = u + (size_t)(2 * (s & 1)) * fsz + (size_t)y * g.pitch;
        const C* fb = fa + fsz;
        const int kk = k <= H ? k : N - k;
        C A = fa[kk], B = fb[kk];
        if (kk == 0 || kk == H) {
          A.y = T(0);
          B.y = T(0);
        }
        z = (k <= H) ? mkc<T>(A.x - B.y, A.y + B.x) : mkc<T>(A.x + B.y, -A.y + B.x);
      }
      sm[sl * SL + k] = z;
    }
    __syncthreads();
    fft_path<T, N, true, G, R>(sm + slot * SL, lane, true, tw);
    TARA_ELEM_LOOP(e, RP * N, RC::THREADS) {
      const int x = e % N, pp = e / N;
      C* b = sm + (size_t)pp * 4 * SL;
      const C c1a = b[x], c2a = b[SL + x], c1b = b[2 * SL + x], c2b = b[3 * SL + x];
      const T na = fma(c1a.x, c2a.x, c1a.y * c2a.y);
      const T nb = fma(c1b.x, c2b.x, c1b.y * c2b.y);
      b[x] = mkc<T>(na, nb);
    }
    __syncthreads();
    fft_path<T, N, false, 4 * G, R>(sm + (tid / (4 * G)) * 4 * SL, tid % (4 * G), true, tw);
    TARA_ELEM_LOOP(e, RP * (H + 1), RC::THREADS) {
      const int k = e % (H + 1), pp = e / (H + 1);
      const int ya = y_base + 2 * pp;
      if (ya < g.ny) {
        const C* b = sm + (size_t)pp * 4 * SL;
        const C z = b[k], m = b[(N - k) & (N - 1)];
        nl[(size_t)ya * g.pitch + k] = mkc<T>(z.x + m.x, z.y - m.y);
        nl[(size_t)(ya + 1) * g.pitch + k] = mkc<T>(z.y + m.y, -(z.x - m.x));
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Pass C
// ---------------------------------------------------------------------------
struct StepBufs {
  const double2* win;  // RHS input (w0 or ws); may alias ws
  double2* w0;         // state
  double2* ws;         // RK stage input
  double2* acc;        // RK sum k1 + 2k2 + 2k3
  double2* fold;       // AB2 history
  double2* fout;       // MODE_DERIVE output
  unsigned int* flag;  // bit 0: a non-finite value was produced
  const double2* force;  // optional spectrum added to every right-hand side (nullptr: none)
};

// blockIdx.y = run of a batch.  The double-float form's 512-thread variant asks
// for two CTAs per SM (64 registers, 90 bytes of spill): its warps wait on the
// state loads, and a second CTA hides them (115 -> 103 us at 2048^2).
template <typename T, int N, int V, int R>
__device__ __forceinline__ void col_forward_cta(unsigned bx, unsigned run, const typename cplx_of<T>::type* __restrict__ nl,
                                                StepBufs sb, const Grid2D& g, const RhsParams& p, int mode,
                                                const typename cplx_of<T>::type* __restrict__ tw) {
  typedef typename cplx_of<T>::type C;
  typedef ColCfg<T, N, V> CF;
  constexpr int TC = CF::TCC, S = CF::S, G = CF::G;
  extern __shared__ __align__(16) unsigned char smraw[];
  C* sm = reinterpret_cast<C*>(smraw);  // [TC][S]
  const int x0 = bx * TC;
  const int tid = threadIdx.x;
  {
    const size_t off = run * (size_t)g.ny * g.pitch;
    nl += off;
    sb.win += off;
    if (sb.w0) sb.w0 += off;
    if (sb.ws) sb.ws += off;
    if (sb.acc) sb.acc += off;
    if (sb.fold) sb.fold += off;
    if (sb.fout) sb.fout += off;
    if (sb.force) sb.force += off;
  }
  // Tiles whose columns all lie at kx >= i0max lose the whole nonlinear term to
  // the 2/3 rule: their transform is skipped (uniform per CTA, so the barriers
  // inside fft_slot stay matched).
  const bool live = x0 < g.i0max;
  if (live) {
    TARA_ELEM_LOOP(e, N * TC, CF::THREADS_C) {
      const int y = e / TC, c = e % TC, x = x0 + c;
      sm[c * S + y] = (x < g.nh) ? nl[(size_t)y * g.pitch + x] : mkc<T>(T(0), T(0));
    }
    __syncthreads();
    fft_path<T, N, false, G, R>(sm + (tid / G) * S, tid % G, true, tw);
  }
  // Pass 1: the right-hand side of every element of this thread (reads only,
  // so the unrolled loop issues all its loads together).
  // The FP32 form keeps its right-hand side in FP32 registers until the update
  // (its value is an FP32 number either way); the optional forcing is added in
  // pass 2 in FP64.
  typedef typename std::conditional<sizeof(T) == 4, float, double>::type RT;
  constexpr int PER = (N * TC + CF::THREADS_C - 1) / CF::THREADS_C;
  RT frv[PER], fiv[PER];
  bool bad = false;
#pragma unroll
  for (int i = 0; i < PER; ++i) {
    const int e = tid + i * CF::THREADS_C;
    const int y = e / TC, c = e % TC, x = x0 + c;
    frv[i] = RT(0);
    fiv[i] = RT(0);
    if (e >= N * TC || x >= g.nh) continue;
    const size_t q = (size_t)y * g.pitch + x;
    double fr, fi;
    if constexpr (sizeof(T) == 4) {  // FP32 right-hand side, FP64 update below
      float nr = 0.f, ni = 0.f;
      if (x < g.i0[y]) {
        const C v = sm[c * S + y];
        nr = v.x * p.nl_scale_f;
        ni = v.y * p.nl_scale_f;
      }
      const float kx = g.kxf[x], ky = g.kyf[y];
      const float k2 = kx * kx + ky * ky;
      const float vk2 = p.nu_f * k2;
      const double2 wd = sb.win[q];
      const float wx = (float)wd.x, wy = (float)wd.y;
      if (p.rhs == 0) {
        fr = (double)(-(nr + vk2 * wx));
        fi = (double)(-(ni + vk2 * wy));
      } else {
        const float inv = g.invf[(size_t)y * g.nh + x];
        fr = (double)(-(p.alpha_f * nr + vk2 * (k2 * (wx * inv))));
        fi = (double)(-(p.alpha_f * ni + vk2 * (k2 * (wy * inv))));
      }
    } else if constexpr (is_df64<T>()) {  // double-float right-hand side, one FP64 add to widen
      df64 nr(0.f, 0.f), ni(0.f, 0.f);
      if (x < g.i0[y]) {
        const C v = sm[c * S + y];
        nr = v.x * p.nl_scale_d;
        ni = v.y * p.nl_scale_d;
      }
      const df64 kx = g.kxd[x], ky = g.kyd[y];
      const df64 k2 = kx * kx + ky * ky;
      const df64 vk2 = p.nu_d * k2;
      const double2 wd = sb.win[q];
      const df64 wx = split_double(wd.x), wy = split_double(wd.y);
      df64 rr, ri;
      if (p.rhs == 0) {
        rr = -(nr + vk2 * wx);
        ri = -(ni + vk2 * wy);
      } else {
        const df64 inv = g.invd[(size_t)y * g.nh + x];
        rr = -(p.alpha_d * nr + vk2 * (k2 * (wx * inv)));
        ri = -(p.alpha_d * ni + vk2 * (k2 * (wy * inv)));
      }
      bad |= !(isfinite(rr.hi) && isfinite(ri.hi));
      fr = to_double(rr);
      fi = to_double(ri);
    } else {
      double nr = 0.0, ni = 0.0;
      if (x < g.i0[y]) {  // 2/3 truncation of the nonlinear term only
        const C v = sm[c * S + y];
        nr = (double)v.x * p.nl_scale;
        ni = (double)v.y * p.nl_scale;
      }
      const double kx = g.kx[x], ky = g.ky[y];
      const double k2 = kx * kx + ky * ky;
      const double vk2 = p.nu * k2;
      const double2 w = sb.win[q];
      if (p.rhs == 0) {
        fr = -(nr + vk2 * w.x);
        fi = -(ni + vk2 * w.y);
      } else {
        const double inv = g.inv[(size_t)y * g.nh + x];  // 1/(k^2+lambda), 0 at k = 0
        const double dr = k2 * (w.x * inv), di = k2 * (w.y * inv);
        fr = -(p.alpha * nr + vk2 * dr);
        fi = -(p.alpha * ni + vk2 * di);
      }
    }
    if constexpr (std::is_same<T, double>::value) {
      if (sb.force) {
        const double2 fc = sb.force[q];
        fr += fc.x;
        fi += fc.y;
      }
      bad |= !(finite_bits(fr) && finite_bits(fi));
    } else if constexpr (is_df64<T>()) {
      if (sb.force) {
        const double2 fc = sb.force[q];
        fr += fc.x;
        fi += fc.y;
        bad |= !(finite_bits(fr) && finite_bits(fi));
      }
    }
    frv[i] = (RT)fr;  // exact: an FP32 value in the FP32 form, unchanged in FP64
    fiv[i] = (RT)fi;
  }
  // Pass 2: the stage update, in chunks whose loads all precede their stores
  // (the state arrays may alias the RHS input, so loads cannot move past stores).
  constexpr int CH = PER < 8 ? PER : 8;
  const double dt = p.dt;
#pragma unroll
  for (int i0 = 0; i0 < PER; i0 += CH) {
    double2 a0[CH], a1[CH];
    size_t qv[CH];
    bool ok[CH];
#pragma unroll
    for (int u = 0; u < CH; ++u) {
      const int e = tid + (i0 + u) * CF::THREADS_C;
      const int y = e / TC, x = x0 + e % TC;
      ok[u] = i0 + u < PER && e < N * TC && x < g.nh;
      qv[u] = (size_t)y * g.pitch + x;
      a0[u] = make_double2(0.0, 0.0);
      a1[u] = a0[u];
      if (ok[u]) {
        if (mode == MODE_AB2) {
          a0[u] = sb.w0[qv[u]];
          a1[u] = sb.fold[qv[u]];
        } else if (mode != MODE_DERIVE) {
          a0[u] = sb.w0[qv[u]];
          if (mode != MODE_RK1) a1[u] = sb.acc[qv[u]];
        }
      }
    }
#pragma unroll
    for (int u = 0; u < CH; ++u) {
      if (!ok[u]) continue;
      double fr = (double)frv[i0 + u], fi = (double)fiv[i0 + u];
      const size_t q = qv[u];
      if constexpr (sizeof(T) == 4) {  // the FP32 form adds the forcing here, in FP64
        if (sb.force) {
          const double2 fc = sb.force[q];
          fr += fc.x;
          fi += fc.y;
        }
        bad |= !(finite_bits(fr) && finite_bits(fi));
      }
      const double2 s = a0[u];
      switch (mode) {
        case MODE_DERIVE:
          sb.fout[q] = make_double2(fr, fi);
          break;
        case MODE_AB2: {
          const double2 fo = a1[u];
          sb.w0[q] = make_double2(s.x + (1.5 * fr - 0.5 * fo.x) * dt, s.y + (1.5 * fi - 0.5 * fo.y) * dt);
          sb.fold[q] = make_double2(fr, fi);
          break;
        }
        case MODE_RK1:
          sb.acc[q] = make_double2(fr, fi);
          sb.ws[q] = make_double2(s.x + fr * dt / 2.0, s.y + fi * dt / 2.0);
          break;
        case MODE_RK2:
        case MODE_RK3: {
          const double2 a = a1[u];
          const double h = (mode == MODE_RK2) ? dt / 2.0 : dt;
          sb.acc[q] = make_double2(a.x + 2.0 * fr, a.y + 2.0 * fi);
          sb.ws[q] = make_double2(s.x + fr * h, s.y + fi * h);
          break;
        }
        default: {  // MODE_RK4
          const double2 a = a1[u];
          sb.w0[q] = make_double2(s.x + dt / 6.0 * (a.x + fr), s.y + dt / 6.0 * (a.y + fi));
          break;
        }
      }
    }
  }
  if (bad) atomicOr(sb.flag, 1u);
}

template <typename T, int N, int V, int R = 4>
__global__ void __launch_bounds__(ColCfg<T, N, V>::THREADS_C,
                                  (is_df64<T>() && ColCfg<T, N, V>::THREADS_C == 512) ? 2 : 1)
    k_col_forward(const typename cplx_of<T>::type* __restrict__ nl, StepBufs sb, Grid2D g,
                  RhsParams p, int mode, const typename cplx_of<T>::type* __restrict__ tw) {
  col_forward_cta<T, N, V, R>(blockIdx.x, blockIdx.y, nl, sb, g, p, mode, tw);
}

// ---------------------------------------------------------------------------
// Plain transforms (initial conditions, diagnostics and the transform API)
// ---------------------------------------------------------------------------
// Column transform of a half spectrum along y, in place or out of place.
template <typename T, int N, bool INV, int V = 0>
__global__ void __launch_bounds__(ColCfg<T, N, V>::THREADS_C)
    k_col_fft(const typename cplx_of<T>::type* in, typename cplx_of<T>::type* out, int nh,
              int pitch, size_t fs, const typename cplx_of<T>::type* __restrict__ tw) {
  typedef typename cplx_of<T>::type C;
  typedef ColCfg<T, N, V> CF;
  constexpr int TC = CF::TCC, S = CF::S, G = CF::G;
  extern __shared__ __align__(16) unsigned char smraw[];
  C* sm = reinterpret_cast<C*>(smraw);
  const int x0 = blockIdx.x * TC, tid = threadIdx.x;
  in += blockIdx.y * fs;  // field of a batch (blockIdx.y), fs elements apart
  out += blockIdx.y * fs;
  TARA_ELEM_LOOP(e, N * TC, CF::THREADS_C) {
    const int y = e / TC, c = e % TC, x = x0 + c;
    sm[c * S + y] = (x < nh) ? in[(size_t)y * pitch + x] : mkc<T>(T(0), T(0));
  }
  __syncthreads();
  fft_slot<T, N, INV, G>(sm + (tid / G) * S, tid % G, true, tw);
  TARA_ELEM_LOOP(e, N * TC, CF::THREADS_C) {
    const int y = e / TC, c = e % TC, x = x0 + c;
    if (x < nh) out[(size_t)y * pitch + x] = sm[c * S + y];
  }
}

// Row pairs per CTA of the plain row transforms (one slot per pair): four per
// row pair of the RHS row pass, or a single pair for the small-grid variant.
// Largest power-of-two count of row pairs, at most np, whose slots fit `budget`.
__host__ __device__ constexpr int fit_pairs(int np, int slot_bytes, int budget = 128 * 1024) {
  return (np > 1 && np * slot_bytes > budget) ? fit_pairs(np / 2, slot_bytes, budget) : np;
}

template <typename T, int N, int V> struct RowXCfg {
  static constexpr int NP = V == 2 ? 1
                                   : fit_pairs(4 * RowCfg<T, N, V>::RP,
                                               N * (int)sizeof(typename cplx_of<T>::type));
  // the single-pair tile gives its transform 4x the threads (one radix-4
  // butterfly per thread per stage), as the one-column tile of the column pass does
  static constexpr int G = V == 2 ? 4 * fft_group(N) : fft_group(N);
  static constexpr int THREADS = NP * G;
  static constexpr int SMEM = NP * N * (int)sizeof(typename cplx_of<T>::type);
};

// 1D c2r along x for pairs of rows (after the y pass): out rows are real with
// row pitch rpitch.  Unnormalised.
template <typename T, int N, int V = 0>
__global__ void __launch_bounds__(RowXCfg<T, N, V>::THREADS)
    k_row_c2r(const typename cplx_of<T>::type* __restrict__ in, T* __restrict__ out, int ny,
              int pitch, int rpitch, size_t fs_in, size_t fs_out,
              const typename cplx_of<T>::type* __restrict__ tw) {
  typedef typename cplx_of<T>::type C;
  typedef RowXCfg<T, N, V> RC;
  constexpr int G = RC::G, H = N / 2, NP = RC::NP, SL = N;  // NP row pairs per CTA
  extern __shared__ __align__(16) unsigned char smraw[];
  C* sm = reinterpret_cast<C*>(smraw);  // [NP][N]
  const int tid = threadIdx.x, y_base = blockIdx.x * (2 * NP);
  in += blockIdx.y * fs_in;  // field of a batch (blockIdx.y)
  out += blockIdx.y * fs_out;
  TARA_ELEM_LOOP(e, NP * N, RC::THREADS) {
    const int k = e % N, pp = e / N, ya = y_base + 2 * pp;
    C z = mkc<T>(T(0), T(0));
    if (ya < ny) {
      const int kk = k <= H ? k : N - k;
      C A = in[(size_t)ya * pitch + kk], B = in[(size_t)(ya + 1) * pitch + kk];
      if (kk == 0 || kk == H) {
        A.y = T(0);
        B.y = T(0);
      }
      z = (k <= H) ? mkc<T>(A.x - B.y, A.y + B.x) : mkc<T>(A.x + B.y, -A.y + B.x);
    }
    sm[pp * SL + k] = z;
  }
  __syncthreads();
  fft_slot<T, N, true, G>(sm + (tid / G) * SL, tid % G, true, tw);
  TARA_ELEM_LOOP(e, NP * N, RC::THREADS) {
    const int x = e % N, pp = e / N, ya = y_base + 2 * pp;
    if (ya < ny) {
      const C z = sm[pp * SL + x];
      out[(size_t)ya * rpitch + x] = z.x;
      out[(size_t)(ya + 1) * rpitch + x] = z.y;
    }
  }
}

// 1D r2c along x for pairs of real rows (before the y pass).  Unnormalised.
template <typename T, int N, int V = 0>
__global__ void __launch_bounds__(RowXCfg<T, N, V>::THREADS)
    k_row_r2c(const T* __restrict__ in, typename cplx_of<T>::type* __restrict__ out, int ny,
              int rpitch, int pitch, size_t fs_in, size_t fs_out,
              const typename cplx_of<T>::type* __restrict__ tw) {
  typedef typename cplx_of<T>::type C;
  typedef RowXCfg<T, N, V> RC;
  constexpr int G = RC::G, H = N / 2, NP = RC::NP, SL = N;
  extern __shared__ __align__(16) unsigned char smraw[];
  C* sm = reinterpret_cast<C*>(smraw);
  const int tid = threadIdx.x, y_base = blockIdx.x * (2 * NP);
  in += blockIdx.y * fs_in;  // field of a batch (blockIdx.y)
  out += blockIdx.y * fs_out;
  TARA_ELEM_LOOP(e, NP * N, RC::THREADS) {
    const int x = e % N, pp = e / N, ya = y_base + 2 * pp;
    sm[pp * SL + x] = (ya < ny) ? mkc<T>(in[(size_t)ya * rpitch + x], in[(size_t)(ya + 1) * rpitch + x])
                               : mkc<T>(T(0), T(0));
  }
  __syncthreads();
  fft_slot<T, N, false, G>(sm + (tid / G) * SL, tid % G, true, tw);
  TARA_ELEM_LOOP(e, NP * (H + 1), RC::THREADS) {
    const int k = e % (H + 1), pp = e / (H + 1), ya = y_base + 2 * pp;
    if (ya < ny) {
      const C z = sm[pp * SL + k], m = sm[pp * SL + ((N - k) & (N - 1))];
      out[(size_t)ya * pitch + k] = mkc<T>(T(0.5) * (z.x + m.x), T(0.5) * (z.y - m.y));
      out[(size_t)(ya + 1) * pitch + k] = mkc<T>(T(0.5) * (z.y + m.y), T(-0.5) * (z.x - m.x));
    }
  }
}

// ---------------------------------------------------------------------------
// Diagnostics: 1/2<|u|^2> and 1/2<omega^2> by Parseval over the half spectrum
// (weight 1 on the kx = 0 and kx = Nx/2 columns, 2 elsewhere).
// ---------------------------------------------------------------------------
__global__ void k_diag_partial(const double2* __restrict__ w, Grid2D g, double* __restrict__ part);
__global__ void k_diag_final(const double* __restrict__ part, int nparts, double inv,
                             double* __restrict__ out, unsigned int* flag);
__global__ void k_mul(double2* __restrict__ w, size_t n, double s);
// out = w + (3/2 fn - 1/2 fo) dt over n elements (src/ab2csh.f95:10-14)
__global__ void k_ab2_dense(const double2* w, double2* out, const double2* __restrict__ fo,
                            const double2* __restrict__ fn, size_t n, double dt);

}  // namespace tara
