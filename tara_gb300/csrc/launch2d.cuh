// Launchers for the 2D kernels: runtime grid size -> compile-time transform
// length.  Included once per precision (launch_fp64.cu, launch_fp32.cu) so the
// two instantiation sets compile in parallel.
#pragma once
#include <type_traits>

#include "internal.h"

namespace tara {

// Opt a kernel into more than 48 KB of dynamic shared memory (once per process).
template <typename K>
static cudaError_t allow_smem(K kernel, int bytes) {
  if (bytes <= 48 * 1024) return cudaSuccess;
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

#define TARA_SWITCH_N(n, CALL)         \
  switch (n) {                         \
    case 16: { constexpr int N = 16; CALL; } break;     \
    case 32: { constexpr int N = 32; CALL; } break;     \
    case 64: { constexpr int N = 64; CALL; } break;     \
    case 128: { constexpr int N = 128; CALL; } break;   \
    case 256: { constexpr int N = 256; CALL; } break;   \
    case 512: { constexpr int N = 512; CALL; } break;   \
    case 1024: { constexpr int N = 1024; CALL; } break; \
    case 2048: { constexpr int N = 2048; CALL; } break; \
    case 4096: { constexpr int N = 4096; CALL; } break; \
    default: return set_error(TARA_ERR_ARGS, "grid size must be a power of two in [16, 4096]"); \
  }

static inline int no_tile() {
  return set_error(TARA_ERR_ARGS, "this tile variant does not fit one CTA at this length");
}

template <typename T, int N, int V, int R>
static int launch_col_inverse(int nh, const double2* win, void* u, const Grid2D& g,
                              const RhsParams& p, const void* tw, cudaStream_t s, int nb) {
  typedef typename cplx_of<T>::type C;
  typedef ColCfg<T, N, V> CF;
  if constexpr (!CF::VALID_A) {
    return no_tile();
  } else {
    static cudaError_t attr = allow_smem(k_col_inverse<T, N, V, R>, CF::SMEM_A);
    TARA_CK(attr);
    const dim3 blocks((nh + CF::TCA - 1) / CF::TCA, 2, nb);
    k_col_inverse<T, N, V, R><<<blocks, CF::THREADS_A, CF::SMEM_A, s>>>(win, (C*)u, g, p, (const C*)tw);
    TARA_CK(cudaGetLastError());
    return TARA_OK;
  }
}

template <typename T, int N, int V, int R>
static int launch_row_nl(int ny, const void* u, void* nl, const Grid2D& g, const void* tw,
                         cudaStream_t s, int nb) {
  typedef typename cplx_of<T>::type C;
  typedef RowCfg<T, N, V> RC;
  if constexpr (!RC::VALID) {
    return no_tile();
  } else {
    static cudaError_t attr = allow_smem(k_row_nl<T, N, V, R>, RC::SMEM);
    TARA_CK(attr);
    const dim3 blocks((ny + 2 * RC::RP - 1) / (2 * RC::RP), nb);
    k_row_nl<T, N, V, R><<<blocks, RC::THREADS, RC::SMEM, s>>>((const C*)u, (C*)nl, g, (const C*)tw);
    TARA_CK(cudaGetLastError());
    return TARA_OK;
  }
}

template <typename T, int N, int V, int R>
static int launch_col_forward(int nh, const void* nl, const StepBufs& sb, const Grid2D& g,
                              const RhsParams& p, int mode, const void* tw, cudaStream_t s, int nb) {
  typedef typename cplx_of<T>::type C;
  typedef ColCfg<T, N, V> CF;
  if constexpr (!CF::VALID_C) {
    return no_tile();
  } else {
    static cudaError_t attr = allow_smem(k_col_forward<T, N, V, R>, CF::SMEM_C);
    TARA_CK(attr);
    const dim3 blocks((nh + CF::TCC - 1) / CF::TCC, nb);
    k_col_forward<T, N, V, R><<<blocks, CF::THREADS_C, CF::SMEM_C, s>>>((const C*)nl, sb, g, p, mode,
                                                                         (const C*)tw);
    TARA_CK(cudaGetLastError());
    return TARA_OK;
  }
}

template <typename T, int N, bool INV, int V>
static int launch_col_fft(int nh, int pitch, const void* in, void* out, const void* tw,
                          cudaStream_t s, int nf, size_t fs) {
  typedef typename cplx_of<T>::type C;
  typedef ColCfg<T, N, V> CF;
  static cudaError_t attr = allow_smem(k_col_fft<T, N, INV, V>, CF::SMEM_C);
  TARA_CK(attr);
  const dim3 blocks((nh + CF::TCC - 1) / CF::TCC, nf);
  k_col_fft<T, N, INV, V><<<blocks, CF::THREADS_C, CF::SMEM_C, s>>>((const C*)in, (C*)out, nh, pitch, fs,
                                                                     (const C*)tw);
  TARA_CK(cudaGetLastError());
  return TARA_OK;
}

template <typename T, int N, int V>
static int launch_row_c2r(int ny, int pitch, int rpitch, const void* in, void* out, const void* tw,
                          cudaStream_t s, int nf, size_t fs_in, size_t fs_out) {
  typedef typename cplx_of<T>::type C;
  typedef RowXCfg<T, N, V> RC;
  static cudaError_t attr = allow_smem(k_row_c2r<T, N, V>, RC::SMEM);
  TARA_CK(attr);
  const int per = 2 * RC::NP;
  const dim3 blocks((ny + per - 1) / per, nf);
  k_row_c2r<T, N, V><<<blocks, RC::THREADS, RC::SMEM, s>>>((const C*)in, (T*)out, ny, pitch, rpitch, fs_in,
                                                           fs_out, (const C*)tw);
  TARA_CK(cudaGetLastError());
  return TARA_OK;
}

template <typename T, int N, int V>
static int launch_row_r2c(int ny, int rpitch, int pitch, const void* in, void* out, const void* tw,
                          cudaStream_t s, int nf, size_t fs_in, size_t fs_out) {
  typedef typename cplx_of<T>::type C;
  typedef RowXCfg<T, N, V> RC;
  static cudaError_t attr = allow_smem(k_row_r2c<T, N, V>, RC::SMEM);
  TARA_CK(attr);
  const int per = 2 * RC::NP;
  const dim3 blocks((ny + per - 1) / per, nf);
  k_row_r2c<T, N, V><<<blocks, RC::THREADS, RC::SMEM, s>>>((const T*)in, (C*)out, ny, rpitch, pitch, fs_in,
                                                           fs_out, (const C*)tw);
  TARA_CK(cudaGetLastError());
  return TARA_OK;
}

// The plain transforms take the one-column / one-row-pair tiles when the
// default tiles would leave most SMs idle (FP64 work then spreads over more SMs).
constexpr int kFewCtas = 152;

template <typename T, int N>
static bool small_col(int nh, int nf) {
  return nf * ((nh + ColCfg<T, N>::TCC - 1) / ColCfg<T, N>::TCC) < kFewCtas;
}

template <typename T, int N>
static bool small_row(int ny, int nf) {
  return nf * ((ny + 2 * RowXCfg<T, N, 0>::NP - 1) / (2 * RowXCfg<T, N, 0>::NP)) < kFewCtas;
}

// The step kernels along radix path R, tile variant v (0-2; 3 for the row pass).
template <typename T, int R>
int step_col_inverse(int ny, int nh, const double2* win, void* u, const Grid2D& g, const RhsParams& p,
                     const void* twy, cudaStream_t s, int nb, int v) {
  if (v == 2) {
    TARA_SWITCH_N(ny, return (launch_col_inverse<T, N, 2, R>(nh, win, u, g, p, twy, s, nb)));
  } else if (v == 1) {
    TARA_SWITCH_N(ny, return (launch_col_inverse<T, N, 1, R>(nh, win, u, g, p, twy, s, nb)));
  } else {
    TARA_SWITCH_N(ny, return (launch_col_inverse<T, N, 0, R>(nh, win, u, g, p, twy, s, nb)));
  }
  return TARA_OK;
}

template <typename T, int R>
int step_row_nl(int nx, int ny, const void* u, void* nl, const Grid2D& g, const void* twx, cudaStream_t s,
                int nb, int v) {
  if (v == 3) {
    TARA_SWITCH_N(nx, return (launch_row_nl<T, N, 3, R>(ny, u, nl, g, twx, s, nb)));
  } else if (v == 2) {
    TARA_SWITCH_N(nx, return (launch_row_nl<T, N, 2, R>(ny, u, nl, g, twx, s, nb)));
  } else if (v == 1) {
    TARA_SWITCH_N(nx, return (launch_row_nl<T, N, 1, R>(ny, u, nl, g, twx, s, nb)));
  } else {
    TARA_SWITCH_N(nx, return (launch_row_nl<T, N, 0, R>(ny, u, nl, g, twx, s, nb)));
  }
  return TARA_OK;
}

template <typename T, int R>
int step_col_forward(int ny, int nh, const void* nl, const StepBufs& sb, const Grid2D& g, const RhsParams& p,
                     int mode, const void* twy, cudaStream_t s, int nb, int v) {
  if (v == 2) {
    TARA_SWITCH_N(ny, return (launch_col_forward<T, N, 2, R>(nh, nl, sb, g, p, mode, twy, s, nb)));
  } else if (v == 1) {
    TARA_SWITCH_N(ny, return (launch_col_forward<T, N, 1, R>(nh, nl, sb, g, p, mode, twy, s, nb)));
  } else {
    TARA_SWITCH_N(ny, return (launch_col_forward<T, N, 0, R>(nh, nl, sb, g, p, mode, twy, s, nb)));
  }
  return TARA_OK;
}

// Whether step kernel k (0 column inverse, 1 row, 2 column forward) has tile
// variant v (0-3) at length n.
template <typename T, int N>
static bool tile_fits_n(int k, int v) {
  if (k == 0)
    return v == 0 ? ColCfg<T, N, 0>::VALID_A : v == 1 ? ColCfg<T, N, 1>::VALID_A
           : v == 2 ? ColCfg<T, N, 2>::VALID_A : false;
  if (k == 1)
    return v == 0 ? RowCfg<T, N, 0>::VALID : v == 1 ? RowCfg<T, N, 1>::VALID
           : v == 2 ? RowCfg<T, N, 2>::VALID : v == 3 ? RowCfg<T, N, 3>::VALID : false;
  return v == 0 ? ColCfg<T, N, 0>::VALID_C : v == 1 ? ColCfg<T, N, 1>::VALID_C
         : v == 2 ? ColCfg<T, N, 2>::VALID_C : false;
}

// Lengths that are not powers of two go to the mixed-radix FP64 passes
// (generic2d.cu); they have one configuration (variant 0).
#define TARA_ANY_2D(n, CALL)                                                                 \
  if (!is_pow2_in_range(n)) {                                                                \
    if constexpr (std::is_same<T, double>::value) {                                          \
      if (any_size_2d(n)) return CALL;                                                       \
    }                                                                                        \
    return set_error(TARA_ERR_ARGS, "grid sizes that are not powers of two need FP64, even " \
                                    "lengths 8 to 3600 with factors 2, 3, 5, 7");            \
  }

template <typename T>
bool Launch2D<T>::tile_fits(int k, int n, int v) {
  if (!is_pow2_in_range(n)) return std::is_same<T, double>::value && any_size_2d(n) && v == 0;
  switch (n) {
    case 16: return tile_fits_n<T, 16>(k, v);
    case 32: return tile_fits_n<T, 32>(k, v);
    case 64: return tile_fits_n<T, 64>(k, v);
    case 128: return tile_fits_n<T, 128>(k, v);
    case 256: return tile_fits_n<T, 256>(k, v);
    case 512: return tile_fits_n<T, 512>(k, v);
    case 1024: return tile_fits_n<T, 1024>(k, v);
    case 2048: return tile_fits_n<T, 2048>(k, v);
    case 4096: return tile_fits_n<T, 4096>(k, v);
    default: return false;
  }
}

// The variant index of the step launchers carries the radix path in bit 2
// (v | 4: radix-8 path, FP64 and FP32 only; the double-float form ignores the
// bit) and the tile variant in bits 0-1.
template <typename T>
int Launch2D<T>::col_inverse(int ny, int nh, const double2* win, void* u, const Grid2D& g,
                             const RhsParams& p, const void* twy, cudaStream_t s, int nb, int v) {
  TARA_ANY_2D(ny, any2d::col_inverse(ny, nh, win, u, g, p, twy, s, nb))
  if constexpr (!is_df64<T>())
    if (v & 4) return step_col_inverse<T, 8>(ny, nh, win, u, g, p, twy, s, nb, v & 3);
  return step_col_inverse<T, 4>(ny, nh, win, u, g, p, twy, s, nb, v & 3);
}

template <typename T>
int Launch2D<T>::row_nl(int nx, int ny, const void* u, void* nl, const Grid2D& g, const void* twx,
                        cudaStream_t s, int nb, int v) {
  TARA_ANY_2D(nx, any2d::row_nl(nx, ny, u, nl, g, twx, s, nb))
  if constexpr (!is_df64<T>())
    if (v & 4) return step_row_nl<T, 8>(nx, ny, u, nl, g, twx, s, nb, v & 3);
  return step_row_nl<T, 4>(nx, ny, u, nl, g, twx, s, nb, v & 3);
}

template <typename T>
int Launch2D<T>::col_forward(int ny, int nh, const void* nl, const StepBufs& sb, const Grid2D& g,
                             const RhsParams& p, int mode, const void* twy, cudaStream_t s, int nb,
                             int v) {
  TARA_ANY_2D(ny, any2d::col_forward(ny, nh, nl, sb, g, p, mode, twy, s, nb))
  if constexpr (!is_df64<T>())
    if (v & 4) return step_col_forward<T, 8>(ny, nh, nl, sb, g, p, mode, twy, s, nb, v & 3);
  return step_col_forward<T, 4>(ny, nh, nl, sb, g, p, mode, twy, s, nb, v & 3);
}

// Explicit instantiations of the radix-8 step launchers live in their own
// translation units (launch_fp64_r8.cu, launch_fp32_r8.cu), which compile in
// parallel with the radix-4 ones.
#define TARA_STEP_R8_INSTANCES(EXT, T)                                                              \
  EXT template int step_col_inverse<T, 8>(int, int, const double2*, void*, const Grid2D&,            \
                                          const RhsParams&, const void*, cudaStream_t, int, int);    \
  EXT template int step_row_nl<T, 8>(int, int, const void*, void*, const Grid2D&, const void*,       \
                                     cudaStream_t, int, int);                                        \
  EXT template int step_col_forward<T, 8>(int, int, const void*, const StepBufs&, const Grid2D&,     \
                                          const RhsParams&, int, const void*, cudaStream_t, int, int);

template <typename T>
int Launch2D<T>::col_fft(int ny, int nh, int pitch, const void* in, void* out, bool inverse,
                         const void* twy, cudaStream_t s, int nf, size_t fs) {
  TARA_ANY_2D(ny, any2d::col_fft(ny, nh, pitch, in, out, inverse, twy, s, nf, fs))
  if (inverse) {
    TARA_SWITCH_N(ny, return (small_col<T, N>(nh, nf)
                                  ? launch_col_fft<T, N, true, 2>(nh, pitch, in, out, twy, s, nf, fs)
                                  : launch_col_fft<T, N, true, 0>(nh, pitch, in, out, twy, s, nf, fs)));
  } else {
    TARA_SWITCH_N(ny, return (small_col<T, N>(nh, nf)
                                  ? launch_col_fft<T, N, false, 2>(nh, pitch, in, out, twy, s, nf, fs)
                                  : launch_col_fft<T, N, false, 0>(nh, pitch, in, out, twy, s, nf, fs)));
  }
  return TARA_OK;
}

template <typename T>
int Launch2D<T>::row_c2r(int nx, int ny, int pitch, int rpitch, const void* in, void* out,
                         const void* twx, cudaStream_t s, int nf, size_t fs_in, size_t fs_out) {
  TARA_ANY_2D(nx, any2d::row_c2r(nx, ny, pitch, rpitch, in, out, twx, s, nf, fs_in, fs_out))
  TARA_SWITCH_N(nx, return (small_row<T, N>(ny, nf)
                                ? launch_row_c2r<T, N, 2>(ny, pitch, rpitch, in, out, twx, s, nf, fs_in, fs_out)
                                : launch_row_c2r<T, N, 0>(ny, pitch, rpitch, in, out, twx, s, nf, fs_in, fs_out)));
  return TARA_OK;
}

template <typename T>
int Launch2D<T>::row_r2c(int nx, int ny, int rpitch, int pitch, const void* in, void* out,
                         const void* twx, cudaStream_t s, int nf, size_t fs_in, size_t fs_out) {
  TARA_ANY_2D(nx, any2d::row_r2c(nx, ny, rpitch, pitch, in, out, twx, s, nf, fs_in, fs_out))
  TARA_SWITCH_N(nx, return (small_row<T, N>(ny, nf)
                                ? launch_row_r2c<T, N, 2>(ny, rpitch, pitch, in, out, twx, s, nf, fs_in, fs_out)
                                : launch_row_r2c<T, N, 0>(ny, rpitch, pitch, in, out, twx, s, nf, fs_in, fs_out)));
  return TARA_OK;
}

}  // namespace tara
