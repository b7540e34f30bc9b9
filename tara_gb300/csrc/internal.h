// Internal host-side declarations shared by the translation units of libtara.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

#include <string>

#include "../../include/tara.h"
#include "kernels2d.cuh"
#include "status.h"

namespace tara {

// thread-local status (tara_last_error): set_error, set_ok, save/restore_error in status.h
int cuda_fail(cudaError_t e, const char* what);

#define TARA_CK(call)                                   \
  do {                                                  \
    cudaError_t e_ = (call);                            \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
  } while (0)

// Largest transform length: a 4096-point FP64 row pair fits the three-slot row
// tile (192 KB of shared memory), a column the one-column tiles (128 KB with
// its two field slots); longer lines would need a split transform.
constexpr int kMaxN = 4096;
inline bool is_pow2_in_range(int n) { return n >= 16 && n <= kMaxN && (n & (n - 1)) == 0; }
inline int round_up(int v, int m) { return (v + m - 1) / m * m; }

// Tile variants per step kernel (column inverse pass, row pass, column forward
// pass).  A kernel's configuration index is its tile variant in bits 0-1 and
// the radix-8 path in bit 2, so the autotuner weighs kCandidates indices.
constexpr int kVariants[3] = {3, 4, 3};
constexpr int kCandidates = 8;

// Philox4x32-10 on the host (Salmon et al., SC'11): ten rounds with the
// published multipliers and Weyl key increments, for the seeded phases of the
// random initial states.
inline void philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3], k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    c0 = hi1 ^ c1 ^ k0;
    c1 = lo1;
    c2 = hi0 ^ c3 ^ k1;
    c3 = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

// Host tables shared with the oracle's arithmetic: kx = 2*kpi*i/lx etc.
void make_wavenumbers(int nx, int ny, double kpi, double lx, double ly, double* kx, double* ky,
                      int* i0);
// inv[j*nh+i] = 1/(kx^2+ky^2 [+lambda]) (0 at the origin), same operation order as
// the RHS's denominators.
void make_inverse_table(int nx, int ny, const double* kx, const double* ky, bool screened,
                        double lambda, double* inv);

// Precision-dispatched launchers (one translation unit per precision).
template <typename T>
struct Launch2D {
  // nb: runs in the batch (grid dimension); v: tile variant (0 default, 1 half tile)
  static int col_inverse(int ny, int nh, const double2* win, void* u, const Grid2D& g,
                         const RhsParams& p, const void* twy, cudaStream_t s, int nb = 1,
                         int v = 0);
  static int row_nl(int nx, int ny, const void* u, void* nl, const Grid2D& g, const void* twx,
                    cudaStream_t s, int nb = 1, int v = 0);
  static int col_forward(int ny, int nh, const void* nl, const StepBufs& sb, const Grid2D& g,
                         const RhsParams& p, int mode, const void* twy, cudaStream_t s,
                         int nb = 1, int v = 0);
  // plain transforms of nf fields (fs / fs_in / fs_out elements apart)
  static int col_fft(int ny, int nh, int pitch, const void* in, void* out, bool inverse,
                     const void* twy, cudaStream_t s, int nf = 1, size_t fs = 0);
  static int row_c2r(int nx, int ny, int pitch, int rpitch, const void* in, void* out,
                     const void* twx, cudaStream_t s, int nf = 1, size_t fs_in = 0, size_t fs_out = 0);
  static int row_r2c(int nx, int ny, int rpitch, int pitch, const void* in, void* out,
                     const void* twx, cudaStream_t s, int nf = 1, size_t fs_in = 0, size_t fs_out = 0);
  // whether step kernel k (0 column inverse, 1 row pass, 2 column forward) has
  // tile variant v at length n (a tile must fit one CTA)
  static bool tile_fits(int k, int n, int v);
};

// Grid sizes that are not powers of two (generic2d.cu, fft_any.cuh): even,
// 8 to 3600, factors 2, 3, 5 and 7; FP64 only.  The Launch2D entry points route
// such lengths there.
bool any_size_2d(int n);
inline bool is_size_2d(int n) { return is_pow2_in_range(n) || any_size_2d(n); }
namespace any2d {
int col_inverse(int ny, int nh, const double2* win, void* u, const Grid2D& g, const RhsParams& p, const void* twy,
                cudaStream_t s, int nb);
int row_nl(int nx, int ny, const void* u, void* nl, const Grid2D& g, const void* twx, cudaStream_t s, int nb);
int col_forward(int ny, int nh, const void* nl, const StepBufs& sb, const Grid2D& g, const RhsParams& p, int mode,
                const void* twy, cudaStream_t s, int nb);
int col_fft(int ny, int nh, int pitch, const void* in, void* out, bool inverse, const void* twy, cudaStream_t s,
            int nf, size_t fs);
int row_c2r(int nx, int ny, int pitch, int rpitch, const void* in, void* out, const void* twx, cudaStream_t s, int nf,
            size_t fs_in, size_t fs_out);
int row_r2c(int nx, int ny, int rpitch, int pitch, const void* in, void* out, const void* twx, cudaStream_t s, int nf,
            size_t fs_in, size_t fs_out);
int make_roots(int n, void** dev);  // exp(-2 pi i t / n), t < n, FP64
}  // namespace any2d

// Twiddle exp(-2 pi i m/n) in FP64 with tw[n - m] = conj(tw[m]) exactly.
void twiddle(int n, int m, double* re, double* im);
// Entry idx < tw_count(n) of the length-n twiddle table (layout in fft.cuh).
void twiddle_entry(int n, int idx, double* re, double* im);
// The FP64 table's entry idx: the radix-4 stage entries in ratio form (fft.cuh).
void twiddle_entry_fp64(int n, int idx, double* a, double* b);
// Twiddle table exp(-2 pi i m/n), m < n, in precision T, uploaded to device.
int make_twiddles(int n, bool fp32, void** dev);
// The same table as double-float (hi, lo) pairs: float4 {re.hi, re.lo, im.hi, im.lo}.
int make_twiddles_df64(int n, void** dev);

}  // namespace tara

struct tara2d {
  tara2d_config cfg;
  int batch = 1;          // runs advanced together (ensembles)
  int var[3] = {0, 0, 0};  // tile variants of the three kernels (autotuner)
  int dev = 0;
  int nx = 0, ny = 0, nh = 0, pitch = 0;
  cudaStream_t stream = nullptr;
  double2 *w0 = nullptr, *ws = nullptr, *acc = nullptr, *fold = nullptr, *fout = nullptr;
  void* u = nullptr;   // 4 fields of the y-inverse pass, precision of cfg
  void* nl = nullptr;  // x-r2c output of the products
  double *kx = nullptr, *ky = nullptr, *inv = nullptr;
  float* tabf = nullptr;  // kx, ky, inv in FP32 (nh + ny + nh*ny floats)
  tara::df64* tabd = nullptr;  // kx, ky, inv in double-float (double-float mode only)
  int* i0 = nullptr;
  void *twx = nullptr, *twy = nullptr;
  double *diag_part = nullptr, *diag_out = nullptr;
  unsigned int* flag = nullptr;
  const double2* force = nullptr;  // closure forcing spectrum (batch fields), not owned
  void* scratch = nullptr;         // filter / spectrum / real-state work space
  void* stage = nullptr;           // one dense field for page-locked host copies (lazy)
  size_t scratch_bytes = 0;
  void *twx64 = nullptr, *twy64 = nullptr;  // FP64 twiddles when the solver runs FP32
  tara::Grid2D grid;
  tara::RhsParams rp;
};

// Fortran common block /comm/: one symbol shared by the reference programs, each
// reading its own layout over it (the 3D code's below; the 2D compressible
// code's Lx, Ly, mux, muy, ms, CS, dt in coh2d.cu).  A Fortran caller that links
// libtara supplies it; mhd3d.cu holds a weak definition so the library loads alone.
struct TaraMhdCommon {
  int32_t iret, thread_num;
  double time_max, Lx, Ly, Lz, dx, dy, dz, spheat, mu, ms, CS, mu_0, eta, dt, kf;
};
extern "C" TaraMhdCommon comm_;

namespace tara {
// One RHS evaluation of `win` followed by the update of `mode`; when ev is not
// null, ev[0..2] are recorded on the handle's stream after the three launches.
int rhs_and_update(tara2d* h, const double2* win, int mode, cudaEvent_t* ev);
int copy_in_dense(tara2d* h, double2* dst, const double* host);
int copy_out_dense(tara2d* h, double* host, const double2* src);
int refresh_tables(tara2d* h);
// Scratch of at least `bytes` on the handle (kept until destroy).
int scratch(tara2d* h, size_t bytes, void** out);
// FP64 twiddles for the handle's grid, whatever the solver's precision.
int twiddles64(tara2d* h, const void** twx, const void** twy);

// Learned-closure internals (fno.cu).
int fno_forward_async(tara_fno* f, const float* x_dev, int B, const float** y);
void fno_bind_stream(tara_fno* f, cudaStream_t s);
void fno_bind_error(tara_fno* f, unsigned int* w);  // nullptr: the handle's own word
const tara_fno_config& fno_config(const tara_fno* f);
float* fno_input(tara_fno* f);  // the handle's input buffer (max_batch samples)
unsigned long long fno_param_version(const tara_fno* f);
int fno_prepare(tara_fno* f);
// Destroy the contexts the Fortran drop-ins keep per grid shape.  Each file
// that holds such a cache defines its function; tara_finalize calls them all.
int release_dropins_2d();
int release_dropins_3d();
int release_dropins_coh();
int release_dropins_com();
}  // namespace tara
