// tara_derive2csh_noalloc: the plain RHS (derive2csh) on caller-owned device
// arrays, with no device allocation of any kind.
//
// Who needs it: callers that cannot call cudaMalloc -- a host program whose
// device memory is entirely owned by another allocator (a framework's caching
// allocator, or a Fortran/C++ code that reserves its memory pool up front and
// forbids further allocation), and callers that must not pay the implicit
// device-wide synchronisation that cudaMalloc and cudaFree can trigger in the
// middle of a time loop.  The regular entry points allocate their work buffers
// on first use; this one never does.
//
// Where its scratch lives: one file-scope `static __device__` array,
// g_noalloc_scratch, of fixed size (kScratchBytes, about 2.9 MB) that every GPU
// which loads libtara holds until the process exits.  It carries the four
// y-inverse spectra, the products' spectrum, the twiddle tables, the
// wavenumber and 1/k^2 tables and the flag word that the forward column kernel
// sets on a non-finite value, for grids up to kNoAllocMaxN^2 = 256^2; larger
// grids are rejected with TARA_ERR_ARGS.
//
// Non-finite results are NOT reported: reading the flag back would need a
// device-to-host copy and a wait on the caller's stream, which this entry
// point leaves to the caller.  It returns TARA_OK whenever the launches were
// accepted, even if the right-hand side holds NaN or Inf; a caller that needs
// the check tests its output array (the regular drop-in derive2csh_ reports
// TARA_ERR_NONFINITE through tara_last_error instead).
//
// Host code cannot use the name g_noalloc_scratch as a device address (on the
// host it names a shadow variable).  The first call on each device, with that
// device current, resolves the real address with cudaGetSymbolAddress and
// uploads the twiddle tables with cudaMemcpy followed by cudaDeviceSynchronize
// (a copy from pageable memory may return before its DMA has landed, and a
// caller's non-blocking stream is not ordered after the legacy stream that
// carries it); that first call should therefore come before any stream
// capture.  Later calls only enqueue kernels on the caller's stream.
//
// Every call on a device shares the one array, and the array keeps what the last
// call wrote.  Each call rewrites everything it reads before reading it (the
// wavenumber tables are recomputed and the error flag is cleared at the start of
// every call), so results never depend on an earlier call.  Calls whose GPU work
// overlaps -- on different streams, or from different host threads -- race on
// the array and must be serialised by the caller.
#include <cmath>
#include <cstdint>
#include <mutex>

#include "internal.h"

namespace {

constexpr int kNoAllocMaxN = 256;
constexpr int kNhMax = kNoAllocMaxN / 2 + 1;
constexpr size_t kFieldElems = (size_t)kNoAllocMaxN * kNhMax;  // dense [Ny][Nh] at the maximum
using tara::tw_count;
constexpr int kTwElems = tw_count(16) + tw_count(32) + tw_count(64) + tw_count(128) + tw_count(256);

constexpr size_t align256(size_t b) { return (b + 255) / 256 * 256; }
constexpr size_t kOffU = 0;
constexpr size_t kOffNL = kOffU + align256(4 * kFieldElems * sizeof(double2));
constexpr size_t kOffTw = kOffNL + align256(kFieldElems * sizeof(double2));
constexpr size_t kOffKx = kOffTw + align256(kTwElems * sizeof(double2));
constexpr size_t kOffKy = kOffKx + align256(kNhMax * sizeof(double));
constexpr size_t kOffI0 = kOffKy + align256(kNoAllocMaxN * sizeof(double));
constexpr size_t kOffInv = kOffI0 + align256(kNoAllocMaxN * sizeof(int));
constexpr size_t kOffFlag = kOffInv + align256(kFieldElems * sizeof(double));
constexpr size_t kScratchBytes = kOffFlag + 256;

// offset of the length-n twiddle table inside the twiddle region (tables for
// 16, 32, ... n/2 precede it)
constexpr int tw_offset(int n) { return n <= 16 ? 0 : tw_offset(n / 2) + tw_count(n / 2); }

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
unsigned char* g_dev_ptr[kMaxDevices] = {};

}  // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

namespace tara {

// Wavenumbers and the 2/3-rule index of derive2csh in IEEE double with the
// host's operation order and no contraction (explicit _rn intrinsics), so the
// tables equal make_wavenumbers()'s bit for bit.
__global__ void k_noalloc_tables(int nx, int ny, double* kx, double* ky, int* i0, double* inv,
                                 unsigned int* flag) {
  const double kpi = (double)3.1428f;
  const double l = __dmul_rn(2.0, kpi);
  const int nh = nx / 2 + 1;
  const int t = threadIdx.x;
  if (t == 0) *flag = 0u;
  for (int i = t; i < nh; i += blockDim.x) kx[i] = __ddiv_rn(__dmul_rn(l, (double)i), l);
  for (int j = t; j < ny; j += blockDim.x)
    ky[j] = (j < ny / 2) ? __ddiv_rn(__dmul_rn(l, (double)j), l)
                         : __ddiv_rn(__dmul_rn(l, __dsub_rn((double)j, (double)ny)), l);
  __syncthreads();
  const double cut = __ddiv_rn(__ddiv_rn((double)(nx + ny), 2.0), 3.0);
  for (int j = t; j < ny; j += blockDim.x) {
    int first = nh;
    for (int i = nh - 1; i >= 0; --i) {
      const double k2 = __dadd_rn(__dmul_rn(kx[i], kx[i]), __dmul_rn(ky[j], ky[j]));
      if (__dsqrt_rn(k2) >= cut)
        first = i;
      else
        break;
    }
    i0[j] = first;
  }
  for (int q = t; q < ny * nh; q += blockDim.x) {
    const int j = q / nh, i = q % nh;
    const double k2 = __dadd_rn(__dmul_rn(kx[i], kx[i]), __dmul_rn(ky[j], ky[j]));
    inv[q] = (i == 0 && j == 0) ? 0.0 : __ddiv_rn(1.0, k2);
  }
}

// Resolve the device address of g_noalloc_scratch for the current device and
// upload the twiddle tables (once per device).
static int noalloc_setup(unsigned char** out) {
  int dev = 0;
  TARA_CK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return set_error(TARA_ERR_ARGS, "device index out of range");
  std::lock_guard<std::mutex> lk(g_setup_mu);
  if (!g_dev_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    double2 tw[kTwElems];
    for (int n = 16; n <= kNoAllocMaxN; n *= 2)
      for (int m = 0; m < tw_count(n); ++m) {
        double c, sn;
        twiddle_entry_fp64(n, m, &c, &sn);
        tw[tw_offset(n) + m] = make_double2(c, sn);
      }
    e = cudaMemcpy((unsigned char*)p + kOffTw, tw, sizeof(tw), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy(twiddles)");
    // the tables must be in device memory before any stream of the caller reads them
    e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return cuda_fail(e, "cudaDeviceSynchronize(twiddles)");
    g_dev_ptr[dev] = (unsigned char*)p;
  }
  *out = g_dev_ptr[dev];
  return TARA_OK;
}

}  // namespace tara

using namespace tara;

extern "C" int tara_derive2csh_noalloc(int nx, int ny, double nu, const void* omegak_dev,
                                       void* dt_omegak_dev, void* stream) {
  if (!is_pow2_in_range(nx) || !is_pow2_in_range(ny) || nx > kNoAllocMaxN || ny > kNoAllocMaxN)
    return set_error(TARA_ERR_ARGS,
                     "tara_derive2csh_noalloc: Nx and Ny must be powers of two in [16, 256]");
  if (!omegak_dev || !dt_omegak_dev || ((uintptr_t)omegak_dev & 15) || ((uintptr_t)dt_omegak_dev & 15))
    return set_error(TARA_ERR_ARGS, "tara_derive2csh_noalloc: null or misaligned device array");
  unsigned char* base = nullptr;
  int rc = noalloc_setup(&base);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  const int nh = nx / 2 + 1;
  double* kx = (double*)(base + kOffKx);
  double* ky = (double*)(base + kOffKy);
  int* i0 = (int*)(base + kOffI0);
  double* inv = (double*)(base + kOffInv);
  unsigned int* flag = (unsigned int*)(base + kOffFlag);
  double2* u = (double2*)(base + kOffU);
  double2* nl = (double2*)(base + kOffNL);
  const double2* tw = (const double2*)(base + kOffTw);
  k_noalloc_tables<<<1, 256, 0, s>>>(nx, ny, kx, ky, i0, inv, flag);
  TARA_CK(cudaGetLastError());
  Grid2D g;
  g.nx = nx;
  g.ny = ny;
  g.nh = nh;
  g.pitch = nh;  // the caller's dense Fortran layout; scratch uses the same pitch
  g.kx = kx;
  g.ky = ky;
  g.i0 = i0;
  g.inv = inv;
  {  // the same tables on the host (stack arrays) give the last column the 2/3 rule keeps
    double hkx[kNhMax], hky[kNoAllocMaxN];
    int hi0[kNoAllocMaxN];
    make_wavenumbers(nx, ny, (double)3.1428f, 2.0 * (double)3.1428f, 2.0 * (double)3.1428f, hkx,
                     hky, hi0);
    g.i0max = 0;
    for (int j = 0; j < ny; ++j) g.i0max = hi0[j] > g.i0max ? hi0[j] : g.i0max;
  }
  RhsParams p;
  p.rhs = TARA_RHS_PLAIN;
  p.nu = nu;
  p.alpha = 1.0;
  p.lambda = 0.0;
  p.dt = 0.0;
  const double nn = (double)nx * (double)ny;
  p.nl_scale = 0.5 / (nn * nn);
  p.nu_f = (float)nu;
  p.alpha_f = 1.0f;
  p.nl_scale_f = (float)p.nl_scale;
  g.kxf = g.kyf = g.invf = nullptr;  // FP64 kernels only
  g.kxd = g.kyd = g.invd = nullptr;
  StepBufs sb = {};
  sb.win = (const double2*)omegak_dev;
  sb.fout = (double2*)dt_omegak_dev;
  sb.flag = flag;
  if ((rc = Launch2D<double>::col_inverse(ny, nh, sb.win, u, g, p, tw + tw_offset(ny), s))) return rc;
  if ((rc = Launch2D<double>::row_nl(nx, ny, u, nl, g, tw + tw_offset(nx), s))) return rc;
  if ((rc = Launch2D<double>::col_forward(ny, nh, nl, sb, g, p, MODE_DERIVE, tw + tw_offset(ny), s)))
    return rc;
  return set_ok();
}
