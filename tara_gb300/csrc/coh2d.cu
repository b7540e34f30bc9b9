// 2D compressible isothermal hydrodynamics: the reference's derive2coh
// (src/derive2coh.f95:6-265) and ab2coh (src/ab2coh.f95:5-34) on the GPU, and
// the initial state of its driver tara2dHydOMP (src/main2coh.f95:140-210).
//
// State: density and velocity spectra (nk, ukx, uky), each a half spectrum
// [Ny][pitch] of double2 like the vorticity solver's.  One right-hand side:
//   1. k_coh_spectra   11 spectra from the state: n, ux, uy, i kx n, i ky n,
//                      i kx ux, i ky ux, i kx uy, i ky uy, and the viscous
//                      spectra (mux kx^2 + muy ky^2) ux, (mux kx^2 + muy ky^2) uy
//   2. col_fft + row_c2r   the 11 inverse transforms (FFTW c2r semantics)
//   3. k_coh_real      per grid point, after the 1/(Nx Ny) normalisation:
//                        F_n = ux dn_dx + uy dn_dy + n (dux_dx + duy_dy)
//                        F_x = ux dux_dx + uy dux_dy + visc_x / n + CS^2 dn_dx / n
//                        F_y = ux duy_dx + uy duy_dy + visc_y / n + CS^2 dn_dy / n
//   4. row_r2c + col_fft   the 3 forward transforms
//   5. k_coh_final     the 2/3 rule (|k| >= (Nx+Ny)/6 removed), d/dt = -F, and
//                      the AB2 update with the history rotation of
//                      src/main2coh.f95:277-298 (or the bare derivative)
// The reference transforms 13 fields back and 9 forward and combines the 9
// forward spectra afterwards (src/derive2coh.f95:249-256); the transforms are
// linear and share one truncation mask, so here the viscous pairs are combined
// before the inverse transform (mux Viscxx + muy Viscxy = (mux d2ux_dx2 +
// muy d2ux_dy2)/n) and the momentum terms before the forward one: 11 c2r and
// 3 r2c per RHS instead of 13 and 9, equal up to rounding.
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "internal.h"

struct tara_coh2d {
  tara_coh2d_config cfg;
  int dev = 0, nx = 0, ny = 0, nh = 0, pitch = 0, rpitch = 0;
  size_t fs = 0, rfs = 0;  // elements of one spectrum / one real field
  cudaStream_t stream = nullptr;
  double2 *st = nullptr, *hist = nullptr, *dnew = nullptr, *spec = nullptr;
  double *real = nullptr, *prod = nullptr;
  double *kx = nullptr, *ky = nullptr;
  double* diag = nullptr;  // per-block partial sums of the driver diagnostics
  int* i0 = nullptr;
  void *twx = nullptr, *twy = nullptr;
  unsigned int* flag = nullptr;
};

namespace tara {
namespace {

constexpr int kCohSpectra = 11;
constexpr int kElemBlocks = 152 * 8, kElemThreads = 256;

__global__ void k_coh_spectra(const double2* __restrict__ st, size_t fs, const double* __restrict__ kx,
                              const double* __restrict__ ky, int nh, int ny, int pitch, double mux,
                              double muy, double2* __restrict__ sp) {
  const size_t total = (size_t)ny * nh;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const int y = (int)(t / nh), x = (int)(t % nh);
    const size_t q = (size_t)y * pitch + x;
    const double2 n = st[q], ux = st[fs + q], uy = st[2 * fs + q];
    const double a = kx[x], b = ky[y];
    sp[q] = n;
    sp[fs + q] = ux;
    sp[2 * fs + q] = uy;
    // (0,1) k f = (-k Im f, k Re f)  (src/derive2coh.f95:57-65)
    sp[3 * fs + q] = make_double2(-a * n.y, a * n.x);
    sp[4 * fs + q] = make_double2(-b * n.y, b * n.x);
    sp[5 * fs + q] = make_double2(-a * ux.y, a * ux.x);
    sp[6 * fs + q] = make_double2(-b * ux.y, b * ux.x);
    sp[7 * fs + q] = make_double2(-a * uy.y, a * uy.x);
    sp[8 * fs + q] = make_double2(-b * uy.y, b * uy.x);
    // mux kx^2 f + muy ky^2 f  (:66-69, combined as :249-250 combines them)
    const double vk = mux * (a * a) + muy * (b * b);
    sp[9 * fs + q] = make_double2(vk * ux.x, vk * ux.y);
    sp[10 * fs + q] = make_double2(vk * uy.x, vk * uy.y);
  }
}

// src/derive2coh.f95:140-169 with the momentum terms combined
__global__ void k_coh_real(const double* __restrict__ re, size_t rfs, int nx, int ny, int rpitch,
                           double inv_nn, double cs2, double* __restrict__ pr) {
  const size_t total = (size_t)ny * nx;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const size_t r = (t / nx) * rpitch + (t % nx);
    double v[kCohSpectra];
#pragma unroll
    for (int f = 0; f < kCohSpectra; ++f) v[f] = re[f * rfs + r] * inv_nn;
    const double n = v[0], ux = v[1], uy = v[2], dn_dx = v[3], dn_dy = v[4];
    const double dux_dx = v[5], dux_dy = v[6], duy_dx = v[7], duy_dy = v[8];
    const double inv_n = 1.0 / n;
    pr[r] = ux * dn_dx + uy * dn_dy + n * (dux_dx + duy_dy);
    pr[rfs + r] = (ux * dux_dx + uy * dux_dy) + v[9] * inv_n + cs2 * (dn_dx * inv_n);
    pr[2 * rfs + r] = (ux * duy_dx + uy * duy_dy) + v[10] * inv_n + cs2 * (dn_dy * inv_n);
  }
}

// 2/3 rule, d/dt = -F (:205-256); mode 0 writes the derivative to dnew, mode 1
// advances the state by AB2 and rotates the history (src/ab2coh.f95:19-27).
__global__ void k_coh_final(const double2* __restrict__ sp, size_t fs, const int* __restrict__ i0, int nh,
                            int ny, int pitch, int mode, double dt, double2* st, double2* hist,
                            double2* __restrict__ dnew, unsigned int* flag) {
  const size_t total = (size_t)ny * nh;
  bool bad = false;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const int y = (int)(t / nh), x = (int)(t % nh);
    const size_t q = (size_t)y * pitch + x;
    const bool keep = x < i0[y];
#pragma unroll
    for (int f = 0; f < 3; ++f) {
      const size_t o = f * fs + q;
      double2 d = make_double2(0.0, 0.0);
      if (keep) {
        const double2 v = sp[o];
        d = make_double2(-v.x, -v.y);
      }
      bad |= !(finite_bits(d.x) && finite_bits(d.y));
      if (mode == 0) {
        dnew[o] = d;
      } else {
        const double2 s = st[o], fo = hist[o];
        st[o] = make_double2(s.x + ((3.0 / 2.0) * d.x - (1.0 / 2.0) * fo.x) * dt,
                             s.y + ((3.0 / 2.0) * d.y - (1.0 / 2.0) * fo.y) * dt);
        hist[o] = d;
      }
    }
  }
  if (bad) atomicOr(flag, 1u);
}

// velocity spectra from the vorticity spectrum, psi = omega/k^2 (psi(1,1) = 0),
// ukx = (0,1) ky psi, uky = -(0,1) kx psi  (src/main2coh.f95:174-205)
__global__ void k_coh_velocity(const double2* __restrict__ wk, const double* __restrict__ kx,
                               const double* __restrict__ ky, int nh, int ny, int pitch,
                               double2* __restrict__ ukx, double2* __restrict__ uky) {
  const size_t total = (size_t)ny * nh;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const int y = (int)(t / nh), x = (int)(t % nh);
    const size_t q = (size_t)y * pitch + x;
    double2 a = make_double2(0.0, 0.0), b = a;
    if (x != 0 || y != 0) {
      const double k2 = kx[x] * kx[x] + ky[y] * ky[y];
      const double2 w = wk[q];
      const double pr = w.x / k2, pim = w.y / k2;
      a = make_double2(-ky[y] * pim, ky[y] * pr);
      b = make_double2(kx[x] * pim, -(kx[x] * pr));
    }
    ukx[q] = a;
    uky[q] = b;
  }
}

// Driver diagnostics (src/main2coh.f95:301-429): n, ux, uy and the vorticity
// omega_k = (0,1) kx uky - (0,1) ky ukx on the grid.
__global__ void k_coh_diag_spec(const double2* __restrict__ st, size_t fs, const double* __restrict__ kx,
                                const double* __restrict__ ky, int nh, int ny, int pitch,
                                double2* __restrict__ sp) {
  const size_t total = (size_t)ny * nh;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const int y = (int)(t / nh), x = (int)(t % nh);
    const size_t q = (size_t)y * pitch + x;
    const double2 ux = st[fs + q], uy = st[2 * fs + q];
    const double a = kx[x], b = ky[y];
    sp[q] = st[q];
    sp[fs + q] = ux;
    sp[2 * fs + q] = uy;
    sp[3 * fs + q] = make_double2((-a * uy.y) - (-b * ux.y), (a * uy.x) - (b * ux.x));
  }
}

constexpr int kDiagBlocksC = 304;

// Per-block sums of ux^2 + uy^2, uy^2, omega^0..3 (:396-405); the real fields
// are the unnormalised c2r outputs, divided by Nx Ny here as the reference does.
__global__ void __launch_bounds__(256) k_coh_diag_sum(const double* __restrict__ re, size_t rfs, int nx, int ny,
                                                      int rpitch, double nn, double* __restrict__ part) {
  double acc[6] = {0, 0, 0, 0, 0, 0};
  const size_t total = (size_t)ny * nx;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const size_t r = (t / nx) * rpitch + (t % nx);
    const double ux = re[rfs + r] / nn, uy = re[2 * rfs + r] / nn, w = re[3 * rfs + r] / nn;
    acc[0] += ux * ux + uy * uy;
    acc[1] += uy * uy;
    acc[2] += pow(w, 0.0);
    acc[3] += pow(w, 1.0);
    acc[4] += pow(w, 2.0);
    acc[5] += pow(w, 3.0);
  }
  __shared__ double sh[6][8];
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    double v = acc[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) sh[k][threadIdx.x >> 5] = v;
  }
  __syncthreads();
  if (threadIdx.x < 6) {
    double v = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += sh[threadIdx.x][w];
    part[blockIdx.x * 6 + threadIdx.x] = v;
  }
}

int coh_copy_in(tara_coh2d* h, double2* dst, const double* host) {
  TARA_CK(cudaMemcpy2DAsync(dst, h->pitch * sizeof(double2), host, h->nh * sizeof(double2),
                            h->nh * sizeof(double2), h->ny, cudaMemcpyHostToDevice, h->stream));
  return TARA_OK;
}

int coh_copy_out(tara_coh2d* h, double* host, const double2* src) {
  TARA_CK(cudaMemcpy2DAsync(host, h->nh * sizeof(double2), src, h->pitch * sizeof(double2),
                            h->nh * sizeof(double2), h->ny, cudaMemcpyDeviceToHost, h->stream));
  return TARA_OK;
}

// One right-hand side of the current state; mode 0 derivative into dnew, 1 AB2.
int coh_rhs(tara_coh2d* h, int mode) {
  const tara_coh2d_config& c = h->cfg;
  cudaStream_t s = h->stream;
  int rc;
  k_coh_spectra<<<kElemBlocks, kElemThreads, 0, s>>>(h->st, h->fs, h->kx, h->ky, h->nh, h->ny, h->pitch,
                                                      c.mux, c.muy, h->spec);
  TARA_CK(cudaGetLastError());
  if ((rc = Launch2D<double>::col_fft(h->ny, h->nh, h->pitch, h->spec, h->spec, true, h->twy, s, kCohSpectra,
                                      h->fs)))
    return rc;
  if ((rc = Launch2D<double>::row_c2r(h->nx, h->ny, h->pitch, h->rpitch, h->spec, h->real, h->twx, s,
                                      kCohSpectra, h->fs, h->rfs)))
    return rc;
  const double nn = (double)h->nx * (double)h->ny;
  k_coh_real<<<kElemBlocks, kElemThreads, 0, s>>>(h->real, h->rfs, h->nx, h->ny, h->rpitch, 1.0 / nn,
                                                   c.cs * c.cs, h->prod);
  TARA_CK(cudaGetLastError());
  if ((rc = Launch2D<double>::row_r2c(h->nx, h->ny, h->rpitch, h->pitch, h->prod, h->spec, h->twx, s, 3,
                                      h->rfs, h->fs)))
    return rc;
  if ((rc = Launch2D<double>::col_fft(h->ny, h->nh, h->pitch, h->spec, h->spec, false, h->twy, s, 3, h->fs)))
    return rc;
  k_coh_final<<<kElemBlocks, kElemThreads, 0, s>>>(h->spec, h->fs, h->i0, h->nh, h->ny, h->pitch, mode, c.dt,
                                                    h->st, h->hist, h->dnew, h->flag);
  TARA_CK(cudaGetLastError());
  return TARA_OK;
}

int coh_check(tara_coh2d* h) {
  unsigned int f = 0;
  TARA_CK(cudaMemcpyAsync(&f, h->flag, sizeof(f), cudaMemcpyDeviceToHost, h->stream));
  TARA_CK(cudaStreamSynchronize(h->stream));
  if (f) return set_error(TARA_ERR_NONFINITE, "non-finite value in the compressible update");
  return TARA_OK;
}

// Fortran common block /comm/ as src/derive2coh.f95:30 and src/ab2coh.f95:13 read it.
struct CohCommon {
  double Lx, Ly, mux, muy, ms, CS, dt;
};
static_assert(sizeof(CohCommon) <= sizeof(TaraMhdCommon), "the common block storage holds both views");

std::mutex g_coh_mu;
std::map<std::tuple<int, int>, tara_coh2d*> g_coh_ctx;

// Context of a shape for the drop-ins, its parameters refreshed per call.
tara_coh2d* coh_ctx(int nx, int ny, double pi) {
  CohCommon cm;  // a copy: the block's storage is declared with the 3D layout
  std::memcpy(&cm, &comm_, sizeof cm);
  if (!(cm.Lx > 0.0) || !(cm.Ly > 0.0)) {
    set_error(TARA_ERR_ARGS, "/comm/ Lx and Ly must be positive");
    return nullptr;
  }
  auto key = std::make_tuple(nx, ny);
  tara_coh2d* h = nullptr;
  auto it = g_coh_ctx.find(key);
  if (it != g_coh_ctx.end()) {
    h = it->second;
  } else {
    tara_coh2d_config c;
    c.nx = nx;
    c.ny = ny;
    c.kpi = pi;
    c.lx = cm.Lx;
    c.ly = cm.Ly;
    c.mux = cm.mux;
    c.muy = cm.muy;
    c.cs = cm.CS;
    c.dt = cm.dt;
    if (tara_coh2d_create(&c, &h) != TARA_OK) return nullptr;
    g_coh_ctx[key] = h;
  }
  tara_coh2d_config& c = h->cfg;
  if (c.kpi != pi || c.lx != cm.Lx || c.ly != cm.Ly) {
    c.kpi = pi;
    c.lx = cm.Lx;
    c.ly = cm.Ly;
    std::vector<double> kx(h->nh), ky(h->ny);
    std::vector<int> i0(h->ny);
    make_wavenumbers(h->nx, h->ny, c.kpi, c.lx, c.ly, kx.data(), ky.data(), i0.data());
    if (cudaMemcpy(h->kx, kx.data(), h->nh * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(h->ky, ky.data(), h->ny * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(h->i0, i0.data(), h->ny * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess) {
      set_error(TARA_ERR_CUDA, "wavenumber upload");
      return nullptr;
    }
  }
  c.mux = cm.mux;
  c.muy = cm.muy;
  c.cs = cm.CS;
  c.dt = cm.dt;
  return h;
}

bool coh_dims(const int* Nx, const int* Ny, const int* Nh, const double* pi) {
  if (!Nx || !Ny || !Nh || !pi) {
    set_error(TARA_ERR_ARGS, "null argument");
    return false;
  }
  if (!is_size_2d(*Nx) || !is_size_2d(*Ny) || *Nh != *Nx / 2 + 1) {
    set_error(TARA_ERR_ARGS,
              "Nx, Ny must be powers of two in [16, 4096] or even lengths 8 to 3600 with factors 2, 3, 5, 7, "
              "and Nh = Nx/2+1");
    return false;
  }
  return true;
}

}  // namespace
}  // namespace tara

using namespace tara;

extern "C" {

void tara_coh2d_default_config(tara_coh2d_config* c, int nx, int ny) {
  if (!c) return;
  const double pi = 3.14159265358979323846;
  c->nx = nx;
  c->ny = ny;
  c->kpi = pi;
  c->lx = 2.0 * pi;
  c->ly = 2.0 * pi;
  c->mux = 0.00020;  // src/main2coh.f95:120-121
  c->muy = 0.00020;
  c->cs = 1.8850 / 0.50;  // U0/M (:127-133)
  c->dt = 1e-3;
}

int tara_coh2d_destroy(tara_coh2d* h) {
  if (!h) return set_ok();
  cudaSetDevice(h->dev);
  if (h->stream) cudaStreamSynchronize(h->stream);
  void* ptrs[] = {h->st, h->hist, h->dnew, h->spec, h->real, h->prod, h->kx, h->ky, h->diag, h->i0, h->twx, h->twy,
                  h->flag};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return set_ok();
}

int tara_coh2d_create(const tara_coh2d_config* cfg, tara_coh2d** out) {
  if (!cfg || !out) return set_error(TARA_ERR_ARGS, "null argument");
  *out = nullptr;
  if (!is_size_2d(cfg->nx) || !is_size_2d(cfg->ny))
    return set_error(TARA_ERR_ARGS,
                     "nx and ny must be powers of two in [16, 4096] or even lengths 8 to 3600 with factors 2, 3, 5, 7");
  if (!(cfg->lx > 0.0) || !(cfg->ly > 0.0) || !(cfg->kpi > 0.0))
    return set_error(TARA_ERR_ARGS, "box lengths and kpi must be positive");
  tara_coh2d* h = new tara_coh2d();
  h->cfg = *cfg;
  h->nx = cfg->nx;
  h->ny = cfg->ny;
  h->nh = cfg->nx / 2 + 1;
  h->pitch = round_up(h->nh, 8);
  h->rpitch = round_up(h->nx, 8);
  h->fs = (size_t)h->ny * h->pitch;
  h->rfs = (size_t)h->ny * h->rpitch;
  auto fail = [&](int code) {  // free the half-built handle, keep the error
    const ErrorState saved = save_error();
    tara_coh2d_destroy(h);
    restore_error(saved);
    return code;
  };
#define CKC(call)                                              \
  do {                                                         \
    cudaError_t e_ = (call);                                   \
    if (e_ != cudaSuccess) return fail(cuda_fail(e_, #call)); \
  } while (0)
  CKC(cudaGetDevice(&h->dev));
  CKC(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
  const size_t sb = h->fs * sizeof(double2), rb = h->rfs * sizeof(double);
  CKC(cudaMalloc(&h->st, 3 * sb));
  CKC(cudaMalloc(&h->hist, 3 * sb));
  CKC(cudaMalloc(&h->dnew, 3 * sb));
  CKC(cudaMalloc(&h->spec, kCohSpectra * sb));
  CKC(cudaMalloc(&h->real, kCohSpectra * rb));
  CKC(cudaMalloc(&h->prod, 3 * rb));
  CKC(cudaMalloc(&h->kx, h->nh * sizeof(double)));
  CKC(cudaMalloc(&h->ky, h->ny * sizeof(double)));
  CKC(cudaMalloc(&h->i0, h->ny * sizeof(int)));
  CKC(cudaMalloc(&h->flag, sizeof(unsigned int)));
  CKC(cudaMalloc(&h->diag, 6 * kDiagBlocksC * sizeof(double)));
  CKC(cudaMemsetAsync(h->st, 0, 3 * sb, h->stream));
  CKC(cudaMemsetAsync(h->hist, 0, 3 * sb, h->stream));
  CKC(cudaMemsetAsync(h->dnew, 0, 3 * sb, h->stream));
  CKC(cudaMemsetAsync(h->spec, 0, kCohSpectra * sb, h->stream));
  CKC(cudaMemsetAsync(h->flag, 0, sizeof(unsigned int), h->stream));
#undef CKC
  int rc;
  if ((rc = make_twiddles(h->nx, false, &h->twx)) || (rc = make_twiddles(h->ny, false, &h->twy))) return fail(rc);
  std::vector<double> kx(h->nh), ky(h->ny);
  std::vector<int> i0(h->ny);
  make_wavenumbers(h->nx, h->ny, cfg->kpi, cfg->lx, cfg->ly, kx.data(), ky.data(), i0.data());
  if (cudaMemcpy(h->kx, kx.data(), h->nh * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(h->ky, ky.data(), h->ny * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(h->i0, i0.data(), h->ny * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess)
    return fail(set_error(TARA_ERR_CUDA, "wavenumber upload"));
  if (cudaStreamSynchronize(h->stream) != cudaSuccess) return fail(set_error(TARA_ERR_CUDA, "create"));
  *out = h;
  return set_ok();
}

int tara_coh2d_set_state(tara_coh2d* h, const double* state3, const double* hist3) {
  if (!h || !state3) return set_error(TARA_ERR_ARGS, "null argument");
  TARA_CK(cudaSetDevice(h->dev));
  const size_t dn = 2 * (size_t)h->nh * h->ny;  // doubles of one dense spectrum
  int rc;
  for (int f = 0; f < 3; ++f) {
    if ((rc = coh_copy_in(h, h->st + f * h->fs, state3 + f * dn))) return rc;
    if (hist3) {
      if ((rc = coh_copy_in(h, h->hist + f * h->fs, hist3 + f * dn))) return rc;
    }
  }
  if (!hist3) TARA_CK(cudaMemsetAsync(h->hist, 0, 3 * h->fs * sizeof(double2), h->stream));
  TARA_CK(cudaStreamSynchronize(h->stream));
  return set_ok();
}

int tara_coh2d_get_state(tara_coh2d* h, double* state3, double* hist3) {
  if (!h || !state3) return set_error(TARA_ERR_ARGS, "null argument");
  TARA_CK(cudaSetDevice(h->dev));
  const size_t dn = 2 * (size_t)h->nh * h->ny;
  int rc;
  for (int f = 0; f < 3; ++f) {
    if ((rc = coh_copy_out(h, state3 + f * dn, h->st + f * h->fs))) return rc;
    if (hist3 && (rc = coh_copy_out(h, hist3 + f * dn, h->hist + f * h->fs))) return rc;
  }
  TARA_CK(cudaStreamSynchronize(h->stream));
  return set_ok();
}

int tara_coh2d_rhs(tara_coh2d* h, double* d3) {
  if (!h || !d3) return set_error(TARA_ERR_ARGS, "null argument");
  TARA_CK(cudaSetDevice(h->dev));
  int rc;
  if ((rc = coh_rhs(h, 0))) return rc;
  const size_t dn = 2 * (size_t)h->nh * h->ny;
  for (int f = 0; f < 3; ++f)
    if ((rc = coh_copy_out(h, d3 + f * dn, h->dnew + f * h->fs))) return rc;
  if ((rc = coh_check(h))) return rc;
  return set_ok();
}

int tara_coh2d_step(tara_coh2d* h, int nsteps) {
  if (!h || nsteps < 0) return set_error(TARA_ERR_ARGS, "bad argument");
  TARA_CK(cudaSetDevice(h->dev));
  int rc;
  for (int s = 0; s < nsteps; ++s)
    if ((rc = coh_rhs(h, 1))) return rc;
  return set_ok();
}

int tara_coh2d_synchronize(tara_coh2d* h) {
  if (!h) return set_error(TARA_ERR_ARGS, "null handle");
  TARA_CK(cudaSetDevice(h->dev));
  int rc;
  if ((rc = coh_check(h))) return rc;
  return set_ok();
}

void* tara_coh2d_stream(tara_coh2d* h) { return h ? (void*)h->stream : nullptr; }

// n, ux, uy, omega of the current state on the grid (real spectra of the c2r
// divided by Nx Ny) into h->real[0..3].
static int coh_grid_fields(tara_coh2d* h) {
  int rc;
  k_coh_diag_spec<<<kElemBlocks, kElemThreads, 0, h->stream>>>(h->st, h->fs, h->kx, h->ky, h->nh, h->ny,
                                                                h->pitch, h->spec);
  TARA_CK(cudaGetLastError());
  if ((rc = Launch2D<double>::col_fft(h->ny, h->nh, h->pitch, h->spec, h->spec, true, h->twy, h->stream, 4, h->fs)))
    return rc;
  return Launch2D<double>::row_c2r(h->nx, h->ny, h->pitch, h->rpitch, h->spec, h->real, h->twx, h->stream, 4,
                                   h->fs, h->rfs);
}

int tara_coh2d_diag(tara_coh2d* h, double* out6) {
  if (!h || !out6) return set_error(TARA_ERR_ARGS, "null argument");
  TARA_CK(cudaSetDevice(h->dev));
  int rc;
  if ((rc = coh_grid_fields(h))) return rc;
  const double nn = (double)h->nx * (double)h->ny;
  double* part = h->diag;  // 6 x kDiagBlocksC doubles
  k_coh_diag_sum<<<kDiagBlocksC, 256, 0, h->stream>>>(h->real, h->rfs, h->nx, h->ny, h->rpitch, nn, part);
  TARA_CK(cudaGetLastError());
  std::vector<double> hp(6 * kDiagBlocksC);
  TARA_CK(cudaMemcpyAsync(hp.data(), part, hp.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  if ((rc = coh_check(h))) return rc;
  double s[6] = {0, 0, 0, 0, 0, 0};
  for (int b = 0; b < kDiagBlocksC; ++b)
    for (int k = 0; k < 6; ++k) s[k] += hp[b * 6 + k];
  out6[0] = s[0] / (2.0 * nn);  // Energy/(2 Nx Ny)
  out6[1] = s[1] / (2.0 * nn);  // y_Energy/(2 Nx Ny)
  for (int k = 2; k < 6; ++k) out6[k] = s[k] / nn;  // C0..C3/(Nx Ny)
  return set_ok();
}

int tara_coh2d_real_fields(tara_coh2d* h, double* n, double* ux, double* uy, double* omega) {
  if (!h) return set_error(TARA_ERR_ARGS, "null handle");
  TARA_CK(cudaSetDevice(h->dev));
  int rc;
  if ((rc = coh_grid_fields(h))) return rc;
  double* outs[4] = {n, ux, uy, omega};
  std::vector<double> buf(h->rfs);
  const double nn = (double)h->nx * (double)h->ny;
  for (int f = 0; f < 4; ++f) {
    if (!outs[f]) continue;
    TARA_CK(cudaMemcpyAsync(buf.data(), h->real + f * h->rfs, h->rfs * sizeof(double), cudaMemcpyDeviceToHost,
                            h->stream));
    TARA_CK(cudaStreamSynchronize(h->stream));
    for (int j = 0; j < h->ny; ++j)
      for (int i = 0; i < h->nx; ++i) outs[f][(size_t)j * h->nx + i] = buf[(size_t)j * h->rpitch + i] / nn;
  }
  return set_ok();
}

int tara_coh2d_launches_per_step(tara_coh2d* h) { return h ? 7 : 0; }

// src/main2coh.f95:140-210: n = n0 = 1; omega = 1 in the disk of radius
// 0.3*2*pi about the centre, 10 in five disks of radius 0.2 at distance
// 0.4*2*pi; x(i) = 0.0d0+real(i-1)*dx with a default-real real().  The
// reference takes the five angles NPV*theta from an uninitialised counter whose
// residues mod 5 give the same five positions at every grid point: here
// NPV = -1..-5.
int tara_coh2d_init_vortices(tara_coh2d* h, double lx_ini, double ly_ini) {
  if (!h || !(lx_ini > 0.0) || !(ly_ini > 0.0)) return set_error(TARA_ERR_ARGS, "bad argument");
  TARA_CK(cudaSetDevice(h->dev));
  const double pi = 3.14159265358979323846;
  const double lx = lx_ini * pi, ly = ly_ini * pi;
  const double dx = lx / (double)h->nx, dy = ly / (double)h->ny;
  const double d = 0.40 * 2.0 * pi, rb = 0.30 * 2.0 * pi, theta = 2.0 * pi / 5.0;
  std::vector<double> real(2 * h->rfs, 0.0);
  for (int j = 0; j < h->ny; ++j) {
    const double y = (double)(float)j * dy;
    for (int i = 0; i < h->nx; ++i) {
      const double x = (double)(float)i * dx;
      const size_t r = (size_t)j * h->rpitch + i;
      real[r] = 1.0;
      const double ax = x - lx / 2.0, ay = y - ly / 2.0;
      double w = (ax * ax + ay * ay <= rb * rb) ? 1.0 : 0.0;
      for (int pv = 1; pv <= 5; ++pv) {
        const double bx = x - (lx / 2.0 + d * std::cos(-pv * theta));
        const double by = y - (ly / 2.0 + d * std::sin(-pv * theta));
        if (bx * bx + by * by <= 0.20 * 0.20) w = 10.0;
      }
      real[h->rfs + r] = w;
    }
  }
  // the true-pi box of the driver for the velocity inversion
  std::vector<double> kx(h->nh), ky(h->ny);
  std::vector<int> i0(h->ny);
  make_wavenumbers(h->nx, h->ny, pi, lx, ly, kx.data(), ky.data(), i0.data());
  double* kd = nullptr;
  TARA_CK(cudaMalloc(&kd, (h->nh + h->ny) * sizeof(double)));
  int rc = TARA_OK;
  if (cudaMemcpyAsync(h->prod, real.data(), 2 * h->rfs * sizeof(double), cudaMemcpyHostToDevice, h->stream) !=
          cudaSuccess ||
      cudaMemcpyAsync(kd, kx.data(), h->nh * sizeof(double), cudaMemcpyHostToDevice, h->stream) != cudaSuccess ||
      cudaMemcpyAsync(kd + h->nh, ky.data(), h->ny * sizeof(double), cudaMemcpyHostToDevice, h->stream) !=
          cudaSuccess)
    rc = set_error(TARA_ERR_CUDA, "initial-condition upload");
  // r2c of n and omega into spec[0], spec[1]; nk into the state, velocities from omega_hat
  if (!rc)
    rc = Launch2D<double>::row_r2c(h->nx, h->ny, h->rpitch, h->pitch, h->prod, h->spec, h->twx, h->stream, 2,
                                   h->rfs, h->fs);
  if (!rc)
    rc = Launch2D<double>::col_fft(h->ny, h->nh, h->pitch, h->spec, h->spec, false, h->twy, h->stream, 2, h->fs);
  if (!rc && cudaMemcpyAsync(h->st, h->spec, h->fs * sizeof(double2), cudaMemcpyDeviceToDevice, h->stream) !=
                 cudaSuccess)
    rc = set_error(TARA_ERR_CUDA, "initial-condition copy");
  if (!rc) {
    k_coh_velocity<<<kElemBlocks, kElemThreads, 0, h->stream>>>(h->spec + h->fs, kd, kd + h->nh, h->nh, h->ny,
                                                               h->pitch, h->st + h->fs, h->st + 2 * h->fs);
    if (cudaGetLastError() != cudaSuccess) rc = set_error(TARA_ERR_CUDA, "k_coh_velocity");
  }
  if (!rc && cudaMemsetAsync(h->hist, 0, 3 * h->fs * sizeof(double2), h->stream) != cudaSuccess)
    rc = set_error(TARA_ERR_CUDA, "history reset");
  cudaError_t e = cudaStreamSynchronize(h->stream);
  cudaFree(kd);
  if (rc) return rc;
  if (e != cudaSuccess) return cuda_fail(e, "initial condition");
  return set_ok();
}

// ---- Fortran drop-ins ------------------------------------------------------

// Replaces subroutine derive2coh (src/derive2coh.f95:6).
void derive2coh_(const int* Nx, const int* Ny, const int* Nh, const double* pi, const double* time,
                 const double* nk, const double* ukx, const double* uky, double* dn_dt_old, double* dux_dt_old,
                 double* duy_dt_old, double* dn_dt_new, double* dux_dt_new, double* duy_dt_new) {
  (void)time;
  (void)dn_dt_old;
  (void)dux_dt_old;
  (void)duy_dt_old;
  std::lock_guard<std::mutex> lk(g_coh_mu);
  if (!coh_dims(Nx, Ny, Nh, pi)) return;
  if (!nk || !ukx || !uky || !dn_dt_new || !dux_dt_new || !duy_dt_new) {
    set_error(TARA_ERR_ARGS, "null array argument");
    return;
  }
  tara_coh2d* h = coh_ctx(*Nx, *Ny, *pi);
  if (!h) return;
  if (cudaSetDevice(h->dev) != cudaSuccess) {
    set_error(TARA_ERR_CUDA, "cudaSetDevice failed");
    return;
  }
  const double* in[3] = {nk, ukx, uky};
  double* out[3] = {dn_dt_new, dux_dt_new, duy_dt_new};
  for (int f = 0; f < 3; ++f)
    if (coh_copy_in(h, h->st + f * h->fs, in[f])) return;
  if (coh_rhs(h, 0)) return;
  for (int f = 0; f < 3; ++f)
    if (coh_copy_out(h, out[f], h->dnew + f * h->fs)) return;
  if (coh_check(h)) return;
  set_ok();
}

// Replaces subroutine ab2coh (src/ab2coh.f95:5): AB2 with dt from /comm/.
void ab2coh_(const int* Nx, const int* Ny, const int* Nh, const double* pi, const double* time,
             const double* nk, const double* ukx, const double* uky, double* nk_new, double* ukx_new,
             double* uky_new, const double* dn_dt_old, const double* dux_dt_old, const double* duy_dt_old,
             const double* dn_dt_new, const double* dux_dt_new, const double* duy_dt_new) {
  (void)time;
  std::lock_guard<std::mutex> lk(g_coh_mu);
  if (!coh_dims(Nx, Ny, Nh, pi)) return;
  if (!nk || !ukx || !uky || !nk_new || !ukx_new || !uky_new || !dn_dt_old || !dux_dt_old || !duy_dt_old ||
      !dn_dt_new || !dux_dt_new || !duy_dt_new) {
    set_error(TARA_ERR_ARGS, "null array argument");
    return;
  }
  tara_coh2d* h = coh_ctx(*Nx, *Ny, *pi);
  if (!h) return;
  if (cudaSetDevice(h->dev) != cudaSuccess) {
    set_error(TARA_ERR_CUDA, "cudaSetDevice failed");
    return;
  }
  const double* in[3] = {nk, ukx, uky};
  const double* old[3] = {dn_dt_old, dux_dt_old, duy_dt_old};
  const double* nw[3] = {dn_dt_new, dux_dt_new, duy_dt_new};
  double* out[3] = {nk_new, ukx_new, uky_new};
  for (int f = 0; f < 3; ++f) {
    if (coh_copy_in(h, h->st + f * h->fs, in[f]) || coh_copy_in(h, h->hist + f * h->fs, old[f]) ||
        coh_copy_in(h, h->dnew + f * h->fs, nw[f]))
      return;
  }
  // padding columns are zero in every input
  const size_t n = 3 * h->fs;
  k_ab2_dense<<<kElemBlocks, kElemThreads, 0, h->stream>>>(h->st, h->st, h->hist, h->dnew, n, h->cfg.dt);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    cuda_fail(e, "k_ab2_dense");
    return;
  }
  for (int f = 0; f < 3; ++f)
    if (coh_copy_out(h, out[f], h->st + f * h->fs)) return;
  e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) {
    cuda_fail(e, "ab2coh");
    return;
  }
  set_ok();
}

}  // extern "C"

namespace tara {
int release_dropins_coh() {
  std::lock_guard<std::mutex> lk(g_coh_mu);
  int rc = TARA_OK;
  for (auto& kv : g_coh_ctx) {
    const int r = tara_coh2d_destroy(kv.second);
    if (r != TARA_OK && rc == TARA_OK) rc = r;
  }
  g_coh_ctx.clear();
  return rc;
}
}  // namespace tara
