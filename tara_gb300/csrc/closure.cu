// Learned subgrid closure around the plain vorticity solver: box filtering of
// fine-grid states into training pairs, shell energy spectra, real-space state
// input, and the coarse-grid stepper corrected by the FNO's subgrid flux.
//
// None of this has a counterpart in the reference; it reuses the solver's
// FP64 transform kernels (Stockham column and row passes) and adds the
// pointwise kernels below.
#include <algorithm>
#include <cmath>
#include <vector>

#include "internal.h"

struct tara_closure {
  tara2d* h = nullptr;
  tara_fno* f = nullptr;
  int nf = 1;                  // input feature channels
  double* in_scale = nullptr;  // device, nf values (the input scale / (NxNy))
  double out_scale = 1.0;
  int rpitch = 0;
  double2* spec = nullptr;   // max(nf, 2) * batch spectra
  double* real = nullptr;    // max(nf, 2) * batch real fields
  double2* force = nullptr;  // batch forcing spectra
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  unsigned long long pver = 0;  // network parameter version the graph was captured with
  bool warmed = false;
};

namespace tara {
namespace {

// Spectra of omega, u_x = i ky psi, u_y = -i kx psi with psi = omega * inv
// (inv = 1/k^2, 0 at k = 0), into three pitched fields.
__global__ void k_vel_spectra(const double2* __restrict__ w, Grid2D g, double2* __restrict__ out) {
  const size_t total = (size_t)g.ny * g.nh, fsz = (size_t)g.ny * g.pitch;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const int y = (int)(t / g.nh), x = (int)(t % g.nh);
    const size_t q = (size_t)y * g.pitch + x;
    const double2 v = w[q];
    const double inv = g.inv[(size_t)y * g.nh + x];
    const double pr = v.x * inv, pim = v.y * inv;
    const double kx = g.kx[x], ky = g.ky[y];
    // the odd derivatives of the Nyquist modes (kx = Nx/2 or ky = -Ny/2) are
    // dropped: a real field's derivative has no such component, and keeping
    // the one-sided value would break the reflection symmetry of the data
    const bool nyq = 2 * x == g.nx || 2 * y == g.ny;
    out[q] = v;
    out[fsz + q] = nyq ? make_double2(0.0, 0.0) : make_double2(-ky * pim, ky * pr);
    out[2 * fsz + q] = nyq ? make_double2(0.0, 0.0) : make_double2(kx * pim, -(kx * pr));
  }
}

// Block means over f x f cells of the unnormalised c2r outputs w, u, v (three
// real fields rf apart, row pitch rp), scaled by s = 1/(NxNy); one thread per
// coarse cell.
__global__ void k_box_filter(const double* __restrict__ r, size_t rf, int rp, int f, int ncx, int ncy,
                             double s, float* __restrict__ wbar, float* __restrict__ flux,
                             double* __restrict__ wbar64) {
  const int n = ncx * ncy;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int cy = t / ncx, cx = t % ncx;
    double sw = 0.0, su = 0.0, sv = 0.0, suw = 0.0, svw = 0.0;
    for (int j = 0; j < f; ++j) {
      const size_t row = (size_t)(cy * f + j) * rp + (size_t)cx * f;
      for (int i = 0; i < f; ++i) {
        const double w = r[row + i] * s, u = r[rf + row + i] * s, v = r[2 * rf + row + i] * s;
        sw += w;
        su += u;
        sv += v;
        suw += u * w;
        svw += v * w;
      }
    }
    const double a = 1.0 / ((double)f * (double)f);
    const double mw = sw * a, mu = su * a, mv = sv * a;
    if (wbar) wbar[t] = (float)mw;
    if (wbar64) wbar64[t] = mw;
    if (flux) {
      flux[2 * t] = (float)(suw * a - mu * mw);
      flux[2 * t + 1] = (float)(svw * a - mv * mw);
    }
  }
}

// dense (ny, nx) -> pitched real rows
__global__ void k_to_pitched(const double* __restrict__ in, int nx, int ny, int rp, double* __restrict__ out) {
  const size_t n = (size_t)nx * ny;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    const size_t y = t / nx, x = t % nx;
    out[y * rp + x] = in[t];
  }
}

// Shell sums of 1/2 |omega_hat|^2 inv (= 1/2 |u_hat|^2), weight 1 on the kx = 0 and
// kx = Nx/2 columns and 2 elsewhere (the half spectrum stands for both halves).
__global__ void k_shell_spectrum(const double2* __restrict__ w, Grid2D g, int kmax, double* __restrict__ E) {
  extern __shared__ double sh[];
  for (int k = threadIdx.x; k <= kmax; k += blockDim.x) sh[k] = 0.0;
  __syncthreads();
  const size_t total = (size_t)g.ny * g.nh;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const int y = (int)(t / g.nh), x = (int)(t % g.nh);
    const double kx = g.kx[x], ky = g.ky[y];
    const int shell = (int)rint(sqrt(kx * kx + ky * ky));
    if (shell > kmax) continue;
    const double2 v = w[(size_t)y * g.pitch + x];
    const double wt = (x == 0 || 2 * x == g.nx) ? 0.5 : 1.0;
    atomicAdd(&sh[shell], wt * (v.x * v.x + v.y * v.y) * g.inv[(size_t)y * g.nh + x]);
  }
  __syncthreads();
  for (int k = threadIdx.x; k <= kmax; k += blockDim.x)
    if (sh[k] != 0.0) atomicAdd(&E[k], sh[k]);
}

// Feature spectra of the closure network for one run, `nf` of the fields
// 0 w, 1 dw/dx, 2 dw/dy, 3 du/dx, 4 du/dy, 5 dv/dx  with u = i ky psi, v = -i kx psi,
// psi = w inv (inv = 1/k^2, 0 at k = 0), into nf pitched fields.
constexpr int kMaxFeat = 6;
__global__ void k_feature_spectra(const double2* __restrict__ w, Grid2D g, int nf, double2* __restrict__ out) {
  const size_t total = (size_t)g.ny * g.nh, fsz = (size_t)g.ny * g.pitch;
  w += blockIdx.y * fsz;  // run blockIdx.y: state fsz apart, features nf * fsz apart
  out += blockIdx.y * nf * fsz;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const int y = (int)(t / g.nh), x = (int)(t % g.nh);
    const size_t q = (size_t)y * g.pitch + x;
    const double2 v = w[q];
    const double inv = g.inv[(size_t)y * g.nh + x];
    const double pr = v.x * inv, pim = v.y * inv;
    const double kx = g.kx[x], ky = g.ky[y];
    double2 f[kMaxFeat];
    const bool nyq = 2 * x == g.nx || 2 * y == g.ny;  // odd derivatives dropped there
    f[0] = v;
    f[1] = make_double2(-kx * v.y, kx * v.x);                 // i kx w
    f[2] = make_double2(-ky * v.y, ky * v.x);                 // i ky w
    f[3] = make_double2(-(kx * ky) * pr, -(kx * ky) * pim);   // i kx u = -kx ky psi
    f[4] = make_double2(-(ky * ky) * pr, -(ky * ky) * pim);   // i ky u = -ky^2 psi
    f[5] = make_double2((kx * kx) * pr, (kx * kx) * pim);     // i kx v = kx^2 psi
    for (int c = 0; c < nf; ++c) out[c * fsz + q] = (c > 0 && nyq) ? make_double2(0.0, 0.0) : f[c];
  }
}

// FNO input: x[b][y][x][c] = s[c] * r[b*nf + c][y][x] (pitched FP64 fields -> NHWC FP32)
__global__ void k_real_to_input(const double* __restrict__ r, int nx, int ny, int rp, size_t rf, int B,
                                int nf, const double* __restrict__ s, float* __restrict__ x) {
  const size_t n = (size_t)B * nx * ny * nf;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    const int c = (int)(t % nf);
    const size_t p = t / nf;
    const size_t b = p / ((size_t)nx * ny), e = p % ((size_t)nx * ny);
    const size_t y = e / nx, xx = e % nx;
    x[t] = (float)(r[(b * nf + c) * rf + y * rp + xx] * s[c]);
  }
}

// FNO output (B, ny, nx, 2) FP32 -> 2B pitched FP64 fields (flux_x of run b at
// field 2b, flux_y at 2b+1), times s
__global__ void k_output_to_real(const float* __restrict__ y, int nx, int ny, int rp, size_t rf, int B,
                                 double s, double* __restrict__ r) {
  const size_t n = (size_t)B * nx * ny;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    const size_t b = t / ((size_t)nx * ny), e = t % ((size_t)nx * ny);
    const size_t yy = e / nx, xx = e % nx;
    r[(2 * b) * rf + yy * rp + xx] = (double)y[2 * t] * s;
    r[(2 * b + 1) * rf + yy * rp + xx] = (double)y[2 * t + 1] * s;
  }
}

// force_b = -s (i kx Fx + i ky Fy) on the modes the 2/3 rule keeps, 0 elsewhere.  The
// flux spectra F are unnormalised r2c outputs, the state's own normalisation, so s = 1.
__global__ void k_div_forcing(const double2* __restrict__ fl, Grid2D g, int B, double s,
                              double2* __restrict__ force) {
  const size_t fsz = (size_t)g.ny * g.pitch, n = (size_t)B * g.ny * g.nh;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    const size_t b = t / ((size_t)g.ny * g.nh), e = t % ((size_t)g.ny * g.nh);
    const int y = (int)(e / g.nh), x = (int)(e % g.nh);
    const size_t q = (size_t)y * g.pitch + x;
    double2 o = make_double2(0.0, 0.0);
    if (x < g.i0[y]) {
      const double2 a = fl[(2 * b) * fsz + q], c = fl[(2 * b + 1) * fsz + q];
      const double kx = g.kx[x], ky = g.ky[y];
      // -(i kx a + i ky c) = (kx a.y + ky c.y) - i (kx a.x + ky c.x)
      o = make_double2((kx * a.y + ky * c.y) * s, -(kx * a.x + ky * c.x) * s);
    }
    force[b * fsz + q] = o;
  }
}

// The eight symmetries of the square periodic grid (bit 0: x -> -x, bit 1:
// y -> -y, bit 2: transpose x <-> y, applied in that order) acting on closure
// samples.  Under x -> -x, w and its y derivatives change sign
// (w' = -w(-x, y), u' = (-u_x, u_y)(-x, y)); under transpose w' = -w(y, x) and
// the velocity components swap.  Sign and channel tables per channel of the
// features (w, dw/dx, dw/dy, du/dx, du/dy, dv/dx) and of the flux (x, y).
__constant__ float kSgnFx[6] = {-1.f, 1.f, -1.f, 1.f, -1.f, -1.f};
__constant__ float kSgnFy[6] = {-1.f, -1.f, 1.f, 1.f, -1.f, -1.f};
__constant__ float kSgnFt[6] = {-1.f, -1.f, -1.f, -1.f, 1.f, 1.f};
__constant__ int kPermFt[6] = {0, 2, 1, 3, 5, 4};
__constant__ float kSgnPx[2] = {1.f, -1.f};
__constant__ float kSgnPy[2] = {-1.f, 1.f};
__constant__ float kSgnPt[2] = {-1.f, -1.f};
__constant__ int kPermPt[2] = {1, 0};

// out[g*N + i] = symmetry g of sample i, for (N, n, n, nc) arrays; flux != 0
// selects the flux tables, else the feature tables.
__global__ void k_augment(const float* __restrict__ in, int N, int n, int nc, int flux, float* __restrict__ out) {
  const size_t per = (size_t)n * n * nc, total = (size_t)8 * N * per;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
    const size_t smp = t / per, e = t % per;
    const int g = (int)(smp / N), i = (int)(smp % N);
    const int c = (int)(e % nc), x = (int)((e / nc) % n), y = (int)(e / ((size_t)nc * n));
    int xs = x, ys = y, cs = c;
    float sg = 1.f;
    if (g & 4) {  // undo the transpose first (it was applied last)
      xs = y;
      ys = x;
      sg *= flux ? kSgnPt[c] : kSgnFt[c];
      cs = flux ? kPermPt[c] : kPermFt[c];
    }
    if (g & 2) {
      ys = n - 1 - ys;
      sg *= flux ? kSgnPy[cs] : kSgnFy[cs];
    }
    if (g & 1) {
      xs = n - 1 - xs;
      sg *= flux ? kSgnPx[cs] : kSgnFx[cs];
    }
    out[t] = sg * in[(size_t)i * per + ((size_t)ys * n + xs) * nc + cs];
  }
}

constexpr int kBlocks = 152 * 4, kThreads = 256;

// c2r of `nf` pitched spectra (fields fsz apart; `in` is left untouched when
// spec != in) into real rows rpitch apart, FP64.
int c2r_fields(tara2d* h, const double2* in, double2* spec, double* real, int nf, int rpitch) {
  const void *tx, *ty;
  int rc;
  if ((rc = twiddles64(h, &tx, &ty))) return rc;
  const size_t fsz = (size_t)h->ny * h->pitch, rfs = (size_t)h->ny * rpitch;
  if ((rc = Launch2D<double>::col_fft(h->ny, h->nh, h->pitch, in, spec, true, ty, h->stream, nf, fsz)))
    return rc;
  return Launch2D<double>::row_c2r(h->nx, h->ny, h->pitch, rpitch, spec, real, tx, h->stream, nf, fsz, rfs);
}

int r2c_fields(tara2d* h, const double* real, double2* spec, int nf, int rpitch) {
  const void *tx, *ty;
  int rc;
  if ((rc = twiddles64(h, &tx, &ty))) return rc;
  const size_t fsz = (size_t)h->ny * h->pitch, rfs = (size_t)h->ny * rpitch;
  if ((rc = Launch2D<double>::row_r2c(h->nx, h->ny, rpitch, h->pitch, real, spec, tx, h->stream, nf, rfs, fsz)))
    return rc;
  return Launch2D<double>::col_fft(h->ny, h->nh, h->pitch, spec, spec, false, ty, h->stream, nf, fsz);
}

// Feature fields of runs [r0, r0+nr) as NHWC FP32 (nf channels) at dst, each
// channel multiplied by s[c] (device, already divided by NxNy).  spec/real hold
// nf*nr fields.
int features(tara2d* h, int r0, int nr, int nf, double2* spec, double* real, int rpitch,
             const double* s, float* dst) {
  const size_t fsz = (size_t)h->ny * h->pitch, rfs = (size_t)h->ny * rpitch;
  int rc;
  k_feature_spectra<<<dim3(kBlocks / 4, nr), kThreads, 0, h->stream>>>(h->w0 + (size_t)r0 * fsz, h->grid, nf,
                                                                        spec);
  TARA_CK(cudaGetLastError());
  if ((rc = c2r_fields(h, spec, spec, real, nf * nr, rpitch))) return rc;
  k_real_to_input<<<kBlocks, kThreads, 0, h->stream>>>(real, h->nx, h->ny, rpitch, rfs, nr, nf, s, dst);
  TARA_CK(cudaGetLastError());
  return TARA_OK;
}

// one closure step, enqueued on the handle's stream
int closure_step_once(tara_closure* c) {
  tara2d* h = c->h;
  const int B = h->batch;
  const size_t rfs = (size_t)h->ny * c->rpitch;
  int rc;
  if ((rc = features(h, 0, B, c->nf, c->spec, c->real, c->rpitch, c->in_scale, fno_input(c->f)))) return rc;
  const float* y = nullptr;
  fno_bind_stream(c->f, h->stream);
  fno_bind_error(c->f, h->flag);  // reported by the solver's synchronize
  rc = fno_forward_async(c->f, nullptr, B, &y);
  fno_bind_error(c->f, nullptr);
  fno_bind_stream(c->f, nullptr);
  if (rc) return rc;
  k_output_to_real<<<kBlocks, kThreads, 0, h->stream>>>(y, h->nx, h->ny, c->rpitch, rfs, B, c->out_scale,
                                                         c->real);
  TARA_CK(cudaGetLastError());
  if ((rc = r2c_fields(h, c->real, c->spec, 2 * B, c->rpitch))) return rc;
  k_div_forcing<<<kBlocks, kThreads, 0, h->stream>>>(c->spec, h->grid, B, 1.0, c->force);
  TARA_CK(cudaGetLastError());
  h->force = c->force;
  rc = tara2d_step(h, 1);
  h->force = nullptr;
  return rc;
}

}  // namespace
}  // namespace tara

using namespace tara;

extern "C" {

int tara2d_filter(tara2d* h, int run, int factor, float* omega_bar, float* flux, double* omega_bar64) {
  if (!h || run < 0 || run >= h->batch || factor < 1 || h->nx % factor || h->ny % factor)
    return set_error(TARA_ERR_ARGS, "bad filter arguments");
  TARA_CK(cudaSetDevice(h->dev));
  const size_t fsz = (size_t)h->ny * h->pitch;
  const int rpitch = round_up(h->nx, 8);
  const size_t rfs = (size_t)h->ny * rpitch;
  void* ws = nullptr;
  int rc;
  if ((rc = scratch(h, 3 * fsz * sizeof(double2) + 3 * rfs * sizeof(double), &ws))) return rc;
  double2* sp = (double2*)ws;
  double* real = (double*)(sp + 3 * fsz);
  k_vel_spectra<<<kBlocks, kThreads, 0, h->stream>>>(h->w0 + (size_t)run * fsz, h->grid, sp);
  TARA_CK(cudaGetLastError());
  if ((rc = c2r_fields(h, sp, sp, real, 3, rpitch))) return rc;
  const int ncx = h->nx / factor, ncy = h->ny / factor;
  const double nn = (double)h->nx * (double)h->ny;
  k_box_filter<<<(ncx * ncy + 255) / 256, 256, 0, h->stream>>>(real, rfs, rpitch, factor, ncx, ncy, 1.0 / nn,
                                                                omega_bar, flux, omega_bar64);
  TARA_CK(cudaGetLastError());
  TARA_CK(cudaStreamSynchronize(h->stream));
  return set_ok();
}

int tara2d_set_state_real_device(tara2d* h, int run, const double* omega_dev) {
  if (!h || !omega_dev || run < 0 || run >= h->batch) return set_error(TARA_ERR_ARGS, "bad arguments");
  TARA_CK(cudaSetDevice(h->dev));
  const size_t fsz = (size_t)h->ny * h->pitch;
  const int rpitch = round_up(h->nx, 8);
  void* ws = nullptr;
  int rc;
  if ((rc = scratch(h, (size_t)h->ny * rpitch * sizeof(double), &ws))) return rc;
  double* real = (double*)ws;
  k_to_pitched<<<kBlocks, kThreads, 0, h->stream>>>(omega_dev, h->nx, h->ny, rpitch, real);
  TARA_CK(cudaGetLastError());
  if ((rc = r2c_fields(h, real, h->w0 + run * fsz, 1, rpitch))) return rc;
  TARA_CK(cudaMemsetAsync(h->fold + run * fsz, 0, fsz * sizeof(double2), h->stream));
  TARA_CK(cudaStreamSynchronize(h->stream));
  return set_ok();
}

int tara2d_spectrum(tara2d* h, int run, int kmax, double* E) {
  if (!h || !E || run < 0 || run >= h->batch || kmax < 0 || kmax > 4096)
    return set_error(TARA_ERR_ARGS, "bad spectrum arguments");
  TARA_CK(cudaSetDevice(h->dev));
  void* ws = nullptr;
  int rc;
  if ((rc = scratch(h, (size_t)(kmax + 1) * sizeof(double), &ws))) return rc;
  double* dE = (double*)ws;
  TARA_CK(cudaMemsetAsync(dE, 0, (kmax + 1) * sizeof(double), h->stream));
  k_shell_spectrum<<<kBlocks, kThreads, (kmax + 1) * sizeof(double), h->stream>>>(
      h->w0 + (size_t)run * h->ny * h->pitch, h->grid, kmax, dE);
  TARA_CK(cudaGetLastError());
  std::vector<double> out(kmax + 1);
  TARA_CK(cudaMemcpyAsync(out.data(), dE, out.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  TARA_CK(cudaStreamSynchronize(h->stream));
  const double nn = (double)h->nx * (double)h->ny;
  for (int k = 0; k <= kmax; ++k) E[k] = out[k] / (nn * nn);
  return set_ok();
}

int tara_closure_destroy(tara_closure* c) {
  if (!c) return set_ok();
  cudaSetDevice(c->h->dev);
  cudaStreamSynchronize(c->h->stream);
  if (c->exec) cudaGraphExecDestroy(c->exec);
  if (c->graph) cudaGraphDestroy(c->graph);
  cudaFree(c->spec);
  cudaFree(c->real);
  cudaFree(c->in_scale);
  cudaFree(c->force);
  delete c;
  return set_ok();
}

int tara_closure_create(tara2d* h, tara_fno* f, const double* in_scales, double out_scale,
                        tara_closure** out) {
  if (!h || !f || !out || !in_scales) return set_error(TARA_ERR_ARGS, "null argument");
  *out = nullptr;
  const tara_fno_config& fc = fno_config(f);
  if (fc.h != h->ny || fc.w != h->nx || fc.ci < 1 || fc.ci > kMaxFeat || fc.co != 2 ||
      fc.max_batch < h->batch)
    return set_error(TARA_ERR_ARGS, "network grid, channels or batch do not fit the handle");
  if (h->cfg.rhs != TARA_RHS_PLAIN) return set_error(TARA_ERR_ARGS, "the closure drives the plain RHS");
  TARA_CK(cudaSetDevice(h->dev));
  tara_closure* c = new tara_closure();
  c->h = h;
  c->f = f;
  c->nf = fc.ci;
  c->out_scale = out_scale;
  c->rpitch = round_up(h->nx, 8);
  const int B = h->batch;
  const int nfield = std::max(c->nf, 2) * B;
  const size_t fsz = (size_t)h->ny * h->pitch, rfs = (size_t)h->ny * c->rpitch;
  if (cudaMalloc(&c->spec, nfield * fsz * sizeof(double2)) != cudaSuccess ||
      cudaMalloc(&c->real, nfield * rfs * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&c->in_scale, kMaxFeat * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&c->force, B * fsz * sizeof(double2)) != cudaSuccess) {
    tara_closure_destroy(c);
    return set_error(TARA_ERR_NOMEM, "cudaMalloc in tara_closure_create");
  }
  double sc[kMaxFeat];
  const double nn = (double)h->nx * (double)h->ny;
  for (int i = 0; i < c->nf; ++i) sc[i] = in_scales[i] / nn;
  if (cudaMemcpy(c->in_scale, sc, c->nf * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) {
    tara_closure_destroy(c);
    return set_error(TARA_ERR_CUDA, "scale upload");
  }
  const void *tx, *ty;
  int rc;
  if ((rc = twiddles64(h, &tx, &ty))) {
    const ErrorState saved = save_error();
    tara_closure_destroy(c);
    restore_error(saved);
    return rc;
  }
  *out = c;
  return set_ok();
}

int tara_closure_augment(const float* x_dev, const float* t_dev, int n_samples, int n, int nf, float* x_out,
                         float* t_out) {
  if (n_samples < 1 || n < 2 || nf < 1 || nf > kMaxFeat || (!x_dev && !t_dev) || (x_dev && !x_out) ||
      (t_dev && !t_out))
    return set_error(TARA_ERR_ARGS, "bad augmentation arguments");
  if (x_dev) {
    k_augment<<<kBlocks * 4, kThreads>>>(x_dev, n_samples, n, nf, 0, x_out);
    TARA_CK(cudaGetLastError());
  }
  if (t_dev) {
    k_augment<<<kBlocks * 4, kThreads>>>(t_dev, n_samples, n, 2, 1, t_out);
    TARA_CK(cudaGetLastError());
  }
  TARA_CK(cudaDeviceSynchronize());
  return set_ok();
}

int tara2d_features(tara2d* h, int run, int nf, const double* scales, float* out_dev) {
  if (!h || !out_dev || run < 0 || run >= h->batch || nf < 1 || nf > kMaxFeat)
    return set_error(TARA_ERR_ARGS, "bad feature arguments");
  TARA_CK(cudaSetDevice(h->dev));
  const int rpitch = round_up(h->nx, 8);
  const size_t fsz = (size_t)h->ny * h->pitch, rfs = (size_t)h->ny * rpitch;
  void* ws = nullptr;
  int rc;
  if ((rc = scratch(h, nf * (fsz * sizeof(double2) + rfs * sizeof(double)) + kMaxFeat * sizeof(double), &ws)))
    return rc;
  double2* spec = (double2*)ws;
  double* real = (double*)(spec + nf * fsz);
  double* ds = real + nf * rfs;
  double sc[kMaxFeat];
  const double nn = (double)h->nx * (double)h->ny;
  for (int i = 0; i < nf; ++i) sc[i] = (scales ? scales[i] : 1.0) / nn;
  TARA_CK(cudaMemcpyAsync(ds, sc, nf * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  if ((rc = features(h, run, 1, nf, spec, real, rpitch, ds, out_dev))) return rc;
  TARA_CK(cudaStreamSynchronize(h->stream));
  return set_ok();
}

// The first step runs eagerly (it sets the kernels' shared-memory attributes);
// the next ones replay a CUDA graph of one step, captured again when the
// network's parameters have changed since.
int tara_closure_step(tara_closure* c, int nsteps) {
  if (!c || nsteps < 0) return set_error(TARA_ERR_ARGS, "bad arguments");
  tara2d* h = c->h;
  TARA_CK(cudaSetDevice(h->dev));
  int rc;
  int s = 0;
  if (!c->warmed && nsteps > 0) {
    if ((rc = closure_step_once(c))) return rc;
    c->warmed = true;
    s = 1;
  }
  if (c->exec && c->pver != fno_param_version(c->f)) {
    cudaGraphExecDestroy(c->exec);
    cudaGraphDestroy(c->graph);
    c->exec = nullptr;
    c->graph = nullptr;
  }
  if (s < nsteps && !c->exec) {
    fno_bind_stream(c->f, h->stream);
    rc = fno_prepare(c->f);  // block matrices outside the capture
    fno_bind_stream(c->f, nullptr);
    if (rc) return rc;
    c->pver = fno_param_version(c->f);
    TARA_CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    rc = closure_step_once(c);
    cudaGraph_t g = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(h->stream, &g);
    if (rc) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (ec != cudaSuccess) return cuda_fail(ec, "cudaStreamEndCapture");
    c->graph = g;
    TARA_CK(cudaGraphInstantiate(&c->exec, c->graph, 0));
  }
  for (; s < nsteps; ++s) TARA_CK(cudaGraphLaunch(c->exec, h->stream));
  return set_ok();
}

}  // extern "C"
