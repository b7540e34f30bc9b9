// Fortran drop-ins (gfortran-mangled derive2csh_, ab2csh_, derive2css_,
// ab2css_, rk42css_) and the standalone 2D transform entry points.
//
// The drop-ins keep one solver context per (shape, RHS kind, scheme) and move
// the caller's host arrays through it on every call: the reference's callers
// rewrite omegak and the histories on the host between calls
// (src/main2csh.f95:121-126), so nothing can stay cached on the device.
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "internal.h"

using namespace tara;

namespace {

std::mutex g_mu;
std::map<std::tuple<int, int, int, int>, tara2d*> g_ctx;
double g_css_lx = 2.0 * (double)3.1428f, g_css_ly = 2.0 * (double)3.1428f, g_css_lambda = 10.0;

// Context for a shape; rhs/scheme select the buffers.  Parameters that the
// reference passes per call (nu, alpha, dt) are refreshed by the caller.
tara2d* get_ctx(int nx, int ny, int rhs, int scheme) {
  auto key = std::make_tuple(nx, ny, rhs, scheme);
  auto it = g_ctx.find(key);
  if (it != g_ctx.end()) return it->second;
  tara2d_config cfg;
  tara2d_default_config(&cfg, nx, ny);
  cfg.rhs = rhs;
  cfg.scheme = scheme;
  if (rhs == TARA_RHS_SCREEN) {
    cfg.lx = g_css_lx;
    cfg.ly = g_css_ly;
    cfg.lambda = g_css_lambda;
  }
  tara2d* h = nullptr;
  if (tara2d_create(&cfg, &h) != TARA_OK) return nullptr;
  g_ctx[key] = h;
  return h;
}

bool check_dims(const int* Nx, const int* Ny, const int* Nh) {
  if (!Nx || !Ny || !Nh) {
    set_error(TARA_ERR_ARGS, "null dimension argument");
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

// Screened contexts follow the current tara_set_css_params values.
int sync_css(tara2d* h) {
  if (h->cfg.lx == g_css_lx && h->cfg.ly == g_css_ly && h->cfg.lambda == g_css_lambda)
    return TARA_OK;
  h->cfg.lx = g_css_lx;
  h->cfg.ly = g_css_ly;
  h->cfg.lambda = g_css_lambda;
  return refresh_tables(h);
}

void derive_common(int rhs, const int* Nx, const int* Ny, const int* Nh, double alpha, double nu,
                   const double* omegak, double* dt_omegak_new) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!check_dims(Nx, Ny, Nh)) return;
  if (!omegak || !dt_omegak_new) {
    set_error(TARA_ERR_ARGS, "null array argument");
    return;
  }
  tara2d* h = get_ctx(*Nx, *Ny, rhs, TARA_SCHEME_AB2);
  if (!h) return;
  if (cudaSetDevice(h->dev) != cudaSuccess) {
    set_error(TARA_ERR_CUDA, "cudaSetDevice failed");
    return;
  }
  if (rhs == TARA_RHS_SCREEN && sync_css(h)) return;
  h->rp.nu = nu;
  h->rp.alpha = alpha;
  h->rp.nu_f = (float)nu;
  h->rp.alpha_f = (float)alpha;
  if (copy_in_dense(h, h->w0, omegak)) return;
  if (rhs_and_update(h, h->w0, MODE_DERIVE, nullptr)) return;
  if (copy_out_dense(h, dt_omegak_new, h->fout)) return;
  cudaError_t e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) {
    cuda_fail(e, "derive");
    return;
  }
  set_ok();
}

void ab2_common(const int* Nx, const int* Ny, const int* Nh, double dt, const double* omegak,
                double* omegak_new, const double* dt_old, const double* dt_new) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!check_dims(Nx, Ny, Nh)) return;
  if (!omegak || !omegak_new || !dt_old || !dt_new) {
    set_error(TARA_ERR_ARGS, "null array argument");
    return;
  }
  tara2d* h = get_ctx(*Nx, *Ny, TARA_RHS_PLAIN, TARA_SCHEME_AB2);
  if (!h) return;
  if (cudaSetDevice(h->dev) != cudaSuccess) {
    set_error(TARA_ERR_CUDA, "cudaSetDevice failed");
    return;
  }
  if (copy_in_dense(h, h->w0, omegak) || copy_in_dense(h, h->fold, dt_old) ||
      copy_in_dense(h, h->fout, dt_new))
    return;
  const size_t n = (size_t)h->ny * h->pitch;  // padding columns are zero in all inputs
  k_ab2_dense<<<304, 256, 0, h->stream>>>(h->w0, h->w0, h->fold, h->fout, n, dt);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    cuda_fail(e, "k_ab2_dense");
    return;
  }
  if (copy_out_dense(h, omegak_new, h->w0)) return;
  e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) {
    cuda_fail(e, "ab2");
    return;
  }
  set_ok();
}

}  // namespace

extern "C" {

void tara_set_css_params(double lx, double ly, double lambda) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_css_lx = lx;
  g_css_ly = ly;
  g_css_lambda = lambda;
}

void derive2csh_(const int* Nx, const int* Ny, const int* Nh, const double* nu,
                 const double* time, double* omegak, double* omegak_new, double* dt_omegak_old,
                 double* dt_omegak_new) {
  (void)time; (void)omegak_new; (void)dt_omegak_old;
  derive_common(TARA_RHS_PLAIN, Nx, Ny, Nh, 1.0, nu ? *nu : 0.0, omegak, dt_omegak_new);
}

void ab2csh_(const int* Nx, const int* Ny, const int* Nh, const double* nu, const double* time,
             const double* dt, double* omegak, double* omegak_new, double* dt_omegak_old,
             double* dt_omegak_new) {
  (void)nu; (void)time;
  ab2_common(Nx, Ny, Nh, dt ? *dt : 0.0, omegak, omegak_new, dt_omegak_old, dt_omegak_new);
}

void derive2css_(const int* Nx, const int* Ny, const int* Nh, const double* alpha,
                 const double* nu, const double* time, double* omegak, double* omegak_new,
                 double* dt_omegak_old, double* dt_omegak_new) {
  (void)time; (void)omegak_new; (void)dt_omegak_old;
  derive_common(TARA_RHS_SCREEN, Nx, Ny, Nh, alpha ? *alpha : 1.0, nu ? *nu : 0.0, omegak,
                dt_omegak_new);
}

void ab2css_(const int* Nx, const int* Ny, const int* Nh, const double* alpha, const double* nu,
             const double* time, const double* dt, double* omegak, double* omegak_new,
             double* dt_omegak_old, double* dt_omegak_new) {
  (void)alpha; (void)nu; (void)time;
  ab2_common(Nx, Ny, Nh, dt ? *dt : 0.0, omegak, omegak_new, dt_omegak_old, dt_omegak_new);
}

void rk42css_(const int* Nx, const int* Ny, const int* Nh, const double* alpha, const double* nu,
              const double* time, const double* dt, double* omegak, double* omegak_new,
              double* dt_omegak_old, double* dt_omegak_new) {
  (void)time; (void)dt_omegak_old; (void)dt_omegak_new;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!check_dims(Nx, Ny, Nh)) return;
  if (!omegak || !omegak_new || !alpha || !nu || !dt) {
    set_error(TARA_ERR_ARGS, "null argument");
    return;
  }
  tara2d* h = get_ctx(*Nx, *Ny, TARA_RHS_SCREEN, TARA_SCHEME_RK4);
  if (!h) return;
  if (cudaSetDevice(h->dev) != cudaSuccess) {
    set_error(TARA_ERR_CUDA, "cudaSetDevice failed");
    return;
  }
  if (sync_css(h)) return;
  h->rp.nu = *nu;
  h->rp.alpha = *alpha;
  h->rp.nu_f = (float)*nu;
  h->rp.alpha_f = (float)*alpha;
  h->rp.dt = *dt;
  h->cfg.dt = *dt;
  if (copy_in_dense(h, h->w0, omegak)) return;
  if (rhs_and_update(h, h->w0, MODE_RK1, nullptr) || rhs_and_update(h, h->ws, MODE_RK2, nullptr) ||
      rhs_and_update(h, h->ws, MODE_RK3, nullptr) || rhs_and_update(h, h->ws, MODE_RK4, nullptr))
    return;
  if (copy_out_dense(h, omegak_new, h->w0)) return;
  cudaError_t e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) {
    cuda_fail(e, "rk4");
    return;
  }
  set_ok();
}

// ---- standalone transforms (FFTW rank-2 semantics, unnormalised) ----------
// in: real (Nx,Ny) x-fastest; out: complex (Nh,Ny) interleaved.
// Eight independent FMA chains per thread; the store happens only for a value
// the chains never reach, but depends on all of them, so none is removed.
__global__ void __launch_bounds__(256) k_dfma_probe(double* out, int iters, double b, double c) {
  double a[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = 1.0 + 1e-3 * k + 1e-9 * threadIdx.x;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = fma(a[k], b, c);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += a[k];
  if (s == -1.0) out[0] = s;
}

int tara_twiddle_table(int n, int precision, double* out, int capacity, int* count) {
  if (!count || !is_pow2_in_range(n) || (precision != TARA_PREC_FP64 && precision != TARA_PREC_FP32))
    return set_error(TARA_ERR_ARGS, "tara_twiddle_table: n a power of two in [16, 4096], FP64 or FP32");
  const int cnt = tw_count(n);
  *count = cnt;
  if (!out) return TARA_OK;
  if (capacity < cnt) return set_error(TARA_ERR_ARGS, "tara_twiddle_table: capacity below the entry count");
  for (int m = 0; m < cnt; ++m) {
    if (precision == TARA_PREC_FP64)
      twiddle_entry_fp64(n, m, out + 2 * m, out + 2 * m + 1);
    else
      twiddle_entry(n, m, out + 2 * m, out + 2 * m + 1);
  }
  return TARA_OK;
}

int tara_measure_dfma_rate(int reps, double* inst_per_s) {
  if (!inst_per_s || reps < 1) return set_error(TARA_ERR_ARGS, "bad argument");
  int dev, sms;
  TARA_CK(cudaGetDevice(&dev));
  TARA_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int blocks = sms * 8, threads = 256, iters = 4096;
  double* out = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaStream_t s = nullptr;
  auto done = [&](int rc) {
    if (s) cudaStreamSynchronize(s);
    cudaFree(out);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (s) cudaStreamDestroy(s);
    return rc;
  };
  if (cudaMalloc(&out, sizeof(double)) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
      cudaEventCreate(&e1) != cudaSuccess || cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess)
    return done(set_error(TARA_ERR_CUDA, "probe setup"));
  k_dfma_probe<<<blocks, threads, 0, s>>>(out, iters, 0.9999999, 1e-7);
  cudaEventRecord(e0, s);
  for (int r = 0; r < reps; ++r) k_dfma_probe<<<blocks, threads, 0, s>>>(out, iters, 0.9999999, 1e-7);
  cudaEventRecord(e1, s);
  cudaError_t e = cudaEventSynchronize(e1);
  if (e != cudaSuccess) return done(cuda_fail(e, "dfma probe"));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  *inst_per_s = (double)blocks * threads * iters * 8.0 * reps / (ms * 1e-3);
  return done(set_ok());
}

int tara_fft2d_r2c(int nx, int ny, int precision, const double* in, double* out) {
  if (!is_size_2d(nx) || !is_size_2d(ny) || !in || !out)
    return set_error(TARA_ERR_ARGS, "bad transform arguments");
  const bool f32 = precision == TARA_PREC_FP32;
  if (f32 && (!is_pow2_in_range(nx) || !is_pow2_in_range(ny)))
    return set_error(TARA_ERR_ARGS, "FP32 transforms take powers of two only");
  const int nh = nx / 2 + 1, pitch = round_up(nh, 8), rpitch = round_up(nx, 8);
  const size_t cs = f32 ? sizeof(float2) : sizeof(double2), rs = f32 ? sizeof(float) : sizeof(double);
  std::vector<unsigned char> hr((size_t)ny * rpitch * rs, 0), hc((size_t)ny * pitch * cs, 0);
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
      const double v = in[(size_t)j * nx + i];
      if (f32) ((float*)hr.data())[(size_t)j * rpitch + i] = (float)v;
      else ((double*)hr.data())[(size_t)j * rpitch + i] = v;
    }
  void *dr = nullptr, *dc = nullptr, *tx = nullptr, *ty = nullptr;
  int rc = TARA_OK;
  cudaStream_t s = nullptr;
  auto done = [&](int code) {
    if (s) cudaStreamSynchronize(s);
    cudaFree(dr); cudaFree(dc); cudaFree(tx); cudaFree(ty);
    if (s) cudaStreamDestroy(s);
    return code;
  };
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess)
    return done(set_error(TARA_ERR_CUDA, "stream"));
  if ((rc = make_twiddles(nx, f32, &tx)) || (rc = make_twiddles(ny, f32, &ty))) return done(rc);
  if (cudaMalloc(&dr, hr.size()) != cudaSuccess || cudaMalloc(&dc, hc.size()) != cudaSuccess)
    return done(set_error(TARA_ERR_NOMEM, "cudaMalloc"));
  cudaMemcpyAsync(dr, hr.data(), hr.size(), cudaMemcpyHostToDevice, s);
  rc = f32 ? Launch2D<float>::row_r2c(nx, ny, rpitch, pitch, dr, dc, tx, s)
           : Launch2D<double>::row_r2c(nx, ny, rpitch, pitch, dr, dc, tx, s);
  if (!rc)
    rc = f32 ? Launch2D<float>::col_fft(ny, nh, pitch, dc, dc, false, ty, s)
             : Launch2D<double>::col_fft(ny, nh, pitch, dc, dc, false, ty, s);
  if (rc) return done(rc);
  cudaMemcpyAsync(hc.data(), dc, hc.size(), cudaMemcpyDeviceToHost, s);
  cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return done(cuda_fail(e, "r2c"));
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nh; ++i) {
      const size_t q = (size_t)j * pitch + i, o = 2 * ((size_t)j * nh + i);
      if (f32) {
        const float2 v = ((float2*)hc.data())[q];
        out[o] = v.x; out[o + 1] = v.y;
      } else {
        const double2 v = ((double2*)hc.data())[q];
        out[o] = v.x; out[o + 1] = v.y;
      }
    }
  return done(set_ok());
}

// in: complex (Nh,Ny) interleaved (left untouched); out: real (Nx,Ny).
int tara_fft2d_c2r(int nx, int ny, int precision, const double* in, double* out) {
  if (!is_size_2d(nx) || !is_size_2d(ny) || !in || !out)
    return set_error(TARA_ERR_ARGS, "bad transform arguments");
  const bool f32 = precision == TARA_PREC_FP32;
  if (f32 && (!is_pow2_in_range(nx) || !is_pow2_in_range(ny)))
    return set_error(TARA_ERR_ARGS, "FP32 transforms take powers of two only");
  const int nh = nx / 2 + 1, pitch = round_up(nh, 8), rpitch = round_up(nx, 8);
  const size_t cs = f32 ? sizeof(float2) : sizeof(double2), rs = f32 ? sizeof(float) : sizeof(double);
  std::vector<unsigned char> hr((size_t)ny * rpitch * rs, 0), hc((size_t)ny * pitch * cs, 0);
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nh; ++i) {
      const size_t q = (size_t)j * pitch + i, o = 2 * ((size_t)j * nh + i);
      if (f32) ((float2*)hc.data())[q] = make_float2((float)in[o], (float)in[o + 1]);
      else ((double2*)hc.data())[q] = make_double2(in[o], in[o + 1]);
    }
  void *dr = nullptr, *dc = nullptr, *tx = nullptr, *ty = nullptr;
  int rc = TARA_OK;
  cudaStream_t s = nullptr;
  auto done = [&](int code) {
    if (s) cudaStreamSynchronize(s);
    cudaFree(dr); cudaFree(dc); cudaFree(tx); cudaFree(ty);
    if (s) cudaStreamDestroy(s);
    return code;
  };
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess)
    return done(set_error(TARA_ERR_CUDA, "stream"));
  if ((rc = make_twiddles(nx, f32, &tx)) || (rc = make_twiddles(ny, f32, &ty))) return done(rc);
  if (cudaMalloc(&dr, hr.size()) != cudaSuccess || cudaMalloc(&dc, hc.size()) != cudaSuccess)
    return done(set_error(TARA_ERR_NOMEM, "cudaMalloc"));
  cudaMemcpyAsync(dc, hc.data(), hc.size(), cudaMemcpyHostToDevice, s);
  rc = f32 ? Launch2D<float>::col_fft(ny, nh, pitch, dc, dc, true, ty, s)
           : Launch2D<double>::col_fft(ny, nh, pitch, dc, dc, true, ty, s);
  if (!rc)
    rc = f32 ? Launch2D<float>::row_c2r(nx, ny, pitch, rpitch, dc, dr, tx, s)
             : Launch2D<double>::row_c2r(nx, ny, pitch, rpitch, dc, dr, tx, s);
  if (rc) return done(rc);
  cudaMemcpyAsync(hr.data(), dr, hr.size(), cudaMemcpyDeviceToHost, s);
  cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return done(cuda_fail(e, "c2r"));
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i)
      out[(size_t)j * nx + i] = f32 ? (double)((float*)hr.data())[(size_t)j * rpitch + i]
                                    : ((double*)hr.data())[(size_t)j * rpitch + i];
  return done(set_ok());
}

}  // extern "C"

namespace tara {
int release_dropins_2d() {
  std::lock_guard<std::mutex> lk(g_mu);
  int rc = TARA_OK;
  for (auto& kv : g_ctx) {
    const int r = tara2d_destroy(kv.second);
    if (r != TARA_OK && rc == TARA_OK) rc = r;
  }
  g_ctx.clear();
  return rc;
}
}  // namespace tara

extern "C" int tara_finalize(void) {
  const int rcs[4] = {release_dropins_2d(), release_dropins_3d(), release_dropins_coh(),
                      release_dropins_com()};
  for (int r : rcs)
    if (r != TARA_OK) return r;
  return set_ok();
}
