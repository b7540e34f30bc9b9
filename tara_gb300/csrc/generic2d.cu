// The 2D FP64 passes for grid sizes that are not powers of two (even sizes with
// factors 2, 3, 5 and 7, up to 3600 per axis): the same three passes per right-hand
// side as kernels2d.cuh -- the y-direction inverse transforms of the four
// spectral fields, the x-direction c2r / product / r2c per pair of ky rows, the
// y-direction forward transform with the 2/3 truncation, the nu k^2 term and
// the stage update -- and the plain transforms, with the mixed-radix transform
// of fft_any.cuh in place of the power-of-two Stockham kernels.  One CTA per
// column or row pair; the element arithmetic is that of the power-of-two FP64
// path line for line (src/derive2csh.f95:29-145, src/derive2css.f95:22-104,
// src/ab2csh.f95:10-14, src/rk42css.f95), so both paths give the same results
// up to the transforms' rounding.
#include <cmath>
#include <vector>

#include "fft_any.cuh"
#include "internal.h"
#include "kernels2d.cuh"

namespace tara {

namespace {

constexpr int kAnyT = 256;

// Hermitian extension of two half rows A, B (kx in [0, n/2]) into entry k of
// Z = A + i B (FFTW's c2r reads only the real parts of the kx = 0 and n/2 bins).
__device__ __forceinline__ double2 any_pair_entry(const double2* __restrict__ fa, const double2* __restrict__ fb,
                                                  int k, int n) {
  const int h = n / 2, kk = k <= h ? k : n - k;
  double2 A = fa[kk], B = fb[kk];
  if (kk == 0 || kk == h) {
    A.y = 0.0;
    B.y = 0.0;
  }
  return (k <= h) ? make_double2(A.x - B.y, A.y + B.x) : make_double2(A.x + B.y, -A.y + B.x);
}

}  // namespace

// Pass A: column x = blockIdx.x of run blockIdx.z; u_x, u_y, i kx w, i ky w
// formed and inverse-transformed along y one after another.
__global__ void __launch_bounds__(kAnyT) k_any_col_inverse(const double2* __restrict__ win, double2* __restrict__ u,
                                                          Grid2D g, RhsParams p, AnyPlan py,
                                                          const double2* __restrict__ wy) {
  extern __shared__ __align__(16) double2 any_sm[];
  double2* buf = any_sm;
  double2* tmp = any_sm + g.ny;
  const int x = blockIdx.x, tid = threadIdx.x;
  const size_t fsz = (size_t)g.ny * g.pitch;
  win += blockIdx.z * fsz;
  u += blockIdx.z * 4 * fsz;
  const double kx = g.kx[x];
  for (int f = 0; f < 4; ++f) {
    for (int y = tid; y < g.ny; y += kAnyT) {
      const double2 w = win[(size_t)y * g.pitch + x];
      const double ky = g.ky[y];
      const double inv = g.inv[(size_t)y * g.nh + x];
      double2 val;
      if (f < 2) {  // psi = omega/(k^2 [+lambda]); u_x = (0,1) ky psi, u_y = -(0,1) kx psi
        const double pr = w.x * inv, pim = w.y * inv;
        val = f == 0 ? make_double2(-ky * pim, ky * pr) : make_double2(kx * pim, -(kx * pr));
      } else {  // i kx w, i ky w with w = omega_hat (plain) or k^2 psi (screened)
        double dr = w.x, di = w.y;
        if (p.rhs) {
          const double k2 = kx * kx + ky * ky;
          dr = k2 * (w.x * inv);
          di = k2 * (w.y * inv);
        }
        val = f == 2 ? make_double2(-kx * di, kx * dr) : make_double2(-ky * di, ky * dr);
      }
      buf[y] = val;
    }
    __syncthreads();
    fft_any(buf, tmp, py, wy, true, tid, kAnyT);
    for (int y = tid; y < g.ny; y += kAnyT) u[(size_t)f * fsz + (size_t)y * g.pitch + x] = buf[y];
    __syncthreads();
  }
}

// Pass B: ky rows 2 blockIdx.x and 2 blockIdx.x + 1 of run blockIdx.y: the
// x-direction c2r of (u_x + i u_y) and (w_x + i w_y) per row, the products
// u_x w_x + u_y w_y packed as (row a) + i (row b), one forward transform, the
// split into the two rows' half spectra (unnormalised; the factor 2 of the
// split is in nl_scale).
__global__ void __launch_bounds__(kAnyT) k_any_row_nl(const double2* __restrict__ u, double2* __restrict__ nl,
                                                     Grid2D g, AnyPlan px, const double2* __restrict__ wx) {
  extern __shared__ __align__(16) double2 any_sm[];
  const int n = g.nx, h = n / 2, tid = threadIdx.x;
  double2* buf = any_sm;
  double2* tmp = buf + n;
  double2* keep = tmp + n;
  double2* prod = keep + n;
  const size_t fsz = (size_t)g.ny * g.pitch;
  u += blockIdx.y * 4 * fsz;
  nl += blockIdx.y * fsz;
  const int ya = 2 * blockIdx.x;
  for (int r = 0; r < 2; ++r) {
    const int y = ya + r;
    for (int s = 0; s < 2; ++s) {
      for (int k = tid; k < n; k += kAnyT) {
        double2 z = make_double2(0.0, 0.0);
        if (y < g.ny) {
          const double2* fa = u + (size_t)(2 * s) * fsz + (size_t)y * g.pitch;
          z = any_pair_entry(fa, fa + fsz, k, n);
        }
        buf[k] = z;
      }
      __syncthreads();
      fft_any(buf, tmp, px, wx, true, tid, kAnyT);
      for (int x = tid; x < n; x += kAnyT) {
        if (s == 0) {
          keep[x] = buf[x];
        } else {
          const double2 c1 = keep[x], c2 = buf[x];
          const double v = fma(c1.x, c2.x, c1.y * c2.y);
          if (r == 0)
            prod[x].x = v;
          else
            prod[x].y = v;
        }
      }
      __syncthreads();
    }
  }
  for (int x = tid; x < n; x += kAnyT) buf[x] = prod[x];
  __syncthreads();
  fft_any(buf, tmp, px, wx, false, tid, kAnyT);
  for (int k = tid; k <= h; k += kAnyT) {
    const double2 z = buf[k], m = buf[(n - k) % n];
    if (ya < g.ny) nl[(size_t)ya * g.pitch + k] = make_double2(z.x + m.x, z.y - m.y);
    if (ya + 1 < g.ny) nl[(size_t)(ya + 1) * g.pitch + k] = make_double2(z.y + m.y, -(z.x - m.x));
  }
}

// Pass C: column x = blockIdx.x of run blockIdx.y: forward transform along y,
// then per element the right-hand side (2/3 truncation of the nonlinear term,
// scaling, nu k^2 term) and the update of `mode`.
__global__ void __launch_bounds__(kAnyT) k_any_col_forward(const double2* __restrict__ nl, StepBufs sb, Grid2D g,
                                                          RhsParams p, int mode, AnyPlan py,
                                                          const double2* __restrict__ wy) {
  extern __shared__ __align__(16) double2 any_sm[];
  double2* buf = any_sm;
  double2* tmp = any_sm + g.ny;
  const int x = blockIdx.x, tid = threadIdx.x;
  {
    const size_t off = blockIdx.y * (size_t)g.ny * g.pitch;
    nl += off;
    sb.win += off;
    if (sb.w0) sb.w0 += off;
    if (sb.ws) sb.ws += off;
    if (sb.acc) sb.acc += off;
    if (sb.fold) sb.fold += off;
    if (sb.fout) sb.fout += off;
    if (sb.force) sb.force += off;
  }
  for (int y = tid; y < g.ny; y += kAnyT) buf[y] = nl[(size_t)y * g.pitch + x];
  __syncthreads();
  fft_any(buf, tmp, py, wy, false, tid, kAnyT);
  bool bad = false;
  const double dt = p.dt;
  for (int y = tid; y < g.ny; y += kAnyT) {
    const size_t q = (size_t)y * g.pitch + x;
    double nr = 0.0, ni = 0.0;
    if (x < g.i0[y]) {  // 2/3 truncation of the nonlinear term only
      nr = buf[y].x * p.nl_scale;
      ni = buf[y].y * p.nl_scale;
    }
    const double kx = g.kx[x], ky = g.ky[y];
    const double k2 = kx * kx + ky * ky;
    const double vk2 = p.nu * k2;
    const double2 w = sb.win[q];
    double fr, fi;
    if (p.rhs == 0) {
      fr = -(nr + vk2 * w.x);
      fi = -(ni + vk2 * w.y);
    } else {
      const double inv = g.inv[(size_t)y * g.nh + x];  // 1/(k^2+lambda), 0 at k = 0
      const double dr = k2 * (w.x * inv), di = k2 * (w.y * inv);
      fr = -(p.alpha * nr + vk2 * dr);
      fi = -(p.alpha * ni + vk2 * di);
    }
    if (sb.force) {
      const double2 fc = sb.force[q];
      fr += fc.x;
      fi += fc.y;
    }
    bad |= !(finite_bits(fr) && finite_bits(fi));
    double2 s = make_double2(0.0, 0.0), a1 = s;
    if (mode == MODE_AB2) {
      s = sb.w0[q];
      a1 = sb.fold[q];
    } else if (mode != MODE_DERIVE) {
      s = sb.w0[q];
      if (mode != MODE_RK1) a1 = sb.acc[q];
    }
    switch (mode) {
      case MODE_DERIVE:
        sb.fout[q] = make_double2(fr, fi);
        break;
      case MODE_AB2:
        sb.w0[q] = make_double2(s.x + (1.5 * fr - 0.5 * a1.x) * dt, s.y + (1.5 * fi - 0.5 * a1.y) * dt);
        sb.fold[q] = make_double2(fr, fi);
        break;
      case MODE_RK1:
        sb.acc[q] = make_double2(fr, fi);
        sb.ws[q] = make_double2(s.x + fr * dt / 2.0, s.y + fi * dt / 2.0);
        break;
      case MODE_RK2:
      case MODE_RK3: {
        const double hh = (mode == MODE_RK2) ? dt / 2.0 : dt;
        sb.acc[q] = make_double2(a1.x + 2.0 * fr, a1.y + 2.0 * fi);
        sb.ws[q] = make_double2(s.x + fr * hh, s.y + fi * hh);
        break;
      }
      default:  // MODE_RK4
        sb.w0[q] = make_double2(s.x + dt / 6.0 * (a1.x + fr), s.y + dt / 6.0 * (a1.y + fi));
        break;
    }
  }
  if (bad) atomicOr(sb.flag, 1u);
}

// Plain transforms: columns along y (field blockIdx.y), in or out of place.
__global__ void __launch_bounds__(kAnyT) k_any_col_fft(const double2* in, double2* out, int nh, int pitch,
                                                      size_t fs, AnyPlan py, const double2* __restrict__ wy,
                                                      int inverse) {
  extern __shared__ __align__(16) double2 any_sm[];
  const int n = py.n, x = blockIdx.x, tid = threadIdx.x;
  double2* buf = any_sm;
  double2* tmp = any_sm + n;
  in += blockIdx.y * fs;
  out += blockIdx.y * fs;
  for (int y = tid; y < n; y += kAnyT) buf[y] = in[(size_t)y * pitch + x];
  __syncthreads();
  fft_any(buf, tmp, py, wy, inverse != 0, tid, kAnyT);
  for (int y = tid; y < n; y += kAnyT) out[(size_t)y * pitch + x] = buf[y];
  (void)nh;
}

// 1D c2r along x of the row pair (2 blockIdx.x, +1) of field blockIdx.y.
__global__ void __launch_bounds__(kAnyT) k_any_row_c2r(const double2* __restrict__ in, double* __restrict__ out,
                                                      int ny, int pitch, int rpitch, size_t fs_in, size_t fs_out,
                                                      AnyPlan px, const double2* __restrict__ wx) {
  extern __shared__ __align__(16) double2 any_sm[];
  const int n = px.n, tid = threadIdx.x, ya = 2 * blockIdx.x;
  double2* buf = any_sm;
  double2* tmp = any_sm + n;
  in += blockIdx.y * fs_in;
  out += blockIdx.y * fs_out;
  for (int k = tid; k < n; k += kAnyT) {
    // (ny is even on this path)
    const double2* fa = in + (size_t)ya * pitch;
    buf[k] = any_pair_entry(fa, fa + pitch, k, n);
  }
  __syncthreads();
  fft_any(buf, tmp, px, wx, true, tid, kAnyT);
  for (int x = tid; x < n; x += kAnyT) {
    if (ya < ny) out[(size_t)ya * rpitch + x] = buf[x].x;
    if (ya + 1 < ny) out[(size_t)(ya + 1) * rpitch + x] = buf[x].y;
  }
}

// 1D r2c along x of the real row pair (2 blockIdx.x, +1) of field blockIdx.y.
__global__ void __launch_bounds__(kAnyT) k_any_row_r2c(const double* __restrict__ in, double2* __restrict__ out,
                                                      int ny, int rpitch, int pitch, size_t fs_in, size_t fs_out,
                                                      AnyPlan px, const double2* __restrict__ wx) {
  extern __shared__ __align__(16) double2 any_sm[];
  const int n = px.n, h = n / 2, tid = threadIdx.x, ya = 2 * blockIdx.x;
  double2* buf = any_sm;
  double2* tmp = any_sm + n;
  in += blockIdx.y * fs_in;
  out += blockIdx.y * fs_out;
  for (int x = tid; x < n; x += kAnyT)
    buf[x] = make_double2(ya < ny ? in[(size_t)ya * rpitch + x] : 0.0,
                          ya + 1 < ny ? in[(size_t)(ya + 1) * rpitch + x] : 0.0);
  __syncthreads();
  fft_any(buf, tmp, px, wx, false, tid, kAnyT);
  for (int k = tid; k <= h; k += kAnyT) {
    const double2 z = buf[k], m = buf[(n - k) % n];
    if (ya < ny) out[(size_t)ya * pitch + k] = make_double2(0.5 * (z.x + m.x), 0.5 * (z.y - m.y));
    if (ya + 1 < ny) out[(size_t)(ya + 1) * pitch + k] = make_double2(0.5 * (z.y + m.y), -0.5 * (z.x - m.x));
  }
}

// ---------------------------------------------------------------------------
// host side
bool any_size_2d(int n) { return !is_pow2_in_range(n) && any_size_ok(n); }

namespace any2d {

static int plan_of(int n, AnyPlan* p) {
  if (!any_plan(n, p)) return set_error(TARA_ERR_ARGS, "grid size has a prime factor other than 2, 3, 5, 7");
  return TARA_OK;
}

template <typename K>
static cudaError_t smem_attr(K kernel, size_t bytes) {
  if (bytes <= 48 * 1024) return cudaSuccess;
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

int col_inverse(int ny, int nh, const double2* win, void* u, const Grid2D& g, const RhsParams& p, const void* twy,
                cudaStream_t s, int nb) {
  AnyPlan py;
  int rc;
  if ((rc = plan_of(ny, &py))) return rc;
  const size_t sm = 2 * (size_t)ny * sizeof(double2);
  TARA_CK(smem_attr(k_any_col_inverse, sm));
  k_any_col_inverse<<<dim3(nh, 1, nb), kAnyT, sm, s>>>(win, (double2*)u, g, p, py, (const double2*)twy);
  TARA_CK(cudaGetLastError());
  return TARA_OK;
}

int row_nl(int nx, int ny, const void* u, void* nl, const Grid2D& g, const void* twx, cudaStream_t s, int nb) {
  AnyPlan px;
  int rc;
  if ((rc = plan_of(nx, &px))) return rc;
  const size_t sm = 4 * (size_t)nx * sizeof(double2);
  TARA_CK(smem_attr(k_any_row_nl, sm));
  k_any_row_nl<<<dim3((ny + 1) / 2, nb), kAnyT, sm, s>>>((const double2*)u, (double2*)nl, g, px,
                                                        (const double2*)twx);
  TARA_CK(cudaGetLastError());
  return TARA_OK;
}

int col_forward(int ny, int nh, const void* nl, const StepBufs& sb, const Grid2D& g, const RhsParams& p, int mode,
                const void* twy, cudaStream_t s, int nb) {
  AnyPlan py;
  int rc;
  if ((rc = plan_of(ny, &py))) return rc;
  const size_t sm = 2 * (size_t)ny * sizeof(double2);
  TARA_CK(smem_attr(k_any_col_forward, sm));
  k_any_col_forward<<<dim3(nh, nb), kAnyT, sm, s>>>((const double2*)nl, sb, g, p, mode, py, (const double2*)twy);
  TARA_CK(cudaGetLastError());
  return TARA_OK;
}

int col_fft(int ny, int nh, int pitch, const void* in, void* out, bool inverse, const void* twy, cudaStream_t s,
            int nf, size_t fs) {
  AnyPlan py;
  int rc;
  if ((rc = plan_of(ny, &py))) return rc;
  const size_t sm = 2 * (size_t)ny * sizeof(double2);
  TARA_CK(smem_attr(k_any_col_fft, sm));
  k_any_col_fft<<<dim3(nh, nf), kAnyT, sm, s>>>((const double2*)in, (double2*)out, nh, pitch, fs, py,
                                                (const double2*)twy, inverse ? 1 : 0);
  TARA_CK(cudaGetLastError());
  return TARA_OK;
}

int row_c2r(int nx, int ny, int pitch, int rpitch, const void* in, void* out, const void* twx, cudaStream_t s, int nf,
            size_t fs_in, size_t fs_out) {
  AnyPlan px;
  int rc;
  if ((rc = plan_of(nx, &px))) return rc;
  const size_t sm = 2 * (size_t)nx * sizeof(double2);
  TARA_CK(smem_attr(k_any_row_c2r, sm));
  k_any_row_c2r<<<dim3((ny + 1) / 2, nf), kAnyT, sm, s>>>((const double2*)in, (double*)out, ny, pitch, rpitch,
                                                         fs_in, fs_out, px, (const double2*)twx);
  TARA_CK(cudaGetLastError());
  return TARA_OK;
}

int row_r2c(int nx, int ny, int rpitch, int pitch, const void* in, void* out, const void* twx, cudaStream_t s, int nf,
            size_t fs_in, size_t fs_out) {
  AnyPlan px;
  int rc;
  if ((rc = plan_of(nx, &px))) return rc;
  const size_t sm = 2 * (size_t)nx * sizeof(double2);
  TARA_CK(smem_attr(k_any_row_r2c, sm));
  k_any_row_r2c<<<dim3((ny + 1) / 2, nf), kAnyT, sm, s>>>((const double*)in, (double2*)out, ny, rpitch, pitch,
                                                         fs_in, fs_out, px, (const double2*)twx);
  TARA_CK(cudaGetLastError());
  return TARA_OK;
}

// The root table of a mixed-radix length: exp(-2 pi i t / n), t < n.
int make_roots(int n, void** dev) {
  std::vector<double2> w(n);
  for (int t = 0; t < n; ++t) {
    const long double a = 6.283185307179586476925286766559005768L * (long double)t / (long double)n;
    w[t] = make_double2((double)cosl(a), (double)-sinl(a));
  }
  TARA_CK(cudaMalloc(dev, n * sizeof(double2)));
  TARA_CK(cudaMemcpy(*dev, w.data(), n * sizeof(double2), cudaMemcpyHostToDevice));
  return TARA_OK;
}

}  // namespace any2d
}  // namespace tara
