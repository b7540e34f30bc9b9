// 2D compressible MHD: the reference's derive2com (src/derive2com.f95:5-426)
// and ab2com (src/ab2com.f95) on the GPU, and the initial state of its driver
// tara2dMHDOMP (src/main2com.f95:229-291).
//
// State: six half spectra [Ny][pitch] of double2 -- rho, rho ux, rho uy, E, Bx,
// By.  One right-hand side (13 launches):
//   1. k_com_prep + col_fft + row_c2r  the six fields on the grid (and, in the
//      defined mode, dBx/dy and dBy/dx)
//   2. k_com_vel     ux = rho ux / rho, uy, and the forcing -rho A sin(kf y),
//                    rho A sin(kf x) (skipped when A = 0)
//   3. row_r2c + col_fft   ux_k, uy_k (and the forcing spectra)
//   4. k_com_dspec + col_fft + row_c2r   d ux/dx, d uy/dy
//   5. k_com_terms   the flux fields of :181-213: Mom_x_1, Mom_x_2, Mom_y_2,
//                    Energy_x, Energy_y, E_Visc, Mag_x
//   6. row_r2c + col_fft   their spectra
//   7. k_com_final   the spectral derivatives, the 2/3 rule (on every term but the
//                    forcing, as :296-338), the sums of :345-364, and AB2 with the
//                    driver's history rotation (src/main2com.f95:375-414)
// Two of the reference's nine forward transforms are exact copies: Mom_y_1 is
// Mom_x_2 (both rho_ux uy - Bx By) and Mag_y is -Mag_x (the same two products
// subtracted the other way round), so seven are computed.  The reference also
// transforms dBx/dy and dBy/dx and then overwrites them with d_ux_dx/(Nx Ny) and
// d_uy_dy/(Nx Ny) (:186-187); the faithful mode skips those two transforms and
// forms curl B as the reference does, the defined mode transforms and uses them.
// The forcing's x(i), y(j) are local arrays the reference never sets
// (:16,109-110): here they are the driver's grid, (i-1) Lx/Nx and (j-1) Ly/Ny.
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "internal.h"

struct tara_com2d {
  tara_com2d_config cfg;
  int dev = 0, nx = 0, ny = 0, nh = 0, pitch = 0, rpitch = 0;
  size_t fs = 0, rfs = 0;
  cudaStream_t stream = nullptr;
  double2 *st = nullptr, *hist = nullptr, *dnew = nullptr;
  double2 *specA = nullptr;  // 8 spectra: the state's inverse transforms, later the fluxes'
  double2 *specB = nullptr;  // 4 spectra: ux_k, uy_k, Fx_k, Fy_k
  double *reA = nullptr, *reB = nullptr, *reC = nullptr, *reD = nullptr;  // 8, 4, 2, 7 real fields
  double *kx = nullptr, *ky = nullptr, *sx = nullptr, *sy = nullptr;
  double* diag = nullptr;  // per-block partial sums of the driver diagnostics
  int* i0 = nullptr;
  void *twx = nullptr, *twy = nullptr;
  unsigned int* flag = nullptr;
};

namespace tara {
namespace {

constexpr int kElemBlocks = 152 * 8, kElemThreads = 256;
constexpr int kFlux = 7;

__global__ void k_com_prep(const double2* __restrict__ st, size_t fs, const double* __restrict__ kx,
                           const double* __restrict__ ky, int nh, int ny, int pitch, int defined,
                           double2* __restrict__ sp) {
  const size_t total = (size_t)ny * nh;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const int y = (int)(t / nh), x = (int)(t % nh);
    const size_t q = (size_t)y * pitch + x;
#pragma unroll
    for (int f = 0; f < 6; ++f) sp[f * fs + q] = st[f * fs + q];
    if (defined) {  // (0,1) ky Bx_k, (0,1) kx By_k  (:146-147)
      const double2 bx = st[4 * fs + q], by = st[5 * fs + q];
      sp[6 * fs + q] = make_double2(-ky[y] * bx.y, ky[y] * bx.x);
      sp[7 * fs + q] = make_double2(-kx[x] * by.y, kx[x] * by.x);
    }
  }
}

// :88-118: normalisation, velocity, forcing
__global__ void k_com_vel(const double* __restrict__ re, size_t rfs, int nx, int ny, int rpitch, double inv_nn,
                          double a, const double* __restrict__ sx, const double* __restrict__ sy,
                          double* __restrict__ out) {
  const size_t total = (size_t)ny * nx;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const int j = (int)(t / nx), i = (int)(t % nx);
    const size_t r = (size_t)j * rpitch + i;
    const double rho = re[r] * inv_nn;
    out[r] = (re[rfs + r] * inv_nn) / rho;
    out[rfs + r] = (re[2 * rfs + r] * inv_nn) / rho;
    if (a != 0.0) {
      out[2 * rfs + r] = -(rho * a * sy[j]);
      out[3 * rfs + r] = rho * a * sx[i];
    }
  }
}

// (0,1) kx ux_k, (0,1) ky uy_k  (:136-160)
__global__ void k_com_dspec(const double2* __restrict__ vk, size_t fs, const double* __restrict__ kx,
                            const double* __restrict__ ky, int nh, int ny, int pitch, double2* __restrict__ sp) {
  const size_t total = (size_t)ny * nh;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const int y = (int)(t / nh), x = (int)(t % nh);
    const size_t q = (size_t)y * pitch + x;
    const double2 u = vk[q], v = vk[fs + q];
    sp[q] = make_double2(-kx[x] * u.y, kx[x] * u.x);
    sp[fs + q] = make_double2(-ky[y] * v.y, ky[y] * v.x);
  }
}

// :181-213 (seven of the nine fields; see the file comment)
__global__ void k_com_terms(const double* __restrict__ reA, const double* __restrict__ reB,
                            const double* __restrict__ reC, size_t rfs, int nx, int ny, int rpitch, double inv_nn,
                            double cs2, double eta, int defined, double* __restrict__ out) {
  const size_t total = (size_t)ny * nx;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const size_t r = (t / nx) * rpitch + (t % nx);
    const double d_ux_dx = reC[r] * inv_nn, d_uy_dy = reC[rfs + r] * inv_nn;
    double d_Bx_dy, d_By_dx;
    if (defined) {
      d_Bx_dy = reA[6 * rfs + r] * inv_nn;
      d_By_dx = reA[7 * rfs + r] * inv_nn;
    } else {  // :186-187
      d_Bx_dy = d_ux_dx * inv_nn;
      d_By_dx = d_uy_dy * inv_nn;
    }
    const double curl_B = d_By_dx - d_Bx_dy;
    const double rho = reA[r] * inv_nn, rho_ux = reA[rfs + r] * inv_nn, rho_uy = reA[2 * rfs + r] * inv_nn;
    const double E = reA[3 * rfs + r] * inv_nn, Bx = reA[4 * rfs + r] * inv_nn, By = reA[5 * rfs + r] * inv_nn;
    const double ux = reB[r], uy = reB[rfs + r];
    const double B2 = Bx * Bx + By * By;
    const double P = cs2 * rho;
    out[r] = rho_ux * ux + P + B2 / 2.0 - Bx * Bx;            // Mom_x_1
    out[rfs + r] = rho_ux * uy - Bx * By;                     // Mom_x_2 (= Mom_y_1)
    out[2 * rfs + r] = rho_uy * uy + P + B2 / 2.0 - By * By;  // Mom_y_2
    const double h = E + P + B2 / 2.0;
    out[3 * rfs + r] = (h * ux - ux * Bx * Bx - uy * Bx * By) - eta * By * curl_B;  // Energy_x
    out[4 * rfs + r] = (h * uy - ux * Bx * By - uy * By * By) + eta * Bx * curl_B;  // Energy_y
    const double dv = d_ux_dx + d_uy_dy;
    out[5 * rfs + r] = dv * dv;                               // E_Visc
    out[6 * rfs + r] = uy * Bx - By * ux;                     // Mag_x (= -Mag_y)
  }
}

__device__ __forceinline__ double ik_re(double k, double2 f) { return -k * f.y; }
__device__ __forceinline__ double ik_im(double k, double2 f) { return k * f.x; }

// :248-364 and the AB2 update (mode 1) or the bare derivative (mode 0)
__global__ void k_com_final(const double2* __restrict__ fl, const double2* __restrict__ vk, size_t fs,
                            const double* __restrict__ kx, const double* __restrict__ ky,
                            const int* __restrict__ i0, int nh, int ny, int pitch, double mu, double eta,
                            int forced, int mode, double dt, double2* st, double2* hist,
                            double2* __restrict__ dnew, unsigned int* flag) {
  const size_t total = (size_t)ny * nh;
  bool bad = false;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const int y = (int)(t / nh), x = (int)(t % nh);
    const size_t q = (size_t)y * pitch + x;
    const double a = kx[x], b = ky[y];
    const double m = x < i0[y] ? 1.0 : 0.0;  // the 2/3 rule zeroes every term but the forcing
    const double2 rux = st[fs + q], ruy = st[2 * fs + q], bx = st[4 * fs + q], by = st[5 * fs + q];
    const double2 m11 = fl[q], m12 = fl[fs + q], m22 = fl[2 * fs + q], ex = fl[3 * fs + q];
    const double2 ey = fl[4 * fs + q], ev = fl[5 * fs + q], mgx = fl[6 * fs + q];
    const double2 ux = vk[q], uy = vk[fs + q];
    const double2 fx = forced ? vk[2 * fs + q] : make_double2(0.0, 0.0);
    const double2 fy = forced ? vk[3 * fs + q] : make_double2(0.0, 0.0);
    double2 d[6];
#pragma unroll
    for (int c = 0; c < 2; ++c) {
#define CMP(v) ((c) == 0 ? (v).x : (v).y)
#define IK(k, v) ((c) == 0 ? ik_re(k, v) : ik_im(k, v))
      const double drho = -(m * IK(a, rux) + m * IK(b, ruy));
      double dux = -(m * IK(a, m11) + m * IK(b, m12));
      dux = dux - mu * (m * (a * a * CMP(ux)) + m * (b * b * CMP(ux))) + CMP(fx);
      double duy = -(m * IK(a, m12) + m * IK(b, m22));
      duy = duy - mu * (m * (a * a * CMP(uy)) + m * (b * b * CMP(uy))) + CMP(fy);
      double dE = -(m * IK(a, ex) + m * IK(b, ey));
      dE = dE + mu * (m * CMP(ev));
      const double dbx = -(m * IK(b, mgx)) - eta * (m * (a * a * CMP(bx)) + m * (b * b * CMP(bx)));
      // Mag_y = -Mag_x: -(0,1) kx Mag_y_k = (0,1) kx Mag_x_k
      const double dby = (m * IK(a, mgx)) - eta * (m * (a * a * CMP(by)) + m * (b * b * CMP(by)));
#undef CMP
#undef IK
      const double v[6] = {drho, dux, duy, dE, dbx, dby};
#pragma unroll
      for (int f = 0; f < 6; ++f) {
        if (c == 0)
          d[f].x = v[f];
        else
          d[f].y = v[f];
      }
    }
#pragma unroll
    for (int f = 0; f < 6; ++f) {
      const size_t o = f * fs + q;
      bad |= !(finite_bits(d[f].x) && finite_bits(d[f].y));
      if (mode == 0) {
        dnew[o] = d[f];
      } else {
        const double2 s = st[o], fo = hist[o];
        st[o] = make_double2(s.x + ((3.0 / 2.0) * d[f].x - (1.0 / 2.0) * fo.x) * dt,
                             s.y + ((3.0 / 2.0) * d[f].y - (1.0 / 2.0) * fo.y) * dt);
        hist[o] = d[f];
      }
    }
  }
  if (bad) atomicOr(flag, 1u);
}

// Driver diagnostics (src/main2com.f95:415-586).
// The six fields and div B = (0,1) kx Bx_k + (0,1) ky By_k on the grid.
__global__ void k_com_diag_spec(const double2* __restrict__ st, size_t fs, const double* __restrict__ kx,
                                const double* __restrict__ ky, int nh, int ny, int pitch,
                                double2* __restrict__ sp) {
  const size_t total = (size_t)ny * nh;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const int y = (int)(t / nh), x = (int)(t % nh);
    const size_t q = (size_t)y * pitch + x;
#pragma unroll
    for (int f = 0; f < 6; ++f) sp[f * fs + q] = st[f * fs + q];
    const double2 bx = st[4 * fs + q], by = st[5 * fs + q];
    const double a = kx[x], b = ky[y];
    sp[6 * fs + q] = make_double2((-a * bx.y) + (-b * by.y), (a * bx.x) + (b * by.x));
  }
}

// ux = rho_ux / rho, uy from the normalised fields (:473-488)
__global__ void k_com_diag_vel(const double* __restrict__ re, size_t rfs, int nx, int ny, int rpitch, double nn,
                               double* __restrict__ out) {
  const size_t total = (size_t)ny * nx;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const size_t r = (t / nx) * rpitch + (t % nx);
    const double rho = re[r] / nn;
    out[r] = (re[rfs + r] / nn) / rho;
    out[rfs + r] = (re[2 * rfs + r] / nn) / rho;
  }
}

// omega_k = (0,1) kx uy_k - (0,1) ky ux_k, j_k = (0,1) kx By_k - (0,1) ky Bx_k (:500-520)
__global__ void k_com_diag_curl(const double2* __restrict__ vk, const double2* __restrict__ st, size_t fs,
                                const double* __restrict__ kx, const double* __restrict__ ky, int nh, int ny,
                                int pitch, double2* __restrict__ sp) {
  const size_t total = (size_t)ny * nh;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const int y = (int)(t / nh), x = (int)(t % nh);
    const size_t q = (size_t)y * pitch + x;
    const double a = kx[x], b = ky[y];
    const double2 ux = vk[q], uy = vk[fs + q], bx = st[4 * fs + q], by = st[5 * fs + q];
    sp[q] = make_double2((-a * uy.y) - (-b * ux.y), (a * uy.x) - (b * ux.x));
    sp[fs + q] = make_double2((-a * by.y) - (-b * bx.y), (a * by.x) - (b * bx.x));
  }
}

constexpr int kDiagBlocksM = 304;

// Per-block sums of (ux^2+uy^2)/N^2, (Bx^2+By^2)/N^2, omega^2/N^2, j^2/N^2,
// divB/N^2 (:560-575); reA holds the six unnormalised fields and div B.
__global__ void __launch_bounds__(256) k_com_diag_sum(const double* __restrict__ reA, const double* __restrict__ reB,
                                                      const double* __restrict__ reC, size_t rfs, int nx, int ny,
                                                      int rpitch, double nn, double* __restrict__ part) {
  double acc[5] = {0, 0, 0, 0, 0};
  const size_t total = (size_t)ny * nx;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const size_t r = (t / nx) * rpitch + (t % nx);
    const double ux = reB[r], uy = reB[rfs + r];
    const double bx = reA[4 * rfs + r] / nn, by = reA[5 * rfs + r] / nn, divb = reA[6 * rfs + r] / nn;
    const double w = reC[r] / nn, jb = reC[rfs + r] / nn;
    acc[0] += (ux * ux + uy * uy) / nn;
    acc[1] += (bx * bx + by * by) / nn;
    acc[2] += pow(w, 2.0) / nn;
    acc[3] += pow(jb, 2.0) / nn;
    acc[4] += divb / nn;
  }
  __shared__ double sh[5][8];
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    double v = acc[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) sh[k][threadIdx.x >> 5] = v;
  }
  __syncthreads();
  if (threadIdx.x < 5) {
    double v = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += sh[threadIdx.x][w];
    part[blockIdx.x * 5 + threadIdx.x] = v;
  }
}

int com_copy_in(tara_com2d* h, double2* dst, const double* host) {
  TARA_CK(cudaMemcpy2DAsync(dst, h->pitch * sizeof(double2), host, h->nh * sizeof(double2),
                            h->nh * sizeof(double2), h->ny, cudaMemcpyHostToDevice, h->stream));
  return TARA_OK;
}

int com_copy_out(tara_com2d* h, double* host, const double2* src) {
  TARA_CK(cudaMemcpy2DAsync(host, h->nh * sizeof(double2), src, h->pitch * sizeof(double2),
                            h->nh * sizeof(double2), h->ny, cudaMemcpyDeviceToHost, h->stream));
  return TARA_OK;
}

int com_rhs(tara_com2d* h, int mode) {
  const tara_com2d_config& c = h->cfg;
  cudaStream_t s = h->stream;
  const int nA = c.defined ? 8 : 6;
  const bool forced = c.a != 0.0;
  const double inv_nn = 1.0 / ((double)h->nx * (double)h->ny);
  int rc;
  k_com_prep<<<kElemBlocks, kElemThreads, 0, s>>>(h->st, h->fs, h->kx, h->ky, h->nh, h->ny, h->pitch, c.defined,
                                                   h->specA);
  TARA_CK(cudaGetLastError());
  if ((rc = Launch2D<double>::col_fft(h->ny, h->nh, h->pitch, h->specA, h->specA, true, h->twy, s, nA, h->fs)))
    return rc;
  if ((rc = Launch2D<double>::row_c2r(h->nx, h->ny, h->pitch, h->rpitch, h->specA, h->reA, h->twx, s, nA, h->fs,
                                      h->rfs)))
    return rc;
  k_com_vel<<<kElemBlocks, kElemThreads, 0, s>>>(h->reA, h->rfs, h->nx, h->ny, h->rpitch, inv_nn, c.a, h->sx,
                                                  h->sy, h->reB);
  TARA_CK(cudaGetLastError());
  const int nB = forced ? 4 : 2;
  if ((rc = Launch2D<double>::row_r2c(h->nx, h->ny, h->rpitch, h->pitch, h->reB, h->specB, h->twx, s, nB, h->rfs,
                                      h->fs)))
    return rc;
  if ((rc = Launch2D<double>::col_fft(h->ny, h->nh, h->pitch, h->specB, h->specB, false, h->twy, s, nB, h->fs)))
    return rc;
  k_com_dspec<<<kElemBlocks, kElemThreads, 0, s>>>(h->specB, h->fs, h->kx, h->ky, h->nh, h->ny, h->pitch,
                                                    h->specA);
  TARA_CK(cudaGetLastError());
  if ((rc = Launch2D<double>::col_fft(h->ny, h->nh, h->pitch, h->specA, h->specA, true, h->twy, s, 2, h->fs)))
    return rc;
  if ((rc = Launch2D<double>::row_c2r(h->nx, h->ny, h->pitch, h->rpitch, h->specA, h->reC, h->twx, s, 2, h->fs,
                                      h->rfs)))
    return rc;
  k_com_terms<<<kElemBlocks, kElemThreads, 0, s>>>(h->reA, h->reB, h->reC, h->rfs, h->nx, h->ny, h->rpitch, inv_nn,
                                                    c.cs * c.cs, c.eta, c.defined, h->reD);
  TARA_CK(cudaGetLastError());
  if ((rc = Launch2D<double>::row_r2c(h->nx, h->ny, h->rpitch, h->pitch, h->reD, h->specA, h->twx, s, kFlux,
                                      h->rfs, h->fs)))
    return rc;
  if ((rc = Launch2D<double>::col_fft(h->ny, h->nh, h->pitch, h->specA, h->specA, false, h->twy, s, kFlux, h->fs)))
    return rc;
  k_com_final<<<kElemBlocks, kElemThreads, 0, s>>>(h->specA, h->specB, h->fs, h->kx, h->ky, h->i0, h->nh, h->ny,
                                                    h->pitch, c.mu, c.eta, forced ? 1 : 0, mode, c.dt, h->st,
                                                    h->hist, h->dnew, h->flag);
  TARA_CK(cudaGetLastError());
  return TARA_OK;
}

int com_check(tara_com2d* h) {
  unsigned int f = 0;
  TARA_CK(cudaMemcpyAsync(&f, h->flag, sizeof(f), cudaMemcpyDeviceToHost, h->stream));
  TARA_CK(cudaStreamSynchronize(h->stream));
  if (f) return set_error(TARA_ERR_NONFINITE, "non-finite value in the compressible MHD update");
  return TARA_OK;
}

// Wavenumbers, the 2/3 rule's first removed column per row and the forcing's
// sine tables sin(kf x_i), sin(kf y_j) (host libm, as the oracle).
int com_tables(tara_com2d* h) {
  const tara_com2d_config& c = h->cfg;
  std::vector<double> kx(h->nh), ky(h->ny), sx(h->nx), sy(h->ny);
  std::vector<int> i0(h->ny);
  make_wavenumbers(h->nx, h->ny, c.kpi, c.lx, c.ly, kx.data(), ky.data(), i0.data());
  const double dx = c.lx / (double)h->nx, dy = c.ly / (double)h->ny;
  for (int i = 0; i < h->nx; ++i) sx[i] = std::sin(c.kf * ((double)(float)i * dx));
  for (int j = 0; j < h->ny; ++j) sy[j] = std::sin(c.kf * ((double)(float)j * dy));
  if (cudaMemcpy(h->kx, kx.data(), h->nh * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(h->ky, ky.data(), h->ny * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(h->sx, sx.data(), h->nx * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(h->sy, sy.data(), h->ny * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(h->i0, i0.data(), h->ny * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess)
    return set_error(TARA_ERR_CUDA, "table upload");
  return TARA_OK;
}

// Fortran common block /comm/ as src/derive2com.f95:43 and src/ab2com.f95 read it.
struct ComCommon {
  double Lx, Ly, spheat, mu, ms, CS, mu_0, eta, dt, kf, A;
};
static_assert(sizeof(ComCommon) <= sizeof(TaraMhdCommon), "the common block storage holds both views");

std::mutex g_com_mu;
std::map<std::tuple<int, int>, tara_com2d*> g_com_ctx;

tara_com2d* com_ctx(int nx, int ny, double pi) {
  ComCommon cm;  // a copy: the block's storage is declared with the 3D layout
  std::memcpy(&cm, &comm_, sizeof cm);
  if (!(cm.Lx > 0.0) || !(cm.Ly > 0.0)) {
    set_error(TARA_ERR_ARGS, "/comm/ Lx and Ly must be positive");
    return nullptr;
  }
  auto key = std::make_tuple(nx, ny);
  tara_com2d* h = nullptr;
  auto it = g_com_ctx.find(key);
  tara_com2d_config want;
  tara_com2d_default_config(&want, nx, ny);
  want.kpi = pi;
  want.lx = cm.Lx;
  want.ly = cm.Ly;
  want.mu = cm.mu;
  want.eta = cm.eta;
  want.cs = cm.CS;
  want.kf = cm.kf;
  want.a = cm.A;
  want.dt = cm.dt;
  if (it != g_com_ctx.end()) {
    h = it->second;
  } else {
    if (tara_com2d_create(&want, &h) != TARA_OK) return nullptr;
    g_com_ctx[key] = h;
    return h;
  }
  tara_com2d_config& c = h->cfg;
  const bool geom = c.kpi != want.kpi || c.lx != want.lx || c.ly != want.ly || c.kf != want.kf;
  const int defined = c.defined;
  c = want;
  c.defined = defined;
  if (geom && com_tables(h)) return nullptr;
  return h;
}

bool com_dims(const int* Nx, const int* Ny, const int* Nh, const double* pi) {
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

void tara_com2d_default_config(tara_com2d_config* c, int nx, int ny) {
  if (!c) return;
  const double pi = 3.14159265358979323846;
  c->nx = nx;
  c->ny = ny;
  c->defined = 0;
  c->kpi = pi;
  c->lx = 2.0 * pi;
  c->ly = 2.0 * pi;
  c->mu = 1e-3;     // the ini's nu (src/main2com.f95:164)
  c->eta = 1e-4;    // :167
  c->cs = 100.0;    // 1/M, M = 0.01 (:181-193)
  c->kf = 1.0;      // :209
  c->a = 1.0;       // :215
  c->dt = 1e-4;
}

int tara_com2d_destroy(tara_com2d* h) {
  if (!h) return set_ok();
  cudaSetDevice(h->dev);
  if (h->stream) cudaStreamSynchronize(h->stream);
  void* ptrs[] = {h->st, h->hist, h->dnew, h->specA, h->specB, h->reA, h->reB, h->reC, h->reD,
                  h->kx, h->ky,   h->sx,   h->sy,    h->diag,  h->i0,  h->twx, h->twy, h->flag};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return set_ok();
}

int tara_com2d_create(const tara_com2d_config* cfg, tara_com2d** out) {
  if (!cfg || !out) return set_error(TARA_ERR_ARGS, "null argument");
  *out = nullptr;
  if (!is_size_2d(cfg->nx) || !is_size_2d(cfg->ny))
    return set_error(TARA_ERR_ARGS,
                     "nx and ny must be powers of two in [16, 4096] or even lengths 8 to 3600 with factors 2, 3, 5, 7");
  if (!(cfg->lx > 0.0) || !(cfg->ly > 0.0) || !(cfg->kpi > 0.0))
    return set_error(TARA_ERR_ARGS, "box lengths and kpi must be positive");
  tara_com2d* h = new tara_com2d();
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
    tara_com2d_destroy(h);
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
  CKC(cudaMalloc(&h->st, 6 * sb));
  CKC(cudaMalloc(&h->hist, 6 * sb));
  CKC(cudaMalloc(&h->dnew, 6 * sb));
  CKC(cudaMalloc(&h->specA, 8 * sb));
  CKC(cudaMalloc(&h->specB, 4 * sb));
  CKC(cudaMalloc(&h->reA, 8 * rb));
  CKC(cudaMalloc(&h->reB, 4 * rb));
  CKC(cudaMalloc(&h->reC, 2 * rb));
  CKC(cudaMalloc(&h->reD, kFlux * rb));
  CKC(cudaMalloc(&h->kx, h->nh * sizeof(double)));
  CKC(cudaMalloc(&h->ky, h->ny * sizeof(double)));
  CKC(cudaMalloc(&h->sx, h->nx * sizeof(double)));
  CKC(cudaMalloc(&h->sy, h->ny * sizeof(double)));
  CKC(cudaMalloc(&h->i0, h->ny * sizeof(int)));
  CKC(cudaMalloc(&h->flag, sizeof(unsigned int)));
  CKC(cudaMalloc(&h->diag, 5 * kDiagBlocksM * sizeof(double)));
  CKC(cudaMemsetAsync(h->st, 0, 6 * sb, h->stream));
  CKC(cudaMemsetAsync(h->hist, 0, 6 * sb, h->stream));
  CKC(cudaMemsetAsync(h->dnew, 0, 6 * sb, h->stream));
  CKC(cudaMemsetAsync(h->specA, 0, 8 * sb, h->stream));
  CKC(cudaMemsetAsync(h->specB, 0, 4 * sb, h->stream));
  CKC(cudaMemsetAsync(h->reB, 0, 4 * rb, h->stream));
  CKC(cudaMemsetAsync(h->flag, 0, sizeof(unsigned int), h->stream));
#undef CKC
  int rc;
  if ((rc = make_twiddles(h->nx, false, &h->twx)) || (rc = make_twiddles(h->ny, false, &h->twy))) return fail(rc);
  if ((rc = com_tables(h))) return fail(rc);
  if (cudaStreamSynchronize(h->stream) != cudaSuccess) return fail(set_error(TARA_ERR_CUDA, "create"));
  *out = h;
  return set_ok();
}

int tara_com2d_set_state(tara_com2d* h, const double* state6, const double* hist6) {
  if (!h || !state6) return set_error(TARA_ERR_ARGS, "null argument");
  TARA_CK(cudaSetDevice(h->dev));
  const size_t dn = 2 * (size_t)h->nh * h->ny;
  int rc;
  for (int f = 0; f < 6; ++f) {
    if ((rc = com_copy_in(h, h->st + f * h->fs, state6 + f * dn))) return rc;
    if (hist6 && (rc = com_copy_in(h, h->hist + f * h->fs, hist6 + f * dn))) return rc;
  }
  if (!hist6) TARA_CK(cudaMemsetAsync(h->hist, 0, 6 * h->fs * sizeof(double2), h->stream));
  TARA_CK(cudaStreamSynchronize(h->stream));
  return set_ok();
}

int tara_com2d_get_state(tara_com2d* h, double* state6, double* hist6) {
  if (!h || !state6) return set_error(TARA_ERR_ARGS, "null argument");
  TARA_CK(cudaSetDevice(h->dev));
  const size_t dn = 2 * (size_t)h->nh * h->ny;
  int rc;
  for (int f = 0; f < 6; ++f) {
    if ((rc = com_copy_out(h, state6 + f * dn, h->st + f * h->fs))) return rc;
    if (hist6 && (rc = com_copy_out(h, hist6 + f * dn, h->hist + f * h->fs))) return rc;
  }
  TARA_CK(cudaStreamSynchronize(h->stream));
  return set_ok();
}

int tara_com2d_rhs(tara_com2d* h, double* d6) {
  if (!h || !d6) return set_error(TARA_ERR_ARGS, "null argument");
  TARA_CK(cudaSetDevice(h->dev));
  int rc;
  if ((rc = com_rhs(h, 0))) return rc;
  const size_t dn = 2 * (size_t)h->nh * h->ny;
  for (int f = 0; f < 6; ++f)
    if ((rc = com_copy_out(h, d6 + f * dn, h->dnew + f * h->fs))) return rc;
  if ((rc = com_check(h))) return rc;
  return set_ok();
}

int tara_com2d_step(tara_com2d* h, int nsteps) {
  if (!h || nsteps < 0) return set_error(TARA_ERR_ARGS, "bad argument");
  TARA_CK(cudaSetDevice(h->dev));
  int rc;
  for (int s = 0; s < nsteps; ++s)
    if ((rc = com_rhs(h, 1))) return rc;
  return set_ok();
}

int tara_com2d_synchronize(tara_com2d* h) {
  if (!h) return set_error(TARA_ERR_ARGS, "null handle");
  TARA_CK(cudaSetDevice(h->dev));
  int rc;
  if ((rc = com_check(h))) return rc;
  return set_ok();
}

void* tara_com2d_stream(tara_com2d* h) { return h ? (void*)h->stream : nullptr; }

// The six fields, div B, u, omega and j on the grid: reA[0..6] (unnormalised),
// reB[0..1] = ux, uy, reC[0..1] = omega, j (unnormalised).
static int com_grid_fields(tara_com2d* h) {
  cudaStream_t s = h->stream;
  const double nn = (double)h->nx * (double)h->ny;
  int rc;
  k_com_diag_spec<<<kElemBlocks, kElemThreads, 0, s>>>(h->st, h->fs, h->kx, h->ky, h->nh, h->ny, h->pitch,
                                                        h->specA);
  TARA_CK(cudaGetLastError());
  if ((rc = Launch2D<double>::col_fft(h->ny, h->nh, h->pitch, h->specA, h->specA, true, h->twy, s, 7, h->fs)))
    return rc;
  if ((rc = Launch2D<double>::row_c2r(h->nx, h->ny, h->pitch, h->rpitch, h->specA, h->reA, h->twx, s, 7, h->fs,
                                      h->rfs)))
    return rc;
  k_com_diag_vel<<<kElemBlocks, kElemThreads, 0, s>>>(h->reA, h->rfs, h->nx, h->ny, h->rpitch, nn, h->reB);
  TARA_CK(cudaGetLastError());
  if ((rc = Launch2D<double>::row_r2c(h->nx, h->ny, h->rpitch, h->pitch, h->reB, h->specB, h->twx, s, 2, h->rfs,
                                      h->fs)))
    return rc;
  if ((rc = Launch2D<double>::col_fft(h->ny, h->nh, h->pitch, h->specB, h->specB, false, h->twy, s, 2, h->fs)))
    return rc;
  k_com_diag_curl<<<kElemBlocks, kElemThreads, 0, s>>>(h->specB, h->st, h->fs, h->kx, h->ky, h->nh, h->ny,
                                                        h->pitch, h->specA);
  TARA_CK(cudaGetLastError());
  if ((rc = Launch2D<double>::col_fft(h->ny, h->nh, h->pitch, h->specA, h->specA, true, h->twy, s, 2, h->fs)))
    return rc;
  return Launch2D<double>::row_c2r(h->nx, h->ny, h->pitch, h->rpitch, h->specA, h->reC, h->twx, s, 2, h->fs,
                                   h->rfs);
}

int tara_com2d_diag(tara_com2d* h, double* out5) {
  if (!h || !out5) return set_error(TARA_ERR_ARGS, "null argument");
  TARA_CK(cudaSetDevice(h->dev));
  int rc;
  if ((rc = com_grid_fields(h))) return rc;
  const double nn = (double)h->nx * (double)h->ny;
  k_com_diag_sum<<<kDiagBlocksM, 256, 0, h->stream>>>(h->reA, h->reB, h->reC, h->rfs, h->nx, h->ny, h->rpitch, nn,
                                                       h->diag);
  TARA_CK(cudaGetLastError());
  std::vector<double> hp(5 * kDiagBlocksM);
  TARA_CK(cudaMemcpyAsync(hp.data(), h->diag, hp.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  if ((rc = com_check(h))) return rc;
  for (int k = 0; k < 5; ++k) out5[k] = 0.0;
  for (int b = 0; b < kDiagBlocksM; ++b)
    for (int k = 0; k < 5; ++k) out5[k] += hp[b * 5 + k];
  return set_ok();
}

// rho, ux, uy, P = CS^2 rho, E, Bx, By on the grid (the driver's snapshot
// fields, :571-573), each [Ny][Nx]; a null pointer skips a field.
int tara_com2d_real_fields(tara_com2d* h, double* rho, double* ux, double* uy, double* P, double* E, double* Bx,
                           double* By) {
  if (!h) return set_error(TARA_ERR_ARGS, "null handle");
  TARA_CK(cudaSetDevice(h->dev));
  int rc;
  if ((rc = com_grid_fields(h))) return rc;
  const double nn = (double)h->nx * (double)h->ny, cs2 = h->cfg.cs * h->cfg.cs;
  std::vector<double> buf(h->rfs);
  struct F {
    double* out;
    const double* src;
    int mode;  // 0 normalise, 1 as is (ux, uy), 2 CS^2 times the normalised rho
  } fl[7] = {{rho, h->reA, 0}, {ux, h->reB, 1}, {uy, h->reB + h->rfs, 1}, {P, h->reA, 2},
             {E, h->reA + 3 * h->rfs, 0}, {Bx, h->reA + 4 * h->rfs, 0}, {By, h->reA + 5 * h->rfs, 0}};
  for (const F& f : fl) {
    if (!f.out) continue;
    TARA_CK(cudaMemcpyAsync(buf.data(), f.src, h->rfs * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    TARA_CK(cudaStreamSynchronize(h->stream));
    for (int j = 0; j < h->ny; ++j)
      for (int i = 0; i < h->nx; ++i) {
        const double v = buf[(size_t)j * h->rpitch + i];
        f.out[(size_t)j * h->nx + i] = f.mode == 1 ? v : f.mode == 2 ? cs2 * (v / nn) : v / nn;
      }
  }
  return set_ok();
}

int tara_com2d_launches_per_step(tara_com2d* h) { return h ? 13 : 0; }

// src/main2com.f95:229-291 (rho0 = 1, U0 = M CS, B0 = U0/MA sqrt(mu_0 rho0)
// with MA = mu_0 = 1; spheat = 5/3)
int tara_com2d_init_reference(tara_com2d* h, double lx_ini, double ly_ini, double b0) {
  if (!h || !(lx_ini > 0.0) || !(ly_ini > 0.0)) return set_error(TARA_ERR_ARGS, "bad argument");
  TARA_CK(cudaSetDevice(h->dev));
  const double pi = 3.14159265358979323846;
  const double lx = lx_ini * pi, ly = ly_ini * pi;
  const double dx = lx / (double)h->nx, dy = ly / (double)h->ny;
  const double cs = h->cfg.cs, kf = h->cfg.kf, spheat = 5.0 / 3.0;
  std::vector<double> re(6 * h->rfs, 0.0);
  for (int j = 0; j < h->ny; ++j) {
    const double y = (double)(float)j * dy;
    for (int i = 0; i < h->nx; ++i) {
      const double x = (double)(float)i * dx;
      const size_t r = (size_t)j * h->rpitch + i;
      const double rho = 1.0, ux = -std::sin(kf * y), uy = std::sin(kf * x);
      const double P = cs * cs * rho;
      const double E = P / (spheat - 1.0) + 0.50 * rho * (ux * ux + uy * uy) + 0.50 * (b0 * b0 + b0 * b0);
      const double v[6] = {rho, rho * ux, rho * uy, E, b0, b0};
      for (int f = 0; f < 6; ++f) re[f * h->rfs + r] = v[f];
    }
  }
  int rc = TARA_OK;
  if (cudaMemcpyAsync(h->reA, re.data(), 6 * h->rfs * sizeof(double), cudaMemcpyHostToDevice, h->stream) !=
      cudaSuccess)
    rc = set_error(TARA_ERR_CUDA, "initial-condition upload");
  if (!rc)
    rc = Launch2D<double>::row_r2c(h->nx, h->ny, h->rpitch, h->pitch, h->reA, h->st, h->twx, h->stream, 6, h->rfs,
                                   h->fs);
  if (!rc)
    rc = Launch2D<double>::col_fft(h->ny, h->nh, h->pitch, h->st, h->st, false, h->twy, h->stream, 6, h->fs);
  if (!rc && cudaMemsetAsync(h->hist, 0, 6 * h->fs * sizeof(double2), h->stream) != cudaSuccess)
    rc = set_error(TARA_ERR_CUDA, "history reset");
  cudaError_t e = cudaStreamSynchronize(h->stream);
  if (rc) return rc;
  if (e != cudaSuccess) return cuda_fail(e, "initial condition");
  return set_ok();
}

// ---- Fortran drop-ins ------------------------------------------------------

// Replaces subroutine derive2com (src/derive2com.f95:5).
void derive2com_(const int* Nx, const int* Ny, const int* Nh, const double* pi, const double* time,
                 const double* rho_k, const double* rho_ux_k, const double* rho_uy_k, const double* E_k,
                 const double* Bx_k, const double* By_k, double* d_rho_k_dt_old, double* d_rho_k_dt_new,
                 double* d_rho_ux_k_dt_old, double* d_rho_ux_k_dt_new, double* d_rho_uy_k_dt_old,
                 double* d_rho_uy_k_dt_new, double* d_E_k_dt_old, double* d_E_k_dt_new, double* d_Bx_k_dt_old,
                 double* d_Bx_k_dt_new, double* d_By_k_dt_old, double* d_By_k_dt_new) {
  (void)time;
  (void)d_rho_k_dt_old;
  (void)d_rho_ux_k_dt_old;
  (void)d_rho_uy_k_dt_old;
  (void)d_E_k_dt_old;
  (void)d_Bx_k_dt_old;
  (void)d_By_k_dt_old;
  std::lock_guard<std::mutex> lk(g_com_mu);
  if (!com_dims(Nx, Ny, Nh, pi)) return;
  const double* in[6] = {rho_k, rho_ux_k, rho_uy_k, E_k, Bx_k, By_k};
  double* out[6] = {d_rho_k_dt_new, d_rho_ux_k_dt_new, d_rho_uy_k_dt_new, d_E_k_dt_new, d_Bx_k_dt_new, d_By_k_dt_new};
  for (int f = 0; f < 6; ++f)
    if (!in[f] || !out[f]) {
      set_error(TARA_ERR_ARGS, "null array argument");
      return;
    }
  tara_com2d* h = com_ctx(*Nx, *Ny, *pi);
  if (!h) return;
  if (cudaSetDevice(h->dev) != cudaSuccess) {
    set_error(TARA_ERR_CUDA, "cudaSetDevice failed");
    return;
  }
  for (int f = 0; f < 6; ++f)
    if (com_copy_in(h, h->st + f * h->fs, in[f])) return;
  if (com_rhs(h, 0)) return;
  for (int f = 0; f < 6; ++f)
    if (com_copy_out(h, out[f], h->dnew + f * h->fs)) return;
  if (com_check(h)) return;
  set_ok();
}

// Replaces subroutine ab2com (src/ab2com.f95): AB2 of the six fields, dt from /comm/.
void ab2com_(const int* Nx, const int* Ny, const int* Nh, const double* pi, const double* time,
             const double* rho_k, const double* rho_ux_k, const double* rho_uy_k, const double* E_k,
             const double* Bx_k, const double* By_k, double* rho_k_new, double* rho_ux_k_new, double* rho_uy_k_new,
             double* E_k_new, double* Bx_k_new, double* By_k_new, const double* d_rho_k_dt_old,
             const double* d_rho_k_dt_new, const double* d_rho_ux_k_dt_old, const double* d_rho_ux_k_dt_new,
             const double* d_rho_uy_k_dt_old, const double* d_rho_uy_k_dt_new, const double* d_E_k_dt_old,
             const double* d_E_k_dt_new, const double* d_Bx_k_dt_old, const double* d_Bx_k_dt_new,
             const double* d_By_k_dt_old, const double* d_By_k_dt_new) {
  (void)time;
  std::lock_guard<std::mutex> lk(g_com_mu);
  if (!com_dims(Nx, Ny, Nh, pi)) return;
  const double* in[6] = {rho_k, rho_ux_k, rho_uy_k, E_k, Bx_k, By_k};
  double* out[6] = {rho_k_new, rho_ux_k_new, rho_uy_k_new, E_k_new, Bx_k_new, By_k_new};
  const double* old[6] = {d_rho_k_dt_old, d_rho_ux_k_dt_old, d_rho_uy_k_dt_old,
                          d_E_k_dt_old,   d_Bx_k_dt_old,     d_By_k_dt_old};
  const double* nw[6] = {d_rho_k_dt_new, d_rho_ux_k_dt_new, d_rho_uy_k_dt_new,
                         d_E_k_dt_new,   d_Bx_k_dt_new,     d_By_k_dt_new};
  for (int f = 0; f < 6; ++f)
    if (!in[f] || !out[f] || !old[f] || !nw[f]) {
      set_error(TARA_ERR_ARGS, "null array argument");
      return;
    }
  tara_com2d* h = com_ctx(*Nx, *Ny, *pi);
  if (!h) return;
  if (cudaSetDevice(h->dev) != cudaSuccess) {
    set_error(TARA_ERR_CUDA, "cudaSetDevice failed");
    return;
  }
  for (int f = 0; f < 6; ++f) {
    if (com_copy_in(h, h->st + f * h->fs, in[f]) || com_copy_in(h, h->hist + f * h->fs, old[f]) ||
        com_copy_in(h, h->dnew + f * h->fs, nw[f]))
      return;
  }
  const size_t n = 6 * h->fs;  // padding columns are zero in every input
  k_ab2_dense<<<kElemBlocks, kElemThreads, 0, h->stream>>>(h->st, h->st, h->hist, h->dnew, n, h->cfg.dt);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    cuda_fail(e, "k_ab2_dense");
    return;
  }
  for (int f = 0; f < 6; ++f)
    if (com_copy_out(h, out[f], h->st + f * h->fs)) return;
  e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) {
    cuda_fail(e, "ab2com");
    return;
  }
  set_ok();
}

}  // extern "C"

namespace tara {
int release_dropins_com() {
  std::lock_guard<std::mutex> lk(g_com_mu);
  int rc = TARA_OK;
  for (auto& kv : g_com_ctx) {
    const int r = tara_com2d_destroy(kv.second);
    if (r != TARA_OK && rc == TARA_OK) rc = r;
  }
  g_com_ctx.clear();
  return rc;
}
}  // namespace tara
