// Lagrangian passive particles of the plain serial driver tara2dHydSer
// (src/main2csh.f95:93-96, 187-273): after every vorticity step the driver
// forms u_x = i ky psi, u_y = -i kx psi with psi = omega/(kx^2+ky^2) and its own
// wavenumbers kx = 2 pi (i-1)/Lx (true pi, ini box; :128-155), transforms them to
// the grid (c2r, divided by Nx*Ny; :157-172), interpolates them bilinearly at
// every particle (:187-255) and moves the particle one Euler step with a
// periodic wrap into (0, L] (:257-271).
//
// Defined behaviour where the reference reads outside its arrays: its branches
// for the last cell column or row (m = Nx or n = Ny) read ux(Nx+1, n),
// ux(m, Ny+1) -- past the array end, or the next column in memory -- where the
// periodic neighbour ux(1, n), ux(m, 1) is meant; here the neighbour wraps
// periodically, with the far cell edge at Lx (Ly) as in those branches.
#include <cmath>
#include <vector>

#include "internal.h"

struct tara_particles {
  tara2d* h = nullptr;
  int np = 0;
  double lx = 0, ly = 0;
  double *xp = nullptr, *yp = nullptr;  // device positions
  double2* spec = nullptr;              // 2 spectra (u_x, u_y)
  double* real = nullptr;               // 2 real fields, row pitch rpitch
  double* k = nullptr;                  // driver wavenumbers kx[nh], ky[ny]
  int rpitch = 0;
};

namespace tara {
namespace {

// u_x, u_y spectra with the plain driver's psi (src/main2csh.f95:128-155)
__global__ void k_driver_velocity(const double2* __restrict__ w, const double* __restrict__ kx,
                                  const double* __restrict__ ky, int nh, int ny, int pitch,
                                  double2* __restrict__ out) {
  const size_t total = (size_t)ny * nh, fsz = (size_t)ny * pitch;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const int y = (int)(t / nh), x = (int)(t % nh);
    const size_t q = (size_t)y * pitch + x;
    double2 a = make_double2(0.0, 0.0), b = a;
    if (x != 0 || y != 0) {
      const double k2 = kx[x] * kx[x] + ky[y] * ky[y];
      const double2 v = w[q];
      const double pr = v.x / k2, pim = v.y / k2;
      a = make_double2(-ky[y] * pim, ky[y] * pr);
      b = make_double2(kx[x] * pim, -(kx[x] * pr));
    }
    out[q] = a;
    out[fsz + q] = b;
  }
}

// One Euler step of every particle (src/main2csh.f95:187-271), defined
// periodic neighbours.  u fields are unnormalised c2r outputs (divided by nn).
__global__ void k_particles_step(const double* __restrict__ ur, size_t rf, int rp, int nx, int ny, double lx,
                                 double ly, double nn, double dt, int np, double* __restrict__ xp,
                                 double* __restrict__ yp) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  const double dx = lx / (double)nx, dy = ly / (double)ny;
  const double h = 1.0 / (dx * dy);
  double x = xp[i], y = yp[i];
  int m = (int)(x / dx), n = (int)(y / dy);  // aint(xp/dx), 0-based
  if (m > nx - 1) m = nx - 1;                // x = Lx lies in the last cell
  if (n > ny - 1) n = ny - 1;
  const int m1 = m + 1 < nx ? m + 1 : 0, n1 = n + 1 < ny ? n + 1 : 0;
  const double xm = (double)m * dx, xm1 = m + 1 < nx ? (double)(m + 1) * dx : lx;
  const double yn = (double)n * dy, yn1 = n + 1 < ny ? (double)(n + 1) * dy : ly;
  double v[2];
  for (int c = 0; c < 2; ++c) {
    const double* u = ur + c * rf;
    const double u00 = u[(size_t)n * rp + m] / nn, u10 = u[(size_t)n * rp + m1] / nn;
    const double u01 = u[(size_t)n1 * rp + m] / nn, u11 = u[(size_t)n1 * rp + m1] / nn;
    v[c] = u00 * (xm1 - x) * (yn1 - y) * h + u10 * (x - xm) * (yn1 - y) * h +
           u01 * (xm1 - x) * (y - yn) * h + u11 * (x - xm) * (y - yn) * h;
  }
  x = x + v[0] * dt;
  y = y + v[1] * dt;
  x = x - (double)(int)(x / lx) * lx;  // xp - int(xp/Lx)*Lx
  if (x <= 0.0) x = x + lx;
  y = y - (double)(int)(y / ly) * ly;
  if (y <= 0.0) y = y + ly;
  xp[i] = x;
  yp[i] = y;
}

}  // namespace
}  // namespace tara

using namespace tara;

extern "C" {

int tara_particles_destroy(tara_particles* p) {
  if (!p) return set_ok();
  cudaSetDevice(p->h->dev);
  cudaStreamSynchronize(p->h->stream);
  cudaFree(p->xp);
  cudaFree(p->yp);
  cudaFree(p->spec);
  cudaFree(p->real);
  cudaFree(p->k);
  delete p;
  return set_ok();
}

int tara_particles_create(tara2d* h, double kpi, double lx, double ly, int np, const double* xp,
                          const double* yp, tara_particles** out) {
  if (!h || !out || np < 1 || !xp || !yp || !(kpi > 0) || !(lx > 0) || !(ly > 0))
    return set_error(TARA_ERR_ARGS, "bad particle arguments");
  *out = nullptr;
  TARA_CK(cudaSetDevice(h->dev));
  tara_particles* p = new tara_particles();
  p->h = h;
  p->np = np;
  p->lx = lx;
  p->ly = ly;
  p->rpitch = round_up(h->nx, 8);
  const size_t fsz = (size_t)h->ny * h->pitch, rfs = (size_t)h->ny * p->rpitch;
  if (cudaMalloc(&p->xp, np * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&p->yp, np * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&p->spec, 2 * fsz * sizeof(double2)) != cudaSuccess ||
      cudaMalloc(&p->real, 2 * rfs * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&p->k, (h->nh + h->ny) * sizeof(double)) != cudaSuccess) {
    tara_particles_destroy(p);
    return set_error(TARA_ERR_NOMEM, "cudaMalloc in tara_particles_create");
  }
  std::vector<double> kx(h->nh), ky(h->ny);
  std::vector<int> i0(h->ny);
  make_wavenumbers(h->nx, h->ny, kpi, lx, ly, kx.data(), ky.data(), i0.data());
  const void *tx, *ty;
  int rc = twiddles64(h, &tx, &ty);
  if (!rc && (cudaMemcpy(p->k, kx.data(), h->nh * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
              cudaMemcpy(p->k + h->nh, ky.data(), h->ny * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
              cudaMemcpy(p->xp, xp, np * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
              cudaMemcpy(p->yp, yp, np * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess))
    rc = set_error(TARA_ERR_CUDA, "particle upload");
  if (rc) {
    const ErrorState saved = save_error();
    tara_particles_destroy(p);
    restore_error(saved);
    return rc;
  }
  *out = p;
  return set_ok();
}

// Moves every particle one Euler step of length dt with the velocity of run 0's
// current state (enqueued on the solver's stream).
int tara_particles_advance(tara_particles* p, double dt) {
  if (!p) return set_error(TARA_ERR_ARGS, "null handle");
  tara2d* h = p->h;
  TARA_CK(cudaSetDevice(h->dev));
  const void *tx, *ty;
  int rc;
  if ((rc = twiddles64(h, &tx, &ty))) return rc;
  const size_t fsz = (size_t)h->ny * h->pitch, rfs = (size_t)h->ny * p->rpitch;
  k_driver_velocity<<<152 * 2, 256, 0, h->stream>>>(h->w0, p->k, p->k + h->nh, h->nh, h->ny, h->pitch, p->spec);
  TARA_CK(cudaGetLastError());
  if ((rc = Launch2D<double>::col_fft(h->ny, h->nh, h->pitch, p->spec, p->spec, true, ty, h->stream, 2, fsz)))
    return rc;
  if ((rc = Launch2D<double>::row_c2r(h->nx, h->ny, h->pitch, p->rpitch, p->spec, p->real, tx, h->stream, 2, fsz,
                                      rfs)))
    return rc;
  const double nn = (double)h->nx * (double)h->ny;
  k_particles_step<<<(p->np + 127) / 128, 128, 0, h->stream>>>(p->real, rfs, p->rpitch, h->nx, h->ny, p->lx, p->ly,
                                                               nn, dt, p->np, p->xp, p->yp);
  TARA_CK(cudaGetLastError());
  return set_ok();
}

int tara_particles_get(tara_particles* p, double* xp, double* yp) {
  if (!p || !xp || !yp) return set_error(TARA_ERR_ARGS, "null argument");
  TARA_CK(cudaSetDevice(p->h->dev));
  TARA_CK(cudaMemcpyAsync(xp, p->xp, p->np * sizeof(double), cudaMemcpyDeviceToHost, p->h->stream));
  TARA_CK(cudaMemcpyAsync(yp, p->yp, p->np * sizeof(double), cudaMemcpyDeviceToHost, p->h->stream));
  TARA_CK(cudaStreamSynchronize(p->h->stream));
  return set_ok();
}

// Minimal-standard multiplicative LCG (Park & Miller 1988: a = 16807,
// m = 2^31 - 1), the generator GNU Fortran documents for its RAND intrinsic,
// returning the REAL(4) value (state-1) truncated to 24 significant bits * 2^-31.
float tara_park_miller_rand(uint64_t* state) {
  *state = (16807ull * *state) % 2147483647ull;
  const uint32_t j = (uint32_t)*state - 1u;
  const uint32_t mask = ~0u << (32 - 24 + 1);
  return (float)(j & mask) * 0x1.p-31f;
}

}  // extern "C"
