// 3D compressible MHD: device-resident solver (tara3d_*) and the Fortran
// drop-ins derive3com_ / ab3com_.
//
// One RHS evaluation (src/derive3com.f95:6-1047) on the GPU:
//   c2r of the 8 state spectra (z pass, y pass, x rows)            8 transforms
//   k3_prim: u, P, B^2, momentum and induction fluxes in real space
//   r2c of u (3) and the 9 distinct fluxes                         12 transforms
//   [drop-in only] div u and curl B (4 c2r), energy fluxes and
//   E_Visc (4 r2c) for dE/dt                                       8 transforms
//   k3_assemble: i k . flux, viscous/resistive terms, the |k| >= (Nx+Ny+Nz)/9
//   sphere, and the AB2 update (E frozen, as ab3com leaves it) fused in.
// The reference runs 42 transforms per RHS; the forcing it transforms is never
// used (:201-217 vs :1009-1040), and six of its 19 product fields are the same
// expressions (Mom_x_2 = Mom_y_1, Mag_x_1 = Mag_y_1, Mag_x_2 = Mag_z_1,
// Mag_y_2 = Mag_z_2) or the same up to rounding (Mom_x_3 / Mom_z_1,
// Mom_y_3 / Mom_z_2), so each distinct field is transformed once.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "internal.h"
#include "kernels3d.cuh"

namespace tara {

// Largest 3D length: 512^3 holds about 85 GB of FP64 state and work fields.
constexpr int kMax3D = 512;

// ---------------------------------------------------------------------------
// pointwise kernels
// ---------------------------------------------------------------------------
__global__ void k3_prim(const double* __restrict__ rl, double* __restrict__ pr, Grid3D g,
                        Mhd3DParams p) {
  const size_t total = (size_t)g.nz * g.ny * g.nx;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const size_t row = t / g.nx;
    const size_t r = row * g.rpitch + (t % g.nx);
    const double rho = rl[S_RHO * g.rfs + r] * p.inv_n;
    const double rux = rl[S_RUX * g.rfs + r] * p.inv_n;
    const double ruy = rl[S_RUY * g.rfs + r] * p.inv_n;
    const double ruz = rl[S_RUZ * g.rfs + r] * p.inv_n;
    const double bx = rl[S_BX * g.rfs + r] * p.inv_n;
    const double by = rl[S_BY * g.rfs + r] * p.inv_n;
    const double bz = rl[S_BZ * g.rfs + r] * p.inv_n;
    const double ux = rux / rho, uy = ruy / rho, uz = ruz / rho;
    const double b2 = bx * bx + by * by + bz * bz;
    const double P = p.cs2 * rho;
    const double iso = P + b2 / 2.0;
    pr[P_UX * g.rfs + r] = ux;
    pr[P_UY * g.rfs + r] = uy;
    pr[P_UZ * g.rfs + r] = uz;
    pr[P_MXX * g.rfs + r] = rux * ux + iso - bx * bx;
    pr[P_MXY * g.rfs + r] = rux * uy - bx * by;
    pr[P_MXZ * g.rfs + r] = rux * uz - bx * bz;
    pr[P_MYY * g.rfs + r] = ruy * uy + iso - by * by;
    pr[P_MYZ * g.rfs + r] = ruy * uz - by * bz;
    pr[P_MZZ * g.rfs + r] = ruz * uz + iso - bz * bz;
    pr[P_G1 * g.rfs + r] = ux * by - uy * bx;
    pr[P_G2 * g.rfs + r] = ux * bz - uz * bx;
    pr[P_G3 * g.rfs + r] = uy * bz - uz * by;
  }
}

__global__ void k3_energy(const double* __restrict__ rl, double* __restrict__ pr,
                          const double* __restrict__ dr, Grid3D g, Mhd3DParams p) {
  const size_t total = (size_t)g.nz * g.ny * g.nx;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const size_t r = (t / g.nx) * g.rpitch + (t % g.nx);
    const double rho = rl[S_RHO * g.rfs + r] * p.inv_n;
    const double E = rl[S_E * g.rfs + r] * p.inv_n;
    const double bx = rl[S_BX * g.rfs + r] * p.inv_n;
    const double by = rl[S_BY * g.rfs + r] * p.inv_n;
    const double bz = rl[S_BZ * g.rfs + r] * p.inv_n;
    const double ux = pr[P_UX * g.rfs + r], uy = pr[P_UY * g.rfs + r], uz = pr[P_UZ * g.rfs + r];
    const double dv = dr[D_DIV * g.rfs + r] * p.inv_n;
    const double cx = dr[D_CX * g.rfs + r] * p.inv_n;
    const double cy = dr[D_CY * g.rfs + r] * p.inv_n;
    const double cz = dr[D_CZ * g.rfs + r] * p.inv_n;
    const double b2 = bx * bx + by * by + bz * bz;
    const double h = E + p.cs2 * rho + b2 / 2.0;
    pr[P_ENX * g.rfs + r] =
        h * ux - ux * bx * bx - uy * bx * by - uz * bx * bz - p.eta * (by * cz + bz * cy);
    pr[P_ENY * g.rfs + r] =
        h * uy - ux * bx * by - uy * by * by - uz * by * bz + p.eta * (bx * cz - bz * cx);
    pr[P_ENZ * g.rfs + r] =
        h * uz - ux * bz * bx - uy * bz * by - uz * bz * bz + p.eta * (bx * cy + by * cx);
    pr[P_EVISC * g.rfs + r] = dv * dv;
  }
}

// The Orszag-Tang-type initial state on the grid: rl holds the unnormalised c2r
// of the u and B spectra in the rho u and B slots; normalise them (rho = 1, so
// rho u = u) and fill rho = 1 and E = 1 + |u|^2/2 + |B|^2/2.
__global__ void k3_ot_fill(double* __restrict__ rl, Grid3D g, double inv_n) {
  const size_t total = (size_t)g.nz * g.ny * g.nx;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const size_t r = (t / g.nx) * g.rpitch + (t % g.nx);
    const double ux = rl[S_RUX * g.rfs + r] * inv_n, uy = rl[S_RUY * g.rfs + r] * inv_n,
                 uz = rl[S_RUZ * g.rfs + r] * inv_n;
    const double bx = rl[S_BX * g.rfs + r] * inv_n, by = rl[S_BY * g.rfs + r] * inv_n,
                 bz = rl[S_BZ * g.rfs + r] * inv_n;
    rl[S_RHO * g.rfs + r] = 1.0;
    rl[S_RUX * g.rfs + r] = ux;
    rl[S_RUY * g.rfs + r] = uy;
    rl[S_RUZ * g.rfs + r] = uz;
    rl[S_BX * g.rfs + r] = bx;
    rl[S_BY * g.rfs + r] = by;
    rl[S_BZ * g.rfs + r] = bz;
    const double u2 = __dadd_rn(__dadd_rn(__dmul_rn(ux, ux), __dmul_rn(uy, uy)), __dmul_rn(uz, uz));
    const double b2 = __dadd_rn(__dadd_rn(__dmul_rn(bx, bx), __dmul_rn(by, by)), __dmul_rn(bz, bz));
    rl[S_E * g.rfs + r] = __dadd_rn(__dadd_rn(1.0, __dmul_rn(0.5, u2)), __dmul_rn(0.5, b2));
  }
}

__device__ __forceinline__ double2 ik(double k, double2 f) { return make_double2(-k * f.y, k * f.x); }

__global__ void k3_derivs(const double2* __restrict__ st, const double2* __restrict__ pk,
                          double2* __restrict__ dk, Grid3D g) {
  const size_t total = (size_t)g.nz * g.ny * g.nh;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const int x = (int)(t % g.nh);
    const size_t row = t / g.nh;
    const int y = (int)(row % g.ny), z = (int)(row / g.ny);
    const size_t q = row * g.pitch + x;
    const double kx = g.kx[x], ky = g.ky[y], kz = g.kz[z];
    const double2 a = ik(kx, pk[P_UX * g.fs + q]), b = ik(ky, pk[P_UY * g.fs + q]),
                  c = ik(kz, pk[P_UZ * g.fs + q]);
    dk[D_DIV * g.fs + q] = make_double2(a.x + b.x + c.x, a.y + b.y + c.y);
    const double2 bx = st[S_BX * g.fs + q], by = st[S_BY * g.fs + q], bz = st[S_BZ * g.fs + q];
    const double2 bzy = ik(ky, bz), byz = ik(kz, by), bzx = ik(kx, bz), bxz = ik(kz, bx),
                  byx = ik(kx, by), bxy = ik(ky, bx);
    dk[D_CX * g.fs + q] = make_double2(bzy.x - byz.x, bzy.y - byz.y);
    dk[D_CY * g.fs + q] = make_double2(bzx.x - bxz.x, bzx.y - bxz.y);
    dk[D_CZ * g.fs + q] = make_double2(byx.x - bxy.x, byx.y - bxy.y);
  }
}

__global__ void k3_assemble(double2* __restrict__ st, const double2* __restrict__ pk,
                            double2* __restrict__ dout, double2* __restrict__ hist, Grid3D g,
                            Mhd3DParams p, int mode, int with_energy, unsigned int* flag) {
  const size_t total = (size_t)g.nz * g.ny * g.nh;
  bool bad = false;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const int x = (int)(t % g.nh);
    const size_t row = t / g.nh;
    const int y = (int)(row % g.ny), z = (int)(row / g.ny);
    const size_t q = row * g.pitch + x;
    double2 d[S_N];
    if (x >= g.i0[row]) {
      for (int f = 0; f < S_N; ++f) d[f] = make_double2(0.0, 0.0);
    } else {
      const double kx = g.kx[x], ky = g.ky[y], kz = g.kz[z];
      const double kx2 = kx * kx, ky2 = ky * ky, kz2 = kz * kz;
#define PK(i) pk[(size_t)(i) * g.fs + q]
#define ST(i) st[(size_t)(i) * g.fs + q]
      // -(i kx a + i ky b + i kz c)
      auto divneg = [&](double2 a, double2 b, double2 c) {
        const double2 u = ik(kx, a), v = ik(ky, b), w = ik(kz, c);
        return make_double2(-(u.x + v.x + w.x), -(u.y + v.y + w.y));
      };
      // k^2 f / 450 (faithful) or coefficient * k^2 f (defined)
      auto diss = [&](double2 f, double coef) {
        const double2 s = make_double2(kx2 * f.x + ky2 * f.x + kz2 * f.x,
                                       kx2 * f.y + ky2 * f.y + kz2 * f.y);
        return p.defined ? make_double2(coef * s.x, coef * s.y)
                         : make_double2(s.x / 450.0, s.y / 450.0);
      };
      d[S_RHO] = divneg(ST(S_RUX), ST(S_RUY), ST(S_RUZ));
      double2 m = divneg(PK(P_MXX), PK(P_MXY), PK(P_MXZ)), v = diss(PK(P_UX), p.nu_u);
      d[S_RUX] = make_double2(m.x - v.x, m.y - v.y);
      m = divneg(PK(P_MXY), PK(P_MYY), PK(P_MYZ));
      v = diss(PK(P_UY), p.nu_u);
      d[S_RUY] = make_double2(m.x - v.x, m.y - v.y);
      m = divneg(PK(P_MXZ), PK(P_MYZ), PK(P_MZZ));
      v = diss(PK(P_UZ), p.nu_u);
      d[S_RUZ] = make_double2(m.x - v.x, m.y - v.y);
      if (with_energy) {
        m = divneg(PK(P_ENX), PK(P_ENY), PK(P_ENZ));
        const double2 ev = PK(P_EVISC);
        d[S_E] = make_double2(m.x + p.mu * ev.x, m.y + p.mu * ev.y);
      } else {
        d[S_E] = make_double2(0.0, 0.0);
      }
      // dBx = +(i ky G1 + i kz G2), dBy = -(i kx G1 - i kz G3), dBz = -(i kx G2 + i ky G3)
      const double2 g1y = ik(ky, PK(P_G1)), g2z = ik(kz, PK(P_G2)), g1x = ik(kx, PK(P_G1)),
                    g3z = ik(kz, PK(P_G3)), g2x = ik(kx, PK(P_G2)), g3y = ik(ky, PK(P_G3));
      v = diss(ST(S_BX), p.eta_b);
      d[S_BX] = make_double2((g1y.x + g2z.x) - v.x, (g1y.y + g2z.y) - v.y);
      v = diss(ST(S_BY), p.eta_b);
      d[S_BY] = make_double2(-(g1x.x - g3z.x) - v.x, -(g1x.y - g3z.y) - v.y);
      v = diss(ST(S_BZ), p.eta_b);
      d[S_BZ] = make_double2(-(g2x.x + g3y.x) - v.x, -(g2x.y + g3y.y) - v.y);
#undef PK
#undef ST
    }
    for (int f = 0; f < S_N; ++f) bad |= !(isfinite(d[f].x) && isfinite(d[f].y));
    if (mode == MODE_DERIVE) {
      for (int f = 0; f < S_N; ++f) dout[(size_t)f * g.fs + q] = d[f];
    } else {  // AB2, E frozen
      for (int f = 0; f < S_N; ++f) {
        const size_t o = (size_t)f * g.fs + q;
        if (f != S_E) {
          const double2 s = st[o], h = hist[o];
          st[o] = make_double2(s.x + ((3.0 / 2.0) * d[f].x - (1.0 / 2.0) * h.x) * p.dt,
                               s.y + ((3.0 / 2.0) * d[f].y - (1.0 / 2.0) * h.y) * p.dt);
        }
        hist[o] = d[f];
      }
    }
  }
  if (bad) atomicOr(flag, 1u);
}

// Grid sums of the reference's 3D diagnostics (src/main3com.f95:1024-1043):
// part[4*b + 0..3] = sum rho, sum |u|^2, sum E, sum |B|^2 over this block's points.
__global__ void k3_diag_partial(const double* __restrict__ rl, const double* __restrict__ pr,
                                Grid3D g, double inv_n, double* __restrict__ part) {
  const size_t total = (size_t)g.nz * g.ny * g.nx;
  double a[4] = {0.0, 0.0, 0.0, 0.0};
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const size_t r = (t / g.nx) * g.rpitch + (t % g.nx);
    const double ux = pr[P_UX * g.rfs + r], uy = pr[P_UY * g.rfs + r], uz = pr[P_UZ * g.rfs + r];
    const double bx = rl[S_BX * g.rfs + r] * inv_n, by = rl[S_BY * g.rfs + r] * inv_n,
                 bz = rl[S_BZ * g.rfs + r] * inv_n;
    a[0] += rl[S_RHO * g.rfs + r] * inv_n;
    a[1] += ux * ux + uy * uy + uz * uz;
    a[2] += rl[S_E * g.rfs + r] * inv_n;
    a[3] += bx * bx + by * by + bz * bz;
  }
  __shared__ double sh[4][8];
  for (int k = 0; k < 4; ++k) {
    for (int o = 16; o > 0; o >>= 1) a[k] += __shfl_down_sync(0xffffffffu, a[k], o);
    if ((threadIdx.x & 31) == 0) sh[k][threadIdx.x >> 5] = a[k];
  }
  __syncthreads();
  if (threadIdx.x < 4) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += sh[threadIdx.x][w];
    part[4 * blockIdx.x + threadIdx.x] = s;
  }
}

// dense AB2 of ab3com on 8 fields: out = s + (3/2 dn - 1/2 do) dt, E copied
__global__ void k3_ab2_dense(const double2* __restrict__ s, double2* __restrict__ out,
                             const double2* __restrict__ dold, const double2* __restrict__ dnew,
                             size_t fs, double dt) {
  const size_t total = fs * S_N;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const int f = (int)(i / fs);
    const double2 a = s[i];
    if (f == S_E) {
      out[i] = a;
    } else {
      const double2 b = dold[i], c = dnew[i];
      out[i] = make_double2(a.x + ((3.0 / 2.0) * c.x - (1.0 / 2.0) * b.x) * dt,
                            a.y + ((3.0 / 2.0) * c.y - (1.0 / 2.0) * b.y) * dt);
    }
  }
}

// ---------------------------------------------------------------------------
// transform launchers (FP64)
// ---------------------------------------------------------------------------
template <typename K>
static cudaError_t allow_smem3(K kernel, int bytes) {
  if (bytes <= 48 * 1024) return cudaSuccess;
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

#define TARA_SWITCH_N3(n, CALL)                            \
  switch (n) {                                             \
    case 16: { constexpr int N = 16; CALL; } break;        \
    case 32: { constexpr int N = 32; CALL; } break;        \
    case 64: { constexpr int N = 64; CALL; } break;        \
    case 128: { constexpr int N = 128; CALL; } break;      \
    case 256: { constexpr int N = 256; CALL; } break;      \
    case 512: { constexpr int N = 512; CALL; } break;      \
    default: return set_error(TARA_ERR_ARGS, "3D sizes must be powers of two in [16, 512]"); \
  }

template <int N, bool INV>
static int lines_n(const double2* in, double2* out, int nh, size_t ps, size_t os, int n_outer,
                   size_t fs_in, size_t fs_out, int nf, const double2* tw, cudaStream_t s) {
  typedef ColCfg<double, N> CF;
  static cudaError_t attr = allow_smem3(k_lines<double, N, INV>, CF::SMEM_C);
  TARA_CK(attr);
  const dim3 grid((nh + CF::TCC - 1) / CF::TCC, n_outer, nf);
  k_lines<double, N, INV><<<grid, CF::THREADS_C, CF::SMEM_C, s>>>(in, out, nh, ps, os, fs_in,
                                                                  fs_out, tw);
  TARA_CK(cudaGetLastError());
  return TARA_OK;
}

static int lines(int n, bool inv, const double2* in, double2* out, int nh, size_t ps, size_t os,
                 int n_outer, size_t fs_in, size_t fs_out, int nf, const void* tw,
                 cudaStream_t s) {
  const double2* t = (const double2*)tw;
  if (inv) {
    TARA_SWITCH_N3(n, return (lines_n<N, true>(in, out, nh, ps, os, n_outer, fs_in, fs_out, nf, t, s)));
  } else {
    TARA_SWITCH_N3(n, return (lines_n<N, false>(in, out, nh, ps, os, n_outer, fs_in, fs_out, nf, t, s)));
  }
  return TARA_OK;
}

template <int N>
static int rows_c2r_n(const double2* in, double* out, int rows, int pitch, int rpitch, size_t fsi,
                      size_t fso, int nf, const double2* tw, cudaStream_t s) {
  typedef RowCfg<double, N> RC;
  static cudaError_t attr = allow_smem3(k_rows_c2r<double, N>, RC::SMEM);
  TARA_CK(attr);
  const int per = 2 * 4 * RC::RP;
  k_rows_c2r<double, N><<<dim3((rows + per - 1) / per, nf), RC::THREADS, RC::SMEM, s>>>(
      in, out, rows, pitch, rpitch, fsi, fso, tw);
  TARA_CK(cudaGetLastError());
  return TARA_OK;
}

template <int N>
static int rows_r2c_n(const double* in, double2* out, int rows, int rpitch, int pitch, size_t fsi,
                      size_t fso, int nf, const double2* tw, cudaStream_t s) {
  typedef RowCfg<double, N> RC;
  static cudaError_t attr = allow_smem3(k_rows_r2c<double, N>, RC::SMEM);
  TARA_CK(attr);
  const int per = 2 * 4 * RC::RP;
  k_rows_r2c<double, N><<<dim3((rows + per - 1) / per, nf), RC::THREADS, RC::SMEM, s>>>(
      in, out, rows, rpitch, pitch, fsi, fso, tw);
  TARA_CK(cudaGetLastError());
  return TARA_OK;
}

}  // namespace tara

using namespace tara;

// Fortran common block /comm/ of the reference's 3D code
// (common/comm/iret,thread_num,time_max,Lx,Ly,Lz,dx,dy,dz,spheat,mu,ms,CS,mu_0,eta,dt,kf,
// src/derive3com.f95:62, src/ab3com.f95:29).  A Fortran caller that links
// libtara supplies it; this weak definition (the reference's main3com values for
// a 2*pi box) lets the library load on its own.
extern "C" __attribute__((weak)) TaraMhdCommon comm_ = {
    0, 1, 1.0, 2.0 * 3.14159265358979323846, 2.0 * 3.14159265358979323846,
    2.0 * 3.14159265358979323846, 0.0, 0.0, 0.0, 1.0, 0.01, 1.0, 10.0, 1.0, 0.005, 1e-3, 1.0};

struct tara3d {
  tara3d_config cfg;
  int dev = 0, nx = 0, ny = 0, nz = 0, nh = 0, pitch = 0, rpitch = 0;
  size_t fs = 0, rfs = 0;
  cudaStream_t stream = nullptr;
  double2 *st = nullptr, *hist = nullptr, *dout = nullptr, *cw = nullptr, *pk = nullptr;
  double *rl = nullptr, *dr = nullptr, *pr = nullptr;
  double *kx = nullptr, *ky = nullptr, *kz = nullptr;
  int* i0 = nullptr;
  void *twx = nullptr, *twy = nullptr, *twz = nullptr;
  unsigned int* flag = nullptr;
  Grid3D g;
  Mhd3DParams p;
};

namespace {

int refresh3(tara3d* h) {
  const tara3d_config& c = h->cfg;
  std::vector<double> kx(h->nh), ky(h->ny), kz(h->nz);
  std::vector<int> i0((size_t)h->ny * h->nz);
  // kx = 2.0d0*pi*dfloat(i-1)/Lx; ky, kz with (j-1)-Ny above Ny/2 (src/derive3com.f95:213-215)
  for (int i = 0; i < h->nh; ++i) kx[i] = 2.0 * c.kpi * (double)i / c.lx;
  for (int j = 0; j < h->ny; ++j)
    ky[j] = j < h->ny / 2 ? 2.0 * c.kpi * (double)j / c.ly : 2.0 * c.kpi * (double)(j - h->ny) / c.ly;
  for (int k = 0; k < h->nz; ++k)
    kz[k] = k < h->nz / 2 ? 2.0 * c.kpi * (double)k / c.lz : 2.0 * c.kpi * (double)(k - h->nz) / c.lz;
  // dsqrt(kx*kx+ky*ky+kz*kz) .ge. (dfloat(Nx+Ny+Nz)/3.0)/3.0 (src/derive3com.f95:796)
  const double cut = ((double)(h->nx + h->ny + h->nz) / 3.0) / 3.0 + 0;
  for (int k = 0; k < h->nz; ++k)
    for (int j = 0; j < h->ny; ++j) {
      int first = h->nh;
      for (int i = h->nh - 1; i >= 0; --i) {
        if (std::sqrt(kx[i] * kx[i] + ky[j] * ky[j] + kz[k] * kz[k]) >= cut)
          first = i;
        else
          break;
      }
      i0[(size_t)k * h->ny + j] = first;
    }
  TARA_CK(cudaMemcpyAsync(h->kx, kx.data(), kx.size() * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  TARA_CK(cudaMemcpyAsync(h->ky, ky.data(), ky.size() * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  TARA_CK(cudaMemcpyAsync(h->kz, kz.data(), kz.size() * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  TARA_CK(cudaMemcpyAsync(h->i0, i0.data(), i0.size() * sizeof(int), cudaMemcpyHostToDevice, h->stream));
  TARA_CK(cudaStreamSynchronize(h->stream));
  h->p.inv_n = 1.0 / ((double)h->nx * (double)h->ny * (double)h->nz);
  h->p.cs2 = c.cs * c.cs;
  h->p.eta = c.eta;
  h->p.mu = c.mu;
  h->p.defined = c.defined;
  h->p.nu_u = c.nu_u;
  h->p.eta_b = c.eta_b;
  h->p.dt = c.dt;
  return TARA_OK;
}

// c2r of nf spectral fields `in` (left untouched) into real fields `out`,
// through the workspace cw.
int c2r3(tara3d* h, const double2* in, double* out, int nf) {
  int rc;
  const size_t pitch = h->pitch, ny = h->ny;
  if ((rc = lines(h->nz, true, in, h->cw, h->nh, ny * pitch, pitch, h->ny, h->fs, h->fs, nf, h->twz,
                  h->stream)))
    return rc;
  if ((rc = lines(h->ny, true, h->cw, h->cw, h->nh, pitch, ny * pitch, h->nz, h->fs, h->fs, nf,
                  h->twy, h->stream)))
    return rc;
  TARA_SWITCH_N3(h->nx, return rows_c2r_n<N>(h->cw, out, h->ny * h->nz, h->pitch, h->rpitch, h->fs,
                                             h->rfs, nf, (const double2*)h->twx, h->stream));
  return TARA_OK;
}

// r2c of nf real fields into spectral fields `out`.
int r2c3(tara3d* h, const double* in, double2* out, int nf) {
  int rc;
  const size_t pitch = h->pitch, ny = h->ny;
  switch (h->nx) {
    case 16: rc = rows_r2c_n<16>(in, out, h->ny * h->nz, h->rpitch, h->pitch, h->rfs, h->fs, nf, (const double2*)h->twx, h->stream); break;
    case 32: rc = rows_r2c_n<32>(in, out, h->ny * h->nz, h->rpitch, h->pitch, h->rfs, h->fs, nf, (const double2*)h->twx, h->stream); break;
    case 64: rc = rows_r2c_n<64>(in, out, h->ny * h->nz, h->rpitch, h->pitch, h->rfs, h->fs, nf, (const double2*)h->twx, h->stream); break;
    case 128: rc = rows_r2c_n<128>(in, out, h->ny * h->nz, h->rpitch, h->pitch, h->rfs, h->fs, nf, (const double2*)h->twx, h->stream); break;
    case 256: rc = rows_r2c_n<256>(in, out, h->ny * h->nz, h->rpitch, h->pitch, h->rfs, h->fs, nf, (const double2*)h->twx, h->stream); break;
    case 512: rc = rows_r2c_n<512>(in, out, h->ny * h->nz, h->rpitch, h->pitch, h->rfs, h->fs, nf, (const double2*)h->twx, h->stream); break;
    default: return set_error(TARA_ERR_ARGS, "3D sizes must be powers of two in [16, 512]");
  }
  if (rc) return rc;
  if ((rc = lines(h->ny, false, out, out, h->nh, pitch, ny * pitch, h->nz, h->fs, h->fs, nf, h->twy,
                  h->stream)))
    return rc;
  return lines(h->nz, false, out, out, h->nh, ny * pitch, pitch, h->ny, h->fs, h->fs, nf, h->twz,
               h->stream);
}

// Spectra of u and B of the Orszag-Tang-type initial state, in the r2c
// convention of the state (unnormalised: F(k) = sum_x f(x) exp(-i k.x)), six
// dense (Nh,Ny,Nz) arrays in the order ux, uy, uz, Bx, By, Bz.
//   u = (-sin y, sin x, 0) + du,  B = (-sin y, sin 2x, 0) + dB  (2 pi box)
// du and dB are random-phase solenoidal fields on the modes 0 < |k| <= kmax
// (integer wavenumbers): for each such mode of the half space and component c,
// phase theta = 2 pi U with U = word 0 of Philox4x32-10 at counter
// (i, j, k, 3 f + c) (f = 0 for u, 1 for B; (i, j, k) the array indices of the
// mode) and key (seed low, seed high), a_c = exp(i theta); then
// a <- a - k (k.a)/|k|^2.  On the kx = 0 plane only the half with ky > 0, or
// ky = 0 and kz > 0, is drawn and the other half is its conjugate, so the field
// is real.  Each perturbation is scaled so that its r.m.s. (sum over the
// components of <f_c^2>) is amp times that of the base field, which is 1 for
// both u and B.
static void ot_spectra(int nx, int ny, int nz, double amp, int kmax, uint64_t seed,
                       std::vector<double2>& out) {
  const int nh = nx / 2 + 1;
  const size_t fs = (size_t)nh * ny * nz;
  const double nn = (double)nx * (double)ny * (double)nz;
  const double two_pi = 2.0 * 3.14159265358979323846;
  out.assign(6 * fs, make_double2(0.0, 0.0));
  const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  auto sgn = [](int j, int n) { return j <= n / 2 ? j : j - n; };
  for (int f = 0; f < 2; ++f) {
    double2* P = out.data() + 3 * f * fs;
    double norm2 = 0.0;
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nh; ++i) {
          const int kxi = i, kyi = sgn(j, ny), kzi = sgn(k, nz);
          const int k2i = kxi * kxi + kyi * kyi + kzi * kzi;
          if (k2i == 0 || k2i > kmax * kmax) continue;
          if (i == 0 && (kyi < 0 || (kyi == 0 && kzi < 0))) continue;  // the conjugate half
          double ar[3], ai[3];
          for (int c = 0; c < 3; ++c) {
            const uint32_t ctr[4] = {(uint32_t)i, (uint32_t)j, (uint32_t)k, (uint32_t)(3 * f + c)};
            uint32_t r[4];
            philox4x32_10(ctr, key, r);
            const double theta = two_pi * ((double)r[0] * (1.0 / 4294967296.0));
            ar[c] = std::cos(theta);
            ai[c] = std::sin(theta);
          }
          const double kv[3] = {(double)kxi, (double)kyi, (double)kzi};
          const double k2 = (double)k2i;
          const double dr = (kv[0] * ar[0] + kv[1] * ar[1] + kv[2] * ar[2]) / k2;
          const double di = (kv[0] * ai[0] + kv[1] * ai[1] + kv[2] * ai[2]) / k2;
          for (int c = 0; c < 3; ++c) {
            const double pr = ar[c] - kv[c] * dr, pi = ai[c] - kv[c] * di;
            P[c * fs + ((size_t)k * ny + j) * nh + i] = make_double2(pr, pi);
            if (i == 0) {
              const int jm = (ny - j) % ny, km = (nz - k) % nz;
              P[c * fs + ((size_t)km * ny + jm) * nh] = make_double2(pr, -pi);
            }
            // the mode and its conjugate at -k both count in the full spectrum
            norm2 += 2.0 * (pr * pr + pi * pi);
          }
        }
    const double s = norm2 > 0.0 ? amp * nn / std::sqrt(norm2) : 0.0;
    for (size_t q = 0; q < 3 * fs; ++q) P[q] = make_double2(P[q].x * s, P[q].y * s);
    // base modes: -sin y at ky = +-1 (kx = 0), sin(m x) at kx = m (m = 1 for u, 2 for B)
    const double h = 0.5 * nn;
    P[0 * fs + (size_t)1 * nh].y += h;         // x component: -sin y, F(0, 1, 0) = +i N/2
    P[0 * fs + (size_t)(ny - 1) * nh].y -= h;  // F(0, -1, 0) = -i N/2
    P[1 * fs + (size_t)(f == 0 ? 1 : 2)].y -= h;  // y component: sin(m x), F(m, 0, 0) = -i N/2
  }
}

constexpr int kPwBlocks = 152 * 4, kPwThreads = 256;

int rhs3(tara3d* h, int mode, int with_energy) {
  int rc;
  if ((rc = c2r3(h, h->st, h->rl, S_N))) return rc;
  k3_prim<<<kPwBlocks, kPwThreads, 0, h->stream>>>(h->rl, h->pr, h->g, h->p);
  TARA_CK(cudaGetLastError());
  if ((rc = r2c3(h, h->pr, h->pk, P_G3 + 1))) return rc;
  if (with_energy) {
    k3_derivs<<<kPwBlocks, kPwThreads, 0, h->stream>>>(h->st, h->pk, h->cw + 4 * h->fs, h->g);
    TARA_CK(cudaGetLastError());
    if ((rc = c2r3(h, h->cw + 4 * h->fs, h->dr, D_N))) return rc;
    k3_energy<<<kPwBlocks, kPwThreads, 0, h->stream>>>(h->rl, h->pr, h->dr, h->g, h->p);
    TARA_CK(cudaGetLastError());
    if ((rc = r2c3(h, h->pr + P_ENX * h->rfs, h->pk + P_ENX * h->fs, 4))) return rc;
  }
  k3_assemble<<<kPwBlocks, kPwThreads, 0, h->stream>>>(h->st, h->pk, h->dout, h->hist, h->g, h->p,
                                                       mode, with_energy, h->flag);
  TARA_CK(cudaGetLastError());
  return TARA_OK;
}

int copy3(tara3d* h, double2* dev, const double* host, cudaMemcpyKind kind, double* host_out) {
  const size_t row = h->nh * sizeof(double2), dp = h->pitch * sizeof(double2);
  const size_t rows = (size_t)h->ny * h->nz;
  if (kind == cudaMemcpyHostToDevice)
    TARA_CK(cudaMemcpy2DAsync(dev, dp, host, row, row, rows, kind, h->stream));
  else
    TARA_CK(cudaMemcpy2DAsync(host_out, row, dev, dp, row, rows, kind, h->stream));
  return TARA_OK;
}

}  // namespace

extern "C" {

void tara3d_default_config(tara3d_config* c, int nx, int ny, int nz) {
  std::memset(c, 0, sizeof(*c));
  c->nx = nx;
  c->ny = ny;
  c->nz = nz;
  c->kpi = 3.14159265358979323846;
  c->lx = c->ly = c->lz = 2.0 * c->kpi;
  c->mu = 0.01;
  c->eta = 0.005;
  c->cs = 10.0;
  c->defined = 0;
  c->nu_u = 0.01;
  c->eta_b = 0.01;
  c->dt = 1e-3;
}

int tara3d_destroy(tara3d* h) {
  if (!h) return set_ok();
  cudaSetDevice(h->dev);
  if (h->stream) cudaStreamSynchronize(h->stream);
  void* ptrs[] = {h->st, h->hist, h->dout, h->cw, h->pk, h->rl, h->dr, h->pr, h->kx, h->ky,
                  h->kz, h->i0, h->twx, h->twy, h->twz, h->flag};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return set_ok();
}

int tara3d_create(const tara3d_config* cfg, tara3d** out) {
  if (!cfg || !out) return set_error(TARA_ERR_ARGS, "null argument");
  *out = nullptr;
  auto ok = [](int n) { return n >= 16 && n <= kMax3D && (n & (n - 1)) == 0; };
  if (!ok(cfg->nx) || !ok(cfg->ny) || !ok(cfg->nz))
    return set_error(TARA_ERR_ARGS, "3D sizes must be powers of two in [16, 512]");
  if (!(cfg->lx > 0 && cfg->ly > 0 && cfg->lz > 0 && cfg->kpi > 0))
    return set_error(TARA_ERR_ARGS, "box lengths and kpi must be positive");
  tara3d* h = new tara3d();
  h->cfg = *cfg;
  h->nx = cfg->nx;
  h->ny = cfg->ny;
  h->nz = cfg->nz;
  h->nh = cfg->nx / 2 + 1;
  h->pitch = round_up(h->nh, 8);
  h->rpitch = round_up(h->nx, 8);
  h->fs = (size_t)h->nz * h->ny * h->pitch;
  h->rfs = (size_t)h->nz * h->ny * h->rpitch;
  int rc;
  auto fail = [&](int code) {  // free the half-built handle, keep the error
    const ErrorState saved = save_error();
    tara3d_destroy(h);
    restore_error(saved);
    return code;
  };
#define CK3(call)                                              \
  do {                                                         \
    cudaError_t e_ = (call);                                   \
    if (e_ != cudaSuccess) return fail(cuda_fail(e_, #call)); \
  } while (0)
  CK3(cudaGetDevice(&h->dev));
  CK3(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
  const size_t sb = h->fs * sizeof(double2), rb = h->rfs * sizeof(double);
  CK3(cudaMalloc(&h->st, S_N * sb));
  CK3(cudaMalloc(&h->hist, S_N * sb));
  CK3(cudaMalloc(&h->dout, S_N * sb));
  CK3(cudaMalloc(&h->cw, S_N * sb));
  CK3(cudaMalloc(&h->pk, P_N * sb));
  CK3(cudaMalloc(&h->rl, S_N * rb));
  CK3(cudaMalloc(&h->dr, D_N * rb));
  CK3(cudaMalloc(&h->pr, P_N * rb));
  CK3(cudaMalloc(&h->kx, h->nh * sizeof(double)));
  CK3(cudaMalloc(&h->ky, h->ny * sizeof(double)));
  CK3(cudaMalloc(&h->kz, h->nz * sizeof(double)));
  CK3(cudaMalloc(&h->i0, (size_t)h->ny * h->nz * sizeof(int)));
  CK3(cudaMalloc(&h->flag, sizeof(unsigned int)));
  CK3(cudaMemsetAsync(h->st, 0, S_N * sb, h->stream));
  CK3(cudaMemsetAsync(h->hist, 0, S_N * sb, h->stream));
  CK3(cudaMemsetAsync(h->dout, 0, S_N * sb, h->stream));
  CK3(cudaMemsetAsync(h->cw, 0, S_N * sb, h->stream));
  CK3(cudaMemsetAsync(h->pk, 0, P_N * sb, h->stream));
  CK3(cudaMemsetAsync(h->flag, 0, sizeof(unsigned int), h->stream));
#undef CK3
  if ((rc = make_twiddles(h->nx, false, &h->twx)) || (rc = make_twiddles(h->ny, false, &h->twy)) ||
      (rc = make_twiddles(h->nz, false, &h->twz)))
    return fail(rc);
  h->g.nx = h->nx;
  h->g.ny = h->ny;
  h->g.nz = h->nz;
  h->g.nh = h->nh;
  h->g.pitch = h->pitch;
  h->g.rpitch = h->rpitch;
  h->g.fs = h->fs;
  h->g.rfs = h->rfs;
  h->g.kx = h->kx;
  h->g.ky = h->ky;
  h->g.kz = h->kz;
  h->g.i0 = h->i0;
  if ((rc = refresh3(h))) return fail(rc);
  *out = h;
  return set_ok();
}

int tara3d_set_state(tara3d* h, const double* state8, const double* hist8) {
  if (!h || !state8) return set_error(TARA_ERR_ARGS, "null argument");
  TARA_CK(cudaSetDevice(h->dev));
  const size_t dense = (size_t)2 * h->nh * h->ny * h->nz;
  int rc;
  for (int f = 0; f < S_N; ++f) {
    if ((rc = copy3(h, h->st + f * h->fs, state8 + f * dense, cudaMemcpyHostToDevice, nullptr)))
      return rc;
    if (hist8) {
      if ((rc = copy3(h, h->hist + f * h->fs, hist8 + f * dense, cudaMemcpyHostToDevice, nullptr)))
        return rc;
    }
  }
  if (!hist8) TARA_CK(cudaMemsetAsync(h->hist, 0, S_N * h->fs * sizeof(double2), h->stream));
  TARA_CK(cudaStreamSynchronize(h->stream));
  return set_ok();
}

int tara3d_get_state(tara3d* h, double* state8, double* hist8) {
  if (!h || !state8) return set_error(TARA_ERR_ARGS, "null argument");
  TARA_CK(cudaSetDevice(h->dev));
  const size_t dense = (size_t)2 * h->nh * h->ny * h->nz;
  int rc;
  for (int f = 0; f < S_N; ++f) {
    if ((rc = copy3(h, h->st + f * h->fs, nullptr, cudaMemcpyDeviceToHost, state8 + f * dense)))
      return rc;
    if (hist8 && (rc = copy3(h, h->hist + f * h->fs, nullptr, cudaMemcpyDeviceToHost, hist8 + f * dense)))
      return rc;
  }
  TARA_CK(cudaStreamSynchronize(h->stream));
  return set_ok();
}

// real fields (Nx,Ny,Nz) x-fastest in the state order -> state spectra (r2c on the GPU)
int tara3d_set_state_real(tara3d* h, const double* real8) {
  if (!h || !real8) return set_error(TARA_ERR_ARGS, "null argument");
  TARA_CK(cudaSetDevice(h->dev));
  const size_t rowb = h->nx * sizeof(double), rp = h->rpitch * sizeof(double);
  const size_t rows = (size_t)h->ny * h->nz, dense = (size_t)h->nx * h->ny * h->nz;
  for (int f = 0; f < S_N; ++f)
    TARA_CK(cudaMemcpy2DAsync(h->rl + f * h->rfs, rp, real8 + f * dense, rowb, rowb, rows,
                              cudaMemcpyHostToDevice, h->stream));
  int rc;
  if ((rc = r2c3(h, h->rl, h->st, S_N))) return rc;
  TARA_CK(cudaMemsetAsync(h->hist, 0, S_N * h->fs * sizeof(double2), h->stream));
  TARA_CK(cudaStreamSynchronize(h->stream));
  return set_ok();
}

int tara3d_init_orszag_tang(tara3d* h, double amp, int kmax, uint64_t seed) {
  if (!h || !(amp >= 0.0) || kmax < 0) return set_error(TARA_ERR_ARGS, "bad arguments");
  if (2 * kmax >= h->nx || 2 * kmax >= h->ny || 2 * kmax >= h->nz || h->nx < 8)
    return set_error(TARA_ERR_ARGS, "kmax must stay below the Nyquist modes (2 kmax < Nx, Ny, Nz)");
  TARA_CK(cudaSetDevice(h->dev));
  std::vector<double2> spec;
  ot_spectra(h->nx, h->ny, h->nz, amp, kmax, seed, spec);
  const size_t fs = (size_t)h->nh * h->ny * h->nz;
  int rc;
  const int slot[6] = {S_RUX, S_RUY, S_RUZ, S_BX, S_BY, S_BZ};
  for (int f = 0; f < 6; ++f)
    if ((rc = copy3(h, h->st + slot[f] * h->fs, (const double*)(spec.data() + f * fs),
                    cudaMemcpyHostToDevice, nullptr)))
      return rc;
  if ((rc = c2r3(h, h->st + S_RUX * h->fs, h->rl + S_RUX * h->rfs, 3))) return rc;
  if ((rc = c2r3(h, h->st + S_BX * h->fs, h->rl + S_BX * h->rfs, 3))) return rc;
  k3_ot_fill<<<kPwBlocks, kPwThreads, 0, h->stream>>>(h->rl, h->g, h->p.inv_n);
  TARA_CK(cudaGetLastError());
  if ((rc = r2c3(h, h->rl, h->st, S_N))) return rc;
  TARA_CK(cudaMemsetAsync(h->hist, 0, S_N * h->fs * sizeof(double2), h->stream));
  TARA_CK(cudaStreamSynchronize(h->stream));
  return set_ok();
}

int tara3d_step(tara3d* h, int nsteps) {
  if (!h || nsteps < 0) return set_error(TARA_ERR_ARGS, "bad arguments");
  TARA_CK(cudaSetDevice(h->dev));
  int rc;
  for (int s = 0; s < nsteps; ++s)
    if ((rc = rhs3(h, MODE_AB2, 0))) return rc;
  return set_ok();
}

int tara3d_rhs(tara3d* h, double* d8) {
  if (!h || !d8) return set_error(TARA_ERR_ARGS, "null argument");
  TARA_CK(cudaSetDevice(h->dev));
  int rc;
  if ((rc = rhs3(h, MODE_DERIVE, 1))) return rc;
  const size_t dense = (size_t)2 * h->nh * h->ny * h->nz;
  for (int f = 0; f < S_N; ++f)
    if ((rc = copy3(h, h->dout + f * h->fs, nullptr, cudaMemcpyDeviceToHost, d8 + f * dense)))
      return rc;
  TARA_CK(cudaStreamSynchronize(h->stream));
  return set_ok();
}

void* tara3d_stream(tara3d* h) { return h ? (void*)h->stream : nullptr; }

int tara3d_diag(tara3d* h, double* out4) {
  if (!h || !out4) return set_error(TARA_ERR_ARGS, "null argument");
  TARA_CK(cudaSetDevice(h->dev));
  int rc;
  if ((rc = c2r3(h, h->st, h->rl, S_N))) return rc;
  k3_prim<<<kPwBlocks, kPwThreads, 0, h->stream>>>(h->rl, h->pr, h->g, h->p);
  TARA_CK(cudaGetLastError());
  double* part = nullptr;
  TARA_CK(cudaMalloc(&part, 4 * kPwBlocks * sizeof(double)));
  k3_diag_partial<<<kPwBlocks, kPwThreads, 0, h->stream>>>(h->rl, h->pr, h->g, h->p.inv_n, part);
  std::vector<double> hp(4 * kPwBlocks);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(hp.data(), part, hp.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  cudaFree(part);
  if (e != cudaSuccess) return cuda_fail(e, "tara3d_diag");
  double a[4] = {0, 0, 0, 0};
  for (int b = 0; b < kPwBlocks; ++b)
    for (int k = 0; k < 4; ++k) a[k] += hp[4 * b + k];
  const double n = (double)h->nx * (double)h->ny * (double)h->nz;
  out4[0] = h->cfg.cs * h->cfg.cs * a[0] / n;  // Pressure = <CS^2 rho>
  out4[1] = a[1] / (2.0 * n);                  // Energy = <|u|^2>/2
  out4[2] = a[2] / n;                          // T_Energy = <E>
  out4[3] = a[3] / (2.0 * n);                  // B_Field = <|B|^2>/(2 mu_0), mu_0 = 1
  for (int k = 0; k < 4; ++k)
    if (!std::isfinite(out4[k])) return set_error(TARA_ERR_NONFINITE, "non-finite 3D diagnostics");
  return set_ok();
}

int tara3d_synchronize(tara3d* h) {
  if (!h) return set_error(TARA_ERR_ARGS, "null handle");
  TARA_CK(cudaSetDevice(h->dev));
  unsigned int f = 0;
  TARA_CK(cudaMemcpyAsync(&f, h->flag, sizeof(f), cudaMemcpyDeviceToHost, h->stream));
  TARA_CK(cudaStreamSynchronize(h->stream));
  if (f) return set_error(TARA_ERR_NONFINITE, "non-finite value in the MHD update");
  return set_ok();
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Fortran drop-ins
// ---------------------------------------------------------------------------
namespace {
std::mutex g_mu3;
std::map<std::tuple<int, int, int>, tara3d*> g_ctx3;

// Context for a shape, parameters refreshed from /comm/ and the pi argument.
tara3d* ctx3(int nx, int ny, int nz, double pi) {
  auto key = std::make_tuple(nx, ny, nz);
  tara3d* h = nullptr;
  auto it = g_ctx3.find(key);
  if (it != g_ctx3.end()) {
    h = it->second;
  } else {
    tara3d_config c;
    tara3d_default_config(&c, nx, ny, nz);
    if (tara3d_create(&c, &h) != TARA_OK) return nullptr;
    g_ctx3[key] = h;
  }
  tara3d_config& c = h->cfg;
  if (c.kpi != pi || c.lx != comm_.Lx || c.ly != comm_.Ly || c.lz != comm_.Lz ||
      c.mu != comm_.mu || c.eta != comm_.eta || c.cs != comm_.CS || c.dt != comm_.dt) {
    c.kpi = pi;
    c.lx = comm_.Lx;
    c.ly = comm_.Ly;
    c.lz = comm_.Lz;
    c.mu = comm_.mu;
    c.eta = comm_.eta;
    c.cs = comm_.CS;
    c.dt = comm_.dt;
    c.defined = 0;  // the reference's 1/450 viscosity and resistivity
    if (refresh3(h)) return nullptr;
  }
  return h;
}

bool dims3(const int* Nx, const int* Ny, const int* Nz, const int* Nh) {
  auto ok = [](int n) { return n >= 16 && n <= kMax3D && (n & (n - 1)) == 0; };
  if (!Nx || !Ny || !Nz || !Nh || !ok(*Nx) || !ok(*Ny) || !ok(*Nz) || *Nh != *Nx / 2 + 1) {
    set_error(TARA_ERR_ARGS, "Nx, Ny, Nz must be powers of two in [16, 512] and Nh = Nx/2+1");
    return false;
  }
  return true;
}
}  // namespace

extern "C" {

void derive3com_(const int* Nx, const int* Ny, const int* Nz, const int* Nh, const double* pi,
                 const double* time, const double* rho_k, const double* rho_ux_k,
                 const double* rho_uy_k, const double* rho_uz_k, const double* E_k,
                 const double* Bx_k, const double* By_k, const double* Bz_k, double* d_rho_old,
                 double* d_rho_new, double* d_rux_old, double* d_rux_new, double* d_ruy_old,
                 double* d_ruy_new, double* d_ruz_old, double* d_ruz_new, double* d_E_old,
                 double* d_E_new, double* d_Bx_old, double* d_Bx_new, double* d_By_old,
                 double* d_By_new, double* d_Bz_old, double* d_Bz_new) {
  (void)time; (void)d_rho_old; (void)d_rux_old; (void)d_ruy_old; (void)d_ruz_old; (void)d_E_old;
  (void)d_Bx_old; (void)d_By_old; (void)d_Bz_old;
  std::lock_guard<std::mutex> lk(g_mu3);
  if (!dims3(Nx, Ny, Nz, Nh) || !pi) return;
  const double* in[S_N] = {rho_k, rho_ux_k, rho_uy_k, rho_uz_k, E_k, Bx_k, By_k, Bz_k};
  double* outp[S_N] = {d_rho_new, d_rux_new, d_ruy_new, d_ruz_new, d_E_new, d_Bx_new, d_By_new, d_Bz_new};
  for (int f = 0; f < S_N; ++f)
    if (!in[f] || !outp[f]) {
      set_error(TARA_ERR_ARGS, "null array argument");
      return;
    }
  tara3d* h = ctx3(*Nx, *Ny, *Nz, *pi);
  if (!h) return;
  if (cudaSetDevice(h->dev) != cudaSuccess) {
    set_error(TARA_ERR_CUDA, "cudaSetDevice failed");
    return;
  }
  for (int f = 0; f < S_N; ++f)
    if (copy3(h, h->st + f * h->fs, in[f], cudaMemcpyHostToDevice, nullptr)) return;
  if (rhs3(h, MODE_DERIVE, 1)) return;
  for (int f = 0; f < S_N; ++f)
    if (copy3(h, h->dout + f * h->fs, nullptr, cudaMemcpyDeviceToHost, outp[f])) return;
  cudaError_t e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) {
    cuda_fail(e, "derive3com");
    return;
  }
  set_ok();
}

void ab3com_(const int* Nx, const int* Ny, const int* Nz, const int* Nh, const double* pi,
             const double* time, const double* rho_k, const double* rho_ux_k,
             const double* rho_uy_k, const double* rho_uz_k, const double* E_k, const double* Bx_k,
             const double* By_k, const double* Bz_k, double* rho_k_new, double* rho_ux_k_new,
             double* rho_uy_k_new, double* rho_uz_k_new, double* E_k_new, double* Bx_k_new,
             double* By_k_new, double* Bz_k_new, const double* d_rho_old, const double* d_rho_new,
             const double* d_rux_old, const double* d_rux_new, const double* d_ruy_old,
             const double* d_ruy_new, const double* d_ruz_old, const double* d_ruz_new,
             const double* d_E_old, const double* d_E_new, const double* d_Bx_old,
             const double* d_Bx_new, const double* d_By_old, const double* d_By_new,
             const double* d_Bz_old, const double* d_Bz_new) {
  (void)time;
  std::lock_guard<std::mutex> lk(g_mu3);
  if (!dims3(Nx, Ny, Nz, Nh) || !pi) return;
  const double* s[S_N] = {rho_k, rho_ux_k, rho_uy_k, rho_uz_k, E_k, Bx_k, By_k, Bz_k};
  double* sn[S_N] = {rho_k_new, rho_ux_k_new, rho_uy_k_new, rho_uz_k_new, E_k_new, Bx_k_new, By_k_new, Bz_k_new};
  const double* dold[S_N] = {d_rho_old, d_rux_old, d_ruy_old, d_ruz_old, d_E_old, d_Bx_old, d_By_old, d_Bz_old};
  const double* dnew[S_N] = {d_rho_new, d_rux_new, d_ruy_new, d_ruz_new, d_E_new, d_Bx_new, d_By_new, d_Bz_new};
  for (int f = 0; f < S_N; ++f)
    if (!s[f] || !sn[f] || !dold[f] || !dnew[f]) {
      set_error(TARA_ERR_ARGS, "null array argument");
      return;
    }
  tara3d* h = ctx3(*Nx, *Ny, *Nz, *pi);
  if (!h) return;
  if (cudaSetDevice(h->dev) != cudaSuccess) {
    set_error(TARA_ERR_CUDA, "cudaSetDevice failed");
    return;
  }
  for (int f = 0; f < S_N; ++f)
    if (copy3(h, h->st + f * h->fs, s[f], cudaMemcpyHostToDevice, nullptr) ||
        copy3(h, h->hist + f * h->fs, dold[f], cudaMemcpyHostToDevice, nullptr) ||
        copy3(h, h->dout + f * h->fs, dnew[f], cudaMemcpyHostToDevice, nullptr))
      return;
  k3_ab2_dense<<<kPwBlocks, kPwThreads, 0, h->stream>>>(h->st, h->cw, h->hist, h->dout, h->fs,
                                                        comm_.dt);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    cuda_fail(e, "k3_ab2_dense");
    return;
  }
  for (int f = 0; f < S_N; ++f)
    if (copy3(h, h->cw + f * h->fs, nullptr, cudaMemcpyDeviceToHost, sn[f])) return;
  e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) {
    cuda_fail(e, "ab3com");
    return;
  }
  set_ok();
}

}  // extern "C"

namespace tara {
int release_dropins_3d() {
  std::lock_guard<std::mutex> lk(g_mu3);
  int rc = TARA_OK;
  for (auto& kv : g_ctx3) {
    const int r = tara3d_destroy(kv.second);
    if (r != TARA_OK && rc == TARA_OK) rc = r;
  }
  g_ctx3.clear();
  return rc;
}
}  // namespace tara
