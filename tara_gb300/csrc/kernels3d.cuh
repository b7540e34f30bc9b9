// 3D pseudo-spectral kernels for the compressible MHD right-hand side of
// derive3com (src/derive3com.f95) and the AB2 update of ab3com
// (src/ab3com.f95), FP64.
//
// Layout: a half spectrum is field[(z*Ny + y)*pitch + x], x in [0,Nh), the
// reference's complex(8) a(Nh,Ny,Nz) with padded rows; a real field is
// field[(z*Ny + y)*rpitch + x], x in [0,Nx).  Fields of one kind are stored back
// to back so that one launch transforms a batch of them (blockIdx.z or
// blockIdx.y selects the field).
//
// A rank-3 c2r follows FFTW's order: complex DFTs along z and y for every kx
// column, then the 1D c2r along x that reads only the real parts of the kx = 0
// and kx = Nx/2 bins; r2c runs the same passes in reverse.
#pragma once
#include "fft.cuh"
#include "kernels2d.cuh"

namespace tara {

// Strided line transforms: element (f, o, p, x) of a batch lives at
// f*fs + o*os + p*ps + x; a CTA transforms the lines of TC consecutive x for one
// outer index o = blockIdx.y of field f = blockIdx.z.  in == out is allowed.
template <typename T, int N, bool INV>
__global__ void __launch_bounds__(ColCfg<T, N>::THREADS_C)
    k_lines(const typename cplx_of<T>::type* in, typename cplx_of<T>::type* out, int nh,
            size_t ps, size_t os, size_t fs_in, size_t fs_out,
            const typename cplx_of<T>::type* __restrict__ tw) {
  typedef typename cplx_of<T>::type C;
  typedef ColCfg<T, N> CF;
  constexpr int TC = CF::TCC, S = CF::S, G = CF::G;
  extern __shared__ __align__(16) unsigned char smraw[];
  C* sm = reinterpret_cast<C*>(smraw);
  const int x0 = blockIdx.x * TC, tid = threadIdx.x;
  const size_t bi = (size_t)blockIdx.z * fs_in + (size_t)blockIdx.y * os;
  const size_t bo = (size_t)blockIdx.z * fs_out + (size_t)blockIdx.y * os;
  for (int e = tid; e < N * TC; e += CF::THREADS_C) {
    const int p = e / TC, c = e % TC, x = x0 + c;
    sm[c * S + p] = (x < nh) ? in[bi + (size_t)p * ps + x] : mkc<T>(T(0), T(0));
  }
  __syncthreads();
  fft_slot<T, N, INV>(sm + (tid / G) * S, tid % G, true, tw);
  for (int e = tid; e < N * TC; e += CF::THREADS_C) {
    const int p = e / TC, c = e % TC, x = x0 + c;
    if (x < nh) out[bo + (size_t)p * ps + x] = sm[c * S + p];
  }
}

// x-direction c2r of `rows` rows per field (pairs of rows per complex transform),
// field = blockIdx.y.  Unnormalised.
template <typename T, int N>
__global__ void __launch_bounds__(RowCfg<T, N>::THREADS)
    k_rows_c2r(const typename cplx_of<T>::type* __restrict__ in, T* __restrict__ out, int rows,
               int pitch, int rpitch, size_t fs_in, size_t fs_out,
               const typename cplx_of<T>::type* __restrict__ tw) {
  typedef typename cplx_of<T>::type C;
  typedef RowCfg<T, N> RC;
  constexpr int G = RC::G, H = N / 2, NP = 4 * RC::RP, SL = RC::SL;
  extern __shared__ __align__(16) unsigned char smraw[];
  C* sm = reinterpret_cast<C*>(smraw);
  const int tid = threadIdx.x, y_base = blockIdx.x * (2 * NP);
  const C* fin = in + (size_t)blockIdx.y * fs_in;
  T* fout = out + (size_t)blockIdx.y * fs_out;
  for (int e = tid; e < NP * N; e += RC::THREADS) {
    const int k = e % N, pp = e / N, ya = y_base + 2 * pp;
    C z = mkc<T>(T(0), T(0));
    if (ya < rows) {
      const int kk = k <= H ? k : N - k;
      C A = fin[(size_t)ya * pitch + kk], B = fin[(size_t)(ya + 1) * pitch + kk];
      if (kk == 0 || kk == H) {
        A.y = T(0);
        B.y = T(0);
      }
      z = (k <= H) ? mkc<T>(A.x - B.y, A.y + B.x) : mkc<T>(A.x + B.y, -A.y + B.x);
    }
    sm[pp * SL + k] = z;
  }
  __syncthreads();
  fft_slot<T, N, true>(sm + (tid / G) * SL, tid % G, true, tw);
  for (int e = tid; e < NP * N; e += RC::THREADS) {
    const int x = e % N, pp = e / N, ya = y_base + 2 * pp;
    if (ya < rows) {
      const C z = sm[pp * SL + x];
      fout[(size_t)ya * rpitch + x] = z.x;
      fout[(size_t)(ya + 1) * rpitch + x] = z.y;
    }
  }
}

// x-direction r2c of `rows` real rows per field, field = blockIdx.y.
template <typename T, int N>
__global__ void __launch_bounds__(RowCfg<T, N>::THREADS)
    k_rows_r2c(const T* __restrict__ in, typename cplx_of<T>::type* __restrict__ out, int rows,
               int rpitch, int pitch, size_t fs_in, size_t fs_out,
               const typename cplx_of<T>::type* __restrict__ tw) {
  typedef typename cplx_of<T>::type C;
  typedef RowCfg<T, N> RC;
  constexpr int G = RC::G, H = N / 2, NP = 4 * RC::RP, SL = RC::SL;
  extern __shared__ __align__(16) unsigned char smraw[];
  C* sm = reinterpret_cast<C*>(smraw);
  const int tid = threadIdx.x, y_base = blockIdx.x * (2 * NP);
  const T* fin = in + (size_t)blockIdx.y * fs_in;
  C* fout = out + (size_t)blockIdx.y * fs_out;
  for (int e = tid; e < NP * N; e += RC::THREADS) {
    const int x = e % N, pp = e / N, ya = y_base + 2 * pp;
    sm[pp * SL + x] = (ya < rows) ? mkc<T>(fin[(size_t)ya * rpitch + x], fin[(size_t)(ya + 1) * rpitch + x])
                                 : mkc<T>(T(0), T(0));
  }
  __syncthreads();
  fft_slot<T, N, false>(sm + (tid / G) * SL, tid % G, true, tw);
  for (int e = tid; e < NP * (H + 1); e += RC::THREADS) {
    const int k = e % (H + 1), pp = e / (H + 1), ya = y_base + 2 * pp;
    if (ya < rows) {
      const C z = sm[pp * SL + k], m = sm[pp * SL + ((N - k) & (N - 1))];
      fout[(size_t)ya * pitch + k] = mkc<T>(T(0.5) * (z.x + m.x), T(0.5) * (z.y - m.y));
      fout[(size_t)(ya + 1) * pitch + k] = mkc<T>(T(0.5) * (z.y + m.y), T(-0.5) * (z.x - m.x));
    }
  }
}

struct Grid3D {
  int nx, ny, nz, nh, pitch, rpitch;
  size_t fs, rfs;                   // spectral / real field strides (elements)
  const double* __restrict__ kx;    // [nh]
  const double* __restrict__ ky;    // [ny]
  const double* __restrict__ kz;    // [nz]
  const int* __restrict__ i0;       // [nz*ny]: first kx index outside the dealiasing sphere
};

struct Mhd3DParams {
  double inv_n;   // 1/(Nx Ny Nz)
  double cs2;     // CS*CS
  double eta;     // resistivity in the energy flux
  double mu;      // coefficient of E_Visc
  int defined;    // 0: k^2 f / 450 ; 1: nu_u k^2 u, eta_b k^2 B
  double nu_u, eta_b;
  double dt;
};

// State field order (the reference's argument order).
enum { S_RHO = 0, S_RUX, S_RUY, S_RUZ, S_E, S_BX, S_BY, S_BZ, S_N };
// Product field order in the work arrays.
enum { P_UX = 0, P_UY, P_UZ, P_MXX, P_MXY, P_MXZ, P_MYY, P_MYZ, P_MZZ, P_G1, P_G2, P_G3,
       P_ENX, P_ENY, P_ENZ, P_EVISC, P_N };
// Real derivative fields of the energy equation.
enum { D_DIV = 0, D_CX, D_CY, D_CZ, D_N };

// Primitive variables and fluxes in real space (src/derive3com.f95:147-175,
// 363-436): u = rho u / rho, P = CS^2 rho, B^2, the symmetric momentum flux
// (Mom_x_2 = Mom_y_1 exactly; Mom_x_3 / Mom_z_1 and Mom_y_3 / Mom_z_2 differ
// only in rounding) and the three distinct induction products
// (Mag_x_1 = Mag_y_1, Mag_x_2 = Mag_z_1, Mag_y_2 = Mag_z_2).
__global__ void k3_prim(const double* __restrict__ rl, double* __restrict__ pr, Grid3D g,
                        Mhd3DParams p);
// Energy fluxes and E_Visc (src/derive3com.f95:411-423), from the real fields,
// the velocities and the c2r of div u and curl B.
__global__ void k3_energy(const double* __restrict__ rl, double* __restrict__ pr,
                          const double* __restrict__ dr, Grid3D g, Mhd3DParams p);
// Spectral fields of div u and curl B for the energy equation (src/derive3com.f95:224-298).
__global__ void k3_derivs(const double2* __restrict__ st, const double2* __restrict__ pk,
                          double2* __restrict__ dk, Grid3D g);
// Assembly (src/derive3com.f95:561-1043) with the dealiasing sphere, then
// MODE_DERIVE (write all 8 derivatives) or MODE_AB2 (src/ab3com.f95:39-59,
// E frozen; the history rotation of src/main3com.f95:570-586 fused in).
__global__ void k3_assemble(double2* __restrict__ st, const double2* __restrict__ pk,
                            double2* __restrict__ dout, double2* __restrict__ hist, Grid3D g,
                            Mhd3DParams p, int mode, int with_energy, unsigned int* flag);

}  // namespace tara
