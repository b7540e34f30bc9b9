/* CPU oracle for the TARA 2D pseudo-spectral path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference subroutines on the hot path, used by
 * the test suite, smoke() and the bench's CPU-baseline leg as the oracle.  It
 * is never linked into the product library.
 *
 * Arrays follow the reference's Fortran layout: a half spectrum complex(8)
 * omegak(Nh,Ny) is Nh*Ny interleaved (re,im) doubles with the kx index fastest;
 * a real field omega(Nx,Ny) is Nx*Ny doubles with x fastest.
 *
 * Two FFT backends share this source: the default build uses the oracle's own
 * radix-2 FFT (builds anywhere); -DORACLE_USE_FFTW routes every transform
 * through FFTW 3.3.9 compiled from the reference's vendored sources, planned
 * with FFTW_ESTIMATE before each transform exactly as the reference does
 * (src/derive2csh.f95:73-106).  The FFTW build pins the own-FFT build and makes
 * the golden vectors.
 */
#ifndef TARA_ORACLE_H
#define TARA_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* 1 when the loaded library routes transforms through FFTW, 0 for the own FFT */
int oracle_backend_is_fftw(void);
/* OpenMP threads used by the own-FFT backend (<=0: all available) */
void oracle_set_threads(int n);
int oracle_get_threads(void);

/* Unnormalised 2D transforms with FFTW's r2c/c2r semantics
 * (dfftw_plan_dft_{r2c,c2r}_2d with Fortran dims (Nx,Ny), see
 * lib/fftw/api/f77funcs.h:206-209,300-303).  c2r leaves `in` untouched. */
void oracle_r2c_2d(int nx, int ny, const double* in, double* out);
void oracle_c2r_2d(int nx, int ny, const double* in, double* out);

/* src/derive2csh.f95:3-149 (plain RHS, faithful: pi=3.1428 real*4, Lx=Ly=2*pi) */
void oracle_derive2csh(const int* Nx, const int* Ny, const int* Nh, const double* nu,
                       const double* time, double* omegak, double* omegak_new,
                       double* dt_omegak_old, double* dt_omegak_new);
/* src/ab2csh.f95:3-16 */
void oracle_ab2csh(const int* Nx, const int* Ny, const int* Nh, const double* nu,
                   const double* time, const double* dt, double* omegak, double* omegak_new,
                   double* dt_omegak_old, double* dt_omegak_new);
/* src/derive2css.f95:6-136 in defined mode: Lx, Ly, lambda come from
 * oracle_set_css_params (defaults 2*3.1428f, 2*3.1428f, 10) */
void oracle_set_css_params(double lx, double ly, double lambda);
void oracle_derive2css(const int* Nx, const int* Ny, const int* Nh, const double* alpha,
                       const double* nu, const double* time, double* omegak, double* omegak_new,
                       double* dt_omegak_old, double* dt_omegak_new);
/* src/ab2css.f95:6-22 */
void oracle_ab2css(const int* Nx, const int* Ny, const int* Nh, const double* alpha,
                   const double* nu, const double* time, const double* dt, double* omegak,
                   double* omegak_new, double* dt_omegak_old, double* dt_omegak_new);
/* Classic RK4 with the signature of src/rk42css.f95:6-13 (the reference body is
 * non-functional); rhs_kind 0 = derive2csh, 1 = derive2css. */
void oracle_rk42css(const int* Nx, const int* Ny, const int* Nh, const double* alpha,
                    const double* nu, const double* time, const double* dt, double* omegak,
                    double* omegak_new, double* dt_omegak_old, double* dt_omegak_new);
void oracle_rk4csh(const int* Nx, const int* Ny, const int* Nh, const double* nu,
                   const double* time, const double* dt, double* omegak, double* omegak_new);

/* Step driver: nsteps of scheme (0 AB2 with the driver's history rotation,
 * src/main2csh.f95:114-126; 1 classic RK4) over rhs_kind (0 plain, 1 screened).
 * omegak is updated in place; dt_old holds the AB2 history (zero before the
 * first step, as the reference's fresh allocation reads). */
void oracle_run(int nx, int ny, int rhs_kind, int scheme, double alpha, double nu, double dt,
                int nsteps, double* omegak, double* dt_old);

/* Double-shear-layer initial vorticity in real space (src/main2css.f95:78-104 when
 * variant 0, src/main2csh.f95:84-106 when variant 1). */
void oracle_ic_shear(int nx, int ny, double lx_ini, double ly_ini, double w0, double m0,
                     double d_ini, int variant, double* omega);

/* Philox4x32-10 (Salmon et al., SC'11), one block. */
void oracle_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* Seeded random-phase initial spectrum: |w(k)| = sqrt(|k| E(|k|)/pi),
 * E(k) = k^4 exp(-(k/k0)^2), phase 2*pi*u with u from Philox (counter (i,j,0,0),
 * key (seed lo, seed hi)), Hermitian-projected by a c2r/r2c round trip and
 * mean mode set to zero, rescaled to 1/2<|u|^2> = energy.  Box Lx=Ly=2*pi. */
void oracle_ic_random(int nx, int ny, double k0, double energy, uint64_t seed, double* omegak);

/* Physical-space diagnostics of a half spectrum for a box (lx, ly) (true lengths):
 * out[0] = 1/2<|u|^2>, out[1] = 1/2<omega^2>; velocity from psi = omega/k^2. */
void oracle_energy_enstrophy(int nx, int ny, double lx, double ly, const double* omegak,
                             double* out);

/* Reference diagnostic of the screened driver (src/main2css.f95:206-275):
 * out[0] = Energy = sum(ux^2+uy^2), out[1] = sum(uy^2), out[2..5] = C0..C3, with
 * lambda applied to ky >= 0 rows only, as the reference does. */
void oracle_diag_css(int nx, int ny, double lx, double ly, double lambda, const double* omegak,
                     double* out);

/* Velocity of the plain driver on the grid (src/main2csh.f95:128-172): psi =
 * omegak/(kx^2+ky^2) (0 at the origin), ux = c2r(i ky psi)/(Nx*Ny), uy =
 * c2r(-i kx psi)/(Nx*Ny), kx = 2*pi*i/lx with the true pi (lx, ly true lengths).
 * ux, uy are (Ny, Nx) real arrays, x fastest. */
void oracle_driver_velocity(int nx, int ny, double lx, double ly, const double* omegak, double* ux,
                            double* uy);

/* One Euler step of np particles with bilinear interpolation of ux, uy
 * (src/main2csh.f95:187-271); the last column / row take the periodic neighbour
 * (the reference reads outside its arrays there). */
void oracle_particles_step(int nx, int ny, double lx, double ly, const double* ux, const double* uy,
                           int np, double* xp, double* yp, double dt);

/* ---- 3D compressible MHD (src/derive3com.f95, src/ab3com.f95) ---------- */
/* Half spectra are (Nh,Ny,Nz) complex(8), x fastest; real fields (Nx,Ny,Nz).
 * The state is 8 consecutive half spectra in the order of the reference's
 * arguments: rho, rho_ux, rho_uy, rho_uz, E, Bx, By, Bz. */
typedef struct oracle_mhd_params {
  double lx, ly, lz; /* true box lengths (Lx = Lx_ini*pi, src/main3com.f95) */
  double mu;         /* coefficient of E_Visc in the energy equation (ini nu) */
  double eta;        /* resistivity in the energy flux (0.005 in the reference) */
  double cs;         /* sound speed, P = CS^2 rho (CS = 1/M = 10) */
  int defined;       /* 0: viscous/resistive terms k^2 f / 450 (faithful);
                        1: nu_u k^2 u and eta_b k^2 B (defined mode) */
  double nu_u, eta_b;
} oracle_mhd_params;

void oracle_r2c_3d(int nx, int ny, int nz, const double* in, double* out);
void oracle_c2r_3d(int nx, int ny, int nz, const double* in, double* out);
/* src/derive3com.f95:6-1047 (the forcing, computed but unused there, is left out) */
void oracle_derive3com(int nx, int ny, int nz, const oracle_mhd_params* p, const double* state,
                       double* dstate);
/* src/ab3com.f95:6-66: AB2 for all fields except E, which stays frozen (:51) */
void oracle_ab3com(int nx, int ny, int nz, double dt, const double* state, double* state_new,
                   const double* d_old, const double* d_new);
/* derive3com + ab3com + the rotation of src/main3com.f95:560-614, nsteps times */
void oracle_run3d(int nx, int ny, int nz, const oracle_mhd_params* p, double dt, int nsteps,
                  double* state, double* hist);
/* Reference initial condition (src/main3com.f95:292-347): rho=1, ABC flow of
 * amplitude U0=0.1 (A=B=C=kf=1), uniform B = B0 = 0.1, P = 1, E from them; real
 * fields in the state order. */
void oracle_ic3d_abc(int nx, int ny, int nz, double lx_ini, double ly_ini, double lz_ini,
                     double* real8);
/* The 3D MHD benchmark's Orszag-Tang-type initial state with a seeded
 * solenoidal perturbation (spectral state (8, Nz, Ny, Nh); see tara_oracle.c). */
void oracle_ic3d_ot(int nx, int ny, int nz, double amp, int kmax, uint64_t seed, double* state);

/* ---- 2D compressible isothermal hydro (src/derive2coh.f95, src/ab2coh.f95) ---- */
typedef struct {
  double pi;       /* the pi argument of kx = 2 pi (i-1)/Lx */
  double lx, ly;   /* /comm/ Lx, Ly */
  double mux, muy; /* /comm/ viscosities */
  double cs;       /* /comm/ sound speed CS */
} oracle_coh_params;

/* src/derive2coh.f95:6-265: state = (nk, ukx, uky), three complex (Nh,Ny) spectra
 * back to back; writes (dn_dt_new, dux_dt_new, duy_dt_new) likewise. */
void oracle_derive2coh(int nx, int ny, const oracle_coh_params* p, const double* state,
                       double* dstate);
/* src/ab2coh.f95:5-34: AB2 of the three fields */
void oracle_ab2coh(int nx, int ny, double dt, const double* state, double* state_new,
                   const double* d_old, const double* d_new);
/* derive2coh + ab2coh + the rotation of src/main2coh.f95:277-298, nsteps times */
void oracle_run_coh(int nx, int ny, const oracle_coh_params* p, double dt, int nsteps,
                    double* state, double* hist);
/* Initial state of src/main2coh.f95:140-210: uniform density n0 = 1, vorticity 1
 * in a disk of radius 0.6 pi about the centre and 10 in five disks of radius 0.2
 * at distance 0.8 pi, velocity from psi = omega_hat/k^2 (true pi, Lx = lx_ini pi).
 * The reference's vortex angles come from an uninitialised counter whose
 * residues mod 5 give the same five positions at every grid point; they are
 * taken here as 2 pi r/5 with r = -1..-5. */
void oracle_ic_coh(int nx, int ny, double lx_ini, double ly_ini, double* state);

/* ---- 2D compressible MHD (src/derive2com.f95, src/ab2com.f95) ---------- */
typedef struct {
  double pi;       /* the pi argument of kx = 2 pi (i-1)/Lx */
  double lx, ly;   /* /comm/ Lx, Ly */
  double mu, eta;  /* /comm/ viscosity, resistivity */
  double cs;       /* /comm/ sound speed, P = CS^2 rho */
  double kf, a;    /* /comm/ forcing wavenumber and amplitude */
  int defined;     /* 0: curl B from d_ux_dx, d_uy_dy / (Nx Ny) as the reference
                      (src/derive2com.f95:186-187); 1: from dBx/dy, dBy/dx */
} oracle_com_params;

/* src/derive2com.f95:5-426: state = (rho, rho ux, rho uy, E, Bx, By), six
 * complex (Nh,Ny) spectra back to back; writes the six d/dt spectra.  The
 * forcing's coordinates x(i), y(j) are local arrays the reference never sets
 * (:16,109-110); here they are the driver's grid, (i-1) Lx/Nx and (j-1) Ly/Ny. */
void oracle_derive2com(int nx, int ny, const oracle_com_params* p, const double* state,
                       double* dstate);
/* src/ab2com.f95: AB2 of the six fields */
void oracle_ab2com(int nx, int ny, double dt, const double* state, double* state_new,
                   const double* d_old, const double* d_new);
/* derive2com + ab2com + the rotation of src/main2com.f95:375-414, nsteps times */
void oracle_run_com(int nx, int ny, const oracle_com_params* p, double dt, int nsteps,
                    double* state, double* hist);
/* Initial state of src/main2com.f95:229-291: rho = 1, ux = -sin(kf y),
 * uy = sin(kf x), P = CS^2 rho, Bx = By = B0, E = P/(5/3 - 1) + rho |u|^2/2 +
 * |B|^2/2 (x = 0.0d0+real(i-1)*dx, Lx = lx_ini pi). */
void oracle_ic_com(int nx, int ny, double lx_ini, double ly_ini, double cs, double kf, double b0,
                   double* state);

#ifdef __cplusplus
}
#endif
#endif
