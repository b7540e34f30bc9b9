/* CPU oracle for the TARA 2D pseudo-spectral path -- TEST INFRASTRUCTURE ONLY.
 *
 * Only the test suite, smoke() and the bench's CPU-baseline leg load this
 * library, and only as the checker.  The product library never links it.
 *
 * Each function restates one reference subroutine; the citation on each names
 * the file:line it follows.  All arithmetic is IEEE double without FMA
 * contraction (see the Makefile), in the reference's expression order where
 * the order changes the rounding.
 *
 * Parity pinning: the reference Fortran cannot be compiled here (no Fortran
 * compiler), so the restatement is pinned by building the same source against
 * FFTW 3.3.9 compiled from the reference's vendored sources (-DORACLE_USE_FFTW,
 * oracle/_ref) and comparing it with this own-FFT build; golden vectors are made
 * from the FFTW build.
 */
#include "tara_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#ifdef ORACLE_USE_FFTW
#include <fftw3.h>
#endif

/* real(kind=8), parameter :: pi = 3.1428 -- a default-real literal
 * (src/derive2csh.f95:16, src/derive2css.f95:18) */
#define PI_R4 ((double)3.1428f)
/* real(kind=8), parameter :: pi = 3.14159265358979323846d0 (src/main2css.f95:9) */
#define PI_R8 3.14159265358979323846

static int g_threads = 0;

void oracle_set_threads(int n) { g_threads = n; }

int oracle_get_threads(void) {
#ifdef _OPENMP
  return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
  return 1;
#endif
}

static void* xcalloc(size_t n, size_t sz) {
  void* p = calloc(n ? n : 1, sz);
  if (!p) abort();
  return p;
}

/* ------------------------------------------------------------------------- */
/* FFT backends                                                               */
/* ------------------------------------------------------------------------- */
#ifdef ORACLE_USE_FFTW
int oracle_backend_is_fftw(void) { return 1; }

/* dfftw_plan_dft_r2c_2d_(plan, Nx, Ny, in, out, FFTW_ESTIMATE) reverses the
 * dimensions to C order (lib/fftw/api/f77funcs.h:206-209); plan, execute and
 * destroy per call as the reference does. */
void oracle_r2c_2d(int nx, int ny, const double* in, double* out) {
  fftw_plan p = fftw_plan_dft_r2c_2d(ny, nx, (double*)in, (fftw_complex*)out, FFTW_ESTIMATE);
  fftw_execute(p);
  fftw_destroy_plan(p);
}

/* c2r may destroy its input, which is why the reference copies into *_dum
 * arrays first (src/derive2csh.f95:42-45); copy here so `in` stays intact. */
void oracle_c2r_2d(int nx, int ny, const double* in, double* out) {
  const size_t ns = (size_t)(nx / 2 + 1) * ny;
  double* tmp = (double*)xcalloc(2 * ns, sizeof(double));
  memcpy(tmp, in, 2 * ns * sizeof(double));
  fftw_plan p = fftw_plan_dft_c2r_2d(ny, nx, (fftw_complex*)tmp, out, FFTW_ESTIMATE);
  fftw_execute(p);
  fftw_destroy_plan(p);
  free(tmp);
}
#else
int oracle_backend_is_fftw(void) { return 0; }

/* Own FFT: iterative radix-2 decimation in time, twiddles from long-double
 * sin/cos rounded once.  Powers of two only. */
typedef struct {
  int n;
  double* w; /* w[2k] = cos(2 pi k/n), w[2k+1] = -sin(2 pi k/n), k < n/2 */
  int* rev;
} fft_plan;

static fft_plan g_plans[32];

static fft_plan* get_plan(int n) {
  int lg = 0;
  while ((1 << lg) < n) ++lg;
  fft_plan* p = &g_plans[lg];
  if (p->n == n) return p;
  p->w = (double*)xcalloc((size_t)n + 2, sizeof(double));
  p->rev = (int*)xcalloc((size_t)n, sizeof(int));
  for (int k = 0; k < n / 2; ++k) {
    long double a = 2.0L * 3.141592653589793238462643383279502884L * (long double)k / (long double)n;
    p->w[2 * k] = (double)cosl(a);
    p->w[2 * k + 1] = (double)-sinl(a);
  }
  for (int i = 0; i < n; ++i) {
    int r = 0;
    for (int b = 0; b < lg; ++b)
      if (i & (1 << b)) r |= 1 << (lg - 1 - b);
    p->rev[i] = r;
  }
  p->n = n;
  return p;
}

/* in-place complex DFT of z[n] (interleaved); sign -1 forward, +1 backward */
static void fft1d(double* z, int n, int sign, const fft_plan* p) {
  for (int i = 0; i < n; ++i) {
    int r = p->rev[i];
    if (r > i) {
      double tr = z[2 * i], ti = z[2 * i + 1];
      z[2 * i] = z[2 * r];
      z[2 * i + 1] = z[2 * r + 1];
      z[2 * r] = tr;
      z[2 * r + 1] = ti;
    }
  }
  for (int len = 2; len <= n; len <<= 1) {
    const int half = len >> 1, step = n / len;
    for (int b = 0; b < n; b += len) {
      for (int k = 0; k < half; ++k) {
        const double wr = p->w[2 * k * step];
        const double wi = sign < 0 ? p->w[2 * k * step + 1] : -p->w[2 * k * step + 1];
        double* a = z + 2 * (b + k);
        double* c = z + 2 * (b + k + half);
        const double tr = c[0] * wr - c[1] * wi;
        const double ti = c[0] * wi + c[1] * wr;
        c[0] = a[0] - tr;
        c[1] = a[1] - ti;
        a[0] = a[0] + tr;
        a[1] = a[1] + ti;
      }
    }
  }
}

/* rank-2 c2r as FFTW's rank-geq2-rdft2 orders it: complex backward DFTs along y
 * for every kx column, then 1D c2r along x, where the 1D c2r reads only the real
 * parts of the kx=0 and kx=Nx/2 bins.  Two rows share one complex transform. */
void oracle_c2r_2d(int nx, int ny, const double* in, double* out) {
  const int nh = nx / 2 + 1;
  const size_t ns = (size_t)nh * ny;
  double* tmp = (double*)xcalloc(2 * ns, sizeof(double));
  memcpy(tmp, in, 2 * ns * sizeof(double));
  const fft_plan* py = get_plan(ny);
  const fft_plan* px = get_plan(nx);
#pragma omp parallel num_threads(oracle_get_threads())
  {
    double* col = (double*)xcalloc(2 * (size_t)ny, sizeof(double));
#pragma omp for schedule(static)
    for (int i = 0; i < nh; ++i) {
      for (int j = 0; j < ny; ++j) {
        col[2 * j] = tmp[2 * ((size_t)j * nh + i)];
        col[2 * j + 1] = tmp[2 * ((size_t)j * nh + i) + 1];
      }
      fft1d(col, ny, +1, py);
      for (int j = 0; j < ny; ++j) {
        tmp[2 * ((size_t)j * nh + i)] = col[2 * j];
        tmp[2 * ((size_t)j * nh + i) + 1] = col[2 * j + 1];
      }
    }
    free(col);
    double* z = (double*)xcalloc(2 * (size_t)nx, sizeof(double));
#pragma omp for schedule(static)
    for (int j = 0; j < ny; j += 2) {
      const double* a = tmp + 2 * (size_t)j * nh;
      const double* b = (j + 1 < ny) ? tmp + 2 * (size_t)(j + 1) * nh : NULL;
      for (int k = 0; k <= nx / 2; ++k) {
        const int edge = (k == 0 || k == nx / 2);
        const double ar = a[2 * k], ai = edge ? 0.0 : a[2 * k + 1];
        const double br = b ? b[2 * k] : 0.0, bi = (b && !edge) ? b[2 * k + 1] : 0.0;
        z[2 * k] = ar - bi; /* A + iB */
        z[2 * k + 1] = ai + br;
        if (k > 0 && k < nx / 2) {
          z[2 * (nx - k)] = ar + bi; /* conj(A) + i conj(B) */
          z[2 * (nx - k) + 1] = -ai + br;
        }
      }
      fft1d(z, nx, +1, px);
      for (int x = 0; x < nx; ++x) {
        out[(size_t)j * nx + x] = z[2 * x];
        if (b) out[(size_t)(j + 1) * nx + x] = z[2 * x + 1];
      }
    }
    free(z);
  }
  free(tmp);
}

/* rank-2 r2c: 1D r2c along x per row (two rows per complex transform), then
 * forward complex DFTs along y per kx column. */
void oracle_r2c_2d(int nx, int ny, const double* in, double* out) {
  const int nh = nx / 2 + 1;
  const fft_plan* py = get_plan(ny);
  const fft_plan* px = get_plan(nx);
#pragma omp parallel num_threads(oracle_get_threads())
  {
    double* z = (double*)xcalloc(2 * (size_t)nx, sizeof(double));
#pragma omp for schedule(static)
    for (int j = 0; j < ny; j += 2) {
      const int two = (j + 1 < ny);
      for (int x = 0; x < nx; ++x) {
        z[2 * x] = in[(size_t)j * nx + x];
        z[2 * x + 1] = two ? in[(size_t)(j + 1) * nx + x] : 0.0;
      }
      fft1d(z, nx, -1, px);
      double* a = out + 2 * (size_t)j * nh;
      double* b = two ? out + 2 * (size_t)(j + 1) * nh : NULL;
      for (int k = 0; k <= nx / 2; ++k) {
        const int m = (nx - k) % nx;
        const double zr = z[2 * k], zi = z[2 * k + 1];
        const double mr = z[2 * m], mi = -z[2 * m + 1]; /* conj(Z[N-k]) */
        a[2 * k] = 0.5 * (zr + mr);
        a[2 * k + 1] = 0.5 * (zi + mi);
        if (b) { /* (Z - conj Z[N-k]) / 2i */
          b[2 * k] = 0.5 * (zi - mi);
          b[2 * k + 1] = -0.5 * (zr - mr);
        }
      }
    }
    free(z);
    double* col = (double*)xcalloc(2 * (size_t)ny, sizeof(double));
#pragma omp for schedule(static)
    for (int i = 0; i < nh; ++i) {
      for (int j = 0; j < ny; ++j) {
        col[2 * j] = out[2 * ((size_t)j * nh + i)];
        col[2 * j + 1] = out[2 * ((size_t)j * nh + i) + 1];
      }
      fft1d(col, ny, -1, py);
      for (int j = 0; j < ny; ++j) {
        out[2 * ((size_t)j * nh + i)] = col[2 * j];
        out[2 * ((size_t)j * nh + i) + 1] = col[2 * j + 1];
      }
    }
    free(col);
  }
}
#endif

/* ------------------------------------------------------------------------- */
/* Wavenumbers as the reference computes them                                 */
/* ------------------------------------------------------------------------- */
/* kx = 2.0d0*pi*dfloat(i-1)/Lx; ky likewise for j <= Ny/2 and
 * 2.0d0*pi*(dfloat(j-1)-Ny)/Ly above (src/derive2csh.f95:30,32,48). */
static double kx_of(int i0, double pi, double lx) { return 2.0 * pi * (double)i0 / lx; }
static double ky_of(int j0, int ny, double pi, double ly) {
  return (j0 < ny / 2) ? 2.0 * pi * (double)j0 / ly : 2.0 * pi * ((double)j0 - (double)ny) / ly;
}

/* ------------------------------------------------------------------------- */
/* derive2csh -- src/derive2csh.f95:3-149                                     */
/* ------------------------------------------------------------------------- */
void oracle_derive2csh(const int* Nx, const int* Ny, const int* Nh, const double* nu,
                       const double* time, double* omegak, double* omegak_new,
                       double* dt_omegak_old, double* dt_omegak_new) {
  (void)time; (void)omegak_new; (void)dt_omegak_old;
  const int nx = *Nx, ny = *Ny, nh = *Nh;
  const size_t ns = (size_t)nh * ny, nr = (size_t)nx * ny;
  const double pi = PI_R4, lx = 2.0 * pi, ly = 2.0 * pi; /* :16,20-21 */
  double* ukx = (double*)xcalloc(2 * ns, sizeof(double));
  double* uky = (double*)xcalloc(2 * ns, sizeof(double));
  double* ikxw = (double*)xcalloc(2 * ns, sizeof(double));
  double* ikyw = (double*)xcalloc(2 * ns, sizeof(double));
  double* nlkx = (double*)xcalloc(2 * ns, sizeof(double));
  double* nlky = (double*)xcalloc(2 * ns, sizeof(double));
  double* ux = (double*)xcalloc(nr, sizeof(double));
  double* uy = (double*)xcalloc(nr, sizeof(double));
  double* dwx = (double*)xcalloc(nr, sizeof(double));
  double* dwy = (double*)xcalloc(nr, sizeof(double));
  double* p1 = (double*)xcalloc(nr, sizeof(double));
  double* p2 = (double*)xcalloc(nr, sizeof(double));

  /* psi = omega/k^2 (psi(1,1)=0), u_x = i ky psi, u_y = -i kx psi  (:29-57);
   * i kx omega, i ky omega (:59-71) */
  for (int i = 0; i < nh; ++i) {
    const double kx = kx_of(i, pi, lx);
    for (int j = 0; j < ny; ++j) {
      const double ky = ky_of(j, ny, pi, ly);
      const size_t q = 2 * ((size_t)j * nh + i);
      const double wr = omegak[q], wi = omegak[q + 1];
      if (i == 0 && j == 0) {
        ukx[q] = ukx[q + 1] = uky[q] = uky[q + 1] = 0.0;
      } else {
        const double k2 = kx * kx + ky * ky;
        const double pr = wr / k2, pim = wi / k2;
        ukx[q] = -ky * pim; /* (0,1)*ky*psi */
        ukx[q + 1] = ky * pr;
        uky[q] = kx * pim; /* -(0,1)*kx*psi */
        uky[q + 1] = -(kx * pr);
      }
      ikxw[q] = -kx * wi;
      ikxw[q + 1] = kx * wr;
      ikyw[q] = -ky * wi;
      ikyw[q + 1] = ky * wr;
    }
  }
  /* four c2r (:73-87) */
  oracle_c2r_2d(nx, ny, ukx, ux);
  oracle_c2r_2d(nx, ny, uky, uy);
  oracle_c2r_2d(nx, ny, ikxw, dwx);
  oracle_c2r_2d(nx, ny, ikyw, dwy);
  /* normalise and form the products (:89-98) */
  const double nn = (double)nx * (double)ny;
  for (size_t r = 0; r < nr; ++r) {
    const double a = ux[r] / nn, b = uy[r] / nn, c = dwx[r] / nn, d = dwy[r] / nn;
    p1[r] = a * c;
    p2[r] = b * d;
  }
  /* two r2c (:100-106) */
  oracle_r2c_2d(nx, ny, p1, nlkx);
  oracle_r2c_2d(nx, ny, p2, nlky);
  /* 2/3 truncation on both spectra (:108-125), then NL + nu k^2 omega and
   * dt_omegak_new = -NLk (:127-145) */
  const double cut = ((double)(nx + ny) / 2.0) / 3.0;
  for (int i = 0; i < nh; ++i) {
    const double kx = kx_of(i, pi, lx);
    for (int j = 0; j < ny; ++j) {
      const double ky = ky_of(j, ny, pi, ly);
      const size_t q = 2 * ((size_t)j * nh + i);
      if (sqrt(kx * kx + ky * ky) >= cut) {
        nlkx[q] = nlkx[q + 1] = nlky[q] = nlky[q + 1] = 0.0;
      }
      const double vk2 = *nu * (kx * kx + ky * ky);
      const double nr_ = (nlkx[q] + nlky[q]) + vk2 * omegak[q];
      const double ni_ = (nlkx[q + 1] + nlky[q + 1]) + vk2 * omegak[q + 1];
      dt_omegak_new[q] = -nr_;
      dt_omegak_new[q + 1] = -ni_;
    }
  }
  free(ukx); free(uky); free(ikxw); free(ikyw); free(nlkx); free(nlky);
  free(ux); free(uy); free(dwx); free(dwy); free(p1); free(p2);
}

/* ab2csh -- src/ab2csh.f95:10-14, ab2css -- src/ab2css.f95:14-18:
 * omegak_new = omegak + (3/2 dt_new - 1/2 dt_old) dt */
static void ab2_update(int nh, int ny, double dt, const double* w, double* wn, const double* fo,
                       const double* fn) {
  const size_t n2 = 2 * (size_t)nh * ny;
  for (size_t q = 0; q < n2; ++q) wn[q] = w[q] + ((3.0 / 2.0) * fn[q] - (1.0 / 2.0) * fo[q]) * dt;
}

void oracle_ab2csh(const int* Nx, const int* Ny, const int* Nh, const double* nu,
                   const double* time, const double* dt, double* omegak, double* omegak_new,
                   double* dt_omegak_old, double* dt_omegak_new) {
  (void)Nx; (void)nu; (void)time;
  ab2_update(*Nh, *Ny, *dt, omegak, omegak_new, dt_omegak_old, dt_omegak_new);
}

void oracle_ab2css(const int* Nx, const int* Ny, const int* Nh, const double* alpha,
                   const double* nu, const double* time, const double* dt, double* omegak,
                   double* omegak_new, double* dt_omegak_old, double* dt_omegak_new) {
  (void)Nx; (void)alpha; (void)nu; (void)time;
  ab2_update(*Nh, *Ny, *dt, omegak, omegak_new, dt_omegak_old, dt_omegak_new);
}

/* ------------------------------------------------------------------------- */
/* derive2css -- src/derive2css.f95:6-136, defined mode                       */
/* ------------------------------------------------------------------------- */
/* The reference reads Lx, Ly and lambda as uninitialised locals (:12); the
 * defined mode takes them from here.  Defaults: the plain RHS's box
 * (2*3.1428, integer wavenumbers) and the driver's lambda = 10
 * (src/main2css.f95:87). */
static double g_css_lx = 2.0 * PI_R4, g_css_ly = 2.0 * PI_R4, g_css_lambda = 10.0;

void oracle_set_css_params(double lx, double ly, double lambda) {
  g_css_lx = lx;
  g_css_ly = ly;
  g_css_lambda = lambda;
}

void oracle_derive2css(const int* Nx, const int* Ny, const int* Nh, const double* alpha,
                       const double* nu, const double* time, double* omegak, double* omegak_new,
                       double* dt_omegak_old, double* dt_omegak_new) {
  (void)time; (void)omegak_new; (void)dt_omegak_old;
  const int nx = *Nx, ny = *Ny, nh = *Nh;
  const size_t ns = (size_t)nh * ny, nr = (size_t)nx * ny;
  const double pi = PI_R4, lx = g_css_lx, ly = g_css_ly, lambda = g_css_lambda; /* :18 */
  double* ukx = (double*)xcalloc(2 * ns, sizeof(double));
  double* uky = (double*)xcalloc(2 * ns, sizeof(double));
  double* wd = (double*)xcalloc(2 * ns, sizeof(double)); /* omegak_dum = k^2 psi */
  double* ikxw = (double*)xcalloc(2 * ns, sizeof(double));
  double* ikyw = (double*)xcalloc(2 * ns, sizeof(double));
  double* nlkx = (double*)xcalloc(2 * ns, sizeof(double));
  double* nlky = (double*)xcalloc(2 * ns, sizeof(double));
  double* ux = (double*)xcalloc(nr, sizeof(double));
  double* uy = (double*)xcalloc(nr, sizeof(double));
  double* dwx = (double*)xcalloc(nr, sizeof(double));
  double* dwy = (double*)xcalloc(nr, sizeof(double));
  double* p1 = (double*)xcalloc(nr, sizeof(double));
  double* p2 = (double*)xcalloc(nr, sizeof(double));

  /* :22-55 */
  for (int i = 0; i < nh; ++i) {
    const double kx = kx_of(i, pi, lx);
    for (int j = 0; j < ny; ++j) {
      const double ky = ky_of(j, ny, pi, ly);
      const size_t q = 2 * ((size_t)j * nh + i);
      double pr = 0.0, pim = 0.0;
      if (i == 0 && j == 0) {
        ukx[q] = ukx[q + 1] = uky[q] = uky[q + 1] = 0.0;
      } else {
        const double den = (kx * kx + ky * ky) + lambda;
        pr = omegak[q] / den;
        pim = omegak[q + 1] / den;
        ukx[q] = -ky * pim;
        ukx[q + 1] = ky * pr;
        uky[q] = kx * pim;
        uky[q + 1] = -(kx * pr);
      }
      const double k2 = kx * kx + ky * ky;
      const double dr = k2 * pr, di = k2 * pim;
      wd[q] = dr;
      wd[q + 1] = di;
      ikxw[q] = -kx * di;
      ikxw[q + 1] = kx * dr;
      ikyw[q] = -ky * di;
      ikyw[q + 1] = ky * dr;
    }
  }
  oracle_c2r_2d(nx, ny, ukx, ux); /* :57-71 */
  oracle_c2r_2d(nx, ny, uky, uy);
  oracle_c2r_2d(nx, ny, ikxw, dwx);
  oracle_c2r_2d(nx, ny, ikyw, dwy);
  const double nn = (double)nx * (double)ny; /* :73-82 */
  for (size_t r = 0; r < nr; ++r) {
    const double a = ux[r] / nn, b = uy[r] / nn, c = dwx[r] / nn, d = dwy[r] / nn;
    p1[r] = a * c;
    p2[r] = b * d;
  }
  oracle_r2c_2d(nx, ny, p1, nlkx); /* :84-90 */
  oracle_r2c_2d(nx, ny, p2, nlky);
  const double cut = ((double)(nx + ny) / 2.0) / 3.0 + 0; /* :92-111 */
  for (int i = 0; i < nh; ++i) {
    const double kx = kx_of(i, pi, lx);
    for (int j = 0; j < ny; ++j) {
      const double ky = ky_of(j, ny, pi, ly);
      const size_t q = 2 * ((size_t)j * nh + i);
      if (sqrt(kx * kx + ky * ky) >= cut) {
        nlkx[q] = nlkx[q + 1] = nlky[q] = nlky[q + 1] = 0.0;
      }
      /* NL = alpha (NLx + NLy) + nu k^2 omegak_dum; dt = -NL  (:113-132) */
      const double vk2 = *nu * (kx * kx + ky * ky);
      const double nr_ = *alpha * (nlkx[q] + nlky[q]) + vk2 * wd[q];
      const double ni_ = *alpha * (nlkx[q + 1] + nlky[q + 1]) + vk2 * wd[q + 1];
      dt_omegak_new[q] = -nr_;
      dt_omegak_new[q + 1] = -ni_;
    }
  }
  free(ukx); free(uky); free(wd); free(ikxw); free(ikyw); free(nlkx); free(nlky);
  free(ux); free(uy); free(dwx); free(dwy); free(p1); free(p2);
}

/* ------------------------------------------------------------------------- */
/* Classic RK4 (the R4 signature of src/rk42css.f95:6-13)                     */
/* ------------------------------------------------------------------------- */
/* Stage inputs omegak + k*dt/2.0 and the final omegak + dt/6*(k1+2k2+2k3+k4)
 * follow the expression forms of src/rk42css.f95:176,185,194,203; the stage
 * derivatives are the RHS outputs (the reference reads an uninitialised local
 * instead, which is why its body is not restated). */
typedef void (*rhs_fn)(int nx, int ny, int nh, double alpha, double nu, double* w, double* f);

static void rhs_plain(int nx, int ny, int nh, double alpha, double nu, double* w, double* f) {
  (void)alpha;
  const double t = 0.0;
  oracle_derive2csh(&nx, &ny, &nh, &nu, &t, w, NULL, NULL, f);
}

static void rhs_screen(int nx, int ny, int nh, double alpha, double nu, double* w, double* f) {
  const double t = 0.0;
  oracle_derive2css(&nx, &ny, &nh, &alpha, &nu, &t, w, NULL, NULL, f);
}

static void rk4_step(rhs_fn rhs, int nx, int ny, int nh, double alpha, double nu, double dt,
                     const double* w, double* wn) {
  const size_t n2 = 2 * (size_t)nh * ny;
  double* ys = (double*)xcalloc(n2, sizeof(double));
  double* k = (double*)xcalloc(n2, sizeof(double));
  double* s = (double*)xcalloc(n2, sizeof(double));
  memcpy(ys, w, n2 * sizeof(double));
  rhs(nx, ny, nh, alpha, nu, ys, k); /* k1 */
  for (size_t q = 0; q < n2; ++q) { s[q] = k[q]; ys[q] = w[q] + k[q] * dt / 2.0; }
  rhs(nx, ny, nh, alpha, nu, ys, k); /* k2 */
  for (size_t q = 0; q < n2; ++q) { s[q] = s[q] + 2.0 * k[q]; ys[q] = w[q] + k[q] * dt / 2.0; }
  rhs(nx, ny, nh, alpha, nu, ys, k); /* k3 */
  for (size_t q = 0; q < n2; ++q) { s[q] = s[q] + 2.0 * k[q]; ys[q] = w[q] + k[q] * dt; }
  rhs(nx, ny, nh, alpha, nu, ys, k); /* k4 */
  for (size_t q = 0; q < n2; ++q) wn[q] = w[q] + dt / 6.0 * (s[q] + k[q]);
  free(ys); free(k); free(s);
}

void oracle_rk42css(const int* Nx, const int* Ny, const int* Nh, const double* alpha,
                    const double* nu, const double* time, const double* dt, double* omegak,
                    double* omegak_new, double* dt_omegak_old, double* dt_omegak_new) {
  (void)time; (void)dt_omegak_old; (void)dt_omegak_new;
  rk4_step(rhs_screen, *Nx, *Ny, *Nh, *alpha, *nu, *dt, omegak, omegak_new);
}

void oracle_rk4csh(const int* Nx, const int* Ny, const int* Nh, const double* nu,
                   const double* time, const double* dt, double* omegak, double* omegak_new) {
  (void)time;
  rk4_step(rhs_plain, *Nx, *Ny, *Nh, 1.0, *nu, *dt, omegak, omegak_new);
}

/* Driver loop: derive, step, then the history rotation of
 * src/main2csh.f95:118-126 / src/main2css.f95:194-204. */
void oracle_run(int nx, int ny, int rhs_kind, int scheme, double alpha, double nu, double dt,
                int nsteps, double* omegak, double* dt_old) {
  const int nh = nx / 2 + 1;
  const size_t n2 = 2 * (size_t)nh * ny;
  double* wn = (double*)xcalloc(n2, sizeof(double));
  double* fn = (double*)xcalloc(n2, sizeof(double));
  rhs_fn rhs = rhs_kind ? rhs_screen : rhs_plain;
  for (int s = 0; s < nsteps; ++s) {
    if (scheme == 0) {
      rhs(nx, ny, nh, alpha, nu, omegak, fn);
      ab2_update(nh, ny, dt, omegak, wn, dt_old, fn);
      memcpy(dt_old, fn, n2 * sizeof(double));
      memcpy(omegak, wn, n2 * sizeof(double));
    } else {
      rk4_step(rhs, nx, ny, nh, alpha, nu, dt, omegak, wn);
      memcpy(omegak, wn, n2 * sizeof(double));
    }
  }
  free(wn); free(fn);
}

/* ------------------------------------------------------------------------- */
/* Initial conditions                                                         */
/* ------------------------------------------------------------------------- */
/* variant 0: src/main2css.f95:78-104 (x = 0.0d0+real(i-1)*dx with a default-real
 * real(), eps = 0.01 default real); variant 1: src/main2csh.f95:84-106
 * (x = (i-1)*dx, eps = 0.10d0).  x**2.0 is evaluated as x*x. */
void oracle_ic_shear(int nx, int ny, double lx_ini, double ly_ini, double w0, double m0,
                     double d_ini, int variant, double* omega) {
  const double pi = PI_R8;
  const double lx = lx_ini * pi, ly = ly_ini * pi;
  const double dx = lx / (double)nx, dy = ly / (double)ny;
  const double d = d_ini * pi;
  for (int i = 0; i < nx; ++i) {
    const double x = variant == 0 ? 0.0 + (double)(float)i * dx : (double)i * dx;
    for (int j = 0; j < ny; ++j) {
      const double y = variant == 0 ? (double)0.0f + (double)(float)j * dy : (double)j * dy;
      const double c1 = cosh((y + 0.5 * pi) / d), c2 = cosh((y - 0.5 * pi) / d);
      const double c3 = cosh((y + 1.5 * pi) / d), c4 = cosh((y - 1.5 * pi) / d);
      double w = w0 / (c1 * c1) - w0 / (c2 * c2);
      w = w - w0 / (c3 * c3) + w0 / (c4 * c4);
      const double eps = variant == 0 ? (double)0.01f : 0.10;
      w = w + eps * cos(m0 * x);
      omega[(size_t)j * nx + i] = w;
    }
  }
}

/* Philox4x32-10: ten rounds of the Philox-4x32 S-box with the published
 * multipliers and Weyl key increments. */
void oracle_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    c0 = hi1 ^ c1 ^ k0;
    c1 = lo1;
    c2 = hi0 ^ c3 ^ k1;
    c3 = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

static void spectral_energy_rescale(int nx, int ny, double energy, double* w);

void oracle_ic_random(int nx, int ny, double k0, double energy, uint64_t seed, double* omegak) {
  const int nh = nx / 2 + 1;
  const double two_pi = 2.0 * PI_R8;
  const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  for (int j = 0; j < ny; ++j) {
    const double ky = (j < ny / 2) ? (double)j : (double)(j - ny);
    for (int i = 0; i < nh; ++i) {
      const double kx = (double)i;
      const size_t q = 2 * ((size_t)j * nh + i);
      const double k = sqrt(kx * kx + ky * ky);
      if (i == 0 && j == 0) {
        omegak[q] = omegak[q + 1] = 0.0;
        continue;
      }
      const uint32_t ctr[4] = {(uint32_t)i, (uint32_t)j, 0u, 0u};
      uint32_t r[4];
      oracle_philox4x32_10(ctr, key, r);
      const double theta = two_pi * ((double)r[0] * (1.0 / 4294967296.0));
      const double ek = k * k * k * k * exp(-(k / k0) * (k / k0));
      const double amp = sqrt(k * ek / PI_R8);
      omegak[q] = amp * cos(theta);
      omegak[q + 1] = amp * sin(theta);
    }
  }
  /* Hermitian projection: c2r then r2c, divided by Nx*Ny */
  const size_t nr = (size_t)nx * ny;
  double* re = (double*)xcalloc(nr, sizeof(double));
  oracle_c2r_2d(nx, ny, omegak, re);
  oracle_r2c_2d(nx, ny, re, omegak);
  const double nn = (double)nx * (double)ny;
  for (size_t q = 0; q < 2 * (size_t)nh * ny; ++q) omegak[q] /= nn;
  omegak[0] = omegak[1] = 0.0; /* zero mean vorticity (round-off of the round trip) */
  free(re);
  spectral_energy_rescale(nx, ny, energy, omegak);
}

/* ------------------------------------------------------------------------- */
/* Diagnostics                                                                */
/* ------------------------------------------------------------------------- */
void oracle_energy_enstrophy(int nx, int ny, double lx, double ly, const double* omegak,
                             double* out) {
  const int nh = nx / 2 + 1;
  const size_t ns = (size_t)nh * ny, nr = (size_t)nx * ny;
  double* ukx = (double*)xcalloc(2 * ns, sizeof(double));
  double* uky = (double*)xcalloc(2 * ns, sizeof(double));
  double* ux = (double*)xcalloc(nr, sizeof(double));
  double* uy = (double*)xcalloc(nr, sizeof(double));
  double* om = (double*)xcalloc(nr, sizeof(double));
  const double pi = PI_R8;
  for (int i = 0; i < nh; ++i) {
    const double kx = kx_of(i, pi, lx);
    for (int j = 0; j < ny; ++j) {
      const double ky = ky_of(j, ny, pi, ly);
      const size_t q = 2 * ((size_t)j * nh + i);
      if (i == 0 && j == 0) continue;
      const double k2 = kx * kx + ky * ky;
      const double pr = omegak[q] / k2, pim = omegak[q + 1] / k2;
      ukx[q] = -ky * pim;
      ukx[q + 1] = ky * pr;
      uky[q] = kx * pim;
      uky[q + 1] = -(kx * pr);
    }
  }
  oracle_c2r_2d(nx, ny, ukx, ux);
  oracle_c2r_2d(nx, ny, uky, uy);
  oracle_c2r_2d(nx, ny, omegak, om);
  const double nn = (double)nx * (double)ny;
  double e = 0.0, z = 0.0;
  for (size_t r = 0; r < nr; ++r) {
    const double a = ux[r] / nn, b = uy[r] / nn, c = om[r] / nn;
    e += a * a + b * b;
    z += c * c;
  }
  out[0] = 0.5 * e / nn;
  out[1] = 0.5 * z / nn;
  free(ukx); free(uky); free(ux); free(uy); free(om);
}

static void spectral_energy_rescale(int nx, int ny, double energy, double* w) {
  double ez[2];
  oracle_energy_enstrophy(nx, ny, 2.0 * PI_R8, 2.0 * PI_R8, w, ez);
  const double s = ez[0] > 0.0 ? sqrt(energy / ez[0]) : 1.0;
  for (size_t q = 0; q < 2 * (size_t)(nx / 2 + 1) * ny; ++q) w[q] *= s;
}

/* src/main2css.f95:206-275 (summation order i outer, j inner, as the loops run) */
void oracle_diag_css(int nx, int ny, double lx, double ly, double lambda, const double* omegak,
                     double* out) {
  const int nh = nx / 2 + 1;
  const size_t ns = (size_t)nh * ny, nr = (size_t)nx * ny;
  double* wd = (double*)xcalloc(2 * ns, sizeof(double));
  double* ukx = (double*)xcalloc(2 * ns, sizeof(double));
  double* uky = (double*)xcalloc(2 * ns, sizeof(double));
  double* om = (double*)xcalloc(nr, sizeof(double));
  double* ux = (double*)xcalloc(nr, sizeof(double));
  double* uy = (double*)xcalloc(nr, sizeof(double));
  const double pi = PI_R8;
  for (int i = 0; i < nh; ++i) {
    const double kx = kx_of(i, pi, lx);
    for (int j = 0; j < ny; ++j) {
      const double ky = ky_of(j, ny, pi, ly);
      const size_t q = 2 * ((size_t)j * nh + i);
      double pr = 0.0, pim = 0.0;
      if (!(i == 0 && j == 0)) {
        /* lambda only on the j <= Ny/2 half (:215 vs :226) */
        const double den = (j < ny / 2) ? (kx * kx + ky * ky) + lambda : (kx * kx + ky * ky);
        pr = omegak[q] / den;
        pim = omegak[q + 1] / den;
      }
      ukx[q] = -ky * pim;
      ukx[q + 1] = ky * pr;
      uky[q] = kx * pim;
      uky[q + 1] = -(kx * pr);
      const double k2 = kx * kx + ky * ky;
      wd[q] = k2 * pr;
      wd[q + 1] = k2 * pim;
    }
  }
  oracle_c2r_2d(nx, ny, wd, om);
  oracle_c2r_2d(nx, ny, ukx, ux);
  oracle_c2r_2d(nx, ny, uky, uy);
  const double nn = (double)nx * (double)ny;
  double e = 0.0, ye = 0.0, c0 = 0.0, c1 = 0.0, c2 = 0.0, c3 = 0.0;
  for (int i = 0; i < nx; ++i) {
    for (int j = 0; j < ny; ++j) {
      const size_t r = (size_t)j * nx + i;
      const double o = om[r] / nn, a = ux[r] / nn, b = uy[r] / nn;
      e = e + (a * a + b * b);
      ye = ye + b * b;
      c0 = c0 + pow(o, 0.0);
      c1 = c1 + pow(o, 1.0);
      c2 = c2 + o * o;
      c3 = c3 + pow(o, 3.0);
    }
  }
  out[0] = e; out[1] = ye; out[2] = c0; out[3] = c1; out[4] = c2; out[5] = c3;
  free(wd); free(ukx); free(uky); free(om); free(ux); free(uy);
}
