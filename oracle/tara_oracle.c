/* CPU oracle for the TARA 2D pseudo-spectral path -- TEST INFRASTRUCTURE ONLY.
 *
 * Only the test suite, smoke() and the bench's CPU-baseline leg load this
 * library, and only as the oracle.  The product library never links it.
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
#include <stdio.h>
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
/* dfftw_plan_dft_{r2c,c2r}_3d_(plan, Nx, Ny, Nz, ...) -> dims (Nz, Ny, Nx) in C order */
void oracle_r2c_3d(int nx, int ny, int nz, const double* in, double* out) {
  fftw_plan p = fftw_plan_dft_r2c_3d(nz, ny, nx, (double*)in, (fftw_complex*)out, FFTW_ESTIMATE);
  fftw_execute(p);
  fftw_destroy_plan(p);
}

void oracle_c2r_3d(int nx, int ny, int nz, const double* in, double* out) {
  const size_t ns = (size_t)(nx / 2 + 1) * ny * nz;
  double* tmp = (double*)xcalloc(2 * ns, sizeof(double));
  memcpy(tmp, in, 2 * ns * sizeof(double));
  fftw_plan p = fftw_plan_dft_c2r_3d(nz, ny, nx, (fftw_complex*)tmp, out, FFTW_ESTIMATE);
  fftw_execute(p);
  fftw_destroy_plan(p);
  free(tmp);
}
#else
int oracle_backend_is_fftw(void) { return 0; }

/* Own FFT: iterative radix-2 decimation in time, twiddles from long-double
 * sin/cos rounded once.  Lengths that are not powers of two take a direct DFT
 * (O(n^2), same twiddle table over all n roots): the test sizes of the
 * mixed-radix GPU path are small. */
typedef struct {
  int n;
  double* w; /* w[2k] = cos(2 pi k/n), w[2k+1] = -sin(2 pi k/n), k < n/2 (k < n for a direct DFT) */
  int* rev;  /* NULL: direct DFT */
} fft_plan;

static fft_plan g_plans[32];
static fft_plan g_any_plans[64];

static fft_plan* get_plan(int n) {
  if (n & (n - 1)) { /* not a power of two */
    for (int i = 0; i < 64; ++i) {
      fft_plan* q = &g_any_plans[i];
      if (q->n == n) return q;
      if (q->n == 0) {
        q->w = (double*)xcalloc(2 * (size_t)n, sizeof(double));
        for (int k = 0; k < n; ++k) {
          long double a = 2.0L * 3.141592653589793238462643383279502884L * (long double)k / (long double)n;
          q->w[2 * k] = (double)cosl(a);
          q->w[2 * k + 1] = (double)-sinl(a);
        }
        q->rev = NULL;
        q->n = n;
        return q;
      }
    }
    fprintf(stderr, "oracle: too many transform lengths\n");
    abort();
  }
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
  if (!p->rev) { /* direct DFT: Z[k] = sum_j z[j] exp(sign 2 pi i j k / n) */
    double* t = (double*)xcalloc(2 * (size_t)n, sizeof(double));
    for (int k = 0; k < n; ++k) {
      double sr = 0.0, si = 0.0;
      for (int j = 0; j < n; ++j) {
        const int m = (int)(((long long)j * k) % n);
        const double wr = p->w[2 * m], wi = sign < 0 ? p->w[2 * m + 1] : -p->w[2 * m + 1];
        sr += z[2 * j] * wr - z[2 * j + 1] * wi;
        si += z[2 * j] * wi + z[2 * j + 1] * wr;
      }
      t[2 * k] = sr;
      t[2 * k + 1] = si;
    }
    memcpy(z, t, 2 * (size_t)n * sizeof(double));
    free(t);
    return;
  }
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
 * parts of the kx=0 bin and, for even Nx, the kx=Nx/2 bin (odd Nx has no
 * self-conjugate bin but kx=0).  Two rows share one complex transform. */
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
        const int edge = (k == 0 || 2 * k == nx); /* self-conjugate bins (Nyquist for even nx only) */
        const double ar = a[2 * k], ai = edge ? 0.0 : a[2 * k + 1];
        const double br = b ? b[2 * k] : 0.0, bi = (b && !edge) ? b[2 * k + 1] : 0.0;
        z[2 * k] = ar - bi; /* A + iB */
        z[2 * k + 1] = ai + br;
        if (!edge) {
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

/* strided complex transforms of all lines along one axis of a (nh, ny, nz) array */
static void lines_fft(double* a, int nlines_outer, int nlines_inner, size_t outer_stride,
                      size_t inner_stride, int n, size_t point_stride, int sign) {
  const fft_plan* p = get_plan(n);
#pragma omp parallel num_threads(oracle_get_threads())
  {
    double* col = (double*)xcalloc(2 * (size_t)n, sizeof(double));
#pragma omp for collapse(2) schedule(static)
    for (int o = 0; o < nlines_outer; ++o)
      for (int i = 0; i < nlines_inner; ++i) {
        double* base = a + 2 * ((size_t)o * outer_stride + (size_t)i * inner_stride);
        for (int q = 0; q < n; ++q) {
          col[2 * q] = base[2 * q * point_stride];
          col[2 * q + 1] = base[2 * q * point_stride + 1];
        }
        fft1d(col, n, sign, p);
        for (int q = 0; q < n; ++q) {
          base[2 * q * point_stride] = col[2 * q];
          base[2 * q * point_stride + 1] = col[2 * q + 1];
        }
      }
    free(col);
  }
}

/* rank-3 c2r: complex DFTs along z and y for all Nh columns, then the 1D c2r
 * along x reading only the real parts of the kx = 0 and kx = Nx/2 bins. */
void oracle_c2r_3d(int nx, int ny, int nz, const double* in, double* out) {
  const int nh = nx / 2 + 1;
  const size_t ns = (size_t)nh * ny * nz;
  double* tmp = (double*)xcalloc(2 * ns, sizeof(double));
  memcpy(tmp, in, 2 * ns * sizeof(double));
  lines_fft(tmp, ny, nh, nh, 1, nz, (size_t)nh * ny, +1);       /* z */
  lines_fft(tmp, nz, nh, (size_t)nh * ny, 1, ny, (size_t)nh, +1); /* y */
  /* x rows as pairs through the 2D row code: rows r = k*ny + j */
  const int rows = ny * nz;
  const fft_plan* px = get_plan(nx);
#pragma omp parallel num_threads(oracle_get_threads())
  {
    double* z = (double*)xcalloc(2 * (size_t)nx, sizeof(double));
#pragma omp for schedule(static)
    for (int r = 0; r < rows; r += 2) {
      const double* a = tmp + 2 * (size_t)r * nh;
      const double* b = (r + 1 < rows) ? tmp + 2 * (size_t)(r + 1) * nh : NULL;
      for (int k = 0; k <= nx / 2; ++k) {
        const int edge = (k == 0 || k == nx / 2);
        const double ar = a[2 * k], ai = edge ? 0.0 : a[2 * k + 1];
        const double br = b ? b[2 * k] : 0.0, bi = (b && !edge) ? b[2 * k + 1] : 0.0;
        z[2 * k] = ar - bi;
        z[2 * k + 1] = ai + br;
        if (k > 0 && k < nx / 2) {
          z[2 * (nx - k)] = ar + bi;
          z[2 * (nx - k) + 1] = -ai + br;
        }
      }
      fft1d(z, nx, +1, px);
      for (int x = 0; x < nx; ++x) {
        out[(size_t)r * nx + x] = z[2 * x];
        if (b) out[(size_t)(r + 1) * nx + x] = z[2 * x + 1];
      }
    }
    free(z);
  }
  free(tmp);
}

void oracle_r2c_3d(int nx, int ny, int nz, const double* in, double* out) {
  const int nh = nx / 2 + 1;
  const int rows = ny * nz;
  const fft_plan* px = get_plan(nx);
#pragma omp parallel num_threads(oracle_get_threads())
  {
    double* z = (double*)xcalloc(2 * (size_t)nx, sizeof(double));
#pragma omp for schedule(static)
    for (int r = 0; r < rows; r += 2) {
      const int two = (r + 1 < rows);
      for (int x = 0; x < nx; ++x) {
        z[2 * x] = in[(size_t)r * nx + x];
        z[2 * x + 1] = two ? in[(size_t)(r + 1) * nx + x] : 0.0;
      }
      fft1d(z, nx, -1, px);
      double* a = out + 2 * (size_t)r * nh;
      double* b = two ? out + 2 * (size_t)(r + 1) * nh : NULL;
      for (int k = 0; k <= nx / 2; ++k) {
        const int m = (nx - k) % nx;
        const double zr = z[2 * k], zi = z[2 * k + 1];
        const double mr = z[2 * m], mi = -z[2 * m + 1];
        a[2 * k] = 0.5 * (zr + mr);
        a[2 * k + 1] = 0.5 * (zi + mi);
        if (b) {
          b[2 * k] = 0.5 * (zi - mi);
          b[2 * k + 1] = -0.5 * (zr - mr);
        }
      }
    }
    free(z);
  }
  lines_fft(out, nz, nh, (size_t)nh * ny, 1, ny, (size_t)nh, -1); /* y */
  lines_fft(out, ny, nh, nh, 1, nz, (size_t)nh * ny, -1);         /* z */
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

/* ------------------------------------------------------------------------- */
/* 3D compressible MHD -- src/derive3com.f95, src/ab3com.f95                  */
/* ------------------------------------------------------------------------- */
enum { F_RHO = 0, F_RUX, F_RUY, F_RUZ, F_E, F_BX, F_BY, F_BZ, NF3 };

/* kx = 2.0d0*pi*dfloat(i-1)/Lx, ky/kz with (j-1)-Ny above Ny/2 (derive3com.f95:213-215) */
static double k3_of(int i0, int n, double pi, double l, int signed_) {
  if (!signed_ || i0 < n / 2) return 2.0 * pi * (double)i0 / l;
  return 2.0 * pi * (double)(i0 - n) / l;
}

/* src/main2csh.f95:128-172 */
void oracle_driver_velocity(int nx, int ny, double lx, double ly, const double* omegak, double* ux,
                            double* uy) {
  const double pi = 3.14159265358979323846;
  const int nh = nx / 2 + 1;
  double* a = (double*)calloc((size_t)2 * nh * ny, sizeof(double));
  double* b = (double*)calloc((size_t)2 * nh * ny, sizeof(double));
  for (int i = 0; i < nh; ++i) {
    const double kx = 2.0 * pi * (double)i / lx;
    for (int j = 0; j < ny; ++j) {
      const double ky = j < ny / 2 ? 2.0 * pi * (double)j / ly : 2.0 * pi * ((double)j - ny) / ly;
      const size_t q = (size_t)j * nh + i;
      if (i == 0 && j == 0) continue;
      const double k2 = kx * kx + ky * ky;
      const double pr = omegak[2 * q] / k2, pim = omegak[2 * q + 1] / k2;
      a[2 * q] = -ky * pim;  /* (0,1)*ky*psik */
      a[2 * q + 1] = ky * pr;
      b[2 * q] = kx * pim;   /* -(0,1)*kx*psik */
      b[2 * q + 1] = -(kx * pr);
    }
  }
  oracle_c2r_2d(nx, ny, a, ux);
  oracle_c2r_2d(nx, ny, b, uy);
  const double nn = (double)(nx * ny);
  for (size_t t = 0; t < (size_t)nx * ny; ++t) {
    ux[t] = ux[t] / nn;
    uy[t] = uy[t] / nn;
  }
  free(a);
  free(b);
}

/* src/main2csh.f95:187-271 (defined periodic neighbours at the last column/row) */
void oracle_particles_step(int nx, int ny, double lx, double ly, const double* ux, const double* uy,
                           int np, double* xp, double* yp, double dt) {
  const double dx = lx / (double)nx, dy = ly / (double)ny;
  const double h = 1.0 / (dx * dy);
  for (int i = 0; i < np; ++i) {
    const double x = xp[i], y = yp[i];
    int m = (int)(x / dx), n = (int)(y / dy); /* aint, 0-based */
    if (m > nx - 1) m = nx - 1;
    if (n > ny - 1) n = ny - 1;
    const int m1 = m + 1 < nx ? m + 1 : 0, n1 = n + 1 < ny ? n + 1 : 0;
    const double xm = (double)m * dx, xm1 = m + 1 < nx ? (double)(m + 1) * dx : lx;
    const double yn = (double)n * dy, yn1 = n + 1 < ny ? (double)(n + 1) * dy : ly;
    const double* f[2] = {ux, uy};
    double v[2];
    for (int c = 0; c < 2; ++c) {
      const double* u = f[c];
      v[c] = u[(size_t)n * nx + m] * (xm1 - x) * (yn1 - y) * h + u[(size_t)n * nx + m1] * (x - xm) * (yn1 - y) * h +
             u[(size_t)n1 * nx + m] * (xm1 - x) * (y - yn) * h + u[(size_t)n1 * nx + m1] * (x - xm) * (y - yn) * h;
    }
    double a = x + v[0] * dt, b = y + v[1] * dt;
    a = a - (double)(int)(a / lx) * lx;
    if (a <= 0.0) a = a + lx;
    b = b - (double)(int)(b / ly) * ly;
    if (b <= 0.0) b = b + ly;
    xp[i] = a;
    yp[i] = b;
  }
}

void oracle_derive3com(int nx, int ny, int nz, const oracle_mhd_params* p, const double* state,
                       double* dstate) {
  const int nh = nx / 2 + 1;
  const size_t ns = (size_t)nh * ny * nz, nr = (size_t)nx * ny * nz;
  const double pi = PI_R8;
  const double nn = (double)nx * (double)ny * (double)nz;
  const double* sk[NF3];
  for (int f = 0; f < NF3; ++f) sk[f] = state + 2 * ns * f;
  /* eight c2r of the state (:73-135), normalised (:147-159) */
  double* rl[NF3];
  for (int f = 0; f < NF3; ++f) {
    rl[f] = (double*)xcalloc(nr, sizeof(double));
    oracle_c2r_3d(nx, ny, nz, sk[f], rl[f]);
    for (size_t r = 0; r < nr; ++r) rl[f][r] = rl[f][r] / nn;
  }
  double *ux = (double*)xcalloc(nr, sizeof(double)), *uy = (double*)xcalloc(nr, sizeof(double)),
         *uz = (double*)xcalloc(nr, sizeof(double)), *b2 = (double*)xcalloc(nr, sizeof(double));
  for (size_t r = 0; r < nr; ++r) { /* :162-175 */
    const double rho = rl[F_RHO][r];
    ux[r] = rl[F_RUX][r] / rho;
    uy[r] = rl[F_RUY][r] / rho;
    uz[r] = rl[F_RUZ][r] / rho;
    b2[r] = rl[F_BX][r] * rl[F_BX][r] + rl[F_BY][r] * rl[F_BY][r] + rl[F_BZ][r] * rl[F_BZ][r];
  }
  /* velocity spectra (:201-217) */
  double* uk[3];
  double* ur[3] = {ux, uy, uz};
  for (int c = 0; c < 3; ++c) {
    uk[c] = (double*)xcalloc(2 * ns, sizeof(double));
    oracle_r2c_3d(nx, ny, nz, ur[c], uk[c]);
  }
  /* first derivatives (:224-298): i kx ux, i ky uy, i kz uz, i ky Bx, i kz Bx,
   * i kx By, i kz By, i kx Bz, i ky Bz */
  enum { D_UXX, D_UYY, D_UZZ, D_BXY, D_BXZ, D_BYX, D_BYZ, D_BZX, D_BZY, ND };
  double* dk[ND];
  for (int d = 0; d < ND; ++d) dk[d] = (double*)xcalloc(2 * ns, sizeof(double));
  for (int k = 0; k < nz; ++k) {
    const double kz = k3_of(k, nz, pi, p->lz, 1);
    for (int j = 0; j < ny; ++j) {
      const double ky = k3_of(j, ny, pi, p->ly, 1);
      for (int i = 0; i < nh; ++i) {
        const double kx = k3_of(i, nx, pi, p->lx, 0);
        const size_t q = 2 * (((size_t)k * ny + j) * nh + i);
#define IK(dst, kk, src) do { dk[dst][q] = -(kk) * (src)[q + 1]; dk[dst][q + 1] = (kk) * (src)[q]; } while (0)
        IK(D_UXX, kx, uk[0]); IK(D_UYY, ky, uk[1]); IK(D_UZZ, kz, uk[2]);
        IK(D_BXY, ky, sk[F_BX]); IK(D_BXZ, kz, sk[F_BX]);
        IK(D_BYX, kx, sk[F_BY]); IK(D_BYZ, kz, sk[F_BY]);
        IK(D_BZX, kx, sk[F_BZ]); IK(D_BZY, ky, sk[F_BZ]);
#undef IK
      }
    }
  }
  double* dr[ND];
  for (int d = 0; d < ND; ++d) {
    dr[d] = (double*)xcalloc(nr, sizeof(double));
    oracle_c2r_3d(nx, ny, nz, dk[d], dr[d]); /* :300-352 */
    for (size_t r = 0; r < nr; ++r) dr[d][r] = dr[d][r] / nn;
  }
  /* fluxes (:363-436) */
  enum { M_X1, M_X2, M_X3, M_Y1, M_Y2, M_Y3, M_Z1, M_Z2, M_Z3, EN_X, EN_Y, EN_Z, E_VISC,
         MG_X1, MG_X2, MG_Y1, MG_Y2, MG_Z1, MG_Z2, NFL };
  double* fl[NFL];
  for (int f = 0; f < NFL; ++f) fl[f] = (double*)xcalloc(nr, sizeof(double));
  const double eta = p->eta, cs = p->cs;
  for (size_t r = 0; r < nr; ++r) {
    const double rho = rl[F_RHO][r], rux = rl[F_RUX][r], ruy = rl[F_RUY][r], ruz = rl[F_RUZ][r];
    const double E = rl[F_E][r], bx = rl[F_BX][r], by = rl[F_BY][r], bz = rl[F_BZ][r];
    const double vx = ux[r], vy = uy[r], vz = uz[r], B2 = b2[r];
    const double cx = dr[D_BZY][r] - dr[D_BYZ][r]; /* curl_x_B */
    const double cy = dr[D_BZX][r] - dr[D_BXZ][r]; /* curl_y_B as the reference defines it */
    const double cz = dr[D_BYX][r] - dr[D_BXY][r]; /* curl_z_B */
    const double P = cs * cs * rho;
    fl[M_X1][r] = rux * vx + P + B2 / 2.0 - bx * bx;
    fl[M_X2][r] = rux * vy - bx * by;
    fl[M_X3][r] = rux * vz - bx * bz;
    fl[M_Y1][r] = rux * vy - bx * by;
    fl[M_Y2][r] = ruy * vy + P + B2 / 2.0 - by * by;
    fl[M_Y3][r] = ruy * vz - by * bz;
    fl[M_Z1][r] = ruz * vx - bz * bx;
    fl[M_Z2][r] = ruz * vy - bz * by;
    fl[M_Z3][r] = ruz * vz + P + B2 / 2.0 - bz * bz;
    fl[EN_X][r] = (E + P + B2 / 2.0) * vx - vx * bx * bx - vy * bx * by - vz * bx * bz -
                  eta * (by * cz + bz * cy);
    fl[EN_Y][r] = (E + P + B2 / 2.0) * vy - vx * bx * by - vy * by * by - vz * by * bz +
                  eta * (bx * cz - bz * cx);
    fl[EN_Z][r] = (E + P + B2 / 2.0) * vz - vx * bz * bx - vy * bz * by - vz * bz * bz +
                  eta * (bx * cy + by * cx);
    const double dv = dr[D_UXX][r] + dr[D_UYY][r] + dr[D_UZZ][r];
    fl[E_VISC][r] = dv * dv;
    fl[MG_X1][r] = vx * by - vy * bx;
    fl[MG_X2][r] = vx * bz - vz * bx;
    fl[MG_Y1][r] = vx * by - vy * bx;
    fl[MG_Y2][r] = vy * bz - vz * by;
    fl[MG_Z1][r] = vx * bz - vz * bx;
    fl[MG_Z2][r] = vy * bz - vz * by;
  }
  double* fk[NFL];
  for (int f = 0; f < NFL; ++f) {
    fk[f] = (double*)xcalloc(2 * ns, sizeof(double));
    oracle_r2c_3d(nx, ny, nz, fl[f], fk[f]); /* :444-556 */
  }
  /* spectral derivatives, the |k| >= (Nx+Ny+Nz)/9 sphere and the assembly
   * (:561-1043) */
  const double cut = ((double)(nx + ny + nz) / 3.0) / 3.0 + 0;
  for (int k = 0; k < nz; ++k) {
    const double kz = k3_of(k, nz, pi, p->lz, 1);
    for (int j = 0; j < ny; ++j) {
      const double ky = k3_of(j, ny, pi, p->ly, 1);
      for (int i = 0; i < nh; ++i) {
        const double kx = k3_of(i, nx, pi, p->lx, 0);
        const size_t q = 2 * (((size_t)k * ny + j) * nh + i);
        const int keep = !(sqrt(kx * kx + ky * ky + kz * kz) >= cut);
        double out[NF3][2];
        for (int c = 0; c < 2; ++c) { /* c = 0 real part, 1 imaginary part */
          /* i k f: real = -k*Im f, imag = k*Re f */
#define IKC(kk, f) ((c == 0) ? -(kk) * (f)[q + 1] : (kk) * (f)[q])
#define K2(kk, f) ((kk) * (kk) * (f)[q + c])
          if (!keep) {
            for (int f = 0; f < NF3; ++f) out[f][c] = 0.0;
            continue;
          }
          const double drho = -(IKC(kx, sk[F_RUX]) + IKC(ky, sk[F_RUY]) + IKC(kz, sk[F_RUZ]));
          const double lux = K2(kx, uk[0]) + K2(ky, uk[0]) + K2(kz, uk[0]);
          const double luy = K2(kx, uk[1]) + K2(ky, uk[1]) + K2(kz, uk[1]);
          const double luz = K2(kx, uk[2]) + K2(ky, uk[2]) + K2(kz, uk[2]);
          const double lbx = K2(kx, sk[F_BX]) + K2(ky, sk[F_BX]) + K2(kz, sk[F_BX]);
          const double lby = K2(kx, sk[F_BY]) + K2(ky, sk[F_BY]) + K2(kz, sk[F_BY]);
          const double lbz = K2(kx, sk[F_BZ]) + K2(ky, sk[F_BZ]) + K2(kz, sk[F_BZ]);
          const double vux = p->defined ? p->nu_u * lux : lux / 450.0;
          const double vuy = p->defined ? p->nu_u * luy : luy / 450.0;
          const double vuz = p->defined ? p->nu_u * luz : luz / 450.0;
          const double vbx = p->defined ? p->eta_b * lbx : lbx / 450.0;
          const double vby = p->defined ? p->eta_b * lby : lby / 450.0;
          const double vbz = p->defined ? p->eta_b * lbz : lbz / 450.0;
          out[F_RHO][c] = drho;
          out[F_RUX][c] = -(IKC(kx, fk[M_X1]) + IKC(ky, fk[M_X2]) + IKC(kz, fk[M_X3])) - vux;
          out[F_RUY][c] = -(IKC(kx, fk[M_Y1]) + IKC(ky, fk[M_Y2]) + IKC(kz, fk[M_Y3])) - vuy;
          out[F_RUZ][c] = -(IKC(kx, fk[M_Z1]) + IKC(ky, fk[M_Z2]) + IKC(kz, fk[M_Z3])) - vuz;
          out[F_E][c] = -(IKC(kx, fk[EN_X]) + IKC(ky, fk[EN_Y]) + IKC(kz, fk[EN_Z])) +
                        p->mu * fk[E_VISC][q + c];
          out[F_BX][c] = +(IKC(ky, fk[MG_X1]) + IKC(kz, fk[MG_X2])) - vbx;
          out[F_BY][c] = -(IKC(kx, fk[MG_Y1]) - IKC(kz, fk[MG_Y2])) - vby;
          out[F_BZ][c] = -(IKC(kx, fk[MG_Z1]) + IKC(ky, fk[MG_Z2])) - vbz;
#undef IKC
#undef K2
        }
        for (int f = 0; f < NF3; ++f) {
          dstate[2 * ns * f + q] = out[f][0];
          dstate[2 * ns * f + q + 1] = out[f][1];
        }
      }
    }
  }
  for (int f = 0; f < NF3; ++f) free(rl[f]);
  free(ux); free(uy); free(uz); free(b2);
  for (int c = 0; c < 3; ++c) free(uk[c]);
  for (int d = 0; d < ND; ++d) { free(dk[d]); free(dr[d]); }
  for (int f = 0; f < NFL; ++f) { free(fl[f]); free(fk[f]); }
}

void oracle_ab3com(int nx, int ny, int nz, double dt, const double* state, double* state_new,
                   const double* d_old, const double* d_new) {
  const size_t n2 = 2 * (size_t)(nx / 2 + 1) * ny * nz;
  for (int f = 0; f < NF3; ++f) {
    const size_t o = n2 * f;
    for (size_t q = 0; q < n2; ++q)
      state_new[o + q] = (f == F_E) ? state[o + q] /* E_k_new = E_k (:51) */
                                    : state[o + q] + ((3.0 / 2.0) * d_new[o + q] -
                                                      (1.0 / 2.0) * d_old[o + q]) * dt;
  }
}

void oracle_run3d(int nx, int ny, int nz, const oracle_mhd_params* p, double dt, int nsteps,
                  double* state, double* hist) {
  const size_t n = 2 * (size_t)(nx / 2 + 1) * ny * nz * NF3;
  double* dn = (double*)xcalloc(n, sizeof(double));
  double* sn = (double*)xcalloc(n, sizeof(double));
  for (int s = 0; s < nsteps; ++s) {
    oracle_derive3com(nx, ny, nz, p, state, dn);
    oracle_ab3com(nx, ny, nz, dt, state, sn, hist, dn);
    memcpy(hist, dn, n * sizeof(double));
    memcpy(state, sn, n * sizeof(double));
  }
  free(dn); free(sn);
}

/* src/main3com.f95:202-347 with U0 = 0.1, A = B = C = kf = 1, B0 = 0.1, P0 = 1 */
void oracle_ic3d_abc(int nx, int ny, int nz, double lx_ini, double ly_ini, double lz_ini,
                     double* real8) {
  const double pi = PI_R8;
  const double lx = lx_ini * pi, ly = ly_ini * pi, lz = lz_ini * pi;
  const double dx = lx / (double)nx, dy = ly / (double)ny, dz = lz / (double)nz;
  const double U0 = 0.10, A = 1.0, B = 1.0, C = 1.0, kf = 1.0, M = 0.10, MA = 1.0;
  const double rho0 = 1.0, P0 = 1.0, mu_0 = 1.0;
  (void)M;
  const double VA = U0 / MA, B0 = VA * sqrt(mu_0 * rho0);
  const size_t nr = (size_t)nx * ny * nz;
  for (int i = 0; i < nx; ++i) {
    const double x = 0.0 + (double)(float)i * dx;
    for (int j = 0; j < ny; ++j) {
      const double y = 0.0 + (double)(float)j * dy;
      for (int k = 0; k < nz; ++k) {
        const double z = 0.0 + (double)(float)k * dz;
        const size_t r = ((size_t)k * ny + j) * nx + i;
        const double rho = rho0;
        const double vx = U0 * (A * sin(kf * z) + C * cos(kf * y));
        const double vy = U0 * (B * sin(kf * x) + A * cos(kf * z));
        const double vz = U0 * (C * sin(kf * y) + B * cos(kf * x));
        const double P = P0, bx = B0, by = B0, bz = B0;
        const double E = P + 0.50 * rho * (vx * vx + vy * vy + vz * vz) +
                         0.50 * (bx * bx + by * by + bz * bz);
        real8[nr * F_RHO + r] = rho;
        real8[nr * F_RUX + r] = rho * vx;
        real8[nr * F_RUY + r] = rho * vy;
        real8[nr * F_RUZ + r] = rho * vz;
        real8[nr * F_E + r] = E;
        real8[nr * F_BX + r] = bx;
        real8[nr * F_BY + r] = by;
        real8[nr * F_BZ + r] = bz;
      }
    }
  }
}

/* The 3D MHD benchmark's initial state (the library's tara3d_init_orszag_tang;
 * no counterpart in the reference, whose 3D driver starts from the ABC flow
 * above): rho = 1, u = (-sin y, sin x, 0) + du, B = (-sin y, sin 2x, 0) + dB,
 * E = 1 + |u|^2/2 + |B|^2/2 on the 2 pi grid.  du, dB: for every mode
 * 0 < |k|^2 <= kmax^2 of the half space (the kx = 0 plane only where ky > 0,
 * or ky = 0 and kz > 0; the other half is the conjugate) and component c,
 * phase 2 pi U (U from word 0 of Philox4x32-10 at counter (i, j, k, 3 f + c),
 * f = 0 for u and 1 for B, key = seed), projected onto k.a = 0 and scaled so
 * that sum_c <f_c^2> = amp^2 (the base fields' r.m.s. is 1).  Writes the
 * spectral state (8, Nz, Ny, Nh) in the unnormalised r2c convention: u and B
 * spectra through c2r (divided by Nx Ny Nz), E and rho formed on the grid, then
 * r2c of all eight fields. */
void oracle_ic3d_ot(int nx, int ny, int nz, double amp, int kmax, uint64_t seed, double* state) {
  const int nh = nx / 2 + 1;
  const size_t fs = (size_t)nh * ny * nz, nr = (size_t)nx * ny * nz;
  const double nn = (double)nx * (double)ny * (double)nz;
  const double two_pi = 2.0 * PI_R8;
  const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  double* spec = (double*)xcalloc(2 * 6 * fs, sizeof(double));
  for (int f = 0; f < 2; ++f) {
    double* P = spec + 2 * 3 * f * fs;
    double norm2 = 0.0;
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nh; ++i) {
          const int kxi = i, kyi = j <= ny / 2 ? j : j - ny, kzi = k <= nz / 2 ? k : k - nz;
          const int k2i = kxi * kxi + kyi * kyi + kzi * kzi;
          if (k2i == 0 || k2i > kmax * kmax) continue;
          if (i == 0 && (kyi < 0 || (kyi == 0 && kzi < 0))) continue;
          double ar[3], ai[3];
          for (int c = 0; c < 3; ++c) {
            const uint32_t ctr[4] = {(uint32_t)i, (uint32_t)j, (uint32_t)k, (uint32_t)(3 * f + c)};
            uint32_t r[4];
            oracle_philox4x32_10(ctr, key, r);
            const double theta = two_pi * ((double)r[0] * (1.0 / 4294967296.0));
            ar[c] = cos(theta);
            ai[c] = sin(theta);
          }
          const double kv[3] = {(double)kxi, (double)kyi, (double)kzi};
          const double k2 = (double)k2i;
          const double dr = (kv[0] * ar[0] + kv[1] * ar[1] + kv[2] * ar[2]) / k2;
          const double di = (kv[0] * ai[0] + kv[1] * ai[1] + kv[2] * ai[2]) / k2;
          for (int c = 0; c < 3; ++c) {
            const double pr = ar[c] - kv[c] * dr, pim = ai[c] - kv[c] * di;
            const size_t q = c * fs + ((size_t)k * ny + j) * nh + i;
            P[2 * q] = pr;
            P[2 * q + 1] = pim;
            if (i == 0) {
              const int jm = (ny - j) % ny, km = (nz - k) % nz;
              const size_t qm = c * fs + ((size_t)km * ny + jm) * nh;
              P[2 * qm] = pr;
              P[2 * qm + 1] = -pim;
            }
            norm2 += 2.0 * (pr * pr + pim * pim);
          }
        }
    const double sc = norm2 > 0.0 ? amp * nn / sqrt(norm2) : 0.0;
    for (size_t q = 0; q < 2 * 3 * fs; ++q) P[q] *= sc;
    const double h = 0.5 * nn;
    P[2 * ((size_t)1 * nh) + 1] += h;                 /* -sin y: F(0, 1, 0) = +i N/2 */
    P[2 * ((size_t)(ny - 1) * nh) + 1] -= h;          /*         F(0, -1, 0) = -i N/2 */
    P[2 * (fs + (size_t)(f == 0 ? 1 : 2)) + 1] -= h;  /* sin(m x): F(m, 0, 0) = -i N/2 */
  }
  double* real = (double*)xcalloc(8 * nr, sizeof(double));
  const int slot[6] = {F_RUX, F_RUY, F_RUZ, F_BX, F_BY, F_BZ};
  for (int f = 0; f < 6; ++f) {
    oracle_c2r_3d(nx, ny, nz, spec + 2 * f * fs, real + slot[f] * nr);
    for (size_t r = 0; r < nr; ++r) real[slot[f] * nr + r] *= 1.0 / nn;
  }
  for (size_t r = 0; r < nr; ++r) {
    const double ux = real[F_RUX * nr + r], uy = real[F_RUY * nr + r], uz = real[F_RUZ * nr + r];
    const double bx = real[F_BX * nr + r], by = real[F_BY * nr + r], bz = real[F_BZ * nr + r];
    const double u2 = (ux * ux + uy * uy) + uz * uz, b2 = (bx * bx + by * by) + bz * bz;
    real[F_RHO * nr + r] = 1.0;
    real[F_E * nr + r] = (1.0 + 0.5 * u2) + 0.5 * b2;
  }
  for (int f = 0; f < 8; ++f) oracle_r2c_3d(nx, ny, nz, real + f * nr, state + 2 * f * fs);
  free(real);
  free(spec);
}

/* ------------------------------------------------------------------------- */
/* derive2coh -- src/derive2coh.f95:6-265                                     */
/* ------------------------------------------------------------------------- */
void oracle_derive2coh(int nx, int ny, const oracle_coh_params* p, const double* state,
                       double* dstate) {
  const int nh = nx / 2 + 1;
  const size_t ns = (size_t)nh * ny, nr = (size_t)nx * ny;
  const double* nk = state;
  const double* ukx = state + 2 * ns;
  const double* uky = state + 4 * ns;
  /* 13 spectra in the order of the c2r calls (:95-132): nk, ukx, uky, i kx nk,
   * i ky nk, i kx ukx, i ky ukx, i kx uky, i ky uky, kx^2 ukx, ky^2 ukx,
   * kx^2 uky, ky^2 uky */
  double* sp = (double*)xcalloc(13 * 2 * ns, sizeof(double));
  double* re = (double*)xcalloc(13 * nr, sizeof(double));
  double* pr = (double*)xcalloc(9 * nr, sizeof(double));  /* Px Py Vxx Vxy Vyx Vyy NLn NLx NLy */
  double* pk = (double*)xcalloc(9 * 2 * ns, sizeof(double));
  for (int i = 0; i < nh; ++i) {
    const double kx = kx_of(i, p->pi, p->lx);
    for (int j = 0; j < ny; ++j) {
      const double ky = ky_of(j, ny, p->pi, p->ly);
      const size_t q = 2 * ((size_t)j * nh + i);
      const double a[3][2] = {{nk[q], nk[q + 1]}, {ukx[q], ukx[q + 1]}, {uky[q], uky[q + 1]}};
      double* o = sp + q;
#define SET(f, r_, i_) (o[2 * ns * (f)] = (r_), o[2 * ns * (f) + 1] = (i_))
      SET(0, a[0][0], a[0][1]);
      SET(1, a[1][0], a[1][1]);
      SET(2, a[2][0], a[2][1]);
      /* (0,1)*k*f = (-k Im f, k Re f) (:57-82) */
      SET(3, -kx * a[0][1], kx * a[0][0]);
      SET(4, -ky * a[0][1], ky * a[0][0]);
      SET(5, -kx * a[1][1], kx * a[1][0]);
      SET(6, -ky * a[1][1], ky * a[1][0]);
      SET(7, -kx * a[2][1], kx * a[2][0]);
      SET(8, -ky * a[2][1], ky * a[2][0]);
      /* kx*kx*f (:66-69) */
      SET(9, kx * kx * a[1][0], kx * kx * a[1][1]);
      SET(10, ky * ky * a[1][0], ky * ky * a[1][1]);
      SET(11, kx * kx * a[2][0], kx * kx * a[2][1]);
      SET(12, ky * ky * a[2][0], ky * ky * a[2][1]);
#undef SET
    }
  }
  for (int f = 0; f < 13; ++f) oracle_c2r_2d(nx, ny, sp + 2 * ns * f, re + nr * f); /* :95-132 */
  const double nn = (double)nx * (double)ny;
  for (size_t r = 0; r < nr; ++r) { /* :140-169 */
    double v[13];
    for (int f = 0; f < 13; ++f) v[f] = re[nr * f + r] / nn;
    const double n = v[0], ux = v[1], uy = v[2], dn_dx = v[3], dn_dy = v[4], dux_dx = v[5],
                 dux_dy = v[6], duy_dx = v[7], duy_dy = v[8];
    pr[0 * nr + r] = dn_dx / n;  /* Px */
    pr[1 * nr + r] = dn_dy / n;  /* Py */
    pr[2 * nr + r] = v[9] / n;   /* Viscxx */
    pr[3 * nr + r] = v[10] / n;  /* Viscxy */
    pr[4 * nr + r] = v[11] / n;  /* Viscyx */
    pr[5 * nr + r] = v[12] / n;  /* Viscyy */
    pr[6 * nr + r] = ux * dn_dx + uy * dn_dy + n * (dux_dx + duy_dy); /* NLn */
    pr[7 * nr + r] = ux * dux_dx + uy * dux_dy;                        /* NLx */
    pr[8 * nr + r] = ux * duy_dx + uy * duy_dy;                        /* NLy */
  }
  for (int f = 0; f < 9; ++f) oracle_r2c_2d(nx, ny, pr + nr * f, pk + 2 * ns * f); /* :173-198 */
  const double cut = ((double)(nx + ny) / 2.0) / 3.0;
  const double cs2 = p->cs * p->cs;
  double* dn = dstate;
  double* dux = dstate + 2 * ns;
  double* duy = dstate + 4 * ns;
  for (int i = 0; i < nh; ++i) {
    const double kx = kx_of(i, p->pi, p->lx);
    for (int j = 0; j < ny; ++j) {
      const double ky = ky_of(j, ny, p->pi, p->ly);
      const size_t q = 2 * ((size_t)j * nh + i);
      if (sqrt(kx * kx + ky * ky) >= cut) { /* :205-242: all nine spectra */
        for (int f = 0; f < 9; ++f) pk[2 * ns * f + q] = pk[2 * ns * f + q + 1] = 0.0;
      }
      for (int c = 0; c < 2; ++c) { /* :249-256 */
        const double Pkx = pk[0 * 2 * ns + q + c], Pky = pk[1 * 2 * ns + q + c];
        const double Vxx = pk[2 * 2 * ns + q + c], Vxy = pk[3 * 2 * ns + q + c];
        const double Vyx = pk[4 * 2 * ns + q + c], Vyy = pk[5 * 2 * ns + q + c];
        const double NLkn = pk[6 * 2 * ns + q + c];
        const double NLkx = pk[7 * 2 * ns + q + c] + (p->mux * Vxx + p->muy * Vxy) + cs2 * Pkx;
        const double NLky = pk[8 * 2 * ns + q + c] + (p->mux * Vyx + p->muy * Vyy) + cs2 * Pky;
        dn[q + c] = -NLkn;
        dux[q + c] = -NLkx;
        duy[q + c] = -NLky;
      }
    }
  }
  free(sp); free(re); free(pr); free(pk);
}

/* ab2coh -- src/ab2coh.f95:19-27 */
void oracle_ab2coh(int nx, int ny, double dt, const double* state, double* state_new,
                   const double* d_old, const double* d_new) {
  const int nh = nx / 2 + 1;
  const size_t n2 = 2 * (size_t)nh * ny;
  for (int f = 0; f < 3; ++f)
    ab2_update(nh, ny, dt, state + f * n2, state_new + f * n2, d_old + f * n2, d_new + f * n2);
}

void oracle_run_coh(int nx, int ny, const oracle_coh_params* p, double dt, int nsteps,
                    double* state, double* hist) {
  const int nh = nx / 2 + 1;
  const size_t n6 = 6 * (size_t)nh * ny;
  double* sn = (double*)xcalloc(n6, sizeof(double));
  double* dn = (double*)xcalloc(n6, sizeof(double));
  for (int s = 0; s < nsteps; ++s) {
    oracle_derive2coh(nx, ny, p, state, dn);
    oracle_ab2coh(nx, ny, dt, state, sn, hist, dn);
    memcpy(hist, dn, n6 * sizeof(double));
    memcpy(state, sn, n6 * sizeof(double));
  }
  free(sn); free(dn);
}

/* src/main2coh.f95:140-210 */
void oracle_ic_coh(int nx, int ny, double lx_ini, double ly_ini, double* state) {
  const double pi = PI_R8;
  const double lx = lx_ini * pi, ly = ly_ini * pi;
  const double dx = lx / (double)nx, dy = ly / (double)ny;
  const double n0 = 1.0, d = 0.40 * 2.0 * pi, rb = 0.30 * 2.0 * pi;
  const int pvn = 5;
  const double theta = 2.0 * pi / (double)pvn;
  const int nh = nx / 2 + 1;
  const size_t ns = (size_t)nh * ny, nr = (size_t)nx * ny;
  double* n = (double*)xcalloc(nr, sizeof(double));
  double* w = (double*)xcalloc(nr, sizeof(double));
  double* wk = (double*)xcalloc(2 * ns, sizeof(double));
  for (int i = 0; i < nx; ++i) {
    const double x = (double)(float)(i) * dx; /* 0.0d0+real(i-1)*dx */
    for (int j = 0; j < ny; ++j) {
      const double y = (double)(float)(j) * dy;
      const size_t r = (size_t)j * nx + i;
      n[r] = n0;
      const double ax = x - lx / 2.0, ay = y - ly / 2.0;
      w[r] = (ax * ax + ay * ay <= rb * rb) ? 1.0 : 0.0;
      for (int pv = 1; pv <= pvn; ++pv) {
        const int npv = -pv;
        const double bx = x - (lx / 2.0 + d * cos(npv * theta));
        const double by = y - (ly / 2.0 + d * sin(npv * theta));
        if (bx * bx + by * by <= 0.20 * 0.20) w[r] = 10.0;
      }
    }
  }
  double* nk = state;
  double* ukx = state + 2 * ns;
  double* uky = state + 4 * ns;
  oracle_r2c_2d(nx, ny, n, nk);
  oracle_r2c_2d(nx, ny, w, wk);
  for (int i = 0; i < nh; ++i) {
    const double kx = kx_of(i, pi, lx);
    for (int j = 0; j < ny; ++j) {
      const double ky = ky_of(j, ny, pi, ly);
      const size_t q = 2 * ((size_t)j * nh + i);
      if (i == 0 && j == 0) {
        ukx[q] = ukx[q + 1] = uky[q] = uky[q + 1] = 0.0;
      } else {
        const double k2 = kx * kx + ky * ky;
        const double pr = wk[q] / k2, pim = wk[q + 1] / k2;
        ukx[q] = -ky * pim; /* + (0,1) ky psi */
        ukx[q + 1] = ky * pr;
        uky[q] = kx * pim;  /* - (0,1) kx psi */
        uky[q + 1] = -(kx * pr);
      }
    }
  }
  free(n); free(w); free(wk);
}

/* ------------------------------------------------------------------------- */
/* derive2com -- src/derive2com.f95:5-426                                     */
/* ------------------------------------------------------------------------- */
void oracle_derive2com(int nx, int ny, const oracle_com_params* p, const double* state,
                       double* dstate) {
  const int nh = nx / 2 + 1;
  const size_t ns = (size_t)nh * ny, nr = (size_t)nx * ny, s2 = 2 * ns;
  const double* rho_ux_k = state + s2;
  const double* rho_uy_k = state + 2 * s2;
  const double* Bx_k = state + 4 * s2;
  const double* By_k = state + 5 * s2;
  double* re = (double*)xcalloc(6 * nr, sizeof(double));  /* rho rho_ux rho_uy E Bx By */
  double* vel = (double*)xcalloc(4 * nr, sizeof(double)); /* ux uy Fx Fy */
  double* vk = (double*)xcalloc(4 * s2, sizeof(double));  /* ux_k uy_k Fx_k Fy_k */
  double* dk = (double*)xcalloc(4 * s2, sizeof(double));  /* i kx ux, i ky uy, i ky Bx, i kx By */
  double* dr = (double*)xcalloc(4 * nr, sizeof(double));
  double* tr = (double*)xcalloc(9 * nr, sizeof(double));  /* the nine flux fields */
  double* tk = (double*)xcalloc(9 * s2, sizeof(double));
  for (int f = 0; f < 6; ++f) oracle_c2r_2d(nx, ny, state + f * s2, re + f * nr); /* :68-84 */
  const double nn = (double)nx * (double)ny;
  const double dx = p->lx / (double)nx, dy = p->ly / (double)ny;
  for (int j = 0; j < ny; ++j) {
    const double y = (double)(float)j * dy;
    for (int i = 0; i < nx; ++i) {
      const double x = (double)(float)i * dx;
      const size_t r = (size_t)j * nx + i;
      for (int f = 0; f < 6; ++f) re[f * nr + r] = re[f * nr + r] / nn; /* :90-101 */
      const double rho = re[r];
      vel[r] = re[nr + r] / rho;          /* ux (:104) */
      vel[nr + r] = re[2 * nr + r] / rho; /* uy (:105) */
      vel[2 * nr + r] = -(rho * p->a * sin(p->kf * y)); /* Fx (:108) */
      vel[3 * nr + r] = +rho * p->a * sin(p->kf * x);   /* Fy (:109) */
    }
  }
  for (int f = 0; f < 4; ++f) oracle_r2c_2d(nx, ny, vel + f * nr, vk + f * s2); /* :122-132 */
  for (int i = 0; i < nh; ++i) { /* :136-160 */
    const double kx = kx_of(i, p->pi, p->lx);
    for (int j = 0; j < ny; ++j) {
      const double ky = ky_of(j, ny, p->pi, p->ly);
      const size_t q = 2 * ((size_t)j * nh + i);
      dk[q] = -kx * vk[q + 1];            dk[q + 1] = kx * vk[q];
      dk[s2 + q] = -ky * vk[s2 + q + 1];  dk[s2 + q + 1] = ky * vk[s2 + q];
      dk[2 * s2 + q] = -ky * Bx_k[q + 1]; dk[2 * s2 + q + 1] = ky * Bx_k[q];
      dk[3 * s2 + q] = -kx * By_k[q + 1]; dk[3 * s2 + q + 1] = kx * By_k[q];
    }
  }
  for (int f = 0; f < 4; ++f) oracle_c2r_2d(nx, ny, dk + f * s2, dr + f * nr); /* :165-175 */
  for (size_t r = 0; r < nr; ++r) { /* :181-213 */
    const double d_ux_dx = dr[r] / nn, d_uy_dy = dr[nr + r] / nn;
    double d_Bx_dy, d_By_dx;
    if (p->defined) {
      d_Bx_dy = dr[2 * nr + r] / nn;
      d_By_dx = dr[3 * nr + r] / nn;
    } else { /* :186-187 */
      d_Bx_dy = d_ux_dx / nn;
      d_By_dx = d_uy_dy / nn;
    }
    const double curl_B = d_By_dx - d_Bx_dy;
    const double rho = re[r], rho_ux = re[nr + r], rho_uy = re[2 * nr + r], E = re[3 * nr + r];
    const double Bx = re[4 * nr + r], By = re[5 * nr + r];
    const double ux = vel[r], uy = vel[nr + r];
    const double B2 = Bx * Bx + By * By;
    const double P = p->cs * p->cs * rho;
    tr[0 * nr + r] = rho_ux * ux + P + B2 / 2.0 - Bx * Bx; /* Mom_x_1 */
    tr[1 * nr + r] = rho_ux * uy - Bx * By;                /* Mom_x_2 */
    tr[2 * nr + r] = rho_ux * uy - Bx * By;                /* Mom_y_1 */
    tr[3 * nr + r] = rho_uy * uy + P + B2 / 2.0 - By * By; /* Mom_y_2 */
    double ex = (E + P + B2 / 2.0) * ux - ux * Bx * Bx - uy * Bx * By;
    ex = ex - p->eta * By * curl_B;
    double ey = (E + P + B2 / 2.0) * uy - ux * Bx * By - uy * By * By;
    ey = ey + p->eta * Bx * curl_B;
    tr[4 * nr + r] = ex;                                   /* Energy_x */
    tr[5 * nr + r] = ey;                                   /* Energy_y */
    const double dv = d_ux_dx + d_uy_dy;
    tr[6 * nr + r] = dv * dv;                              /* E_Visc */
    tr[7 * nr + r] = uy * Bx - By * ux;                    /* Mag_x */
    tr[8 * nr + r] = ux * By - Bx * uy;                    /* Mag_y */
  }
  for (int f = 0; f < 9; ++f) oracle_r2c_2d(nx, ny, tr + f * nr, tk + f * s2); /* :217-241 */
  const double cut = ((double)(nx + ny) / 2.0) / 3.0;
  for (int i = 0; i < nh; ++i) { /* :248-414 */
    const double kx = kx_of(i, p->pi, p->lx);
    for (int j = 0; j < ny; ++j) {
      const double ky = ky_of(j, ny, p->pi, p->ly);
      const size_t q = 2 * ((size_t)j * nh + i);
      const int cut_here = sqrt(kx * kx + ky * ky) >= cut;
      for (int c = 0; c < 2; ++c) {
        /* (0,1) k f: real part -k Im f, imaginary part k Re f */
#define IK(k_, f_) ((c) == 0 ? -(k_) * (f_)[q + 1] : (k_) * (f_)[q])
        double ikx_rux = IK(kx, rho_ux_k), iky_ruy = IK(ky, rho_uy_k);
        double ikx_m11 = IK(kx, tk), iky_m12 = IK(ky, tk + s2);
        double ikx_m21 = IK(kx, tk + 2 * s2), iky_m22 = IK(ky, tk + 3 * s2);
        double kx2ux = kx * kx * vk[q + c], ky2ux = ky * ky * vk[q + c];
        double kx2uy = kx * kx * vk[s2 + q + c], ky2uy = ky * ky * vk[s2 + q + c];
        double ikx_ex = IK(kx, tk + 4 * s2), iky_ey = IK(ky, tk + 5 * s2);
        double ev = tk[6 * s2 + q + c];
        double iky_mgx = IK(ky, tk + 7 * s2), ikx_mgy = IK(kx, tk + 8 * s2);
        double kx2bx = kx * kx * Bx_k[q + c], ky2bx = ky * ky * Bx_k[q + c];
        double kx2by = kx * kx * By_k[q + c], ky2by = ky * ky * By_k[q + c];
#undef IK
        if (cut_here) {
          ikx_rux = iky_ruy = ikx_m11 = iky_m12 = ikx_m21 = iky_m22 = 0.0;
          kx2ux = ky2ux = kx2uy = ky2uy = ikx_ex = iky_ey = ev = iky_mgx = ikx_mgy = 0.0;
          kx2bx = ky2bx = kx2by = ky2by = 0.0;
        }
        const double fx = vk[2 * s2 + q + c], fy = vk[3 * s2 + q + c];
        double d;
        dstate[q + c] = -(ikx_rux + iky_ruy);
        d = -(ikx_m11 + iky_m12);
        dstate[s2 + q + c] = d - p->mu * (kx2ux + ky2ux) + fx;
        d = -(ikx_m21 + iky_m22);
        dstate[2 * s2 + q + c] = d - p->mu * (kx2uy + ky2uy) + fy;
        d = -(ikx_ex + iky_ey);
        dstate[3 * s2 + q + c] = d + p->mu * ev;
        dstate[4 * s2 + q + c] = -iky_mgx - p->eta * (kx2bx + ky2bx);
        dstate[5 * s2 + q + c] = -ikx_mgy - p->eta * (kx2by + ky2by);
      }
    }
  }
  free(re); free(vel); free(vk); free(dk); free(dr); free(tr); free(tk);
}

void oracle_ab2com(int nx, int ny, double dt, const double* state, double* state_new,
                   const double* d_old, const double* d_new) {
  const int nh = nx / 2 + 1;
  const size_t n2 = 2 * (size_t)nh * ny;
  for (int f = 0; f < 6; ++f)
    ab2_update(nh, ny, dt, state + f * n2, state_new + f * n2, d_old + f * n2, d_new + f * n2);
}

void oracle_run_com(int nx, int ny, const oracle_com_params* p, double dt, int nsteps,
                    double* state, double* hist) {
  const int nh = nx / 2 + 1;
  const size_t n12 = 12 * (size_t)nh * ny;
  double* sn = (double*)xcalloc(n12, sizeof(double));
  double* dn = (double*)xcalloc(n12, sizeof(double));
  for (int s = 0; s < nsteps; ++s) {
    oracle_derive2com(nx, ny, p, state, dn);
    oracle_ab2com(nx, ny, dt, state, sn, hist, dn);
    memcpy(hist, dn, n12 * sizeof(double));
    memcpy(state, sn, n12 * sizeof(double));
  }
  free(sn); free(dn);
}

void oracle_ic_com(int nx, int ny, double lx_ini, double ly_ini, double cs, double kf, double b0,
                   double* state) {
  const double pi = PI_R8;
  const double lx = lx_ini * pi, ly = ly_ini * pi;
  const double dx = lx / (double)nx, dy = ly / (double)ny;
  const double spheat = 5.0 / 3.0, rho0 = 1.0;
  const int nh = nx / 2 + 1;
  const size_t ns = (size_t)nh * ny, nr = (size_t)nx * ny;
  double* re = (double*)xcalloc(6 * nr, sizeof(double));
  for (int i = 0; i < nx; ++i) {
    const double x = (double)(float)i * dx;
    for (int j = 0; j < ny; ++j) {
      const double y = (double)(float)j * dy;
      const size_t r = (size_t)j * nx + i;
      const double rho = rho0, ux = -sin(kf * y), uy = sin(kf * x);
      const double P = cs * cs * rho, Bx = b0, By = b0;
      const double E = P / (spheat - 1.0) + 0.50 * rho * (ux * ux + uy * uy) + 0.50 * (Bx * Bx + By * By);
      re[r] = rho;
      re[nr + r] = rho * ux;
      re[2 * nr + r] = rho * uy;
      re[3 * nr + r] = E;
      re[4 * nr + r] = Bx;
      re[5 * nr + r] = By;
    }
  }
  for (int f = 0; f < 6; ++f) oracle_r2c_2d(nx, ny, re + f * nr, state + f * 2 * ns);
  free(re);
}

