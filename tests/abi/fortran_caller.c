/* A caller in the shape gfortran gives an external subroutine with an implicit
 * interface (src/main2csh.f95:118-119 calls derive2csh/ab2csh this way): no
 * header, every argument by reference, complex(8) arrays as double _Complex,
 * names in lowercase with one trailing underscore.  It calls the drop-ins with
 * shapes that the library must refuse before touching a GPU, and checks that
 * nothing was written and the failure was recorded. */
#include <complex.h>
#include <string.h>

extern void derive2csh_(int*, int*, int*, double*, double*, double _Complex*, double _Complex*,
                        double _Complex*, double _Complex*);
extern void ab2csh_(int*, int*, int*, double*, double*, double*, double _Complex*, double _Complex*,
                    double _Complex*, double _Complex*);
extern void rk42css_(int*, int*, int*, double*, double*, double*, double*, double _Complex*,
                     double _Complex*, double _Complex*, double _Complex*);
extern int tara_last_error(void);
extern void tara_clear_error(void);

enum { NX = 32, NY = 32, NH = NX / 2 + 1 };

static int untouched(const double _Complex* a, size_t n, double _Complex v) {
  for (size_t i = 0; i < n; ++i)
    if (a[i] != v) return 0;
  return 1;
}

/* Returns 0 when every call was refused with status 1 (bad arguments) and no
 * array changed; otherwise the number of the failing check. */
int fortran_style_calls(void) {
  static double _Complex w[NH * NY], wn[NH * NY], d_old[NH * NY], d_new[NH * NY];
  const double _Complex fill = 7.0 + 3.0 * I;
  for (size_t i = 0; i < NH * NY; ++i) w[i] = wn[i] = d_old[i] = d_new[i] = fill;
  int nx = NX, ny = NY, nh_bad = NH + 1, nx_bad = 88, nh_of_bad = 45;
  double nu = 0.01, t = 0.0, dt = 1e-4, alpha = 1.0;

  tara_clear_error();
  derive2csh_(&nx, &ny, &nh_bad, &nu, &t, w, wn, d_old, d_new);  /* Nh != Nx/2+1 */
  if (tara_last_error() != 1) return 1;
  tara_clear_error();
  derive2csh_(&nx_bad, &ny, &nh_of_bad, &nu, &t, w, wn, d_old, d_new);  /* Nx = 88: factor 11 */
  if (tara_last_error() != 1) return 2;
  tara_clear_error();
  ab2csh_(&nx, &ny, &nh_bad, &nu, &t, &dt, w, wn, d_old, d_new);
  if (tara_last_error() != 1) return 3;
  tara_clear_error();
  rk42css_(&nx, &ny, &nh_bad, &alpha, &nu, &t, &dt, w, wn, d_old, d_new);
  if (tara_last_error() != 1) return 4;
  if (!untouched(w, NH * NY, fill) || !untouched(wn, NH * NY, fill) || !untouched(d_old, NH * NY, fill) ||
      !untouched(d_new, NH * NY, fill))
    return 5;
  return 0;
}
