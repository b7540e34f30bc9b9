/* The reference's plain driver loop (src/main2csh.f95:114-126) as a compiled
 * caller of the drop-ins, with no header and no Python: every argument by
 * reference, complex(8) arrays as double _Complex in the Fortran layout
 * a(Nh,Ny), names as gfortran mangles them.
 *
 *   reference_loop ab2 <Nx> <Ny> <steps> <nu> <dt> <in> <out>
 *       do time = ...: call derive2csh(...); call ab2csh(...);
 *       dt_omegak_old = dt_omegak_new; omegak = omegak_new
 *   reference_loop rk4 <Nx> <Ny> 1 <nu> <dt> <in> <out>
 *       one call rk42css(Nx,Ny,Nh,alpha=1,nu,time,dt,omegak,omegak_new,...)
 *
 * <in> holds omegak as Nh*Ny interleaved (re,im) doubles; <out> receives
 * omegak after the loop (omegak_new for rk4).  Exit status 0 when every call
 * left tara_last_error() at 0. */
#include <complex.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

extern void derive2csh_(int*, int*, int*, double*, double*, double _Complex*, double _Complex*,
                        double _Complex*, double _Complex*);
extern void ab2csh_(int*, int*, int*, double*, double*, double*, double _Complex*, double _Complex*,
                    double _Complex*, double _Complex*);
extern void rk42css_(int*, int*, int*, double*, double*, double*, double*, double _Complex*,
                     double _Complex*, double _Complex*, double _Complex*);
extern int tara_last_error(void);
extern const char* tara_last_error_message(void);

int main(int argc, char** argv) {
  if (argc != 9) {
    fprintf(stderr, "usage: %s ab2|rk4 Nx Ny steps nu dt in out\n", argv[0]);
    return 2;
  }
  int nx = atoi(argv[2]), ny = atoi(argv[3]), steps = atoi(argv[4]);
  int nh = nx / 2 + 1;
  double nu = atof(argv[5]), dt = atof(argv[6]), time = 0.0, alpha = 1.0;
  const size_t n = (size_t)nh * ny;
  double _Complex* w = calloc(n, sizeof(double _Complex));
  double _Complex* wn = calloc(n, sizeof(double _Complex));
  /* allocate(dt_omegak_old): the reference reads it before the first write;
   * a fresh allocation reads as zero */
  double _Complex* d_old = calloc(n, sizeof(double _Complex));
  double _Complex* d_new = calloc(n, sizeof(double _Complex));
  FILE* f = fopen(argv[7], "rb");
  if (!f || fread(w, sizeof(double _Complex), n, f) != n) {
    fprintf(stderr, "cannot read %s\n", argv[7]);
    return 2;
  }
  fclose(f);
  if (strcmp(argv[1], "ab2") == 0) {
    for (int t = 0; t < steps; ++t) {
      derive2csh_(&nx, &ny, &nh, &nu, &time, w, wn, d_old, d_new);
      ab2csh_(&nx, &ny, &nh, &nu, &time, &dt, w, wn, d_old, d_new);
      if (tara_last_error() != 0) break;
      memcpy(d_old, d_new, n * sizeof(double _Complex)); /* dt_omegak_old = dt_omegak_new */
      memcpy(w, wn, n * sizeof(double _Complex));        /* omegak = omegak_new */
      time += dt;
    }
  } else {
    rk42css_(&nx, &ny, &nh, &alpha, &nu, &time, &dt, w, wn, d_old, d_new);
    memcpy(w, wn, n * sizeof(double _Complex));
  }
  if (tara_last_error() != 0) {
    fprintf(stderr, "tara error %d: %s\n", tara_last_error(), tara_last_error_message());
    return 1;
  }
  f = fopen(argv[8], "wb");
  if (!f || fwrite(w, sizeof(double _Complex), n, f) != n) return 2;
  fclose(f);
  free(w);
  free(wn);
  free(d_old);
  free(d_new);
  return 0;
}
