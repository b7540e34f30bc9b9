// input.ini driver: the reference program's dispatch (src/main.f95) and the
// time loops of the solvers on the path (src/main2css.f95, src/main2csh.f95,
// src/main2coh.f95, src/main2com.f95, src/main3com.f95), with their output files.  Host code over the C ABI; every
// transform and update runs in libtara's kernels.
#include <cmath>
#include <exception>
#include <new>
#include <cstdio>
#include <cstring>
#include <string>
#include <sys/stat.h>
#include <vector>

#include "../../include/tara.h"
#include "ini.h"
#include "status.h"

using namespace tara;

namespace {

// A run that leaves on an error frees its handles on the way out; the public
// destroy records success, so the error is saved and put back around it.
template <typename F>
void keep_error_across(F&& cleanup) {
  const ErrorState saved = save_error();
  cleanup();
  restore_error(saved);
}

const double kPi = 3.14159265358979323846;  // real(kind=8), parameter :: pi (main2css.f95:9)

struct Reader {
  IniFile ini;
  std::string err;
  bool ok = true;

  void str(const char* sec, const char* key, std::string& v) {
    if (!ok) return;
    ok = ini_get(ini, sec, key, v, err);
    if (ok) {  // character(len=90) variables, compared without trailing blanks
      if (v.size() > 90) v.resize(90);
      while (!v.empty() && v.back() == ' ') v.pop_back();
    }
  }
  void i(const char* sec, const char* key, int& v) {
    std::string s;
    str(sec, key, s);
    if (!ok) return;
    long long x = 0;
    ok = fortran_read_int(s, x, err);
    if (!ok) err = std::string(sec) + ":" + key + ": " + err;
    v = (int)x;
  }
  void d(const char* sec, const char* key, double& v) {
    std::string s;
    str(sec, key, s);
    if (!ok) return;
    ok = fortran_read_double(s, v, err);
    if (!ok) err = std::string(sec) + ":" + key + ": " + err;
  }
};

struct Out {
  FILE* f = nullptr;
  explicit Out(const std::string& path) { f = std::fopen(path.c_str(), "w"); }
  ~Out() {
    if (f) std::fclose(f);
  }
  // the refusal to return when the file could not be opened
  int open_error(const std::string& path) const {
    return f ? TARA_OK : set_error(TARA_ERR_ARGS, "cannot open " + path + " for writing");
  }
  void rec(std::initializer_list<double> v) {
    if (!f) return;
    std::vector<double> a(v);
    const std::string r = fortran_list_record(a.data(), (int)a.size());
    std::fprintf(f, "%s\n", r.c_str());
  }
};

// Fortran real DO loop `do time = t0, t1, dt`: the trip count is
// max(int((t1 - t0 + dt)/dt), 0) in the loop variable's type, and the variable
// advances by dt each iteration.
long trip_count(double t0, double t1, double dt) {
  const double n = (t1 - t0 + dt) / dt;
  return n > 0 ? (long)n : 0;
}

long nint(double x) { return (long)std::llround(x); }

std::string fort_name(const std::string& dir, long unit) {
  char buf[64];
  std::snprintf(buf, sizeof buf, "/fort.%08ld", unit);  // '("output/fort.",I8.8)'
  return dir + buf;
}

int fail_rc() { return tara_last_error() ? tara_last_error() : TARA_ERR_CUDA; }

// The reference reads any Nx, Ny (, Nz) (src/main2csh.f95:35-38) and FFTW takes
// any length; these kernels take powers of two, 16 to 4096 in 2D and 16 to 512
// in 3D, and the 2D programs (any_ok) also even lengths 8 to 3600 with
// factors 2, 3, 5, 7 (the mixed-radix FP64 path).  Refuse anything else
// before allocating, naming the supported set.
// even, 8 to 3600, no prime factor above 7 (the mixed-radix path's lengths)
bool mixed_radix_size(int n) {
  if (n < 8 || n > 3600 || (n & 1)) return false;
  for (int p : {2, 3, 5, 7})
    while (n % p == 0) n /= p;
  return n == 1;
}

int check_grid(const char* program, int dims, int nx, int ny, int nz, bool any_ok = false) {
  const int hi = dims == 2 ? 4096 : 512;
  const int n[3] = {nx, ny, nz};
  const char* name[3] = {"Nx", "Ny", "Nz"};
  for (int d = 0; d < dims; ++d) {
    const bool pow2 = n[d] >= 16 && n[d] <= hi && !(n[d] & (n[d] - 1));
    if (pow2 || (any_ok && mixed_radix_size(n[d]))) continue;
    char msg[320];
    if (any_ok)
      std::snprintf(msg, sizeof msg,
                    "%s: %s = %d is not supported; grid sizes here are powers of two from 16 to %d "
                    "(16, 32, 64, ..., %d), or even lengths from 8 to 3600 whose only prime factors are "
                    "2, 3, 5 and 7 (e.g. 48, 96, 384, 448)",
                    program, name[d], n[d], hi, hi);
    else
      std::snprintf(msg, sizeof msg,
                    "%s: %s = %d is not supported; grid sizes here are powers of two from 16 to %d "
                    "(16, 32, 64, ..., %d)",
                    program, name[d], n[d], hi, hi);
    return set_error(TARA_ERR_ARGS, msg);
  }
  return TARA_OK;
}

// ---------------------------------------------------------------------------
// tara2dScrSer (src/main2css.f95) and tara2dHydSer (src/main2csh.f95)
// ---------------------------------------------------------------------------
int run_2d(Reader& R, const std::string& out, int max_steps, bool screened) {
  int np = 0, nx = 0, ny = 0;
  double lx = 0, ly = 0, nu = 0, tmin = 0, tmax = 0, dt = 0, w0 = 0, m0 = 0, d = 0;
  R.i("particle", "Np", np);
  R.i("grid", "Nx", nx);
  R.i("grid", "Ny", ny);
  R.d("length", "Lx", lx);
  R.d("length", "Ly", ly);
  R.d("resistivity", "nu", nu);
  R.d("time", "time_min", tmin);
  R.d("time", "time_max", tmax);
  R.d("time", "dt", dt);
  R.d("initialProfile", "W0", w0);
  R.d("initialProfile", "m0", m0);
  R.d("initialProfile", "d", d);
  if (!R.ok) return set_error(TARA_ERR_INI, R.err);
  if (int rc = check_grid(screened ? "tara2dScrSer" : "tara2dHydSer", 2, nx, ny, 0, true)) return rc;
  lx = lx * kPi;
  ly = ly * kPi;
  const double dx = lx / (double)nx, dy = ly / (double)ny;
  d = d * kPi;
  const double alpha = 1.0, lambda = 10.0;  // src/main2css.f95:86-87
  const int nh = nx / 2 + 1;
  // initial vorticity (src/main2css.f95:89-104, src/main2csh.f95:98-106)
  std::vector<double> xs(nx), ys(ny), omega((size_t)nx * ny);
  for (int i = 0; i < nx; ++i) xs[i] = screened ? 0.0 + (double)(float)i * dx : (double)i * dx;
  for (int j = 0; j < ny; ++j) ys[j] = screened ? (double)0.0f + (double)(float)j * dy : (double)j * dy;
  for (int i = 0; i < nx; ++i)
    for (int j = 0; j < ny; ++j) {
      const double y = ys[j];
      const double c1 = std::cosh((y + 0.5 * kPi) / d), c2 = std::cosh((y - 0.5 * kPi) / d);
      const double c3 = std::cosh((y + 1.5 * kPi) / d), c4 = std::cosh((y - 1.5 * kPi) / d);
      double w = w0 / (c1 * c1) - w0 / (c2 * c2);
      w = w - w0 / (c3 * c3) + w0 / (c4 * c4);
      w = w + (screened ? (double)0.01f : 0.10) * std::cos(m0 * xs[i]);
      omega[(size_t)j * nx + i] = w;
    }
  mkdir(out.c_str(), 0755);
  if (screened) {
    const std::vector<double> zero((size_t)nx * ny, 0.0);
    if (int rc = write_grid_records(out + "/Initial_Condition_Velocity.dat", nx, ny, xs.data(), ys.data(),
                                    {omega.data(), zero.data(), zero.data()}))
      return rc;
  }
  std::vector<double> wk(2 * (size_t)nh * ny);
  if (tara_fft2d_r2c(nx, ny, TARA_PREC_FP64, omega.data(), wk.data())) return fail_rc();
  tara2d_config cfg;
  tara2d_default_config(&cfg, nx, ny);
  cfg.nu = nu;
  cfg.dt = dt;
  if (screened) {  // derive2css in defined mode: its pi = 3.1428 with the driver's box
    cfg.rhs = TARA_RHS_SCREEN;
    cfg.alpha = alpha;
    cfg.lambda = lambda;
    cfg.lx = lx;
    cfg.ly = ly;
  }
  tara2d* h = nullptr;
  if (tara2d_create(&cfg, &h)) return fail_rc();
  struct Guard {
    tara2d* h;
    ~Guard() { keep_error_across([&] { tara2d_destroy(h); }); }
  } guard{h};
  if (tara2d_set_state(h, wk.data(), nullptr)) return fail_rc();
  const size_t nr = (size_t)nx * ny;
  std::vector<double> psi(nr), om(nr), ux(nr), uy(nr);
  if (screened) {  // initial diagnostics use psi = omega/k^2 (src/main2css.f95:112-179)
    tara2d_diag_params p0 = {kPi, lx, ly, 0.0, 0};
    if (tara2d_real_fields(h, &p0, psi.data(), om.data(), ux.data(), uy.data())) return fail_rc();
    if (int rc = write_grid_records(out + "/Initial_Condition_Omega_REP.dat", nx, ny, xs.data(), ys.data(),
                                    {om.data(), psi.data(), ux.data(), uy.data()}))
      return rc;
  }
  // Lagrangian particles of the plain driver (src/main2csh.f95:93-96, 187-273);
  // the screened driver reads Np but moves none
  tara_particles* parts = nullptr;
  struct PGuard {
    tara_particles** p;
    ~PGuard() { keep_error_across([&] { tara_particles_destroy(*p); }); }
  } pguard{&parts};
  std::vector<double> xp, yp;
  if (!screened && np > 0) {
    xp.resize(np);
    yp.resize(np);
    uint64_t state = 1;
    for (int i = 0; i < np; ++i) {
      xp[i] = (double)tara_park_miller_rand(&state) * lx;  // xp(i) = rand()*Lx
      yp[i] = (double)tara_park_miller_rand(&state) * ly;
    }
    if (tara_particles_create(h, kPi, lx, ly, np, xp.data(), yp.data(), &parts)) return fail_rc();
  }
  Out energy(out + "/Energy.dat");  // written every step by the screened driver only
  if (int rc = energy.open_error(out + "/Energy.dat")) return rc;
  const tara2d_diag_params dp = {kPi, lx, ly, screened ? lambda : 0.0, screened ? 1 : 0};
  const long n = trip_count(tmin, tmax, dt);
  const long steps = (max_steps > 0 && max_steps < n) ? max_steps : n;
  const long every = screened ? 100 : 1000;
  double time = tmin, y_energy = 0.0;
  for (long it = 0; it < steps; ++it) {
    const long t = nint(time / dt) - (long)(tmin / dt);
    if (tara2d_step(h, 1)) return fail_rc();  // derive + ab2 + history rotation
    if (screened) {
      double usq = 0.0, uysq = 0.0;
      if (tara2d_diag_reference(h, &dp, &usq, &uysq)) return fail_rc();
      y_energy += uysq;  // never reset by the reference (src/main2css.f95:259)
      if (t % every == 0) {
        if (tara2d_real_fields(h, &dp, nullptr, om.data(), ux.data(), uy.data())) return fail_rc();
        if (int rc = write_grid_records(fort_name(out, t + 100), nx, ny, xs.data(), ys.data(),
                                        {ux.data(), uy.data(), om.data()}))
          return rc;
      }
      energy.rec({time, usq, y_energy});
    } else {
      if (t % every == 0) {
        if (tara2d_real_fields(h, &dp, nullptr, om.data(), ux.data(), uy.data())) return fail_rc();
        if (int rc = write_grid_records(fort_name(out, t + 100), nx, ny, xs.data(), ys.data(),
                                        {om.data(), ux.data(), uy.data()}))
          return rc;
      }
      if (parts) {
        if (tara_particles_advance(parts, dt)) return fail_rc();
        if (t % every == 0) {  // fort.(t+105): one "xp yp" record per particle
          if (tara_particles_get(parts, xp.data(), yp.data())) return fail_rc();
          Out pf(fort_name(out, t + 105));
          if (int rc = pf.open_error(fort_name(out, t + 105))) return rc;
          for (int i = 0; i < np; ++i) pf.rec({xp[i], yp[i]});
        }
      }
    }
    time = time + dt;
  }
  if (tara2d_synchronize(h)) return fail_rc();
  return set_ok();
}

// ---------------------------------------------------------------------------
// tara3dMHDOMP (src/main3com.f95)
// ---------------------------------------------------------------------------
int run_3d(Reader& R, const std::string& out, int max_steps) {
  int nx = 0, ny = 0, nz = 0;
  double lx = 0, ly = 0, lz = 0, tmin = 0, tmax = 0, dt = 0, mu = 0;
  R.i("grid", "Nx", nx);
  R.i("grid", "Ny", ny);
  R.i("grid", "Nz", nz);
  R.d("length", "Lx", lx);
  R.d("length", "Ly", ly);
  R.d("length", "Lz", lz);
  R.d("time", "time_min", tmin);
  R.d("time", "time_max", tmax);
  R.d("time", "dt", dt);
  R.d("resistivity", "nu", mu);
  if (!R.ok) return set_error(TARA_ERR_INI, R.err);
  if (int rc = check_grid("tara3dMHDOMP", 3, nx, ny, nz)) return rc;
  lx = lx * kPi;
  ly = ly * kPi;
  lz = lz * kPi;
  const double dx = lx / (double)nx, dy = ly / (double)ny, dz = lz / (double)nz;
  // src/main3com.f95:216-262: eta = 0.005, M = 0.1 -> CS = 10, U0 = 0.1, B0 = U0/MA
  const double eta = 0.005, U0 = 0.10, cs = 1.0 / 0.10, B0 = U0 / 1.0 * std::sqrt(1.0 * 1.0);
  const double A = 1.0, B = 1.0, C = 1.0, kf = 1.0, P0 = 1.0, rho0 = 1.0;
  const size_t nr = (size_t)nx * ny * nz;
  std::vector<double> real(8 * nr);
  for (int i = 0; i < nx; ++i) {
    const double x = 0.0 + (double)(float)i * dx;
    for (int j = 0; j < ny; ++j) {
      const double y = 0.0 + (double)(float)j * dy;
      for (int k = 0; k < nz; ++k) {
        const double z = 0.0 + (double)(float)k * dz;
        const size_t r = ((size_t)k * ny + j) * nx + i;
        const double vx = U0 * (A * std::sin(kf * z) + C * std::cos(kf * y));
        const double vy = U0 * (B * std::sin(kf * x) + A * std::cos(kf * z));
        const double vz = U0 * (C * std::sin(kf * y) + B * std::cos(kf * x));
        const double E = P0 + 0.50 * rho0 * (vx * vx + vy * vy + vz * vz) +
                         0.50 * (B0 * B0 + B0 * B0 + B0 * B0);
        const double f[8] = {rho0, rho0 * vx, rho0 * vy, rho0 * vz, E, B0, B0, B0};
        for (int q = 0; q < 8; ++q) real[q * nr + r] = f[q];
      }
    }
  }
  tara3d_config cfg;
  tara3d_default_config(&cfg, nx, ny, nz);
  cfg.kpi = kPi;
  cfg.lx = lx;
  cfg.ly = ly;
  cfg.lz = lz;
  cfg.mu = mu;
  cfg.eta = eta;
  cfg.cs = cs;
  cfg.dt = dt;
  cfg.defined = 0;
  tara3d* h = nullptr;
  if (tara3d_create(&cfg, &h)) return fail_rc();
  struct Guard {
    tara3d* h;
    ~Guard() { keep_error_across([&] { tara3d_destroy(h); }); }
  } guard{h};
  if (tara3d_set_state_real(h, real.data())) return fail_rc();
  mkdir(out.c_str(), 0755);
  Out energy(out + "/Energy.dat");
  if (int rc = energy.open_error(out + "/Energy.dat")) return rc;
  const long n = trip_count(tmin, tmax, dt);
  const long steps = (max_steps > 0 && max_steps < n) ? max_steps : n;
  double time = tmin;
  for (long it = 0; it < steps; ++it) {
    if (tara3d_step(h, 1)) return fail_rc();
    double dg[4];
    if (tara3d_diag(h, dg)) return fail_rc();
    energy.rec({time, dg[0], dg[1], dg[2], dg[3]});
    time = time + dt;
  }
  return set_ok();
}

// ---------------------------------------------------------------------------
// tara2dHydOMP (src/main2coh.f95): 2D compressible isothermal hydro
// ---------------------------------------------------------------------------
int run_coh(Reader& R, const std::string& out, int max_steps) {
  int nx = 0, ny = 0;
  double lx = 0, ly = 0, tmin = 0, tmax = 0, dt = 0, nu = 0;
  R.i("grid", "Nx", nx);
  R.i("grid", "Ny", ny);
  R.d("length", "Lx", lx);
  R.d("length", "Ly", ly);
  R.d("time", "time_min", tmin);
  R.d("time", "time_max", tmax);
  R.d("time", "dt", dt);
  R.d("resistivity", "nu", nu);  // read, then replaced by 0.0002 (src/main2coh.f95:119-120)
  if (!R.ok) return set_error(TARA_ERR_INI, R.err);
  if (int rc = check_grid("tara2dHydOMP", 2, nx, ny, 0, true)) return rc;
  const double lx_ini = lx, ly_ini = ly;
  lx = lx * kPi;
  ly = ly * kPi;
  const double dx = lx / (double)nx, dy = ly / (double)ny;
  tara_coh2d_config cfg;
  tara_coh2d_default_config(&cfg, nx, ny);  // mux = muy = 0.0002, CS = U0/M (:119-133)
  cfg.kpi = kPi;
  cfg.lx = lx;
  cfg.ly = ly;
  cfg.dt = dt;
  tara_coh2d* h = nullptr;
  if (tara_coh2d_create(&cfg, &h)) return fail_rc();
  struct Guard {
    tara_coh2d* h;
    ~Guard() { keep_error_across([&] { tara_coh2d_destroy(h); }); }
  } guard{h};
  if (tara_coh2d_init_vortices(h, lx_ini, ly_ini)) return fail_rc();
  mkdir(out.c_str(), 0755);
  const size_t nr = (size_t)nx * ny;
  std::vector<double> xs(nx), ys(ny), dn(nr), ux(nr), uy(nr), om(nr);
  for (int i = 0; i < nx; ++i) xs[i] = 0.0 + (double)(float)i * dx;  // x(i)=0.0d0+real(i-1)*dx
  for (int j = 0; j < ny; ++j) ys[j] = 0.0 + (double)(float)j * dy;
  auto snapshot = [&](const std::string& path) -> int {  // x, y, omega, n, ux, uy
    if (tara_coh2d_real_fields(h, dn.data(), ux.data(), uy.data(), om.data())) return fail_rc();
    return write_grid_records(path, nx, ny, xs.data(), ys.data(), {om.data(), dn.data(), ux.data(), uy.data()});
  };
  int rc;
  if ((rc = snapshot(out + "/Initial_Grid_Data_Reproduced.dat"))) return rc;  // (:214-238)
  Out energy(out + "/Energy.dat");
  if (int rc = energy.open_error(out + "/Energy.dat")) return rc;
  const long n = trip_count(tmin, tmax, dt);
  const long steps = (max_steps > 0 && max_steps < n) ? max_steps : n;
  const double every = 1.0 / (10.0 * dt);  // mod(float(t),1.0d0/(10.0d0*dt)) == 0.0 (:407)
  double time = tmin;
  for (long it = 0; it < steps; ++it) {
    const long t = nint(time / dt) - (long)(tmin / dt);
    if (tara_coh2d_step(h, 1)) return fail_rc();  // derive2coh + ab2coh + rotation (:263-298)
    double d[6];
    if (tara_coh2d_diag(h, d)) return fail_rc();
    if (std::fmod((double)(float)t, every) == 0.0 && (rc = snapshot(fort_name(out, t + 100)))) return rc;
    energy.rec({time, d[0], d[1], d[2], d[3], d[4], d[5]});
    time = time + dt;
  }
  return set_ok();
}

// ---------------------------------------------------------------------------
// tara2dMHDOMP (src/main2com.f95): 2D compressible MHD
// ---------------------------------------------------------------------------
int run_com(Reader& R, const std::string& out, int max_steps) {
  int nx = 0, ny = 0;
  double lx = 0, ly = 0, tmin = 0, tmax = 0, dt = 0, mu = 0;
  R.i("grid", "Nx", nx);
  R.i("grid", "Ny", ny);
  R.d("length", "Lx", lx);
  R.d("length", "Ly", ly);
  R.d("time", "time_min", tmin);
  R.d("time", "time_max", tmax);
  R.d("time", "dt", dt);
  R.d("resistivity", "nu", mu);
  if (!R.ok) return set_error(TARA_ERR_INI, R.err);
  if (int rc = check_grid("tara2dMHDOMP", 2, nx, ny, 0, true)) return rc;
  const double lx_ini = lx, ly_ini = ly;
  lx = lx * kPi;
  ly = ly * kPi;
  const double dx = lx / (double)nx, dy = ly / (double)ny;
  // src/main2com.f95:161-215: eta = 1e-4, M = 0.01 -> CS = 100, U0 = M CS = 1,
  // VA = U0/MA = 1, B0 = VA sqrt(mu_0 rho0) = 1, kf = A = 1
  const double cs = 1.0 / 0.010, U0 = 0.010 * cs, B0 = (U0 / 1.0) * std::sqrt(1.0 * 1.0);
  tara_com2d_config cfg;
  tara_com2d_default_config(&cfg, nx, ny);
  cfg.kpi = kPi;
  cfg.lx = lx;
  cfg.ly = ly;
  cfg.mu = mu;
  cfg.eta = 0.000100;
  cfg.cs = cs;
  cfg.kf = 1.0;
  cfg.a = 1.0;
  cfg.dt = dt;
  cfg.defined = 0;
  tara_com2d* h = nullptr;
  if (tara_com2d_create(&cfg, &h)) return fail_rc();
  struct Guard {
    tara_com2d* h;
    ~Guard() { keep_error_across([&] { tara_com2d_destroy(h); }); }
  } guard{h};
  if (tara_com2d_init_reference(h, lx_ini, ly_ini, B0)) return fail_rc();
  mkdir(out.c_str(), 0755);
  const size_t nr = (size_t)nx * ny;
  std::vector<double> xs(nx), ys(ny);
  for (int i = 0; i < nx; ++i) xs[i] = 0.0 + (double)(float)i * dx;
  for (int j = 0; j < ny; ++j) ys[j] = 0.0 + (double)(float)j * dy;
  Out energy(out + "/Energy.dat");
  if (int rc = energy.open_error(out + "/Energy.dat")) return rc;
  const long n = trip_count(tmin, tmax, dt);
  const long steps = (max_steps > 0 && max_steps < n) ? max_steps : n;
  double time = tmin;
  for (long it = 0; it < steps; ++it) {
    const long t = nint(time / dt) - (long)(tmin / dt);
    if (tara_com2d_step(h, 1)) return fail_rc();  // derive2com + ab2com + rotation (:360-414)
    const double tf = (double)(float)t;
    if (std::fmod(tf, 100000.0) == 0.0) {  // fort.(t+100000): x, y, rho, ux, uy, P, E, Bx, By (:571-573)
      std::vector<double> f[7];
      for (auto& v : f) v.resize(nr);
      if (tara_com2d_real_fields(h, f[0].data(), f[1].data(), f[2].data(), f[3].data(), f[4].data(), f[5].data(),
                                 f[6].data()))
        return fail_rc();
      if (int rc = write_grid_records(fort_name(out, t + 100000), nx, ny, xs.data(), ys.data(),
                                      {f[0].data(), f[1].data(), f[2].data(), f[3].data(), f[4].data(),
                                       f[5].data(), f[6].data()}))
        return rc;
    }
    if (std::fmod(tf, 100.0) == 0.0) {  // Energy.dat every 100 steps (:578-580)
      double d[5];
      if (tara_com2d_diag(h, d)) return fail_rc();
      energy.rec({time, d[0], d[1], d[2], d[3], d[4]});
    }
    time = time + dt;
  }
  return set_ok();
}

// A console line of the driver, flushed at once so that it keeps its place among
// the caller's own output when stdout is a pipe or a file.
void say(const char* line) {
  std::fputs(line, stdout);
  std::fflush(stdout);
}

}  // namespace

namespace {
int run_ini(const char* ini_path, const char* out_dir, int max_steps);
}

// No C++ exception leaves the C ABI: a host allocation that fails (the field
// buffers of a large grid) is reported as TARA_ERR_NOMEM.
extern "C" int tara_run_ini(const char* ini_path, const char* out_dir, int max_steps) {
  try {
    return run_ini(ini_path, out_dir, max_steps);
  } catch (const std::bad_alloc&) {
    return set_error(TARA_ERR_NOMEM, "tara_run_ini: host allocation failed");
  } catch (const std::exception& e) {
    return set_error(TARA_ERR_ARGS, std::string("tara_run_ini: ") + e.what());
  }
}

namespace {
int run_ini(const char* ini_path, const char* out_dir, int max_steps) {
  Reader R;
  if (!ini_path) return set_error(TARA_ERR_ARGS, "null ini path");
  if (!ini_parse_file(ini_path, R.ini, R.err)) return set_error(TARA_ERR_INI, R.err);
  const std::string out = out_dir ? out_dir : "output";
  int dim = 0;
  std::string arch, mode, domain, hydrotype;
  R.i("dimension", "dim", dim);  // src/main.f95:26-30
  R.str("architecture", "arch", arch);
  R.str("parallel", "mode", mode);
  R.str("type", "domain", domain);
  R.str("problem", "hydrotype", hydrotype);
  if (!R.ok) return set_error(TARA_ERR_INI, R.err);
  const bool here = (arch == "cpu" || arch == "single-gpu");
  if (dim == 2 && here && mode == "serial" && hydrotype == "bare") {
    say(" tara-gb300: 2D serial hydrodynamic vorticity solver on the GPU\n");
    return run_2d(R, out, max_steps, false);
  }
  if (dim == 2 && here && mode == "serial" && hydrotype == "screen") {
    say(" tara-gb300: 2D serial screened hydrodynamic vorticity solver on the GPU\n");
    return run_2d(R, out, max_steps, true);
  }
  if (dim == 3 && here && mode == "openmp" && domain == "mhd") {
    say(" tara-gb300: 3D compressible MHD solver on the GPU\n");
    return run_3d(R, out, max_steps);
  }
  if (dim == 2 && here && mode == "openmp" && domain == "hydro") {
    say(" tara-gb300: 2D compressible isothermal hydrodynamic solver on the GPU\n");
    return run_coh(R, out, max_steps);
  }
  if (dim == 2 && here && mode == "openmp" && domain == "mhd") {
    say(" tara-gb300: 2D compressible MHD solver on the GPU\n");
    return run_com(R, out, max_steps);
  }
  if (mode == "mpi" || arch == "multi-gpu" || (dim == 3 && mode == "serial")) {
    say(" Under preparation. Please wait!\n");  // src/main.f95:40-85
    return set_ok();
  }
  if (dim == 1) return set_error(TARA_ERR_ARGS, "the 1D Burgers solver is not implemented by this library");
  say(" Incompatible Input file. Please check TARA user-manual.\n");
  return set_error(TARA_ERR_INI, "incompatible input file");
}
}  // namespace
