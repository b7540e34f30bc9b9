/* tara.h -- C ABI of libtara, the GB300 (sm_103a) implementation of TARA's 2D
 * pseudo-spectral right-hand side and explicit time steppers.
 *
 * Two layers:
 *
 * 1. Drop-in replacements for the reference's Fortran subroutines.  The
 *    reference declares them as external subroutines with implicit interfaces,
 *    so gfortran passes every argument by reference and mangles the names to
 *    lowercase plus one trailing underscore.  Linking libtara.so in place of the
 *    reference's derive2csh.o / ab2csh.o / derive2css.o / ab2css.o / rk42css.o
 *    substitutes them without touching the caller.  Arrays are the caller's
 *    host arrays in Fortran layout: complex(8) a(Nh,Ny) is Nh*Ny interleaved
 *    (re,im) doubles with the kx index fastest, Nh = Nx/2+1.  Each call copies
 *    its inputs to the GPU, runs there and copies its outputs back; only the
 *    outputs the reference writes are written.  The subroutines return nothing
 *    (as in the reference); a failure is recorded and read back with
 *    tara_last_error().
 *
 * 2. A device-resident solver (tara2d_*) that keeps the state in HBM and runs
 *    many steps per call, plus batched ensembles (tara_ens_*).  These return an
 *    int status (TARA_OK = 0).
 *
 * Grid sizes: Nx and Ny powers of two from 16 to 4096 (the 2D paths; 3D: 16 to 512).
 * The 2D paths in FP64 (the derive2csh_ / derive2css_ / ab2csh_ / ab2css_ /
 * rk42css_ / derive2coh_ / derive2com_ drop-ins, tara2d_* with TARA_PREC_FP64,
 * tara_coh2d_* and tara_com2d_*, tara_fft2d_* in FP64 and the tara2dHydSer /
 * tara2dScrSer / tara2dHydOMP / tara2dMHDOMP programs) also take even lengths
 * from 8 to 3600 whose only prime factors are 2, 3, 5 and 7 (mixed-radix passes).
 */
#ifndef TARA_H
#define TARA_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------- */
#define TARA_OK 0
#define TARA_ERR_ARGS 1       /* bad sizes, null pointers, unsupported config   */
#define TARA_ERR_CUDA 2       /* a CUDA runtime call failed                      */
#define TARA_ERR_NONFINITE 3  /* NaN/Inf found by the energy/enstrophy reduction */
#define TARA_ERR_NOMEM 4      /* device allocation failed                        */
#define TARA_ERR_TIMEOUT 5    /* a bounded device-side wait gave up              */
#define TARA_ERR_INI 6        /* input.ini missing, malformed or missing a key    */

/* Last status recorded on the calling thread by any entry point, and its message. */
int tara_last_error(void);
const char* tara_last_error_message(void);
void tara_clear_error(void);

/* ---- 1. Fortran drop-ins (gfortran mangling) ----------------------------- */

/* Replaces subroutine derive2csh (src/derive2csh.f95:3).  Plain vorticity RHS:
 * writes dt_omegak_new = -(dealiased u.grad(omega) + nu k^2 omegak).  Reads
 * omegak; time, omegak_new and dt_omegak_old are unused, as in the reference.
 * Wavenumbers are the reference's: kx = 2*pi*(i-1)/Lx with pi = 3.1428 (real*4)
 * and Lx = Ly = 2*pi, i.e. integers. */
void derive2csh_(const int* Nx, const int* Ny, const int* Nh, const double* nu,
                 const double* time, double* omegak, double* omegak_new,
                 double* dt_omegak_old, double* dt_omegak_new);

/* Replaces subroutine ab2csh (src/ab2csh.f95:3):
 * omegak_new = omegak + (3/2 dt_omegak_new - 1/2 dt_omegak_old) dt. */
void ab2csh_(const int* Nx, const int* Ny, const int* Nh, const double* nu, const double* time,
             const double* dt, double* omegak, double* omegak_new, double* dt_omegak_old,
             double* dt_omegak_new);

/* Replaces subroutine derive2css (src/derive2css.f95:6).  Screened RHS with
 * psi = omega/(k^2+lambda), derivatives of k^2 psi, NL = alpha(...) + nu k^2 (k^2 psi).
 * The reference reads Lx, Ly and lambda from uninitialised locals; here they come
 * from tara_set_css_params (defaults Lx = Ly = 2*3.1428, lambda = 10). */
void derive2css_(const int* Nx, const int* Ny, const int* Nh, const double* alpha,
                 const double* nu, const double* time, double* omegak, double* omegak_new,
                 double* dt_omegak_old, double* dt_omegak_new);

/* Replaces subroutine ab2css (src/ab2css.f95:6); same update as ab2csh_. */
void ab2css_(const int* Nx, const int* Ny, const int* Nh, const double* alpha, const double* nu,
             const double* time, const double* dt, double* omegak, double* omegak_new,
             double* dt_omegak_old, double* dt_omegak_new);

/* Replaces subroutine rk42css (src/rk42css.f95:6) with a working classic RK4 over
 * the derive2css RHS: writes omegak_new; dt_omegak_old and dt_omegak_new are
 * unused.  (The reference body reads an uninitialised local and does not
 * integrate anything.) */
void rk42css_(const int* Nx, const int* Ny, const int* Nh, const double* alpha, const double* nu,
              const double* time, const double* dt, double* omegak, double* omegak_new,
              double* dt_omegak_old, double* dt_omegak_new);

/* Box lengths (true lengths, e.g. 2*pi*Lx_ini) and screening used by
 * derive2css_ / rk42css_.  The reference driver sets lambda = 10
 * (src/main2css.f95:87). */
void tara_set_css_params(double lx, double ly, double lambda);

/* Frees the device contexts (arrays, tables, streams) that the Fortran drop-ins
 * keep per grid shape, the owners of the device side of every drop-in call; the
 * next drop-in call creates its context again.  Handles made by the *_create
 * calls belong to the caller and are not touched.  Call it while no drop-in call
 * runs on another thread.  No counterpart in the reference, whose subroutines
 * allocate their work arrays and FFTW plans per call. */
int tara_finalize(void);

/* ---- 2. Device-resident solver ------------------------------------------- */

#define TARA_RHS_PLAIN 0   /* derive2csh */
#define TARA_RHS_SCREEN 1  /* derive2css (defined mode) */
#define TARA_SCHEME_AB2 0
#define TARA_SCHEME_RK4 1
#define TARA_PREC_FP64 0   /* FFTs, products and state in FP64 */
#define TARA_PREC_FP32 1   /* FP32 FFTs and products; FP64 state and reductions */
#define TARA_PREC_DF64 2   /* double-float (FP32 pair) FFTs and products; FP64 state */

typedef struct tara2d_config {
  int nx, ny;      /* powers of two, 16..4096; in FP64 also even 8..3600 with factors 2, 3, 5, 7 */
  int rhs;         /* TARA_RHS_* */
  int scheme;      /* TARA_SCHEME_* */
  int precision;   /* TARA_PREC_* */
  double nu;       /* viscosity */
  double dt;       /* time step */
  double alpha;    /* screened RHS: coefficient of the nonlinear term */
  double lambda;   /* screened RHS: screening */
  double lx, ly;   /* box lengths used in kx = 2*kpi*(i-1)/lx */
  double kpi;      /* the pi in that formula: 3.1428f for the reference's RHS */
  int batch;       /* independent runs of this shape advanced together (>= 1) */
} tara2d_config;

/* Fills cfg with the reference plain RHS defaults (pi = 3.1428f, Lx = Ly = 2*pi,
 * AB2, FP64). */
void tara2d_default_config(tara2d_config* cfg, int nx, int ny);

typedef struct tara2d tara2d;

int tara2d_create(const tara2d_config* cfg, tara2d** out);
int tara2d_destroy(tara2d* h);
/* Host half spectra in Fortran layout (Nh*Ny complex).  dt_old may be NULL
 * (the AB2 history is then zero, as the reference's fresh allocation reads). */
int tara2d_set_state(tara2d* h, const double* omegak, const double* dt_old);
int tara2d_get_state(tara2d* h, double* omegak, double* dt_old);
/* The same for run `run` of a batched handle (the calls above address run 0). */
int tara2d_set_state_run(tara2d* h, int run, const double* omegak, const double* dt_old);
int tara2d_get_state_run(tara2d* h, int run, double* omegak, double* dt_old);
/* Device pointers (dense Nh*Ny complex) on the handle's device. */
int tara2d_set_state_device(tara2d* h, const void* omegak_dev, const void* dt_old_dev);
int tara2d_get_state_device(tara2d* h, void* omegak_dev);
/* Advance nsteps steps on the handle's stream (asynchronous). */
int tara2d_step(tara2d* h, int nsteps);
/* As tara2d_step, with a CUDA event recorded on the handle's stream after every
 * launch; waits for completion and returns, per kernel kind (0 column inverse
 * pass, 1 row pass, 2 column forward + update pass), the summed milliseconds
 * and launch counts, and the total milliseconds of the nsteps steps (total_ms
 * may be NULL). */
int tara2d_step_timed(tara2d* h, int nsteps, double* kernel_ms, int* kernel_launches,
                      double* total_ms);
/* One RHS evaluation of the current state into a host array (dense Nh*Ny complex). */
int tara2d_rhs(tara2d* h, double* dt_omegak);
/* 1/2<|u|^2> and 1/2<omega^2> of the current state in the box (lx, ly) of the
 * config, from the spectrum by Parseval; TARA_ERR_NONFINITE when NaN/Inf. */
int tara2d_diag(tara2d* h, double* energy, double* enstrophy);
int tara2d_diag_run(tara2d* h, int run, double* energy, double* enstrophy);
int tara2d_synchronize(tara2d* h);
/* The handle's CUDA stream (cudaStream_t) for callers that order work around it. */
void* tara2d_stream(tara2d* h);
/* Number of kernel launches a single step issues (for launch accounting). */
int tara2d_launches_per_step(const tara2d* h);
/* Configurations of the three step kernels (column inverse pass, row pass,
 * column forward pass): an index c = tile variant + 4 * radix-8 path.  Tile
 * variants: 0 the default tile, 1 half of it, 2 one column / one row pair per
 * CTA (small grids, whose FP64 work would otherwise sit on a few SMs; in the
 * column passes also 4x the threads per column); the row pass also has 3, one
 * row pair in three shared-memory slots with half the threads (two CTAs share
 * an SM).  Radix path: the transforms run radix-4 stages (c < 4) or radix-8
 * stages first (c >= 4; FP64 and FP32 only) -- the same transform, rounded
 * differently, so the two paths agree to rounding, not bit for bit; tile
 * variants on one path agree bit for bit.  tara2d_autotune times all kernels
 * per candidate (a settling step, then trial_steps timed steps), then each
 * kernel's candidates with the other two at that first choice (again a
 * settling step and trial_steps timed), keeps the fastest per kernel in that
 * context and restores the state; variants3 and ms24 (per-launch ms in
 * context, candidate-major: 8 candidates x 3 kernels, 0 where a kernel has no
 * such candidate) may be NULL. */
int tara2d_autotune(tara2d* h, int trial_steps, int* variants3, double* ms24);
int tara2d_set_variants(tara2d* h, const int* variants3);

/* Driver diagnostics in the reference's form.  Wavenumbers kx = 2*kpi*i/lx
 * (the drivers use the true pi and Lx = Lx_ini*pi); screened != 0 applies the
 * screened driver's psi = omega/(k^2+lambda) on the ky >= 0 half only
 * (src/main2css.f95:215 vs :226), screened = 0 the plain driver's psi = omega/k^2. */
typedef struct tara2d_diag_params {
  double kpi, lx, ly, lambda;
  int screened;
} tara2d_diag_params;
/* usq = sum over the grid of ux^2+uy^2 and uysq = sum of uy^2, with u from c2r
 * divided by Nx*Ny (src/main2css.f95:253-259 "Energy" and its uy part). */
int tara2d_diag_reference(tara2d* h, const tara2d_diag_params* dp, double* usq, double* uysq);
/* Real (Nx,Ny) fields psi, omega (k^2 psi when screened), ux, uy of the current
 * state, normalised as the drivers normalise them; any pointer may be NULL. */
int tara2d_real_fields(tara2d* h, const tara2d_diag_params* dp, double* psi, double* omega,
                       double* ux, double* uy);

/* Seeded random-phase initial spectrum (Philox4x32-10, E(k) ~ k^4 exp(-(k/k0)^2),
 * Hermitian-projected on the GPU by a c2r/r2c round trip, mean mode zeroed,
 * rescaled to 1/2<|u|^2> = energy with the handle's wavenumbers). */
int tara2d_init_random(tara2d* h, double k0, double energy, uint64_t seed);
int tara2d_init_random_run(tara2d* h, int run, double k0, double energy, uint64_t seed);

/* ---- ensembles of runs of uneven sizes ------------------------------------ */

/* One run: grid n x n (power of two in [16, 4096]) with a seeded random-phase
 * initial spectrum (tara2d_init_random's recipe with this k0 and seed). */
typedef struct tara_ens_run {
  int n;
  double k0;
  uint64_t seed;
} tara_ens_run;

typedef struct tara_ens tara_ens;

/* Runs of one size are advanced by the same launches (a batched handle per size);
 * all sizes share nu, dt, scheme and precision (TARA_PREC_FP32: FP32 transforms
 * and products, FP64 state and reductions).  Plain RHS, 2*pi box. */
int tara_ens_create(int nruns, const tara_ens_run* runs, int precision, int scheme, double nu,
                    double dt, double energy, tara_ens** out);
int tara_ens_destroy(tara_ens* e);
/* Runs tara2d_autotune(trial_steps) on each size group (all kernels per
 * candidate, then each kernel's candidates in the context of the others'
 * choice) and keeps the fastest per kernel and size, then times the graph
 * against the persistent form (both radix paths) and keeps the fastest form;
 * the state is saved and restored around it. */
int tara_ens_autotune(tara_ens* e, int trial_steps);
/* Advances every run nsteps steps, asynchronously, in the ensemble's form:
 * TARA_ENS_GRAPH, one CUDA-graph launch per step (the graph, one parallel
 * branch per size, is captured on first use); TARA_ENS_PERSISTENT4 / 8, one
 * cooperative launch for all nsteps steps of every size (grid-wide barriers
 * between the passes, work items taken from a counter), with the transforms
 * on the radix-4 or radix-8 path -- FP32 form, RK4 and square grids whose
 * tiles fit the kernel's 256-thread CTAs (128, 256, 512) only.
 * tara_ens_autotune times the three and keeps the fastest; tara_ens_set_form
 * fixes one.  No counterpart in the reference. */
#define TARA_ENS_GRAPH 0
#define TARA_ENS_PERSISTENT4 1
#define TARA_ENS_PERSISTENT8 2
int tara_ens_step(tara_ens* e, int nsteps);
int tara_ens_set_form(tara_ens* e, int form);
/* The current form and the autotuner's milliseconds per step of each form
 * (graph, persistent radix-4, persistent radix-8; 0 where not timed). */
int tara_ens_form(tara_ens* e, int* form, double* ms3);
int tara_ens_synchronize(tara_ens* e);
/* The stream the graph launches on (cudaStream_t). */
void* tara_ens_stream(tara_ens* e);
int tara_ens_get_state(tara_ens* e, int run, double* omegak);
int tara_ens_set_state(tara_ens* e, int run, const double* omegak);
int tara_ens_diag(tara_ens* e, int run, double* energy, double* enstrophy);
int tara_ens_groups(tara_ens* e);
/* Size group info: n, number of runs, chosen configurations of the three
 * kernels, and the autotuner's per-launch milliseconds (8 candidates x three
 * kernels, as tara2d_autotune's ms24). */
int tara_ens_group_info(tara_ens* e, int group, int* n, int* runs, int* variants3,
                        double* tuned_ms24);
/* Kernel launches one ensemble step contains (inside its graph). */
int tara_ens_launches_per_step(tara_ens* e);

/* ---- 3D compressible MHD (derive3com / ab3com) --------------------------- */

/* Replaces subroutine derive3com (src/derive3com.f95:6): writes the eight
 * d_*_k_dt_new arrays (rho, rho ux, rho uy, rho uz, E, Bx, By, Bz) from the eight
 * state spectra; the *_old arrays and time are unused.  Arrays are complex(8)
 * (Nh,Ny,Nz).  Lx, Ly, Lz, mu, eta, CS are read from the caller's common block
 * /comm/ (comm_), wavenumbers use the pi argument; viscosity and resistivity are
 * the reference's hard-coded 1/450.  The forcing the reference transforms but
 * never uses is not computed.  Sizes: powers of two in [16, 512]. */
void derive3com_(const int* Nx, const int* Ny, const int* Nz, const int* Nh, const double* pi,
                 const double* time, const double* rho_k, const double* rho_ux_k,
                 const double* rho_uy_k, const double* rho_uz_k, const double* E_k,
                 const double* Bx_k, const double* By_k, const double* Bz_k, double* d_rho_k_dt_old,
                 double* d_rho_k_dt_new, double* d_rho_ux_k_dt_old, double* d_rho_ux_k_dt_new,
                 double* d_rho_uy_k_dt_old, double* d_rho_uy_k_dt_new, double* d_rho_uz_k_dt_old,
                 double* d_rho_uz_k_dt_new, double* d_E_k_dt_old, double* d_E_k_dt_new,
                 double* d_Bx_k_dt_old, double* d_Bx_k_dt_new, double* d_By_k_dt_old,
                 double* d_By_k_dt_new, double* d_Bz_k_dt_old, double* d_Bz_k_dt_new);

/* Replaces subroutine ab3com (src/ab3com.f95:6): AB2 into the *_new state arrays
 * with dt from /comm/; E is carried over unchanged, as the reference leaves it. */
void ab3com_(const int* Nx, const int* Ny, const int* Nz, const int* Nh, const double* pi,
             const double* time, const double* rho_k, const double* rho_ux_k,
             const double* rho_uy_k, const double* rho_uz_k, const double* E_k, const double* Bx_k,
             const double* By_k, const double* Bz_k, double* rho_k_new, double* rho_ux_k_new,
             double* rho_uy_k_new, double* rho_uz_k_new, double* E_k_new, double* Bx_k_new,
             double* By_k_new, double* Bz_k_new, const double* d_rho_k_dt_old,
             const double* d_rho_k_dt_new, const double* d_rho_ux_k_dt_old,
             const double* d_rho_ux_k_dt_new, const double* d_rho_uy_k_dt_old,
             const double* d_rho_uy_k_dt_new, const double* d_rho_uz_k_dt_old,
             const double* d_rho_uz_k_dt_new, const double* d_E_k_dt_old, const double* d_E_k_dt_new,
             const double* d_Bx_k_dt_old, const double* d_Bx_k_dt_new, const double* d_By_k_dt_old,
             const double* d_By_k_dt_new, const double* d_Bz_k_dt_old, const double* d_Bz_k_dt_new);

/* ---- 2D compressible isothermal hydro (derive2coh / ab2coh) ------------- */

/* Replaces subroutine derive2coh (src/derive2coh.f95:6): writes dn_dt_new,
 * dux_dt_new, duy_dt_new from the density and velocity spectra nk, ukx, uky
 * (complex(8) (Nh,Ny)); the *_old arrays and time are unused.  Lx, Ly, mux, muy,
 * CS come from the caller's common block /comm/ (comm_, the layout
 * Lx,Ly,mux,muy,ms,CS,dt of src/derive2coh.f95:30); wavenumbers use the pi
 * argument.  Sizes: powers of two in [16, 4096], or even 8..3600 with factors 2, 3, 5, 7. */
void derive2coh_(const int* Nx, const int* Ny, const int* Nh, const double* pi, const double* time,
                 const double* nk, const double* ukx, const double* uky, double* dn_dt_old,
                 double* dux_dt_old, double* duy_dt_old, double* dn_dt_new, double* dux_dt_new,
                 double* duy_dt_new);

/* Replaces subroutine ab2coh (src/ab2coh.f95:5): AB2 of the three fields with dt
 * from /comm/. */
void ab2coh_(const int* Nx, const int* Ny, const int* Nh, const double* pi, const double* time,
             const double* nk, const double* ukx, const double* uky, double* nk_new, double* ukx_new,
             double* uky_new, const double* dn_dt_old, const double* dux_dt_old,
             const double* duy_dt_old, const double* dn_dt_new, const double* dux_dt_new,
             const double* duy_dt_new);

typedef struct tara_coh2d_config {
  int nx, ny;        /* powers of two, 16..4096, or even 8..3600 with factors 2, 3, 5, 7 */
  double kpi;        /* the pi of kx = 2*pi*(i-1)/Lx */
  double lx, ly;     /* box lengths */
  double mux, muy;   /* viscosities (the reference driver: 0.0002) */
  double cs;         /* sound speed CS (the reference driver: U0/M = 3.77) */
  double dt;         /* AB2 time step */
} tara_coh2d_config;

typedef struct tara_coh2d tara_coh2d;

/* The reference driver's values (src/main2coh.f95): 2 pi box, true pi. */
void tara_coh2d_default_config(tara_coh2d_config* cfg, int nx, int ny);
int tara_coh2d_create(const tara_coh2d_config* cfg, tara_coh2d** out);
int tara_coh2d_destroy(tara_coh2d* h);
/* state3 = nk, ukx, uky as three dense complex (Nh,Ny) arrays back to back;
 * hist3 the AB2 history (dn_dt_old, dux_dt_old, duy_dt_old) or NULL for zero. */
int tara_coh2d_set_state(tara_coh2d* h, const double* state3, const double* hist3);
int tara_coh2d_get_state(tara_coh2d* h, double* state3, double* hist3);
/* derive2coh of the current state into d3 (three dense spectra) */
int tara_coh2d_rhs(tara_coh2d* h, double* d3);
/* nsteps of derive2coh + ab2coh + the history rotation (enqueued on the stream) */
int tara_coh2d_step(tara_coh2d* h, int nsteps);
int tara_coh2d_synchronize(tara_coh2d* h);
void* tara_coh2d_stream(tara_coh2d* h);
int tara_coh2d_launches_per_step(tara_coh2d* h);
/* The driver's initial state (src/main2coh.f95:140-210): n = 1, a vorticity disk
 * and five point vortices, velocity from the streamfunction; Lx = lx_ini*pi.
 * Zero history. */
int tara_coh2d_init_vortices(tara_coh2d* h, double lx_ini, double ly_ini);
/* The driver's per-step record (src/main2coh.f95:388-429) of the current state:
 * out6 = Energy/(2NxNy), y_Energy/(2NxNy), C0..C3/(NxNy) with Energy = sum of
 * ux^2+uy^2, y_Energy = sum of uy^2, Cp = sum of omega^p over the grid. */
int tara_coh2d_diag(tara_coh2d* h, double* out6);
/* n, ux, uy, omega on the grid, each [Ny][Nx] (NULL skips a field). */
int tara_coh2d_real_fields(tara_coh2d* h, double* n, double* ux, double* uy, double* omega);

/* ---- 2D compressible MHD (derive2com / ab2com) --------------------------- */

/* Replaces subroutine derive2com (src/derive2com.f95:5): writes the six
 * d_*_k_dt_new arrays (rho, rho ux, rho uy, E, Bx, By) from the six state spectra;
 * the *_old arrays and time are unused.  Lx, Ly, mu, CS, eta, kf, A come from the
 * caller's /comm/ (comm_, the layout Lx,Ly,spheat,mu,ms,CS,mu_0,eta,dt,kf,A of
 * src/derive2com.f95:43).  Faithful to the reference's curl B (built from
 * d_ux_dx and d_uy_dy, :186-187); the forcing uses the grid coordinates the
 * reference leaves unset.  Sizes: powers of two in [16, 4096], or even 8..3600 with
 * factors 2, 3, 5, 7. */
void derive2com_(const int* Nx, const int* Ny, const int* Nh, const double* pi, const double* time,
                 const double* rho_k, const double* rho_ux_k, const double* rho_uy_k,
                 const double* E_k, const double* Bx_k, const double* By_k, double* d_rho_k_dt_old,
                 double* d_rho_k_dt_new, double* d_rho_ux_k_dt_old, double* d_rho_ux_k_dt_new,
                 double* d_rho_uy_k_dt_old, double* d_rho_uy_k_dt_new, double* d_E_k_dt_old,
                 double* d_E_k_dt_new, double* d_Bx_k_dt_old, double* d_Bx_k_dt_new,
                 double* d_By_k_dt_old, double* d_By_k_dt_new);

/* Replaces subroutine ab2com (src/ab2com.f95): AB2 of the six fields with dt from
 * /comm/. */
void ab2com_(const int* Nx, const int* Ny, const int* Nh, const double* pi, const double* time,
             const double* rho_k, const double* rho_ux_k, const double* rho_uy_k, const double* E_k,
             const double* Bx_k, const double* By_k, double* rho_k_new, double* rho_ux_k_new,
             double* rho_uy_k_new, double* E_k_new, double* Bx_k_new, double* By_k_new,
             const double* d_rho_k_dt_old, const double* d_rho_k_dt_new,
             const double* d_rho_ux_k_dt_old, const double* d_rho_ux_k_dt_new,
             const double* d_rho_uy_k_dt_old, const double* d_rho_uy_k_dt_new,
             const double* d_E_k_dt_old, const double* d_E_k_dt_new, const double* d_Bx_k_dt_old,
             const double* d_Bx_k_dt_new, const double* d_By_k_dt_old, const double* d_By_k_dt_new);

typedef struct tara_com2d_config {
  int nx, ny;      /* powers of two, 16..4096, or even 8..3600 with factors 2, 3, 5, 7 */
  int defined;     /* 0: curl B as the reference (from d_ux_dx, d_uy_dy); 1: from dB/dx, dB/dy */
  double kpi;      /* the pi of kx = 2*pi*(i-1)/Lx */
  double lx, ly;   /* box lengths */
  double mu, eta;  /* viscosity (ini nu), resistivity (the reference driver: 1e-4) */
  double cs;       /* sound speed, P = CS^2 rho (the reference driver: 1/M = 100) */
  double kf, a;    /* forcing wavenumber and amplitude (the reference driver: 1, 1) */
  double dt;       /* AB2 time step */
} tara_com2d_config;

typedef struct tara_com2d tara_com2d;

void tara_com2d_default_config(tara_com2d_config* cfg, int nx, int ny);
int tara_com2d_create(const tara_com2d_config* cfg, tara_com2d** out);
int tara_com2d_destroy(tara_com2d* h);
/* state6 = rho, rho ux, rho uy, E, Bx, By as six dense complex (Nh,Ny) arrays;
 * hist6 the AB2 history or NULL for zero. */
int tara_com2d_set_state(tara_com2d* h, const double* state6, const double* hist6);
int tara_com2d_get_state(tara_com2d* h, double* state6, double* hist6);
int tara_com2d_rhs(tara_com2d* h, double* d6);
int tara_com2d_step(tara_com2d* h, int nsteps);
int tara_com2d_synchronize(tara_com2d* h);
void* tara_com2d_stream(tara_com2d* h);
int tara_com2d_launches_per_step(tara_com2d* h);
/* The driver's initial state (src/main2com.f95:229-291) with the handle's CS
 * and kf: rho = 1, ux = -sin(kf y), uy = sin(kf x), Bx = By = b0, Lx = lx_ini*pi. */
int tara_com2d_init_reference(tara_com2d* h, double lx_ini, double ly_ini, double b0);
/* The driver's record (src/main2com.f95:556-580) of the current state:
 * out5 = Energy, B_Field, C2, C3, div_B_Tot, the sums over the grid of
 * (ux^2+uy^2)/N^2, (Bx^2+By^2)/N^2, omega^2/N^2, j^2/N^2, divB/N^2 (N^2 = NxNy,
 * omega and j the curls of u and B). */
int tara_com2d_diag(tara_com2d* h, double* out5);
/* rho, ux, uy, P = CS^2 rho, E, Bx, By on the grid, each [Ny][Nx] (NULL skips). */
int tara_com2d_real_fields(tara_com2d* h, double* rho, double* ux, double* uy, double* P, double* E,
                           double* Bx, double* By);

typedef struct tara3d_config {
  int nx, ny, nz;      /* powers of two, 16..512 */
  int defined;         /* 0: k^2 f / 450 as the reference; 1: nu_u k^2 u and eta_b k^2 B */
  double kpi;          /* the pi of kx = 2*pi*(i-1)/Lx */
  double lx, ly, lz;   /* box lengths (the reference driver uses Lx = Lx_ini * pi) */
  double mu;           /* coefficient of E_Visc in the energy equation (ini nu) */
  double eta;          /* resistivity in the energy flux (0.005 in the reference) */
  double cs;           /* sound speed, P = CS^2 rho (10 in the reference) */
  double nu_u, eta_b;  /* defined-mode viscosity and resistivity */
  double dt;
} tara3d_config;

typedef struct tara3d tara3d;

/* Reference defaults: 2*pi box, mu = 0.01, eta = 0.005, CS = 10, faithful 1/450. */
void tara3d_default_config(tara3d_config* cfg, int nx, int ny, int nz);
int tara3d_create(const tara3d_config* cfg, tara3d** out);
int tara3d_destroy(tara3d* h);
/* eight dense (Nh,Ny,Nz) complex spectra in the order rho, rho ux, rho uy, rho uz,
 * E, Bx, By, Bz; hist8 (the AB2 history) may be NULL for zero history. */
int tara3d_set_state(tara3d* h, const double* state8, const double* hist8);
int tara3d_get_state(tara3d* h, double* state8, double* hist8);
/* eight real (Nx,Ny,Nz) fields in the same order, transformed on the GPU */
int tara3d_set_state_real(tara3d* h, const double* real8);
/* The 3D MHD benchmark's initial state (no counterpart in the reference, whose
 * own 3D initial state is the ABC flow of src/main3com.f95:301-319):
 * rho = 1, u = (-sin y, sin x, 0) + du, B = (-sin y, sin 2x, 0) + dB,
 * E = 1 + |u|^2/2 + |B|^2/2 on the 2 pi grid x_i = 2 pi i / Nx, where du and dB
 * are seeded random-phase solenoidal fields on the modes 0 < |k| <= kmax
 * (Philox4x32-10 phases at counter (i, j, k, 3 f + c), f = 0 for u and 1 for B,
 * c the component; projected onto k.a = 0; kx = 0 plane Hermitian) scaled to
 * amp times the base fields' r.m.s. (1).  The benchmark uses amp = 0.01,
 * kmax = 4, seed 3.  History set to zero.  Needs 2 kmax < Nx, Ny, Nz. */
int tara3d_init_orszag_tang(tara3d* h, double amp, int kmax, uint64_t seed);
/* nsteps of derive3com + ab3com + the driver's history rotation (E frozen) */
int tara3d_step(tara3d* h, int nsteps);
/* all eight derivatives of the current state (dense spectra), as derive3com */
int tara3d_rhs(tara3d* h, double* d8);
int tara3d_synchronize(tara3d* h);
/* The handle's CUDA stream (cudaStream_t). */
void* tara3d_stream(tara3d* h);
/* The first columns of the reference's 3D Energy.dat (src/main3com.f95:1024-1070)
 * for the current state: out4 = {Pressure = <CS^2 rho>, Energy = <|u|^2>/2,
 * T_Energy = <E>, B_Field = <|B|^2>/2}, u = (rho u)/rho in real space. */
int tara3d_diag(tara3d* h, double* out4);

/* ---- input.ini driver ----------------------------------------------------- */

/* Runs the solver an input.ini selects, as the reference's program TARA2D does
 * (src/main.f95:24-89): dim=2 serial bare -> the plain vorticity loop of
 * tara2dHydSer (src/main2csh.f95), dim=2 serial screen -> tara2dScrSer
 * (src/main2css.f95), dim=3 openmp mhd -> tara3dMHDOMP (src/main3com.f95);
 * arch cpu and single-gpu both run on the GPU.  Output files go to out_dir
 * (the reference writes ./output).  max_steps > 0 caps the number of steps
 * (0: the full time_min..time_max loop).  Returns TARA_ERR_INI for a missing or
 * malformed ini key, TARA_ERR_ARGS for a solver this library does not implement. */
int tara_run_ini(const char* ini_path, const char* out_dir, int max_steps);

/* cfg%gets of the reference's ini parser: the value of section/key with the
 * DEFAULTS fallback, quotes stripped and ${sec:key} interpolated. */
int tara_ini_get(const char* path, const char* section, const char* key, char* buf, int buflen);
/* Fortran list-directed read of one REAL(8) / INTEGER from a string, e.g.
 * "0.010d0" -> 0.01 and "3.0d0/128.0d0" -> 3.0 (the slash ends the read). */
int tara_fortran_read_double(const char* s, double* out);
int tara_fortran_read_int(const char* s, long long* out);
/* One list-directed output record of n REAL(8) values, gfortran style: 26
 * characters per value and a terminating NUL; a smaller buflen is refused
 * (TARA_ERR_ARGS, buf set to the empty string). */
int tara_fortran_list_record(const double* v, int n, char* buf, int buflen);
/* A snapshot file in the reference drivers' fort.* format: one record per grid
 * point, x outer and y inner, holding xs[i], ys[j] and fields[k*nx*ny + j*nx + i]
 * for k < nfields (the same records as tara_fortran_list_record), formatted in
 * parallel on the host's cores. */
int tara_write_grid_records(const char* path, int nx, int ny, const double* xs, const double* ys,
                            const double* fields, int nfields);

/* ---- Lagrangian passive particles ------------------------------------------ */
/* The plain serial driver's particles (src/main2csh.f95:93-96, 187-273): after a
 * step, u_x = i ky psi, u_y = -i kx psi with psi = omega/(kx^2+ky^2) and the
 * driver's wavenumbers kx = 2*kpi*i/lx (true pi, ini box) are transformed to the
 * grid (c2r / (Nx*Ny)), interpolated bilinearly at each particle and the particle
 * moves one Euler step, wrapped into (0, L] as the reference does.  Where the
 * reference's last-column / last-row branches read outside ux(Nx,Ny), the
 * neighbour wraps periodically (defined behaviour).  Positions live on the
 * device; run 0 of the handle drives them. */
typedef struct tara_particles tara_particles;
int tara_particles_create(tara2d* h, double kpi, double lx, double ly, int np, const double* xp,
                          const double* yp, tara_particles** out);
int tara_particles_destroy(tara_particles* p);
/* One Euler step of length dt with the current state's velocity (asynchronous,
 * on the solver's stream; call it after tara2d_step as the reference driver does). */
int tara_particles_advance(tara_particles* p, double dt);
int tara_particles_get(tara_particles* p, double* xp, double* yp);
/* The minimal-standard LCG (Park & Miller 1988, a = 16807, m = 2^31-1) that GNU
 * Fortran documents for its RAND intrinsic, as a REAL(4) in [0,1); the driver
 * draws the initial positions xp = rand()*Lx, yp = rand()*Ly with it (state 1). */
float tara_park_miller_rand(uint64_t* state);

/* ---- standalone transforms ------------------------------------------------ */
/* Unnormalised 2D transforms with FFTW's rank-2 r2c/c2r semantics, i.e. what
 * dfftw_plan_dft_{r2c,c2r}_2d(plan, Nx, Ny, ...) computes in the reference
 * (src/derive2csh.f95:73-106, lib/fftw/api/f77funcs.h:206-209,300-303): c2r runs
 * complex DFTs along y and then a 1D c2r along x that reads only the real parts
 * of the kx = 0 and kx = Nx/2 bins.  Host arrays: real (Nx,Ny) x-fastest,
 * complex (Nh,Ny) interleaved.  precision TARA_PREC_FP64 or TARA_PREC_FP32 (the
 * transform arithmetic; inputs and outputs stay double). */
int tara_fft2d_r2c(int nx, int ny, int precision, const double* in, double* out);
int tara_fft2d_c2r(int nx, int ny, int precision, const double* in, double* out);

/* ---- learned subgrid closure ---------------------------------------------- */
/* No counterpart in the reference: a coarse-grid run of the plain vorticity
 * solver corrected by a Fourier neural operator (FNO) that predicts the
 * subgrid vorticity flux from the filtered vorticity.  The network is trained
 * on the GPU by the library's own forward/backward kernels on filtered
 * fine-grid snapshots that the plain solver generates (tara2d_filter).
 *
 * Network (per sample, activations H x W x channels, FP32):
 *   v0 = x Pw + Pb;  v_l = GELU(S_l(v_{l-1}) + v_{l-1} W_l + b_l), l = 1..L
 *   (no GELU after the last layer);  y = GELU(v_L Q1 + q1) Q2 + q2.
 * S_l keeps the Fourier modes kx in [0, mx), ky in [-my/2, my/2) of rfft2(v),
 * multiplies each by a complex c x c matrix and returns irfft2 of the result.
 * Flat parameter vector order: Pw (ci x c), Pb (c), then per layer R_l
 * (my x mx x c x c complex, ky index j = ky mod my, interleaved re/im), W_l
 * (c x c), b_l (c); then Q1 (c x p), q1 (p), Q2 (p x co), q2 (co).  Matrices
 * are row-major (input index first).  Grids are powers of two, c a multiple of
 * 8, p and co <= 256.  The handle works on its own non-blocking stream, which
 * does not wait for other streams: device inputs must be complete before a call
 * (as for the tara2d_* device-pointer entry points). */
typedef struct tara_fno tara_fno;
#define TARA_FNO_BF16 0  /* channel mixing on BF16 tensor cores, FP32 accumulators */
#define TARA_FNO_FP32 1  /* the same GEMMs on FP32 CUDA cores (gradient checks)    */
#define TARA_FNO_BF16_TMEM 2  /* as BF16, the tall-skinny channel GEMMs on tcgen05 with
                               * accumulators in tensor memory */
typedef struct tara_fno_config {
  int h, w;           /* grid (rows, columns) */
  int ci, c, co;      /* input, hidden and output channels */
  int mx, my;         /* retained modes: mx <= w/2, my even <= h */
  int layers, p;      /* Fourier layers (1..8), projection width */
  int max_batch;      /* samples per call */
  int mode;           /* TARA_FNO_* */
  uint64_t seed;      /* initial parameters: uniform(+-1/sqrt(fan_in)), R uniform(+-1/c^2) */
} tara_fno_config;
/* 128 x 128, ci 1, c 32, co 2, mx 16, my 32, 4 layers, p 128, batch 32, BF16. */
void tara_fno_default_config(tara_fno_config* c);
int tara_fno_create(const tara_fno_config* cfg, tara_fno** out);
int tara_fno_destroy(tara_fno* f);
size_t tara_fno_num_params(const tara_fno* f);
int tara_fno_get_params(tara_fno* f, float* host);
int tara_fno_set_params(tara_fno* f, const float* host);
/* Gradients of the last tara_fno_train_step (same layout as the parameters). */
int tara_fno_get_grads(tara_fno* f, float* host);
int tara_fno_set_mode(tara_fno* f, int mode);
/* Inference path of tara_fno_forward and the closure (enable != 0, the default):
 * in the BF16 modes, batches of at most 4 samples at W = 128, 32 channels,
 * p in {32, 64, 128, 256}, co <= 4, H <= 256, mx <= 16 and mx * my <= 512 run through fused
 * per-row and per-column kernels (lift + 2 launches per Fourier layer, the
 * pointwise and projection products on tcgen05); enable = 0 keeps the
 * layer-by-layer forward of the training step.  Same arithmetic up to the
 * order of FP32 sums. */
int tara_fno_set_fused(tara_fno* f, int enable);
/* y_dev (B,H,W,co) = FNO(x_dev (B,H,W,ci)); device FP32 arrays; synchronous. */
int tara_fno_forward(tara_fno* f, const float* x_dev, float* y_dev, int B);
/* Forward, loss = mean((y - t)^2), backward, then one Adam step (beta 0.9,
 * 0.999, eps 1e-8, bias-corrected) when lr > 0.  With idx_dev (B int32 sample
 * indices, device) the batch is gathered from datasets x_dev / t_dev of
 * n_samples samples (an index outside them returns TARA_ERR_ARGS); with idx_dev
 * NULL, x_dev / t_dev hold the batch itself (n_samples >= B). */
int tara_fno_train_step(tara_fno* f, const float* x_dev, const float* t_dev, const int* idx_dev,
                        int n_samples, int B, float lr, double* loss);
/* Adam steps taken so far; setting it restarts the bias correction count. */
long long tara_fno_adam_steps(const tara_fno* f);
void* tara_fno_stream(tara_fno* f);

/* Box filter of run `run` of a plain-solver handle onto the grid coarsened by
 * `factor` (block means of factor x factor cells; Nx, Ny divisible by it).
 * Device outputs, any may be NULL: omega_bar (Ny/f, Nx/f) FP32, flux
 * (Ny/f, Nx/f, 2) FP32 = the subgrid vorticity flux bar(u w) - bar(u) bar(w),
 * bar(v w) - bar(v) bar(w), omega_bar64 (Ny/f, Nx/f) FP64.  Velocities come
 * from the state with the solver's wavenumbers, in FP64. */
int tara2d_filter(tara2d* h, int run, int factor, float* omega_bar, float* flux,
                  double* omega_bar64);
/* Set run `run` to the r2c of a real vorticity field on the device (Nx x Ny,
 * x fastest, FP64); the AB2 history is zeroed. */
int tara2d_set_state_real_device(tara2d* h, int run, const double* omega_dev);
/* Shell energy spectrum of run `run`: E[k], k = 0..kmax, sums 1/2 |u_hat|^2 / (NxNy)^2
 * over the modes with round(|k|) = k (|k| in the solver's integer wavenumbers),
 * so that sum_k E[k] is the energy when kmax covers the grid. */
int tara2d_spectrum(tara2d* h, int run, int kmax, double* E);

/* Input features of the closure network from run `run`'s state, in real space
 * on the handle's grid: the first nf (1..6) of w, dw/dx, dw/dy, du/dx, du/dy,
 * dv/dx (u = d psi/dy, v = -d psi/dx, spectral derivatives, FP64), each times
 * scales[c] (NULL: 1), written as FP32 (Ny, Nx, nf) at out_dev. */
int tara2d_features(tara2d* h, int run, int nf, const double* scales, float* out_dev);

/* Training-set augmentation by the eight symmetries of the square periodic
 * grid (g = bit 0: x -> -x, bit 1: y -> -y, bit 2: transpose, in that order):
 * sample g*n_samples + i of the outputs is symmetry g of sample i.  x: features
 * (n_samples, n, n, nf) as tara2d_features writes them; t: subgrid fluxes
 * (n_samples, n, n, 2) as tara2d_filter writes them.  Reflections negate w and
 * the derivatives across them; the transpose swaps the x and y components.
 * Either input may be NULL.  Synchronous (legacy default stream). */
int tara_closure_augment(const float* x_dev, const float* t_dev, int n_samples, int n, int nf,
                         float* x_out, float* t_out);

/* A coarse plain-solver handle advanced with the FNO's subgrid flux: every
 * step evaluates y = FNO(features) with the network's ci feature channels
 * (tara2d_features, scaled by in_scales[0..ci-1]) on every run, takes
 * flux = out_scale * y and adds -div(flux) (2/3-truncated) to the right-hand
 * side of every stage of the step.  The handle and the network stay owned by
 * the caller and must outlive the closure; the network's batch must hold the
 * handle's runs and its grid must be the handle's. */
typedef struct tara_closure tara_closure;
int tara_closure_create(tara2d* coarse, tara_fno* fno, const double* in_scales, double out_scale,
                        tara_closure** out);
int tara_closure_destroy(tara_closure* c);
/* Advance nsteps closure steps (enqueued on the handle's stream). */
int tara_closure_step(tara_closure* c, int nsteps);

/* ---- allocation-free RHS ------------------------------------------------- */
/* No counterpart in the reference.  The plain RHS of derive2csh_ (same
 * arithmetic, same kernels) on caller-owned device arrays -- omegak_dev in,
 * dt_omegak_dev out, each a dense (Nh,Ny) complex(8) array, 16-byte aligned --
 * enqueued on `stream` (a cudaStream_t; NULL for the legacy default stream).
 * It performs no device allocation at all, for callers that cannot call
 * cudaMalloc: programs whose device memory is owned by another allocator or
 * reserved up front, and time loops that must not trigger the device-wide
 * synchronisation cudaMalloc/cudaFree can cause.  Its scratch is one
 * file-scope static device array of about 2.9 MB that every GPU loading the
 * library holds until exit, so grids are limited to Nx, Ny <= 256 (powers of
 * two); larger ones return TARA_ERR_ARGS.  The first call on a device resolves
 * the array's address, uploads twiddle tables and waits for the device
 * (cudaDeviceSynchronize), so make it before any stream capture.  All calls on
 * a device share the array: calls whose GPU work overlaps race and must be
 * serialised by the caller; calls one after another on one stream are safe.
 * Non-finite results are not reported: the call returns TARA_OK once its
 * launches are accepted, even when the output holds NaN or Inf (checking would
 * need a device-to-host read and a wait), so a caller that needs the check
 * tests dt_omegak_dev itself. */
int tara_derive2csh_noalloc(int nx, int ny, double nu, const void* omegak_dev,
                            void* dt_omegak_dev, void* stream);

/* Measured FP64 FMA throughput of the current device in thread-instructions
 * per second: one kernel of independent DFMA chains filling every SM, timed with
 * CUDA events over `reps` launches after a warm-up launch (about 20 ms each).
 * The measured denominator of the FP64-pipe roofline. */
int tara_measure_dfma_rate(int reps, double* inst_per_s);

/* The transforms' twiddle table of a power-of-two length n (16..4096) as the
 * device reads it, host only (no device call): *count entries of two doubles.
 * TARA_PREC_FP64 gives the FP64 table, whose twiddled radix-4 stage entries hold
 * the ratio form (tau, c) and (tau3, c3/c1), tau = s/c; TARA_PREC_FP32 the plain
 * twiddles (cos, -sin) before their rounding to FP32.  With out NULL only *count
 * is set; otherwise capacity must be at least *count. */
int tara_twiddle_table(int n, int precision, double* out, int capacity, int* count);

/* Library version string. */
const char* tara_version(void);

#ifdef __cplusplus
}
#endif
#endif
