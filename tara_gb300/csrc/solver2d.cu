// Device-resident 2D solver (tara2d_*), status handling, tables and the
// diagnostics reduction.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "internal.h"

namespace tara {

// ---------------------------------------------------------------------------
// status
// ---------------------------------------------------------------------------
static thread_local int g_err = TARA_OK;
static thread_local std::string g_msg;

int set_error(int code, const std::string& msg) {
  g_err = code;
  g_msg = msg;
  return code;
}
int set_ok() {
  g_err = TARA_OK;
  g_msg.clear();
  return TARA_OK;
}
ErrorState save_error() { return ErrorState{g_err, g_msg}; }
void restore_error(const ErrorState& s) {
  g_err = s.code;
  g_msg = s.msg;
}
int cuda_fail(cudaError_t e, const char* what) {
  const int code = (e == cudaErrorMemoryAllocation) ? TARA_ERR_NOMEM : TARA_ERR_CUDA;
  return set_error(code, std::string(what) + ": " + cudaGetErrorString(e));
}

// ---------------------------------------------------------------------------
// tables
// ---------------------------------------------------------------------------
// kx = 2.0d0*pi*dfloat(i-1)/Lx and ky = 2.0d0*pi*(dfloat(j-1)-Ny)/Ly above
// Ny/2 (src/derive2csh.f95:30,32,48); the 2/3 rule removes the nonlinear term
// where dsqrt(kx*kx+ky*ky) >= (dfloat(Nx+Ny)/2.0)/3.0 (src/derive2csh.f95:113).
// Evaluated on the host with the same expressions (no FMA contraction), so the
// tables equal the reference's values bit for bit; because kx grows with i, the
// removed set of row j is {i >= i0[j]}.
void make_wavenumbers(int nx, int ny, double kpi, double lx, double ly, double* kx, double* ky,
                      int* i0) {
  const int nh = nx / 2 + 1;
  for (int i = 0; i < nh; ++i) kx[i] = 2.0 * kpi * (double)i / lx;
  for (int j = 0; j < ny; ++j)
    ky[j] = (j < ny / 2) ? 2.0 * kpi * (double)j / ly : 2.0 * kpi * ((double)j - (double)ny) / ly;
  const double cut = ((double)(nx + ny) / 2.0) / 3.0;
  for (int j = 0; j < ny; ++j) {
    int first = nh;
    for (int i = nh - 1; i >= 0; --i) {
      if (std::sqrt(kx[i] * kx[i] + ky[j] * ky[j]) >= cut)
        first = i;
      else
        break;
    }
    i0[j] = first;
  }
}

void make_inverse_table(int nx, int ny, const double* kx, const double* ky, bool screened,
                        double lambda, double* inv) {
  const int nh = nx / 2 + 1;
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nh; ++i) {
      const double k2 = kx[i] * kx[i] + ky[j] * ky[j];
      inv[(size_t)j * nh + i] = (i == 0 && j == 0) ? 0.0 : 1.0 / (screened ? k2 + lambda : k2);
    }
}

void twiddle(int n, int m, double* re, double* im) {
  // exp(-2 pi i m/n) from long-double cos/sin on [0, n/2]; the quarter points
  // exact, and tw[n - m] = conj(tw[m]) exactly, so that an inverse transform
  // reads its conjugate twiddle by index instead of negating it
  const long double tp = 6.283185307179586476925286766559005768L;
  const int r = m <= n / 2 ? m : n - m;
  double c, s;
  if (4 * r == n) {
    c = 0.0;
    s = -1.0;
  } else if (r == 0 || 2 * r == n) {
    c = r == 0 ? 1.0 : -1.0;
    s = 0.0;
  } else {
    const long double a = tp * (long double)r / (long double)n;
    c = (double)std::cos(a);
    s = (double)-std::sin(a);
  }
  *re = c;
  *im = m <= n / 2 ? s : -s;
}

void twiddle_entry(int n, int idx, double* re, double* im) {
  if (idx < n) {
    twiddle(n, idx, re, im);
    return;
  }
  if (idx >= tw_m8_base(n)) {  // radix-4 stages after a radix-8 first stage (layout in fft.cuh)
    int t = idx - tw_m8_base(n);
    const int span = tw_m8_span(n);
    const bool inv = t >= span;
    if (inv) t -= span;
    int ns = 8;  // stage Ns owns [Ns - 8, 4 Ns - 8)
    while (4 * ns - 8 <= t) ns *= 4;
    const int off = t - (ns - 8);
    twiddle(n, (off / ns + 1) * (off % ns) * (n / (4 * ns)), re, im);
    if (inv) *im = -*im;
    return;
  }
  if (idx >= tw_r8_base(n)) {  // radix-8 path stage tables (layout in fft.cuh)
    int t = idx - tw_r8_base(n);
    const int span = r8_span(n);
    const bool inv = t >= span;
    if (inv) t -= span;
    int i = 1;
    while (t >= r8_stage_off(n, i) + r8_stage_size(n, i)) ++i;
    const int off = t - r8_stage_off(n, i), ns = r8_ns(n, i);
    const int run = off / ns, k = off % ns;
    int e;
    if (r8_radix(n, i) == 8) {
      const int m = k * (n / (8 * ns));
      e = run == 0 ? m : run == 1 ? 2 * m : run == 2 ? 4 * m : m + n / 8;
    } else {
      e = (run + 1) * k * (n / (4 * ns));
    }
    twiddle(n, e, re, im);
    if (inv) *im = -*im;
    return;
  }
  int t = idx - n;
  const int span = tw_stage_span(n);
  const bool inv = t >= span;
  if (inv) t -= span;
  int ns = 4;  // stage s owns [Ns - 4, 4 Ns - 4)
  while (4 * ns - 4 <= t) ns *= 4;
  const int off = t - (ns - 4);
  const int r = off / ns + 1, k = off % ns;
  twiddle(n, r * k * (n / (4 * ns)), re, im);
  if (inv) *im = -*im;
}

// Entry idx of the FP64 table: as twiddle_entry, except the twiddled radix-4
// stage entries (of the radix-4 path and of the radix-8-first path, fft.cuh),
// which take the ratio form of dft4_tw_ratio: (tau_r, c_r) for r = 1, 2 and
// (tau_3, c_3 / c_1) for r = 3, tau = s / c.  A zero cosine (the quarter turn,
// only ever w2 at k = Ns/2) becomes 2^-256 with tau = s 2^256: both exact
// powers of two, so c tau = s exactly.
void twiddle_entry_fp64(int n, int idx, double* a, double* b) {
  int start, span, first;  // the region, its per-direction size, its first Ns
  if (idx >= n && idx < n + 2 * tw_stage_span(n)) {
    start = n;
    span = tw_stage_span(n);
    first = 4;
  } else if (idx >= tw_m8_base(n) && idx < tw_m8_base(n) + 2 * tw_m8_span(n)) {
    start = tw_m8_base(n);
    span = tw_m8_span(n);
    first = 8;
  } else {
    twiddle_entry(n, idx, a, b);
    return;
  }
  int t = idx - start;
  const int base = t >= span ? start + span : start;
  if (t >= span) t -= span;
  int ns = first;  // stage Ns owns [Ns - first, 4 Ns - first)
  while (4 * ns - first <= t) ns *= 4;
  const int off = t - (ns - first);
  const int r = off / ns + 1, k = off % ns;
  auto entry = [&](int rr, double* c, double* s) {
    twiddle_entry(n, base + (ns - first) + (rr - 1) * ns + k, c, s);
    if (*c == 0.0) *c = std::ldexp(1.0, -256);
  };
  double c, s;
  entry(r, &c, &s);
  *a = s / c;
  if (r < 3) {
    *b = c;
  } else {
    double c1, s1;
    entry(1, &c1, &s1);
    *b = c / c1;
  }
}

int make_twiddles(int n, bool fp32, void** dev) {
  if (!is_pow2_in_range(n)) {  // the mixed-radix path: the n roots, FP64 only
    if (fp32 || !any_size_2d(n)) return set_error(TARA_ERR_ARGS, "twiddles: unsupported length");
    return any2d::make_roots(n, dev);
  }
  const int cnt = tw_count(n);
  if (fp32) {
    std::vector<float2> w(cnt);
    for (int m = 0; m < cnt; ++m) {
      double c, s;
      twiddle_entry(n, m, &c, &s);
      w[m] = make_float2((float)c, (float)s);
    }
    TARA_CK(cudaMalloc(dev, cnt * sizeof(float2)));
    TARA_CK(cudaMemcpy(*dev, w.data(), cnt * sizeof(float2), cudaMemcpyHostToDevice));
  } else {
    std::vector<double2> w(cnt);
    for (int m = 0; m < cnt; ++m) {
      double c, s;
      twiddle_entry_fp64(n, m, &c, &s);
      w[m] = make_double2(c, s);
    }
    TARA_CK(cudaMalloc(dev, cnt * sizeof(double2)));
    TARA_CK(cudaMemcpy(*dev, w.data(), cnt * sizeof(double2), cudaMemcpyHostToDevice));
  }
  return TARA_OK;
}

// The same table as double-float pairs (hi, lo) per component, for the
// double-float transforms: hi = fl32(w), lo = fl32(w - hi).
int make_twiddles_df64(int n, void** dev) {
  if (!is_pow2_in_range(n)) return set_error(TARA_ERR_ARGS, "the double-float form takes powers of two only");
  const int cnt = tw_count(n);
  std::vector<float4> w(cnt);
  for (int m = 0; m < cnt; ++m) {
    double c, s;
    twiddle_entry(n, m, &c, &s);
    const float ch = (float)c, sh = (float)s;
    w[m] = make_float4(ch, (float)(c - (double)ch), sh, (float)(s - (double)sh));
  }
  TARA_CK(cudaMalloc(dev, cnt * sizeof(float4)));
  TARA_CK(cudaMemcpy(*dev, w.data(), cnt * sizeof(float4), cudaMemcpyHostToDevice));
  return TARA_OK;
}

// ---------------------------------------------------------------------------
// diagnostics
// ---------------------------------------------------------------------------
constexpr int kDiagBlocks = 304, kDiagThreads = 256;

// Energy as the reference measures it: u from c2r of i ky psi and -i kx psi,
// psi = omega/k^2, summed over grid points.  The c2r keeps only real parts in the
// kx = 0 and kx = Nx/2 columns, which removes u_y of the whole kx = Nx/2 column
// and u_x of the ky = -Ny/2 row in those two columns (their derivatives vanish
// on the grid); every other mode counts by Parseval with weight 1 on the two
// edge columns and 2 elsewhere.
__global__ void __launch_bounds__(kDiagThreads)
    k_diag_partial(const double2* __restrict__ w, Grid2D g, double* __restrict__ part) {
  double e = 0.0, z = 0.0;
  const size_t total = (size_t)g.ny * g.nh;
  for (size_t t = (size_t)blockIdx.x * kDiagThreads + threadIdx.x; t < total;
       t += (size_t)gridDim.x * kDiagThreads) {
    const int y = (int)(t / g.nh), x = (int)(t % g.nh);
    const double2 v = w[(size_t)y * g.pitch + x];
    const bool edge_x = (x == 0 || 2 * x == g.nx);
    const double wt = edge_x ? 1.0 : 2.0;
    const double a2 = v.x * v.x + v.y * v.y;
    z += wt * a2;
    if (x != 0 || y != 0) {
      const double kx = g.kx[x], ky = g.ky[y];
      const double k2 = kx * kx + ky * ky;
      const double keep_ux = (edge_x && 2 * y == g.ny) ? 0.0 : ky * ky;
      const double keep_uy = (2 * x == g.nx) ? 0.0 : kx * kx;
      e += wt * a2 * (keep_ux + keep_uy) / (k2 * k2);
    }
  }
  __shared__ double se[kDiagThreads / 32], sz[kDiagThreads / 32];
  for (int o = 16; o > 0; o >>= 1) {
    e += __shfl_down_sync(0xffffffffu, e, o);
    z += __shfl_down_sync(0xffffffffu, z, o);
  }
  if ((threadIdx.x & 31) == 0) {
    se[threadIdx.x >> 5] = e;
    sz[threadIdx.x >> 5] = z;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double te = 0.0, tz = 0.0;
    for (int i = 0; i < kDiagThreads / 32; ++i) {
      te += se[i];
      tz += sz[i];
    }
    part[2 * blockIdx.x] = te;
    part[2 * blockIdx.x + 1] = tz;
  }
}

__global__ void k_diag_final(const double* __restrict__ part, int nparts, double inv,
                             double* __restrict__ out, unsigned int* flag) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double e = 0.0, z = 0.0;
  for (int i = 0; i < nparts; ++i) {
    e += part[2 * i];
    z += part[2 * i + 1];
  }
  out[0] = e * inv;
  out[1] = z * inv;
  if (!(isfinite(e) && isfinite(z))) atomicOr(flag, 2u);
}

// w *= s
__global__ void k_mul(double2* __restrict__ w, size_t n, double s) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const double2 v = w[i];
    w[i] = make_double2(v.x * s, v.y * s);
  }
}

// pointwise AB2 on dense arrays: out = w + (3/2 fn - 1/2 fo) dt  (src/ab2csh.f95:12)
__global__ void k_ab2_dense(const double2* w, double2* out, const double2* __restrict__ fo,
                            const double2* __restrict__ fn, size_t n, double dt) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const double2 a = w[i], b = fo[i], c = fn[i];
    out[i] = make_double2(a.x + ((3.0 / 2.0) * c.x - (1.0 / 2.0) * b.x) * dt,
                          a.y + ((3.0 / 2.0) * c.y - (1.0 / 2.0) * b.y) * dt);
  }
}

// ---------------------------------------------------------------------------
// driver diagnostics in the reference's form (src/main2css.f95:206-275,
// src/main2csh.f95:128-168): spectra of psi, omega_dum, u_x, u_y with the
// driver's wavenumbers, and the grid sums of u^2 through the c2r discard rule
// ---------------------------------------------------------------------------
// psi = omega/(k^2 + lam_row) with lam_row = lambda for j < Ny/2 and 0 above (the
// screened driver applies lambda to one half only, :215 vs :226; the plain
// driver passes lambda = 0); out[0..3] = psi, k^2 psi (screened) or omega
// (plain), (0,1) ky psi, -(0,1) kx psi.
__global__ void k_diag_spectra(const double2* __restrict__ w, Grid2D g, double lambda, int screened,
                               double2* __restrict__ out) {
  const size_t total = (size_t)g.ny * g.nh, fsz = (size_t)g.ny * g.pitch;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const int y = (int)(t / g.nh), x = (int)(t % g.nh);
    const size_t q = (size_t)y * g.pitch + x;
    const double2 v = w[q];
    const double kx = g.kx[x], ky = g.ky[y];
    const double k2 = kx * kx + ky * ky;
    double pr = 0.0, pim = 0.0;
    if (x != 0 || y != 0) {
      const double den = (screened && 2 * y < g.ny) ? k2 + lambda : k2;
      pr = v.x / den;
      pim = v.y / den;
    }
    out[q] = make_double2(pr, pim);
    out[fsz + q] = screened ? make_double2(k2 * pr, k2 * pim) : v;
    out[2 * fsz + q] = make_double2(-ky * pim, ky * pr);
    out[3 * fsz + q] = make_double2(kx * pim, -(kx * pr));
  }
}

// Grid sums of u_x^2 + u_y^2 and of u_y^2 over the N^2 points after c2r and
// division by NxNy: (1/(NxNy)) * sum over the full spectrum of |U|^2, where on
// the kx = 0 and kx = Nx/2 columns the c2r keeps only the Hermitian part
// (U(ky) + conj U(-ky))/2 of each column.
__global__ void k_diag_usq(const double2* __restrict__ sp, Grid2D g, double* __restrict__ part) {
  const size_t total = (size_t)g.ny * g.nh, fsz = (size_t)g.ny * g.pitch;
  double sx = 0.0, sy = 0.0;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const int y = (int)(t / g.nh), x = (int)(t % g.nh);
    const size_t q = (size_t)y * g.pitch + x;
    const double2 a = sp[2 * fsz + q], b = sp[3 * fsz + q];
    if (x == 0 || 2 * x == g.nx) {
      const size_t qm = (size_t)((g.ny - y) % g.ny) * g.pitch + x;
      const double2 am = sp[2 * fsz + qm], bm = sp[3 * fsz + qm];
      const double hax = 0.5 * (a.x + am.x), hay = 0.5 * (a.y - am.y);
      const double hbx = 0.5 * (b.x + bm.x), hby = 0.5 * (b.y - bm.y);
      sx += hax * hax + hay * hay;
      sy += hbx * hbx + hby * hby;
    } else {
      sx += 2.0 * (a.x * a.x + a.y * a.y);
      sy += 2.0 * (b.x * b.x + b.y * b.y);
    }
  }
  __shared__ double s1[8], s2[8];
  for (int o = 16; o > 0; o >>= 1) {
    sx += __shfl_down_sync(0xffffffffu, sx, o);
    sy += __shfl_down_sync(0xffffffffu, sy, o);
  }
  if ((threadIdx.x & 31) == 0) {
    s1[threadIdx.x >> 5] = sx;
    s2[threadIdx.x >> 5] = sy;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) {
      a += s1[i];
      b += s2[i];
    }
    part[2 * blockIdx.x] = a;
    part[2 * blockIdx.x + 1] = b;
  }
}

// ---------------------------------------------------------------------------
// solver internals
// ---------------------------------------------------------------------------
template <typename T>
static int rhs_update_t(tara2d* h, const double2* win, int mode, cudaEvent_t* ev) {
  StepBufs sb;
  sb.win = win;
  sb.w0 = h->w0;
  sb.ws = h->ws;
  sb.acc = h->acc;
  sb.fold = h->fold;
  sb.fout = h->fout;
  sb.flag = h->flag;
  sb.force = h->force;
  int rc;
  const int nb = h->batch;
  if ((rc = Launch2D<T>::col_inverse(h->ny, h->nh, win, h->u, h->grid, h->rp, h->twy, h->stream, nb,
                                     h->var[0])))
    return rc;
  if (ev) TARA_CK(cudaEventRecord(ev[0], h->stream));
  if ((rc = Launch2D<T>::row_nl(h->nx, h->ny, h->u, h->nl, h->grid, h->twx, h->stream, nb,
                                h->var[1])))
    return rc;
  if (ev) TARA_CK(cudaEventRecord(ev[1], h->stream));
  if ((rc = Launch2D<T>::col_forward(h->ny, h->nh, h->nl, sb, h->grid, h->rp, mode, h->twy,
                                     h->stream, nb, h->var[2])))
    return rc;
  if (ev) TARA_CK(cudaEventRecord(ev[2], h->stream));
  return TARA_OK;
}

// One RHS evaluation of `win` followed by the update of `mode`; when ev is not
// null, ev[0..2] are recorded after the three launches.
int rhs_and_update(tara2d* h, const double2* win, int mode, cudaEvent_t* ev) {
  switch (h->cfg.precision) {
    case TARA_PREC_FP32: return rhs_update_t<float>(h, win, mode, ev);
    case TARA_PREC_DF64: return rhs_update_t<df64>(h, win, mode, ev);
    default: return rhs_update_t<double>(h, win, mode, ev);
  }
}

// Rows of nh complex values between a dense [ny][nh] and a padded [ny][pitch] layout.
__global__ void k_repitch(const double2* __restrict__ src, int spitch, double2* __restrict__ dst, int dpitch,
                          int nh, int ny) {
  const size_t total = (size_t)ny * nh;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const size_t y = t / nh, x = t % nh;
    dst[y * dpitch + x] = src[y * spitch + x];
  }
}

static bool is_pinned(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

// Page-locked host arrays of a megabyte or more move as one contiguous copy
// through a staging field of the handle and are re-pitched on the device (a
// pitched host<->device copy of 16 KB rows ran at about a third of the link's
// rate); other host memory takes the pitched copy.  The staging field is its
// own allocation, never the scratch that captured graphs may hold.
static int stage_buffer(tara2d* h, void** out) {
  if (!h->stage) TARA_CK(cudaMalloc(&h->stage, (size_t)h->nh * h->ny * sizeof(double2)));
  *out = h->stage;
  return TARA_OK;
}
int copy_in_dense(tara2d* h, double2* dst, const double* host) {
  const size_t bytes = (size_t)h->nh * h->ny * sizeof(double2);
  if (bytes >= (1u << 20) && is_pinned(host)) {
    void* stage = nullptr;
    int rc;
    if ((rc = stage_buffer(h, &stage))) return rc;
    TARA_CK(cudaMemcpyAsync(stage, host, bytes, cudaMemcpyHostToDevice, h->stream));
    k_repitch<<<152 * 8, 256, 0, h->stream>>>((const double2*)stage, h->nh, dst, h->pitch, h->nh, h->ny);
    TARA_CK(cudaGetLastError());
    return TARA_OK;
  }
  TARA_CK(cudaMemcpy2DAsync(dst, h->pitch * sizeof(double2), host, h->nh * sizeof(double2),
                            h->nh * sizeof(double2), h->ny, cudaMemcpyHostToDevice, h->stream));
  return TARA_OK;
}

int copy_out_dense(tara2d* h, double* host, const double2* src) {
  const size_t bytes = (size_t)h->nh * h->ny * sizeof(double2);
  if (bytes >= (1u << 20) && is_pinned(host)) {
    void* stage = nullptr;
    int rc;
    if ((rc = stage_buffer(h, &stage))) return rc;
    k_repitch<<<152 * 8, 256, 0, h->stream>>>(src, h->pitch, (double2*)stage, h->nh, h->nh, h->ny);
    TARA_CK(cudaGetLastError());
    TARA_CK(cudaMemcpyAsync(host, stage, bytes, cudaMemcpyDeviceToHost, h->stream));
    return TARA_OK;
  }
  TARA_CK(cudaMemcpy2DAsync(host, h->nh * sizeof(double2), src, h->pitch * sizeof(double2),
                            h->nh * sizeof(double2), h->ny, cudaMemcpyDeviceToHost, h->stream));
  return TARA_OK;
}

int refresh_tables(tara2d* h) {
  std::vector<double> kx(h->nh), ky(h->ny), inv((size_t)h->nh * h->ny);
  std::vector<int> i0(h->ny);
  make_wavenumbers(h->nx, h->ny, h->cfg.kpi, h->cfg.lx, h->cfg.ly, kx.data(), ky.data(), i0.data());
  make_inverse_table(h->nx, h->ny, kx.data(), ky.data(), h->cfg.rhs == TARA_RHS_SCREEN,
                     h->cfg.lambda, inv.data());
  int i0max = 0;
  for (int j = 0; j < h->ny; ++j) i0max = i0[j] > i0max ? i0[j] : i0max;
  h->grid.i0max = i0max;
  TARA_CK(cudaMemcpyAsync(h->inv, inv.data(), inv.size() * sizeof(double), cudaMemcpyHostToDevice,
                          h->stream));
  std::vector<float> tf(h->nh + h->ny + inv.size());
  for (int i = 0; i < h->nh; ++i) tf[i] = (float)kx[i];
  for (int j = 0; j < h->ny; ++j) tf[h->nh + j] = (float)ky[j];
  for (size_t q = 0; q < inv.size(); ++q) tf[h->nh + h->ny + q] = (float)inv[q];
  TARA_CK(cudaMemcpyAsync(h->tabf, tf.data(), tf.size() * sizeof(float), cudaMemcpyHostToDevice,
                          h->stream));
  std::vector<df64> td;
  if (h->tabd) {  // round-to-nearest splits hi = fl32(v), lo = fl32(v - hi)
    td.resize(tf.size());
    for (int i = 0; i < h->nh; ++i) td[i] = df64(kx[i]);
    for (int j = 0; j < h->ny; ++j) td[h->nh + j] = df64(ky[j]);
    for (size_t q = 0; q < inv.size(); ++q) td[h->nh + h->ny + q] = df64(inv[q]);
    TARA_CK(cudaMemcpyAsync(h->tabd, td.data(), td.size() * sizeof(df64), cudaMemcpyHostToDevice, h->stream));
  }
  TARA_CK(cudaMemcpyAsync(h->kx, kx.data(), h->nh * sizeof(double), cudaMemcpyHostToDevice,
                          h->stream));
  TARA_CK(cudaMemcpyAsync(h->ky, ky.data(), h->ny * sizeof(double), cudaMemcpyHostToDevice,
                          h->stream));
  TARA_CK(cudaMemcpyAsync(h->i0, i0.data(), h->ny * sizeof(int), cudaMemcpyHostToDevice, h->stream));
  TARA_CK(cudaStreamSynchronize(h->stream));  // host vectors go out of scope
  h->grid.kxf = h->tabf;
  h->grid.kyf = h->tabf + h->nh;
  h->grid.invf = h->tabf + h->nh + h->ny;
  h->grid.kxd = h->tabd;
  h->grid.kyd = h->tabd ? h->tabd + h->nh : nullptr;
  h->grid.invd = h->tabd ? h->tabd + h->nh + h->ny : nullptr;
  h->rp.rhs = h->cfg.rhs;
  h->rp.nu = h->cfg.nu;
  h->rp.alpha = h->cfg.alpha;
  h->rp.lambda = h->cfg.lambda;
  h->rp.dt = h->cfg.dt;
  const double nn = (double)h->nx * (double)h->ny;
  h->rp.nl_scale = 0.5 / (nn * nn);
  h->rp.nu_f = (float)h->rp.nu;
  h->rp.alpha_f = (float)h->rp.alpha;
  h->rp.nl_scale_f = (float)h->rp.nl_scale;
  h->rp.nu_d = df64(h->rp.nu);
  h->rp.alpha_d = df64(h->rp.alpha);
  h->rp.nl_scale_d = df64(h->rp.nl_scale);
  return TARA_OK;
}

int scratch(tara2d* h, size_t bytes, void** out) {
  if (h->scratch_bytes < bytes) {
    TARA_CK(cudaStreamSynchronize(h->stream));
    cudaFree(h->scratch);
    h->scratch = nullptr;
    h->scratch_bytes = 0;
    TARA_CK(cudaMalloc(&h->scratch, bytes));
    h->scratch_bytes = bytes;
  }
  *out = h->scratch;
  return TARA_OK;
}

int twiddles64(tara2d* h, const void** twx, const void** twy) {
  if (h->cfg.precision == TARA_PREC_FP64) {
    *twx = h->twx;
    *twy = h->twy;
    return TARA_OK;
  }
  int rc;
  if (!h->twx64 && (rc = make_twiddles(h->nx, false, &h->twx64))) return rc;
  if (!h->twy64 && (rc = make_twiddles(h->ny, false, &h->twy64))) return rc;
  *twx = h->twx64;
  *twy = h->twy64;
  return TARA_OK;
}

static int check_flag(tara2d* h) {
  unsigned int f = 0;
  TARA_CK(cudaMemcpyAsync(&f, h->flag, sizeof(f), cudaMemcpyDeviceToHost, h->stream));
  TARA_CK(cudaStreamSynchronize(h->stream));
  if (f & 4u) return set_error(TARA_ERR_TIMEOUT, "a tensor-memory wait of the closure network gave up");
  if (f) return set_error(TARA_ERR_NONFINITE, "non-finite value in the vorticity update");
  return TARA_OK;
}

}  // namespace tara

using namespace tara;

// ---------------------------------------------------------------------------
// public API
// ---------------------------------------------------------------------------
extern "C" {

int tara_last_error(void) { return g_err; }
const char* tara_last_error_message(void) { return g_msg.c_str(); }
void tara_clear_error(void) { set_ok(); }
const char* tara_version(void) { return "tara-gb300 0.1 (sm_103a)"; }

void tara2d_default_config(tara2d_config* c, int nx, int ny) {
  std::memset(c, 0, sizeof(*c));
  c->nx = nx;
  c->ny = ny;
  c->rhs = TARA_RHS_PLAIN;
  c->scheme = TARA_SCHEME_AB2;
  c->precision = TARA_PREC_FP64;
  c->nu = 0.01;
  c->dt = 1e-4;
  c->alpha = 1.0;
  c->lambda = 10.0;
  c->kpi = (double)3.1428f;
  c->lx = 2.0 * c->kpi;
  c->ly = 2.0 * c->kpi;
  c->batch = 1;
}

int tara2d_destroy(tara2d* h) {
  if (!h) return set_ok();
  cudaSetDevice(h->dev);
  if (h->stream) cudaStreamSynchronize(h->stream);
  void* ptrs[] = {h->w0, h->ws, h->acc, h->fold, h->fout, h->u, h->nl, h->kx, h->ky, h->i0, h->inv, h->tabf,
                  h->tabd, h->twx, h->twy, h->diag_part, h->diag_out, h->flag, h->scratch, h->stage, h->twx64,
                  h->twy64};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return set_ok();
}

// Is configuration index c (tile variant | 4 for the radix-8 path) available
// for step kernel k of handle h?
static bool candidate_ok(const tara2d* h, int k, int c) {
  if ((c & 3) >= kVariants[k] || ((c & 4) && h->cfg.precision == TARA_PREC_DF64)) return false;
  if (!is_pow2_in_range(h->nx) || !is_pow2_in_range(h->ny)) return c == 0;  // mixed-radix path: one form
  const int n = k == 1 ? h->nx : h->ny;  // the row pass transforms along x, the others along y
  switch (h->cfg.precision) {
    case TARA_PREC_FP32: return Launch2D<float>::tile_fits(k, n, c & 3);
    case TARA_PREC_DF64: return Launch2D<df64>::tile_fits(k, n, c & 3);
    default: return Launch2D<double>::tile_fits(k, n, c & 3);
  }
}

int tara2d_create(const tara2d_config* cfg, tara2d** out) {
  if (!cfg || !out) return set_error(TARA_ERR_ARGS, "null argument");
  *out = nullptr;
  if (!is_size_2d(cfg->nx) || !is_size_2d(cfg->ny))
    return set_error(TARA_ERR_ARGS,
                     "nx and ny must be powers of two in [16, 4096], or (FP64) even lengths 8 to 3600 "
                     "with factors 2, 3, 5, 7");
  if ((!is_pow2_in_range(cfg->nx) || !is_pow2_in_range(cfg->ny)) && cfg->precision != TARA_PREC_FP64)
    return set_error(TARA_ERR_ARGS, "grid sizes that are not powers of two take the FP64 precision only");
  if (cfg->rhs != TARA_RHS_PLAIN && cfg->rhs != TARA_RHS_SCREEN)
    return set_error(TARA_ERR_ARGS, "unknown rhs kind");
  if (cfg->scheme != TARA_SCHEME_AB2 && cfg->scheme != TARA_SCHEME_RK4)
    return set_error(TARA_ERR_ARGS, "unknown scheme");
  if (cfg->precision != TARA_PREC_FP64 && cfg->precision != TARA_PREC_FP32 &&
      cfg->precision != TARA_PREC_DF64)
    return set_error(TARA_ERR_ARGS, "unknown precision");
  if (!(cfg->lx > 0.0) || !(cfg->ly > 0.0) || !(cfg->kpi > 0.0))
    return set_error(TARA_ERR_ARGS, "box lengths and kpi must be positive");
  if (cfg->batch < 1 || cfg->batch > 65535) return set_error(TARA_ERR_ARGS, "batch must be in [1, 65535]");
  tara2d* h = new tara2d();
  h->cfg = *cfg;
  h->batch = cfg->batch;
  h->nx = cfg->nx;
  h->ny = cfg->ny;
  h->nh = cfg->nx / 2 + 1;
  h->pitch = round_up(h->nh, 8);
  // default tiles: variant 0, or the first that fits a CTA (at 4096 points the
  // FP64 row pass has only the three-slot tile)
  for (int k = 0; k < 3; ++k)
    for (int v = 0; v < kVariants[k]; ++v)
      if (candidate_ok(h, k, v)) {
        h->var[k] = v;
        break;
      }
  int rc = TARA_OK;
  auto fail = [&](int code) {  // free the half-built handle, keep the error
    const ErrorState saved = save_error();
    tara2d_destroy(h);
    restore_error(saved);
    return code;
  };
#define CKC(call)                                              \
  do {                                                         \
    cudaError_t e_ = (call);                                   \
    if (e_ != cudaSuccess) return fail(cuda_fail(e_, #call)); \
  } while (0)
  CKC(cudaGetDevice(&h->dev));
  CKC(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
  const size_t fbytes = (size_t)h->batch * h->ny * h->pitch * sizeof(double2);
  const size_t csize = cfg->precision == TARA_PREC_FP32 ? sizeof(float2)
                       : cfg->precision == TARA_PREC_DF64 ? sizeof(df64c)
                                                          : sizeof(double2);
  const size_t wbytes = (size_t)h->batch * h->ny * h->pitch * csize;
  CKC(cudaMalloc(&h->w0, fbytes));
  CKC(cudaMalloc(&h->fold, fbytes));
  CKC(cudaMalloc(&h->fout, fbytes));
  if (cfg->scheme == TARA_SCHEME_RK4) {
    CKC(cudaMalloc(&h->ws, fbytes));
    CKC(cudaMalloc(&h->acc, fbytes));
  }
  CKC(cudaMalloc(&h->u, 4 * wbytes));
  CKC(cudaMalloc(&h->nl, wbytes));
  CKC(cudaMalloc(&h->kx, h->nh * sizeof(double)));
  CKC(cudaMalloc(&h->ky, h->ny * sizeof(double)));
  CKC(cudaMalloc(&h->i0, h->ny * sizeof(int)));
  CKC(cudaMalloc(&h->inv, (size_t)h->ny * h->nh * sizeof(double)));
  CKC(cudaMalloc(&h->tabf, ((size_t)h->ny * h->nh + h->nh + h->ny) * sizeof(float)));
  if (cfg->precision == TARA_PREC_DF64)
    CKC(cudaMalloc(&h->tabd, ((size_t)h->ny * h->nh + h->nh + h->ny) * sizeof(df64)));
  CKC(cudaMalloc(&h->diag_part, 2 * kDiagBlocks * sizeof(double)));
  CKC(cudaMalloc(&h->diag_out, 4 * sizeof(double)));
  CKC(cudaMalloc(&h->flag, sizeof(unsigned int)));
  CKC(cudaMemsetAsync(h->w0, 0, fbytes, h->stream));
  CKC(cudaMemsetAsync(h->fold, 0, fbytes, h->stream));
  CKC(cudaMemsetAsync(h->fout, 0, fbytes, h->stream));
  if (h->ws) CKC(cudaMemsetAsync(h->ws, 0, fbytes, h->stream));
  if (h->acc) CKC(cudaMemsetAsync(h->acc, 0, fbytes, h->stream));
  CKC(cudaMemsetAsync(h->u, 0, 4 * wbytes, h->stream));
  CKC(cudaMemsetAsync(h->nl, 0, wbytes, h->stream));
  CKC(cudaMemsetAsync(h->flag, 0, sizeof(unsigned int), h->stream));
#undef CKC
  if (cfg->precision == TARA_PREC_DF64) {
    if ((rc = make_twiddles_df64(h->nx, &h->twx))) return fail(rc);
    if ((rc = make_twiddles_df64(h->ny, &h->twy))) return fail(rc);
  } else {
    const bool f32 = cfg->precision == TARA_PREC_FP32;
    if ((rc = make_twiddles(h->nx, f32, &h->twx))) return fail(rc);
    if ((rc = make_twiddles(h->ny, f32, &h->twy))) return fail(rc);
  }
  h->grid.nx = h->nx;
  h->grid.ny = h->ny;
  h->grid.nh = h->nh;
  h->grid.pitch = h->pitch;
  h->grid.kx = h->kx;
  h->grid.ky = h->ky;
  h->grid.i0 = h->i0;
  h->grid.inv = h->inv;
  if ((rc = refresh_tables(h))) return fail(rc);
  *out = h;
  return set_ok();
}

int tara2d_set_state_run(tara2d* h, int run, const double* omegak, const double* dt_old) {
  if (!h || !omegak || run < 0 || run >= h->batch) return set_error(TARA_ERR_ARGS, "bad argument");
  TARA_CK(cudaSetDevice(h->dev));
  const size_t off = (size_t)run * h->ny * h->pitch;
  int rc;
  if ((rc = copy_in_dense(h, h->w0 + off, omegak))) return rc;
  if (dt_old) {
    if ((rc = copy_in_dense(h, h->fold + off, dt_old))) return rc;
  } else {
    TARA_CK(cudaMemsetAsync(h->fold + off, 0, (size_t)h->ny * h->pitch * sizeof(double2), h->stream));
  }
  TARA_CK(cudaStreamSynchronize(h->stream));
  return set_ok();
}

int tara2d_get_state_run(tara2d* h, int run, double* omegak, double* dt_old) {
  if (!h || !omegak || run < 0 || run >= h->batch) return set_error(TARA_ERR_ARGS, "bad argument");
  TARA_CK(cudaSetDevice(h->dev));
  const size_t off = (size_t)run * h->ny * h->pitch;
  int rc;
  if ((rc = copy_out_dense(h, omegak, h->w0 + off))) return rc;
  if (dt_old && (rc = copy_out_dense(h, dt_old, h->fold + off))) return rc;
  TARA_CK(cudaStreamSynchronize(h->stream));
  return set_ok();
}

int tara2d_set_state(tara2d* h, const double* omegak, const double* dt_old) {
  return tara2d_set_state_run(h, 0, omegak, dt_old);
}

int tara2d_get_state(tara2d* h, double* omegak, double* dt_old) {
  return tara2d_get_state_run(h, 0, omegak, dt_old);
}

int tara2d_set_state_device(tara2d* h, const void* omegak, const void* dt_old) {
  if (!h || !omegak) return set_error(TARA_ERR_ARGS, "null argument");
  TARA_CK(cudaSetDevice(h->dev));
  const size_t row = h->nh * sizeof(double2), dp = h->pitch * sizeof(double2);
  TARA_CK(cudaMemcpy2DAsync(h->w0, dp, omegak, row, row, h->ny, cudaMemcpyDeviceToDevice, h->stream));
  if (dt_old)
    TARA_CK(cudaMemcpy2DAsync(h->fold, dp, dt_old, row, row, h->ny, cudaMemcpyDeviceToDevice,
                              h->stream));
  else
    TARA_CK(cudaMemsetAsync(h->fold, 0, (size_t)h->ny * dp, h->stream));
  return set_ok();
}

int tara2d_get_state_device(tara2d* h, void* omegak) {
  if (!h || !omegak) return set_error(TARA_ERR_ARGS, "null argument");
  TARA_CK(cudaSetDevice(h->dev));
  const size_t row = h->nh * sizeof(double2), dp = h->pitch * sizeof(double2);
  TARA_CK(cudaMemcpy2DAsync(omegak, row, h->w0, dp, row, h->ny, cudaMemcpyDeviceToDevice, h->stream));
  return set_ok();
}

int tara2d_launches_per_step(const tara2d* h) {
  if (!h) return 0;
  return h->cfg.scheme == TARA_SCHEME_RK4 ? 12 : 3;
}

static int step_impl(tara2d* h, int nsteps, cudaEvent_t* ev) {
  int rc;
  const int per = h->cfg.scheme == TARA_SCHEME_RK4 ? 12 : 3;
  for (int s = 0; s < nsteps; ++s) {
    cudaEvent_t* e = ev ? ev + (size_t)s * per : nullptr;
    if (h->cfg.scheme == TARA_SCHEME_AB2) {
      if ((rc = rhs_and_update(h, h->w0, MODE_AB2, e))) return rc;
    } else {
      if ((rc = rhs_and_update(h, h->w0, MODE_RK1, e))) return rc;
      if ((rc = rhs_and_update(h, h->ws, MODE_RK2, e ? e + 3 : nullptr))) return rc;
      if ((rc = rhs_and_update(h, h->ws, MODE_RK3, e ? e + 6 : nullptr))) return rc;
      if ((rc = rhs_and_update(h, h->ws, MODE_RK4, e ? e + 9 : nullptr))) return rc;
    }
  }
  return TARA_OK;
}

int tara2d_step(tara2d* h, int nsteps) {
  if (!h || nsteps < 0) return set_error(TARA_ERR_ARGS, "bad handle or step count");
  TARA_CK(cudaSetDevice(h->dev));
  int rc;
  if ((rc = step_impl(h, nsteps, nullptr))) return rc;
  return set_ok();
}

int tara2d_step_timed(tara2d* h, int nsteps, double* kernel_ms, int* kernel_launches,
                      double* total_ms) {
  if (!h || nsteps <= 0 || !kernel_ms || !kernel_launches)
    return set_error(TARA_ERR_ARGS, "bad arguments");
  TARA_CK(cudaSetDevice(h->dev));
  const int per = h->cfg.scheme == TARA_SCHEME_RK4 ? 12 : 3;
  const size_t nev = (size_t)nsteps * per + 1;
  std::vector<cudaEvent_t> ev(nev, nullptr);
  int rc = TARA_OK;
  for (size_t i = 0; i < nev && !rc; ++i)
    if (cudaEventCreate(&ev[i]) != cudaSuccess) rc = set_error(TARA_ERR_CUDA, "cudaEventCreate");
  if (!rc && cudaEventRecord(ev[0], h->stream) != cudaSuccess)
    rc = set_error(TARA_ERR_CUDA, "cudaEventRecord");
  if (!rc) rc = step_impl(h, nsteps, ev.data() + 1);
  if (!rc && cudaEventSynchronize(ev[nev - 1]) != cudaSuccess)
    rc = set_error(TARA_ERR_CUDA, "cudaEventSynchronize");
  if (!rc) {
    for (int k = 0; k < 3; ++k) {
      kernel_ms[k] = 0.0;
      kernel_launches[k] = 0;
    }
    for (size_t i = 1; i < nev; ++i) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, ev[i - 1], ev[i]);
      const int kind = (int)((i - 1) % 3);  // col_inverse, row_nl, col_forward
      kernel_ms[kind] += ms;
      kernel_launches[kind] += 1;
    }
    if (total_ms) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, ev[0], ev[nev - 1]);
      *total_ms = ms;
    }
  }
  for (cudaEvent_t e : ev)
    if (e) cudaEventDestroy(e);
  return rc ? rc : set_ok();
}

int tara2d_autotune(tara2d* h, int trial_steps, int* variants3, double* ms24) {
  if (!h || trial_steps <= 0) return set_error(TARA_ERR_ARGS, "bad arguments");
  TARA_CK(cudaSetDevice(h->dev));
  const size_t bytes = (size_t)h->batch * h->ny * h->pitch * sizeof(double2);
  double2 *save_w0 = nullptr, *save_fold = nullptr;
  int rc = TARA_OK;
  if (cudaMalloc(&save_w0, bytes) != cudaSuccess || cudaMalloc(&save_fold, bytes) != cudaSuccess)
    rc = set_error(TARA_ERR_NOMEM, "cudaMalloc in tara2d_autotune");
  if (!rc && (cudaMemcpyAsync(save_w0, h->w0, bytes, cudaMemcpyDeviceToDevice, h->stream) != cudaSuccess ||
              cudaMemcpyAsync(save_fold, h->fold, bytes, cudaMemcpyDeviceToDevice, h->stream) != cudaSuccess))
    rc = set_error(TARA_ERR_CUDA, "state save");
  // Candidates: every tile variant on both radix paths (radix 4 only for the
  // double-float form).
  // Pass 1: every kernel in candidate c (a kernel without it keeps its default),
  // one settling step (which also sets the shared-memory attributes on first
  // use), then trial_steps timed.
  // Pass 2: each kernel's candidates with the other two at their pass-1 choice,
  // again one settling step and trial_steps timed -- a kernel's time depends
  // on its neighbours' tiles (cache contents, CTA phases), and a variant timed
  // right after a switch, without the settling step, read up to 15 % slow.
  // Pass 3 (below) settles between each kernel's two best by whole steps.
  double ms[kCandidates][3];
  for (int c = 0; c < kCandidates; ++c)
    for (int k = 0; k < 3; ++k) ms[c][k] = 0.0;
  int dflt[3] = {0, 0, 0};  // the first candidate each kernel has (variant 0 may not fit a CTA)
  for (int k = 0; k < 3; ++k)
    for (int c = kCandidates - 1; c >= 0; --c)
      if (candidate_ok(h, k, c)) dflt[k] = c;
  int best1[3] = {dflt[0], dflt[1], dflt[2]};
  // Warm-up: about 50 ms of steps before anything is timed.  Timed from an idle
  // GPU, the first candidates ran at lower clocks than the later ones, and at
  // small grids that reordered the ranking.
  if (!rc) {
    for (int k = 0; k < 3; ++k) h->var[k] = dflt[k];
    double kms[3] = {0.0, 0.0, 0.0}, tot = 0.0;
    int cnt[3];
    rc = tara2d_step_timed(h, 1, kms, cnt, &tot);
    if (!rc) {
      const int warm = (int)std::min(500.0, std::ceil(50.0 / std::max(tot, 1e-3)));
      rc = tara2d_step(h, warm);
    }
  }
  auto timed = [&](double* t) {
    int r = tara2d_step(h, 1);
    int cnt[3];
    if (!r) r = tara2d_step_timed(h, trial_steps, t, cnt, nullptr);
    if (!r)
      for (int k = 0; k < 3; ++k) t[k] /= (cnt[k] > 0 ? cnt[k] : 1);
    return r;
  };
  for (int c = 0; c < kCandidates && !rc; ++c) {
    bool any = false;
    for (int k = 0; k < 3; ++k) {
      const bool ok = candidate_ok(h, k, c);
      h->var[k] = ok ? c : dflt[k];
      any |= ok;
    }
    if (!any) continue;
    double t[3];
    rc = timed(t);
    if (!rc)
      for (int k = 0; k < 3; ++k)
        if (candidate_ok(h, k, c)) ms[c][k] = t[k];
  }
  if (!rc)
    for (int k = 0; k < 3; ++k)
      for (int c = 0; c < kCandidates; ++c)
        if (candidate_ok(h, k, c) && ms[c][k] < ms[best1[k]][k]) best1[k] = c;
  double ctx[3][kCandidates];
  for (int k = 0; k < 3 && !rc; ++k)
    for (int c = 0; c < kCandidates && !rc; ++c) {
      if (!candidate_ok(h, k, c)) continue;
      for (int q = 0; q < 3; ++q) h->var[q] = best1[q];
      h->var[k] = c;
      double t[3];
      rc = timed(t);
      if (!rc) ctx[k][c] = t[k];
    }
  // Pass 3: whole steps (no events between the launches) over the products of
  // each kernel's two best in-context candidates.  Events between launches
  // add about a microsecond to each timed kernel, which at small grids (a few
  // microseconds per launch) is the size of the differences being ranked.
  int top[3][2];
  if (!rc)
    for (int k = 0; k < 3; ++k) {
      top[k][0] = top[k][1] = -1;
      for (int c = 0; c < kCandidates; ++c) {
        if (!candidate_ok(h, k, c)) continue;
        if (top[k][0] < 0 || ctx[k][c] < ctx[k][top[k][0]]) {
          top[k][1] = top[k][0];
          top[k][0] = c;
        } else if (top[k][1] < 0 || ctx[k][c] < ctx[k][top[k][1]]) {
          top[k][1] = c;
        }
      }
      if (top[k][1] < 0) top[k][1] = top[k][0];
      for (int c = 0; c < kCandidates; ++c)
        ms[c][k] = candidate_ok(h, k, c) ? ctx[k][c] : 0.0;  // reported: the in-context times
    }
  if (!rc) {
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
      rc = set_error(TARA_ERR_CUDA, "cudaEventCreate");
    // repetitions: whole steps worth about 2 ms per combination, from the
    // in-context estimate of one step
    double est = 0.0;
    for (int k = 0; k < 3; ++k) est += ctx[k][top[k][0]] * (h->cfg.scheme == TARA_SCHEME_RK4 ? 4 : 1);
    const int reps = std::max(trial_steps, std::min(200, (int)(2.0 / std::max(est, 1e-3)) + 1));
    float best_ms = 0.f;
    bool have = false;
    int pick[3] = {top[0][0], top[1][0], top[2][0]};
    // every combination twice, the second sweep in reverse order
    for (int it = 0; it < 16 && !rc; ++it) {
      const int m = it < 8 ? it : 15 - it;
      const int v[3] = {top[0][m & 1], top[1][(m >> 1) & 1], top[2][(m >> 2) & 1]};
      bool dup = false;  // a kernel with one candidate repeats a combination
      for (int q = 0; q < 3; ++q) dup |= ((m >> q) & 1) && top[q][1] == top[q][0];
      if (dup) continue;
      for (int q = 0; q < 3; ++q) h->var[q] = v[q];
      float t = 0.f;
      rc = tara2d_step(h, 1);
      if (!rc && (cudaEventRecord(e0, h->stream) != cudaSuccess)) rc = set_error(TARA_ERR_CUDA, "event");
      if (!rc) rc = tara2d_step(h, reps);
      if (!rc && (cudaEventRecord(e1, h->stream) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
                  cudaEventElapsedTime(&t, e0, e1) != cudaSuccess))
        rc = set_error(TARA_ERR_CUDA, "event timing");
      if (!rc && (!have || t < best_ms)) {
        have = true;
        best_ms = t;
        for (int q = 0; q < 3; ++q) pick[q] = v[q];
      }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    for (int k = 0; k < 3; ++k) {
      h->var[k] = pick[k];
      if (variants3) variants3[k] = pick[k];
    }
  }
  if (!rc && ms24)
    for (int c = 0; c < kCandidates; ++c)
      for (int k = 0; k < 3; ++k) ms24[3 * c + k] = ms[c][k];
  if (!rc && (cudaMemcpyAsync(h->w0, save_w0, bytes, cudaMemcpyDeviceToDevice, h->stream) != cudaSuccess ||
              cudaMemcpyAsync(h->fold, save_fold, bytes, cudaMemcpyDeviceToDevice, h->stream) != cudaSuccess ||
              cudaStreamSynchronize(h->stream) != cudaSuccess))
    rc = set_error(TARA_ERR_CUDA, "state restore");
  cudaFree(save_w0);
  cudaFree(save_fold);
  return rc ? rc : set_ok();
}

int tara2d_set_variants(tara2d* h, const int* variants3) {
  if (!h || !variants3) return set_error(TARA_ERR_ARGS, "null argument");
  for (int k = 0; k < 3; ++k)
    if (variants3[k] < 0 || variants3[k] >= kCandidates || !candidate_ok(h, k, variants3[k]))
      return set_error(TARA_ERR_ARGS,
                       "variants: tile 0-2 (row pass 0-3), plus 4 for the radix-8 path (not in the "
                       "double-float form)");
  for (int k = 0; k < 3; ++k) h->var[k] = variants3[k];
  return set_ok();
}

int tara2d_rhs(tara2d* h, double* dt_omegak) {
  if (!h || !dt_omegak) return set_error(TARA_ERR_ARGS, "null argument");
  TARA_CK(cudaSetDevice(h->dev));
  int rc;
  if ((rc = rhs_and_update(h, h->w0, MODE_DERIVE, nullptr))) return rc;
  if ((rc = copy_out_dense(h, dt_omegak, h->fout))) return rc;
  TARA_CK(cudaStreamSynchronize(h->stream));
  return set_ok();
}

int tara2d_diag_run(tara2d* h, int run, double* energy, double* enstrophy) {
  if (!h || run < 0 || run >= h->batch) return set_error(TARA_ERR_ARGS, "bad argument");
  TARA_CK(cudaSetDevice(h->dev));
  k_diag_partial<<<kDiagBlocks, kDiagThreads, 0, h->stream>>>(
      h->w0 + (size_t)run * h->ny * h->pitch, h->grid, h->diag_part);
  TARA_CK(cudaGetLastError());
  const double nn = (double)h->nx * (double)h->ny;
  k_diag_final<<<1, 32, 0, h->stream>>>(h->diag_part, kDiagBlocks, 0.5 / (nn * nn), h->diag_out,
                                        h->flag);
  TARA_CK(cudaGetLastError());
  double out[2];
  TARA_CK(cudaMemcpyAsync(out, h->diag_out, sizeof(out), cudaMemcpyDeviceToHost, h->stream));
  TARA_CK(cudaStreamSynchronize(h->stream));
  if (energy) *energy = out[0];
  if (enstrophy) *enstrophy = out[1];
  int rc;
  if ((rc = check_flag(h))) return rc;
  return set_ok();
}

int tara2d_diag(tara2d* h, double* energy, double* enstrophy) {
  return tara2d_diag_run(h, 0, energy, enstrophy);
}

int tara2d_synchronize(tara2d* h) {
  if (!h) return set_error(TARA_ERR_ARGS, "null handle");
  TARA_CK(cudaSetDevice(h->dev));
  TARA_CK(cudaStreamSynchronize(h->stream));
  return check_flag(h) ? g_err : set_ok();
}

void* tara2d_stream(tara2d* h) { return h ? (void*)h->stream : nullptr; }

// Diagnostic spectra with the driver's wavenumbers (true pi, ini box), into
// four consecutive pitched fields at `sp`.
static int diag_spectra(tara2d* h, const tara2d_diag_params* dp, double2* sp, Grid2D* gout,
                        double** kbuf) {
  std::vector<double> kx(h->nh), ky(h->ny);
  std::vector<int> i0(h->ny);
  make_wavenumbers(h->nx, h->ny, dp->kpi, dp->lx, dp->ly, kx.data(), ky.data(), i0.data());
  double* dk = nullptr;
  TARA_CK(cudaMalloc(&dk, (h->nh + h->ny) * sizeof(double)));
  *kbuf = dk;
  TARA_CK(cudaMemcpyAsync(dk, kx.data(), h->nh * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  TARA_CK(cudaMemcpyAsync(dk + h->nh, ky.data(), h->ny * sizeof(double), cudaMemcpyHostToDevice,
                          h->stream));
  Grid2D g = h->grid;
  g.kx = dk;
  g.ky = dk + h->nh;
  *gout = g;
  k_diag_spectra<<<304, 256, 0, h->stream>>>(h->w0, g, dp->lambda, dp->screened, sp);
  TARA_CK(cudaGetLastError());
  TARA_CK(cudaStreamSynchronize(h->stream));  // host tables go out of scope
  return TARA_OK;
}

int tara2d_diag_reference(tara2d* h, const tara2d_diag_params* dp, double* usq, double* uysq) {
  if (!h || !dp) return set_error(TARA_ERR_ARGS, "null argument");
  TARA_CK(cudaSetDevice(h->dev));
  double2* sp = nullptr;
  double* part = nullptr;
  double* kbuf = nullptr;
  const size_t fsz = (size_t)h->ny * h->pitch;
  int rc = TARA_OK;
  if (cudaMalloc(&sp, 4 * fsz * sizeof(double2)) != cudaSuccess ||
      cudaMalloc(&part, 2 * kDiagBlocks * sizeof(double)) != cudaSuccess)
    rc = set_error(TARA_ERR_NOMEM, "cudaMalloc");
  Grid2D g;
  if (!rc) rc = diag_spectra(h, dp, sp, &g, &kbuf);
  std::vector<double> hp(2 * kDiagBlocks);
  if (!rc) {
    k_diag_usq<<<kDiagBlocks, kDiagThreads, 0, h->stream>>>(sp, g, part);
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpyAsync(hp.data(), part, hp.size() * sizeof(double), cudaMemcpyDeviceToHost,
                        h->stream) != cudaSuccess ||
        cudaStreamSynchronize(h->stream) != cudaSuccess)
      rc = set_error(TARA_ERR_CUDA, "diag reduction");
  }
  if (!rc) {
    double a = 0.0, b = 0.0;
    for (int i = 0; i < kDiagBlocks; ++i) {
      a += hp[2 * i];
      b += hp[2 * i + 1];
    }
    const double nn = (double)h->nx * (double)h->ny;
    if (usq) *usq = (a + b) / nn;
    if (uysq) *uysq = b / nn;
    if (!(std::isfinite(a) && std::isfinite(b)))
      rc = set_error(TARA_ERR_NONFINITE, "non-finite energy");
  }
  cudaFree(sp);
  cudaFree(part);
  cudaFree(kbuf);
  return rc ? rc : set_ok();
}

int tara2d_real_fields(tara2d* h, const tara2d_diag_params* dp, double* psi, double* omega,
                       double* ux, double* uy) {
  if (!h || !dp) return set_error(TARA_ERR_ARGS, "null argument");
  TARA_CK(cudaSetDevice(h->dev));
  const size_t fsz = (size_t)h->ny * h->pitch;
  const int rpitch = round_up(h->nx, 8);
  double2* sp = nullptr;
  double* real = nullptr;
  double* kbuf = nullptr;
  void *tx = nullptr, *ty = nullptr;
  int rc = TARA_OK;
  if (cudaMalloc(&sp, 4 * fsz * sizeof(double2)) != cudaSuccess ||
      cudaMalloc(&real, (size_t)h->ny * rpitch * sizeof(double)) != cudaSuccess)
    rc = set_error(TARA_ERR_NOMEM, "cudaMalloc");
  Grid2D g;
  if (!rc) rc = diag_spectra(h, dp, sp, &g, &kbuf);
  // the diagnostic transforms run in FP64 whatever the solver's precision
  if (!rc) rc = make_twiddles(h->nx, false, &tx);
  if (!rc) rc = make_twiddles(h->ny, false, &ty);
  double* outs[4] = {psi, omega, ux, uy};
  std::vector<double> host((size_t)h->ny * rpitch);
  const double nn = (double)h->nx * (double)h->ny;
  for (int f = 0; f < 4 && !rc; ++f) {
    if (!outs[f]) continue;
    double2* in = sp + f * fsz;
    rc = Launch2D<double>::col_fft(h->ny, h->nh, h->pitch, in, in, true, ty, h->stream);
    if (!rc) rc = Launch2D<double>::row_c2r(h->nx, h->ny, h->pitch, rpitch, in, real, tx, h->stream);
    if (!rc && (cudaMemcpyAsync(host.data(), real, host.size() * sizeof(double),
                                cudaMemcpyDeviceToHost, h->stream) != cudaSuccess ||
                cudaStreamSynchronize(h->stream) != cudaSuccess))
      rc = set_error(TARA_ERR_CUDA, "real field copy");
    if (!rc)
      for (int j = 0; j < h->ny; ++j)
        for (int i = 0; i < h->nx; ++i)
          outs[f][(size_t)j * h->nx + i] = host[(size_t)j * rpitch + i] / nn;
  }
  cudaFree(sp);
  cudaFree(real);
  cudaFree(kbuf);
  cudaFree(tx);
  cudaFree(ty);
  return rc ? rc : set_ok();
}

int tara2d_init_random(tara2d* h, double k0, double energy, uint64_t seed) {
  return tara2d_init_random_run(h, 0, k0, energy, seed);
}

int tara2d_init_random_run(tara2d* h, int run, double k0, double energy, uint64_t seed) {
  if (!h || !(k0 > 0.0) || !(energy > 0.0) || run < 0 || run >= h->batch)
    return set_error(TARA_ERR_ARGS, "bad arguments");
  TARA_CK(cudaSetDevice(h->dev));
  const int nx = h->nx, ny = h->ny, nh = h->nh;
  const double pi = 3.14159265358979323846;
  std::vector<double2> spec((size_t)nh * ny);
  const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  for (int j = 0; j < ny; ++j) {
    const double ky = (j < ny / 2) ? (double)j : (double)(j - ny);
    for (int i = 0; i < nh; ++i) {
      const double kx = (double)i;
      double2 v = make_double2(0.0, 0.0);
      if (i || j) {
        const uint32_t ctr[4] = {(uint32_t)i, (uint32_t)j, 0u, 0u};
        uint32_t r[4];
        philox4x32_10(ctr, key, r);
        const double theta = 2.0 * pi * ((double)r[0] * (1.0 / 4294967296.0));
        const double k = std::sqrt(kx * kx + ky * ky);
        const double ek = k * k * k * k * std::exp(-(k / k0) * (k / k0));
        const double amp = std::sqrt(k * ek / pi);
        v = make_double2(amp * std::cos(theta), amp * std::sin(theta));
      }
      spec[(size_t)j * nh + i] = v;
    }
  }
  int rc;
  const size_t off = (size_t)run * ny * h->pitch;
  double2* w0 = h->w0 + off;
  double2* tmp = h->fout + off;
  if ((rc = copy_in_dense(h, w0, (const double*)spec.data()))) return rc;
  // Hermitian projection: c2r then r2c (FP64 transforms), scaled by 1/(Nx Ny)
  const int rpitch = round_up(nx, 8);
  double* real = nullptr;
  void *tx = nullptr, *ty = nullptr;
  if ((rc = make_twiddles(nx, false, &tx)) || (rc = make_twiddles(ny, false, &ty))) {
    cudaFree(tx);
    cudaFree(ty);
    return rc;
  }
  TARA_CK(cudaMalloc(&real, (size_t)ny * rpitch * sizeof(double)));
  TARA_CK(cudaMemcpyAsync(tmp, w0, (size_t)ny * h->pitch * sizeof(double2),
                          cudaMemcpyDeviceToDevice, h->stream));
  rc = Launch2D<double>::col_fft(ny, nh, h->pitch, tmp, tmp, true, ty, h->stream);
  if (!rc) rc = Launch2D<double>::row_c2r(nx, ny, h->pitch, rpitch, tmp, real, tx, h->stream);
  if (!rc) rc = Launch2D<double>::row_r2c(nx, ny, rpitch, h->pitch, real, w0, tx, h->stream);
  if (!rc) rc = Launch2D<double>::col_fft(ny, nh, h->pitch, w0, w0, false, ty, h->stream);
  if (!rc) {
    const double nn = (double)nx * (double)ny;
    TARA_CK(cudaMemsetAsync(w0, 0, sizeof(double2), h->stream));  // zero mean vorticity
    k_mul<<<304, 256, 0, h->stream>>>(w0, (size_t)ny * h->pitch, 1.0 / nn);
    TARA_CK(cudaGetLastError());
    double e0 = 0.0;
    rc = tara2d_diag_run(h, run, &e0, nullptr);
    if (!rc) {
      k_mul<<<304, 256, 0, h->stream>>>(w0, (size_t)ny * h->pitch,
                                        e0 > 0.0 ? std::sqrt(energy / e0) : 1.0);
      TARA_CK(cudaGetLastError());
      TARA_CK(cudaMemsetAsync(h->fold + off, 0, (size_t)ny * h->pitch * sizeof(double2), h->stream));
    }
  }
  TARA_CK(cudaStreamSynchronize(h->stream));
  cudaFree(real);
  cudaFree(tx);
  cudaFree(ty);
  return rc ? rc : set_ok();
}

}  // extern "C"
