// Fused inference forward of the Fourier neural operator for small batches (the
// closure's one-sample call): the 27 launches of the layer-by-layer forward
// become 2 per Fourier layer plus one, each spread over a CTA per grid row or
// per (kx, mode group) column so that a single 128^2 sample still fills the SMs.
//
//   k_fused_lift     per row (b, y): v_0 = x P + p, and the row's truncated
//                    DFT along x (A[b, y, kx, re/im, c]) for layer 1.
//   k_fused_col      per (b, kx, group of kModeGroup ky modes): the truncated
//                    DFT along y of A's column kx for the group's modes, then
//                    the per-mode complex mixing Y[b, j, kx, :] = X Rb[j, kx]
//                    (BF16-rounded operands, FP32 sums, as the per-mode GEMV of
//                    the layer-by-layer path).
//   k_fused_row<P>   per row (b, y): the inverse DFT along y of Y for this row,
//                    the inverse DFT along x, plus the pointwise channel mixing
//                    v W on tcgen05 (A = the row's 128 x 32 activations, B = W,
//                    both BF16 in shared memory, the FP32 accumulator in tensor
//                    memory) and the bias; then GELU.  P = 0: the row's DFT
//                    along x for the next layer.  P > 0 (last layer): the
//                    projection h = GELU(v Q1 + q1) on tcgen05 (N = P) and
//                    y = h Q2 + q2 on CUDA cores.
//
// Same arithmetic as the layer-by-layer forward (fno.cu) up to the order of FP32
// sums; no activations are kept for a backward pass.  Every wait on the tensor
// cores is bounded: one that gives up sets bit 2 (value 4) of *err, the CTA
// skips what depends on it, waits once more for its MMAs and frees its tensor
// memory.
#include <cstdint>

#include <cuda_bf16.h>

#include "fno_fused.h"
#include "internal.h"
#include "umma.cuh"

namespace tara {

namespace {

constexpr int kW = kFusedW, kC = kFusedC, kThreads = 256, kModeGroup = 4;
// Row kernels: 512 threads, four warps per TMEM lane group (32 rows) -- each
// thread owns one grid point x and kCpt channels, and each 128-thread quarter
// one quarter of the x range in the row DFT.
constexpr int kRT = 512, kQ = kRT / 128, kCpt = kC / kQ;
constexpr int kK2 = 2 * kFusedMaxMX;  // the inverse x-DFT's K: (kx, re/im), padded with zeros past 2 MX

__device__ __forceinline__ void split_store(unsigned char* hi, unsigned char* lo, uint32_t off, float v) {
  const __nv_bfloat16 h = __float2bfloat16_rn(v);
  *reinterpret_cast<__nv_bfloat16*>(hi + off) = h;
  *reinterpret_cast<__nv_bfloat16*>(lo + off) = __float2bfloat16_rn(v - __bfloat162float(h));
}
constexpr uint32_t kFwWait = 1u << 20;  // polls of an mbarrier before a wait gives up
constexpr uint32_t kBulkChunk = 16384;   // bytes per bulk copy instruction

__device__ __forceinline__ float gelu_f(float x) { return 0.5f * x * (1.f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float bf16r(float v) { return __bfloat162float(__float2bfloat16_rn(v)); }

// Programmatic dependent launch: the kernels of the chain are launched with
// programmatic stream serialisation, so each may start while its predecessor
// runs.  A kernel first lets its own successor launch, prepares what does not
// depend on the predecessor (parameters, tables, barriers, tensor memory),
// then waits for the predecessor grid to complete before it touches its
// outputs.  Parameters are only written before the chain starts (a chain
// kernel starts after its predecessor has started, so after every kernel
// before the chain has completed).
__device__ __forceinline__ void chain_release() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void chain_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Shared-memory layout of the row kernels (bytes).  The tensor-core operands
// come first (16-byte aligned, which the no-swizzle layout needs), then the FP32 work arrays.
template <int P> struct RowSmem {
  static constexpr int A = 0;                        // 128 x 32 BF16 activations, canonical layout
  static constexpr int BW = A + kW * kC * 2;         // 32 x 32 BF16 pointwise weights (N x K)
  static constexpr int BQ = BW + kC * kC * 2;        // P x 32 BF16 projection weights (N x K)
  // the inverse x-DFT as a product with the same accumulator: G (x, (kx, re/im))
  // and U ((c), (kx, re/im)), each split into BF16 high and low parts
  static constexpr int GH = BQ + P * kC * 2;         // 128 x 32 BF16
  static constexpr int GL = GH + kW * kK2 * 2;
  static constexpr int UH = GL + kW * kK2 * 2;       // 32 x 32 BF16 (N = channels, K = modes)
  static constexpr int UL = UH + kC * kK2 * 2;
  static constexpr int TWX = UL + kC * kK2 * 2;      // cos, sin (2 pi t / W)
  static constexpr int TWY = TWX + 2 * kW * 4;              // cos, sin (2 pi t / H)
  static constexpr int SV = TWY + 2 * kFusedMaxH * 4;       // [W][C] FP32 activations / y partials
  static constexpr int PART = SV + kW * kC * 4;             // [kQ][MX][2][C] DFT partial sums
  static constexpr int BAR = PART + kQ * kFusedMaxMX * 2 * kC * 4;  // two mbarriers, the TMEM address
  static constexpr int SY = BAR + 128;                             // this sample's mixed modes Y[b]
  static constexpr uint32_t TMEM_COLS = P > kC ? P : kC;  // a power of two >= 32
  // tcgen05.alloc waits while the SM's 512 TMEM columns are taken: the CTA's
  // shared memory is padded so that no more than 512 / TMEM_COLS of them are
  // resident on an SM (228 KB per SM, 1 KB reserved per CTA)
  static constexpr int MIN_BYTES = 228 * 1024 / (512 / (int)TMEM_COLS + 1);
  static constexpr int BYTES = SY + kFusedMaxModes * 2 * kC * 4 > MIN_BYTES ? SY + kFusedMaxModes * 2 * kC * 4
                                                                           : MIN_BYTES;
};

// the lift kernel uses the layout up to the barriers
constexpr int kLiftBytes = RowSmem<0>::BAR + 32;

// v_l row (FP32 in sv, [x][c]) -> A[kx][re/im][c] = sum_x v (cos, -sin)(2 pi kx x / W).
// kRT threads: thread = (x quarter, kx, four channels); the quarters meet in `part`.
__device__ __forceinline__ void row_dft_x(const float* sv, const float* twx, float* part, float* dst, int MX) {
  const int tid = threadIdx.x;
  const int item = tid & 127, half = tid >> 7;  // (the x quarter)
  if (item < MX * (kC / 4)) {
    const int kx = item / (kC / 4), c = (item % (kC / 4)) * 4;
    float4 re = make_float4(0.f, 0.f, 0.f, 0.f), im = re;
    const int x0 = half * (kW / kQ);
    int t = (kx * x0) & (kW - 1);
    for (int x = x0; x < x0 + kW / kQ; ++x) {
      const float4 v = *reinterpret_cast<const float4*>(&sv[x * kC + c]);
      const float co = twx[2 * t], si = twx[2 * t + 1];
      re.x = fmaf(v.x, co, re.x);
      re.y = fmaf(v.y, co, re.y);
      re.z = fmaf(v.z, co, re.z);
      re.w = fmaf(v.w, co, re.w);
      im.x = fmaf(-v.x, si, im.x);
      im.y = fmaf(-v.y, si, im.y);
      im.z = fmaf(-v.z, si, im.z);
      im.w = fmaf(-v.w, si, im.w);
      t = (t + kx) & (kW - 1);
    }
    float* p = part + half * (kFusedMaxMX * 2 * kC);
    *reinterpret_cast<float4*>(&p[(kx * 2) * kC + c]) = re;
    *reinterpret_cast<float4*>(&p[(kx * 2 + 1) * kC + c]) = im;
  }
  __syncthreads();
  for (int e = tid; e < MX * 2 * kC; e += kRT) {
    float v = part[e];
#pragma unroll
    for (int q = 1; q < kQ; ++q) v += part[q * kFusedMaxMX * 2 * kC + e];
    dst[e] = v;
  }
}

}  // namespace

// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kRT) k_fused_lift(FusedFwdArgs a) {
  extern __shared__ __align__(16) unsigned char fused_sm[];
  typedef RowSmem<0> L;
  float* twx = reinterpret_cast<float*>(fused_sm + L::TWX);
  float* sv = reinterpret_cast<float*>(fused_sm + L::SV);
  float* part = reinterpret_cast<float*>(fused_sm + L::PART);
  const int row = blockIdx.x, tid = threadIdx.x;  // row = b * H + y
  float* sx = part;                 // the row's inputs [W][CI] (CI <= 8)
  float* sw = part + kW * 8;        // P [CI][C], then p [C]
  chain_release();
  for (int e = tid; e < 2 * kW; e += kRT) twx[e] = a.csx[e];
  for (int e = tid; e < a.CI * kC; e += kRT) sw[e] = a.Pw[e];
  for (int e = tid; e < kC; e += kRT) sw[a.CI * kC + e] = a.Pb[e];
  chain_wait();
  const float* xr = a.x + (size_t)row * kW * a.CI;
  for (int e = tid; e < kW * a.CI; e += kRT) sx[e] = xr[e];
  __syncthreads();
  float* vout = a.v[0] + (size_t)row * kW * kC;
  for (int e = tid; e < kW * kC; e += kRT) {
    const int x = e / kC, c = e % kC;
    float s = sw[a.CI * kC + c];
    for (int i = 0; i < a.CI; ++i) s = fmaf(sx[x * a.CI + i], sw[i * kC + c], s);
    sv[e] = s;
    vout[e] = s;
  }
  __syncthreads();
  row_dft_x(sv, twx, part, a.A + (size_t)row * a.MX * 2 * kC, a.MX);
}

// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads, 1) k_fused_col(FusedFwdArgs a, int layer) {
  extern __shared__ __align__(16) float smf[];
  constexpr int K2 = 2 * kC;
  const int H = a.H, MX = a.MX, MY = a.MY, C2 = K2;
  float* sa = smf;                         // [H][2C] column kx of A
  float* sr = sa + H * K2;                 // [kModeGroup][2C][2C] the group's block matrices
  float* twy = sr + kModeGroup * K2 * K2;  // [H][2]
  float* part = twy + 2 * H;               // [2][kModeGroup][2C]
  float* xs = part + 2 * kModeGroup * K2;  // [kModeGroup][2C] X (BF16-rounded in BF16 mode)
  unsigned long long* lbar = reinterpret_cast<unsigned long long*>(xs + kModeGroup * K2);
  const uint32_t lb = umma::smem_addr(lbar);
  const int tid = threadIdx.x;
  const int b = blockIdx.x / MX, kx = blockIdx.x % MX, j0 = blockIdx.y * kModeGroup;
  // bulk copies: the group's block matrices (16 KB each) and the H row
  // segments (256 B) of column kx, all in flight together
  const float* Rb = a.Rb[layer];
  chain_release();
  if (tid == 0) {
    umma::mbar_init(lb, 1);
    umma::mbar_expect_tx(lb, (uint32_t)((H * K2 + kModeGroup * K2 * K2) * 4));
    for (int jj = 0; jj < kModeGroup; ++jj)
      umma::bulk_g2s(umma::smem_addr(sr + jj * K2 * K2), Rb + ((size_t)(j0 + jj) * MX + kx) * K2 * K2,
                     K2 * K2 * 4, lb);
  }
  for (int e = tid; e < 2 * H; e += kThreads) twy[e] = a.csy[e];
  __syncthreads();  // the barrier is initialised and armed before the row copies
  chain_wait();
  for (int y = tid; y < H; y += kThreads)
    umma::bulk_g2s(umma::smem_addr(sa + y * K2), a.A + (((size_t)b * H + y) * MX + kx) * K2, K2 * 4, lb);
  const bool ok = umma::mbar_wait(lb, 0, kFwWait);
  if (__syncthreads_or(!ok)) {
    umma::mbar_wait(lb, 0, kFwWait);  // the copies in flight, once more, before the CTA ends
    if (tid == 0) atomicOr(a.err, 4u);
    return;
  }
  {  // X[j, c] = sum_y A[y, c] exp(-2 pi i ky(j) y / H), the y range in two halves
    const int item = tid & (kModeGroup * kC - 1), half = tid / (kModeGroup * kC);
    const int jj = item / kC, c = item % kC, j = j0 + jj;
    const int ky = j < MY / 2 ? j : j - MY;
    const int step = ky & (H - 1), y0 = half * (H / 2);
    float re = 0.f, im = 0.f;
    int t = (step * y0) & (H - 1);
    for (int y = y0; y < y0 + H / 2; ++y) {
      const float co = twy[2 * t], si = -twy[2 * t + 1];
      const float ar = sa[y * C2 + c], ai = sa[y * C2 + kC + c];
      re = fmaf(ar, co, fmaf(-ai, si, re));
      im = fmaf(ar, si, fmaf(ai, co, im));
      t = (t + step) & (H - 1);
    }
    part[(half * kModeGroup + jj) * C2 + c] = re;
    part[(half * kModeGroup + jj) * C2 + kC + c] = im;
  }
  __syncthreads();
  for (int e = tid; e < kModeGroup * C2; e += kThreads) {
    const float v = part[e] + part[kModeGroup * C2 + e];
    xs[e] = a.bf16 ? bf16r(v) : v;
  }
  __syncthreads();
  // Y[b, j, kx, o] = sum_k X[j, k] Rb[j, kx][k, o], one output per thread
  for (int e = tid; e < kModeGroup * K2; e += kThreads) {
    const int jj = e / K2, o = e % K2, j = j0 + jj;
    const float* R = sr + jj * K2 * K2 + o;
    float acc = 0.f;
#pragma unroll 16
    for (int k = 0; k < K2; ++k) {
      const float r = R[k * K2];
      acc = fmaf(xs[jj * K2 + k], a.bf16 ? bf16r(r) : r, acc);
    }
    a.Y[(((size_t)b * MY + j) * MX + kx) * K2 + o] = acc;
  }
}

// ---------------------------------------------------------------------------
template <int P>
__global__ void __launch_bounds__(kRT, 1) k_fused_row(FusedFwdArgs a, int layer) {
  typedef RowSmem<P> L;
  extern __shared__ __align__(16) unsigned char fused_sm[];
  __nv_bfloat16* As = reinterpret_cast<__nv_bfloat16*>(fused_sm + L::A);
  __nv_bfloat16* Bw = reinterpret_cast<__nv_bfloat16*>(fused_sm + L::BW);
  __nv_bfloat16* Bq = reinterpret_cast<__nv_bfloat16*>(fused_sm + L::BQ);
  unsigned char* gh = fused_sm + L::GH;
  unsigned char* gl = fused_sm + L::GL;
  unsigned char* uh = fused_sm + L::UH;
  unsigned char* ul = fused_sm + L::UL;
  float* twx = reinterpret_cast<float*>(fused_sm + L::TWX);
  float* twy = reinterpret_cast<float*>(fused_sm + L::TWY);
  float* sv = reinterpret_cast<float*>(fused_sm + L::SV);
  float* part = reinterpret_cast<float*>(fused_sm + L::PART);
  float* sy = reinterpret_cast<float*>(fused_sm + L::SY);
  unsigned long long* mbar = reinterpret_cast<unsigned long long*>(fused_sm + L::BAR);  // MMA completion
  unsigned long long* lbar = mbar + 1;                                                  // bulk copies
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(fused_sm + L::BAR + 16);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int row = blockIdx.x, H = a.H, MX = a.MX, MY = a.MY, C2 = 2 * kC;
  const int b = row / H, y = row % H;
  const uint32_t mb = umma::smem_addr(mbar), lb = umma::smem_addr(lbar);
  chain_release();
  if (tid == 0) {
    umma::mbar_init(mb, 1);
    umma::mbar_init(lb, 1);
  }
  const float* Wl = a.Wl[layer];
  for (int e = tid; e < kC * kC; e += kRT) {  // B(k, n) = W[k C + n] as row n of an N x K operand
    const int k = e / kC, n = e % kC;
    *reinterpret_cast<__nv_bfloat16*>(reinterpret_cast<char*>(Bw) + umma::elem_offset<kC>(n, k)) =
        __float2bfloat16_rn(Wl[e]);
  }
  if constexpr (P > 0) {
    for (int e = tid; e < kC * P; e += kRT) {  // Q1(k, n) = Q1[k P + n]
      const int k = e / P, n = e % P;
      *reinterpret_cast<__nv_bfloat16*>(reinterpret_cast<char*>(Bq) + umma::elem_offset<kC>(n, k)) =
          __float2bfloat16_rn(a.Q1[e]);
    }
  }
  for (int e = tid; e < 2 * kW; e += kRT) twx[e] = a.csx[e];
  for (int e = tid; e < 2 * H; e += kRT) twy[e] = a.csy[e];
  // G[x, (kx, re)] = cos, G[x, (kx, im)] = -sin (2 pi kx x / W), zero past 2 MX;
  // and the U columns past 2 MX, zero
  for (int e = tid; e < kW * kK2; e += kRT) {
    const int x = e / kK2, k = e % kK2, kx = k >> 1;
    float g = 0.f;
    if (kx < MX) {
      const int t = (kx * x) & (kW - 1);
      g = (k & 1) ? -a.csx[2 * t + 1] : a.csx[2 * t];
    }
    split_store(gh, gl, umma::elem_offset<kK2>(x, k), g);
  }
  for (int e = tid; e < kC * (kK2 - 2 * MX); e += kRT) {
    const int c = e / (kK2 - 2 * MX), k = 2 * MX + e % (kK2 - 2 * MX);
    split_store(uh, ul, umma::elem_offset<kK2>(c, k), 0.f);
  }
  if (warp == 0) umma::alloc(umma::smem_addr(tmem_slot), L::TMEM_COLS);
  // then one thread starts the bulk copies of this sample's mixed modes Y[b]
  // (all rows need all of them) and of v_{l-1}'s row (FP32, into sv)
  chain_wait();
  const float* vin = a.v[layer - 1] + (size_t)row * kW * kC;
  const uint32_t ybytes = (uint32_t)(MY * MX * C2 * 4), vbytes = kW * kC * 4;
  if (tid == 0) {
    umma::mbar_expect_tx(lb, ybytes + vbytes);
    const char* ysrc = reinterpret_cast<const char*>(a.Y + (size_t)b * MY * MX * C2);
    for (uint32_t o = 0; o < ybytes; o += kBulkChunk)
      umma::bulk_g2s(umma::smem_addr(sy) + o, ysrc + o, ybytes - o < kBulkChunk ? ybytes - o : kBulkChunk, lb);
    umma::bulk_g2s(umma::smem_addr(sv), vin, vbytes, lb);
  }
  __syncthreads();  // the barriers are initialised
  bool ok = umma::mbar_wait(lb, 0, kFwWait);
  if (__syncthreads_or(!ok)) {
    umma::mbar_wait(lb, 0, kFwWait);  // the copies in flight, once more, before the CTA ends
    if (tid == 0) atomicOr(a.err, 4u);
  }
  // the pointwise operand: v_{l-1}'s row as BF16, K-major canonical
  for (int e = tid; e < kW * kC / 4; e += kRT) {
    const int r = e / (kC / 4), k4 = (e % (kC / 4)) * 4;
    const float4 v = *reinterpret_cast<const float4*>(sv + r * kC + k4);
    __nv_bfloat162* d = reinterpret_cast<__nv_bfloat162*>(reinterpret_cast<char*>(As) + umma::elem_offset<kC>(r, k4));
    d[0] = __floats2bfloat162_rn(v.x, v.y);
    d[1] = __floats2bfloat162_rn(v.z, v.w);
  }
  umma::fence_proxy_async();
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = *tmem_slot;
  constexpr uint32_t kSbo = (kC / 8) * 128;
  static_assert(kK2 == kC, "one stride serves both K = 32 operands");
  // U[kx, c] = w_kx sum_j Y[b, j, kx, c] exp(+2 pi i ky(j) y / H) for this row
  for (int e = tid; e < MX * kC; e += kRT) {
    const int kx = e / kC, c = e % kC;
    float re = 0.f, im = 0.f;
    for (int j = 0; j < MY; ++j) {
      const int ky = j < MY / 2 ? j : j - MY;
      const int t = (ky * y) & (H - 1);
      const float co = twy[2 * t], si = twy[2 * t + 1];
      const float* yj = sy + (j * MX + kx) * C2;
      const float vr = yj[c], vi = yj[kC + c];
      re = fmaf(vr, co, fmaf(-vi, si, re));
      im = fmaf(vr, si, fmaf(vi, co, im));
    }
    const float s = a.wx[kx];
    split_store(uh, ul, umma::elem_offset<kK2>(c, 2 * kx), re * s);
    split_store(uh, ul, umma::elem_offset<kK2>(c, 2 * kx + 1), im * s);
  }
  umma::fence_proxy_async();
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  // z = v W + G U: M = 128 rows (x), N = 32; v W in BF16 (K = 32 channels) and the
  // inverse x-DFT G U in split BF16 (G_hi U_hi + G_hi U_lo + G_lo U_hi, K = 32 modes)
  if (ok && tid == 0) {
    const uint32_t idesc = umma::idesc_bf16_f32(kW, kC);
    const uint32_t pa[4] = {umma::smem_addr(As), umma::smem_addr(gh), umma::smem_addr(gh), umma::smem_addr(gl)};
    const uint32_t pb[4] = {umma::smem_addr(Bw), umma::smem_addr(uh), umma::smem_addr(ul), umma::smem_addr(uh)};
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
      for (int s = 0; s < kC / 16; ++s)
        umma::mma_bf16(tmem, umma::smem_desc(pa[q] + 2 * s * 128, 128, kSbo),
                       umma::smem_desc(pb[q] + 2 * s * 128, 128, kSbo), idesc, (q > 0 || s > 0) ? 1u : 0u);
    umma::commit(mb);
  }
  // this thread: row x (its TMEM lane) and kCpt channels
  const int lg = warp & 3, x = lg * 32 + lane, c0 = (warp >> 2) * kCpt;
  float z[kCpt];
#pragma unroll
  for (int i = 0; i < kCpt; ++i) z[i] = 0.f;
  if (ok) {  // (uniform over the CTA)
    ok = umma::mbar_wait(mb, 0, kFwWait);
    umma::fence_after_sync();
    if (__syncthreads_or(!ok)) {
      umma::mbar_wait(mb, 0, kFwWait);  // a second bounded wait for the MMAs in flight
      if (tid == 0) atomicOr(a.err, 4u);
      ok = false;
    }
  }
  const bool last = P > 0;
  const float* bl = a.bl[layer];
  if (ok) {
    float acc[kCpt];
    umma::ld_8cols(tmem + ((uint32_t)(lg * 32) << 16) + (uint32_t)c0, acc);
#pragma unroll
    for (int i = 0; i < kCpt; ++i) {
      const float zz = acc[i] + bl[c0 + i];
      z[i] = last ? zz : gelu_f(zz);  // v_l (the last Fourier layer has no activation)
    }
  }
  if constexpr (P == 0) {
    float* vout = a.v[layer] + (size_t)row * kW * kC;
#pragma unroll
    for (int i = 0; i < kCpt; i += 4) {
      const float4 q = make_float4(z[i], z[i + 1], z[i + 2], z[i + 3]);
      *reinterpret_cast<float4*>(&sv[x * kC + c0 + i]) = q;
      *reinterpret_cast<float4*>(&vout[x * kC + c0 + i]) = q;
    }
    __syncthreads();
    row_dft_x(sv, twx, part, a.A + (size_t)row * MX * 2 * kC, MX);
  } else {
    // the projection's A operand: v_L, BF16, over the pointwise operand (consumed)
#pragma unroll
    for (int i = 0; i < kCpt; i += 2)
      *reinterpret_cast<__nv_bfloat162*>(reinterpret_cast<char*>(As) + umma::elem_offset<kC>(x, c0 + i)) =
          __floats2bfloat162_rn(z[i], z[i + 1]);
    umma::fence_proxy_async();
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    if (ok && tid == 0) {  // zh = v_L Q1: N = P
      const uint32_t a0 = umma::smem_addr(As), b0 = umma::smem_addr(Bq);
      const uint32_t idesc = umma::idesc_bf16_f32(kW, P);
#pragma unroll
      for (int s = 0; s < kC / 16; ++s)
        umma::mma_bf16(tmem, umma::smem_desc(a0 + 2 * s * 128, 128, kSbo),
                       umma::smem_desc(b0 + 2 * s * 128, 128, kSbo), idesc, s > 0);
      umma::commit(mb);
    }
    if (ok) {
      ok = umma::mbar_wait(mb, 1, kFwWait);
      umma::fence_after_sync();
      if (__syncthreads_or(!ok)) {
        umma::mbar_wait(mb, 1, kFwWait);
        if (tid == 0) atomicOr(a.err, 4u);
        ok = false;
      }
    }
    // h = GELU(zh + q1) over this thread's quarter of the P columns; y = h Q2 + q2
    float ys[kFusedMaxCO] = {0.f, 0.f, 0.f, 0.f};
    const int p0 = (warp >> 2) * (P / kQ);
    if (ok) {
#pragma unroll 1
      for (int q0 = 0; q0 < P / kQ; q0 += 8) {
        float hv[8];
        umma::ld_8cols(tmem + ((uint32_t)(lg * 32) << 16) + (uint32_t)(p0 + q0), hv);
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const int p = p0 + q0 + i;
          const float h = gelu_f(hv[i] + a.q1[p]);
#pragma unroll
          for (int o = 0; o < kFusedMaxCO; ++o)
            if (o < a.CO) ys[o] = fmaf(h, a.Q2[p * a.CO + o], ys[o]);
        }
      }
    }
    float* yp = sv;  // [kQ][W][4] partial sums of the column quarters
#pragma unroll
    for (int o = 0; o < kFusedMaxCO; ++o) yp[((warp >> 2) * kW + x) * kFusedMaxCO + o] = ys[o];
    __syncthreads();
    for (int e = tid; e < kW * a.CO; e += kRT) {
      const int xx = e / a.CO, o = e % a.CO;
      float v = yp[xx * kFusedMaxCO + o];
#pragma unroll
      for (int q = 1; q < kQ; ++q) v += yp[(q * kW + xx) * kFusedMaxCO + o];
      a.y[(size_t)row * kW * a.CO + e] = v + a.q2[o];
    }
  }
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  if (warp == 0) umma::dealloc(tmem, L::TMEM_COLS);
}

// ---------------------------------------------------------------------------
bool fused_forward_supported(int B, int H, int W, int C, int MX, int MY, int CI, int P, int CO) {
  return B >= 1 && B <= kFusedMaxB && W == kW && C == kC && H >= 16 && H <= kFusedMaxH && (H & (H - 1)) == 0 &&
         MX >= 1 && MX <= kFusedMaxMX && MY >= kModeGroup && MY % kModeGroup == 0 && MY <= H &&
         MX * MY <= kFusedMaxModes && CI >= 1 &&
         CI <= 8 && CO >= 1 && CO <= kFusedMaxCO && (P == 32 || P == 64 || P == 128 || P == 256);
}

// A kernel of the chain, launched with programmatic stream serialisation.
template <typename... KArgs, typename... Args>
static cudaError_t chain_launch(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                                Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}

template <int P>
static int launch_rows(const FusedFwdArgs& a, int layer, cudaStream_t s) {
  typedef RowSmem<P> L;
  static const cudaError_t attr =
      cudaFuncSetAttribute(k_fused_row<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, L::BYTES);
  TARA_CK(attr);
  TARA_CK(chain_launch(k_fused_row<P>, dim3(a.B * a.H), dim3(kRT), L::BYTES, s, a, layer));
  return TARA_OK;
}

int fused_forward_launch(const FusedFwdArgs& a, cudaStream_t s) {
  if (!fused_forward_supported(a.B, a.H, kW, kC, a.MX, a.MY, a.CI, a.P, a.CO) || a.layers < 1 ||
      a.layers > kFusedMaxLayers)
    return set_error(TARA_ERR_ARGS, "shape outside the fused forward");
  static const cudaError_t attr =
      cudaFuncSetAttribute(k_fused_lift, cudaFuncAttributeMaxDynamicSharedMemorySize, kLiftBytes);
  TARA_CK(attr);
  TARA_CK(chain_launch(k_fused_lift, dim3(a.B * a.H), dim3(kRT), kLiftBytes, s, a));
  // column, block matrices, twiddles, partial sums, X; then the mbarrier
  auto col_bytes = [](int h) {
    return (size_t)(h * 2 * kC + kModeGroup * 4 * kC * kC + 2 * h + 3 * kModeGroup * 2 * kC) * sizeof(float) + 16;
  };
  const size_t col_smem = col_bytes(a.H);
  static const cudaError_t cattr =
      cudaFuncSetAttribute(k_fused_col, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)col_bytes(kFusedMaxH));
  TARA_CK(cattr);
  for (int l = 1; l <= a.layers; ++l) {
    TARA_CK(chain_launch(k_fused_col, dim3(a.B * a.MX, a.MY / kModeGroup), dim3(kThreads), col_smem, s, a, l));
    int rc = TARA_OK;
    if (l < a.layers)
      rc = launch_rows<0>(a, l, s);
    else if (a.P == 32)
      rc = launch_rows<32>(a, l, s);
    else if (a.P == 64)
      rc = launch_rows<64>(a, l, s);
    else if (a.P == 128)
      rc = launch_rows<128>(a, l, s);
    else
      rc = launch_rows<256>(a, l, s);
    if (rc) return rc;
  }
  return TARA_OK;
}

}  // namespace tara
