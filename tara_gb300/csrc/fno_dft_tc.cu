// The closure network's truncated DFTs along x on the 5th-generation tensor
// cores (BF16 modes of the network), as products with the DFT matrix:
//
//   k_x2m_tc<C>   A[row, kx, re/im, c] = s_kx sum_x v[row, x, c] (cos, -sin)(2 pi kx x / W)
//                 one tcgen05 product per tile of 128 / C rows: D[(r, c), (kx, re/im)] =
//                 sum_x V[(r, c), x] F[(kx, re/im), x]   (M = 128, N = 2 MX, K = W)
//   k_m2x_tc<C>   out[row, x, c] (+)= sum_kx s_kx (A_re cos - A_im sin)(2 pi kx x / W)
//                 per row: D[x, c] = sum_(kx, re/im) G[x, (kx, re/im)] A'[(kx, re/im), c]
//                 (M = W = 128, N = C, K = 2 MX), four rows per round in four
//                 accumulators of tensor memory.
//
// Operands are FP32 values split into two BF16 parts, v = v_hi + v_lo
// (v_hi = bf16(v), v_lo = bf16(v - v_hi)), and each product is taken as
// a_hi b_hi + a_hi b_lo + a_lo b_hi into the FP32 accumulator (the split-BF16
// form of an FP32 product; the dropped a_lo b_lo term and the rounding of the
// low parts leave about 2^-16 relative per term), so the transforms keep
// FP32-level accuracy, as the CUDA-core kernels they replace in the BF16 modes.
// Operands sit in shared memory in the no-swizzle K-major layout of umma.cuh;
// every mbarrier wait is bounded (a wait that gives up sets value 4 in *err and
// the CTA stops, after a second bounded wait for its MMAs in flight).
#include <cstdint>

#include <cuda_bf16.h>

#include "internal.h"
#include "umma.cuh"

namespace tara {

namespace {

constexpr uint32_t kDftWait = 1u << 20;

// byte offset of element (r, k) of an R x K BF16 operand, K a multiple of 8
__device__ __forceinline__ uint32_t coff(int r, int k, int K) {
  return (uint32_t)(((r >> 3) * (K >> 3) + (k >> 3)) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

__device__ __forceinline__ void split_bf16(float v, __nv_bfloat16& hi, __nv_bfloat16& lo) {
  hi = __float2bfloat16_rn(v);
  lo = __float2bfloat16_rn(v - __bfloat162float(hi));
}

// hi and lo parts of four consecutive K values of row r, as two 8-byte stores
__device__ __forceinline__ void store4(unsigned char* hi_base, unsigned char* lo_base, int r, int k, int K,
                                       float a, float b, float c, float d) {
  __nv_bfloat16 h[4], l[4];
  split_bf16(a, h[0], l[0]);
  split_bf16(b, h[1], l[1]);
  split_bf16(c, h[2], l[2]);
  split_bf16(d, h[3], l[3]);
  const uint32_t o = coff(r, k, K);
  uint2 hv, lv;
  hv.x = (uint32_t)__bfloat16_as_ushort(h[0]) | ((uint32_t)__bfloat16_as_ushort(h[1]) << 16);
  hv.y = (uint32_t)__bfloat16_as_ushort(h[2]) | ((uint32_t)__bfloat16_as_ushort(h[3]) << 16);
  lv.x = (uint32_t)__bfloat16_as_ushort(l[0]) | ((uint32_t)__bfloat16_as_ushort(l[1]) << 16);
  lv.y = (uint32_t)__bfloat16_as_ushort(l[2]) | ((uint32_t)__bfloat16_as_ushort(l[3]) << 16);
  *reinterpret_cast<uint2*>(hi_base + o) = hv;
  *reinterpret_cast<uint2*>(lo_base + o) = lv;
}

// the three split products D (+)= A_hi B_hi + A_hi B_lo + A_lo B_hi, K / 16 steps each
__device__ __forceinline__ void mma3(uint32_t tmem, uint32_t ah, uint32_t al, uint32_t bh, uint32_t bl, int K,
                                     uint32_t idesc) {
  const uint32_t sbo = (uint32_t)(K / 8) * 128;
  for (int p = 0; p < 3; ++p) {
    const uint32_t a = p < 2 ? ah : al, b = p == 1 ? bl : bh;
    for (int s = 0; s < K / 16; ++s)
      umma::mma_bf16(tmem, umma::smem_desc(a + 2 * s * 128, 128, sbo), umma::smem_desc(b + 2 * s * 128, 128, sbo),
                     idesc, (p > 0 || s > 0) ? 1u : 0u);
  }
}

// TMEM columns to allocate for n accumulator columns: a power of two >= 32
__host__ __device__ constexpr uint32_t tmem_cols(int n) { return n <= 32 ? 32u : n <= 64 ? 64u : n <= 128 ? 128u : 256u; }

}  // namespace

// ---------------------------------------------------------------------------
// forward x-DFT: 256 threads; tiles of R = 128 / C rows
template <int C>
__global__ void __launch_bounds__(256, 1) k_x2m_tc(const float* __restrict__ v, float* __restrict__ out,
                                                 long long rows, int W, int MX, const float* __restrict__ cs,
                                                 const float* __restrict__ scale, unsigned int* err) {
  constexpr int R = 128 / C;
  extern __shared__ __align__(16) unsigned char dsm[];
  const int N = 2 * MX, K = W;
  unsigned char* ah = dsm;                     // [128][K] V^T, BF16 high parts
  unsigned char* al = ah + 128 * K * 2;        // low parts
  unsigned char* bh = al + 128 * K * 2;        // [N][K] F, high parts
  unsigned char* bl = bh + N * K * 2;          // low parts
  unsigned long long* mbar = reinterpret_cast<unsigned long long*>(bl + N * K * 2);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(mbar + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // F[(kx, re/im), x] = (cos, -sin)(2 pi kx x / W)
  for (int e = tid; e < N * (K / 4); e += 256) {
    const int n = e / (K / 4), x0 = (e % (K / 4)) * 4, kx = n >> 1;
    float f[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int t = (kx * (x0 + i)) & (W - 1);
      f[i] = (n & 1) ? -cs[2 * t + 1] : cs[2 * t];
    }
    store4(bh, bl, n, x0, K, f[0], f[1], f[2], f[3]);
  }
  const uint32_t cols = tmem_cols(N);
  const uint32_t mb = umma::smem_addr(mbar);
  if (warp == 0) umma::alloc(umma::smem_addr(tslot), cols);
  if (tid == 0) umma::mbar_init(mb, 1);
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = *tslot;
  const uint32_t idesc = umma::idesc_bf16_f32(128, N);
  const uint32_t uah = umma::smem_addr(ah), ual = umma::smem_addr(al), ubh = umma::smem_addr(bh),
                 ubl = umma::smem_addr(bl);
  uint32_t parity = 0;
  bool failed = false;
  const long long tiles = (rows + R - 1) / R;
  for (long long tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const long long row0 = tile * R;
    // V^T: element ((r, c), x) = v[row0 + r, x, c]; a work item is 4 x values of
    // 4 channels (four 16-byte loads, eight 8-byte stores)
    for (int e = tid; e < R * (K / 4) * (C / 4); e += 256) {
      const int c4 = (e % (C / 4)) * 4, x4 = ((e / (C / 4)) % (K / 4)) * 4, r = e / ((C / 4) * (K / 4));
      float4 q[4];
      const bool in = row0 + r < rows;
      const float* src = v + ((row0 + r) * K + x4) * C + c4;
#pragma unroll
      for (int i = 0; i < 4; ++i)
        q[i] = in ? *reinterpret_cast<const float4*>(src + i * C) : make_float4(0.f, 0.f, 0.f, 0.f);
      const int m = r * C + c4;
      store4(ah, al, m + 0, x4, K, q[0].x, q[1].x, q[2].x, q[3].x);
      store4(ah, al, m + 1, x4, K, q[0].y, q[1].y, q[2].y, q[3].y);
      store4(ah, al, m + 2, x4, K, q[0].z, q[1].z, q[2].z, q[3].z);
      store4(ah, al, m + 3, x4, K, q[0].w, q[1].w, q[2].w, q[3].w);
    }
    umma::fence_proxy_async();
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    if (tid == 0) {
      mma3(tmem, uah, ual, ubh, ubl, K, idesc);
      umma::commit(mb);
    }
    const bool ok = umma::mbar_wait(mb, parity, kDftWait);
    if (__syncthreads_or(!ok)) {
      umma::mbar_wait(mb, parity, kDftWait);
      failed = true;
      break;
    }
    parity ^= 1u;
    umma::fence_after_sync();
    // epilogue: thread (lane group = warp % 4, column half = warp / 4) owns
    // accumulator row m = (r, c) and half of the N columns
    const int m = (warp & 3) * 32 + lane, r = m / C, c = m % C;
    const long long row = row0 + r;
    const int n0 = (warp >> 2) * (N / 2);
    for (int nc = 0; nc < N / 2; nc += 8) {
      float d[8];
      umma::ld_8cols(tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)(n0 + nc), d);
      if (row < rows) {
        float* o = out + (size_t)row * N * C + c;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const int n = n0 + nc + i;
          o[(size_t)n * C] = scale ? d[i] * scale[n >> 1] : d[i];
        }
      }
    }
    umma::fence_before_sync();
    __syncthreads();  // the accumulator and the operand buffer are free again
  }
  if (failed && tid == 0) atomicOr(err, 4u);
  __syncthreads();
  umma::fence_after_sync();
  if (warp == 0) umma::dealloc(tmem, cols);
}

// ---------------------------------------------------------------------------
// inverse x-DFT at W = 128: 256 threads, four rows per round
template <int C>
__global__ void __launch_bounds__(256, 1) k_m2x_tc(const float* __restrict__ a, float* __restrict__ out,
                                                 long long rows, int MX, const float* __restrict__ cs,
                                                 const float* __restrict__ scale, int accumulate,
                                                 unsigned int* err) {
  constexpr int W = 128, RB = 4;
  extern __shared__ __align__(16) unsigned char dsm[];
  const int K = 2 * MX;
  unsigned char* gh = dsm;                    // [128][K] G, high parts
  unsigned char* gl = gh + W * K * 2;         // low parts
  unsigned char* bh = gl + W * K * 2;         // [RB][C][K] A'^T of the round's rows, high
  unsigned char* bl = bh + RB * C * K * 2;    // low
  // the round's output rows [RB][W][C + 4] (FP32), staged so that the stores to
  // memory go out as contiguous 16-byte runs across the CTA
  constexpr int SP = C + 4;
  float* stage = reinterpret_cast<float*>(bl + RB * C * K * 2);
  unsigned long long* mbar = reinterpret_cast<unsigned long long*>(stage + RB * W * SP);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(mbar + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // G[x, (kx, re/im)] = (cos, -sin)(2 pi kx x / W)
  for (int e = tid; e < W * (K / 4); e += 256) {
    const int x = e / (K / 4), k0 = (e % (K / 4)) * 4;
    float g[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int k = k0 + i, kx = k >> 1, t = (kx * x) & (W - 1);
      g[i] = (k & 1) ? -cs[2 * t + 1] : cs[2 * t];
    }
    store4(gh, gl, x, k0, K, g[0], g[1], g[2], g[3]);
  }
  constexpr uint32_t cols = tmem_cols(RB * C);
  const uint32_t mb = umma::smem_addr(mbar);
  if (warp == 0) umma::alloc(umma::smem_addr(tslot), cols);
  if (tid == 0) umma::mbar_init(mb, 1);
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = *tslot;
  const uint32_t idesc = umma::idesc_bf16_f32(W, C);
  const uint32_t ugh = umma::smem_addr(gh), ugl = umma::smem_addr(gl), ubh = umma::smem_addr(bh),
                 ubl = umma::smem_addr(bl);
  uint32_t parity = 0;
  bool failed = false;
  const long long rounds = (rows + RB - 1) / RB;
  for (long long rd = blockIdx.x; rd < rounds; rd += gridDim.x) {
    const long long row0 = rd * RB;
    // B operand of row j: element (c, k = (kx, re/im)) = s_kx a[row, kx, re/im, c];
    // a work item is 4 consecutive k of one channel
    for (int e = tid; e < RB * C * (K / 4); e += 256) {
      const int c = e % C, k0 = ((e / C) % (K / 4)) * 4, j = e / (C * (K / 4));
      const long long row = row0 + j;
      float q[4] = {0.f, 0.f, 0.f, 0.f};
      if (row < rows) {
        const float* src = a + (size_t)row * K * C + c;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int k = k0 + i;
          q[i] = src[(size_t)k * C] * (scale ? scale[k >> 1] : 1.f);
        }
      }
      store4(bh + j * C * K * 2, bl + j * C * K * 2, c, k0, K, q[0], q[1], q[2], q[3]);
    }
    umma::fence_proxy_async();
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    if (tid == 0) {
      for (int j = 0; j < RB; ++j)
        mma3(tmem + (uint32_t)(j * C), ugh, ugl, ubh + j * C * K * 2, ubl + j * C * K * 2, K, idesc);
      umma::commit(mb);
    }
    const bool ok = umma::mbar_wait(mb, parity, kDftWait);
    if (__syncthreads_or(!ok)) {
      umma::mbar_wait(mb, parity, kDftWait);
      failed = true;
      break;
    }
    parity ^= 1u;
    umma::fence_after_sync();
    // epilogue: thread (lane group = warp % 4 -> x, warp / 4 -> rows j = 2 (warp / 4) + {0, 1})
    const int x = (warp & 3) * 32 + lane;
    for (int jj = 0; jj < RB / 2; ++jj) {
      const int j = (warp >> 2) * (RB / 2) + jj;
      for (int c0 = 0; c0 < C; c0 += 8) {
        float d[8];
        umma::ld_8cols(tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)(j * C + c0), d);
        float4* st = reinterpret_cast<float4*>(stage + (j * W + x) * SP + c0);
        st[0] = make_float4(d[0], d[1], d[2], d[3]);
        st[1] = make_float4(d[4], d[5], d[6], d[7]);
      }
    }
    umma::fence_before_sync();
    __syncthreads();  // staged; the accumulators are free again
    for (int e = tid; e < RB * W * (C / 4); e += 256) {
      const int c4 = (e % (C / 4)) * 4, xx = (e / (C / 4)) % W, j = e / ((C / 4) * W);
      const long long row = row0 + j;
      if (row >= rows) continue;
      float4 p = *reinterpret_cast<const float4*>(stage + (j * W + xx) * SP + c4);
      float4* o = reinterpret_cast<float4*>(out + ((size_t)row * W + xx) * C + c4);
      if (accumulate) {
        const float4 q = *o;
        p.x += q.x;
        p.y += q.y;
        p.z += q.z;
        p.w += q.w;
      }
      *o = p;
    }
    __syncthreads();  // the stage is read before the next round writes it
  }
  if (failed && tid == 0) atomicOr(err, 4u);
  __syncthreads();
  umma::fence_after_sync();
  if (warp == 0) umma::dealloc(tmem, cols);
}

// ---------------------------------------------------------------------------
// forward y-DFT (sign -1): per tile (b, QK = 128 / C consecutive kx),
//   X[b, j, kx, re/im, c] = sum_y A[b, y, kx, :, c] exp(-2 pi i ky(j) y / H)
// as D[(q, c), (j, re/im)] = sum_(y, re/im) A[(q, c), (y, re/im)] F[(j, re/im), (y, re/im)]
// (M = 128, N = 2 MY, K = 2 H).
template <int C>
__global__ void __launch_bounds__(256, 1) k_y2m_tc(const float* __restrict__ ain, float* __restrict__ out,
                                                 int B, int H, int MX, int MY, const float* __restrict__ cs,
                                                 unsigned int* err) {
  constexpr int QK = 128 / C, C2 = 2 * C;
  extern __shared__ __align__(16) unsigned char dsm[];
  const int N = 2 * MY, K = 2 * H;
  unsigned char* ah = dsm;               // [128][K]
  unsigned char* al = ah + 128 * K * 2;
  unsigned char* bh = al + 128 * K * 2;  // [N][K]
  unsigned char* bl = bh + N * K * 2;
  unsigned long long* mbar = reinterpret_cast<unsigned long long*>(bl + N * K * 2);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(mbar + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // F: row (j, re): (cos, sin) on (y, re), (y, im); row (j, im): (-sin, cos)
  for (int e = tid; e < N * (K / 4); e += 256) {
    const int n = e / (K / 4), y0 = (e % (K / 4)) * 2, j = n >> 1;
    const int ky = j < MY / 2 ? j : j - MY;
    float f[4];
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      const int t = (ky * (y0 + i)) & (H - 1);
      const float co = cs[2 * t], si = cs[2 * t + 1];
      f[2 * i] = (n & 1) ? -si : co;
      f[2 * i + 1] = (n & 1) ? co : si;
    }
    store4(bh, bl, n, 2 * y0, K, f[0], f[1], f[2], f[3]);
  }
  const uint32_t cols = tmem_cols(N);
  const uint32_t mb = umma::smem_addr(mbar);
  if (warp == 0) umma::alloc(umma::smem_addr(tslot), cols);
  if (tid == 0) umma::mbar_init(mb, 1);
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = *tslot;
  const uint32_t idesc = umma::idesc_bf16_f32(128, N);
  const uint32_t uah = umma::smem_addr(ah), ual = umma::smem_addr(al), ubh = umma::smem_addr(bh),
                 ubl = umma::smem_addr(bl);
  uint32_t parity = 0;
  bool failed = false;
  const int groups = MX / QK, tiles = B * groups;
  for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const int b = tile / groups, kx0 = (tile % groups) * QK;
    // A: element ((q, c), (y, re/im)); a work item is two y of one kx and 4 channels
    for (int e = tid; e < QK * (C / 4) * (H / 2); e += 256) {
      const int c4 = (e % (C / 4)) * 4, q = (e / (C / 4)) % QK, y0 = (e / ((C / 4) * QK)) * 2;
      const float* s0 = ain + (((size_t)b * H + y0) * MX + kx0 + q) * C2 + c4;
      const float* s1 = s0 + (size_t)MX * C2;
      const float4 r0 = *reinterpret_cast<const float4*>(s0), i0 = *reinterpret_cast<const float4*>(s0 + C);
      const float4 r1 = *reinterpret_cast<const float4*>(s1), i1 = *reinterpret_cast<const float4*>(s1 + C);
      const int m = q * C + c4;
      store4(ah, al, m + 0, 2 * y0, K, r0.x, i0.x, r1.x, i1.x);
      store4(ah, al, m + 1, 2 * y0, K, r0.y, i0.y, r1.y, i1.y);
      store4(ah, al, m + 2, 2 * y0, K, r0.z, i0.z, r1.z, i1.z);
      store4(ah, al, m + 3, 2 * y0, K, r0.w, i0.w, r1.w, i1.w);
    }
    umma::fence_proxy_async();
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    if (tid == 0) {
      mma3(tmem, uah, ual, ubh, ubl, K, idesc);
      umma::commit(mb);
    }
    const bool ok = umma::mbar_wait(mb, parity, kDftWait);
    if (__syncthreads_or(!ok)) {
      umma::mbar_wait(mb, parity, kDftWait);
      failed = true;
      break;
    }
    parity ^= 1u;
    umma::fence_after_sync();
    const int m = (warp & 3) * 32 + lane, q = m / C, c = m % C;
    const int n0 = (warp >> 2) * (N / 2);
    for (int nc = 0; nc < N / 2; nc += 8) {
      float d[8];
      umma::ld_8cols(tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)(n0 + nc), d);
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int n = n0 + nc + i, j = n >> 1;
        out[(((size_t)b * MY + j) * MX + kx0 + q) * C2 + (n & 1) * C + c] = d[i];
      }
    }
    umma::fence_before_sync();
    __syncthreads();
  }
  if (failed && tid == 0) atomicOr(err, 4u);
  __syncthreads();
  umma::fence_after_sync();
  if (warp == 0) umma::dealloc(tmem, cols);
}

// inverse y-DFT (sign +1): per tile (b, QK consecutive kx),
//   U[b, y, kx, re/im, c] = sum_j V[b, j, kx, :, c] exp(+2 pi i ky(j) y / H)
// as D[(q, c), (y, re/im)] = sum_(j, re/im) V[(q, c), (j, re/im)] G[(y, re/im), (j, re/im)]
// (M = 128, N = 2 H, K = 2 MY).
template <int C>
__global__ void __launch_bounds__(256, 1) k_m2y_tc(const float* __restrict__ vin, float* __restrict__ out,
                                                 int B, int H, int MX, int MY, const float* __restrict__ cs,
                                                 unsigned int* err) {
  constexpr int QK = 128 / C, C2 = 2 * C;
  extern __shared__ __align__(16) unsigned char dsm[];
  const int N = 2 * H, K = 2 * MY;
  unsigned char* ah = dsm;               // [128][K]
  unsigned char* al = ah + 128 * K * 2;
  unsigned char* bh = al + 128 * K * 2;  // [N][K]
  unsigned char* bl = bh + N * K * 2;
  unsigned long long* mbar = reinterpret_cast<unsigned long long*>(bl + N * K * 2);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(mbar + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // G: row (y, re): (cos, -sin) on (j, re), (j, im); row (y, im): (sin, cos)
  for (int e = tid; e < N * (K / 4); e += 256) {
    const int n = e / (K / 4), j0 = (e % (K / 4)) * 2, y = n >> 1;
    float g[4];
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      const int j = j0 + i, ky = j < MY / 2 ? j : j - MY;
      const int t = (ky * y) & (H - 1);
      const float co = cs[2 * t], si = cs[2 * t + 1];
      g[2 * i] = (n & 1) ? si : co;
      g[2 * i + 1] = (n & 1) ? co : -si;
    }
    store4(bh, bl, n, 2 * j0, K, g[0], g[1], g[2], g[3]);
  }
  const uint32_t cols = tmem_cols(N);
  const uint32_t mb = umma::smem_addr(mbar);
  if (warp == 0) umma::alloc(umma::smem_addr(tslot), cols);
  if (tid == 0) umma::mbar_init(mb, 1);
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = *tslot;
  const uint32_t idesc = umma::idesc_bf16_f32(128, N);
  const uint32_t uah = umma::smem_addr(ah), ual = umma::smem_addr(al), ubh = umma::smem_addr(bh),
                 ubl = umma::smem_addr(bl);
  uint32_t parity = 0;
  bool failed = false;
  const int groups = MX / QK, tiles = B * groups;
  for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const int b = tile / groups, kx0 = (tile % groups) * QK;
    for (int e = tid; e < QK * (C / 4) * MY / 2; e += 256) {
      const int c4 = (e % (C / 4)) * 4, q = (e / (C / 4)) % QK, j0 = (e / ((C / 4) * QK)) * 2;
      const float* s0 = vin + (((size_t)b * MY + j0) * MX + kx0 + q) * C2 + c4;
      const float* s1 = s0 + (size_t)MX * C2;
      const float4 r0 = *reinterpret_cast<const float4*>(s0), i0 = *reinterpret_cast<const float4*>(s0 + C);
      const float4 r1 = *reinterpret_cast<const float4*>(s1), i1 = *reinterpret_cast<const float4*>(s1 + C);
      const int m = q * C + c4;
      store4(ah, al, m + 0, 2 * j0, K, r0.x, i0.x, r1.x, i1.x);
      store4(ah, al, m + 1, 2 * j0, K, r0.y, i0.y, r1.y, i1.y);
      store4(ah, al, m + 2, 2 * j0, K, r0.z, i0.z, r1.z, i1.z);
      store4(ah, al, m + 3, 2 * j0, K, r0.w, i0.w, r1.w, i1.w);
    }
    umma::fence_proxy_async();
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    if (tid == 0) {
      mma3(tmem, uah, ual, ubh, ubl, K, idesc);
      umma::commit(mb);
    }
    const bool ok = umma::mbar_wait(mb, parity, kDftWait);
    if (__syncthreads_or(!ok)) {
      umma::mbar_wait(mb, parity, kDftWait);
      failed = true;
      break;
    }
    parity ^= 1u;
    umma::fence_after_sync();
    const int m = (warp & 3) * 32 + lane, q = m / C, c = m % C;
    const int n0 = (warp >> 2) * (N / 2);
    for (int nc = 0; nc < N / 2; nc += 8) {
      float d[8];
      umma::ld_8cols(tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)(n0 + nc), d);
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int n = n0 + nc + i, y = n >> 1;
        out[(((size_t)b * H + y) * MX + kx0 + q) * C2 + (n & 1) * C + c] = d[i];
      }
    }
    umma::fence_before_sync();
    __syncthreads();
  }
  if (failed && tid == 0) atomicOr(err, 4u);
  __syncthreads();
  umma::fence_after_sync();
  if (warp == 0) umma::dealloc(tmem, cols);
}

// ---------------------------------------------------------------------------
// Host launchers: false when the shape is not one these kernels take.
template <typename Kern>
static bool set_smem(Kern k, size_t bytes) {
  return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) == cudaSuccess;
}

bool x2m_tc_launch(const float* v, float* out, long long rows, int W, int C, int MX, const float* cs,
                   const float* scale, unsigned int* err, cudaStream_t s) {
  const int N = 2 * MX;
  if (rows < 1 || W < 16 || W > 256 || (W & (W - 1)) || N % 16 || N > 64) return false;
  const size_t smem = (size_t)(2 * 128 * W + 2 * N * W) * 2 + 16;
  const long long tiles = (rows + 128 / C - 1) / (128 / C);
  const int grid = (int)(tiles < 152 * 2 ? tiles : 152 * 2);
#define X2M(CC)                                                                           \
  if (C == CC) {                                                                          \
    if (!set_smem(k_x2m_tc<CC>, smem)) return false;                                      \
    k_x2m_tc<CC><<<grid, 256, smem, s>>>(v, out, rows, W, MX, cs, scale, err);            \
    return cudaGetLastError() == cudaSuccess;                                             \
  }
  X2M(16)
  X2M(32)
  X2M(64)
#undef X2M
  return false;
}

bool m2x_tc_launch(const float* a, float* out, long long rows, int W, int C, int MX, const float* cs,
                   const float* scale, int accumulate, unsigned int* err, cudaStream_t s) {
  const int K = 2 * MX;
  if (rows < 1 || W != 128 || K % 16 || K > 64) return false;
  // (padded so that the CTAs resident on an SM hold at most 512 TMEM columns:
  // tcgen05.alloc waits while they are taken)
  const size_t cols = tmem_cols(4 * C), need = (size_t)(2 * 128 * K + 2 * 4 * C * K) * 2 + (size_t)4 * 128 * (C + 4) * 4 + 16,
               floor_bytes = (size_t)228 * 1024 / (512 / cols + 1);
  const size_t smem = need > floor_bytes ? need : floor_bytes;
  const long long rounds = (rows + 3) / 4;
  const int grid = (int)(rounds < 152 * 2 ? rounds : 152 * 2);
#define M2X(CC)                                                                                \
  if (C == CC) {                                                                               \
    if (!set_smem(k_m2x_tc<CC>, smem)) return false;                                           \
    k_m2x_tc<CC><<<grid, 256, smem, s>>>(a, out, rows, MX, cs, scale, accumulate, err);        \
    return cudaGetLastError() == cudaSuccess;                                                  \
  }
  M2X(16)
  M2X(32)
  M2X(64)
#undef M2X
  return false;
}

}  // namespace tara

namespace tara {

bool y2m_tc_launch(const float* a, float* out, int B, int H, int C, int MX, int MY, const float* cs,
                   unsigned int* err, cudaStream_t s) {
  const int N = 2 * MY, K = 2 * H;
  if (B < 1 || C < 16 || C > 64 || MX % (128 / C) || H < 16 || H > 128 || (H & (H - 1)) || N % 16 || N > 256)
    return false;
  const size_t cols = N <= 32 ? 32 : N <= 64 ? 64 : N <= 128 ? 128 : 256;
  const size_t need = (size_t)(2 * 128 * K + 2 * N * K) * 2 + 16, floor_bytes = (size_t)228 * 1024 / (512 / cols + 1);
  const size_t smem = need > floor_bytes ? need : floor_bytes;
  if (smem > 227 * 1024) return false;
  const int tiles = B * (MX / (128 / C)), grid = tiles < 152 * 2 ? tiles : 152 * 2;
#define Y2M(CC)                                                                   \
  if (C == CC) {                                                                  \
    if (!set_smem(k_y2m_tc<CC>, smem)) return false;                              \
    k_y2m_tc<CC><<<grid, 256, smem, s>>>(a, out, B, H, MX, MY, cs, err);          \
    return cudaGetLastError() == cudaSuccess;                                     \
  }
  Y2M(16)
  Y2M(32)
  Y2M(64)
#undef Y2M
  return false;
}

bool m2y_tc_launch(const float* v, float* out, int B, int H, int C, int MX, int MY, const float* cs,
                   unsigned int* err, cudaStream_t s) {
  const int N = 2 * H, K = 2 * MY;
  if (B < 1 || C < 16 || C > 64 || MX % (128 / C) || H < 8 || N > 256 || (H & (H - 1)) || K % 16 || K > 128)
    return false;
  const size_t cols = N <= 32 ? 32 : N <= 64 ? 64 : N <= 128 ? 128 : 256;
  const size_t need = (size_t)(2 * 128 * K + 2 * N * K) * 2 + 16, floor_bytes = (size_t)228 * 1024 / (512 / cols + 1);
  const size_t smem = need > floor_bytes ? need : floor_bytes;
  if (smem > 227 * 1024) return false;
  const int tiles = B * (MX / (128 / C)), grid = tiles < 152 * 2 ? tiles : 152 * 2;
#define M2Y(CC)                                                                   \
  if (C == CC) {                                                                  \
    if (!set_smem(k_m2y_tc<CC>, smem)) return false;                              \
    k_m2y_tc<CC><<<grid, 256, smem, s>>>(v, out, B, H, MX, MY, cs, err);          \
    return cudaGetLastError() == cudaSuccess;                                     \
  }
  M2Y(16)
  M2Y(32)
  M2Y(64)
#undef M2Y
  return false;
}

}  // namespace tara
