// The closure network's projection head, fused on the 5th-generation tensor
// cores (BF16 modes, C = 32 channels, P = 128 hidden units, co <= 4 outputs):
//
//   k_head_fwd_tc   per 128-row tile: zh = v Q1 (tcgen05, accumulator in TMEM),
//                   h = GELU(zh + q1), y = h Q2 + q2 (CUDA cores).  Only y is
//                   written: the 128-wide zh and h (256 MB each at batch 32) are
//                   recomputed in the backward pass instead of stored.
//   k_head_bwd_tc   per 128-row tile: zh = v Q1 again, then with g = dy Q2^T:
//                   dh = g GELU'(zh + q1); dv = dh Q1^T (tcgen05); and the weight
//                   gradients as products over the tile's rows accumulated in
//                   tensor memory across the CTA's tiles --
//                   dQ1^T (+)= dh^T [v | 1] (the ones column gives dq1) and
//                   dQ2^T (+)= h^T dy; each CTA leaves its partial sums in `part`
//                   for a fixed-order reduction.
//
// Operands are BF16 in shared memory (no-swizzle K-major layout, umma.cuh), as
// the mma.sync kernels of the layer-by-layer path round them; the transposed
// operands (dh^T, h^T, v^T, dy^T) are written element by element from the
// thread that owns the row.  Every mbarrier wait is bounded (value 4 in *err,
// a second bounded wait for the MMAs in flight, the columns freed).
#include <cstdint>

#include <cuda_bf16.h>

#include "internal.h"
#include "umma.cuh"

namespace tara {

namespace {

constexpr int kHC = 32, kHP = 128, kHT = 256;  // channels, hidden units, threads
constexpr uint32_t kHeadWait = 1u << 20;

__device__ __forceinline__ float gelu_h(float x) { return 0.5f * x * (1.f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ uint32_t hoff(int r, int k, int K) {
  return (uint32_t)(((r >> 3) * (K >> 3) + (k >> 3)) * 128 + (r & 7) * 16 + (k & 7) * 2);
}
__device__ __forceinline__ void st_bf16(unsigned char* base, uint32_t off, float v) {
  *reinterpret_cast<__nv_bfloat16*>(base + off) = __float2bfloat16_rn(v);
}
__device__ __forceinline__ uint32_t pack2(float a, float b) {
  const __nv_bfloat162 t = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<const uint32_t*>(&t);
}
__device__ __forceinline__ void issue(uint32_t tmem_d, uint32_t a, uint32_t b, int K, uint32_t idesc, bool acc) {
  const uint32_t sbo = (uint32_t)(K / 8) * 128;
  for (int s = 0; s < K / 16; ++s)
    umma::mma_bf16(tmem_d, umma::smem_desc(a + 2 * s * 128, 128, sbo), umma::smem_desc(b + 2 * s * 128, 128, sbo),
                   idesc, (acc || s > 0) ? 1u : 0u);
}

// v tile (128 rows x 32 channels, FP32) -> BF16 rows (r, c) of `a1`; rows at or
// past `rows` are zeros.  With `bt`, also the transposed copy (c, r), K = 128.
__device__ __forceinline__ void stage_v(const float* __restrict__ v, long long r0, long long rows,
                                        unsigned char* a1, unsigned char* bt) {
  for (int e = threadIdx.x; e < 128 * kHC / 4; e += kHT) {
    const int r = e / (kHC / 4), c4 = (e % (kHC / 4)) * 4;
    const float4 q = r0 + r < rows ? *reinterpret_cast<const float4*>(v + (r0 + r) * kHC + c4)
                                   : make_float4(0.f, 0.f, 0.f, 0.f);
    *reinterpret_cast<uint2*>(a1 + hoff(r, c4, kHC)) = make_uint2(pack2(q.x, q.y), pack2(q.z, q.w));
    if (bt) {
      st_bf16(bt, hoff(c4 + 0, r, 128), q.x);
      st_bf16(bt, hoff(c4 + 1, r, 128), q.y);
      st_bf16(bt, hoff(c4 + 2, r, 128), q.z);
      st_bf16(bt, hoff(c4 + 3, r, 128), q.w);
    }
  }
}

}  // namespace

// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kHT, 1) k_head_fwd_tc(const float* __restrict__ v, long long rows,
                                                      const float* __restrict__ Q1, const float* __restrict__ q1,
                                                      const float* __restrict__ Q2, const float* __restrict__ q2,
                                                      int CO, float* __restrict__ y, unsigned int* err) {
  extern __shared__ __align__(16) unsigned char hsm[];
  unsigned char* a1 = hsm;                    // [128][32] v
  unsigned char* bq = a1 + 128 * kHC * 2;     // [128 p][32 c] Q1
  float* q1s = reinterpret_cast<float*>(bq + kHP * kHC * 2);
  float* q2w = q1s + kHP;                     // Q2 [p][4]
  float* yp = q2w + kHP * 4;                  // [2][128][4] partial y of the two p halves
  unsigned long long* mbar = reinterpret_cast<unsigned long long*>(yp + 2 * 128 * 4);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(mbar + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (int e = tid; e < kHC * kHP; e += kHT) {  // Q1(k = c, n = p) = Q1[c P + p] as row p
    const int c = e / kHP, p = e % kHP;
    st_bf16(bq, hoff(p, c, kHC), Q1[e]);
  }
  for (int e = tid; e < kHP; e += kHT) q1s[e] = q1[e];
  for (int e = tid; e < kHP * 4; e += kHT) q2w[e] = (e & 3) < CO ? Q2[(e >> 2) * CO + (e & 3)] : 0.f;
  const uint32_t mb = umma::smem_addr(mbar);
  if (warp == 0) umma::alloc(umma::smem_addr(tslot), kHP);
  if (tid == 0) umma::mbar_init(mb, 1);
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = *tslot;
  const uint32_t idesc = umma::idesc_bf16_f32(128, kHP);
  uint32_t parity = 0;
  bool failed = false;
  const long long tiles = (rows + 127) / 128;
  for (long long tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const long long r0 = tile * 128;
    stage_v(v, r0, rows, a1, nullptr);
    umma::fence_proxy_async();
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    if (tid == 0) {
      issue(tmem, umma::smem_addr(a1), umma::smem_addr(bq), kHC, idesc, false);
      umma::commit(mb);
    }
    const bool ok = umma::mbar_wait(mb, parity, kHeadWait);
    if (__syncthreads_or(!ok)) {
      umma::mbar_wait(mb, parity, kHeadWait);
      failed = true;
      break;
    }
    parity ^= 1u;
    umma::fence_after_sync();
    // thread: row r (its TMEM lane) and half of the hidden units
    const int r = (warp & 3) * 32 + lane, p0 = (warp >> 2) * (kHP / 2);
    float ys[4] = {0.f, 0.f, 0.f, 0.f};
    for (int pc = 0; pc < kHP / 2; pc += 16) {
      float z[16];
      umma::ld_16cols(tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)(p0 + pc), z);
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        const int p = p0 + pc + i;
        const float h = gelu_h(z[i] + q1s[p]);
#pragma unroll
        for (int o = 0; o < 4; ++o) ys[o] = fmaf(h, q2w[p * 4 + o], ys[o]);
      }
    }
#pragma unroll
    for (int o = 0; o < 4; ++o) yp[((warp >> 2) * 128 + r) * 4 + o] = ys[o];
    umma::fence_before_sync();
    __syncthreads();
    for (int e = tid; e < 128 * CO; e += kHT) {
      const int rr = e / CO, o = e % CO;
      if (r0 + rr < rows) y[(r0 + rr) * CO + o] = yp[rr * 4 + o] + yp[(128 + rr) * 4 + o] + q2[o];
    }
  }
  if (failed && tid == 0) atomicOr(err, 4u);
  __syncthreads();
  umma::fence_after_sync();
  if (warp == 0) umma::dealloc(tmem, kHP);
}

// ---------------------------------------------------------------------------
// Tensor-memory columns of the backward kernel: zh [0, 128), dv [128, 160),
// dQ1^T with the dq1 column [160, 208), dQ2^T [208, 224).
constexpr int kColDv = 128, kColQ1 = 160, kColQ2 = 208, kNQ1 = 48, kNQ2 = 16;

__global__ void __launch_bounds__(kHT, 1) k_head_bwd_tc(const float* __restrict__ v, const float* __restrict__ dy,
                                                      long long rows, const float* __restrict__ Q1,
                                                      const float* __restrict__ q1, const float* __restrict__ Q2,
                                                      int CO, float* __restrict__ dv, float* __restrict__ part,
                                                      unsigned int* err) {
  extern __shared__ __align__(16) unsigned char hsm[];
  unsigned char* a1 = hsm;                     // [128 r][32 c] v
  unsigned char* bq1 = a1 + 128 * kHC * 2;     // [128 p][32 c] Q1
  unsigned char* bq2 = bq1 + kHP * kHC * 2;    // [32 c][128 p] Q1 (for dh Q1^T)
  unsigned char* a2 = bq2 + kHC * kHP * 2;     // [128 r][128 p] dh
  unsigned char* a3 = a2 + 128 * kHP * 2;      // [128 p][128 r] dh^T
  unsigned char* a4 = a3 + kHP * 128 * 2;      // [128 p][128 r] h^T
  unsigned char* b3 = a4 + kHP * 128 * 2;      // [48][128 r] v^T, a row of ones, zeros
  unsigned char* b4 = b3 + kNQ1 * 128 * 2;     // [16][128 r] dy^T, zeros
  float* q1s = reinterpret_cast<float*>(b4 + kNQ2 * 128 * 2);
  float* q2w = q1s + kHP;                      // Q2 [p][4]
  float* dys = q2w + kHP * 4;                  // [128 r][4] this tile's dy
  unsigned long long* mbar = reinterpret_cast<unsigned long long*>(dys + 128 * 4);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(mbar + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (int e = tid; e < kHC * kHP; e += kHT) {
    const int c = e / kHP, p = e % kHP;
    st_bf16(bq1, hoff(p, c, kHC), Q1[e]);
    st_bf16(bq2, hoff(c, p, kHP), Q1[e]);
  }
  for (int e = tid; e < (kNQ1 - kHC) * 128; e += kHT)  // the ones row (n = 32) and zero rows
    st_bf16(b3, hoff(kHC + e / 128, e % 128, 128), e < 128 ? 1.f : 0.f);
  for (int e = tid; e < kNQ2 * 128; e += kHT) st_bf16(b4, hoff(e / 128, e % 128, 128), 0.f);
  for (int e = tid; e < kHP; e += kHT) q1s[e] = q1[e];
  for (int e = tid; e < kHP * 4; e += kHT) q2w[e] = (e & 3) < CO ? Q2[(e >> 2) * CO + (e & 3)] : 0.f;
  const uint32_t mb = umma::smem_addr(mbar);
  if (warp == 0) umma::alloc(umma::smem_addr(tslot), 256);
  if (tid == 0) umma::mbar_init(mb, 1);
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = *tslot;
  uint32_t parity = 0;
  bool failed = false, first = true;
  const long long tiles = (rows + 127) / 128;
  const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;
  for (long long tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const long long r0 = tile * 128;
    stage_v(v, r0, rows, a1, b3);
    for (int e = tid; e < 128 * 4; e += kHT) {
      const int r = e >> 2, o = e & 3;
      const float d = (o < CO && r0 + r < rows) ? dy[(r0 + r) * CO + o] : 0.f;
      dys[e] = d;
      if (o < CO) st_bf16(b4, hoff(o, r, 128), d);
    }
    umma::fence_proxy_async();
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    if (tid == 0) {  // zh = v Q1
      issue(tmem, umma::smem_addr(a1), umma::smem_addr(bq1), kHC, umma::idesc_bf16_f32(128, kHP), false);
      umma::commit(mb);
    }
    bool ok = umma::mbar_wait(mb, parity, kHeadWait);
    if (__syncthreads_or(!ok)) {
      umma::mbar_wait(mb, parity, kHeadWait);
      failed = true;
      break;
    }
    parity ^= 1u;
    umma::fence_after_sync();
    {  // dh = (dy Q2^T) GELU'(zh + q1) and h = GELU(zh + q1) for row r, half of p
      const int r = (warp & 3) * 32 + lane, p0 = (warp >> 2) * (kHP / 2);
      float dyr[4];
#pragma unroll
      for (int o = 0; o < 4; ++o) dyr[o] = dys[r * 4 + o];
      for (int pc = 0; pc < kHP / 2; pc += 16) {
        float z[16], dh[16];
        umma::ld_16cols(tmem + lane_base + (uint32_t)(p0 + pc), z);
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          const int p = p0 + pc + i;
          const float zz = z[i] + q1s[p];
          float g = 0.f;
#pragma unroll
          for (int o = 0; o < 4; ++o) g = fmaf(dyr[o], q2w[p * 4 + o], g);
          // GELU and its derivative share one erf
          const float t = erff(zz * 0.70710678118654752f);
          dh[i] = g * (0.5f * (1.f + t) + zz * 0.39894228040143268f * expf(-0.5f * zz * zz));
          st_bf16(a3, hoff(p, r, 128), dh[i]);
          st_bf16(a4, hoff(p, r, 128), 0.5f * zz * (1.f + t));
        }
        *reinterpret_cast<uint4*>(a2 + hoff(r, p0 + pc, kHP)) =
            make_uint4(pack2(dh[0], dh[1]), pack2(dh[2], dh[3]), pack2(dh[4], dh[5]), pack2(dh[6], dh[7]));
        *reinterpret_cast<uint4*>(a2 + hoff(r, p0 + pc + 8, kHP)) =
            make_uint4(pack2(dh[8], dh[9]), pack2(dh[10], dh[11]), pack2(dh[12], dh[13]), pack2(dh[14], dh[15]));
      }
    }
    umma::fence_proxy_async();
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    if (tid == 0) {
      // dv = dh Q1^T (K = 128 hidden units)
      issue(tmem + kColDv, umma::smem_addr(a2), umma::smem_addr(bq2), kHP, umma::idesc_bf16_f32(128, kHC), false);
      // dQ1^T (+)= dh^T [v | 1] and dQ2^T (+)= h^T dy over the tile's 128 rows
      issue(tmem + kColQ1, umma::smem_addr(a3), umma::smem_addr(b3), 128, umma::idesc_bf16_f32(128, kNQ1), !first);
      issue(tmem + kColQ2, umma::smem_addr(a4), umma::smem_addr(b4), 128, umma::idesc_bf16_f32(128, kNQ2), !first);
      umma::commit(mb);
    }
    first = false;
    ok = umma::mbar_wait(mb, parity, kHeadWait);
    if (__syncthreads_or(!ok)) {
      umma::mbar_wait(mb, parity, kHeadWait);
      failed = true;
      break;
    }
    parity ^= 1u;
    umma::fence_after_sync();
    {  // dv row r, half of the channels
      const int r = (warp & 3) * 32 + lane, c0 = (warp >> 2) * (kHC / 2);
      float d[16];
      umma::ld_16cols(tmem + lane_base + (uint32_t)(kColDv + c0), d);
      if (r0 + r < rows) {
        float4* o = reinterpret_cast<float4*>(dv + (r0 + r) * kHC + c0);
#pragma unroll
        for (int i = 0; i < 4; ++i) o[i] = make_float4(d[4 * i], d[4 * i + 1], d[4 * i + 2], d[4 * i + 3]);
      }
    }
    umma::fence_before_sync();
    __syncthreads();
  }
  // this CTA's partial weight gradients: lane p of the accumulators
  const size_t nq1 = (size_t)kHC * kHP;
  const size_t nparts = gridDim.x;
  float* pq1 = part + (size_t)blockIdx.x * nq1;                            // dQ1 [c][p]
  float* pb1 = part + nparts * nq1 + (size_t)blockIdx.x * kHP;             // dq1 [p]
  float* pq2 = part + nparts * (nq1 + kHP) + (size_t)blockIdx.x * kHP * CO;  // dQ2 [p][o]
  if (!failed && warp < 4) {
    const int p = warp * 32 + lane;
    float d[16];
    for (int c0 = 0; c0 < kNQ1; c0 += 16) {
      if (!first) umma::ld_16cols(tmem + lane_base + (uint32_t)(kColQ1 + c0), d);
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        const int c = c0 + i;
        const float val = first ? 0.f : d[i];
        if (c < kHC)
          pq1[(size_t)c * kHP + p] = val;
        else if (c == kHC)
          pb1[p] = val;
      }
    }
    if (!first) umma::ld_16cols(tmem + lane_base + (uint32_t)kColQ2, d);
    for (int o = 0; o < CO; ++o) pq2[(size_t)p * CO + o] = first ? 0.f : d[o];
  }
  if (failed && tid == 0) atomicOr(err, 4u);
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  if (warp == 0) umma::dealloc(tmem, 256);
}

// ---------------------------------------------------------------------------
bool head_tc_supported(int C, int P, int CO) { return C == kHC && P == kHP && CO >= 1 && CO <= 4; }

static size_t fwd_smem() { return (size_t)128 * kHC * 2 + kHP * kHC * 2 + (kHP + kHP * 4 + 2 * 128 * 4) * 4 + 16; }
static size_t bwd_smem() {
  return (size_t)128 * kHC * 2 + 2 * kHP * kHC * 2 + 3 * 128 * kHP * 2 + (kNQ1 + kNQ2) * 128 * 2 +
         (kHP + kHP * 4 + 128 * 4) * 4 + 16;
}

bool head_fwd_tc_launch(const float* v, long long rows, const float* Q1, const float* q1, const float* Q2,
                        const float* q2, int CO, float* y, unsigned int* err, cudaStream_t s) {
  if (rows < 1) return false;
  // (padded to 57 KB: at most 4 CTAs, 4 x 128 TMEM columns, per SM)
  const size_t smem = fwd_smem() > 57 * 1024 ? fwd_smem() : 57 * 1024;
  static const cudaError_t attr =
      cudaFuncSetAttribute(k_head_fwd_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(57 * 1024));
  if (attr != cudaSuccess || smem > 57 * 1024) return false;
  const long long tiles = (rows + 127) / 128;
  const int grid = (int)(tiles < 152 * 4 ? tiles : 152 * 4);
  k_head_fwd_tc<<<grid, kHT, smem, s>>>(v, rows, Q1, q1, Q2, q2, CO, y, err);
  return cudaGetLastError() == cudaSuccess;
}

// Grid of the backward kernel (one CTA per SM: 256 TMEM columns, ~140 KB of
// shared memory); `part` must hold grid * (C P + P + P co) floats.
int head_bwd_tc_grid(long long rows) {
  const long long tiles = (rows + 127) / 128;
  return (int)(tiles < 152 ? tiles : 152);
}

bool head_bwd_tc_launch(const float* v, const float* dy, long long rows, const float* Q1, const float* q1,
                        const float* Q2, int CO, float* dv, float* part, unsigned int* err, cudaStream_t s) {
  if (rows < 1) return false;
  static const cudaError_t attr =
      cudaFuncSetAttribute(k_head_bwd_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bwd_smem());
  if (attr != cudaSuccess) return false;
  k_head_bwd_tc<<<head_bwd_tc_grid(rows), kHT, bwd_smem(), s>>>(v, dy, rows, Q1, q1, Q2, CO, dv, part, err);
  return cudaGetLastError() == cudaSuccess;
}

}  // namespace tara
