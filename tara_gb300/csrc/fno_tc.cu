// Tall-skinny channel-mixing GEMMs of the closure network on the 5th-generation
// tensor cores (the TARA_FNO_BF16_TMEM mode): C[r, n] (+)= sum_k A[r, k] B(k, n)
// (+ bias[n]), r over the B*H*W grid points, K x N the small weight matrix
// (32 x 32 for the pointwise layers, 32 x 128 for the projection, 128 x 32 for
// the projection's input gradient).
//
// Per 128-row tile: the CTA's 128 threads load the rows (FP32), round them to
// BF16 and store them in the K-major canonical layout (umma.cuh); one thread
// issues K/16 tcgen05.mma (M = 128, N, K = 16) into an FP32 accumulator in
// tensor memory and commits to an mbarrier; after the wait each warp reads its
// 32 rows back with tcgen05.ld (one row per thread, 32 columns per load) and
// applies the epilogue -- bias, accumulation into C, the GELU or copy second
// output -- exactly as the mma.sync kernel of the BF16 mode does.  The weight
// matrix is staged once per CTA; the CTAs loop over tiles.
//
// Every wait is bounded: a wait that gives up sets bit 2 (value 4) of *err, the
// CTA stops taking tiles, and the host reports TARA_ERR_TIMEOUT.
#include <cstdint>

#include <cuda_bf16.h>

#include "internal.h"
#include "umma.cuh"

namespace tara {

namespace {
__device__ __forceinline__ float gelu_tc(float x) { return 0.5f * x * (1.f + erff(x * 0.70710678118654752f)); }

constexpr int kTcRows = 128;        // rows per tile = the MMA's M
constexpr uint32_t kTcWait = 1u << 20;  // polls before a wait gives up (far above any tile's time)
}  // namespace

template <int K, int N>
__global__ void __launch_bounds__(128) k_ts_gemm_tc(const float* __restrict__ A, long long M,
                                                    const float* __restrict__ Bw, int transB,
                                                    const float* __restrict__ bias, float* C, int accumulate,
                                                    float* act, int act_mode, unsigned int* err) {
  static_assert(K % 16 == 0 && N % 32 == 0 && N <= 256, "MMA shape");
  constexpr uint32_t kCols = N;  // TMEM columns: a power of two >= 32 (32 or 128 here)
  __shared__ __align__(128) __nv_bfloat16 As[kTcRows * K];
  __shared__ __align__(128) __nv_bfloat16 Bs[N * K];
  __shared__ __align__(8) unsigned long long mbar;
  __shared__ uint32_t tmem_slot;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // weights as the N x K operand (row n holds B(:, n)), K-major
  for (int e = tid; e < K * N; e += 128) {
    const int k = transB ? e % K : e / N, n = transB ? e / K : e % N;
    *reinterpret_cast<__nv_bfloat16*>(reinterpret_cast<char*>(Bs) + umma::elem_offset<K>(n, k)) =
        __float2bfloat16_rn(Bw[e]);
  }
  const uint32_t mb = umma::smem_addr(&mbar);
  if (warp == 0) umma::alloc(umma::smem_addr(&tmem_slot), kCols);
  if (tid == 0) umma::mbar_init(mb, 1);
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = tmem_slot;
  const uint32_t idesc = umma::idesc_bf16_f32(kTcRows, N);
  const uint32_t a0 = umma::smem_addr(As), b0 = umma::smem_addr(Bs);
  constexpr uint32_t kSbo = (K / 8) * 128;  // 8-row groups
  uint32_t parity = 0;
  int failed = 0;
  const long long tiles = (M + kTcRows - 1) / kTcRows;
  for (long long tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const long long r0 = tile * kTcRows;
    for (int e = tid; e < kTcRows * K / 4; e += 128) {
      const int r = e / (K / 4), k4 = (e % (K / 4)) * 4;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (r0 + r < M) v = *reinterpret_cast<const float4*>(A + (r0 + r) * K + k4);
      __nv_bfloat162* d = reinterpret_cast<__nv_bfloat162*>(reinterpret_cast<char*>(As) +
                                                            umma::elem_offset<K>(r, k4));
      d[0] = __floats2bfloat162_rn(v.x, v.y);
      d[1] = __floats2bfloat162_rn(v.z, v.w);
    }
    umma::fence_proxy_async();  // the rows just stored are read by the tensor cores
    __syncthreads();
    if (tid == 0) {
      umma::fence_after_sync();
#pragma unroll
      for (int s = 0; s < K / 16; ++s)  // K = 16 per MMA: two core matrices along K
        umma::mma_bf16(tmem, umma::smem_desc(a0 + 2 * s * 128, 128, kSbo),
                       umma::smem_desc(b0 + 2 * s * 128, 128, kSbo), idesc, s > 0);
      umma::commit(mb);
    }
    const bool ok = umma::mbar_wait(mb, parity, kTcWait);
    if (__syncthreads_or(!ok)) {
      // give the MMAs in flight a second bounded wait before the TMEM is freed
      umma::mbar_wait(mb, parity, kTcWait);
      failed = 1;
      break;
    }
    parity ^= 1u;
    umma::fence_after_sync();
    const long long r = r0 + warp * 32 + lane;  // this thread's row (TMEM lane)
#pragma unroll
    for (int c0 = 0; c0 < N; c0 += 32) {
      float v[32];
      umma::ld_32cols(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
      if (r < M) {
#pragma unroll
        for (int q = 0; q < 32; q += 4) {
          float4 o = make_float4(v[q], v[q + 1], v[q + 2], v[q + 3]);
          if (bias) {
            o.x += bias[c0 + q];
            o.y += bias[c0 + q + 1];
            o.z += bias[c0 + q + 2];
            o.w += bias[c0 + q + 3];
          }
          float4* pc = reinterpret_cast<float4*>(C + r * N + c0 + q);
          if (accumulate) {
            const float4 p = *pc;
            o.x += p.x;
            o.y += p.y;
            o.z += p.z;
            o.w += p.w;
          }
          *pc = o;
          if (act)
            *reinterpret_cast<float4*>(act + r * N + c0 + q) =
                act_mode == 1 ? make_float4(gelu_tc(o.x), gelu_tc(o.y), gelu_tc(o.z), gelu_tc(o.w)) : o;
        }
      }
    }
    umma::fence_before_sync();
    __syncthreads();  // TMEM read and As consumed before the next tile's MMA and loads
  }
  if (failed && tid == 0) atomicOr(err, 4u);
  __syncthreads();
  umma::fence_after_sync();
  if (warp == 0) umma::dealloc(tmem, kCols);
}

// Static shared memory of k_ts_gemm_tc<K, N>: both operands in BF16, the mbarrier
// and the TMEM address slot.
constexpr size_t tc_static_smem(int K, int N) { return (size_t)(kTcRows + N) * K * 2 + 16; }

// Host launcher: true when (K, N) is one of the shapes above.
bool ts_gemm_tc_launch(const float* A, long long M, int K, int N, const float* Bw, int transB, const float* bias,
                       float* C, int accumulate, float* act, int act_mode, unsigned int* err, cudaStream_t s) {
  const long long tiles = (M + kTcRows - 1) / kTcRows;
  if (tiles < 1) return true;
  const int grid = (int)(tiles < 152 * 4 ? tiles : 152 * 4);
  // tcgen05.alloc waits while the SM's 512 TMEM columns are taken, so the
  // CTAs resident on one SM must not ask for more than 512 together: 16 CTAs
  // (the thread limit) x 32 columns fit; for 128 columns the shared memory of
  // a CTA is padded to 50 KB, which leaves room for at most 4 of them.
#define TC_CASE(KK, NN)                                                                                    \
  if (K == KK && N == NN) {                                                                                \
    const int pad = NN > 32 ? 50 * 1024 - (int)tc_static_smem(KK, NN) : 0;                               \
    if (pad > 0) cudaFuncSetAttribute(k_ts_gemm_tc<KK, NN>, cudaFuncAttributeMaxDynamicSharedMemorySize, pad); \
    k_ts_gemm_tc<KK, NN><<<grid, 128, pad > 0 ? pad : 0, s>>>(A, M, Bw, transB, bias, C, accumulate, act,  \
                                                               act_mode, err);                             \
    return true;                                                                                           \
  }
  TC_CASE(32, 32)
  TC_CASE(32, 128)
  TC_CASE(128, 32)
#undef TC_CASE
  return false;
}

}  // namespace tara
