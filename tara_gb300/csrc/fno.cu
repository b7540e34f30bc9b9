// Fourier neural operator (FNO) subgrid closure: forward, backward and Adam on
// the GPU with the project's own kernels.
//
// Network (per sample, grid H x W, activations NHWC in FP32):
//   v0 = x * Pw + Pb                                     lifting, CI -> C channels
//   for l = 1..L:  z_l = S_l(v_{l-1}) + v_{l-1} W_l + b_l,  v_l = GELU(z_l) (l < L), v_L = z_L
//   h = GELU(v_L Q1 + q1),  y = h Q2 + q2                projection C -> P -> CO
// S_l is the spectral convolution on the retained modes kx in [0, MX),
// ky in [0, MY/2) U [-MY/2, 0): forward truncated DFT along x then y, a complex
// C x C matrix per mode, inverse along y then x (irfft restricted to the modes,
// weight 2 on kx >= 1, divided by H*W).
//
// Tensor cores: the channel mixing -- the pointwise W_l, the projection Q1 and
// the per-mode complex mixing (as a 2C x 2C real block matrix) in forward and
// backward, and the weight gradients -- runs through gemm_bf16: operands
// rounded to BF16 in shared memory, mma.sync.m16n8k16 with FP32 accumulators.
// In mode TARA_FNO_BF16_TMEM the tall-skinny GEMMs run on the 5th-generation
// tensor cores instead (fno_tc.cu: tcgen05.mma, accumulators in tensor memory).
// The same GEMM has an FP32 CUDA-core path (mode TARA_FNO_FP32) used to check
// gradients against the FP64 oracle.  The truncated DFTs (16 and 32 modes of a
// 128-point axis) run on FP32 CUDA cores, and so does the per-mode mixing of
// batches of at most four samples (a GEMV per mode), with BF16-rounded operands.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include <cuda_bf16.h>

#include "fno_fused.h"
#include "internal.h"

namespace tara {

// fno_dft_tc.cu: the truncated DFTs on tcgen05 (split-BF16 operands).
bool x2m_tc_launch(const float* v, float* out, long long rows, int W, int C, int MX, const float* cs,
                   const float* scale, unsigned int* err, cudaStream_t s);
bool m2x_tc_launch(const float* a, float* out, long long rows, int W, int C, int MX, const float* cs,
                   const float* scale, int accumulate, unsigned int* err, cudaStream_t s);
bool y2m_tc_launch(const float* a, float* out, int B, int H, int C, int MX, int MY, const float* cs,
                   unsigned int* err, cudaStream_t s);
bool m2y_tc_launch(const float* v, float* out, int B, int H, int C, int MX, int MY, const float* cs,
                   unsigned int* err, cudaStream_t s);
// fno_head_tc.cu: the projection head fused on tcgen05 (forward without stored
// hidden activations; backward recomputing them, with the weight gradients).
bool head_tc_supported(int C, int P, int CO);
bool head_fwd_tc_launch(const float* v, long long rows, const float* Q1, const float* q1, const float* Q2,
                        const float* q2, int CO, float* y, unsigned int* err, cudaStream_t s);
int head_bwd_tc_grid(long long rows);
bool head_bwd_tc_launch(const float* v, const float* dy, long long rows, const float* Q1, const float* q1,
                        const float* Q2, int CO, float* dv, float* part, unsigned int* err, cudaStream_t s);
// fno_tc.cu: the tall-skinny GEMMs on tcgen05 with TMEM accumulators.
bool ts_gemm_tc_launch(const float* A, long long M, int K, int N, const float* Bw, int transB, const float* bias,
                       float* C, int accumulate, float* act, int act_mode, unsigned int* err, cudaStream_t s);

// ---------------------------------------------------------------------------
// strided batched GEMM:  C[b](m,n) = alpha * sum_k A[b](m,k) B[b](k,n)
//                                    (+ C[b](m,n) if accumulate) (+ bias[n])
// Element addresses: A + b*sab + m*sam + k*sak, likewise B and C.
// ---------------------------------------------------------------------------
struct GemmArgs {
  int M, N, K, batch;
  const float* A;
  long long sab, sam, sak;
  const float* B;
  long long sbb, sbk, sbn;
  float* C;
  long long scb, scm, scn;
  float alpha;
  int accumulate;
  const float* bias;
  float* act;    // optional second output at C's offsets: act_mode 1 GELU(c), 2 c
  int act_mode;
};

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x) {
  return 0.5f * (1.f + erff(x * 0.70710678118654752f)) + x * 0.39894228040143268f * expf(-0.5f * x * x);
}

__device__ __forceinline__ void gemm_store(const GemmArgs& g, float* C, int m, int n, float acc) {
  float v = g.alpha * acc;
  if (g.bias) v += g.bias[n];
  float* p = C + m * g.scm + n * g.scn;
  if (g.accumulate) v += *p;
  *p = v;
  if (g.act) g.act[m * g.scm + n * g.scn] = g.act_mode == 1 ? gelu(v) : v;
}

constexpr int GT_M = 64, GT_N = 64, GT_K = 32;

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  const __nv_bfloat16 l = __float2bfloat16_rn(lo), h = __float2bfloat16_rn(hi);
  return (uint32_t)__bfloat16_as_ushort(l) | ((uint32_t)__bfloat16_as_ushort(h) << 16);
}

// 128 threads = 4 warps in a 2 x 2 arrangement; each warp owns a 32 x 32 block
// of the 64 x 64 tile as 2 x 4 mma tiles of 16 x 8.  Operands are staged in
// shared memory as FP32 (any stride pattern in global memory) and rounded to
// BF16 when the fragments are formed.
__global__ void __launch_bounds__(128) k_gemm_bf16(GemmArgs g) {
  __shared__ float As[GT_M][GT_K + 1];
  __shared__ float Bs[GT_K][GT_N + 1];
  const int b = blockIdx.z;
  const int m0 = blockIdx.y * GT_M, n0 = blockIdx.x * GT_N;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
  const int gid = lane >> 2, tig = lane & 3;
  const float* A = g.A + b * g.sab;
  const float* Bm = g.B + b * g.sbb;
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int r = 0; r < 4; ++r) acc[i][j][r] = 0.f;
  for (int k0 = 0; k0 < g.K; k0 += GT_K) {
    for (int e = tid; e < GT_M * GT_K; e += 128) {
      const int mm = e / GT_K, kk = e % GT_K, m = m0 + mm, k = k0 + kk;
      As[mm][kk] = (m < g.M && k < g.K) ? A[m * g.sam + k * g.sak] : 0.f;
    }
    for (int e = tid; e < GT_K * GT_N; e += 128) {
      const int kk = e / GT_N, nn = e % GT_N, k = k0 + kk, n = n0 + nn;
      Bs[kk][nn] = (k < g.K && n < g.N) ? Bm[k * g.sbk + n * g.sbn] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int ks = 0; ks < GT_K; ks += 16) {
      uint32_t af[2][4], bf[4][2];
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const int r = wm + 16 * i + gid, c = ks + 2 * tig;
        af[i][0] = pack_bf16(As[r][c], As[r][c + 1]);
        af[i][1] = pack_bf16(As[r + 8][c], As[r + 8][c + 1]);
        af[i][2] = pack_bf16(As[r][c + 8], As[r][c + 9]);
        af[i][3] = pack_bf16(As[r + 8][c + 8], As[r + 8][c + 9]);
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int n = wn + 8 * j + gid, k = ks + 2 * tig;
        bf[j][0] = pack_bf16(Bs[k][n], Bs[k + 1][n]);
        bf[j][1] = pack_bf16(Bs[k + 8][n], Bs[k + 9][n]);
      }
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
          asm volatile(
              "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
              "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
              : "+f"(acc[i][j][0]), "+f"(acc[i][j][1]), "+f"(acc[i][j][2]), "+f"(acc[i][j][3])
              : "r"(af[i][0]), "r"(af[i][1]), "r"(af[i][2]), "r"(af[i][3]), "r"(bf[j][0]),
                "r"(bf[j][1]));
    }
    __syncthreads();
  }
  float* C = g.C + b * g.scb;
  if (g.act) g.act += b * g.scb;
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const int m = m0 + wm + 16 * i + gid + (r >= 2 ? 8 : 0);
        const int n = n0 + wn + 8 * j + 2 * tig + (r & 1);
        if (m < g.M && n < g.N) gemm_store(g, C, m, n, acc[i][j][r]);
      }
}

// FP32 CUDA-core path with the same tiling (verification mode).
__global__ void __launch_bounds__(256) k_gemm_fp32(GemmArgs g) {
  __shared__ float As[GT_M][GT_K + 1];
  __shared__ float Bs[GT_K][GT_N + 1];
  const int b = blockIdx.z;
  const int m0 = blockIdx.y * GT_M, n0 = blockIdx.x * GT_N;
  const int tid = threadIdx.x, tm = (tid / 16) * 4, tn = (tid % 16) * 4;
  const float* A = g.A + b * g.sab;
  const float* Bm = g.B + b * g.sbb;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < g.K; k0 += GT_K) {
    for (int e = tid; e < GT_M * GT_K; e += 256) {
      const int mm = e / GT_K, kk = e % GT_K, m = m0 + mm, k = k0 + kk;
      As[mm][kk] = (m < g.M && k < g.K) ? A[m * g.sam + k * g.sak] : 0.f;
    }
    for (int e = tid; e < GT_K * GT_N; e += 256) {
      const int kk = e / GT_N, nn = e % GT_N, k = k0 + kk, n = n0 + nn;
      Bs[kk][nn] = (k < g.K && n < g.N) ? Bm[k * g.sbk + n * g.sbn] : 0.f;
    }
    __syncthreads();
    for (int kk = 0; kk < GT_K; ++kk)
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(As[tm + i][kk], Bs[kk][tn + j], acc[i][j]);
    __syncthreads();
  }
  float* C = g.C + b * g.scb;
  if (g.act) g.act += b * g.scb;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      const int m = m0 + tm + i, n = n0 + tn + j;
      if (m < g.M && n < g.N) gemm_store(g, C, m, n, acc[i][j]);
    }
}

// ---------------------------------------------------------------------------
// Tall-skinny tensor-core GEMMs of the channel mixing (BF16 mode): the rows are
// the B*H*W grid points and stream through; the small weight matrix (K, N in
// {32, 128}) stays in shared memory as BF16.  Operand tiles are loaded with
// float4 reads, rounded to BF16 in shared memory (rows padded by 8 BF16 so the
// fragment loads are conflict-free), multiplied with mma.sync.m16n8k16 into
// FP32 accumulators.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void mma_bf16_16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
      "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t lds32(const __nv_bfloat16* p) { return *reinterpret_cast<const uint32_t*>(p); }

constexpr int kTsRows = 128;  // rows per tile: 8 warps x 16

// C[r, n] (+)= sum_k A[r, k] B(k, n) (+ bias[n]) for r < M; B(k, n) = Bw[k*N + n],
// or Bw[n*K + k] with transB.  act: a second output at C's offsets
// (act_mode 1: GELU, 2: copy).  Persistent CTAs loop over 128-row tiles.
template <int K, int N>
__global__ void __launch_bounds__(256) k_ts_gemm(const float* __restrict__ A, long long M,
                                                 const float* __restrict__ Bw, int transB,
                                                 const float* __restrict__ bias, float* C, int accumulate,
                                                 float* act, int act_mode) {
  constexpr int KP = K + 8, NT = N / 8;
  __shared__ __align__(16) __nv_bfloat16 Bs[N * KP];
  __shared__ __align__(16) __nv_bfloat16 As[kTsRows * KP];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, gid = lane >> 2, tig = lane & 3;
  for (int e = tid; e < K * N; e += 256) {
    const int k = transB ? e % K : e / N, n = transB ? e / K : e % N;
    Bs[n * KP + k] = __float2bfloat16_rn(Bw[e]);
  }
  const long long tiles = (M + kTsRows - 1) / kTsRows;
  const int ra = warp * 16 + gid;
  for (long long tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const long long r0 = tile * kTsRows;
    __syncthreads();  // Bs written / previous tile's As consumed
    for (int e = tid; e < kTsRows * K / 4; e += 256) {
      const int r = e / (K / 4), k4 = (e % (K / 4)) * 4;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (r0 + r < M) v = *reinterpret_cast<const float4*>(A + (r0 + r) * K + k4);
      *reinterpret_cast<__nv_bfloat162*>(&As[r * KP + k4]) = __floats2bfloat162_rn(v.x, v.y);
      *reinterpret_cast<__nv_bfloat162*>(&As[r * KP + k4 + 2]) = __floats2bfloat162_rn(v.z, v.w);
    }
    __syncthreads();
    float acc[NT][4];
#pragma unroll
    for (int nt = 0; nt < NT; ++nt)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[nt][q] = 0.f;
#pragma unroll
    for (int ks = 0; ks < K; ks += 16) {
      uint32_t a[4];
      a[0] = lds32(&As[ra * KP + ks + 2 * tig]);
      a[1] = lds32(&As[(ra + 8) * KP + ks + 2 * tig]);
      a[2] = lds32(&As[ra * KP + ks + 2 * tig + 8]);
      a[3] = lds32(&As[(ra + 8) * KP + ks + 2 * tig + 8]);
#pragma unroll
      for (int nt = 0; nt < NT; ++nt) {
        const __nv_bfloat16* b = &Bs[(nt * 8 + gid) * KP + ks + 2 * tig];
        mma_bf16_16816(acc[nt], a, lds32(b), lds32(b + 8));
      }
    }
#pragma unroll
    for (int nt = 0; nt < NT; ++nt)
#pragma unroll
      for (int hh = 0; hh < 2; ++hh) {
        const long long r = r0 + ra + 8 * hh;
        if (r >= M) continue;
        const int n = nt * 8 + 2 * tig;
        float2 v = make_float2(acc[nt][2 * hh], acc[nt][2 * hh + 1]);
        if (bias) {
          v.x += bias[n];
          v.y += bias[n + 1];
        }
        float2* pc = reinterpret_cast<float2*>(C + r * N + n);
        if (accumulate) {
          const float2 o = *pc;
          v.x += o.x;
          v.y += o.y;
        }
        *pc = v;
        if (act)
          *reinterpret_cast<float2*>(act + r * N + n) =
              act_mode == 1 ? make_float2(gelu(v.x), gelu(v.y)) : v;
      }
  }
}

// Weight gradient dW(k, n) = sum_r A[r, k] B[r, n] over the rows of this CTA's
// chunk, as a partial sum into part[blockIdx.x] (K x N), and with bias_part the
// FP32 column sums of B (the bias gradient) into bias_part[blockIdx.x] (N).
// Sub-tiles of 64 rows are staged transposed (rows contiguous) so that the row
// index is the MMA reduction dimension.
template <int K, int N>
__global__ void __launch_bounds__(256) k_ts_wgrad(const float* __restrict__ A, const float* __restrict__ B,
                                                  long long M, long long rows_per_cta, float* __restrict__ part,
                                                  float* __restrict__ bias_part) {
  constexpr int RT = 64, RP = RT + 8;
  constexpr int TM = K / 16, TN = N / 8, TPW = TM * TN / 8;  // output tiles per warp
  static_assert(TM * TN % 8 == 0 && 256 % (N / 4) == 0, "tile split");
  __shared__ __align__(16) __nv_bfloat16 At[K * RP];
  __shared__ __align__(16) __nv_bfloat16 Bt[N * RP];
  __shared__ float bsum[N];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, gid = lane >> 2, tig = lane & 3;
  const long long rb = (long long)blockIdx.x * rows_per_cta;
  const long long re = rb + rows_per_cta < M ? rb + rows_per_cta : M;
  float acc[TPW][4];
#pragma unroll
  for (int t = 0; t < TPW; ++t)
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[t][q] = 0.f;
  float bs[4] = {0.f, 0.f, 0.f, 0.f};  // this thread's column sums (fixed columns)
  for (int e = tid; e < N; e += 256) bsum[e] = 0.f;
  for (long long r0 = rb; r0 < re; r0 += RT) {
    __syncthreads();
    for (int e = tid; e < RT * K / 4; e += 256) {
      const int r = e / (K / 4), k4 = (e % (K / 4)) * 4;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (r0 + r < re) v = *reinterpret_cast<const float4*>(A + (r0 + r) * K + k4);
      At[(k4 + 0) * RP + r] = __float2bfloat16_rn(v.x);
      At[(k4 + 1) * RP + r] = __float2bfloat16_rn(v.y);
      At[(k4 + 2) * RP + r] = __float2bfloat16_rn(v.z);
      At[(k4 + 3) * RP + r] = __float2bfloat16_rn(v.w);
    }
    for (int e = tid; e < RT * N / 4; e += 256) {
      const int r = e / (N / 4), n4 = (e % (N / 4)) * 4;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (r0 + r < re) v = *reinterpret_cast<const float4*>(B + (r0 + r) * N + n4);
      bs[0] += v.x;
      bs[1] += v.y;
      bs[2] += v.z;
      bs[3] += v.w;
      Bt[(n4 + 0) * RP + r] = __float2bfloat16_rn(v.x);
      Bt[(n4 + 1) * RP + r] = __float2bfloat16_rn(v.y);
      Bt[(n4 + 2) * RP + r] = __float2bfloat16_rn(v.z);
      Bt[(n4 + 3) * RP + r] = __float2bfloat16_rn(v.w);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < RT; kk += 16) {
#pragma unroll
      for (int t = 0; t < TPW; ++t) {
        const int tile = warp * TPW + t, tm = tile / TN, tn = tile % TN;
        uint32_t a[4];
        const int ma = tm * 16 + gid;
        a[0] = lds32(&At[ma * RP + kk + 2 * tig]);
        a[1] = lds32(&At[(ma + 8) * RP + kk + 2 * tig]);
        a[2] = lds32(&At[ma * RP + kk + 2 * tig + 8]);
        a[3] = lds32(&At[(ma + 8) * RP + kk + 2 * tig + 8]);
        const __nv_bfloat16* b = &Bt[(tn * 8 + gid) * RP + kk + 2 * tig];
        mma_bf16_16816(acc[t], a, lds32(b), lds32(b + 8));
      }
    }
  }
  float* out = part + (size_t)blockIdx.x * K * N;
#pragma unroll
  for (int t = 0; t < TPW; ++t) {
    const int tile = warp * TPW + t, tm = tile / TN, tn = tile % TN;
    const int m = tm * 16 + gid, n = tn * 8 + 2 * tig;
    out[m * N + n] = acc[t][0];
    out[m * N + n + 1] = acc[t][1];
    out[(m + 8) * N + n] = acc[t][2];
    out[(m + 8) * N + n + 1] = acc[t][3];
  }
  if (bias_part) {
    __syncthreads();
    const int n4 = (tid % (N / 4)) * 4;
#pragma unroll
    for (int q = 0; q < 4; ++q) atomicAdd(&bsum[n4 + q], bs[q]);
    __syncthreads();
    for (int e = tid; e < N; e += 256) bias_part[(size_t)blockIdx.x * N + e] = bsum[e];
  }
}

// Weight gradient for a small side (K*N <= 1024 outputs, e.g. the 128 x 2 output
// projection or the ci x 32 lifting), CUDA cores: thread t owns outputs
// t, t + 256, ... of the K x N matrix; per-CTA partial sums into part.
__global__ void __launch_bounds__(256) k_wgrad_small(const float* __restrict__ A, int K, const float* __restrict__ B,
                                                     int N, long long M, long long rows_per_cta,
                                                     float* __restrict__ part) {
  const long long rb = (long long)blockIdx.x * rows_per_cta;
  const long long re = rb + rows_per_cta < M ? rb + rows_per_cta : M;
  for (int o = threadIdx.x; o < K * N; o += blockDim.x) {
    const int k = o / N, n = o % N;
    float s = 0.f;
#pragma unroll 8
    for (long long r = rb; r < re; ++r) s = fmaf(A[r * K + k], B[r * N + n], s);
    part[(size_t)blockIdx.x * K * N + o] = s;
  }
}

// dh = GELU'(zh) * (dy Q2^T), the output projection's and the head GELU's
// backward.  Launch with blockDim.x = P (<= 256): thread p keeps its row of Q2
// (co <= 4) in registers; rows are strided over the grid.
__global__ void k_head_back(const float* __restrict__ dy, const float* __restrict__ Q2,
                            const float* __restrict__ zh, float* __restrict__ dh, long long rows, int P, int CO) {
  const int p = threadIdx.x;
  float q[4];
  for (int o = 0; o < 4; ++o) q[o] = o < CO ? Q2[p * CO + o] : 0.f;
  for (long long r = blockIdx.x; r < rows; r += gridDim.x) {
    float s = 0.f;
    for (int o = 0; o < CO; ++o) s = fmaf(dy[r * CO + o], q[o], s);
    const long long t = r * P + p;
    dh[t] = s * gelu_grad(zh[t]);
  }
}

// Per-mode mixing for small batches (a GEMV per mode: tensor-core tiles would be
// all padding): Y[b, m, :] = X[b, m, :] Rb[m] for b < B <= kMixB, one CTA per
// mode, thread o owns output column o.  With bf16 != 0 both operands are
// rounded to BF16 first, as the tensor-core path does; sums in FP32.
constexpr int kMixB = 4;
__global__ void __launch_bounds__(128) k_mode_mix(const float* __restrict__ X, const float* __restrict__ Rb,
                                                  float* __restrict__ Y, int B, int C2, long long sbm,
                                                  int bf16) {
  __shared__ float sx[kMixB * 128];
  const int m = blockIdx.x;
  for (int e = threadIdx.x; e < B * C2; e += blockDim.x) {
    const float v = X[(e / C2) * sbm + (size_t)m * C2 + e % C2];
    sx[e] = bf16 ? __bfloat162float(__float2bfloat16_rn(v)) : v;
  }
  __syncthreads();
  const float* R = Rb + (size_t)m * C2 * C2;
  for (int o = threadIdx.x; o < C2; o += blockDim.x) {
    float acc[kMixB] = {0.f, 0.f, 0.f, 0.f};
    for (int k = 0; k < C2; ++k) {
      float r = R[(size_t)k * C2 + o];
      if (bf16) r = __bfloat162float(__float2bfloat16_rn(r));
#pragma unroll
      for (int b = 0; b < kMixB; ++b)
        if (b < B) acc[b] = fmaf(sx[b * C2 + k], r, acc[b]);
    }
#pragma unroll
    for (int b = 0; b < kMixB; ++b)
      if (b < B) Y[b * sbm + (size_t)m * C2 + o] = acc[b];
  }
}

// sum over `parts` partial results of length n (split-K reduction)
// Launch with blockDim (32, 8): threadIdx.y splits the parts, a fixed-order tree
// in shared memory combines them (deterministic).
__global__ void __launch_bounds__(256) k_sum_parts(const float* __restrict__ part, int parts, int n,
                                                   float* __restrict__ out, int accumulate) {
  __shared__ float sh[8][33];
  for (int i0 = blockIdx.x * 32; i0 < n; i0 += gridDim.x * 32) {
    const int i = i0 + threadIdx.x;
    float s = 0.f;
    if (i < n)
      for (int p = threadIdx.y; p < parts; p += 8) s += part[(size_t)p * n + i];
    sh[threadIdx.y][threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.y == 0 && i < n) {
      float t = 0.f;
      for (int y = 0; y < 8; ++y) t += sh[y][threadIdx.x];
      out[i] = accumulate ? out[i] + t : t;
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// truncated DFTs on NHWC activations.  H and W are powers of two, so the phase
// index k*n mod N is a mask; cs[2t], cs[2t+1] = cos, sin(2 pi t / N) are staged
// in shared memory.  The y kernels split the channels over blockIdx.y (CPB
// channels per CTA) so that a batch of one sample still fills the SMs.
// ---------------------------------------------------------------------------
constexpr int kCpb = 8;

// x_to_modes: A[b,y,kx,r,c] = s_kx * sum_x v[b,y,x,c] * (cos, -sin)(2 pi kx x / W).
// One CTA per row (b, y); a thread owns one kx and four channels, so each
// step of the x sum is one 16-byte activation load, one twiddle load and
// eight FMAs.  C is a multiple of 4 (8 in practice).
__global__ void __launch_bounds__(256) k_x_to_modes(const float* __restrict__ v, float* __restrict__ a,
                                                    int W, int C, int MX, const float* __restrict__ cs,
                                                    const float* __restrict__ scale) {
  extern __shared__ __align__(16) float sm[];
  float* sv = sm;          // [W][C]
  float* tw = sm + W * C;  // [W][2]
  const int row = blockIdx.x;  // b*H + y
  const float4* src = reinterpret_cast<const float4*>(v + (size_t)row * W * C);
  for (int e = threadIdx.x; e < W * C / 4; e += blockDim.x) reinterpret_cast<float4*>(sv)[e] = src[e];
  for (int e = threadIdx.x; e < 2 * W; e += blockDim.x) tw[e] = cs[e];
  __syncthreads();
  float* dst = a + (size_t)row * MX * 2 * C;
  const int mask = W - 1, C4 = C / 4;
  for (int e = threadIdx.x; e < MX * C4; e += blockDim.x) {
    const int kx = e / C4, c = (e % C4) * 4;
    float4 re = make_float4(0.f, 0.f, 0.f, 0.f), im = re;
    int t = 0;
    for (int x = 0; x < W; ++x) {
      const float4 val = *reinterpret_cast<const float4*>(&sv[x * C + c]);
      const float2 w = *reinterpret_cast<const float2*>(&tw[2 * t]);
      re.x = fmaf(val.x, w.x, re.x);
      re.y = fmaf(val.y, w.x, re.y);
      re.z = fmaf(val.z, w.x, re.z);
      re.w = fmaf(val.w, w.x, re.w);
      im.x = fmaf(-val.x, w.y, im.x);
      im.y = fmaf(-val.y, w.y, im.y);
      im.z = fmaf(-val.z, w.y, im.z);
      im.w = fmaf(-val.w, w.y, im.w);
      t = (t + kx) & mask;
    }
    const float s = scale ? scale[kx] : 1.f;
    *reinterpret_cast<float4*>(&dst[(kx * 2 + 0) * C + c]) = make_float4(s * re.x, s * re.y, s * re.z, s * re.w);
    *reinterpret_cast<float4*>(&dst[(kx * 2 + 1) * C + c]) = make_float4(s * im.x, s * im.y, s * im.z, s * im.w);
  }
}

// modes_to_x: out[b,y,x,c] (+)= sum_kx s_kx * (Ar cos - Ai sin)(2 pi kx x / W);
// a thread owns one x and four channels.
__global__ void __launch_bounds__(256) k_modes_to_x(const float* __restrict__ a, float* __restrict__ out,
                                                    int W, int C, int MX, const float* __restrict__ cs,
                                                    const float* __restrict__ scale, int accumulate) {
  extern __shared__ __align__(16) float sm[];
  float* sa = sm;               // [MX][2][C], pre-scaled by s_kx
  float* tw = sm + MX * 2 * C;  // [W][2]
  const int row = blockIdx.x;
  const float* src = a + (size_t)row * MX * 2 * C;
  for (int e = threadIdx.x; e < MX * 2 * C; e += blockDim.x)
    sa[e] = scale ? src[e] * scale[e / (2 * C)] : src[e];
  for (int e = threadIdx.x; e < 2 * W; e += blockDim.x) tw[e] = cs[e];
  __syncthreads();
  float* dst = out + (size_t)row * W * C;
  const int mask = W - 1, C4 = C / 4;
  for (int e = threadIdx.x; e < W * C4; e += blockDim.x) {
    const int x = e / C4, c = (e % C4) * 4;
    float4 s4 = make_float4(0.f, 0.f, 0.f, 0.f);
    int t = 0;
    for (int kx = 0; kx < MX; ++kx) {
      const float4 ar = *reinterpret_cast<const float4*>(&sa[(kx * 2) * C + c]);
      const float4 ai = *reinterpret_cast<const float4*>(&sa[(kx * 2 + 1) * C + c]);
      const float2 w = *reinterpret_cast<const float2*>(&tw[2 * t]);
      s4.x = fmaf(ar.x, w.x, fmaf(-ai.x, w.y, s4.x));
      s4.y = fmaf(ar.y, w.x, fmaf(-ai.y, w.y, s4.y));
      s4.z = fmaf(ar.z, w.x, fmaf(-ai.z, w.y, s4.z));
      s4.w = fmaf(ar.w, w.x, fmaf(-ai.w, w.y, s4.w));
      t = (t + x) & mask;
    }
    float4* pd = reinterpret_cast<float4*>(&dst[x * C + c]);
    if (accumulate) {
      const float4 o = *pd;
      s4.x += o.x;
      s4.y += o.y;
      s4.z += o.z;
      s4.w += o.w;
    }
    *pd = s4;
  }
}

// y_to_modes: V[b,j,kx,:,c] = sum_y A[b,y,kx,:,c] * exp(sign*2 pi i ky(j) y / H),
// ky(j) = j for j < MY/2, j - MY above.  CTA (b*MX + kx, channel group).
__global__ void __launch_bounds__(256) k_y_to_modes(const float* __restrict__ a, float* __restrict__ out,
                                                    int H, int C, int MX, int MY,
                                                    const float* __restrict__ cs, float sign) {
  extern __shared__ float sm[];
  float* sa = sm;               // [H][2][kCpb]
  float* tw = sm + H * 2 * kCpb;  // [H][2]
  const int b = blockIdx.x / MX, kx = blockIdx.x % MX, c0 = blockIdx.y * kCpb;
  for (int e = threadIdx.x; e < H * 2 * kCpb; e += blockDim.x) {
    const int y = e / (2 * kCpb), r = (e / kCpb) & 1, cc = e % kCpb;
    sa[e] = a[(((size_t)b * H + y) * MX + kx) * 2 * C + r * C + c0 + cc];
  }
  for (int e = threadIdx.x; e < 2 * H; e += blockDim.x) tw[e] = cs[e];
  __syncthreads();
  const int mask = H - 1;
  for (int e = threadIdx.x; e < MY * kCpb; e += blockDim.x) {
    const int j = e / kCpb, cc = e % kCpb;
    const int ky = j < MY / 2 ? j : j - MY;
    const int step = ky & mask;
    float re = 0.f, im = 0.f;
    int t = 0;
    for (int y = 0; y < H; ++y) {
      const float co = tw[2 * t], si = sign * tw[2 * t + 1];
      const float ar = sa[(y * 2) * kCpb + cc], ai = sa[(y * 2 + 1) * kCpb + cc];
      re = fmaf(ar, co, fmaf(-ai, si, re));
      im = fmaf(ar, si, fmaf(ai, co, im));
      t = (t + step) & mask;
    }
    float* o = out + (((size_t)b * MY + j) * MX + kx) * 2 * C;
    o[c0 + cc] = re;
    o[C + c0 + cc] = im;
  }
}

// modes_to_y: U[b,y,kx,:,c] = sum_j V[b,j,kx,:,c] * exp(sign*2 pi i ky(j) y / H)
__global__ void __launch_bounds__(256) k_modes_to_y(const float* __restrict__ v, float* __restrict__ out,
                                                    int H, int C, int MX, int MY,
                                                    const float* __restrict__ cs, float sign) {
  extern __shared__ float sm[];
  float* sv = sm;                  // [MY][2][kCpb]
  float* tw = sm + MY * 2 * kCpb;  // [H][2]
  const int b = blockIdx.x / MX, kx = blockIdx.x % MX, c0 = blockIdx.y * kCpb;
  for (int e = threadIdx.x; e < MY * 2 * kCpb; e += blockDim.x) {
    const int j = e / (2 * kCpb), r = (e / kCpb) & 1, cc = e % kCpb;
    sv[e] = v[(((size_t)b * MY + j) * MX + kx) * 2 * C + r * C + c0 + cc];
  }
  for (int e = threadIdx.x; e < 2 * H; e += blockDim.x) tw[e] = cs[e];
  __syncthreads();
  const int mask = H - 1;
  for (int e = threadIdx.x; e < H * kCpb; e += blockDim.x) {
    const int y = e / kCpb, cc = e % kCpb;
    float re = 0.f, im = 0.f;
    for (int j = 0; j < MY; ++j) {
      const int ky = j < MY / 2 ? j : j - MY;
      const int t = (ky * y) & mask;
      const float co = tw[2 * t], si = sign * tw[2 * t + 1];
      const float vr = sv[(j * 2) * kCpb + cc], vi = sv[(j * 2 + 1) * kCpb + cc];
      re = fmaf(vr, co, fmaf(-vi, si, re));
      im = fmaf(vr, si, fmaf(vi, co, im));
    }
    float* o = out + (((size_t)b * H + y) * MX + kx) * 2 * C;
    o[c0 + cc] = re;
    o[C + c0 + cc] = im;
  }
}

// Block matrix of the complex mixing per mode: Rbig[m][(ri,c)][(ro,o)] from
// R[m][c][o][2]: [[Rr, Ri], [-Ri, Rr]].
__global__ void k_expand_r(const float* __restrict__ R, float* __restrict__ Rb, int modes, int C) {
  const size_t total = (size_t)modes * C * C;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const int m = (int)(t / (C * C)), c = (int)((t / C) % C), o = (int)(t % C);
    const float rr = R[2 * t], ri = R[2 * t + 1];
    float* B = Rb + (size_t)m * 4 * C * C;
    const int n2 = 2 * C;
    B[c * n2 + o] = rr;
    B[c * n2 + C + o] = ri;
    B[(C + c) * n2 + o] = -ri;
    B[(C + c) * n2 + C + o] = rr;
  }
}

// Fold the gradient of the block matrix back to the complex weights.
__global__ void k_fold_r(const float* __restrict__ dRb, float* __restrict__ dR, int modes, int C) {
  const size_t total = (size_t)modes * C * C;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const int m = (int)(t / (C * C)), c = (int)((t / C) % C), o = (int)(t % C);
    const float* B = dRb + (size_t)m * 4 * C * C;
    const int n2 = 2 * C;
    dR[2 * t] = B[c * n2 + o] + B[(C + c) * n2 + C + o];
    dR[2 * t + 1] = B[c * n2 + C + o] - B[(C + c) * n2 + o];
  }
}

__global__ void k_gelu(const float* __restrict__ z, float* __restrict__ v, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    v[i] = gelu(z[i]);
}

// dz may be dv (in place), so neither is declared __restrict__
__global__ void k_gelu_back(const float* __restrict__ z, const float* dv, float* dz, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    dz[i] = dv[i] * gelu_grad(z[i]);
}

// column sums of an (M x N) row-major matrix (N <= 256) into per-block partial
// sums part[block][N] (bias gradients): each CTA covers 256/N rows per pass
__global__ void __launch_bounds__(256) k_colsum_part(const float* __restrict__ x, long long M, int N,
                                                     float* __restrict__ part) {
  __shared__ float sh[256];
  const int rpi = 256 / N, t = threadIdx.x;
  const int n = t % N, r0 = t / N;
  float s = 0.f;
  if (r0 < rpi)
    for (long long m = (long long)blockIdx.x * rpi + r0; m < M; m += (long long)gridDim.x * rpi)
      s += x[m * N + n];
  sh[t] = s;
  __syncthreads();
  if (t < N) {
    float a = 0.f;
    for (int i = 0; i < rpi; ++i) a += sh[i * N + t];
    part[(size_t)blockIdx.x * N + t] = a;
  }
}

// lifting with CI input channels
// v = x Pw + Pb; thread (row slot, channel): blockDim.x = C (<= 64), rows
// strided over blockDim.y and the grid.
__global__ void k_lift(const float* __restrict__ x, const float* __restrict__ Pw,
                       const float* __restrict__ Pb, float* __restrict__ v, long long rows, int CI, int C) {
  const int c = threadIdx.x;
  float w[8];
  for (int i = 0; i < CI && i < 8; ++i) w[i] = Pw[i * C + c];
  const float b = Pb[c];
  for (long long r = (long long)blockIdx.x * blockDim.y + threadIdx.y; r < rows;
       r += (long long)gridDim.x * blockDim.y) {
    float s = b;
    for (int i = 0; i < CI; ++i) s = fmaf(x[r * CI + i], i < 8 ? w[i] : Pw[i * C + c], s);
    v[r * C + c] = s;
  }
}

// out = h Q2 + q2 (N = CO is tiny: CUDA cores)
__global__ void k_proj_out(const float* __restrict__ h, const float* __restrict__ Q2,
                           const float* __restrict__ q2, float* __restrict__ y, long long rows, int P, int CO) {
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < rows * CO;
       t += (long long)gridDim.x * blockDim.x) {
    const long long r = t / CO;
    const int o = (int)(t % CO);
    float s = q2[o];
    for (int p = 0; p < P; ++p) s = fmaf(h[r * P + p], Q2[p * CO + o], s);
    y[t] = s;
  }
}

// out = h Q2 + q2 with one warp per row (co <= 4): lanes split the p sum
__global__ void __launch_bounds__(256) k_proj_out_warp(const float* __restrict__ h, const float* __restrict__ Q2,
                                                       const float* __restrict__ q2, float* __restrict__ y,
                                                       long long rows, int P, int CO) {
  const int lane = threadIdx.x & 31;
  const long long w0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long r = w0; r < rows; r += nw) {
    float s[4] = {0.f, 0.f, 0.f, 0.f};
    for (int p = lane; p < P; p += 32) {
      const float hv = h[r * P + p];
#pragma unroll
      for (int o = 0; o < 4; ++o)
        if (o < CO) s[o] = fmaf(hv, Q2[p * CO + o], s[o]);
    }
#pragma unroll
    for (int o = 0; o < 4; ++o)
      for (int d = 16; d > 0; d >>= 1) s[o] += __shfl_xor_sync(0xffffffffu, s[o], d);
    if (lane < CO) {
      float v = s[0];
#pragma unroll
      for (int o = 1; o < 4; ++o)
        if (lane == o) v = s[o];
      y[r * CO + lane] = v + q2[lane];
    }
  }
}

// dh = dy Q2^T
__global__ void k_proj_out_back(const float* __restrict__ dy, const float* __restrict__ Q2,
                                float* __restrict__ dh, long long rows, int P, int CO) {
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < rows * P;
       t += (long long)gridDim.x * blockDim.x) {
    const long long r = t / P;
    const int p = (int)(t % P);
    float s = 0.f;
    for (int o = 0; o < CO; ++o) s = fmaf(dy[r * CO + o], Q2[p * CO + o], s);
    dh[t] = s;
  }
}

// loss = mean((y - t)^2) partial sums; dy = 2 (y - t) / n
__global__ void k_mse(const float* __restrict__ y, const float* __restrict__ t, float* __restrict__ dy,
                      size_t n, double* __restrict__ part) {
  double s = 0.0;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float d = y[i] - t[i];
    s += (double)d * d;
    dy[i] = 2.f * d / (float)n;
  }
  __shared__ double sh[8];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) a += sh[w];
    part[blockIdx.x] = a;
  }
}

__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, size_t n, float lr, float b1, float b2, float eps,
                       float c1, float c2) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

// dst[b] = src[idx[b]] for samples of n floats (idx NULL: dst[b] = src[b]); an
// index outside [0, nsrc) yields zeros and sets *bad
__global__ void k_gather(const float* __restrict__ src, const int* __restrict__ idx, int nsrc, int B,
                         size_t n, float* __restrict__ dst, unsigned int* __restrict__ bad) {
  const size_t total = (size_t)B * n;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const size_t b = t / n, e = t % n;
    const int sb = idx ? idx[b] : (int)b;
    if (sb < 0 || sb >= nsrc) {
      dst[t] = 0.f;
      if (e == 0) atomicOr(bad, 1u);
    } else {
      dst[t] = src[(size_t)sb * n + e];
    }
  }
}

}  // namespace tara

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
using namespace tara;

struct tara_fno {
  tara_fno_config cfg;
  int dev = 0;
  cudaStream_t stream = nullptr;      // where the work is launched
  cudaStream_t own_stream = nullptr;  // the handle's own stream
  int bmax = 0;
  // parameters, gradients, Adam moments (FP32, same layout)
  size_t np = 0;
  float *p = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;
  size_t off_Pw, off_Pb, off_Q1, off_q1, off_Q2, off_q2;
  std::vector<size_t> off_R, off_W, off_b;
  long long step = 0;
  bool rb_valid = false;   // Rb holds the block matrices of the current parameters
  unsigned long long pver = 0;  // bumped whenever the parameters change
  // tables
  float *csx = nullptr, *csy = nullptr, *wx = nullptr;  // twiddles and the irfft weights 2/(HW)
  // activations for backward
  float *x = nullptr, *tgt = nullptr, *vact = nullptr, *zact = nullptr, *X = nullptr, *zh = nullptr, *h = nullptr,
        *y = nullptr, *dy = nullptr;
  // work
  float *A = nullptr, *Y = nullptr, *U = nullptr, *S = nullptr, *Rb = nullptr, *dRb = nullptr,
        *dv = nullptr, *dz = nullptr, *dh = nullptr, *part = nullptr;
  size_t part_n = 0;
  double* lpart = nullptr;
  unsigned int* bad = nullptr;
  unsigned int* errw = nullptr;  // where tensor-core waits that gave up are flagged (value 4): bad, or a
                                 // word of the caller the handle is bound to (the closure's solver flag)
  bool fused = true;             // inference forward of small batches through fno_fused.cu
};

namespace {

constexpr int kPw = 152 * 4, kTh = 256;

// BF16 operands on the tensor cores (either form of the tall-skinny GEMMs).
bool bf16_mode(const tara_fno* f) { return f->cfg.mode == TARA_FNO_BF16 || f->cfg.mode == TARA_FNO_BF16_TMEM; }

// The truncated DFTs along x over `rows` grid rows: on the tensor cores in the
// BF16 modes where the shape allows (fno_dft_tc.cu), else on FP32 CUDA cores.
int x_to_modes(tara_fno* f, const float* v, float* out, int rows, const float* scale) {
  const auto& c = f->cfg;
  if (bf16_mode(f) && x2m_tc_launch(v, out, rows, c.w, c.c, c.mx, f->csx, scale, f->errw, f->stream))
    return TARA_OK;
  const size_t sx = (size_t)(c.w * c.c + 2 * c.w) * sizeof(float);
  k_x_to_modes<<<rows, 256, sx, f->stream>>>(v, out, c.w, c.c, c.mx, f->csx, scale);
  TARA_CK(cudaGetLastError());
  return TARA_OK;
}
int modes_to_x(tara_fno* f, const float* a, float* out, int rows, const float* scale, int accumulate) {
  const auto& c = f->cfg;
  if (bf16_mode(f) && m2x_tc_launch(a, out, rows, c.w, c.c, c.mx, f->csx, scale, accumulate, f->errw, f->stream))
    return TARA_OK;
  const size_t smx = (size_t)(c.mx * 2 * c.c + 2 * c.w) * sizeof(float);
  k_modes_to_x<<<rows, 256, smx, f->stream>>>(a, out, c.w, c.c, c.mx, f->csx, scale, accumulate);
  TARA_CK(cudaGetLastError());
  return TARA_OK;
}

// The truncated DFTs along y (forward: sign -1 into the modes; inverse: +1 back
// to the rows), likewise.
int y_to_modes(tara_fno* f, const float* a, float* out, int B) {
  const auto& c = f->cfg;
  if (bf16_mode(f) && y2m_tc_launch(a, out, B, c.h, c.c, c.mx, c.my, f->csy, f->errw, f->stream)) return TARA_OK;
  const dim3 gy(B * c.mx, c.c / kCpb);
  const size_t sy = (size_t)(c.h * 2 * kCpb + 2 * c.h) * sizeof(float);
  k_y_to_modes<<<gy, 256, sy, f->stream>>>(a, out, c.h, c.c, c.mx, c.my, f->csy, -1.f);
  TARA_CK(cudaGetLastError());
  return TARA_OK;
}
int modes_to_y(tara_fno* f, const float* v, float* out, int B) {
  const auto& c = f->cfg;
  if (bf16_mode(f) && m2y_tc_launch(v, out, B, c.h, c.c, c.mx, c.my, f->csy, f->errw, f->stream)) return TARA_OK;
  const dim3 gy(B * c.mx, c.c / kCpb);
  const size_t smy = (size_t)(c.my * 2 * kCpb + 2 * c.h) * sizeof(float);
  k_modes_to_y<<<gy, 256, smy, f->stream>>>(v, out, c.h, c.c, c.mx, c.my, f->csy, 1.f);
  TARA_CK(cudaGetLastError());
  return TARA_OK;
}

// The fused head (fno_head_tc.cu) replaces the stored zh, h of the projection in
// the BF16 modes at 32 channels and 128 hidden units; forward and backward
// decide the same way.
bool head_fused(const tara_fno* f) { return bf16_mode(f) && head_tc_supported(f->cfg.c, f->cfg.p, f->cfg.co); }

int gemm(tara_fno* f, const GemmArgs& a) {
  const dim3 grid((a.N + GT_N - 1) / GT_N, (a.M + GT_M - 1) / GT_M, a.batch);
  if (f->cfg.mode == TARA_FNO_FP32)
    k_gemm_fp32<<<grid, 256, 0, f->stream>>>(a);
  else
    k_gemm_bf16<<<grid, 128, 0, f->stream>>>(a);
  TARA_CK(cudaGetLastError());
  return TARA_OK;
}

constexpr int kTsCtas = 152 * 2;

// C (M x N) (+)= A (M x K) B(K x N) (+bias) with the tall-skinny tensor-core kernel
// in BF16 mode for the shapes it is instantiated for; false when not handled.
bool ts_gemm(tara_fno* f, const float* A, long long M, int K, int N, const float* Bw, int transB,
             const float* bias, float* C, int accumulate, float* act, int act_mode) {
  if (f->cfg.mode == TARA_FNO_BF16_TMEM)
    return ts_gemm_tc_launch(A, M, K, N, Bw, transB, bias, C, accumulate, act, act_mode, f->errw, f->stream);
  if (f->cfg.mode != TARA_FNO_BF16) return false;
  const long long tiles = (M + kTsRows - 1) / kTsRows;
  const int grid = (int)std::min<long long>(tiles, kTsCtas * 2);
#define TS_CASE(KK, NN)                                                                          \
  if (K == KK && N == NN) {                                                                      \
    k_ts_gemm<KK, NN><<<grid, 256, 0, f->stream>>>(A, M, Bw, transB, bias, C, accumulate, act, act_mode); \
    return true;                                                                                 \
  }
  TS_CASE(32, 32)
  TS_CASE(32, 128)
  TS_CASE(128, 32)
#undef TS_CASE
  return false;
}

// dW (K x N) = A^T B over M rows (+ bias gradient = column sums of B) with the
// tensor-core reduction kernel in BF16 mode; false when not handled.
bool ts_wgrad(tara_fno* f, const float* A, int K, const float* B, int N, long long M, float* dW, float* dbias) {
  if (!bf16_mode(f)) return false;
  const int ctas = (int)std::min<long long>(kTsCtas, (M + 63) / 64);
  const long long per = ((M + ctas - 1) / ctas + 63) / 64 * 64;
  float* bias_part = f->part + (size_t)ctas * K * N;
  if ((size_t)ctas * (K * N + N) > f->part_n) return false;
#define TW_CASE(KK, NN)                                                                            \
  if (K == KK && N == NN) {                                                                        \
    k_ts_wgrad<KK, NN><<<ctas, 256, 0, f->stream>>>(A, B, M, per, f->part, dbias ? bias_part : nullptr); \
    k_sum_parts<<<64, dim3(32, 8), 0, f->stream>>>(f->part, ctas, K * N, dW, 0);                           \
    if (dbias) k_sum_parts<<<1, dim3(32, 8), 0, f->stream>>>(bias_part, ctas, N, dbias, 0);                \
    return true;                                                                                   \
  }
  TW_CASE(32, 32)
  TW_CASE(32, 128)
#undef TW_CASE
  return false;
}

// dW (K x N) = A^T B for a small K*N (<= 1024), CUDA cores
int wgrad_small(tara_fno* f, const float* A, int K, const float* B, int N, long long M, float* dW) {
  const int ctas = (int)std::min<long long>(std::max<size_t>(1, f->part_n / ((size_t)K * N)),
                                            std::min<long long>(4096, (M + 127) / 128));
  const long long per = (M + ctas - 1) / ctas;
  k_wgrad_small<<<ctas, 256, 0, f->stream>>>(A, K, B, N, M, per, f->part);
  k_sum_parts<<<64, dim3(32, 8), 0, f->stream>>>(f->part, ctas, K * N, dW, 0);
  TARA_CK(cudaGetLastError());
  return TARA_OK;
}

// C[M x N] (+)= A^T B over a long shared dimension K (rows): split-K into the
// `part` buffer, then one reduction.  A is (K x M) row-major with leading dim lda,
// B is (K x N) row-major with leading dim ldb.
int gemm_tn_long(tara_fno* f, const float* A, long long lda, const float* B, long long ldb, float* C,
                 int M, int N, long long K, int accumulate) {
  int parts = (int)std::min<long long>(256, (K + 4095) / 4096);
  if ((size_t)parts * M * N > f->part_n) parts = (int)(f->part_n / ((size_t)M * N));
  if (parts < 1) return set_error(TARA_ERR_ARGS, "split-K buffer too small");
  const long long chunk = (K + parts - 1) / parts;
  GemmArgs a{};
  a.M = M;
  a.N = N;
  a.K = (int)chunk;
  a.batch = parts;
  a.A = A;
  a.sab = chunk * lda;
  a.sam = 1;
  a.sak = lda;
  a.B = B;
  a.sbb = chunk * ldb;
  a.sbk = ldb;
  a.sbn = 1;
  a.C = f->part;
  a.scb = (long long)M * N;
  a.scm = N;
  a.scn = 1;
  a.alpha = 1.f;
  // the last chunk may run past K: those rows read zeros only if K divides evenly,
  // so clamp by giving the kernel the true K of each chunk via a second call
  if (chunk * parts != K) {
    a.batch = parts - 1;
    int rc = a.batch > 0 ? gemm(f, a) : TARA_OK;
    if (rc) return rc;
    GemmArgs t = a;
    t.batch = 1;
    t.K = (int)(K - chunk * (parts - 1));
    t.A = A + (parts - 1) * chunk * lda;
    t.B = B + (parts - 1) * chunk * ldb;
    t.C = f->part + (size_t)(parts - 1) * M * N;
    if ((rc = gemm(f, t))) return rc;
  } else {
    int rc = gemm(f, a);
    if (rc) return rc;
  }
  k_sum_parts<<<64, dim3(32, 8), 0, f->stream>>>(f->part, parts, M * N, C, accumulate);
  TARA_CK(cudaGetLastError());
  return TARA_OK;
}

int colsum(tara_fno* f, const float* x, long long M, int N, float* out) {
  const int parts = 128;
  k_colsum_part<<<parts, 256, 0, f->stream>>>(x, M, N, f->part);
  TARA_CK(cudaGetLastError());
  k_sum_parts<<<64, dim3(32, 8), 0, f->stream>>>(f->part, parts, N, out, 0);
  TARA_CK(cudaGetLastError());
  return TARA_OK;
}

void make_cs(int n, std::vector<float>& cs) {
  cs.resize(2 * n);
  for (int t = 0; t < n; ++t) {
    const long double a = 6.283185307179586476925286766559005768L * t / n;
    cs[2 * t] = (float)std::cos(a);
    cs[2 * t + 1] = (float)std::sin(a);
  }
}

float* act_v(tara_fno* f, int l) {  // v_l, l = 0..L
  return f->vact + (size_t)l * f->bmax * f->cfg.h * f->cfg.w * f->cfg.c;
}
float* act_z(tara_fno* f, int l) {  // z_l, l = 1..L
  return f->zact + (size_t)(l - 1) * f->bmax * f->cfg.h * f->cfg.w * f->cfg.c;
}
float* act_X(tara_fno* f, int l) {  // spectral input of layer l
  return f->X + (size_t)(l - 1) * f->bmax * f->cfg.my * f->cfg.mx * 2 * f->cfg.c;
}

// spectral convolution of v (B rows of H x W x C) into out (overwritten), with
// the layer's block weights Rb; the mode coefficients go to Xsave.
int spectral_fwd(tara_fno* f, const float* v, float* out, float* Xsave, const float* Rb, int B) {
  const auto& c = f->cfg;
  const int C = c.c, H = c.h, MX = c.mx, MY = c.my;
  int rc;
  if ((rc = x_to_modes(f, v, f->A, B * H, nullptr))) return rc;
  if ((rc = y_to_modes(f, f->A, Xsave, B))) return rc;
  // per-mode complex mixing: Y[b, m, :] = X[b, m, :] Rb[m]  (M = B, K = N = 2C)
  GemmArgs a{};
  a.M = B;
  a.N = 2 * C;
  a.K = 2 * C;
  a.batch = MY * MX;
  a.A = Xsave;
  a.sab = 2 * C;
  a.sam = (long long)MY * MX * 2 * C;
  a.sak = 1;
  a.B = Rb;
  a.sbb = 4LL * C * C;
  a.sbk = 2 * C;
  a.sbn = 1;
  a.C = f->Y;
  a.scb = 2 * C;
  a.scm = (long long)MY * MX * 2 * C;
  a.scn = 1;
  a.alpha = 1.f;
  if (B <= kMixB && 2 * C <= 128) {
    k_mode_mix<<<MY * MX, 128, 0, f->stream>>>(Xsave, Rb, f->Y, B, 2 * C, (long long)MY * MX * 2 * C,
                                               bf16_mode(f));
    TARA_CK(cudaGetLastError());
  } else if ((rc = gemm(f, a))) {
    return rc;
  }
  if ((rc = modes_to_y(f, f->Y, f->U, B))) return rc;
  if ((rc = modes_to_x(f, f->U, out, B * H, f->wx, 0))) return rc;
  return TARA_OK;
}

float* layer_rb(tara_fno* f, int l) {  // block matrices of layer l = 1..L
  return f->Rb + (size_t)(l - 1) * f->cfg.my * f->cfg.mx * 4 * f->cfg.c * f->cfg.c;
}

// Expand every layer's complex weights into the block matrices once per
// parameter change.
int refresh_rb(tara_fno* f) {
  if (f->rb_valid) return TARA_OK;
  const auto& c = f->cfg;
  for (int l = 1; l <= c.layers; ++l)
    k_expand_r<<<kPw, kTh, 0, f->stream>>>(f->p + f->off_R[l - 1], layer_rb(f, l), c.my * c.mx, c.c);
  TARA_CK(cudaGetLastError());
  f->rb_valid = true;
  return TARA_OK;
}

void params_changed(tara_fno* f) {
  f->rb_valid = false;
  f->pver += 1;
}

// Forward pass of the B samples already in f->x.
int forward(tara_fno* f, int B) {
  const auto& c = f->cfg;
  const int C = c.c;
  const long long rows = (long long)B * c.h * c.w;
  int rc;
  if ((rc = refresh_rb(f))) return rc;
  k_lift<<<(int)std::min<long long>((rows + 7) / 8, 152 * 32), dim3(C, 256 / C), 0, f->stream>>>(
      f->x, f->p + f->off_Pw, f->p + f->off_Pb, act_v(f, 0), rows, c.ci, C);
  TARA_CK(cudaGetLastError());
  for (int l = 1; l <= c.layers; ++l) {
    float* z = act_z(f, l);
    if ((rc = spectral_fwd(f, act_v(f, l - 1), z, act_X(f, l), layer_rb(f, l), B))) return rc;
    GemmArgs a{};  // z += v W + b ; v_l = GELU(z) (last layer: v_L = z)
    a.M = (int)rows;
    a.N = C;
    a.K = C;
    a.batch = 1;
    a.A = act_v(f, l - 1);
    a.sam = C;
    a.sak = 1;
    a.B = f->p + f->off_W[l - 1];
    a.sbk = C;
    a.sbn = 1;
    a.C = z;
    a.scm = C;
    a.scn = 1;
    a.alpha = 1.f;
    a.accumulate = 1;
    a.bias = f->p + f->off_b[l - 1];
    a.act = act_v(f, l);
    a.act_mode = l < c.layers ? 1 : 2;
    if (!ts_gemm(f, a.A, rows, C, C, a.B, 0, a.bias, z, 1, a.act, a.act_mode) && (rc = gemm(f, a))) return rc;
  }
  if (head_fused(f)) {  // y = GELU(v_L Q1 + q1) Q2 + q2, nothing else stored
    if (!head_fwd_tc_launch(act_v(f, c.layers), rows, f->p + f->off_Q1, f->p + f->off_q1, f->p + f->off_Q2,
                            f->p + f->off_q2, c.co, f->y, f->errw, f->stream))
      return set_error(TARA_ERR_CUDA, "fused head launch");
    return TARA_OK;
  }
  GemmArgs a{};  // zh = v_L Q1 + q1 ; h = GELU(zh)
  a.M = (int)rows;
  a.N = c.p;
  a.K = C;
  a.batch = 1;
  a.A = act_v(f, c.layers);
  a.sam = C;
  a.sak = 1;
  a.B = f->p + f->off_Q1;
  a.sbk = c.p;
  a.sbn = 1;
  a.C = f->zh;
  a.scm = c.p;
  a.scn = 1;
  a.alpha = 1.f;
  a.bias = f->p + f->off_q1;
  a.act = f->h;
  a.act_mode = 1;
  if (!ts_gemm(f, a.A, rows, C, c.p, a.B, 0, a.bias, f->zh, 0, f->h, 1) && (rc = gemm(f, a))) return rc;
  if (c.co <= 4)
    k_proj_out_warp<<<(int)std::min<long long>((rows + 7) / 8, 152 * 16), 256, 0, f->stream>>>(
        f->h, f->p + f->off_Q2, f->p + f->off_q2, f->y, rows, c.p, c.co);
  else
    k_proj_out<<<kPw, kTh, 0, f->stream>>>(f->h, f->p + f->off_Q2, f->p + f->off_q2, f->y, rows, c.p, c.co);
  TARA_CK(cudaGetLastError());
  return TARA_OK;
}

int backward(tara_fno* f, int B) {
  const auto& c = f->cfg;
  const int C = c.c, H = c.h, W = c.w, MX = c.mx, MY = c.my;
  const long long rows = (long long)B * H * W;
  int rc;
  TARA_CK(cudaMemsetAsync(f->g, 0, f->np * sizeof(float), f->stream));
  // projection
  if ((rc = colsum(f, f->dy, rows, c.co, f->g + f->off_q2))) return rc;
  if (head_fused(f)) {
    // dv = dh Q1^T and the partial dQ1, dq1, dQ2 of every CTA, then their sums
    const int parts = head_bwd_tc_grid(rows);
    const size_t nq1 = (size_t)C * c.p;
    if ((size_t)parts * (nq1 + c.p + (size_t)c.p * c.co) > f->part_n)
      return set_error(TARA_ERR_ARGS, "partial-sum buffer too small for the fused head");
    if (!head_bwd_tc_launch(act_v(f, c.layers), f->dy, rows, f->p + f->off_Q1, f->p + f->off_q1,
                            f->p + f->off_Q2, c.co, f->dv, f->part, f->errw, f->stream))
      return set_error(TARA_ERR_CUDA, "fused head backward launch");
    k_sum_parts<<<64, dim3(32, 8), 0, f->stream>>>(f->part, parts, (int)nq1, f->g + f->off_Q1, 0);
    k_sum_parts<<<64, dim3(32, 8), 0, f->stream>>>(f->part + parts * nq1, parts, c.p, f->g + f->off_q1, 0);
    k_sum_parts<<<64, dim3(32, 8), 0, f->stream>>>(f->part + parts * (nq1 + c.p), parts, c.p * c.co,
                                                   f->g + f->off_Q2, 0);
    TARA_CK(cudaGetLastError());
  } else {
  if (c.p * c.co <= 1024) {
    if ((rc = wgrad_small(f, f->h, c.p, f->dy, c.co, rows, f->g + f->off_Q2))) return rc;
  } else if ((rc = gemm_tn_long(f, f->h, c.p, f->dy, c.co, f->g + f->off_Q2, c.p, c.co, rows, 0))) {
    return rc;
  }
  if (c.co <= 4) {
    k_head_back<<<(int)std::min<long long>(rows, 152 * 64), c.p, 0, f->stream>>>(f->dy, f->p + f->off_Q2, f->zh,
                                                                               f->dh, rows, c.p, c.co);
  } else {
    k_proj_out_back<<<kPw, kTh, 0, f->stream>>>(f->dy, f->p + f->off_Q2, f->dh, rows, c.p, c.co);
    k_gelu_back<<<kPw, kTh, 0, f->stream>>>(f->zh, f->dh, f->dh, (size_t)rows * c.p);
  }
  TARA_CK(cudaGetLastError());
  if (!ts_wgrad(f, act_v(f, c.layers), C, f->dh, c.p, rows, f->g + f->off_Q1, f->g + f->off_q1)) {
    if ((rc = colsum(f, f->dh, rows, c.p, f->g + f->off_q1))) return rc;
    if ((rc = gemm_tn_long(f, act_v(f, c.layers), C, f->dh, c.p, f->g + f->off_Q1, C, c.p, rows, 0)))
      return rc;
  }
  if (!ts_gemm(f, f->dh, rows, c.p, C, f->p + f->off_Q1, 1, nullptr, f->dv, 0, nullptr, 0)) {
    GemmArgs a{};  // dv = dh Q1^T
    a.M = (int)rows;
    a.N = C;
    a.K = c.p;
    a.batch = 1;
    a.A = f->dh;
    a.sam = c.p;
    a.sak = 1;
    a.B = f->p + f->off_Q1;
    a.sbk = 1;
    a.sbn = c.p;
    a.C = f->dv;
    a.scm = C;
    a.scn = 1;
    a.alpha = 1.f;
    if ((rc = gemm(f, a))) return rc;
  }
  }  // layer-by-layer head
  for (int l = c.layers; l >= 1; --l) {
    float* dz = f->dz;
    if (l < c.layers) {
      k_gelu_back<<<kPw, kTh, 0, f->stream>>>(act_z(f, l), f->dv, dz, (size_t)rows * C);
      TARA_CK(cudaGetLastError());
    } else {
      TARA_CK(cudaMemcpyAsync(dz, f->dv, (size_t)rows * C * sizeof(float), cudaMemcpyDeviceToDevice, f->stream));
    }
    const float* vprev = act_v(f, l - 1);
    if (!ts_wgrad(f, vprev, C, dz, C, rows, f->g + f->off_W[l - 1], f->g + f->off_b[l - 1])) {
      if ((rc = colsum(f, dz, rows, C, f->g + f->off_b[l - 1]))) return rc;
      if ((rc = gemm_tn_long(f, vprev, C, dz, C, f->g + f->off_W[l - 1], C, C, rows, 0))) return rc;
    }
    if (!ts_gemm(f, dz, rows, C, C, f->p + f->off_W[l - 1], 1, nullptr, f->dv, 0, nullptr, 0)) {
      GemmArgs a{};  // dv = dz W^T
      a.M = (int)rows;
      a.N = C;
      a.K = C;
      a.batch = 1;
      a.A = dz;
      a.sam = C;
      a.sak = 1;
      a.B = f->p + f->off_W[l - 1];
      a.sbk = 1;
      a.sbn = C;
      a.C = f->dv;
      a.scm = C;
      a.scn = 1;
      a.alpha = 1.f;
      if ((rc = gemm(f, a))) return rc;
    }
    // spectral part: adjoints in reverse order
    if ((rc = x_to_modes(f, dz, f->A, B * H, f->wx))) return rc;
    if ((rc = y_to_modes(f, f->A, f->Y, B))) return rc;
    TARA_CK(cudaGetLastError());
    {
      GemmArgs a{};  // dRb[m] = X[:, m, :]^T dY[:, m, :]   (M = N = 2C, K = B)
      a.M = 2 * C;
      a.N = 2 * C;
      a.K = B;
      a.batch = MY * MX;
      a.A = act_X(f, l);
      a.sab = 2 * C;
      a.sam = 1;
      a.sak = (long long)MY * MX * 2 * C;
      a.B = f->Y;
      a.sbb = 2 * C;
      a.sbk = (long long)MY * MX * 2 * C;
      a.sbn = 1;
      a.C = f->dRb;
      a.scb = 4LL * C * C;
      a.scm = 2 * C;
      a.scn = 1;
      a.alpha = 1.f;
      if ((rc = gemm(f, a))) return rc;
      k_fold_r<<<kPw, kTh, 0, f->stream>>>(f->dRb, f->g + f->off_R[l - 1], MY * MX, C);
      TARA_CK(cudaGetLastError());
      GemmArgs t{};  // dX[:, m, :] = dY[:, m, :] Rb[m]^T
      t.M = B;
      t.N = 2 * C;
      t.K = 2 * C;
      t.batch = MY * MX;
      t.A = f->Y;
      t.sab = 2 * C;
      t.sam = (long long)MY * MX * 2 * C;
      t.sak = 1;
      t.B = layer_rb(f, l);
      t.sbb = 4LL * C * C;
      t.sbk = 1;
      t.sbn = 2 * C;
      t.C = f->U;  // dX, reusing the U buffer (same size)
      t.scb = 2 * C;
      t.scm = (long long)MY * MX * 2 * C;
      t.scn = 1;
      t.alpha = 1.f;
      if ((rc = gemm(f, t))) return rc;
    }
    if ((rc = modes_to_y(f, f->U, f->A, B))) return rc;
    if ((rc = modes_to_x(f, f->A, f->dv, B * H, nullptr, 1))) return rc;
    TARA_CK(cudaGetLastError());
  }
  // lifting
  if ((rc = colsum(f, f->dv, rows, C, f->g + f->off_Pb))) return rc;
  if (c.ci * C <= 1024) {
    if ((rc = wgrad_small(f, f->x, c.ci, f->dv, C, rows, f->g + f->off_Pw))) return rc;
  } else if ((rc = gemm_tn_long(f, f->x, c.ci, f->dv, C, f->g + f->off_Pw, c.ci, C, rows, 0))) {
    return rc;
  }
  return TARA_OK;
}

}  // namespace

namespace tara {

// Forward pass on the handle's current stream, leaving the output in the
// handle (valid until the next call); x is copied in first.
// Inference forward (nothing kept for a backward pass): the fused kernels of
// fno_fused.cu for small batches of the shapes they take, in the BF16 modes;
// otherwise the layer-by-layer forward.
int forward_infer(tara_fno* f, int B) {
  const auto& c = f->cfg;
  if (!f->fused || !bf16_mode(f) || c.layers > kFusedMaxLayers ||
      !fused_forward_supported(B, c.h, c.w, c.c, c.mx, c.my, c.ci, c.p, c.co))
    return forward(f, B);
  int rc;
  if ((rc = refresh_rb(f))) return rc;
  FusedFwdArgs a{};
  a.B = B;
  a.H = c.h;
  a.MX = c.mx;
  a.MY = c.my;
  a.CI = c.ci;
  a.P = c.p;
  a.CO = c.co;
  a.layers = c.layers;
  a.bf16 = 1;
  a.x = f->x;
  a.Pw = f->p + f->off_Pw;
  a.Pb = f->p + f->off_Pb;
  for (int l = 1; l <= c.layers; ++l) {
    a.Wl[l] = f->p + f->off_W[l - 1];
    a.bl[l] = f->p + f->off_b[l - 1];
    a.Rb[l] = layer_rb(f, l);
  }
  for (int l = 0; l < c.layers; ++l) a.v[l] = act_v(f, l);
  a.Q1 = f->p + f->off_Q1;
  a.q1 = f->p + f->off_q1;
  a.Q2 = f->p + f->off_Q2;
  a.q2 = f->p + f->off_q2;
  a.csx = f->csx;
  a.csy = f->csy;
  a.wx = f->wx;
  a.A = f->A;
  a.Y = f->Y;
  a.y = f->y;
  a.err = f->errw;
  return fused_forward_launch(a, f->stream);
}

int fno_forward_async(tara_fno* f, const float* x_dev, int B, const float** y) {
  if (!f || B < 1 || B > f->bmax) return set_error(TARA_ERR_ARGS, "bad arguments");
  const size_t n = (size_t)B * f->cfg.h * f->cfg.w * f->cfg.ci;
  if (x_dev && x_dev != f->x)
    TARA_CK(cudaMemcpyAsync(f->x, x_dev, n * sizeof(float), cudaMemcpyDeviceToDevice, f->stream));
  const int rc = forward_infer(f, B);
  if (rc) return rc;
  *y = f->y;
  return TARA_OK;
}

// Launch the network's work on `s` (nullptr: back to its own stream).
void fno_bind_stream(tara_fno* f, cudaStream_t s) { f->stream = s ? s : f->own_stream; }
// Flag tensor-core waits that gave up in `w` (nullptr: back to the handle's own word).
void fno_bind_error(tara_fno* f, unsigned int* w) { f->errw = w ? w : f->bad; }

const tara_fno_config& fno_config(const tara_fno* f) { return f->cfg; }
float* fno_input(tara_fno* f) { return f->x; }
unsigned long long fno_param_version(const tara_fno* f) { return f->pver; }
// Expand the block matrices now (outside any stream capture).
int fno_prepare(tara_fno* f) { return refresh_rb(f); }

}  // namespace tara

extern "C" {

void tara_fno_default_config(tara_fno_config* c) {
  std::memset(c, 0, sizeof(*c));
  c->h = c->w = 128;
  c->ci = 1;
  c->c = 32;
  c->mx = 16;
  c->my = 32;
  c->layers = 4;
  c->p = 128;
  c->co = 2;
  c->max_batch = 32;
  c->mode = TARA_FNO_BF16;
  c->seed = 1234;
}

int tara_fno_destroy(tara_fno* f) {
  if (!f) return set_ok();
  cudaSetDevice(f->dev);
  if (f->own_stream) cudaStreamSynchronize(f->own_stream);
  void* ptrs[] = {f->p, f->g, f->m, f->v, f->csx, f->csy, f->wx, f->x, f->tgt, f->vact, f->zact, f->X,
                  f->zh, f->h, f->y, f->dy, f->A, f->Y, f->U, f->S, f->Rb, f->dRb, f->dv, f->dz,
                  f->dh, f->part, f->lpart, f->bad};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  if (f->own_stream) cudaStreamDestroy(f->own_stream);
  delete f;
  return set_ok();
}

int tara_fno_create(const tara_fno_config* cfg, tara_fno** out) {
  if (!cfg || !out) return set_error(TARA_ERR_ARGS, "null argument");
  *out = nullptr;
  const auto& c = *cfg;
  if (c.h < 16 || c.w < 16 || c.c < 1 || c.c > 64 || c.mx < 1 || c.mx > c.w / 2 || c.my < 2 ||
      (c.my & 1) || c.my > c.h || c.layers < 1 || c.layers > 8 || c.p < 1 || c.co < 1 ||
      c.ci < 1 || c.max_batch < 1)
    return set_error(TARA_ERR_ARGS, "bad FNO shape");
  // the truncated-DFT kernels stage one row / column of channels in shared memory
  const size_t smax = 48 * 1024;
  if ((size_t)(c.w * c.c + 2 * c.w) * 4 > smax || (size_t)(c.mx * 2 * c.c + 2 * c.w) * 4 > smax)
    return set_error(TARA_ERR_ARGS, "FNO grid x channels too large for the DFT kernels");
  if ((c.h & (c.h - 1)) || (c.w & (c.w - 1)) || c.c % kCpb || c.p > 256 || c.co > 256)
    return set_error(TARA_ERR_ARGS, "FNO needs power-of-two grids, channels a multiple of 8, p, co <= 256");
  tara_fno* f = new tara_fno();
  f->cfg = c;
  f->bmax = c.max_batch;
  auto fail = [&](int code) {  // free the half-built handle, keep the error
    const ErrorState saved = save_error();
    tara_fno_destroy(f);
    restore_error(saved);
    return code;
  };
  // parameter layout
  size_t o = 0;
  f->off_Pw = o; o += (size_t)c.ci * c.c;
  f->off_Pb = o; o += c.c;
  for (int l = 0; l < c.layers; ++l) {
    f->off_R.push_back(o); o += (size_t)c.my * c.mx * c.c * c.c * 2;
    f->off_W.push_back(o); o += (size_t)c.c * c.c;
    f->off_b.push_back(o); o += c.c;
  }
  f->off_Q1 = o; o += (size_t)c.c * c.p;
  f->off_q1 = o; o += c.p;
  f->off_Q2 = o; o += (size_t)c.p * c.co;
  f->off_q2 = o; o += c.co;
  f->np = o;
  const size_t rows = (size_t)c.max_batch * c.h * c.w;
  const size_t modes = (size_t)c.max_batch * c.my * c.mx * 2 * c.c;
#define FA(ptr, n)                                                                   \
  do {                                                                               \
    if (cudaMalloc(&ptr, (size_t)(n) * sizeof(*ptr)) != cudaSuccess)                \
      return fail(set_error(TARA_ERR_NOMEM, "cudaMalloc in tara_fno_create"));      \
  } while (0)
  if (cudaGetDevice(&f->dev) != cudaSuccess ||
      cudaStreamCreateWithFlags(&f->own_stream, cudaStreamNonBlocking) != cudaSuccess)
    return fail(set_error(TARA_ERR_CUDA, "device/stream"));
  f->stream = f->own_stream;
  FA(f->p, f->np); FA(f->g, f->np); FA(f->m, f->np); FA(f->v, f->np);
  FA(f->csx, 2 * c.w); FA(f->csy, 2 * c.h); FA(f->wx, c.mx);
  FA(f->x, rows * c.ci);
  FA(f->tgt, rows * c.co);
  FA(f->vact, (size_t)(c.layers + 1) * rows * c.c);
  FA(f->zact, (size_t)c.layers * rows * c.c);
  FA(f->X, (size_t)c.layers * modes);
  FA(f->zh, rows * c.p); FA(f->h, rows * c.p); FA(f->dh, rows * c.p);
  FA(f->y, rows * c.co); FA(f->dy, rows * c.co);
  FA(f->A, (size_t)c.max_batch * c.h * c.mx * 2 * c.c);
  FA(f->Y, modes); FA(f->U, std::max(modes, (size_t)c.max_batch * c.h * c.mx * 2 * c.c));
  FA(f->S, rows * c.c);
  FA(f->Rb, (size_t)c.layers * c.my * c.mx * 4 * c.c * c.c); FA(f->dRb, (size_t)c.my * c.mx * 4 * c.c * c.c);
  FA(f->dv, rows * c.c); FA(f->dz, rows * c.c);
  f->part_n = std::max<size_t>((size_t)256 * c.p * std::max(c.c, c.co), (size_t)128 * std::max(c.p, c.c) * 4);
  f->part_n = std::max<size_t>(f->part_n, (size_t)kTsCtas * 2 *
                                             ((size_t)std::max(c.c * c.p, std::max(c.c * c.c, 1024)) + c.p + c.c));
  FA(f->part, f->part_n);
  FA(f->lpart, kPw);
  FA(f->bad, 1);
  f->errw = f->bad;
#undef FA
  // tables
  std::vector<float> cs;
  make_cs(c.w, cs);
  cudaMemcpy(f->csx, cs.data(), cs.size() * sizeof(float), cudaMemcpyHostToDevice);
  make_cs(c.h, cs);
  cudaMemcpy(f->csy, cs.data(), cs.size() * sizeof(float), cudaMemcpyHostToDevice);
  std::vector<float> wx(c.mx);
  for (int k = 0; k < c.mx; ++k) wx[k] = (k == 0 ? 1.f : 2.f) / ((float)c.h * (float)c.w);
  cudaMemcpy(f->wx, wx.data(), wx.size() * sizeof(float), cudaMemcpyHostToDevice);
  // initial parameters: uniform(-a, a) from a splitmix64 stream, a = 1/sqrt(fan_in)
  // for the linear maps and 1/(C*C) for the spectral weights; biases zero
  std::vector<float> hp(f->np, 0.f);
  uint64_t st = c.seed;
  auto urand = [&]() {
    st += 0x9E3779B97F4A7C15ull;
    uint64_t z = st;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
  };
  auto fill = [&](size_t off, size_t n, double a) {
    for (size_t i = 0; i < n; ++i) hp[off + i] = (float)((2.0 * urand() - 1.0) * a);
  };
  fill(f->off_Pw, (size_t)c.ci * c.c, 1.0 / std::sqrt((double)c.ci));
  for (int l = 0; l < c.layers; ++l) {
    fill(f->off_R[l], (size_t)c.my * c.mx * c.c * c.c * 2, 1.0 / ((double)c.c * c.c));
    fill(f->off_W[l], (size_t)c.c * c.c, 1.0 / std::sqrt((double)c.c));
  }
  fill(f->off_Q1, (size_t)c.c * c.p, 1.0 / std::sqrt((double)c.c));
  fill(f->off_Q2, (size_t)c.p * c.co, 1.0 / std::sqrt((double)c.p));
  if (cudaMemcpy(f->p, hp.data(), f->np * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemset(f->m, 0, f->np * sizeof(float)) != cudaSuccess ||
      cudaMemset(f->v, 0, f->np * sizeof(float)) != cudaSuccess)
    return fail(set_error(TARA_ERR_CUDA, "parameter upload"));
  *out = f;
  return set_ok();
}

size_t tara_fno_num_params(const tara_fno* f) { return f ? f->np : 0; }

int tara_fno_get_params(tara_fno* f, float* host) {
  if (!f || !host) return set_error(TARA_ERR_ARGS, "null argument");
  TARA_CK(cudaSetDevice(f->dev));
  TARA_CK(cudaStreamSynchronize(f->stream));
  TARA_CK(cudaMemcpy(host, f->p, f->np * sizeof(float), cudaMemcpyDeviceToHost));
  return set_ok();
}

int tara_fno_set_params(tara_fno* f, const float* host) {
  if (!f || !host) return set_error(TARA_ERR_ARGS, "null argument");
  TARA_CK(cudaSetDevice(f->dev));
  TARA_CK(cudaStreamSynchronize(f->stream));
  TARA_CK(cudaMemcpy(f->p, host, f->np * sizeof(float), cudaMemcpyHostToDevice));
  params_changed(f);
  return set_ok();
}

int tara_fno_get_grads(tara_fno* f, float* host) {
  if (!f || !host) return set_error(TARA_ERR_ARGS, "null argument");
  TARA_CK(cudaSetDevice(f->dev));
  TARA_CK(cudaStreamSynchronize(f->stream));
  TARA_CK(cudaMemcpy(host, f->g, f->np * sizeof(float), cudaMemcpyDeviceToHost));
  return set_ok();
}

int tara_fno_set_fused(tara_fno* f, int enable) {
  if (!f) return set_error(TARA_ERR_ARGS, "null handle");
  f->fused = enable != 0;
  return set_ok();
}

int tara_fno_set_mode(tara_fno* f, int mode) {
  if (!f || (mode != TARA_FNO_BF16 && mode != TARA_FNO_FP32 && mode != TARA_FNO_BF16_TMEM))
    return set_error(TARA_ERR_ARGS, "bad mode");
  f->cfg.mode = mode;
  return set_ok();
}

// x: device (B, H, W, CI) FP32; y: device (B, H, W, CO) FP32 (written).
int tara_fno_forward(tara_fno* f, const float* x_dev, float* y_dev, int B) {
  if (!f || !x_dev || !y_dev || B < 1 || B > f->bmax) return set_error(TARA_ERR_ARGS, "bad arguments");
  TARA_CK(cudaSetDevice(f->dev));
  int rc;
  const float* y = nullptr;
  TARA_CK(cudaMemsetAsync(f->bad, 0, sizeof(unsigned int), f->stream));
  if ((rc = fno_forward_async(f, x_dev, B, &y))) return rc;
  const size_t n = (size_t)B * f->cfg.h * f->cfg.w * f->cfg.co;
  TARA_CK(cudaMemcpyAsync(y_dev, y, n * sizeof(float), cudaMemcpyDeviceToDevice, f->stream));
  unsigned int bad = 0;
  TARA_CK(cudaMemcpyAsync(&bad, f->bad, sizeof(bad), cudaMemcpyDeviceToHost, f->stream));
  TARA_CK(cudaStreamSynchronize(f->stream));
  if (bad & 4u) return set_error(TARA_ERR_TIMEOUT, "a tensor-memory GEMM wait gave up");
  return set_ok();
}

// Forward + MSE loss + backward (gradients into the handle); optionally an Adam
// step with learning rate lr (lr <= 0: no update).  loss may be NULL.
int tara_fno_train_step(tara_fno* f, const float* x_dev, const float* t_dev, const int* idx_dev,
                        int n_samples, int B, float lr, double* loss) {
  if (!f || !x_dev || !t_dev || B < 1 || B > f->bmax || (idx_dev ? n_samples < 1 : n_samples < B))
    return set_error(TARA_ERR_ARGS, "bad arguments");
  TARA_CK(cudaSetDevice(f->dev));
  const auto& c = f->cfg;
  const size_t per_x = (size_t)c.h * c.w * c.ci, per_y = (size_t)c.h * c.w * c.co;
  TARA_CK(cudaMemsetAsync(f->bad, 0, sizeof(unsigned int), f->stream));
  k_gather<<<kPw, kTh, 0, f->stream>>>(x_dev, idx_dev, n_samples, B, per_x, f->x, f->bad);
  k_gather<<<kPw, kTh, 0, f->stream>>>(t_dev, idx_dev, n_samples, B, per_y, f->tgt, f->bad);
  TARA_CK(cudaGetLastError());
  int rc;
  if ((rc = forward(f, B))) return rc;
  const size_t n = (size_t)B * per_y;
  k_mse<<<kPw, kTh, 0, f->stream>>>(f->y, f->tgt, f->dy, n, f->lpart);
  TARA_CK(cudaGetLastError());
  if ((rc = backward(f, B))) return rc;
  if (lr > 0.f) {
    f->step += 1;
    const double b1 = 0.9, b2 = 0.999;
    const float c1 = (float)(1.0 - std::pow(b1, (double)f->step));
    const float c2 = (float)(1.0 - std::pow(b2, (double)f->step));
    k_adam<<<kPw, kTh, 0, f->stream>>>(f->p, f->g, f->m, f->v, f->np, lr, (float)b1, (float)b2, 1e-8f,
                                       c1, c2);
    TARA_CK(cudaGetLastError());
    params_changed(f);
  }
  std::vector<double> lp(kPw);
  unsigned int bad = 0;
  if (loss)
    TARA_CK(cudaMemcpyAsync(lp.data(), f->lpart, kPw * sizeof(double), cudaMemcpyDeviceToHost, f->stream));
  TARA_CK(cudaMemcpyAsync(&bad, f->bad, sizeof(bad), cudaMemcpyDeviceToHost, f->stream));
  TARA_CK(cudaStreamSynchronize(f->stream));
  if (bad & 4u) return set_error(TARA_ERR_TIMEOUT, "a tensor-memory GEMM wait gave up");
  if (bad) return set_error(TARA_ERR_ARGS, "sample index outside the dataset");
  if (loss) {
    double s = 0.0;
    for (double v : lp) s += v;
    *loss = s / (double)n;
  }
  return set_ok();
}

long long tara_fno_adam_steps(const tara_fno* f) { return f ? f->step : 0; }

void* tara_fno_stream(tara_fno* f) { return f ? (void*)f->stream : nullptr; }

}  // extern "C"
