// Fused small-batch inference forward of the Fourier neural operator
// (fno_fused.cu): arguments and the shapes it takes.
#pragma once
#include <cuda_runtime.h>

namespace tara {

constexpr int kFusedW = 128;        // grid points along x: the rows of one tcgen05 tile
constexpr int kFusedC = 32;         // channels
constexpr int kFusedMaxB = 4;       // samples per call
constexpr int kFusedMaxH = 256;     // grid points along y
constexpr int kFusedMaxMX = 16;     // retained kx modes (one 128-thread half of a CTA per kx and 4 channels)
constexpr int kFusedMaxCO = 4;      // output channels
constexpr int kFusedMaxModes = 512; // mx * my: one sample's mixed modes (128 KB) sit in shared memory
constexpr int kFusedMaxLayers = 8;  // Fourier layers

struct FusedFwdArgs {
  int B, H, MX, MY, CI, P, CO, layers, bf16;
  const float* x;                         // [B][H][W][CI] input
  const float *Pw, *Pb;                   // lift CI x C, C
  const float* Wl[kFusedMaxLayers + 1];   // pointwise weights of layer l (index l = 1..layers), C x C
  const float* bl[kFusedMaxLayers + 1];   // their biases
  const float* Rb[kFusedMaxLayers + 1];   // per-mode block matrices [MY][MX][2C][2C]
  const float *Q1, *q1, *Q2, *q2;         // projection C x P, P, P x CO, CO
  const float *csx, *csy, *wx;            // cos/sin tables along x and y, inverse-DFT weights per kx
  float* v[kFusedMaxLayers + 1];          // activations v_0 .. v_{layers-1}, [B][H][W][C]
  float *A, *Y;                           // [B][H][MX][2][C] row modes, [B][MY][MX][2C] mixed modes
  float* y;                               // [B][H][W][CO] output
  unsigned int* err;                      // bit 2 (value 4) set when a tensor-core wait gave up
};

bool fused_forward_supported(int B, int H, int W, int C, int MX, int MY, int CI, int P, int CO);
int fused_forward_launch(const FusedFwdArgs& a, cudaStream_t s);

}  // namespace tara
