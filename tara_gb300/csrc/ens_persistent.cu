// The ensemble's persistent form: one cooperative launch advances every run
// of every size group by n RK4 steps.
//
// Each RK stage is three passes over whole fields (column inverse, rows, column
// forward), so the kernel walks 12 phases per step with a grid-wide barrier
// (cooperative_groups grid sync; the cooperative launch guarantees that every
// CTA is resident) between them.  Inside a phase the CTAs take work items --
// one CTA tile of one pass of one run of one size -- from a global counter, so
// the uneven sizes pack onto the SMs without one branch per size.  The item
// bodies are the same CTA functions the per-pass kernels run, in the FP32
// form (FP32 transforms and products, FP64 state), with for each size the tile
// variants whose CTAs have kEnsThreads threads; results equal the graph path's
// on the same radix path bit for bit.  Sizes: 128, 256 and 512 (the sizes whose
// three passes all have 256-thread tiles).
//
// The counter only grows: in a phase with T items every CTA makes one failing
// fetch, so the phase takes T + gridDim.x fetches and the next phase's items
// start at a base every CTA can compute.  It is zeroed before each launch.
//
// The kernel carries the registers of its largest item body (about 214), so
// one CTA of 256 threads runs per SM.
#include <cooperative_groups.h>

#include <algorithm>
#include <vector>

#include "internal.h"

namespace cg = cooperative_groups;

namespace tara {

constexpr int kEnsThreads = 256;

// Tile variant of each pass whose CTA has kEnsThreads threads in the FP32 form
// at length N, or -1.
template <int N> constexpr int ens_va() {
  return ColCfg<float, N, 0>::THREADS_A == kEnsThreads   ? 0
         : ColCfg<float, N, 1>::THREADS_A == kEnsThreads ? 1
         : ColCfg<float, N, 2>::THREADS_A == kEnsThreads ? 2
                                                         : -1;
}
template <int N> constexpr int ens_vb() {
  return RowCfg<float, N, 0>::THREADS == kEnsThreads   ? 0
         : RowCfg<float, N, 1>::THREADS == kEnsThreads ? 1
         : RowCfg<float, N, 3>::THREADS == kEnsThreads ? 3
                                                       : -1;
}
template <int N> constexpr int ens_vc() {
  return ColCfg<float, N, 0>::THREADS_C == kEnsThreads   ? 0
         : ColCfg<float, N, 1>::THREADS_C == kEnsThreads ? 1
         : ColCfg<float, N, 2>::THREADS_C == kEnsThreads ? 2
                                                         : -1;
}
template <int N> constexpr bool ens_ok() { return ens_va<N>() >= 0 && ens_vb<N>() >= 0 && ens_vc<N>() >= 0; }
static_assert(ens_ok<128>() && ens_ok<256>() && ens_ok<512>(), "256-thread tiles at 128, 256, 512");

template <int N> constexpr int ens_smem() {
  return std::max(ColCfg<float, N, ens_va<N>()>::SMEM_A,
                  std::max(RowCfg<float, N, ens_vb<N>()>::SMEM, ColCfg<float, N, ens_vc<N>()>::SMEM_C));
}
constexpr int kEnsSmem = std::max(ens_smem<128>(), std::max(ens_smem<256>(), ens_smem<512>()));

// One size group as the kernel sees it (device memory).
struct EnsGroupDev {
  int n, runs;
  int ta, tb, tc;  // CTAs per run of pass A (per field pair), B, C
  Grid2D g;
  RhsParams p;
  double2 *w0, *ws, *acc, *fold;
  unsigned int* flag;
  const double2* force;
  void* u;
  void* nl;
  const void* twx;
  const void* twy;
};

template <int N, int R>
__device__ __forceinline__ void ens_item(const EnsGroupDev& G, int pass, int mode, int rem) {
  constexpr int VA = ens_va<N>(), VB = ens_vb<N>(), VC = ens_vc<N>();
  const double2* win = mode == MODE_RK1 ? G.w0 : G.ws;
  if (pass == 0) {
    const int per = 2 * G.ta, run = rem / per, t = rem % per;
    col_inverse_cta<float, N, VA, R>(t % G.ta, t / G.ta, run, win, (float2*)G.u, G.g, G.p,
                                     (const float2*)G.twy);
  } else if (pass == 1) {
    // coherent loads: this launch wrote u in the previous phase
    row_nl_cta<float, N, VB, R, false>(rem % G.tb, rem / G.tb, (const float2*)G.u, (float2*)G.nl, G.g,
                                (const float2*)G.twx);
  } else {
    StepBufs sb;
    sb.win = win;
    sb.w0 = G.w0;
    sb.ws = G.ws;
    sb.acc = G.acc;
    sb.fold = G.fold;
    sb.fout = nullptr;
    sb.flag = G.flag;
    sb.force = G.force;
    col_forward_cta<float, N, VC, R>(rem % G.tc, rem / G.tc, (const float2*)G.nl, sb, G.g, G.p, mode,
                                     (const float2*)G.twy);
  }
}

__device__ __forceinline__ int ens_items(const EnsGroupDev& G, int pass) {
  return G.runs * (pass == 0 ? 2 * G.ta : pass == 1 ? G.tb : G.tc);
}

template <int R>
__global__ void __launch_bounds__(kEnsThreads)
    k_ens_persistent(const EnsGroupDev* __restrict__ gd, int ngroups, int nsteps,
                     unsigned long long* __restrict__ ctr) {
  cg::grid_group grid = cg::this_grid();
  __shared__ int s_item;
  unsigned long long base = 0;
  for (int step = 0; step < nsteps; ++step)
    for (int st = 0; st < 4; ++st) {
      const int mode = MODE_RK1 + st;
      for (int pass = 0; pass < 3; ++pass) {
        int total = 0;
        for (int i = 0; i < ngroups; ++i) total += ens_items(gd[i], pass);
        for (;;) {
          if (threadIdx.x == 0) s_item = (int)(atomicAdd(ctr, 1ull) - base);
          __syncthreads();
          const int item = s_item;
          __syncthreads();  // everyone has read s_item before it is written again
          if (item >= total) break;
          int gi = 0, rem = item;
          while (rem >= ens_items(gd[gi], pass)) rem -= ens_items(gd[gi++], pass);
          switch (gd[gi].n) {
            case 128: ens_item<128, R>(gd[gi], pass, mode, rem); break;
            case 256: ens_item<256, R>(gd[gi], pass, mode, rem); break;
            case 512: ens_item<512, R>(gd[gi], pass, mode, rem); break;
            default: break;
          }
          __syncthreads();  // the next item reuses the shared memory
        }
        base += (unsigned long long)total + gridDim.x;
        grid.sync();
      }
    }
}

bool ens_persistent_supports(int n) { return n == 128 || n == 256 || n == 512; }

// Device descriptor of a group (a batched handle in the FP32 form with RK4).
template <int N>
static void ens_tiles(int nh, int ny, EnsGroupDev* d) {
  auto tiles = [](int per, int total) { return (total + per - 1) / per; };
  d->ta = tiles(ColCfg<float, N, ens_va<N>()>::TCA, nh);
  d->tb = tiles(2 * RowCfg<float, N, ens_vb<N>()>::RP, ny);
  d->tc = tiles(ColCfg<float, N, ens_vc<N>()>::TCC, nh);
}

static void ens_desc(tara2d* h, EnsGroupDev* d) {
  d->n = h->nx;
  d->runs = h->batch;
  if (h->nx == 128) ens_tiles<128>(h->nh, h->ny, d);
  if (h->nx == 256) ens_tiles<256>(h->nh, h->ny, d);
  if (h->nx == 512) ens_tiles<512>(h->nh, h->ny, d);
  d->g = h->grid;
  d->p = h->rp;
  d->w0 = h->w0;
  d->ws = h->ws;
  d->acc = h->acc;
  d->fold = h->fold;
  d->flag = h->flag;
  d->force = h->force;
  d->u = h->u;
  d->nl = h->nl;
  d->twx = h->twx;
  d->twy = h->twy;
}

size_t ens_desc_bytes(int ngroups) { return (size_t)ngroups * sizeof(EnsGroupDev); }

// One cooperative launch: nsteps RK4 steps of every group on `stream`.
// `desc` and `ctr` are device buffers of ngroups descriptors and one counter;
// radix8 selects the transforms' radix path.
int ens_persistent_launch(tara2d* const* hs, int ngroups, int nsteps, bool radix8, void* desc,
                          unsigned long long* ctr, cudaStream_t stream) {
  if (ngroups <= 0 || nsteps <= 0) return TARA_OK;
  std::vector<EnsGroupDev> d(ngroups);
  for (int i = 0; i < ngroups; ++i) {
    if (!ens_persistent_supports(hs[i]->nx) || hs[i]->nx != hs[i]->ny ||
        hs[i]->cfg.precision != TARA_PREC_FP32 || hs[i]->cfg.scheme != TARA_SCHEME_RK4)
      return set_error(TARA_ERR_ARGS,
                       "persistent ensemble: FP32 form, RK4, square grids of 128, 256 or 512 only");
    ens_desc(hs[i], &d[i]);
  }
  TARA_CK(cudaMemcpyAsync(desc, d.data(), d.size() * sizeof(EnsGroupDev), cudaMemcpyHostToDevice, stream));
  TARA_CK(cudaMemsetAsync(ctr, 0, sizeof(unsigned long long), stream));
  void (*kern)(const EnsGroupDev*, int, int, unsigned long long*) =
      radix8 ? k_ens_persistent<8> : k_ens_persistent<4>;
  static cudaError_t a4 =
      cudaFuncSetAttribute(k_ens_persistent<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, kEnsSmem);
  static cudaError_t a8 =
      cudaFuncSetAttribute(k_ens_persistent<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, kEnsSmem);
  TARA_CK(radix8 ? a8 : a4);
  int dev = 0, sms = 0, per_sm = 0;
  TARA_CK(cudaGetDevice(&dev));
  TARA_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  TARA_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kEnsThreads, kEnsSmem));
  if (per_sm <= 0) return set_error(TARA_ERR_CUDA, "persistent ensemble kernel does not fit on an SM");
  const EnsGroupDev* dd = (const EnsGroupDev*)desc;
  void* args[] = {(void*)&dd, (void*)&ngroups, (void*)&nsteps, (void*)&ctr};
  TARA_CK(cudaLaunchCooperativeKernel((const void*)kern, dim3(sms * per_sm), dim3(kEnsThreads), args,
                                      (size_t)kEnsSmem, stream));
  return TARA_OK;
}

}  // namespace tara
