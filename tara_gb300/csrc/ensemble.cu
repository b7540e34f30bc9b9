// Ensembles of independent 2D runs of uneven grid sizes (tara_ens_*).
//
// Runs of one size form a batched tara2d handle: every kernel launch advances
// all of them (the run index is a grid dimension), so a 128^2 run costs no extra
// launches.  One step of the whole ensemble -- every size group, every RK4
// stage -- is captured once into a CUDA graph with one parallel branch per size
// group (fork/join events on the groups' streams), and replayed with a single
// cudaGraphLaunch per step.  Before capture an autotuner (tara2d_autotune) times
// the three tile variants of each of the three kernels on the real batch
// (tara2d_step_timed reports per-kernel CUDA-event times) and keeps the fastest
// per kernel and size; the state is saved before and restored after the trials.
//
// The persistent form (ens_persistent.cu) replaces the graph by one cooperative
// launch per tara_ens_step call: every size, every RK stage, every step, with a
// grid-wide barrier between passes.  tara_ens_autotune times the graph and the
// persistent form on both radix paths and keeps the fastest; tara_ens_set_form
// fixes a form.
#include <algorithm>
#include <cstring>
#include <map>
#include <vector>

#include "internal.h"

struct tara_ens {
  struct Group {
    int n = 0;
    tara2d* h = nullptr;
    std::vector<int> runs;  // global run index of each slot
    double2* save_w0 = nullptr;
    double2* save_fold = nullptr;
    double tuned_ms[24] = {};  // [candidate][kernel]
  };
  int nruns = 0;
  std::vector<int> group_of, slot_of;
  std::vector<Group> groups;
  cudaStream_t main = nullptr;
  cudaEvent_t fork = nullptr;
  std::vector<cudaEvent_t> join;
  cudaGraphExec_t exec = nullptr;
  cudaGraph_t graph = nullptr;
  int dev = 0;
  int form = TARA_ENS_GRAPH;           // TARA_ENS_GRAPH / _PERSISTENT4 / _PERSISTENT8
  double form_ms[3] = {0, 0, 0};       // autotuner: ms per step of each form (0: not timed)
  void* pdesc = nullptr;               // device descriptors of the groups (persistent form)
  unsigned long long* pctr = nullptr;  // its work counter
};

using namespace tara;

namespace tara {
bool ens_persistent_supports(int n);
int ens_persistent_launch(tara2d* const* hs, int ngroups, int nsteps, bool radix8, void* desc,
                          unsigned long long* ctr, cudaStream_t stream);
size_t ens_desc_bytes(int ngroups);
}  // namespace tara

namespace {

bool persistent_ok(const tara_ens* e) {
  for (const auto& g : e->groups)
    if (!ens_persistent_supports(g.n) || g.h->cfg.precision != TARA_PREC_FP32 ||
        g.h->cfg.scheme != TARA_SCHEME_RK4)
      return false;
  return !e->groups.empty();
}

// nsteps of the persistent form on e->main, ordered after and before the
// groups' own streams.
int persistent_steps(tara_ens* e, int nsteps) {
  if (!e->pdesc) {
    TARA_CK(cudaMalloc(&e->pdesc, ens_desc_bytes((int)e->groups.size())));
    TARA_CK(cudaMalloc((void**)&e->pctr, sizeof(unsigned long long)));
  }
  std::vector<tara2d*> hs;
  for (size_t g = 0; g < e->groups.size(); ++g) {
    hs.push_back(e->groups[g].h);
    TARA_CK(cudaEventRecord(e->join[g], e->groups[g].h->stream));
    TARA_CK(cudaStreamWaitEvent(e->main, e->join[g], 0));
  }
  int rc = ens_persistent_launch(hs.data(), (int)hs.size(), nsteps, e->form == TARA_ENS_PERSISTENT8,
                                 e->pdesc, e->pctr, e->main);
  if (rc) return rc;
  TARA_CK(cudaEventRecord(e->fork, e->main));
  for (auto& g : e->groups) TARA_CK(cudaStreamWaitEvent(g.h->stream, e->fork, 0));
  return TARA_OK;
}

int save_or_restore(tara_ens* e, bool save) {
  for (auto& g : e->groups) {
    const size_t bytes = (size_t)g.h->batch * g.h->ny * g.h->pitch * sizeof(double2);
    if (!g.save_w0) {
      TARA_CK(cudaMalloc(&g.save_w0, bytes));
      TARA_CK(cudaMalloc(&g.save_fold, bytes));
    }
    TARA_CK(cudaMemcpyAsync(save ? g.save_w0 : g.h->w0, save ? g.h->w0 : g.save_w0, bytes,
                            cudaMemcpyDeviceToDevice, g.h->stream));
    TARA_CK(cudaMemcpyAsync(save ? g.save_fold : g.h->fold, save ? g.h->fold : g.save_fold, bytes,
                            cudaMemcpyDeviceToDevice, g.h->stream));
    TARA_CK(cudaStreamSynchronize(g.h->stream));
  }
  return TARA_OK;
}

void drop_graph(tara_ens* e) {
  if (e->exec) cudaGraphExecDestroy(e->exec);
  if (e->graph) cudaGraphDestroy(e->graph);
  e->exec = nullptr;
  e->graph = nullptr;
}

// Capture one ensemble step into a graph: fork on `main`, each group's step on
// its own stream, join back on `main`.
int capture(tara_ens* e) {
  drop_graph(e);
  TARA_CK(cudaStreamBeginCapture(e->main, cudaStreamCaptureModeThreadLocal));
  int rc = TARA_OK;
  if (cudaEventRecord(e->fork, e->main) != cudaSuccess) rc = set_error(TARA_ERR_CUDA, "fork");
  for (size_t g = 0; g < e->groups.size() && !rc; ++g) {
    tara2d* h = e->groups[g].h;
    if (cudaStreamWaitEvent(h->stream, e->fork, 0) != cudaSuccess) rc = set_error(TARA_ERR_CUDA, "wait");
    if (!rc) rc = tara2d_step(h, 1);
    if (!rc && (cudaEventRecord(e->join[g], h->stream) != cudaSuccess ||
                cudaStreamWaitEvent(e->main, e->join[g], 0) != cudaSuccess))
      rc = set_error(TARA_ERR_CUDA, "join");
  }
  cudaGraph_t graph = nullptr;
  const cudaError_t ec = cudaStreamEndCapture(e->main, &graph);
  if (rc) {
    if (graph) cudaGraphDestroy(graph);
    return rc;
  }
  if (ec != cudaSuccess) return cuda_fail(ec, "cudaStreamEndCapture");
  e->graph = graph;
  TARA_CK(cudaGraphInstantiate(&e->exec, e->graph, 0));
  return TARA_OK;
}

}  // namespace

extern "C" {

int tara_ens_destroy(tara_ens* e) {
  if (!e) return set_ok();
  cudaSetDevice(e->dev);
  if (e->main) cudaStreamSynchronize(e->main);
  drop_graph(e);
  for (auto& g : e->groups) {
    tara2d_destroy(g.h);
    cudaFree(g.save_w0);
    cudaFree(g.save_fold);
  }
  cudaFree(e->pdesc);
  cudaFree(e->pctr);
  for (cudaEvent_t ev : e->join)
    if (ev) cudaEventDestroy(ev);
  if (e->fork) cudaEventDestroy(e->fork);
  if (e->main) cudaStreamDestroy(e->main);
  delete e;
  return set_ok();
}

int tara_ens_create(int nruns, const tara_ens_run* runs, int precision, int scheme, double nu,
                    double dt, double energy, tara_ens** out) {
  if (!runs || !out || nruns <= 0) return set_error(TARA_ERR_ARGS, "bad arguments");
  *out = nullptr;
  tara_ens* e = new tara_ens();
  e->nruns = nruns;
  auto fail = [&](int code) {  // free the half-built handle, keep the error
    const ErrorState saved = save_error();
    tara_ens_destroy(e);
    restore_error(saved);
    return code;
  };
  if (cudaGetDevice(&e->dev) != cudaSuccess) return fail(set_error(TARA_ERR_CUDA, "cudaGetDevice"));
  std::map<int, int> by_n;
  e->group_of.resize(nruns);
  e->slot_of.resize(nruns);
  for (int r = 0; r < nruns; ++r) {
    const int n = runs[r].n;
    if (!is_pow2_in_range(n) || !(runs[r].k0 > 0.0))
      return fail(set_error(TARA_ERR_ARGS, "run sizes must be powers of two in [16, 4096], k0 > 0"));
    auto it = by_n.find(n);
    if (it == by_n.end()) {
      it = by_n.emplace(n, (int)e->groups.size()).first;
      e->groups.emplace_back();
      e->groups.back().n = n;
    }
    auto& g = e->groups[it->second];
    e->group_of[r] = it->second;
    e->slot_of[r] = (int)g.runs.size();
    g.runs.push_back(r);
  }
  for (auto& g : e->groups) {
    tara2d_config c;
    tara2d_default_config(&c, g.n, g.n);
    c.scheme = scheme;
    c.precision = precision;
    c.nu = nu;
    c.dt = dt;
    c.batch = (int)g.runs.size();
    int rc = tara2d_create(&c, &g.h);
    if (rc) return fail(rc);
    for (size_t s = 0; s < g.runs.size(); ++s) {
      const tara_ens_run& rr = runs[g.runs[s]];
      if ((rc = tara2d_init_random_run(g.h, (int)s, rr.k0, energy, rr.seed))) return fail(rc);
    }
  }
  if (cudaStreamCreateWithFlags(&e->main, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&e->fork, cudaEventDisableTiming) != cudaSuccess)
    return fail(set_error(TARA_ERR_CUDA, "stream/event"));
  e->join.resize(e->groups.size(), nullptr);
  for (auto& ev : e->join)
    if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess)
      return fail(set_error(TARA_ERR_CUDA, "event"));
  *out = e;
  return set_ok();
}

static int graph_steps(tara_ens* e, int nsteps) {
  int rc;
  if (!e->exec) {
    // one untimed pass sets every kernel's shared-memory attribute outside the
    // capture; the state is restored afterwards
    if ((rc = save_or_restore(e, true))) return rc;
    for (auto& g : e->groups)
      if ((rc = tara2d_step(g.h, 1))) return rc;
    if ((rc = save_or_restore(e, false))) return rc;
    if ((rc = capture(e))) return rc;
  }
  for (int s = 0; s < nsteps; ++s) TARA_CK(cudaGraphLaunch(e->exec, e->main));
  return TARA_OK;
}

int tara_ens_step(tara_ens* e, int nsteps) {
  if (!e || nsteps < 0) return set_error(TARA_ERR_ARGS, "bad arguments");
  TARA_CK(cudaSetDevice(e->dev));
  int rc = e->form == TARA_ENS_GRAPH ? graph_steps(e, nsteps) : persistent_steps(e, nsteps);
  return rc ? rc : set_ok();
}

int tara_ens_set_form(tara_ens* e, int form) {
  if (!e || form < TARA_ENS_GRAPH || form > TARA_ENS_PERSISTENT8)
    return set_error(TARA_ERR_ARGS, "form: TARA_ENS_GRAPH, TARA_ENS_PERSISTENT4 or TARA_ENS_PERSISTENT8");
  if (form != TARA_ENS_GRAPH && !persistent_ok(e))
    return set_error(TARA_ERR_ARGS,
                     "the persistent form needs the FP32 form, RK4 and square grids of 128, 256 or 512");
  TARA_CK(cudaSetDevice(e->dev));
  TARA_CK(cudaStreamSynchronize(e->main));
  e->form = form;
  return set_ok();
}

int tara_ens_form(tara_ens* e, int* form, double* ms3) {
  if (!e) return set_error(TARA_ERR_ARGS, "null handle");
  if (form) *form = e->form;
  if (ms3)
    for (int i = 0; i < 3; ++i) ms3[i] = e->form_ms[i];
  return set_ok();
}

int tara_ens_autotune(tara_ens* e, int trial_steps) {
  if (!e || trial_steps <= 0) return set_error(TARA_ERR_ARGS, "bad arguments");
  TARA_CK(cudaSetDevice(e->dev));
  TARA_CK(cudaStreamSynchronize(e->main));
  int rc;
  for (auto& g : e->groups)  // each group saves and restores its own state
    if ((rc = tara2d_autotune(g.h, trial_steps, nullptr, g.tuned_ms))) return rc;
  drop_graph(e);  // the graph bakes in the launch shapes
  // Form: the graph (with the tiles just chosen) against the persistent launch
  // on both radix paths, each after one settling step, timed over trial_steps
  // steps with CUDA events on the main stream; the state is restored after.
  for (int f = 0; f < 3; ++f) e->form_ms[f] = 0.0;
  const int nforms = persistent_ok(e) ? 3 : 1;
  if ((rc = save_or_restore(e, true))) return rc;
  cudaEvent_t a = nullptr, b = nullptr;
  TARA_CK(cudaEventCreate(&a));
  TARA_CK(cudaEventCreate(&b));
  const int keep = e->form;
  for (int f = 0; f < nforms && !rc; ++f) {
    e->form = f;
    rc = tara_ens_step(e, 1);
    if (!rc && cudaEventRecord(a, e->main) != cudaSuccess) rc = set_error(TARA_ERR_CUDA, "event");
    if (!rc) rc = tara_ens_step(e, trial_steps);
    if (!rc && (cudaEventRecord(b, e->main) != cudaSuccess || cudaEventSynchronize(b) != cudaSuccess))
      rc = set_error(TARA_ERR_CUDA, "event");
    float ms = 0.f;
    if (!rc && cudaEventElapsedTime(&ms, a, b) != cudaSuccess) rc = set_error(TARA_ERR_CUDA, "event time");
    if (!rc) e->form_ms[f] = ms / trial_steps;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  e->form = keep;
  if (rc) return rc;
  int best = 0;
  for (int f = 1; f < nforms; ++f)
    if (e->form_ms[f] < e->form_ms[best]) best = f;
  e->form = best;
  if ((rc = tara_ens_synchronize(e))) return rc;
  if ((rc = save_or_restore(e, false))) return rc;
  return set_ok();
}

int tara_ens_synchronize(tara_ens* e) {
  if (!e) return set_error(TARA_ERR_ARGS, "null handle");
  TARA_CK(cudaSetDevice(e->dev));
  TARA_CK(cudaStreamSynchronize(e->main));
  for (auto& g : e->groups) {
    const int rc = tara2d_synchronize(g.h);
    if (rc) return rc;
  }
  return set_ok();
}

void* tara_ens_stream(tara_ens* e) { return e ? (void*)e->main : nullptr; }

int tara_ens_get_state(tara_ens* e, int run, double* omegak) {
  if (!e || run < 0 || run >= e->nruns) return set_error(TARA_ERR_ARGS, "bad run");
  TARA_CK(cudaSetDevice(e->dev));
  TARA_CK(cudaStreamSynchronize(e->main));
  return tara2d_get_state_run(e->groups[e->group_of[run]].h, e->slot_of[run], omegak, nullptr);
}

int tara_ens_set_state(tara_ens* e, int run, const double* omegak) {
  if (!e || run < 0 || run >= e->nruns) return set_error(TARA_ERR_ARGS, "bad run");
  TARA_CK(cudaSetDevice(e->dev));
  TARA_CK(cudaStreamSynchronize(e->main));
  return tara2d_set_state_run(e->groups[e->group_of[run]].h, e->slot_of[run], omegak, nullptr);
}

int tara_ens_diag(tara_ens* e, int run, double* energy, double* enstrophy) {
  if (!e || run < 0 || run >= e->nruns) return set_error(TARA_ERR_ARGS, "bad run");
  TARA_CK(cudaSetDevice(e->dev));
  TARA_CK(cudaStreamSynchronize(e->main));
  return tara2d_diag_run(e->groups[e->group_of[run]].h, e->slot_of[run], energy, enstrophy);
}

int tara_ens_group_info(tara_ens* e, int group, int* n, int* runs, int* variants3,
                        double* tuned_ms24) {
  if (!e || group < 0 || group >= (int)e->groups.size()) return set_error(TARA_ERR_ARGS, "bad group");
  const auto& g = e->groups[group];
  if (n) *n = g.n;
  if (runs) *runs = (int)g.runs.size();
  if (variants3)
    for (int k = 0; k < 3; ++k) variants3[k] = g.h->var[k];
  if (tuned_ms24)
    for (int i = 0; i < 24; ++i) tuned_ms24[i] = g.tuned_ms[i];
  return set_ok();
}

int tara_ens_groups(tara_ens* e) { return e ? (int)e->groups.size() : 0; }

int tara_ens_launches_per_step(tara_ens* e) {
  if (!e) return 0;
  int n = 0;
  for (auto& g : e->groups) n += tara2d_launches_per_step(g.h);
  return n;
}

}  // extern "C"
