// ep_api.cu - the C ABI of include/eff_pot.h.
//
// One ep_ctx is one solver instance on one GPU: its own stream, its own
// device buffers (Engine<double> for the FP64 drop-in path, Engine<float>
// for the FP32 path) and the small host-side impurity state.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/eff_pot.h"
#include "ep_engine.h"
#include "ep_pairpot.h"

// A captured steppc (one context, or one step of every context of a batch)
// and, per context, its predictor / corrector nodes and the engine state the
// capture depends on (which engine, its launch shapes).
struct StepGraph {
  cudaGraph_t graph = nullptr;  // kept alive: node updates name its nodes
  cudaGraphExec_t exec = nullptr;
  std::vector<std::pair<cudaGraphNode_t, cudaGraphNode_t>> nodes;
  std::vector<const void*> engine;
  std::vector<int> gen;
  std::vector<long long> launches;  // kernels per replay, per context
  // multi-step graphs: steps per replay, and each context's next-step
  // buffers when the capture began (the replay is valid at that phase only)
  int nsteps = 1;
  std::vector<std::array<const void*, 7>> sig0;
  void reset() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    exec = nullptr;
    graph = nullptr;
    nodes.clear();
    engine.clear();
    gen.clear();
    launches.clear();
    sig0.clear();
    nsteps = 1;
  }
};

struct ep_ctx {
  StepGraph graph;
  StepGraph graphk;  // one rotation period of steps
  int use_graphs = 1;  // 0 direct launches, 1 step graphs, 2 multi-step graphs
  ep_config cfg{};
  cudaStream_t st = nullptr;
  Prof prof;
  ImpState imp;
  std::string err;
  Engine<double>* e64 = nullptr;
  Engine<float>* e32 = nullptr;
  Engine<dfloat>* edd = nullptr;
  int active = EP_FP64;
  cudaEvent_t ev[16] = {};
};

struct ep_batch {
  StepGraph graph;
  StepGraph graphk;  // one rotation period of steps
  int use_graphs = 1;  // 0 direct launches, 1 step graphs, 2 multi-step graphs
  std::vector<ep_ctx*> ctx;
  cudaStream_t st = nullptr;
  cudaEvent_t fork = nullptr;
  std::vector<cudaEvent_t> join;
  cudaEvent_t ev[16] = {};
  int device = 0;
};

namespace {

thread_local std::string g_create_error;

bool factor235(int n) {
  if (n < 2) return false;
  while (n % 2 == 0) n /= 2;
  while (n % 3 == 0) n /= 3;
  while (n % 5 == 0) n /= 5;
  return n == 1;
}

int fail(ep_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

// Select_Pot (V_impur.f90:87-932) plus the Morse selector.
double select_pot(const ep_potential& p, double r) {
  return ep_pair_potential(p.kind, p.r_cutoff, p.umax, p.par, p.series, r);
}

// A potential the evaluator knows; a series fit with 0 < n <= EP_SERIES_MAX.
const char* bad_potential(const ep_potential* p) {
  if (!p) return "null potential";
  if (p->kind < EP_POT_NULL || p->kind > EP_POT_EXPFIT) return "unknown potential kind";
  if (p->kind == EP_POT_SERIES || p->kind == EP_POT_EVENPOW || p->kind == EP_POT_EXPFIT) {
    if (!p->series) return "a fitted potential without its fit";
    if (p->series->n < 1 || p->series->n > EP_SERIES_MAX) return "series fit: n outside 1..EP_SERIES_MAX";
    if (p->series->k0 < 0 || p->series->k0 > 64) return "series fit: k0 outside 0..64";
  }
  return nullptr;
}

// Keeps plus for energy(): the fit is copied, the borrowed pointer dropped.
void keep_plus(ImpState& imp, const ep_potential* plus) {
  imp.plus = *plus;
  imp.plus.series = nullptr;
  imp.plus_series = ep_series{};
  if (plus->series) imp.plus_series = *plus->series;
}

template <class F>
int dispatch(ep_ctx* c, F f) {
  if (!c) return EP_ERR_INVALID_ARG;
  if (c->active == EP_FP64 && c->e64) return f(*c->e64);
  if (c->active == EP_FP32 && c->e32) return f(*c->e32);
  if (c->active == EP_DFLOAT && c->edd) return f(*c->edd);
  return fail(c, EP_ERR_STATE, "context has no engine");
}

// ---------------------------------------------------------------------------
// Step graphs.  A steppc of a context with a fixed (or no) impurity launches
// the same kernels every step; only the predictor and corrector see the
// rotating history buffers.  One step (of one context, or of every context
// of a batch on their forked streams) is captured once; later steps update
// the two march nodes per context and launch the graph.
const void* engine_of(ep_ctx* c) {
  return c->active == EP_FP64 ? (const void*)c->e64
         : c->active == EP_FP32 ? (const void*)c->e32 : (const void*)c->edd;
}
int gen_of(ep_ctx* c) {
  return dispatch(c, [](auto& e) -> int { return e.shapes_gen; });
}
bool graph_eligible(ep_ctx* c) {
  return c->use_graphs > 0 && dispatch(c, [](auto& e) -> int { return e.graph_ok() ? 1 : 0; }) == 1;
}
bool graph_valid(const StepGraph& G, const std::vector<ep_ctx*>& cs) {
  if (!G.exec || G.engine.size() != cs.size()) return false;
  for (size_t i = 0; i < cs.size(); ++i)
    if (G.engine[i] != engine_of(cs[i]) || G.gen[i] != gen_of(cs[i])) return false;
  return true;
}

// Every instance stream waits for the batch stream, then the batch stream
// waits for every instance: batch events bracket all instances' work.
void batch_fork(ep_batch* b) {
  cudaEventRecord(b->fork, b->st);
  for (ep_ctx* c : b->ctx) cudaStreamWaitEvent(c->st, b->fork, 0);
}
void batch_join(ep_batch* b) {
  for (size_t i = 0; i < b->ctx.size(); ++i) {
    cudaEventRecord(b->join[i], b->ctx[i]->st);
    cudaStreamWaitEvent(b->st, b->join[i], 0);
  }
}

// Capture one step of every context of cs into G on stream st (forked to the
// contexts' streams when b is given) and run it.
int capture_step(StepGraph& G, const std::vector<ep_ctx*>& cs, cudaStream_t st, ep_batch* b, double dt) {
  G.reset();
  const size_t n = cs.size();
  G.nodes.assign(n, {nullptr, nullptr});
  G.engine.assign(n, nullptr);
  G.gen.assign(n, 0);
  G.launches.assign(n, 0);
  if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return EP_ERR_CUDA;
  if (b) batch_fork(b);
  int r = EP_OK;
  for (size_t i = 0; i < n && !r; ++i) {
    ep_ctx* c = cs[i];
    const long long l0 = c->prof.launches;
    r = dispatch(c, [&](auto& e) -> int {
      e.cap_nodes = &G.nodes[i];
      const int q = e.steppc(dt, nullptr);
      e.cap_nodes = nullptr;
      return q;
    });
    G.launches[i] = c->prof.launches - l0;
    G.engine[i] = engine_of(c);
    G.gen[i] = gen_of(c);
  }
  if (b && !r) batch_join(b);
  cudaGraph_t graph = nullptr;
  const cudaError_t e = cudaStreamEndCapture(st, &graph);
  if (r || e != cudaSuccess || !graph) {
    if (graph) cudaGraphDestroy(graph);
    G.reset();
    cudaGetLastError();
    return r ? r : EP_ERR_CUDA;
  }
  G.graph = graph;
  const cudaError_t ei = cudaGraphInstantiate(&G.exec, graph, 0);
  if (ei != cudaSuccess) {
    G.exec = nullptr;
    G.reset();
    return EP_ERR_CUDA;
  }
  return cudaGraphLaunch(G.exec, st) == cudaSuccess ? EP_OK : EP_ERR_CUDA;
}

// One replayed step: the host half of every context's step, then the graph.
int replay_step(StepGraph& G, const std::vector<ep_ctx*>& cs, cudaStream_t st, double dt) {
  for (size_t i = 0; i < cs.size(); ++i) {
    ep_ctx* c = cs[i];
    const int r = dispatch(c, [&](auto& e) -> int {
      return e.steppc_update(dt, G.exec, G.nodes[i].first, G.nodes[i].second);
    });
    if (r) return r;
    c->prof.launches += G.launches[i];
  }
  return cudaGraphLaunch(G.exec, st) == cudaSuccess ? EP_OK : EP_ERR_CUDA;
}

// ---------------------------------------------------------------------------
// Multi-step graphs.  The buffers a step reads and writes repeat after a
// fixed number of steps (the history rotation: 10 for steppc), so that many
// consecutive steps of every context are captured once and replayed with no
// node updates at all; after a replay the host applies the same number of
// buffer rotations.  A replay is valid only at the phase of the rotation
// where it was captured; single steps realign the phase.
std::array<const void*, 7> signature_of(ep_ctx* c) {
  std::array<const void*, 7> a{};
  dispatch(c, [&](auto& e) -> int {
    const void* s[7];
    e.step_signature(s);
    for (int k = 0; k < 7; ++k) a[k] = s[k];
    return EP_OK;
  });
  return a;
}
int common_period(const std::vector<ep_ctx*>& cs) {
  int P = 0;
  for (ep_ctx* c : cs) {
    const int p = dispatch(c, [](auto& e) -> int { return e.rotation_period(); });
    if (p <= 0) return 0;
    if (P == 0) P = p;
    else if (P != p) return 0;
  }
  return P;
}
bool at_phase(const StepGraph& G, const std::vector<ep_ctx*>& cs) {
  if (G.sig0.size() != cs.size()) return false;
  for (size_t i = 0; i < cs.size(); ++i)
    if (signature_of(cs[i]) != G.sig0[i]) return false;
  return true;
}
int capture_steps(StepGraph& G, const std::vector<ep_ctx*>& cs, cudaStream_t st, ep_batch* b, double dt, int P) {
  G.reset();
  const size_t n = cs.size();
  G.engine.assign(n, nullptr);
  G.gen.assign(n, 0);
  G.launches.assign(n, 0);
  G.sig0.resize(n);
  for (size_t i = 0; i < n; ++i) G.sig0[i] = signature_of(cs[i]);
  if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return EP_ERR_CUDA;
  if (b) batch_fork(b);
  int r = EP_OK;
  for (int p = 0; p < P && !r; ++p) {  // step-major: the contexts' kernels overlap
    for (size_t i = 0; i < n && !r; ++i) {
      ep_ctx* c = cs[i];
      const long long l0 = c->prof.launches;
      r = dispatch(c, [&](auto& e) -> int { return e.steppc(dt, nullptr); });
      G.launches[i] += c->prof.launches - l0;
    }
  }
  for (size_t i = 0; i < n; ++i) {
    G.engine[i] = engine_of(cs[i]);
    G.gen[i] = gen_of(cs[i]);
  }
  if (b && !r) batch_join(b);
  cudaGraph_t graph = nullptr;
  const cudaError_t e = cudaStreamEndCapture(st, &graph);
  if (r || e != cudaSuccess || !graph) {
    if (graph) cudaGraphDestroy(graph);
    G.reset();
    cudaGetLastError();
    return r ? r : EP_ERR_CUDA;
  }
  G.graph = graph;
  if (cudaGraphInstantiate(&G.exec, graph, 0) != cudaSuccess) {
    G.exec = nullptr;
    G.reset();
    return EP_ERR_CUDA;
  }
  G.nsteps = P;
  return cudaGraphLaunch(G.exec, st) == cudaSuccess ? EP_OK : EP_ERR_CUDA;
}
int replay_steps(StepGraph& G, const std::vector<ep_ctx*>& cs, cudaStream_t st) {
  if (cudaGraphLaunch(G.exec, st) != cudaSuccess) return EP_ERR_CUDA;
  for (size_t i = 0; i < cs.size(); ++i) {
    dispatch(cs[i], [&](auto& e) -> int {
      for (int p = 0; p < G.nsteps; ++p) e.rotate_step();
      return EP_OK;
    });
    cs[i]->prof.launches += G.launches[i];
  }
  return EP_OK;
}

// ng graph-eligible steps of every context of cs: whole rotation periods
// from the multi-step graph Gk (captured at the first phase that needs it),
// the rest -- realignment and remainder -- as single replayed steps of G1.
int graph_steps(StepGraph& G1, StepGraph& Gk, const std::vector<ep_ctx*>& cs, cudaStream_t st, ep_batch* b,
                double dt, int ng, int mode) {
  int s = 0, r;
  auto single = [&]() -> int {
    if (!graph_valid(G1, cs)) return capture_step(G1, cs, st, b, dt);
    return replay_step(G1, cs, st, dt);
  };
  const int P = mode >= 2 ? common_period(cs) : 0;
  if (P >= 2 && ng >= P) {
    if (graph_valid(Gk, cs))
      while (s < ng && !at_phase(Gk, cs)) {
        if ((r = single())) return r;
        ++s;
      }
    if (ng - s >= P) {
      if (!graph_valid(Gk, cs) || !at_phase(Gk, cs)) {
        if ((r = capture_steps(Gk, cs, st, b, dt, P))) return r;
        s += P;
      }
      for (; ng - s >= P; s += P)
        if ((r = replay_steps(Gk, cs, st))) return r;
    }
  }
  for (; s < ng; ++s)
    if ((r = single())) return r;
  return EP_OK;
}

}  // namespace

namespace {

// The engine of precision T of c, created on first use.
template <class T> Engine<T>*& engine_slot(ep_ctx* c);
template <> Engine<double>*& engine_slot<double>(ep_ctx* c) { return c->e64; }
template <> Engine<float>*& engine_slot<float>(ep_ctx* c) { return c->e32; }
template <> Engine<dfloat>*& engine_slot<dfloat>(ep_ctx* c) { return c->edd; }

// The active engine's state converted into the engine of precision T.
template <class T>
int switch_to(ep_ctx* c, int precision) {
  Engine<T>*& e = engine_slot<T>(c);
  int r;
  if (!e) {
    ep_config cfg = c->cfg;
    cfg.precision = precision;
    e = new Engine<T>();
    if ((r = e->init(cfg, c->st, &c->prof, &c->imp, &c->err))) { e->release(); delete e; e = nullptr; return r; }
  }
  r = dispatch(c, [&](auto& src) -> int {
    typedef typename std::remove_reference<decltype(src)>::type Src;
    if constexpr (std::is_same<Src, Engine<T>>::value) {
      return EP_OK;
    } else {
      int q = src.ensure_materialized();
      return q ? q : e->import_state(src);
    }
  });
  if (r) return r;
  // an FP64-class engine recomputes the impurity field from the tables and
  // the impurity state instead of widening its FP32 copy: a fixed impurity's
  // field is never refreshed, so the refinement sweeps would otherwise carry
  // its FP32 rounding to the end
  if (!std::is_same<T, float>::value && c->cfg.impurity != EP_IMPURITY_NONE && c->imp.have_tables &&
      (r = e->potenimp()))
    return r;
  return EP_OK;
}

}  // namespace

extern "C" {

int ep_config_init(ep_config* c) {
  if (!c) return EP_ERR_INVALID_ARG;
  std::memset(c, 0, sizeof(*c));
  c->nx = c->ny = c->nz = 64;
  c->xmax = c->ymax = c->zmax = 64.0;
  c->npd = 13;
  c->icon = EP_ICON_ZERO_OUTSIDE;
  c->core = EP_CORE_OT;
  c->cp4 = -2.41186e4;
  c->cpp4 = 1.85850e6;
  c->den4c = 0.062;
  c->alphas = 54.31;
  c->l = 1.0;
  c->den0s = 0.04;
  c->h2o2m4 = 6.05969638298;
  c->C = 3.1577504e4;
  c->beta = 40.0;
  c->den_m = 0.37;
  c->h4ot = 2.190323;
  c->h4op = 2.359665;
  c->eps4 = 10.22;
  c->sigma4 = 2.556;
  c->b4 = -718.99;
  c->time_mode = EP_IMAGINARY_TIME;
  c->renormalize = 1;
  c->n4 = 300.0;
  c->impurity = EP_IMPURITY_NONE;
  c->mimpur = 0.0;
  c->fix_lambda = 0;
  c->als_p = 0.0;
  c->ev0 = 0.0;
  c->z_exciplex_exclusion = 0.0;
  c->precision = EP_FP64;
  c->device = 0;
  c->state = EP_STATE_P;
  c->als_d = 0.0;
  c->filter_exciplex_force = 0;
  return EP_OK;
}

const char* ep_create_error(void) { return g_create_error.c_str(); }

int ep_create(const ep_config* cfg, ep_ctx** out) {
  g_create_error.clear();
  if (!cfg || !out) { g_create_error = "null argument"; return EP_ERR_INVALID_ARG; }
  *out = nullptr;
  const ep_config& c = *cfg;
  if (c.nx % 2 || c.ny % 2 || c.nz % 2 || !factor235(c.nx) || !factor235(c.ny) || !factor235(c.nz)) {
    g_create_error = "grid sizes must be even with prime factors 2, 3, 5 only";
    return EP_ERR_BAD_GRID;
  }
  if (c.npd < 3 || c.npd > 25 || c.npd % 2 == 0) { g_create_error = "npd must be odd, 3..25"; return EP_ERR_INVALID_ARG; }
  if (c.npd > 13) { g_create_error = "stencils wider than 13 points are not built"; return EP_ERR_UNSUPPORTED; }
  if (c.nx < c.npd || c.ny < c.npd || c.nz < c.npd) { g_create_error = "grid smaller than the stencil"; return EP_ERR_BAD_GRID; }
  if (c.icon != EP_ICON_PERIODIC && c.icon != EP_ICON_ZERO_OUTSIDE) {
    g_create_error = "icon must be 8 (periodic) or 13 (zero outside)";
    return EP_ERR_UNSUPPORTED;
  }
  if (c.core != EP_CORE_OT && c.core != EP_CORE_OTC && c.core != EP_CORE_OP) { g_create_error = "unknown core"; return EP_ERR_INVALID_ARG; }
  if (c.impurity == EP_IMPURITY_MOVING && !(c.mimpur > 0.0)) {
    g_create_error = "a moving impurity needs mimpur > 0";
    return EP_ERR_INVALID_ARG;
  }
  if (c.precision != EP_FP64 && c.precision != EP_FP32 && c.precision != EP_DFLOAT) {
    g_create_error = "unknown precision";
    return EP_ERR_INVALID_ARG;
  }
  if (c.state != EP_STATE_P && c.state != EP_STATE_D) { g_create_error = "state must be P or D"; return EP_ERR_INVALID_ARG; }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    g_create_error = "no CUDA device visible";
    return EP_ERR_NO_DEVICE;
  }
  if (c.device < 0 || c.device >= ndev) { g_create_error = "device ordinal out of range"; return EP_ERR_INVALID_ARG; }
  if (cudaSetDevice(c.device) != cudaSuccess) { g_create_error = "cudaSetDevice failed"; return EP_ERR_CUDA; }
  ep_ctx* x = new ep_ctx();
  x->cfg = c;
  if (cudaStreamCreateWithFlags(&x->st, cudaStreamNonBlocking) != cudaSuccess) {
    g_create_error = "stream creation failed";
    delete x;
    return EP_ERR_CUDA;
  }
  int r;
  x->active = c.precision;
  if (c.precision == EP_FP64) {
    x->e64 = new Engine<double>();
    r = x->e64->init(c, x->st, &x->prof, &x->imp, &x->err);
  } else if (c.precision == EP_DFLOAT) {
    x->edd = new Engine<dfloat>();
    r = x->edd->init(c, x->st, &x->prof, &x->imp, &x->err);
  } else {
    x->e32 = new Engine<float>();
    r = x->e32->init(c, x->st, &x->prof, &x->imp, &x->err);
  }
  if (r) {
    g_create_error = x->err;
    ep_destroy(x);
    return r;
  }
  *out = x;
  return EP_OK;
}

int ep_destroy(ep_ctx* c) {
  if (!c) return EP_ERR_INVALID_ARG;
  cudaSetDevice(c->cfg.device);
  if (c->st) cudaStreamSynchronize(c->st);
  c->graph.reset();
  c->graphk.reset();
  if (c->e64) { c->e64->release(); delete c->e64; }
  if (c->e32) { c->e32->release(); delete c->e32; }
  if (c->edd) { c->edd->release(); delete c->edd; }
  if (c->imp.d_potpi) cudaFree(c->imp.d_potpi);
  if (c->imp.d_potdel) cudaFree(c->imp.d_potdel);
  if (c->imp.d_potsigdel) cudaFree(c->imp.d_potsigdel);
  if (c->imp.d_potpi_f) cudaFree(c->imp.d_potpi_f);
  if (c->imp.d_potdel_f) cudaFree(c->imp.d_potdel_f);
  c->prof.release();
  for (cudaEvent_t e : c->ev)
    if (e) cudaEventDestroy(e);
  if (c->st) cudaStreamDestroy(c->st);
  delete c;
  return EP_OK;
}

const char* ep_last_error(const ep_ctx* c) { return c ? c->err.c_str() : "null context"; }

int ep_potential_values(const ep_potential* p, const double* r, double* v, int n) {
  if (!p || (n > 0 && (!r || !v)) || n < 0 || bad_potential(p)) return EP_ERR_INVALID_ARG;
  for (int i = 0; i < n; ++i) v[i] = select_pot(*p, r[i]);
  return EP_OK;
}

// potenimpini (potenimpini.f90:11-58), P state.
int ep_set_impurity_potentials(ep_ctx* c, const ep_potential* pi, const ep_potential* sigma, const ep_potential* plus) {
  if (!c || !pi || !sigma) return EP_ERR_INVALID_ARG;
  if (c->cfg.state != EP_STATE_P) return fail(c, EP_ERR_STATE, "D state: use ep_set_impurity_potentials_d");
  for (const ep_potential* q : {pi, sigma, plus})
    if (q && bad_potential(q)) return fail(c, EP_ERR_INVALID_ARG, bad_potential(q));
  const ep_config& g = c->cfg;
  const int npot = 100 * std::max(g.nx, std::max(g.ny, g.nz)) + 1;
  const double rmax = 4.0 * std::max(g.xmax, std::max(g.ymax, g.zmax));
  const double del = rmax / (double)(npot - 1);
  std::vector<double> tp(npot + 2), td(npot + 2);
  for (int i = 1; i <= npot; ++i) {
    const double r = (double)(i - 1) * del;
    const double a = select_pot(*pi, r);
    tp[i] = a;
    td[i] = select_pot(*sigma, r) - a;
  }
  tp[0] = tp[1]; tp[npot + 1] = tp[npot];
  td[0] = td[1]; td[npot + 1] = td[npot];
  if (plus) keep_plus(c->imp, plus);
  return ep_set_impurity_tables(c, tp.data(), td.data(), npot, del, sigma->umax);
}

// Replaces the device tables (d_potpi, d_potdel, d_potsigdel) by tabs[0..2]
// (NULL: none) of npot + 2 entries each.
static int upload_tables(ep_ctx* c, const double* const tabs[3], int npot) {
  cudaSetDevice(c->cfg.device);
  double** dst[3] = {&c->imp.d_potpi, &c->imp.d_potdel, &c->imp.d_potsigdel};
  for (double** d : dst) {
    if (*d) cudaFree(*d);
    *d = nullptr;
  }
  float** dstf[2] = {&c->imp.d_potpi_f, &c->imp.d_potdel_f};
  for (float** d : dstf) {
    if (*d) cudaFree(*d);
    *d = nullptr;
  }
  c->imp.have_tables = false;
  const size_t n = (size_t)(npot + 2) * sizeof(double);
  for (int i = 0; i < 3; ++i) {
    if (!tabs[i]) continue;
    if (cudaMalloc((void**)dst[i], n) != cudaSuccess) {
      cudaGetLastError();
      *dst[i] = nullptr;
      return fail(c, EP_ERR_OOM, "table allocation failed");
    }
    cudaMemcpyAsync(*dst[i], tabs[i], n, cudaMemcpyHostToDevice, c->st);
  }
  // P state: FP32 copies for the FP32 engine's field evaluation
  std::vector<float> tf((size_t)npot + 2);
  for (int i = 0; i < 2 && c->cfg.state == EP_STATE_P; ++i) {
    for (size_t k = 0; k < tf.size(); ++k) tf[k] = (float)tabs[i][k];
    if (cudaMalloc((void**)dstf[i], tf.size() * sizeof(float)) != cudaSuccess) {
      cudaGetLastError();
      *dstf[i] = nullptr;
      return fail(c, EP_ERR_OOM, "table allocation failed");
    }
    if (cudaMemcpy(*dstf[i], tf.data(), tf.size() * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess)
      return fail(c, EP_ERR_CUDA, "table upload failed");
  }
  if (cudaStreamSynchronize(c->st) != cudaSuccess) return fail(c, EP_ERR_CUDA, "table upload failed");
  return EP_OK;
}

int ep_set_impurity_tables(ep_ctx* c, const double* potpi, const double* potdel, int npot, double delinter,
                           double umax_sigma) {
  if (!c || !potpi || !potdel || npot < 3 || !(delinter > 0)) return EP_ERR_INVALID_ARG;
  if (c->cfg.state != EP_STATE_P) return fail(c, EP_ERR_STATE, "D state: use ep_set_impurity_tables_d");
  const double* tabs[3] = {potpi, potdel, nullptr};
  int r = upload_tables(c, tabs, npot);
  if (r) return r;
  c->imp.npot = npot;
  c->imp.delinter = delinter;
  c->imp.umax_sigma = umax_sigma;
  c->imp.have_tables = true;
  return EP_OK;
}

// potenimpini.f90:28-50, D state: V_Delta, V_Pi - V_Delta, V_Sigma - V_Delta
// on r_i = (i-1)*delinter, end points repeated.
int ep_set_impurity_potentials_d(ep_ctx* c, const ep_potential* pi, const ep_potential* sigma,
                                 const ep_potential* delta, const ep_potential* plus) {
  if (!c || !pi || !sigma || !delta) return EP_ERR_INVALID_ARG;
  if (c->cfg.state != EP_STATE_D) return fail(c, EP_ERR_STATE, "D-state potentials need state = EP_STATE_D");
  for (const ep_potential* q : {pi, sigma, delta, plus})
    if (q && bad_potential(q)) return fail(c, EP_ERR_INVALID_ARG, bad_potential(q));
  const ep_config& g = c->cfg;
  const int npot = 100 * std::max(g.nx, std::max(g.ny, g.nz)) + 1;
  const double rmax = 4.0 * std::max(g.xmax, std::max(g.ymax, g.zmax));
  const double del = rmax / (double)(npot - 1);
  std::vector<double> td(npot + 2), tpd(npot + 2), tsd(npot + 2);
  for (int i = 1; i <= npot; ++i) {
    const double r = (double)(i - 1) * del;
    const double aux = select_pot(*delta, r);
    td[i] = aux;
    tpd[i] = select_pot(*pi, r) - aux;
    tsd[i] = select_pot(*sigma, r) - aux;
  }
  td[0] = td[1]; td[npot + 1] = td[npot];
  tpd[0] = tpd[1]; tpd[npot + 1] = tpd[npot];
  tsd[0] = tsd[1]; tsd[npot + 1] = tsd[npot];
  if (plus) keep_plus(c->imp, plus);
  return ep_set_impurity_tables_d(c, td.data(), tpd.data(), tsd.data(), npot, del, pi->umax, sigma->umax);
}

int ep_set_impurity_tables_d(ep_ctx* c, const double* potdel, const double* potpidel, const double* potsigdel,
                             int npot, double delinter, double umax_pi, double umax_sigma) {
  if (!c || !potdel || !potpidel || !potsigdel || npot < 3 || !(delinter > 0)) return EP_ERR_INVALID_ARG;
  if (c->cfg.state != EP_STATE_D) return fail(c, EP_ERR_STATE, "D-state tables need state = EP_STATE_D");
  const double* tabs[3] = {potpidel, potdel, potsigdel};
  int r = upload_tables(c, tabs, npot);
  if (r) return r;
  c->imp.npot = npot;
  c->imp.delinter = delinter;
  c->imp.umax_pi = umax_pi;
  c->imp.umax_sigma = umax_sigma;
  c->imp.have_tables = true;
  return EP_OK;
}

int ep_set_impurity_state(ep_ctx* c, const double* rimp, const double* vimp, const double* invar) {
  if (!c) return EP_ERR_INVALID_ARG;
  for (int i = 0; i < 3; ++i) {
    if (rimp) c->imp.rimp[i] = rimp[i];
    if (vimp) c->imp.vimp[i] = vimp[i];
  }
  if (invar)
    for (int i = 0; i < 10; ++i) c->imp.invar[i] = std::complex<double>(invar[2 * i], invar[2 * i + 1]);
  return EP_OK;
}

int ep_get_impurity_state(ep_ctx* c, double* rimp, double* vimp, double* aimp, double* invar) {
  if (!c) return EP_ERR_INVALID_ARG;
  for (int i = 0; i < 3; ++i) {
    if (rimp) rimp[i] = c->imp.rimp[i];
    if (vimp) vimp[i] = c->imp.vimp[i];
    if (aimp) aimp[i] = c->imp.aimp[i];
  }
  if (invar)
    for (int i = 0; i < 10; ++i) { invar[2 * i] = c->imp.invar[i].real(); invar[2 * i + 1] = c->imp.invar[i].imag(); }
  return EP_OK;
}

int ep_upload_psi(ep_ctx* c, const double* psi) {
  if (!c || !psi) return EP_ERR_INVALID_ARG;
  return dispatch(c, [&](auto& e) -> int { return e.upload_psi(psi); });
}
int ep_download_psi(ep_ctx* c, double* psi) {
  if (!c || !psi) return EP_ERR_INVALID_ARG;
  return dispatch(c, [&](auto& e) -> int { return e.download_c(EP_CFIELD_PSI, psi); });
}
int ep_download_cfield(ep_ctx* c, int which, double* out) {
  if (!c || !out) return EP_ERR_INVALID_ARG;
  return dispatch(c, [&](auto& e) -> int { return e.download_c(which, out); });
}
int ep_download_field(ep_ctx* c, int which, double* out) {
  if (!c || !out) return EP_ERR_INVALID_ARG;
  return dispatch(c, [&](auto& e) -> int { return e.download_r(which, out); });
}

int ep_potenimp(ep_ctx* c) {
  return dispatch(c, [&](auto& e) -> int {
    int r = e.ensure_materialized();
    if (r) return r;
    r = e.potenimp();
    return r ? r : e.check_flags();
  });
}
int ep_poten(ep_ctx* c) {
  return dispatch(c, [&](auto& e) -> int {
    int r = e.ensure_materialized();
    if (r) return r;
    r = e.poten();
    return r ? r : e.check_flags();
  });
}
int ep_energy(ep_ctx* c, ep_energies* out) {
  if (!out) return EP_ERR_INVALID_ARG;
  return dispatch(c, [&](auto& e) -> int { return e.energy(out); });
}
int ep_forceimp(ep_ctx* c, double* F) {
  if (!F) return EP_ERR_INVALID_ARG;
  const int r = dispatch(c, [&](auto& e) -> int {
    int q = e.ensure_materialized();
    return q ? q : e.forceimp(F);
  });
  // every reference call site follows forceimp with aimp = F / mAg_u
  // (DFT4He3d.f90:454-455, steppc.f90:114-115, steprk.f90:169-170)
  if (!r && c->cfg.impurity == EP_IMPURITY_MOVING) {
    const double m = c->cfg.mimpur * 0.0207569277;
    for (int i = 0; i < 3; ++i) c->imp.aimp[i] = F[i] / m;
  }
  return r;
}
int ep_impurity_moments(ep_ctx* c, double* v6) {
  if (!v6) return EP_ERR_INVALID_ARG;
  return dispatch(c, [&](auto& e) -> int {
    double F[3];
    int r = e.ensure_materialized();
    if (!r) r = e.forceimp(F);
    if (!r) r = e.moments(v6);
    return r;
  });
}

int ep_impurity_matrix_d(ep_ctx* c, double* m25) {
  if (!m25) return EP_ERR_INVALID_ARG;
  return dispatch(c, [&](auto& e) -> int {
    double F[3];
    int r = e.ensure_materialized();
    if (!r) r = e.forceimp(F);
    if (!r) r = e.matrix_d(m25);
    return r;
  });
}

int ep_potinvar(ep_ctx* c, double* hinvar) {
  if (!hinvar) return EP_ERR_INVALID_ARG;
  return dispatch(c, [&](auto& e) -> int {
    double F[3];
    int r = e.ensure_materialized();
    if (r) return r;
    r = e.forceimp(F);
    if (r) return r;
    std::complex<double> H[10];
    r = e.potinvar(H);
    for (int i = 0; i < 10; ++i) { hinvar[2 * i] = H[i].real(); hinvar[2 * i + 1] = H[i].imag(); }
    return r;
  });
}
int ep_steprk(ep_ctx* c, double dt) {
  return dispatch(c, [&](auto& e) -> int { return e.steprk(dt); });
}
int ep_steppc(ep_ctx* c, double dt, ep_step_errors* err) {
  return dispatch(c, [&](auto& e) -> int { return e.steppc(dt, err); });
}

int ep_run(ep_ctx* c, int nsteps, double dt, ep_run_stats* stats) {
  if (!c || nsteps < 0) return EP_ERR_INVALID_ARG;
  const bool renorm = c->cfg.time_mode == EP_IMAGINARY_TIME && c->cfg.renormalize;
  int s0 = 0;
  const int ng = nsteps - (stats ? 1 : 0);  // steps that need no host statistics
  if (ng >= 2 && graph_eligible(c)) {
    std::vector<ep_ctx*> one{c};
    int r;
    if ((r = graph_steps(c->graph, c->graphk, one, c->st, nullptr, dt, ng, c->use_graphs))) return r;
    s0 = ng;
  }
  return dispatch(c, [&](auto& e) -> int {
    ep_step_errors se{};
    for (int s = s0; s < nsteps; ++s) {
      const bool last = (s == nsteps - 1) && stats;
      int r = e.steppc(dt, last ? &se : nullptr);
      if (r) return r;
    }
    (void)renorm;
    if (stats) {
      stats->errHe = se.errHe;
      stats->mu = e.last_mu;
      stats->norm = e.last_norm;
      stats->steps_done = nsteps;
      return e.check_flags();
    }
    return EP_OK;
  });
}

int ep_renormalize(ep_ctx* c, double* norm_before) {
  return dispatch(c, [&](auto& e) -> int { return e.renormalize(norm_before, true); });
}

int ep_set_precision(ep_ctx* c, int precision) {
  if (!c || (precision != EP_FP64 && precision != EP_FP32 && precision != EP_DFLOAT)) return EP_ERR_INVALID_ARG;
  if (precision == c->active) return EP_OK;
  cudaSetDevice(c->cfg.device);
  const int r = precision == EP_FP64   ? switch_to<double>(c, precision)
                : precision == EP_FP32 ? switch_to<float>(c, precision)
                                       : switch_to<dfloat>(c, precision);
  if (r) return r;
  c->active = precision;
  c->cfg.precision = precision;
  return EP_OK;
}

int ep_get_precision(const ep_ctx* c) { return c ? c->active : -1; }

// ---------------------------------------------------------------------------
// Batches.
int ep_batch_create(const ep_config* cfgs, int n, ep_batch** out) {
  if (!cfgs || n < 1 || !out) return EP_ERR_INVALID_ARG;
  *out = nullptr;
  ep_batch* b = new ep_batch();
  b->device = cfgs[0].device;
  for (int i = 0; i < n; ++i) {
    if (cfgs[i].device != b->device) { g_create_error = "a batch lives on one device"; ep_batch_destroy(b); return EP_ERR_INVALID_ARG; }
    ep_ctx* c = nullptr;
    int r = ep_create(&cfgs[i], &c);
    if (r) { ep_batch_destroy(b); return r; }
    b->ctx.push_back(c);
  }
  cudaSetDevice(b->device);
  if (cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess) {
    g_create_error = "batch stream creation failed";
    ep_batch_destroy(b);
    return EP_ERR_CUDA;
  }
  b->join.resize(n);
  for (int i = 0; i < n; ++i) cudaEventCreateWithFlags(&b->join[i], cudaEventDisableTiming);
  *out = b;
  return EP_OK;
}

int ep_batch_destroy(ep_batch* b) {
  if (!b) return EP_ERR_INVALID_ARG;
  if (b->st) cudaStreamSynchronize(b->st);
  b->graph.reset();
  b->graphk.reset();
  for (ep_ctx* c : b->ctx) ep_destroy(c);
  cudaSetDevice(b->device);
  for (cudaEvent_t e : b->join) if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : b->ev) if (e) cudaEventDestroy(e);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->st) cudaStreamDestroy(b->st);
  delete b;
  return EP_OK;
}

int ep_batch_size(const ep_batch* b) { return b ? (int)b->ctx.size() : 0; }

ep_ctx* ep_batch_ctx(ep_batch* b, int i) {
  if (!b || i < 0 || i >= (int)b->ctx.size()) return nullptr;
  return b->ctx[i];
}

int ep_batch_run(ep_batch* b, int nsteps, double dt, ep_run_stats* stats) {
  if (!b || nsteps < 0) return EP_ERR_INVALID_ARG;
  cudaSetDevice(b->device);
  batch_join(b);  // work the caller left on the instance streams comes first
  int s0 = 0;
  const int ng = nsteps - (stats ? 1 : 0);
  bool eligible = b->use_graphs > 0 && ng >= 2;
  for (ep_ctx* c : b->ctx) eligible = eligible && graph_eligible(c);
  if (eligible) {
    int r;
    if ((r = graph_steps(b->graph, b->graphk, b->ctx, b->st, b, dt, ng, b->use_graphs))) return r;
    s0 = ng;
  }
  batch_fork(b);
  // step-major interleaving so the instances' kernels overlap
  for (int s = s0; s < nsteps; ++s) {
    const bool last = (s == nsteps - 1) && stats;
    for (size_t i = 0; i < b->ctx.size(); ++i) {
      ep_ctx* c = b->ctx[i];
      const bool renorm = c->cfg.time_mode == EP_IMAGINARY_TIME && c->cfg.renormalize;
      ep_step_errors se{};
      int r = dispatch(c, [&](auto& e) -> int {
        int q = e.steppc(dt, last ? &se : nullptr);
        if (q) return q;
        (void)renorm;
        if (last) {
          stats[i].errHe = se.errHe;
          stats[i].mu = e.last_mu;
          stats[i].norm = e.last_norm;
          stats[i].steps_done = nsteps;
        }
        return EP_OK;
      });
      if (r) return r;
    }
  }
  batch_join(b);
  if (stats) {
    if (cudaStreamSynchronize(b->st) != cudaSuccess) return EP_ERR_CUDA;
    for (ep_ctx* c : b->ctx) {
      int r = dispatch(c, [&](auto& e) -> int { return e.check_flags(); });
      if (r) return r;
    }
  }
  return EP_OK;
}

// The instances' Runge-Kutta steps are enqueued on their streams first and
// checked afterwards, so that they overlap on the GPU; an instance with a
// moving impurity reads its force every stage and runs on its own.
int ep_batch_steprk(ep_batch* b, double dt) {
  if (!b) return EP_ERR_INVALID_ARG;
  cudaSetDevice(b->device);
  std::vector<char> queued(b->ctx.size(), 0);
  for (size_t i = 0; i < b->ctx.size(); ++i) {
    ep_ctx* c = b->ctx[i];
    const bool mov = c->cfg.impurity == EP_IMPURITY_MOVING;
    int r = dispatch(c, [&](auto& e) -> int { return e.steprk(dt, mov); });
    if (r) return r;
    queued[i] = !mov;
  }
  for (size_t i = 0; i < b->ctx.size(); ++i) {
    if (!queued[i]) continue;
    int r = dispatch(b->ctx[i], [&](auto& e) -> int { return e.check_flags(); });
    if (r) return r;
  }
  return EP_OK;
}

int ep_batch_set_precision(ep_batch* b, int precision) {
  if (!b) return EP_ERR_INVALID_ARG;
  for (ep_ctx* c : b->ctx) {
    int r = ep_set_precision(c, precision);
    if (r) return r;
  }
  return EP_OK;
}

int ep_batch_synchronize(ep_batch* b) {
  if (!b) return EP_ERR_INVALID_ARG;
  for (ep_ctx* c : b->ctx)
    if (cudaStreamSynchronize(c->st) != cudaSuccess) return EP_ERR_CUDA;
  return cudaStreamSynchronize(b->st) == cudaSuccess ? EP_OK : EP_ERR_CUDA;
}

int ep_batch_event_record(ep_batch* b, int slot) {
  if (!b || slot < 0 || slot >= 16) return EP_ERR_INVALID_ARG;
  cudaSetDevice(b->device);
  if (!b->ev[slot] && cudaEventCreate(&b->ev[slot]) != cudaSuccess) return EP_ERR_CUDA;
  batch_join(b);
  return cudaEventRecord(b->ev[slot], b->st) == cudaSuccess ? EP_OK : EP_ERR_CUDA;
}

int ep_batch_event_elapsed(ep_batch* b, int a, int c, double* ms) {
  if (!b || !ms || a < 0 || a >= 16 || c < 0 || c >= 16 || !b->ev[a] || !b->ev[c]) return EP_ERR_INVALID_ARG;
  if (cudaEventSynchronize(b->ev[c]) != cudaSuccess) return EP_ERR_CUDA;
  float t = 0.f;
  if (cudaEventElapsedTime(&t, b->ev[a], b->ev[c]) != cudaSuccess) return EP_ERR_CUDA;
  *ms = t;
  return EP_OK;
}

long long ep_batch_kernel_launches(const ep_batch* b) {
  long long n = 0;
  if (b)
    for (ep_ctx* c : b->ctx) n += c->prof.launches;
  return n;
}

}  // extern "C"

namespace {
template <class E>
void shapes_out(const E& e, int* s) {
  s[0] = e.shp.xnl[0]; s[1] = e.shp.xthr[0]; s[2] = e.shp.ylt; s[3] = e.shp.ythr; s[4] = e.shp.zlt; s[5] = e.shp.zthr;
}
bool shapes_ok(const int* s) {
  auto pow2 = [](int v) { return v >= 1 && v <= 64 && (v & (v - 1)) == 0; };
  auto thr = [](int v) { return v >= 32 && v <= 1024 && v % 32 == 0; };
  return s[0] >= 1 && s[0] <= 64 && thr(s[1]) && pow2(s[2]) && thr(s[3]) && pow2(s[4]) && thr(s[5]);
}
}  // namespace

extern "C" {

int ep_autotune(ep_ctx* c, char* report, int cap) {
  return dispatch(c, [&](auto& e) -> int {
    std::string rep;
    int r = e.autotune(&rep);
    if (report && cap > 0) {
      std::strncpy(report, rep.c_str(), (size_t)cap - 1);
      report[cap - 1] = 0;
    }
    return r;
  });
}

int ep_get_launch_shapes(const ep_ctx* c, int* s) {
  if (!c || !s) return EP_ERR_INVALID_ARG;
  return dispatch(const_cast<ep_ctx*>(c), [&](auto& e) -> int {
    shapes_out(e, s);
    return EP_OK;
  });
}

int ep_set_launch_shapes(ep_ctx* c, const int* s) {
  if (!c || !s || !shapes_ok(s)) return EP_ERR_INVALID_ARG;
  Shapes sh;
  for (int k = 0; k < 4; ++k) { sh.xnl[k] = s[0]; sh.xthr[k] = s[1]; }
  sh.ylt = s[2]; sh.ythr = s[3]; sh.zlt = s[4]; sh.zthr = s[5];
  return dispatch(c, [&](auto& e) -> int {
    e.shp = sh;
    ++e.shapes_gen;
    return EP_OK;
  });
}

int ep_batch_autotune(ep_batch* b) {
  if (!b) return EP_ERR_INVALID_ARG;
  std::vector<int> done(b->ctx.size(), 0);
  for (size_t i = 0; i < b->ctx.size(); ++i) {
    if (done[i]) continue;
    int r = ep_autotune(b->ctx[i], nullptr, 0);
    if (r) return r;
    // the tuned shapes (every X kernel's own) go to the instances of the same
    // grid and precision
    ep_ctx* ci_ = b->ctx[i];
    const ep_config& ci = ci_->cfg;
    for (size_t j = i; j < b->ctx.size(); ++j) {
      ep_ctx* cj_ = b->ctx[j];
      const ep_config& cj = cj_->cfg;
      if (cj.nx == ci.nx && cj.ny == ci.ny && cj.nz == ci.nz && cj_->active == ci_->active) {
        if (j != i) {
          if (ci_->active == EP_FP64 && ci_->e64 && cj_->e64) { cj_->e64->shp = ci_->e64->shp; ++cj_->e64->shapes_gen; }
          if (ci_->active == EP_FP32 && ci_->e32 && cj_->e32) { cj_->e32->shp = ci_->e32->shp; ++cj_->e32->shapes_gen; }
          if (ci_->active == EP_DFLOAT && ci_->edd && cj_->edd) { cj_->edd->shp = ci_->edd->shp; ++cj_->edd->shapes_gen; }
        }
        done[j] = 1;
      }
    }
  }
  return EP_OK;
}

int ep_synchronize(ep_ctx* c) {
  if (!c) return EP_ERR_INVALID_ARG;
  if (cudaStreamSynchronize(c->st) != cudaSuccess) return fail(c, EP_ERR_CUDA, cudaGetErrorString(cudaGetLastError()));
  return EP_OK;
}

void* ep_stream(ep_ctx* c) { return c ? (void*)c->st : nullptr; }

int ep_event_record(ep_ctx* c, int slot) {
  if (!c || slot < 0 || slot >= 16) return EP_ERR_INVALID_ARG;
  if (!c->ev[slot] && cudaEventCreate(&c->ev[slot]) != cudaSuccess) return fail(c, EP_ERR_CUDA, "event create");
  if (cudaEventRecord(c->ev[slot], c->st) != cudaSuccess) return fail(c, EP_ERR_CUDA, "event record");
  return EP_OK;
}

int ep_event_elapsed(ep_ctx* c, int a, int b, double* ms) {
  if (!c || !ms || a < 0 || a >= 16 || b < 0 || b >= 16 || !c->ev[a] || !c->ev[b]) return EP_ERR_INVALID_ARG;
  if (cudaEventSynchronize(c->ev[b]) != cudaSuccess) return fail(c, EP_ERR_CUDA, "event sync");
  float t = 0.f;
  if (cudaEventElapsedTime(&t, c->ev[a], c->ev[b]) != cudaSuccess) return fail(c, EP_ERR_CUDA, "event elapsed");
  *ms = t;
  return EP_OK;
}

long long ep_kernel_launches(const ep_ctx* c) { return c ? c->prof.launches : 0; }

int ep_set_step_graphs(ep_ctx* c, int on) {
  if (!c) return EP_ERR_INVALID_ARG;
  c->use_graphs = on < 0 ? 0 : on > 2 ? 2 : on;
  return EP_OK;
}

int ep_batch_set_step_graphs(ep_batch* b, int on) {
  if (!b) return EP_ERR_INVALID_ARG;
  b->use_graphs = on < 0 ? 0 : on > 2 ? 2 : on;
  for (ep_ctx* c : b->ctx) c->use_graphs = b->use_graphs;
  return EP_OK;
}

int ep_profile_enable(ep_ctx* c, int on) {
  if (!c) return EP_ERR_INVALID_ARG;
  c->prof.collect();
  c->prof.on = on != 0;
  return EP_OK;
}

int ep_profile_read(ep_ctx* c, char* names, int cap, double* ms, long long* launches, int maxn, int* n) {
  if (!c || !n) return EP_ERR_INVALID_ARG;
  c->prof.collect();
  const int k = (int)c->prof.names.size();
  *n = k;
  int off = 0;
  for (int i = 0; i < k && i < maxn; ++i) {
    if (ms) ms[i] = c->prof.ms[i];
    if (launches) launches[i] = c->prof.cnt[i];
    if (names) {
      const std::string& s = c->prof.names[i];
      if (off + (int)s.size() + 1 <= cap) {
        std::memcpy(names + off, s.c_str(), s.size() + 1);
        off += (int)s.size() + 1;
      }
    }
  }
  for (int i = 0; i < k; ++i) { c->prof.ms[i] = 0.0; c->prof.cnt[i] = 0; }
  return EP_OK;
}

long long ep_device_bytes(const ep_ctx* c) {
  if (!c) return 0;
  return (c->e64 ? c->e64->bytes : 0) + (c->e32 ? c->e32->bytes : 0) + (c->edd ? c->edd->bytes : 0);
}

}  // extern "C"
