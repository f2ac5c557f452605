// ep_engine.h - host-side engine of one solver instance in one precision.
#pragma once
#include <cuda_runtime.h>

#include <complex>
#include <string>
#include <utility>
#include <vector>

#include "../../include/eff_pot.h"
#include "ep_common.cuh"
#include "ep_kernels.cuh"

// Launch accounting and optional per-class event timing.
struct Prof {
  long long launches = 0;
  bool on = false;
  std::vector<std::string> names;
  std::vector<double> ms;
  std::vector<long long> cnt;
  struct Rec { int cls; cudaEvent_t a, b; };
  std::vector<Rec> pending;
  std::vector<cudaEvent_t> pool;
  int cls(const char* name);
  cudaEvent_t ev();
  void begin(cudaStream_t st, const char* name, cudaEvent_t& a, int& c);
  void end(cudaStream_t st, int c, cudaEvent_t a);
  void collect();
  void release();
};

// Small-vector state of the classical impurity and the internal variables
// (module classicimp; the steppc/steprk history arrays).
struct ImpState {
  double rimp[3] = {0, 0, 0}, vimp[3] = {0, 0, 0}, aimp[3] = {0, 0, 0};
  std::complex<double> invar[10], hinvar[10];
  double qr[3] = {0, 0, 0}, qv[3] = {0, 0, 0};
  double rimpold[3][3] = {}, vimpold[3][3] = {}, aimpold[3][2] = {};
  int ioldr[3] = {0, 1, 2}, ioldv[3] = {0, 1, 2}, iolda[2] = {0, 1}, ioldiv[3] = {0, 1, 2}, ioldhiv[2] = {0, 1};
  double pcr[3] = {0, 0, 0}, pcv[3] = {0, 0, 0};
  std::complex<double> qiv[10], invarold[10][3], hinvarold[10][2], pciv[10];
  // interpolation tables (module interpol), FP64 on the device
  // P state: d_potpi = V_Pi, d_potdel = V_Sigma - V_Pi.  D state:
  // d_potdel = V_Delta, d_potpi = V_Pi - V_Delta, d_potsigdel = V_Sigma - V_Delta.
  int npot = 0;
  double delinter = 0, umax_sigma = 9.674836e3, umax_pi = 0.0;
  double* d_potpi = nullptr;
  double* d_potdel = nullptr;
  double* d_potsigdel = nullptr;
  // P state: FP32 copies of d_potpi, d_potdel for the FP32 engine
  float* d_potpi_f = nullptr;
  float* d_potdel_f = nullptr;
  ep_potential plus{};  // series pointer cleared: the fit lives in plus_series
  ep_series plus_series{};
  bool have_tables = false;
};

// Launch shapes of the FFT passes (lines per CTA and threads per CTA),
// chosen by Engine::autotune.
struct Shapes {
  int xnl[4] = {16, 16, 16, 16}, xthr[4] = {256, 256, 256, 256};  // X1..X4: x-lines per CTA, threads
  int ylt = 16, ythr = 256;  // Y passes (shared-memory engine)
  int zlt = 16, zthr = 256;  // Z convolution passes (shared-memory engine)
};

template <class T>
class Engine {
 public:
  Shapes shp;
  typedef C2<T> CT;
  ep_config cfg{};
  Geo g{};
  double hx = 0, hy = 0, hz = 0, dxyz = 0;
  cudaStream_t st = nullptr;
  Prof* prof = nullptr;
  ImpState* imp = nullptr;
  std::string* err = nullptr;
  int dev_sm = 0;
  int zc_pc = 16, zc_pr = 16, zc_rk = 16, zc_d1 = 16;  // z planes per CTA of the stencil marches
  // predictor / corrector form: 0 one point per thread, 1 two points per
  // thread staged by cp.async (FP32, even R and nx), 2 the same staged by TMA
  // boxes (also nx % 64 == 0 and ny % 8 == 0)
  int pmode = 0;
  // TMA boxes of each rotating complex buffer ({128 x R}, {128 x EP_TYT},
  // {16 x R}, {16 x EP_TYT} floats x rows) and of pot4 / uimp
  // ({64 x EP_TYT})
  struct BufMaps {
    const void* buf;
    CUtensorMap m[4];
  };
  std::vector<BufMaps> cmaps;
  bool tma_timeout_test = false;  // EP_TEST_TMA_TIMEOUT=1: every TMA wait runs out
  CUtensorMap rmaps[2];
  int build_march_maps();
  const CUtensorMap* maps_of(const void* buf) const;
  bool march_maps(MarchMaps& mm, const CT* marched, const CT* const* cin, int nc) const;
  T* dyz = nullptr;                         // dy(gy) + dz(gz) of term_alfa
  T* sigdel = nullptr;                      // Sig_Del of the D state (vpi holds Pi_Del)
  int d1march(int mode, const T* f, const T* f2, T* o0, T* o1, T* o2);
  int moments(double* v6);
  int matrix_d(double* m25);
  // Step graphs (CUDA-graph replay of steppc): while capturing, cap_nodes
  // receives the predictor / corrector nodes; while replaying, upd_exec is the
  // executable graph whose nodes lap_predict / lap_correct update.
  std::pair<cudaGraphNode_t, cudaGraphNode_t>* cap_nodes = nullptr;
  cudaGraphExec_t upd_exec = nullptr;
  cudaGraphNode_t upd_pred = nullptr, upd_corr = nullptr;
  int shapes_gen = 0;  // bumped whenever launch shapes change (invalidates graphs)
  int launch_march(const void* fn, dim3 grid, dim3 blk, size_t smem, void** args, const char* name, int which);
  int steppc_update(double dt, cudaGraphExec_t x, cudaGraphNode_t np, cudaGraphNode_t nc);
  bool graph_ok() const { return cfg.impurity != EP_IMPURITY_MOVING && !prof->on; }
  // Multi-step graphs.  The buffers the next steppc's predictor and corrector
  // read and write (psi, spare, psiold in age order, hpsiold in age order),
  // the steps after which they repeat, and the host half of one steppc with
  // a fixed (or no) impurity -- the buffer rotation of lap_predict and
  // lap_correct, nothing launched -- applied for each step of a replayed
  // multi-step graph.
  void step_signature(const void* (&sig)[7]) const {
    sig[0] = psi; sig[1] = spare;
    sig[2] = po[ioldp[0]]; sig[3] = po[ioldp[1]]; sig[4] = po[ioldp[2]];
    sig[5] = ph[ioldh[0]]; sig[6] = ph[ioldh[1]];
  }
  void rotate_step() {
    std::swap(psi, po[ioldp[2]]);
    std::swap(ioldh[0], ioldh[1]);
    std::swap(psi, spare);
    const int t = ioldp[2];
    ioldp[2] = ioldp[1];
    ioldp[1] = ioldp[0];
    ioldp[0] = t;
    if (cfg.time_mode == EP_IMAGINARY_TIME && cfg.renormalize) lazy = true;
  }
  int rotation_period() const {
    Engine<T> e;  // host copy of the rotation state only
    e.cfg = cfg;
    e.psi = psi; e.spare = spare;
    for (int k = 0; k < 3; ++k) { e.po[k] = po[k]; e.ioldp[k] = ioldp[k]; }
    for (int k = 0; k < 2; ++k) { e.ph[k] = ph[k]; e.ioldh[k] = ioldh[k]; }
    const void* s0[7];
    step_signature(s0);
    for (int n = 1; n <= 64; ++n) {
      e.rotate_step();
      const void* s[7];
      e.step_signature(s);
      bool same = true;
      for (int k = 0; k < 7; ++k) same = same && s[k] == s0[k];
      if (same) return n;
    }
    return 0;
  }
  int march_zchunk(int blocks_per_sm, int tile_x = EP_TX, int tile_y = EP_TY) const;
  // kernel attributes (dynamic shared memory) and the march z-chunk lengths,
  // set up by init
  int x_attrs();
  int fft_attrs();
  int x_pass(int which, bool otc);
  template <int N2> int x_launch(int which, bool otc);
  template <int N2> int x_attrs_n2();
  int march_setup();
  long long bytes = 0;
  Phys phys{};
  FdW<T> fd{};

  // state (module rho / rkpc / field)
  CT* psi = nullptr;
  CT* spare = nullptr;
  CT* po[3] = {nullptr, nullptr, nullptr};
  CT* ph[2] = {nullptr, nullptr};
  CT* pc = nullptr;
  CT* q = nullptr;
  int ioldp[3] = {0, 1, 2}, ioldh[2] = {0, 1};
  bool have_field = false;
  // real fields
  T *den = nullptr, *pot4 = nullptr, *uimp = nullptr, *dencg = nullptr, *delj4 = nullptr;
  T *dxd = nullptr, *dyd = nullptr, *dzd = nullptr, *falfs = nullptr, *intx = nullptr, *inty = nullptr,
    *intz = nullptr, *ualphas = nullptr, *gy = nullptr, *gz = nullptr, *dgx = nullptr, *vpi = nullptr,
    *delta = nullptr;
  // spectra and kernels
  CT* S[4] = {nullptr, nullptr, nullptr, nullptr};
  CT* Tb[4] = {nullptr, nullptr, nullptr, nullptr};
  T *fvlj4 = nullptr, *wcgk = nullptr, *kalfs = nullptr;
  CT *twx = nullptr, *twy = nullptr, *twz = nullptr;
  FftPlan p2{}, pY{}, pZ{};
  // reductions
  double* partials = nullptr;
  long long npartials = 0;
  DevScalars* sc = nullptr;
  double last_mu = 0, last_norm = 0;

  int init(const ep_config& c, cudaStream_t s, Prof* p, ImpState* im, std::string* e);
  void release();

  // sub-steps
  int poten();
  int potenimp();
  int energy(ep_energies* out);
  int forceimp(double* F);
  int potinvar(std::complex<double>* H);
  // wait = false: return once the step is enqueued (no stream synchronise,
  // no flag check -- the caller runs check_flags() later); only for an
  // impurity that does not move (a moving one reads its force each stage)
  int steprk(double dt, bool wait = true);
  int steppc(double dt, ep_step_errors* err);
  int renormalize(double* norm_before, bool wait);
  int upload_psi(const double* h);
  int download_c(int which, double* h);
  int download_r(int which, double* h);
  int check_flags();
  int autotune(std::string* report);
  int rescale_pending();
  // Apply the lazy renormalisation scales before host-visible operations.
  int ensure_materialized();
  bool lazy = false;
  CT* slot_base[EP_NSLOTS] = {};

  // precision conversion (the other engine's state -> this one)
  template <class U> int import_state(const Engine<U>& o);

 private:
  int alloc(void** p, size_t n);
  int cuda_ok(cudaError_t e, const char* what);
  int refresh();
  int lap_predict(double dt);
  int lap_correct(double dt, bool want);
  int rk_stage(int jr, double dt);
  int reduce_finalize(int nblocks, int nq, int out0, int mode);
  int read_sums(double* h, int n, int off);
  int fft_y(CT** arrs, int n, int dir);
  template <int N> int rfft_y(const Arr8<T>& a, int n, const LineSet& ls, int dir);
  template <int N> int rfft_z(const ConvSpec<T>& cs, int nin, const LineSet& ls);
  int zconv(const CT* const* in, CT* const (*out)[3], const T* const (*ker)[3], const int* nout, int nin);
  int slot_of(const CT* p) const;
  int x_lines(int which, int nreal) const;
  size_t x_smem(int nl, int nreal) const;
  int l_lines(int n, int nbuf) const;
  size_t l_smem(int LT, int n, int nbuf) const;
};
