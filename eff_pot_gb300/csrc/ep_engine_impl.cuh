// ep_engine_impl.cuh - Engine<T> method bodies (instantiated per precision).
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>

#include "ep_dstate.h"
#include "ep_engine.h"
#include "ep_kernels_impl.cuh"
#include "ep_rfft.cuh"

#define EP_RED_BLOCKS 1216
#define EP_SMEM_CAP (110 * 1024)

#define EP_LAUNCH(name, kern, grid, block, smem, ...)                 \
  do {                                                                \
    cudaEvent_t _a = nullptr;                                         \
    int _c = -1;                                                      \
    prof->begin(st, name, _a, _c);                                    \
    kern<<<grid, block, smem, st>>>(__VA_ARGS__);                     \
    prof->end(st, _c, _a);                                            \
    cudaError_t _e = cudaGetLastError();                              \
    if (_e != cudaSuccess) return cuda_ok(_e, name);                  \
  } while (0)


// Stencil radii built per precision: every npd = 3..13 (R = 1..6) in FP64
// and FP32; in double-float only the 13-point stencils (R = 6: npd = 13, the
// reference default and every benchmark workload), whose kernels are several
// times larger than the FP64 ones.
// Parts of the engine's member definitions: a translation unit that defines
// EP_ENGINE_PARTS compiles only those parts (the large double-float engine
// is built from several units in parallel); the default is all of them.
#define EP_PART_REST 1
#define EP_PART_X 2
#define EP_PART_FFT 4
#define EP_PART_MARCH 8
#define EP_PART_XK 16
#ifndef EP_ENGINE_PARTS
#define EP_ENGINE_PARTS 31
#endif

template <class T> constexpr bool r_built(int R) { return !std::is_same<T, dfloat>::value || R == 6; }
// the two-points-per-thread predictor / corrector: FP32 fields, even R
template <class T> constexpr bool pair_built(int R) { return std::is_same<T, float>::value && R % 2 == 0; }

namespace {

// Planes per CTA of a stencil march over a (gx, gy) grid of column tiles:
// minimise waves x (planes + prologue) over the chunk counts, so that the
// last wave is as full as the SM count allows.
inline int march_chunk(long long nxy, int nz, long long slots, int R) {
  int best = nz;
  long long cost = -1;
  for (int nch = 1; nch <= nz; ++nch) {
    const int zc = (nz + nch - 1) / nch;
    if (zc < 4 && nch > 1) break;
    const long long nblk = nxy * ((nz + zc - 1) / zc);
    const long long waves = (nblk + slots - 1) / slots;
    const long long c = waves * (zc + R);
    if (cost < 0 || c < cost) { cost = c; best = zc; }
  }
  return best;
}

// Central-row weights of the (2R+1)-point stencils (closed forms of the
// Bickley/Lagrange coefficients), at +k.
inline void fd_weights(int R, long double* w1, long double* w2) {
  long double lf[64];
  lf[0] = 0.0L;
  for (int i = 1; i < 64; ++i) lf[i] = lf[i - 1] + logl((long double)i);
  long double c = 0.0L;
  w1[0] = 0.0L;
  for (int k = 1; k <= R; ++k) {
    const long double mag = expl(2.0L * lf[R] - lf[R - k] - lf[R + k]);
    const long double sg = (k & 1) ? 1.0L : -1.0L;
    w1[k] = sg * mag / k;
    w2[k] = 2.0L * sg * mag / ((long double)k * k);
    c -= 2.0L / ((long double)k * k);
  }
  w2[0] = c;
}

template <class T, class CT>
inline void twiddles(int n, std::vector<CT>& tw) {
  tw.resize(n);
  for (int k = 0; k < n; ++k) {
    const long double a = -2.0L * 3.141592653589793238462643383279502884L * k / n;
    tw[k].x = (T)(double)cosl(a);
    tw[k].y = (T)(double)sinl(a);
  }
}

}  // namespace

#if EP_ENGINE_PARTS & EP_PART_REST
template <class T>
int Engine<T>::cuda_ok(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return EP_OK;
  if (err) *err = std::string(what) + ": " + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? EP_ERR_OOM : EP_ERR_CUDA;
}

template <class T>
int Engine<T>::alloc(void** p, size_t n) {
  cudaError_t e = cudaMalloc(p, n);
  if (e != cudaSuccess) {
    *p = nullptr;
    cudaGetLastError();
    if (err) *err = "device allocation of " + std::to_string(n) + " bytes failed";
    return EP_ERR_OOM;
  }
  bytes += (long long)n;
  return EP_OK;
}

template <class T>
size_t Engine<T>::x_smem(int nl, int nreal) const {
  return x_smem_bytes<T>(nl, g.nx, nreal);
}
template <class T>
int Engine<T>::x_lines(int which, int nreal) const {
  int nl = shp.xnl[which];
  while (nl > 1 && x_smem(nl, nreal) > EP_SMEM_CAP) nl /= 2;
  return nl;
}
template <class T>
size_t Engine<T>::l_smem(int LT, int n, int nbuf) const {
  return (size_t)nbuf * LT * (n + 1) * sizeof(CT) + (size_t)n * sizeof(CT) + (size_t)LT * sizeof(long long);
}
template <class T>
int Engine<T>::l_lines(int n, int nbuf) const {
  int LT = nbuf == 3 ? shp.zlt : shp.ylt;
  while (LT > 1 && l_smem(LT, n, nbuf) > EP_SMEM_CAP) LT /= 2;
  return LT;
}

template <class T>
int Engine<T>::init(const ep_config& c, cudaStream_t s, Prof* p, ImpState* im, std::string* e) {
  cfg = c;
  st = s;
  prof = p;
  imp = im;
  err = e;
  if (!r_built<T>(c.npd / 2)) {
    *err = "double-float fields are built for npd = 13 only";
    return EP_ERR_UNSUPPORTED;
  }
  g.nx = c.nx; g.ny = c.ny; g.nz = c.nz; g.nxh = c.nx / 2 + 1;
  g.N = (long long)c.nx * c.ny * c.nz;
  g.Nh = (long long)g.nxh * c.ny * c.nz;
  hx = 2.0 * std::fabs(c.xmax) / c.nx;
  hy = 2.0 * std::fabs(c.ymax) / c.ny;
  hz = 2.0 * std::fabs(c.zmax) / c.nz;
  dxyz = hx * hy * hz;
  if (!make_plan(c.nx / 2, p2) || !make_plan(c.ny, pY) || !make_plan(c.nz, pZ)) {
    *err = "grid sizes must factor into 2, 3 and 5";
    return EP_ERR_BAD_GRID;
  }
  // finite-difference weights scaled by 1/h^id (Deriv3D_p Sto = 1/h**id)
  const int R = c.npd / 2;
  long double w1[EP_MAX_R + 1], w2[EP_MAX_R + 1];
  fd_weights(R, w1, w2);
  FdW<T> fdl{};
  const double hh[3] = {hx, hy, hz};
  for (int a = 0; a < 3; ++a) {
    const double s1 = 1.0 / hh[a], s2 = 1.0 / (hh[a] * hh[a]);
    for (int k = 0; k <= R; ++k) {
      fdl.w1[a][k] = (T)((double)w1[k] * s1);
      fdl.w2[a][k] = (T)((double)w2[k] * s2);
    }
  }
  fdl.R = R;
  fdl.periodic = (c.icon == EP_ICON_PERIODIC) ? 1 : 0;
  fd = fdl;
  Phys phl{};
  phl.cp4 = c.cp4; phl.cpp4 = c.cpp4; phl.a0 = c.cp4 / 2.0; phl.a1 = c.cpp4 / 3.0;
  phl.den0s = c.den0s; phl.h2o2m4 = c.h2o2m4; phl.alphas = c.alphas;
  phl.C = c.C; phl.beta = c.beta; phl.den_m = c.den_m;
  phl.renor = 1.0 / ((double)c.nx * c.ny * c.nz);
  phl.dxyz = dxyz;
  phl.core = c.core;
  phl.time_mode = c.time_mode;
  phl.rden0s = 1.0 / c.den0s;
  phl.f = PhysF{(float)phl.cp4, (float)phl.cpp4, (float)phl.a0, (float)phl.a1, (float)phl.rden0s,
                (float)phl.h2o2m4, (float)phl.alphas, (float)phl.C, (float)phl.beta, (float)phl.den_m,
                (float)phl.renor};
  phl.d = PhysD{dfloat(phl.cp4), dfloat(phl.cpp4), dfloat(phl.a0), dfloat(phl.a1), dfloat(phl.rden0s),
                dfloat(phl.h2o2m4), dfloat(phl.alphas), dfloat(phl.C), dfloat(phl.beta), dfloat(phl.den_m),
                dfloat(phl.renor)};
  phys = phl;

  const size_t N = (size_t)g.N, Nh = (size_t)g.Nh;
  int r;
  CT** cbufs[] = {&psi, &spare, &po[0], &po[1], &po[2], &ph[0], &ph[1], &pc, &q};
  for (CT** b : cbufs) if ((r = alloc((void**)b, N * sizeof(CT)))) return r;
  T** rbufs[] = {&den, &pot4, &uimp, &dencg, &delj4, &dxd, &dyd, &dzd, &falfs, &intx, &inty, &intz,
                 &ualphas, &gy, &gz, &dgx, &vpi, &delta, &dyz};
  for (T** b : rbufs) if ((r = alloc((void**)b, N * sizeof(T)))) return r;
  if (c.state == EP_STATE_D && (r = alloc((void**)&sigdel, N * sizeof(T)))) return r;
  for (int i = 0; i < 4; ++i) {
    if ((r = alloc((void**)&S[i], Nh * sizeof(CT)))) return r;
    if ((r = alloc((void**)&Tb[i], Nh * sizeof(CT)))) return r;
  }
  T** kbufs[] = {&fvlj4, &wcgk, &kalfs};
  for (T** b : kbufs) if ((r = alloc((void**)b, Nh * sizeof(T)))) return r;
  if ((r = alloc((void**)&twx, c.nx * sizeof(CT)))) return r;
  if ((r = alloc((void**)&twy, c.ny * sizeof(CT)))) return r;
  if ((r = alloc((void**)&twz, c.nz * sizeof(CT)))) return r;
  if ((r = alloc((void**)&sc, sizeof(DevScalars)))) return r;

  {
    CT* sb[EP_NSLOTS] = {psi, spare, po[0], po[1], po[2], ph[0], ph[1], pc};
    for (int k = 0; k < EP_NSLOTS; ++k) slot_base[k] = sb[k];
  }
  for (CT** b : cbufs) if ((r = cuda_ok(cudaMemsetAsync(*b, 0, N * sizeof(CT), st), "memset"))) return r;
  for (T** b : rbufs) if ((r = cuda_ok(cudaMemsetAsync(*b, 0, N * sizeof(T), st), "memset"))) return r;
  if ((r = cuda_ok(cudaMemsetAsync(sc, 0, sizeof(DevScalars), st), "memset"))) return r;
  {
    auto kr = k_reset_scales;
    EP_LAUNCH("reset_scales", kr, 1, 32, 0, sc);
  }

  std::vector<CT> tw;
  twiddles<T>(c.nx, tw);
  cudaMemcpyAsync(twx, tw.data(), c.nx * sizeof(CT), cudaMemcpyHostToDevice, st);
  cudaStreamSynchronize(st);
  twiddles<T>(c.ny, tw);
  cudaMemcpyAsync(twy, tw.data(), c.ny * sizeof(CT), cudaMemcpyHostToDevice, st);
  cudaStreamSynchronize(st);
  twiddles<T>(c.nz, tw);
  cudaMemcpyAsync(twz, tw.data(), c.nz * sizeof(CT), cudaMemcpyHostToDevice, st);
  cudaStreamSynchronize(st);

  // FFT-ordered momentum grid (DFT4He3d.f90:213-219,266-300).
  {
    const int nx = c.nx, ny = c.ny, nz = c.nz;
    const double hpx = 1.0 / (nx * hx), hpy = 1.0 / (ny * hy), hpz = 1.0 / (nz * hz);
    const double pmx = 1.0 / (2.0 * hx), pmy = 1.0 / (2.0 * hy), pmz = 1.0 / (2.0 * hz);
    std::vector<double> pg(nx + ny + nz);
    for (int i = 1; i <= nx / 2 + 1; ++i) pg[i - 1] = hpx * (i - 1);
    for (int i = nx / 2 + 2; i <= nx; ++i) pg[i - 1] = -pmx + hpx * (i - (nx / 2 + 1));
    for (int i = 1; i <= ny / 2 + 1; ++i) pg[nx + i - 1] = hpy * (i - 1);
    for (int i = ny / 2 + 2; i <= ny; ++i) pg[nx + i - 1] = -pmy + hpy * (i - (ny / 2 + 1));
    for (int i = 1; i <= nz / 2 + 1; ++i) pg[nx + ny + i - 1] = hpz * (i - 1);
    for (int i = nz / 2 + 2; i <= nz; ++i) pg[nx + ny + i - 1] = -pmz + hpz * (i - (nz / 2 + 1));
    double* dpg = nullptr;
    if ((r = cuda_ok(cudaMalloc((void**)&dpg, pg.size() * sizeof(double)), "pgrid"))) return r;
    cudaMemcpyAsync(dpg, pg.data(), pg.size() * sizeof(double), cudaMemcpyHostToDevice, st);
    const double h4 = (c.core == EP_CORE_OP) ? c.h4op : c.h4ot;
    // bforce (fforma.f90:256-280)
    const double pi4 = 4.0 * 3.14159265358979323846, eps4 = 4.0 * c.eps4;
    const double xx = std::pow(c.sigma4 / h4, 6), v0 = xx * (xx - 1.0) / std::pow(h4, 4);
    const double s6 = std::pow(c.sigma4, 6), s12 = s6 * s6;
    double bf = pi4 * eps4 * s12 / (9.0 * std::pow(h4, 9)) - pi4 * eps4 * s6 / (3.0 * std::pow(h4, 3));
    if (c.core == EP_CORE_OP) bf += pi4 * eps4 * (v0 * std::pow(h4, 7)) / 7.0;
    auto kf = k_formfactors<T>;
    EP_LAUNCH("formfactors", kf, 4 * 152, 256, 0, g, dpg, dpg + nx, dpg + nx + ny, c.core, h4, c.eps4, c.sigma4,
              bf, c.l, fvlj4, wcgk, kalfs);
    cudaStreamSynchronize(st);
    cudaFree(dpg);
  }
  {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&dev_sm, cudaDevAttrMultiProcessorCount, dev);
    if (dev_sm <= 0) dev_sm = 152;
  }
  if ((r = x_attrs()) || (r = fft_attrs()) || (r = march_setup())) return r;
  {
    const long long nxy = (long long)((c.nx + EP_TX - 1) / EP_TX) * ((c.ny + EP_TY - 1) / EP_TY);
    const long long nxy2 = (long long)((c.nx + EP_PX - 1) / EP_PX) * ((c.ny + EP_TY - 1) / EP_TY);
    const int zmin = std::min(std::min(zc_pc, zc_pr), zc_rk);
    const long long nbs = std::max(nxy, nxy2) * ((c.nz + zmin - 1) / zmin);
    // block partials are compensated (hi, lo) pairs: the hi parts of a
    // reduction's nblocks*nq sums, then their lo parts
    npartials = 2 * std::max(nbs * 4, (long long)EP_RED_BLOCKS * 18);
    if ((r = alloc((void**)&partials, npartials * sizeof(double)))) return r;
  }
  return cuda_ok(cudaStreamSynchronize(st), "init");
}

template <class T>
int Engine<T>::march_zchunk(int blocks_per_sm, int tile_x, int tile_y) const {
  const long long nxy = (long long)((g.nx + tile_x - 1) / tile_x) * ((g.ny + tile_y - 1) / tile_y);
  const long long slots = (long long)dev_sm * std::max(1, blocks_per_sm);
  return march_chunk(nxy, g.nz, slots, fd.R);
}

template <class T>
void Engine<T>::release() {
  void* bufs[] = {psi, spare, po[0], po[1], po[2], ph[0], ph[1], pc, q, den, pot4, uimp, dencg, delj4, dxd, dyd,
                  dzd, falfs, intx, inty, intz, ualphas, gy, gz, dgx, vpi, delta, dyz, S[0], S[1], S[2], S[3], Tb[0],
                  Tb[1], Tb[2], Tb[3], fvlj4, wcgk, kalfs, twx, twy, twz, partials, sc, sigdel};
  for (void* b : bufs)
    if (b) cudaFree(b);
  sigdel = nullptr;
  psi = nullptr;
  bytes = 0;
}

// ---------------------------------------------------------------------------
// Register-resident transforms (ep_rfft.cuh) of lines of length N.
#endif
#if EP_ENGINE_PARTS & EP_PART_FFT
template <class T>
template <int N>
int Engine<T>::rfft_y(const Arr8<T>& a, int n, const LineSet& ls, int dir) {
  dim3 grid((unsigned)((ls.nlines + 31) / 32), (unsigned)n), blk(32, rfft::Shape<N>::P);
  const size_t sm = rfft::smem_bytes<T, N>();
  if (dir < 0) {
    auto k = k_c2c_r<T, N, -1>;
    EP_LAUNCH("fft_y_fwd", k, grid, blk, sm, a, ls, twy);
  } else {
    auto k = k_c2c_r<T, N, +1>;
    EP_LAUNCH("fft_y_inv", k, grid, blk, sm, a, ls, twy);
  }
  return EP_OK;
}

template <class T>
template <int N>
int Engine<T>::rfft_z(const ConvSpec<T>& cs, int nin, const LineSet& ls) {
  dim3 grid((unsigned)((ls.nlines + 31) / 32), (unsigned)nin), blk(32, rfft::Shape<N>::P);
  bool one = true;
  for (int i = 0; i < nin; ++i) one = one && cs.nout[i] == 1;
  if (one) {
    auto k = k_zconv_r<T, N, true>;
    EP_LAUNCH("fft_z_conv", k, grid, blk, (rfft::conv_smem_bytes<T, N, true>()), cs, ls, twz);
  } else {
    auto k = k_zconv_r<T, N, false>;
    EP_LAUNCH("fft_z_conv", k, grid, blk, (rfft::conv_smem_bytes<T, N, false>()), cs, ls, twz);
  }
  return EP_OK;
}

template <class T>
int Engine<T>::fft_y(CT** arrs, int n, int dir) {
  Arr8<T> a{};
  for (int i = 0; i < n; ++i) a.a[i] = arrs[i];
  LineSet ls{(long long)g.nxh, (long long)g.nxh * g.ny, (long long)g.nxh, (long long)g.nxh * g.nz};
  switch (g.ny) {
    case 32: return rfft_y<32>(a, n, ls, dir);
    case 64: return rfft_y<64>(a, n, ls, dir);
    case 128: return rfft_y<128>(a, n, ls, dir);
    case 256: return rfft_y<256>(a, n, ls, dir);
    case 96: if constexpr (sizeof(T) == 4) return rfft_y<96>(a, n, ls, dir); break;
    case 192: if constexpr (sizeof(T) == 4) return rfft_y<192>(a, n, ls, dir); break;
    default: break;
  }
  const int LT = l_lines(g.ny, 2);
  dim3 grid((unsigned)((ls.nlines + LT - 1) / LT), (unsigned)n);
  const size_t sm = l_smem(LT, g.ny, 2);
  if (dir < 0) {
    auto k = k_c2c<T, -1>;
    EP_LAUNCH("fft_y_fwd", k, grid, shp.ythr, sm, a, ls, pY, twy, LT);
  } else {
    auto k = k_c2c<T, +1>;
    EP_LAUNCH("fft_y_inv", k, grid, shp.ythr, sm, a, ls, pY, twy, LT);
  }
  return EP_OK;
}

template <class T>
int Engine<T>::zconv(const CT* const* in, CT* const (*out)[3], const T* const (*ker)[3], const int* nout, int nin) {
  ConvSpec<T> cs{};
  for (int i = 0; i < nin; ++i) {
    cs.in[i] = in[i];
    cs.nout[i] = nout[i];
    for (int j = 0; j < nout[i]; ++j) { cs.out[i][j] = out[i][j]; cs.ker[i][j] = ker[i][j]; }
  }
  LineSet ls{(long long)g.nxh * g.ny, 0, (long long)g.nxh * g.ny, (long long)g.nxh * g.ny};
  switch (g.nz) {
    case 32: return rfft_z<32>(cs, nin, ls);
    case 64: return rfft_z<64>(cs, nin, ls);
    case 128: return rfft_z<128>(cs, nin, ls);
    case 256: return rfft_z<256>(cs, nin, ls);
    case 96: if constexpr (sizeof(T) == 4) return rfft_z<96>(cs, nin, ls); break;
    case 192: if constexpr (sizeof(T) == 4) return rfft_z<192>(cs, nin, ls); break;
    default: break;
  }
  const int LT = l_lines(g.nz, 3);
  dim3 grid((unsigned)((ls.nlines + LT - 1) / LT), (unsigned)nin);
  auto k = k_zconv<T>;
  EP_LAUNCH("fft_z_conv", k, grid, shp.zthr, l_smem(LT, g.nz, 3), cs, ls, pZ, twz, LT);
  return EP_OK;
}

// First-derivative marches (k_d1march): mode 0 = grad f, mode 1 = dy f + dz f2.
#endif
#if EP_ENGINE_PARTS & EP_PART_MARCH
template <class T>
int Engine<T>::d1march(int mode, const T* f, const T* f2, T* o0, T* o1, T* o2) {
  dim3 grid((g.nx + EP_D1_TX - 1) / EP_D1_TX, (g.ny + EP_TY - 1) / EP_TY, (g.nz + zc_d1 - 1) / zc_d1);
  dim3 blk(EP_TX, EP_TY);
#define EP_D1(RR)                                                                                  \
  case RR:                                                                                         \
    if constexpr (!r_built<T>(RR)) {                                                               \
      *err = "double-float fields are built for npd = 13 only";                                    \
      return EP_ERR_UNSUPPORTED;                                                                   \
    } else if (mode == 0) {                                                                        \
      auto k = k_d1march<T, RR, 0>;                                                                \
      EP_LAUNCH("grad_march", k, grid, blk, 0, g, fd, zc_d1, f, f2, o0, o1, o2);                  \
    } else {                                                                                       \
      auto k = k_d1march<T, RR, 1>;                                                                \
      EP_LAUNCH("div_march", k, grid, blk, 0, g, fd, zc_d1, f, f2, o0, o1, o2);                   \
    }                                                                                              \
    break;
  switch (fd.R) {
    EP_D1(1) EP_D1(2) EP_D1(3) EP_D1(4) EP_D1(5) EP_D1(6)
    default: *err = "npd > 13 not built"; return EP_ERR_UNSUPPORTED;
  }
#undef EP_D1
  return EP_OK;
}

// poten() + derden() + term_alfa() (poten.f90:5-131, term_alfa.f90:5-109).
#endif
#if EP_ENGINE_PARTS & EP_PART_X
template <class T>
int Engine<T>::poten() {
  const bool otc = cfg.core == EP_CORE_OTC;
  const bool grad = otc || cfg.impurity != EP_IMPURITY_NONE;
  int r;
  if ((r = x_pass(1, otc))) return r;
  if (grad && (r = d1march(0, den, nullptr, dxd, dyd, dzd))) return r;
  CT* a1[1] = {S[0]};
  if ((r = fft_y(a1, 1, -1))) return r;
  {
    const CT* in[1] = {S[0]};
    CT* const out[1][3] = {{Tb[0], Tb[1], Tb[2]}};
    const T* const ker[1][3] = {{wcgk, fvlj4, kalfs}};
    const int no[1] = {otc ? 3 : 2};
    if ((r = zconv(in, out, ker, no, 1))) return r;
  }
  CT* b3[3] = {Tb[0], Tb[1], Tb[2]};
  if ((r = fft_y(b3, otc ? 3 : 2, +1))) return r;
  if ((r = x_pass(2, otc))) return r;
  CT* c4[4] = {S[0], S[1], S[2], S[3]};
  if ((r = fft_y(c4, otc ? 4 : 1, -1))) return r;
  {
    const CT* in[4] = {S[0], S[1], S[2], S[3]};
    CT* const out[4][3] = {{Tb[0]}, {Tb[1]}, {Tb[2]}, {Tb[3]}};
    const T* const ker[4][3] = {{wcgk}, {kalfs}, {kalfs}, {kalfs}};
    const int no[4] = {1, 1, 1, 1};
    if ((r = zconv(in, out, ker, no, otc ? 4 : 1))) return r;
  }
  CT* d4[4] = {Tb[0], Tb[1], Tb[2], Tb[3]};
  if ((r = fft_y(d4, otc ? 4 : 1, +1))) return r;
  if ((r = x_pass(3, otc))) return r;
  if (otc) {
    if ((r = d1march(1, gy, gz, dyz, nullptr, nullptr))) return r;
    if ((r = fft_y(a1, 1, -1))) return r;
    const CT* in[1] = {S[0]};
    CT* const out[1][3] = {{Tb[0]}};
    const T* const ker[1][3] = {{kalfs}};
    const int no[1] = {1};
    if ((r = zconv(in, out, ker, no, 1))) return r;
    CT* e1[1] = {Tb[0]};
    if ((r = fft_y(e1, 1, +1))) return r;
    if ((r = x_pass(4, otc))) return r;
  }
  have_field = true;
  return EP_OK;
}

#endif
#if EP_ENGINE_PARTS & EP_PART_REST
template <class T>
int Engine<T>::potenimp() {
  if (cfg.impurity == EP_IMPURITY_NONE) return cuda_ok(cudaMemsetAsync(uimp, 0, g.N * sizeof(T), st), "uimp");
  if (!imp->have_tables) {
    *err = "impurity tables not set";
    return EP_ERR_STATE;
  }
  const double rmax = (imp->npot - 1) * imp->delinter;
  if (cfg.state == EP_STATE_D) {
    // Re G_ij of the internal variables for the per-point quadratic form
    DGram G{};
    int k = 0;
    for (int i = 0; i < 5; ++i)
      for (int j = i; j < 5; ++j, ++k) {
        const std::complex<double> gij = std::conj(imp->invar[2 * i]) * imp->invar[2 * j] +
                                         std::conj(imp->invar[2 * i + 1]) * imp->invar[2 * j + 1];
        G.g[k] = (i == j ? 1.0 : 2.0) * gij.real();
      }
    auto kd = k_potenimp_d<T>;
    EP_LAUNCH("potenimp", kd, 4 * 152, 256, 0, g, cfg.xmax, cfg.ymax, cfg.zmax, hx, hy, hz, imp->rimp[0],
              imp->rimp[1], imp->rimp[2], imp->d_potdel, imp->d_potpi, imp->d_potsigdel, imp->npot, rmax,
              imp->umax_pi, imp->umax_sigma, G, delta, vpi, sigdel, uimp);
    return EP_OK;
  }
  if constexpr (sizeof(T) == 4) {
    if (imp->d_potpi_f) {
      float2 fv[6];
      for (int i = 0; i < 6; ++i) fv[i] = make_float2((float)imp->invar[i].real(), (float)imp->invar[i].imag());
      const double h = rmax / (imp->npot - 1);
      auto kf = k_potenimp_f;
      EP_LAUNCH("potenimp", kf, 4 * 152, 256, 0, g, (float)cfg.xmax, (float)cfg.ymax, (float)cfg.zmax, (float)hx,
                (float)hy, (float)hz, (float)imp->rimp[0], (float)imp->rimp[1], (float)imp->rimp[2], imp->d_potpi_f,
                imp->d_potdel_f, imp->npot, (float)h, (float)(1.0 / h), (float)imp->umax_sigma, fv[0], fv[1], fv[2],
                fv[3], fv[4], fv[5], vpi, delta, uimp);
      return EP_OK;
    }
  }
  double2 iv[6];
  for (int i = 0; i < 6; ++i) iv[i] = make_double2(imp->invar[i].real(), imp->invar[i].imag());
  auto k = k_potenimp<T>;
  EP_LAUNCH("potenimp", k, 4 * 152, 256, 0, g, cfg.xmax, cfg.ymax, cfg.zmax, hx, hy, hz, imp->rimp[0],
            imp->rimp[1], imp->rimp[2], imp->d_potpi, imp->d_potdel, imp->npot, rmax, imp->umax_sigma, iv[0], iv[1],
            iv[2], iv[3], iv[4], iv[5], vpi, delta, uimp);
  return EP_OK;
}

template <class T>
int Engine<T>::reduce_finalize(int nblocks, int nq, int out0, int mode) {
  auto k = k_finalize;
  const int renorm = (cfg.time_mode == EP_IMAGINARY_TIME && cfg.renormalize) ? 1 : 0;
  EP_LAUNCH("finalize", k, 1, 256, 0, partials, nblocks, nq, sc, out0, mode, (double)g.N, dxyz, cfg.n4, renorm);
  return EP_OK;
}

template <class T>
int Engine<T>::read_sums(double* h, int n, int off) {
  int r = cuda_ok(cudaMemcpyAsync(h, sc->sums + off, n * sizeof(double), cudaMemcpyDeviceToHost, st), "read sums");
  if (r) return r;
  return cuda_ok(cudaStreamSynchronize(st), "read sums");
}

template <class T>
int Engine<T>::energy(ep_energies* e) {
  if (!have_field) { *err = "poten() must run before energy()"; return EP_ERR_STATE; }
  int r0 = ensure_materialized();
  if (r0) return r0;
  PotDev vp{};
  vp.kind = imp->plus.kind;
  vp.r_cutoff = imp->plus.r_cutoff;
  vp.umax = imp->plus.umax;
  for (int i = 0; i < 4; ++i) vp.par[i] = imp->plus.par[i];
  vp.s = imp->plus_series;
  auto k = k_energy<T>;
  EP_LAUNCH("energy", k, EP_RED_BLOCKS, 256, 0, g, fd, phys, psi, den, dencg, delj4, falfs, dxd, dyd, dzd, intx,
            inty, intz, uimp, cfg.xmax, cfg.ymax, cfg.zmax, hx, hy, hz, imp->rimp[0], imp->rimp[1], imp->rimp[2],
            cfg.z_exciplex_exclusion, vp, cfg.impurity != EP_IMPURITY_NONE ? 1 : 0, partials);
  int r;
  if ((r = reduce_finalize(EP_RED_BLOCKS, 8, 8, 0))) return r;
  double s[8];
  if ((r = read_sums(s, 8, 8))) return r;
  const ep_config& c = cfg;
  e->ekin4 = c.h2o2m4 * s[0] * dxyz;
  e->elj4 = 0.5 * s[1] * dxyz;
  e->ecor4 = s[2] * dxyz;
  e->ealphas = (c.core == EP_CORE_OTC) ? -c.h2o2m4 * 0.5 * c.alphas * s[3] * dxyz : 0.0;
  e->esolid = c.C * s[4] * dxyz;
  e->etot4 = e->ekin4 + e->elj4 + e->ecor4;
  if (c.core == EP_CORE_OTC) e->etot4 = e->etot4 + e->ealphas;
  const double mAg_u = c.mimpur * 0.0207569277;
  e->ekinx = 0.5 * mAg_u * (imp->vimp[0] * imp->vimp[0] + imp->vimp[1] * imp->vimp[1] + imp->vimp[2] * imp->vimp[2]);
  e->eHeX = s[5] * dxyz;
  e->uplus = s[6] * dxyz;
  const std::complex<double>* iv = imp->invar;
  std::complex<double> ivs[10];
  for (int i = 0; i < 10; ++i) ivs[i] = std::conj(iv[i]);
  if (c.state == EP_STATE_D) {
    // energy.f90:176-190: Als_D * 0.5 * sum_i conj(iv_i) (SOD iv)_i
    std::complex<double> S[10][10];
    dstate::sod(S);
    std::complex<double> vls = 0.0;
    for (int i = 0; i < 10; ++i) {
      std::complex<double> t = 0.0;
      for (int j = 0; j < 10; ++j) t += S[i][j] * iv[j];
      vls += t * ivs[i];
    }
    e->eso = (0.5 * vls * c.als_d).real();
  } else {
    e->eso = 0.5 * c.als_p * (2.0 * (ivs[0] * iv[5] - ivs[1] * iv[4]).real() +
                              2.0 * (ivs[0] * iv[2] + ivs[3] * iv[1] + ivs[2] * iv[5] + ivs[3] * iv[4]).imag());
  }
  e->eimpu = e->ekinx + e->eHeX + e->eso;
  e->etot = e->etot4 + e->eimpu;
  e->n4 = s[7] * dxyz;
  return check_flags();
}

// Planes [lo, hi) of the F_z sum: all of them, or with the exciplex filter
// those beyond z_exciplex_exclusion on the far side of the impurity
// (potenimp.f90:211-248: iz0 / nz0 truncated as Fortran's integer
// assignment does, 1-based there).
inline void fz_planes(const ep_config& c, double rz, double hz, int nz, int& lo, int& hi) {
  lo = 0;
  hi = nz;
  if (!c.filter_exciplex_force) return;
  const double z1 = -c.zmax;
  if (rz < 0.0) {
    const int iz0 = std::max(1, (int)((rz - z1 + c.z_exciplex_exclusion) / hz + 1.5));
    lo = std::min(iz0 - 1, nz);
  } else {
    const int nz0 = std::min(nz, (int)((rz - z1 - c.z_exciplex_exclusion) / hz + 1.5));
    hi = std::max(nz0, 0);
  }
}

template <class T>
int Engine<T>::forceimp(double* F) {
  int izlo, izhi;
  fz_planes(cfg, imp->rimp[2], hz, g.nz, izlo, izhi);
  if (cfg.state == EP_STATE_D) {
    auto kd = k_impmoments_d<T>;
    EP_LAUNCH("impmoments", kd, EP_RED_BLOCKS, 256, 0, g, den, dxd, dyd, dzd, uimp, delta, vpi, sigdel, cfg.xmax,
              cfg.ymax, cfg.zmax, hx, hy, hz, imp->rimp[0], imp->rimp[1], imp->rimp[2], izlo, izhi, partials);
    int r;
    if ((r = reduce_finalize(EP_RED_BLOCKS, 18, 16, 0))) return r;
    double s[3];
    if ((r = read_sums(s, 3, 16))) return r;
    for (int i = 0; i < 3; ++i) F[i] = -s[i] * dxyz;
    return EP_OK;
  }
  if constexpr (sizeof(T) == 4) {
    auto kf = k_impmoments_f;
    EP_LAUNCH("impmoments", kf, EP_RED_BLOCKS, 256, 0, g, den, dxd, dyd, dzd, uimp, vpi, delta, (float)cfg.xmax,
              (float)cfg.ymax, (float)cfg.zmax, (float)hx, (float)hy, (float)hz, (float)imp->rimp[0],
              (float)imp->rimp[1], (float)imp->rimp[2], izlo, izhi, partials);
  } else {
    auto k = k_impmoments<T>;
    EP_LAUNCH("impmoments", k, EP_RED_BLOCKS, 256, 0, g, den, dxd, dyd, dzd, uimp, vpi, delta, cfg.xmax, cfg.ymax,
              cfg.zmax, hx, hy, hz, imp->rimp[0], imp->rimp[1], imp->rimp[2], izlo, izhi, partials);
  }
  int r;
  if ((r = reduce_finalize(EP_RED_BLOCKS, 9, 16, 0))) return r;
  double s[9];
  if ((r = read_sums(s, 9, 16))) return r;
  for (int i = 0; i < 3; ++i) F[i] = -s[i] * dxyz;
  return EP_OK;
}

// (Vx, Vy, Vz, Vxy, Vxz, Vyz) of instates.f90:123-147 from the moments left
// by the last forceimp() call.
template <class T>
int Engine<T>::moments(double* v6) {
  if (cfg.state != EP_STATE_P) { *err = "the six moments belong to the P state"; return EP_ERR_STATE; }
  double s[9];
  int r;
  if ((r = read_sums(s, 9, 16))) return r;
  v6[0] = s[3] * dxyz;
  v6[1] = s[6] * dxyz;
  v6[2] = s[8] * dxyz;
  v6[3] = s[4] * dxyz;
  v6[4] = s[5] * dxyz;
  v6[5] = s[7] * dxyz;
  return EP_OK;
}

// D state: the 5x5 matrix (MP + MS + sumVdel) dxyz of potinvar /
// instates, from the sums left by the last forceimp() call.
template <class T>
int Engine<T>::matrix_d(double* m25) {
  if (cfg.state != EP_STATE_D) { *err = "the D-state matrix needs state = EP_STATE_D"; return EP_ERR_STATE; }
  double s[18];
  int r;
  if ((r = read_sums(s, 18, 16))) return r;
  int k = 3;
  for (int i = 0; i < 5; ++i)
    for (int j = i; j < 5; ++j, ++k) m25[5 * i + j] = m25[5 * j + i] = s[k] * dxyz;
  return EP_OK;
}

// potinvar (potenimp.f90:261-492), from the sums left by the last forceimp()
// call.  D state: Hiv = (M (x) 1_2 + Als_D/2 SOD) iv; P state: the six
// moments and the 6x6 spin-orbit block.  Then -i (Hiv - Ev0 iv).
template <class T>
int Engine<T>::potinvar(std::complex<double>* Hiv) {
  const std::complex<double> uim(0.0, 1.0);
  if (cfg.state == EP_STATE_D) {
    double M[25];
    int r;
    if ((r = matrix_d(M))) return r;
    std::complex<double> S[10][10];
    dstate::sod(S);
    const std::complex<double>* iv = imp->invar;
    for (int i = 0; i < 10; ++i) {
      std::complex<double> h = 0.0;
      for (int j = 0; j < 10; ++j) h += dstate::matdso(M, S, cfg.als_d, i, j) * iv[j];
      Hiv[i] = h;
    }
    for (int i = 0; i < 10; ++i) Hiv[i] = -uim * (Hiv[i] - cfg.ev0 * iv[i]);
    return EP_OK;
  }
  double s[9];
  int r;
  if ((r = read_sums(s, 9, 16))) return r;
  const double uxx = s[3], uxy = s[4], uxz = s[5], uyy = s[6], uyz = s[7], uzz = s[8];
  const std::complex<double>* iv = imp->invar;
  const double A = cfg.als_p / 2.0;
  Hiv[0] = (uxx * iv[0] + uxy * iv[2] + uxz * iv[4]) * dxyz + A * (-uim * iv[2] + iv[5]);
  Hiv[1] = (uxx * iv[1] + uxy * iv[3] + uxz * iv[5]) * dxyz + A * (uim * iv[3] - iv[4]);
  Hiv[2] = (uxy * iv[0] + uyy * iv[2] + uyz * iv[4]) * dxyz + A * (uim * iv[0] - uim * iv[5]);
  Hiv[3] = (uxy * iv[1] + uyy * iv[3] + uyz * iv[5]) * dxyz + A * (-uim * iv[1] - uim * iv[4]);
  Hiv[4] = (uxz * iv[0] + uyz * iv[2] + uzz * iv[4]) * dxyz + A * (-iv[1] + uim * iv[3]);
  Hiv[5] = (uxz * iv[1] + uyz * iv[3] + uzz * iv[5]) * dxyz + A * (iv[0] + uim * iv[2]);
  for (int i = 6; i < 10; ++i) Hiv[i] = 0.0;
  for (int i = 0; i < 10; ++i) Hiv[i] = -uim * (Hiv[i] - cfg.ev0 * iv[i]);
  return EP_OK;
}

template <class T>
int Engine<T>::refresh() {
  const bool mov = cfg.impurity == EP_IMPURITY_MOVING;
  int r;
  if (mov && (r = potenimp())) return r;
  if ((r = poten())) return r;
  if (mov) {
    double F[3];
    if ((r = forceimp(F))) return r;
    const double m = cfg.mimpur * 0.0207569277;
    for (int i = 0; i < 3; ++i) imp->aimp[i] = F[i] / m;
    if (!cfg.fix_lambda && (r = potinvar(imp->hinvar))) return r;
  }
  return EP_OK;
}

// Launch of a stencil-march kernel, or -- while a step graph is replayed --
// an update of its captured node (which = 0 predictor, 1 corrector).  While
// a step is captured the node just recorded is remembered for the updates.
#endif
#if EP_ENGINE_PARTS & EP_PART_MARCH
template <class T>
int Engine<T>::launch_march(const void* fn, dim3 grid, dim3 blk, size_t smem, void** args, const char* name,
                            int which) {
  if (upd_exec) {
    cudaKernelNodeParams p{};
    p.func = const_cast<void*>(fn);
    p.gridDim = grid;
    p.blockDim = blk;
    p.sharedMemBytes = (unsigned)smem;
    p.kernelParams = args;
    p.extra = nullptr;
    return cuda_ok(cudaGraphExecKernelNodeSetParams(upd_exec, which == 0 ? upd_pred : upd_corr, &p), name);
  }
  cudaEvent_t a = nullptr;
  int c = -1;
  prof->begin(st, name, a, c);
  cudaError_t e = cudaLaunchKernel(fn, grid, blk, args, smem, st);
  prof->end(st, c, a);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_ok(e, name);
  if (cap_nodes) {
    cudaStreamCaptureStatus cs;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    e = cudaStreamGetCaptureInfo(st, &cs, nullptr, nullptr, &deps, nullptr, &nd);
    if (e != cudaSuccess) return cuda_ok(e, name);
    if (cs != cudaStreamCaptureStatusActive || nd != 1) {
      *err = "step capture: unexpected dependency set";
      return EP_ERR_CUDA;
    }
    (which == 0 ? cap_nodes->first : cap_nodes->second) = deps[0];
  }
  return EP_OK;
}

template <class T>
int Engine<T>::lap_predict(double dt) {
  const double c112 = 112.0 / 121.0, c4o3 = 4.0 / 3.0;
  CT* po3 = po[ioldp[2]];
  const CT* h1 = ph[ioldh[0]];
  CT* h2 = ph[ioldh[1]];
  const int tile_x = pmode ? EP_PX : EP_TX, tile_y = pmode == 2 ? EP_TYT : EP_TY;
  dim3 grid((g.nx + tile_x - 1) / tile_x, (g.ny + tile_y - 1) / tile_y, (g.nz + zc_pr - 1) / zc_pr);
  dim3 blk(EP_TX, tile_y);
  T f = (T)(c4o3 * dt), c1 = (T)c112;
  Slots sl{slot_of(psi), slot_of(po3), -1, slot_of(h1), slot_of(h2), slot_of(pc), -1};
  const CT* psic = psi;
  const T *pot4c = pot4, *uimpc = uimp;
  int zc = zc_pr;
  NoMaps nomaps{0};
  MarchMaps mm;
  if (pmode == 2) {
    const CT* cin[4] = {po3, h1, h2, pc};
    if (!march_maps(mm, psi, cin, 4)) {
      *err = "predictor: a buffer without tensor maps";
      return EP_ERR_STATE;
    }
  }
  void* args[] = {&g,  &fd, &phys, &zc, &psic, &pot4c, &uimpc, &po3, &h1, &h2,
                  &pc, &den, &f,   &c1, &sc,   &sl,    pmode == 2 ? (void*)&mm : (void*)&nomaps};
  const void* fn = nullptr;
  size_t smem = 0;
#define EP_PRED(RR)                                                                   \
  case RR:                                                                            \
    if constexpr (pair_built<T>(RR)) {                                                \
      if (pmode) {                                                                    \
        fn = pmode == 2 ? (const void*)k_predict<T, RR, 2> : (const void*)k_predict<T, RR, 1>; \
        smem = pmode == 2 ? march_tma_smem<RR, 4, 2>() : march_pair_smem<RR, 4, 2>(); \
        break;                                                                        \
      }                                                                               \
    }                                                                                 \
    if constexpr (r_built<T>(RR)) {                                                   \
      fn = (const void*)k_predict<T, RR, 0>;                                          \
      smem = march_smem<T, RR, 4, 2>();                                               \
    }                                                                                 \
    break;
  switch (fd.R) {
    EP_PRED(1) EP_PRED(2) EP_PRED(3) EP_PRED(4) EP_PRED(5) EP_PRED(6)
    default: *err = "npd > 13 not built"; return EP_ERR_UNSUPPORTED;
  }
#undef EP_PRED
  if (!fn) { *err = "npd not built in this precision"; return EP_ERR_UNSUPPORTED; }
  int r;
  if ((r = launch_march(fn, grid, blk, smem, args, "predict", 0))) return r;
  std::swap(psi, po[ioldp[2]]);
  std::swap(ioldh[0], ioldh[1]);
  return EP_OK;
}

template <class T>
int Engine<T>::lap_correct(double dt, bool want) {
  const double c9 = 9.0 / 121.0;
  const CT* po3 = po[ioldp[2]];
  const CT* po2 = po[ioldp[1]];
  const CT* h1 = ph[ioldh[0]];
  const CT* h2 = ph[ioldh[1]];
  const int tile_x = pmode ? EP_PX : EP_TX, tile_y = pmode == 2 ? EP_TYT : EP_TY;
  dim3 grid((g.nx + tile_x - 1) / tile_x, (g.ny + tile_y - 1) / tile_y, (g.nz + zc_pc - 1) / zc_pc);
  dim3 blk(EP_TX, tile_y);
  T f3 = (T)(3.0 * dt), cc = (T)c9;
  int renorm = (cfg.time_mode == EP_IMAGINARY_TIME && cfg.renormalize) ? 1 : 0;
  Slots sl{slot_of(psi), slot_of(po3), slot_of(po2), slot_of(h1), slot_of(h2), slot_of(pc), slot_of(spare)};
  const CT* psic = psi;
  const T *pot4c = pot4, *uimpc = uimp;
  int zc = zc_pc;
  double n4 = cfg.n4;
  NoMaps nomaps{0};
  MarchMaps mm;
  if (pmode == 2) {
    const CT* cin[5] = {po3, po2, h1, h2, pc};
    if (!march_maps(mm, psi, cin, 5)) {
      *err = "corrector: a buffer without tensor maps";
      return EP_ERR_STATE;
    }
  }
  void* args[] = {&g,  &fd,  &phys, &zc,  &psic, &pot4c, &uimpc,   &po3, &po2, &h1, &h2,
                  &pc, &spare, &den, &f3, &cc,   &partials, &sc,   &renorm, &n4, &sl,
                  pmode == 2 ? (void*)&mm : (void*)&nomaps};
  const void* fn = nullptr;
  size_t smem = 0;
#define EP_CORR(RR)                                                                                   \
  case RR:                                                                                            \
    if constexpr (pair_built<T>(RR)) {                                                                \
      if (pmode == 2) {                                                                               \
        fn = want ? (const void*)k_correct<T, RR, true, 2> : (const void*)k_correct<T, RR, false, 2>; \
        smem = march_tma_smem<RR, 5, 2>();                                                            \
        break;                                                                                        \
      }                                                                                               \
      if (pmode == 1) {                                                                               \
        fn = want ? (const void*)k_correct<T, RR, true, 1> : (const void*)k_correct<T, RR, false, 1>; \
        smem = march_pair_smem<RR, 5, 2>();                                                           \
        break;                                                                                        \
      }                                                                                               \
    }                                                                                                 \
    if constexpr (r_built<T>(RR)) {                                                                   \
      fn = want ? (const void*)k_correct<T, RR, true, 0> : (const void*)k_correct<T, RR, false, 0>;   \
      smem = march_smem<T, RR, 5, 2>();                                                               \
    }                                                                                                 \
    break;
  switch (fd.R) {
    EP_CORR(1) EP_CORR(2) EP_CORR(3) EP_CORR(4) EP_CORR(5) EP_CORR(6)
    default: *err = "npd > 13 not built"; return EP_ERR_UNSUPPORTED;
  }
#undef EP_CORR
  if (!fn) { *err = "npd not built in this precision"; return EP_ERR_UNSUPPORTED; }
  int r;
  if ((r = launch_march(fn, grid, blk, smem, args, "correct", 1))) return r;
  std::swap(psi, spare);
  const int t = ioldp[2];
  ioldp[2] = ioldp[1];
  ioldp[1] = ioldp[0];
  ioldp[0] = t;
  if (renorm) lazy = true;
  return EP_OK;
}

// Host half of one steppc replayed from a step graph (fixed or no impurity):
// the buffer rotation of lap_predict/lap_correct, with the predictor and
// corrector nodes of graph x updated to this step's buffers.  poten() is in
// the graph with fixed buffers.
template <class T>
int Engine<T>::steppc_update(double dt, cudaGraphExec_t x, cudaGraphNode_t np, cudaGraphNode_t nc) {
  upd_exec = x;
  upd_pred = np;
  upd_corr = nc;
  int r = lap_predict(dt);
  if (!r) r = lap_correct(dt, false);
  upd_exec = nullptr;
  return r;
}

template <class T>
int Engine<T>::rk_stage(int jr, double dt) {
  const double s2 = std::sqrt(2.0);
  const double arun[4] = {0.5, 1.0 - 1.0 / s2, 1.0 + 1.0 / s2, 1.0 / 6.0};
  const double brun[4] = {2.0, 1.0, 1.0, 2.0};
  const double crun[4] = {0.5, 1.0 - 1.0 / s2, 1.0 + 1.0 / s2, 0.5};
  CT* out = (jr == 0) ? po[2] : spare;
  CT* hout = (jr == 0) ? ph[1] : nullptr;
  dim3 grid((g.nx + EP_TX - 1) / EP_TX, (g.ny + EP_TY - 1) / EP_TY, (g.nz + zc_rk - 1) / zc_rk);
  dim3 blk(EP_TX, EP_TY);
  const T a = (T)arun[jr], b = (T)brun[jr], cr = (T)crun[jr], d = (T)dt;
#define EP_RK(RR)                                                                                              \
  case RR:                                                                                                     \
    if constexpr (r_built<T>(RR)) {                                                                            \
      auto k = k_rkstage<T, RR>;                                                                               \
      EP_LAUNCH("rkstage", k, grid, blk, (march_smem<T, RR, 1, 2>()), g, fd, phys, zc_rk, psi, pot4, uimp, q, out, \
                hout, den, a, b, cr, d, sc);                                                                   \
    }                                                                                                          \
    break;
  switch (fd.R) {
    EP_RK(1) EP_RK(2) EP_RK(3) EP_RK(4) EP_RK(5) EP_RK(6)
    default: *err = "npd > 13 not built"; return EP_ERR_UNSUPPORTED;
  }
#undef EP_RK
  if (jr == 0) {
    // hpsiold(2) = hpsiold(1); hpsiold(1) = H; psiold(3) = psiold(2);
    // psiold(2) = psiold(1); psiold(1) = psi (steprk.f90:78-84)
    CT* hn = ph[1];
    ph[1] = ph[0];
    ph[0] = hn;
    CT* pn = po[2];
    po[2] = po[1];
    po[1] = po[0];
    po[0] = psi;
    psi = pn;
  } else {
    std::swap(psi, spare);
  }
  return EP_OK;
}

// steprk (steprk.f90:1-191).
#endif
#if EP_ENGINE_PARTS & EP_PART_REST
template <class T>
int Engine<T>::steprk(double dt, bool wait) {
  if (!have_field) { *err = "poten() must run before steprk()"; return EP_ERR_STATE; }
  {
    int r0 = ensure_materialized();
    if (r0) return r0;
  }
  const double s2 = std::sqrt(2.0);
  const double arun[4] = {0.5, 1.0 - 1.0 / s2, 1.0 + 1.0 / s2, 1.0 / 6.0};
  const double brun[4] = {2.0, 1.0, 1.0, 2.0};
  const double crun[4] = {0.5, 1.0 - 1.0 / s2, 1.0 + 1.0 / s2, 0.5};
  const bool mov = cfg.impurity == EP_IMPURITY_MOVING;
  int r;
  for (int jr = 0; jr < 4; ++jr) {
    if ((r = rk_stage(jr, dt))) return r;
    if (mov) {
      ImpState& m = *imp;
      const double a = arun[jr], b = brun[jr], cr = crun[jr];
      for (int k = 0; k < 3; ++k) {
        const double ax = a * (m.vimp[k] - b * m.qr[k]);
        m.qr[k] = m.qr[k] + 3.0 * ax - cr * m.vimp[k];
        if (jr == 0) { m.rimpold[k][2] = m.rimpold[k][1]; m.rimpold[k][1] = m.rimpold[k][0]; m.rimpold[k][0] = m.rimp[k]; }
        m.rimp[k] = m.rimp[k] + dt * ax;
      }
      for (int k = 0; k < 3; ++k) {
        const double ax = a * (m.aimp[k] - b * m.qv[k]);
        m.qv[k] = m.qv[k] + 3.0 * ax - cr * m.aimp[k];
        if (jr == 0) {
          m.aimpold[k][1] = m.aimpold[k][0]; m.aimpold[k][0] = m.aimp[k];
          m.vimpold[k][2] = m.vimpold[k][1]; m.vimpold[k][1] = m.vimpold[k][0]; m.vimpold[k][0] = m.vimp[k];
        }
        m.vimp[k] = m.vimp[k] + dt * ax;
      }
      if (!cfg.fix_lambda) {
        for (int k = 0; k < 10; ++k) {
          const std::complex<double> ax = a * (m.hinvar[k] - b * m.qiv[k]);
          m.qiv[k] = m.qiv[k] + 3.0 * ax - cr * m.hinvar[k];
          if (jr == 0) {
            m.hinvarold[k][1] = m.hinvarold[k][0]; m.hinvarold[k][0] = m.hinvar[k];
            m.invarold[k][2] = m.invarold[k][1]; m.invarold[k][1] = m.invarold[k][0]; m.invarold[k][0] = m.invar[k];
          }
          m.invar[k] = m.invar[k] + dt * ax;
        }
      }
    }
    if (jr <= 2 && (r = refresh())) return r;
  }
  for (int i = 0; i < 3; ++i) { ioldp[i] = i; imp->ioldr[i] = i; imp->ioldv[i] = i; imp->ioldiv[i] = i; }
  for (int i = 0; i < 2; ++i) { ioldh[i] = i; imp->iolda[i] = i; imp->ioldhiv[i] = i; }
  if (!wait && !mov) return EP_OK;
  if ((r = cuda_ok(cudaStreamSynchronize(st), "steprk"))) return r;
  return check_flags();
}

// steppc (steppc.f90:1-230).
template <class T>
int Engine<T>::steppc(double dt, ep_step_errors* e) {
  if (!have_field) { *err = "poten() must run before steppc()"; return EP_ERR_STATE; }
  const double c112 = 112.0 / 121.0, c9 = 9.0 / 121.0, c4o3 = 4.0 / 3.0;
  const bool mov = cfg.impurity == EP_IMPURITY_MOVING;
  int r;
  if ((r = lap_predict(dt))) return r;
  ImpState& m = *imp;
  if (mov) {
    double auxr[3];
    const int r3 = m.ioldr[2], v1 = m.ioldv[0], v2 = m.ioldv[1], v3 = m.ioldv[2], a1 = m.iolda[0], a2 = m.iolda[1];
    for (int k = 0; k < 3; ++k)
      auxr[k] = m.rimpold[k][r3] + c4o3 * dt * (2.0 * m.vimp[k] - m.vimpold[k][v1] + 2.0 * m.vimpold[k][v2]);
    for (int k = 0; k < 3; ++k) { m.rimpold[k][r3] = m.rimp[k]; m.rimp[k] = auxr[k] - c112 * m.pcr[k]; m.pcr[k] = auxr[k]; }
    for (int k = 0; k < 3; ++k)
      auxr[k] = m.vimpold[k][v3] + c4o3 * dt * (2.0 * m.aimp[k] - m.aimpold[k][a1] + 2.0 * m.aimpold[k][a2]);
    for (int k = 0; k < 3; ++k) { m.vimpold[k][v3] = auxr[k] - c112 * m.pcv[k]; m.pcv[k] = auxr[k]; }
    if (!cfg.fix_lambda) {
      const int i3 = m.ioldiv[2], h1 = m.ioldhiv[0], h2 = m.ioldhiv[1];
      std::complex<double> auxc[10];
      for (int k = 0; k < 10; ++k)
        auxc[k] = m.invarold[k][i3] + c4o3 * dt * (2.0 * m.hinvar[k] - m.hinvarold[k][h1] + 2.0 * m.hinvarold[k][h2]);
      for (int k = 0; k < 10; ++k) { m.invarold[k][i3] = m.invar[k]; m.invar[k] = auxc[k] - c112 * m.pciv[k]; m.pciv[k] = auxc[k]; }
    }
    for (int k = 0; k < 3; ++k) m.aimpold[k][a2] = m.aimp[k];
    for (int k = 0; k < 10; ++k) m.hinvarold[k][m.ioldhiv[1]] = m.hinvar[k];
    std::swap(m.iolda[0], m.iolda[1]);
    std::swap(m.ioldhiv[0], m.ioldhiv[1]);
  }
  if ((r = refresh())) return r;
  if ((r = lap_correct(dt, e != nullptr))) return r;
  double errimp = 0, errvimp = 0, erriv = 0;
  if (mov) {
    double auxr[3];
    const int r2 = m.ioldr[1], r3 = m.ioldr[2], v1 = m.ioldv[0], v2 = m.ioldv[1], v3 = m.ioldv[2];
    const int a1 = m.iolda[0], a2 = m.iolda[1];
    for (int k = 0; k < 3; ++k)
      auxr[k] = 0.125 * (9.0 * m.rimpold[k][r3] - m.rimpold[k][r2] + 3.0 * dt * (m.vimpold[k][v3] + 2.0 * m.vimp[k] - m.vimpold[k][v1]));
    for (int k = 0; k < 3; ++k) { m.pcr[k] = m.pcr[k] - auxr[k]; m.rimp[k] = auxr[k] + c9 * m.pcr[k]; errimp += std::fabs(c9 * m.pcr[k]); }
    errimp *= 0.3333333333;
    { const int t = m.ioldr[2]; m.ioldr[2] = m.ioldr[1]; m.ioldr[1] = m.ioldr[0]; m.ioldr[0] = t; }
    for (int k = 0; k < 3; ++k)
      auxr[k] = 0.125 * (9.0 * m.vimp[k] - m.vimpold[k][v2] + 3.0 * dt * (m.aimp[k] + 2.0 * m.aimpold[k][a1] - m.aimpold[k][a2]));
    for (int k = 0; k < 3; ++k) {
      m.pcv[k] = m.pcv[k] - auxr[k];
      m.vimpold[k][v3] = m.vimp[k];
      m.vimp[k] = auxr[k] + c9 * m.pcv[k];
      errvimp += std::fabs(c9 * m.pcv[k]);
    }
    errvimp *= 0.3333333333;
    if (!cfg.fix_lambda) {
      const int i3 = m.ioldiv[2], i2 = m.ioldiv[1], h1 = m.ioldhiv[0], h2 = m.ioldhiv[1];
      std::complex<double> auxc[10];
      for (int k = 0; k < 10; ++k)
        auxc[k] = 0.125 * (9.0 * m.invarold[k][i3] - m.invarold[k][i2] + 3.0 * dt * (m.hinvar[k] + 2.0 * m.hinvarold[k][h1] - m.hinvarold[k][h2]));
      // steppc.f90:199-217: P corrects components 1-6 (7-10 zeroed), D all ten
      const int nc = cfg.state == EP_STATE_D ? 10 : 6;
      for (int k = 0; k < nc; ++k) m.pciv[k] = m.pciv[k] - auxc[k];
      for (int k = 0; k < 10; ++k) m.invar[k] = 0.0;
      for (int k = 0; k < nc; ++k) m.invar[k] = auxc[k] + c9 * m.pciv[k];
      for (int k = 0; k < nc; ++k) erriv += std::abs(c9 * m.pciv[k]);
      erriv *= nc == 10 ? 0.1 : 0.1666666666666;
    }
    { const int t = m.ioldv[2]; m.ioldv[2] = m.ioldv[1]; m.ioldv[1] = m.ioldv[0]; m.ioldv[0] = t; }
    { const int t = m.ioldiv[2]; m.ioldiv[2] = m.ioldiv[1]; m.ioldiv[1] = m.ioldiv[0]; m.ioldiv[0] = t; }
  }
  if (e) {
    double s[4];
    if ((r = read_sums(s, 4, 0))) return r;
    e->errHe = c9 * s[0] / (double)g.N;
    e->errimp = errimp;
    e->errvimp = errvimp;
    e->erriv = erriv;
    last_norm = s[1] * dxyz;
    last_mu = s[2] / s[3];
    return check_flags();
  }
  return EP_OK;
}

template <class T>
int Engine<T>::renormalize(double* norm_before, bool wait) {
  // norm of psi -> scale -> rescale psi, the history and den
  int r0 = ensure_materialized();
  if (r0) return r0;
  auto kn = k_normsum<T>;
  EP_LAUNCH("normsum", kn, EP_RED_BLOCKS, 256, 0, psi, g.N, partials);
  int r;
  if ((r = reduce_finalize(EP_RED_BLOCKS, 1, 25, 2))) return r;
  HistPtrs<T> hp{{po[0], po[1], po[2], ph[0], ph[1], pc}};
  auto ks = k_rescale<T>;
  EP_LAUNCH("rescale", ks, 4 * 152, 256, 0, psi, den, hp, g.N, sc);
  if (wait || norm_before) {
    double s;
    if ((r = read_sums(&s, 1, 25))) return r;
    last_norm = s * dxyz;
    if (norm_before) *norm_before = last_norm;
    return check_flags();
  }
  return EP_OK;
}

template <class T>
int Engine<T>::check_flags() {
  unsigned int f = 0;
  int r = cuda_ok(cudaMemcpyAsync(&f, &sc->flags, sizeof(unsigned), cudaMemcpyDeviceToHost, st), "flags");
  if (r) return r;
  if ((r = cuda_ok(cudaStreamSynchronize(st), "flags"))) return r;
  if (f) {
    cudaMemsetAsync(&sc->flags, 0, sizeof(unsigned), st);
    if (f & EP_FLAG_TIMEOUT) {
      *err = "a stencil march gave up waiting for its TMA copies";
      return EP_ERR_TIMEOUT;
    }
    *err = (f & EP_FLAG_DEN_NONPOS) ? "density not positive (steprk trap)" : "non-finite value in a reduction";
    return EP_ERR_NONFINITE;
  }
  return EP_OK;
}

template <class T>
int Engine<T>::upload_psi(const double* h) {
  int r;
  if ((r = ensure_materialized())) return r;
  if (std::is_same<T, double>::value) {
    if ((r = cuda_ok(cudaMemcpyAsync(psi, h, g.N * sizeof(CT), cudaMemcpyHostToDevice, st), "upload psi"))) return r;
  } else {
    double2* tmp = nullptr;
    if ((r = cuda_ok(cudaMalloc((void**)&tmp, g.N * sizeof(double2)), "upload tmp"))) return r;
    cudaMemcpyAsync(tmp, h, g.N * sizeof(double2), cudaMemcpyHostToDevice, st);
    auto k = k_convert<double2, CT>;
    EP_LAUNCH("convert", k, 4 * 152, 256, 0, tmp, psi, g.N);
    cudaStreamSynchronize(st);
    cudaFree(tmp);
  }
  auto k = k_psi_to_den<T>;
  EP_LAUNCH("psi_to_den", k, 4 * 152, 256, 0, psi, den, g.N);
  return cuda_ok(cudaStreamSynchronize(st), "upload psi");
}

template <class T>
int Engine<T>::download_c(int which, double* h) {
  int r0 = ensure_materialized();
  if (r0) return r0;
  const CT* src = nullptr;
  switch (which) {
    case EP_CFIELD_PSI: src = psi; break;
    case EP_CFIELD_PSIOLD1: src = po[0]; break;
    case EP_CFIELD_PSIOLD2: src = po[1]; break;
    case EP_CFIELD_PSIOLD3: src = po[2]; break;
    case EP_CFIELD_HPSIOLD1: src = ph[0]; break;
    case EP_CFIELD_HPSIOLD2: src = ph[1]; break;
    case EP_CFIELD_PC: src = pc; break;
    case EP_CFIELD_Q: src = q; break;
    default: *err = "unknown complex field"; return EP_ERR_INVALID_ARG;
  }
  int r;
  if (std::is_same<T, double>::value) {
    if ((r = cuda_ok(cudaMemcpyAsync(h, src, g.N * sizeof(CT), cudaMemcpyDeviceToHost, st), "download"))) return r;
  } else {
    double2* tmp = nullptr;
    if ((r = cuda_ok(cudaMalloc((void**)&tmp, g.N * sizeof(double2)), "download tmp"))) return r;
    auto k = k_convert<CT, double2>;
    EP_LAUNCH("convert", k, 4 * 152, 256, 0, src, tmp, g.N);
    cudaMemcpyAsync(h, tmp, g.N * sizeof(double2), cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);
    cudaFree(tmp);
  }
  return cuda_ok(cudaStreamSynchronize(st), "download");
}

template <class T>
int Engine<T>::download_r(int which, double* h) {
  int r0 = ensure_materialized();
  if (r0) return r0;
  const T* src = nullptr;
  switch (which) {
    case EP_FIELD_DEN: src = den; break;
    case EP_FIELD_POT4: src = pot4; break;
    case EP_FIELD_UIMP: src = uimp; break;
    case EP_FIELD_DENCG: src = dencg; break;
    case EP_FIELD_DELJ4: src = delj4; break;
    case EP_FIELD_DXDEN: src = dxd; break;
    case EP_FIELD_DYDEN: src = dyd; break;
    case EP_FIELD_DZDEN: src = dzd; break;
    case EP_FIELD_FALFS: src = falfs; break;
    case EP_FIELD_INTXALF: src = intx; break;
    case EP_FIELD_INTYALF: src = inty; break;
    case EP_FIELD_INTZALF: src = intz; break;
    case EP_FIELD_UALPHAS: src = ualphas; break;
    case EP_FIELD_VPI: src = vpi; break;
    case EP_FIELD_DELTA: src = delta; break;
    case EP_FIELD_SIGDEL:
      if (!sigdel) { *err = "SIGDEL exists in the D state only"; return EP_ERR_INVALID_ARG; }
      src = sigdel;
      break;
    default: *err = "unknown field"; return EP_ERR_INVALID_ARG;
  }
  int r;
  if (std::is_same<T, double>::value) {
    if ((r = cuda_ok(cudaMemcpyAsync(h, src, g.N * sizeof(T), cudaMemcpyDeviceToHost, st), "download"))) return r;
  } else {
    double* tmp = nullptr;
    if ((r = cuda_ok(cudaMalloc((void**)&tmp, g.N * sizeof(double)), "download tmp"))) return r;
    auto k = k_convert<T, double>;
    EP_LAUNCH("convert", k, 4 * 152, 256, 0, src, tmp, g.N);
    cudaMemcpyAsync(h, tmp, g.N * sizeof(double), cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);
    cudaFree(tmp);
  }
  return cuda_ok(cudaStreamSynchronize(st), "download");
}

template <class T>
int Engine<T>::slot_of(const CT* p) const {
  for (int k = 0; k < EP_NSLOTS; ++k)
    if (slot_base[k] == p) return k;
  return 0;
}

template <class T>
int Engine<T>::ensure_materialized() {
  if (!lazy) return EP_OK;
  SlotPtrs<T> sp{};
  for (int k = 0; k < EP_NSLOTS; ++k) sp.b[k] = slot_base[k];
  auto km = k_materialize<T>;
  EP_LAUNCH("materialize", km, 4 * 152, 256, 0, sp, den, g.N, sc);
  auto kr = k_reset_scales;
  EP_LAUNCH("reset_scales", kr, 1, 32, 0, sc);
  lazy = false;
  return EP_OK;
}

template <class T>
int Engine<T>::rescale_pending() {
  HistPtrs<T> hp{{po[0], po[1], po[2], ph[0], ph[1], pc}};
  auto ks = k_rescale<T>;
  EP_LAUNCH("rescale", ks, 4 * 152, 256, 0, psi, den, hp, g.N, sc);
  return EP_OK;
}

// Precision switch: convert the state of the other engine role by role
// (psi, the multistep history, pc, q and every real field) into this one.
template <class T>
template <class U>
int Engine<T>::import_state(const Engine<U>& o) {
  typedef C2<U> OT;
  const OT* cs[9] = {o.psi, o.spare, o.po[0], o.po[1], o.po[2], o.ph[0], o.ph[1], o.pc, o.q};
  CT* cd[9] = {psi, spare, po[0], po[1], po[2], ph[0], ph[1], pc, q};
  for (int i = 0; i < 9; ++i) {
    auto k = k_convert<OT, CT>;
    EP_LAUNCH("convert", k, 4 * 152, 256, 0, cs[i], cd[i], g.N);
  }
  const U* rs[15] = {o.den, o.pot4, o.uimp, o.dencg, o.delj4, o.dxd, o.dyd, o.dzd, o.falfs,
                     o.intx, o.inty, o.intz, o.ualphas, o.vpi, o.delta};
  T* rd[15] = {den, pot4, uimp, dencg, delj4, dxd, dyd, dzd, falfs, intx, inty, intz, ualphas, vpi, delta};
  for (int i = 0; i < 15; ++i) {
    auto k = k_convert<U, T>;
    EP_LAUNCH("convert", k, 4 * 152, 256, 0, rs[i], rd[i], g.N);
  }
  if (sigdel && o.sigdel) {
    auto k = k_convert<U, T>;
    EP_LAUNCH("convert", k, 4 * 152, 256, 0, o.sigdel, sigdel, g.N);
  }
  for (int i = 0; i < 3; ++i) ioldp[i] = o.ioldp[i];
  for (int i = 0; i < 2; ++i) ioldh[i] = o.ioldh[i];
  have_field = o.have_field;
  last_mu = o.last_mu;
  last_norm = o.last_norm;
  return EP_OK;
}

// Autotuner of the FFT-pass launch shapes: times the idempotent poten()
// pipeline on the current density for candidate (lines, threads) per pass
// class, coordinate by coordinate, and keeps the fastest.
template <class T>
int Engine<T>::autotune(std::string* report) {
  int r;
  if ((r = ensure_materialized())) return r;
  cudaEvent_t a = nullptr, b = nullptr;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  auto timed = [&](float& best) -> int {
    best = 1e30f;
    for (int rep = 0; rep < 3; ++rep) {
      cudaEventRecord(a, st);
      int q = poten();
      if (q) return q;
      cudaEventRecord(b, st);
      cudaEventSynchronize(b);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, a, b);
      if (rep > 0) best = std::min(best, ms);
    }
    return EP_OK;
  };
  const int lts[] = {4, 8, 16, 32};
  const int nls[] = {2, 4, 8, 16, 32};
  const int thrs[] = {64, 128, 256};
  float base = 0.f;
  if ((r = timed(base))) goto done;
  // coordinate descent: each X kernel's shape, then the Y and Z shapes of the
  // shared-memory engine; a candidate replaces the current shape only when
  // poten gets faster by more than 1% (timing noise)
  {
    float cur = base;
    const int xreal[4] = {0, 4, 4, 1};
    for (int round = 0; round < 2; ++round) {
      for (int cls = 0; cls < 6; ++cls) {
        if ((cls == 4 && rfft::supported<T>(g.ny)) || (cls == 5 && rfft::supported<T>(g.nz))) continue;
        const Shapes keep = shp;
        Shapes bestS = shp;
        float best = cur;
        for (int li = 0; li < (cls < 4 ? 5 : 4); ++li) {
          for (int th : thrs) {
            Shapes c = keep;
            if (cls < 4) {
              c.xnl[cls] = nls[li];
              c.xthr[cls] = th;
              if (x_smem(c.xnl[cls], xreal[cls]) > EP_SMEM_CAP) continue;
            } else if (cls == 4) {
              c.ylt = lts[li]; c.ythr = th;
              if (l_smem(c.ylt, g.ny, 2) > EP_SMEM_CAP) continue;
            } else {
              c.zlt = lts[li]; c.zthr = th;
              if (l_smem(c.zlt, g.nz, 3) > EP_SMEM_CAP) continue;
            }
            shp = c;
            float t = 0.f;
            if ((r = timed(t))) goto done;
            if (t < 0.99f * best) { best = t; bestS = c; }
          }
        }
        shp = bestS;
        cur = best;
      }
    }
  }
  {
    float fin = 0.f;
    if ((r = timed(fin))) goto done;
    if (report) {
      char buf[256];
      snprintf(buf, sizeof buf,
               "poten %.3f -> %.3f ms; X1..X4 %dx%d %dx%d %dx%d %dx%d (lines x threads), Y %d x %d, Z %d x %d", base,
               fin, shp.xnl[0], shp.xthr[0], shp.xnl[1], shp.xthr[1], shp.xnl[2], shp.xthr[2], shp.xnl[3],
               shp.xthr[3], shp.ylt, shp.ythr, shp.zlt, shp.zthr);
      *report = buf;
    }
  }
done:
  ++shapes_gen;  // captured step graphs used the old shapes
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return r;
}

#endif
#if EP_ENGINE_PARTS & EP_PART_X
template <class T>
int Engine<T>::x_attrs() {
  int r;
  if ((r = x_attrs_n2<0>())) return r;
  if constexpr (std::is_same<T, dfloat>::value) return EP_OK;  // general engine only
  if ((r = x_attrs_n2<16>()) || (r = x_attrs_n2<32>()) || (r = x_attrs_n2<64>()) || (r = x_attrs_n2<128>()))
    return r;
  if constexpr (sizeof(T) == 4) {
    if ((r = x_attrs_n2<48>()) || (r = x_attrs_n2<80>()) || (r = x_attrs_n2<96>())) return r;
  }
  return EP_OK;
}

// X pass `which` (1..4) of poten on the register transform of this grid's
// half-lines (N2 = 0: the general engine).
template <class T>
int Engine<T>::x_pass(int which, bool otc) {
  if constexpr (std::is_same<T, dfloat>::value) return x_launch<0>(which, otc);
  switch (x_reg_n2<T>(g.nx / 2)) {
    case 16: return x_launch<16>(which, otc);
    case 32: return x_launch<32>(which, otc);
    case 64: return x_launch<64>(which, otc);
    case 128: return x_launch<128>(which, otc);
    case 48: if constexpr (sizeof(T) == 4) return x_launch<48>(which, otc); break;
    case 80: if constexpr (sizeof(T) == 4) return x_launch<80>(which, otc); break;
    case 96: if constexpr (sizeof(T) == 4) return x_launch<96>(which, otc); break;
    default: break;
  }
  return x_launch<0>(which, otc);
}
#endif

#if EP_ENGINE_PARTS & EP_PART_XK
template <class T>
template <int N2>
int Engine<T>::x_attrs_n2() {
  const int big = 220 * 1024;
  cudaFuncSetAttribute(k_x1<T, N2>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(k_x2<T, N2>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(k_x3<T, N2>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(k_x4<T, N2>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  return EP_OK;
}

template <class T>
template <int N2>
int Engine<T>::x_launch(int which, bool otc) {
  const long long nlines = (long long)g.ny * g.nz;
  if (which == 1) {
    const int nl = x_lines(0, 0);
    auto k = k_x1<T, N2>;
    EP_LAUNCH("x1_r2c_den", k, (unsigned)((nlines + nl - 1) / nl), shp.xthr[0], x_smem(nl, 0), g, den, S[0], p2, twx, nl);
  } else if (which == 2) {
    const int nl = x_lines(1, otc ? 3 : 2);
    auto k = k_x2<T, N2>;
    EP_LAUNCH("x2_c2r_r2c", k, (unsigned)((nlines + nl - 1) / nl), shp.xthr[1], x_smem(nl, otc ? 3 : 2), g, phys, Tb[0],
              Tb[1], Tb[2], den, dxd, dyd, dzd, dencg, delj4, pot4, falfs, S[0], S[1], S[2], S[3], p2, twx, nl);
  } else if (which == 3) {
    const int nl = x_lines(2, otc ? 4 : 1);
    auto k = k_x3<T, N2>;
    EP_LAUNCH("x3_c2r_r2c", k, (unsigned)((nlines + nl - 1) / nl), shp.xthr[2], x_smem(nl, otc ? 4 : 1), g, phys, fd,
              Tb[0], Tb[1], Tb[2], Tb[3], den, dxd, dyd, dzd, falfs, pot4, intx, inty, intz, gy, gz, dgx, S[0], p2, twx,
              nl);
  } else {
    const int nl = x_lines(3, 1);
    auto k = k_x4<T, N2>;
    EP_LAUNCH("x4_c2r_ualpha", k, (unsigned)((nlines + nl - 1) / nl), shp.xthr[3], x_smem(nl, 1), g, phys, Tb[0], den,
              dgx, dyz, pot4, ualphas, p2, twx, nl);
  }
  return EP_OK;
}
#endif

#if EP_ENGINE_PARTS & EP_PART_FFT
template <class T>
int Engine<T>::fft_attrs() {
  const int big = 220 * 1024;
  cudaFuncSetAttribute(k_c2c<T, -1>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(k_c2c<T, +1>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(k_zconv<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
#define EP_RFFT_ATTR(NN)                                                                                  \
  cudaFuncSetAttribute(k_c2c_r<T, NN, -1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rfft::smem_bytes<T, NN>()); \
  cudaFuncSetAttribute(k_c2c_r<T, NN, +1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rfft::smem_bytes<T, NN>()); \
  cudaFuncSetAttribute(k_zconv_r<T, NN, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rfft::conv_smem_bytes<T, NN, true>()); \
  cudaFuncSetAttribute(k_zconv_r<T, NN, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rfft::conv_smem_bytes<T, NN, false>());
  EP_RFFT_ATTR(32) EP_RFFT_ATTR(64) EP_RFFT_ATTR(128) EP_RFFT_ATTR(256)
  if constexpr (sizeof(T) == 4) { EP_RFFT_ATTR(96) EP_RFFT_ATTR(192) }
#undef EP_RFFT_ATTR
  return EP_OK;
}
#endif

#if EP_ENGINE_PARTS & EP_PART_MARCH
// TMA tensor maps of the pair march.  A complex field is a float tensor of
// 2 nx x ny x nz (row pitch 8 nx bytes, a multiple of 16 for even nx);
// boxes reaching outside it read zeros.
template <class T>
int Engine<T>::build_march_maps() {
  typedef CUresult (*EncodeTiled)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
  void* fp = nullptr;
  cudaDriverEntryPointQueryResult qres{};
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fp, 12000, cudaEnableDefault, &qres) !=
          cudaSuccess ||
      qres != cudaDriverEntryPointSuccess || !fp) {
    cudaGetLastError();
    *err = "cuTensorMapEncodeTiled is not available";
    return EP_ERR_CUDA;
  }
  EncodeTiled encode = reinterpret_cast<EncodeTiled>(fp);
  auto make = [&](CUtensorMap* m, const void* base, int xfloats, int bx, int by) -> bool {
    const cuuint64_t dim[3] = {(cuuint64_t)xfloats, (cuuint64_t)g.ny, (cuuint64_t)g.nz};
    const cuuint64_t str[2] = {(cuuint64_t)xfloats * 4, (cuuint64_t)xfloats * 4 * g.ny};
    const cuuint32_t box[3] = {(cuuint32_t)bx, (cuuint32_t)by, 1};
    const cuuint32_t est[3] = {1, 1, 1};
    return encode(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<void*>(base), dim, str, box, est,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
  };
  const void* cb[] = {psi, spare, po[0], po[1], po[2], ph[0], ph[1], pc, q};
  cmaps.clear();
  for (const void* b : cb) {
    BufMaps bm{};
    bm.buf = b;
    if (!make(&bm.m[0], b, 2 * g.nx, 2 * EP_PX, fd.R) || !make(&bm.m[1], b, 2 * g.nx, 2 * EP_PX, EP_TYT) ||
        !make(&bm.m[2], b, 2 * g.nx, 16, fd.R) || !make(&bm.m[3], b, 2 * g.nx, 16, EP_TYT)) {
      *err = "tensor map of a complex field refused";
      return EP_ERR_CUDA;
    }
    cmaps.push_back(bm);
  }
  if (!make(&rmaps[0], pot4, g.nx, EP_PX, EP_TYT) || !make(&rmaps[1], uimp, g.nx, EP_PX, EP_TYT)) {
    *err = "tensor map of a real field refused";
    return EP_ERR_CUDA;
  }
  return EP_OK;
}

template <class T>
const CUtensorMap* Engine<T>::maps_of(const void* buf) const {
  for (const BufMaps& b : cmaps)
    if (b.buf == buf) return b.m;
  return nullptr;
}

// The maps of one predictor / corrector launch: the marched field's four
// boxes, the {128 x EP_TYT} box of each complex input, pot4 and uimp.
template <class T>
bool Engine<T>::march_maps(MarchMaps& mm, const CT* marched, const CT* const* cin, int nc) const {
  memset(&mm, 0, sizeof(mm));
  const CUtensorMap* m = maps_of(marched);
  if (!m) return false;
  for (int k = 0; k < 4; ++k) mm.halo[k] = m[k];
  for (int i = 0; i < nc; ++i) {
    const CUtensorMap* mi = maps_of(cin[i]);
    if (!mi) return false;
    mm.cin[i] = mi[1];
  }
  mm.rin[0] = rmaps[0];
  mm.rin[1] = rmaps[1];
  // the failure-detection test: bytes announced that no copy delivers, and a
  // short wait limit
  mm.polls = tma_timeout_test ? 4096u : EP_MBAR_POLLS;
  mm.no_copies = tma_timeout_test ? 1u : 0u;
  return true;
}

template <class T>
int Engine<T>::march_setup() {
#define EP_ATTR(RR)                                                                                      \
  if constexpr (r_built<T>(RR)) {                                                                        \
  cudaFuncSetAttribute(k_predict<T, RR, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)march_smem<T, RR, 4, 2>()); \
  cudaFuncSetAttribute(k_correct<T, RR, true, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)march_smem<T, RR, 5, 2>()); \
  cudaFuncSetAttribute(k_correct<T, RR, false, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)march_smem<T, RR, 5, 2>()); \
  cudaFuncSetAttribute(k_rkstage<T, RR>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)march_smem<T, RR, 1, 2>()); } \
  if constexpr (pair_built<T>(RR)) {                                                                     \
  cudaFuncSetAttribute(k_predict<T, RR, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)march_pair_smem<RR, 4, 2>()); \
  cudaFuncSetAttribute(k_correct<T, RR, true, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)march_pair_smem<RR, 5, 2>()); \
  cudaFuncSetAttribute(k_correct<T, RR, false, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)march_pair_smem<RR, 5, 2>()); \
  cudaFuncSetAttribute(k_predict<T, RR, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)march_tma_smem<RR, 4, 2>()); \
  cudaFuncSetAttribute(k_correct<T, RR, true, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)march_tma_smem<RR, 5, 2>()); \
  cudaFuncSetAttribute(k_correct<T, RR, false, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)march_tma_smem<RR, 5, 2>()); }
  EP_ATTR(1) EP_ATTR(2) EP_ATTR(3) EP_ATTR(4) EP_ATTR(5) EP_ATTR(6)
#undef EP_ATTR
  {
    // the pair forms need an even stencil radius and even nx (a pair never
    // straddles the box edge), the TMA form whole 64 x 16 tiles as well;
    // EP_MARCH_PAIRS=0 keeps the one-point form, EP_MARCH_TMA=0 the cp.async
    // staging
    const char* ev = getenv("EP_MARCH_PAIRS");
    const char* et = getenv("EP_MARCH_TMA");
    const char* ex = getenv("EP_TEST_TMA_TIMEOUT");
    tma_timeout_test = ex && ex[0] == '1';
    bool can = g.nx % 2 == 0 && !(ev && ev[0] == '0');
    switch (fd.R) {
      case 2: can = can && pair_built<T>(2); break;
      case 4: can = can && pair_built<T>(4); break;
      case 6: can = can && pair_built<T>(6); break;
      default: can = false;
    }
    const bool tma = can && g.nx % EP_PX == 0 && g.ny % EP_TYT == 0 && !(et && et[0] == '0');
    pmode = tma ? 2 : (can ? 1 : 0);
    if (pmode == 2) {
      int r = build_march_maps();
      if (r) return r;
    }
  }
  {
    // z-chunk lengths of the stencil marches from their resident blocks per SM
    int occ_pc = 0, occ_pr = 0, occ_rk = 0, occ_d1 = 0;
    const int nt = EP_TX * EP_TY;
#define EP_OCC(RR)                                                                                         \
  case RR:                                                                                                 \
    if constexpr (r_built<T>(RR)) {                                                                        \
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_pc, k_correct<T, RR, true, 0>, nt, march_smem<T, RR, 5, 2>()); \
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_pr, k_predict<T, RR, 0>, nt, march_smem<T, RR, 4, 2>());      \
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_rk, k_rkstage<T, RR>, nt, march_smem<T, RR, 1, 2>()); \
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_d1, k_d1march<T, RR, 0>, nt, 0); }                  \
    if constexpr (pair_built<T>(RR)) {                                                                     \
    if (pmode == 1) {                                                                                      \
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_pc, k_correct<T, RR, true, 1>, nt, march_pair_smem<RR, 5, 2>()); \
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_pr, k_predict<T, RR, 1>, nt, march_pair_smem<RR, 4, 2>()); } \
    if (pmode == 2) {                                                                                      \
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_pc, k_correct<T, RR, true, 2>, EP_TX * EP_TYT, march_tma_smem<RR, 5, 2>()); \
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_pr, k_predict<T, RR, 2>, EP_TX * EP_TYT, march_tma_smem<RR, 4, 2>()); } } \
    break;
    switch (fd.R) { EP_OCC(1) EP_OCC(2) EP_OCC(3) EP_OCC(4) EP_OCC(5) EP_OCC(6) default: break; }
#undef EP_OCC
    const int tile_x = pmode ? EP_PX : EP_TX, tile_y = pmode == 2 ? EP_TYT : EP_TY;
    zc_pc = march_zchunk(occ_pc, tile_x, tile_y);
    zc_pr = march_zchunk(occ_pr, tile_x, tile_y);
    zc_rk = march_zchunk(occ_rk);
    zc_d1 = march_zchunk(occ_d1, EP_D1_TX);
  }
  return EP_OK;
}
#endif
