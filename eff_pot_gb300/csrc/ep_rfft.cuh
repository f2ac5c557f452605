// ep_rfft.cuh - register-resident FFTs of strided lines (the Y and Z passes)
// for line lengths N in {32, 64, 128, 256} and, in FP32, {96, 192}.
//
// A CTA owns 32 lines whose first elements are (nearly) contiguous in memory
// (the x index runs fastest) and P threads per line: lane = line, warp = t.
// With N = E * P every thread holds E elements, and the transform is the
// two-factor decomposition
//
//   n = t + P a   (t < P, a < E),     k = ka + E kt   (ka < E, kt < P)
//   X[ka + E kt] = sum_t w_P^(t kt) w_N^(t ka) sum_a x[t + P a] w_E^(a ka)
//
// step 1: thread t loads x[t + P a] straight from global memory (each warp
//         load touches 32 consecutive lines: coalesced), runs the E-point
//         DFT over a in registers and applies w_N^(t ka);
// exchange: one pass through shared memory (row stride N+1: conflict-free);
// step 2: thread w runs the P-point DFTs of ka = w + P j (j < E/P) and then
//         holds X[w + P m] with m = j + (E/P) kt -- the same stride-P
//         subsequence step 1 reads, so a product in k-space followed by the
//         inverse transform needs no further exchange, and stores are again
//         coalesced.
// The general shared-memory Stockham engine (ep_fft.cuh) covers every other
// length.  Conventions are those of ep_fft.cuh: forward exp(-2 pi i kn/N),
// unnormalised both ways.
#pragma once
#include "ep_fft.cuh"
#include "ep_kernels.cuh"

namespace rfft {

template <int N> struct Shape;
template <> struct Shape<32> { static constexpr int P = 4, E = 8; };
template <> struct Shape<64> { static constexpr int P = 8, E = 8; };
template <> struct Shape<128> { static constexpr int P = 8, E = 16; };
template <> struct Shape<256> { static constexpr int P = 16, E = 16; };
template <> struct Shape<96> { static constexpr int P = 4, E = 24; };
template <> struct Shape<192> { static constexpr int P = 8, E = 24; };

// the mixed-radix lengths only in FP32 (the FP64 passes are bound by the
// arithmetic pipe, where the shared-memory engine does as well)
template <class T>
constexpr bool supported(int n) {
  return n == 32 || n == 64 || n == 128 || n == 256 || (sizeof(T) == 4 && (n == 96 || n == 192));
}

// Transform of the CTA's lines: on entry v[a] = x[t + P a], on return
// v[m] = X[t + P m].  S: this line's exchange row (N + 1 entries); tw: the
// table exp(-2 pi i k / N), k < N.  All threads of the CTA must call it.
template <class T, int N, int DIR>
EP_DEV void lines(C2<T>* v, C2<T>* S, const C2<T>* __restrict__ tw, int t) {
  constexpr int P = Shape<N>::P, E = Shape<N>::E;
  epfft::dft<T, E, DIR>(v);
  if (t != 0) {
#pragma unroll
    for (int ka = 1; ka < E; ++ka) {
      const C2<T> w = tw[t * ka];
      v[ka] = DIR < 0 ? cmul(v[ka], w) : cmulc(v[ka], w);
    }
  }
  __syncthreads();  // the previous transform has read its exchange rows
#pragma unroll
  for (int ka = 0; ka < E; ++ka) S[ka * P + t] = v[ka];
  __syncthreads();
#pragma unroll
  for (int j = 0; j < E / P; ++j) {
    C2<T> u[P];
#pragma unroll
    for (int tt = 0; tt < P; ++tt) u[tt] = S[(t + P * j) * P + tt];
    epfft::dft<T, P, DIR>(u);
#pragma unroll
    for (int kt = 0; kt < P; ++kt) v[j + (E / P) * kt] = u[kt];
  }
}

template <class T, int N>
constexpr size_t smem_bytes() {
  return (size_t)(32 * (N + 1) + N) * sizeof(C2<T>);
}
// The convolution pass up to 128-point lines stages each thread's
// form-factor values of its line (one table, or up to three) in shared
// memory while the forward transform runs; longer lines read them after the
// transform (the staging would cost resident CTAs, or not fit).
template <class T, int N>
__host__ __device__ constexpr bool conv_stage() {
  return N <= 128;
}
template <class T, int N, bool ONE>
constexpr size_t conv_smem_bytes() {
  return smem_bytes<T, N>() + (conv_stage<T, N>() ? (size_t)(ONE ? 1 : 3) * 32 * N * sizeof(T) : 0);
}


// Line base address of line L of a LineSet-like description.
EP_DEV long long line_base(long long L, long long Mi, long long So) { return (L % Mi) + (L / Mi) * So; }

}  // namespace rfft

// Blocks per SM the launch bounds ask for (FP32 / FP64).
template <class T, int N> struct Occ {
  // the in-place Y pass fits 64 registers at N = 128 without spilling: four
  // CTAs per SM keep more lines in flight (the pass is load-latency bound)
  static constexpr int c2c = sizeof(T) == 4 ? (N <= 128 ? 4 : 2) : (N <= 64 ? 2 : 1);
  static constexpr int conv = sizeof(T) == 4 ? (N <= 96 ? 3 : (N <= 192 ? 2 : 1)) : 1;
  // one output per input (no spectrum kept): 3 CTAs per SM at N = 128 (64
  // registers would spill)
  static constexpr int conv1 = sizeof(T) == 4 ? (N <= 96 ? 4 : (N == 128 ? 3 : 2)) : (N <= 64 ? 2 : 1);
};

// In-place transforms along a strided axis of up to 8 arrays (blockIdx.y).
// Element m of a thread sits at offset m * (P Sa) from its first one (32-bit
// offsets: N Sa < 2^31 for every supported grid).
template <class T, int N, int DIR>
__global__ void __launch_bounds__(32 * rfft::Shape<N>::P, (Occ<T, N>::c2c))
    k_c2c_r(const __grid_constant__ Arr8<T> arr, LineSet ls, const C2<T>* __restrict__ twg) {
  constexpr int P = rfft::Shape<N>::P, E = rfft::Shape<N>::E;
  extern __shared__ __align__(16) unsigned char smraw[];
  C2<T>* S = reinterpret_cast<C2<T>*>(smraw);
  C2<T>* tw = S + 32 * (N + 1);
  const int lane = threadIdx.x, t = threadIdx.y;
  for (int i = t * 32 + lane; i < N; i += 32 * P) tw[i] = twg[i];
  const long long L = (long long)blockIdx.x * 32 + lane;
  const bool valid = L < ls.nlines;
  const int stp = P * (int)ls.Sa;
  C2<T>* a = arr.a[blockIdx.y] + (valid ? rfft::line_base(L, ls.Mi, ls.So) : 0) + (long long)t * ls.Sa;
  C2<T> v[E];
#pragma unroll
  for (int m = 0; m < E; ++m) v[m] = valid ? a[m * stp] : cmk<T>(T(0), T(0));
  __syncthreads();  // tw complete
  rfft::lines<T, N, DIR>(v, S + lane * (N + 1), tw, t);
  if (valid) {
#pragma unroll
    for (int m = 0; m < E; ++m) a[m * stp] = v[m];
  }
}

// Forward transform along the pass axis, then per kernel table the k-space
// product and the inverse transform (poten.f90:34-36,46-48,69-71,95-97 and
// term_alfa.f90:172-176,203-205), all in registers between the exchanges.
template <class T, int N, bool ONE>
__global__ void __launch_bounds__(32 * rfft::Shape<N>::P, (ONE ? Occ<T, N>::conv1 : Occ<T, N>::conv))
    k_zconv_r(const __grid_constant__ ConvSpec<T> cs, LineSet ls, const C2<T>* __restrict__ twg) {
  constexpr int P = rfft::Shape<N>::P, E = rfft::Shape<N>::E;
  extern __shared__ __align__(16) unsigned char smraw[];
  C2<T>* S = reinterpret_cast<C2<T>*>(smraw);
  C2<T>* tw = S + 32 * (N + 1);
  const int lane = threadIdx.x, t = threadIdx.y;
  for (int i = t * 32 + lane; i < N; i += 32 * P) tw[i] = twg[i];
  const int which = blockIdx.y;
  const long long L = (long long)blockIdx.x * 32 + lane;
  const bool valid = L < ls.nlines;
  const long long b = (valid ? rfft::line_base(L, ls.Mi, ls.So) : 0) + (long long)t * ls.Sa;
  const int stp = P * (int)ls.Sa;
  C2<T>* Srow = S + lane * (N + 1);
  // the thread's form-factor values, copied in while the forward transform
  // runs (each thread reads back only its own copies)
  constexpr bool STAGE = rfft::conv_stage<T, N>();
  constexpr int NT = 32 * P;
  T* kb = reinterpret_cast<T*>(tw + N);
  const int tid = t * 32 + lane;
  auto kval = [&](int j, int m) -> T {
    if (!valid) return T(0);
    if constexpr (STAGE) return kb[(j * E + m) * NT + tid];
    return cs.ker[which][j][b + (long long)m * stp];
  };
  if constexpr (STAGE) {
    const int ntab = ONE ? 1 : cs.nout[which];
    if (valid) {
      for (int j = 0; j < ntab; ++j) {
        const T* ker = cs.ker[which][j] + b;
#pragma unroll
        for (int m = 0; m < E; ++m) cp_async<sizeof(T)>(kb + (j * E + m) * NT + tid, ker + m * stp);
      }
    }
    cp_commit();
  }
  C2<T> v[E];
  {
    const C2<T>* in = cs.in[which] + b;
#pragma unroll
    for (int m = 0; m < E; ++m) v[m] = valid ? in[m * stp] : cmk<T>(T(0), T(0));
  }
  __syncthreads();  // tw complete
  rfft::lines<T, N, -1>(v, Srow, tw, t);
  if constexpr (STAGE) cp_wait<0>();
  if (ONE) {
    // a single kernel table: the product overwrites the spectrum
#pragma unroll
    for (int m = 0; m < E; ++m) {
      const T kv = kval(0, m);
      v[m] = cmk<T>(v[m].x * kv, v[m].y * kv);
    }
    rfft::lines<T, N, +1>(v, Srow, tw, t);
    if (valid) {
      C2<T>* o = cs.out[which][0] + b;
#pragma unroll
      for (int m = 0; m < E; ++m) o[m * stp] = v[m];
    }
    return;
  }
  const int nout = cs.nout[which];
  for (int j = 0; j < nout; ++j) {
    C2<T> u[E];
#pragma unroll
    for (int m = 0; m < E; ++m) {
      const T kv = kval(j, m);
      u[m] = cmk<T>(v[m].x * kv, v[m].y * kv);
    }
    rfft::lines<T, N, +1>(u, Srow, tw, t);
    if (valid) {
      C2<T>* o = cs.out[which][j] + b;
#pragma unroll
      for (int m = 0; m < E; ++m) o[m * stp] = u[m];
    }
  }
}
