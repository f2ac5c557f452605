// ep_reduce.cuh - compensated reductions shared by the eff_pot kernels.
//
// Every sum the kernels return (norm, errHe, <psi|H|psi>, the energy
// integrals of energy.f90:67-165, the impurity force and moments) is carried
// as an unevaluated pair (hi, lo) from the first addition to the last:
//  * per thread: Neumaier's variant of Kahan-Babuska summation in FP64,
//    Kahan summation in FP32 for FP32 fields and in the stencil marches;
//  * across a warp, across the warps of a block and across the blocks:
//    pairs added with Knuth's error-free TwoSum, hi + e into hi, the lows
//    and e into lo (FP32 pairs up to the block's result for FP32 fields);
//  * block partials are stored as pairs: partials[b*nq + q] holds hi and
//    partials[nblocks*nq + b*nq + q] holds lo (the buffer holds twice the
//    partial count).
// The result is hi + lo rounded once: its error is about one rounding of the
// sum plus n u^2 times the sum of magnitudes, instead of the log2(n) u of a
// plain pairwise tree, so sums whose terms cancel keep their digits.
#pragma once
#include "ep_common.cuh"

// Knuth's TwoSum: s = fl(a + b) and s + e == a + b exactly.
EP_DEV void two_sum(double a, double b, double& s, double& e) {
  s = a + b;
  const double bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
EP_DEV void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// (s, c) += (s2, c2) for unevaluated pairs.
template <class F>
EP_DEV void pair_add(F& s, F& c, F s2, F c2) {
  F t, e;
  two_sum(s, s2, t, e);
  s = t;
  c = (c + c2) + e;
}

// Per-thread accumulators: the running sum s and its compensation c.
// Neumaier: the correction of each addition, whichever operand is larger in
// magnitude, goes into c (value s + c).
template <class T> struct Neumaier {
  typedef T value_type;
  T s = T(0), c = T(0);
  EP_DEV void add(T v) {
    const T t = s + v;
    c += (fabs(s) >= fabs(v)) ? ((s - t) + v) : ((v - t) + s);
    s = t;
  }
  EP_DEV T lo() const { return c; }
  EP_DEV double get() const { return (double)s + (double)c; }
};
// Kahan: c holds minus the low part lost so far (value s - c); four
// operations per addition, for the per-point sums of the stencil marches,
// whose running sums are short (one term per plane of the CTA's z range).
template <class T> struct Kahan {
  typedef T value_type;
  T s = T(0), c = T(0);
  EP_DEV void add(T v) {
    const T y = v - c;
    const T t = s + y;
    c = (t - s) - y;
    s = t;
  }
  EP_DEV T lo() const { return -c; }
  EP_DEV double get() const { return (double)s - (double)c; }
};
// Double-float terms: the pair (s, c) of FP32 values, each high part added
// to s with the error-free TwoSum and its rounding error and the low part
// collected in c (Ogita, Rump and Oishi's Sum2 kept as a pair: the error is
// about n u^2 of the magnitudes, where Kahan's s - c in FP32 keeps an error
// of up to 2u of the sum -- enough to move the renormalisation factor of the
// double-float path by 1e-12 a step).
template <> struct Kahan<dfloat> {
  typedef float value_type;
  float s = 0.0f, c = 0.0f;
  EP_DEV void add(dfloat v) {
    const float t = s + v.hi;
    const float bb = t - s;
    c += ((s - (t - bb)) + (v.hi - bb)) + v.lo;
    s = t;
  }
  EP_DEV float lo() const { return c; }
  EP_DEV double get() const { return (double)s + (double)c; }
};
// The accumulator of sums of T values: Neumaier in FP64, Kahan in FP32 and
// double-float.
template <class T> struct AccOf { typedef Neumaier<T> type; };
template <> struct AccOf<float> { typedef Kahan<float> type; };
template <> struct AccOf<dfloat> { typedef Kahan<dfloat> type; };
template <class T> using Acc = typename AccOf<T>::type;

template <class F>
EP_DEV void warp_pair_sum(F& s, F& c) {
  for (int o = 16; o > 0; o >>= 1) {
    const F s2 = __shfl_down_sync(0xffffffffu, s, o), c2 = __shfl_down_sync(0xffffffffu, c, o);
    pair_add(s, c, s2, c2);
  }
}

// Warp 0 finishes the per-warp pairs red_s/red_c[q][warp] of a block and
// stores the block's pair of every q in QMASK.
template <int NQ, unsigned QMASK, class F>
EP_DEV void block_pairs_store(F (&red_s)[NQ][32], F (&red_c)[NQ][32], int lane, int warp, int nw,
                              double* __restrict__ partials) {
  if (warp == 0) {
    const long long nb = (long long)gridDim.x * gridDim.y * gridDim.z;
    const long long b = blockIdx.x + (long long)gridDim.x * (blockIdx.y + (long long)gridDim.y * blockIdx.z);
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      if (!((QMASK >> q) & 1u)) continue;
      F s = lane < nw ? red_s[q][lane] : F(0), c = lane < nw ? red_c[q][lane] : F(0);
      warp_pair_sum(s, c);
      if (lane == 0) {
        // the pair widened to FP64 exactly (an FP32 pair gives its two
        // values; TwoSum of them is exact in FP64)
        double hs, he;
        two_sum((double)s, (double)c, hs, he);
        partials[b * NQ + q] = hs;
        partials[nb * NQ + b * NQ + q] = he;
      }
    }
  }
}

// Block reduction of per-thread accumulators into the block's pairs, for
// the sums q whose bit is set in QMASK (the others are not stored).  FP32
// accumulators stay FP32 pairs up to the block's result (the FP64 pipe is
// about 1/64 of the FP32 rate on this part; a pair of FP32 values carries
// about 48 significant bits).
template <int NQ, unsigned QMASK = ~0u, class A>
EP_DEV void block_reduce_store_acc(A (&acc)[NQ], double* __restrict__ partials) {
  typedef typename A::value_type T;
  __shared__ T red_s[NQ][32], red_c[NQ][32];
  const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int nth = blockDim.x * blockDim.y * blockDim.z;
  const int lane = tid & 31, warp = tid >> 5, nw = (nth + 31) >> 5;
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    if (!((QMASK >> q) & 1u)) continue;
    T s = acc[q].s, c = acc[q].lo();
    warp_pair_sum(s, c);
    if (lane == 0) {
      red_s[q][warp] = s;
      red_c[q][warp] = c;
    }
  }
  __syncthreads();
  block_pairs_store<NQ, QMASK>(red_s, red_c, lane, warp, nw, partials);
}

// Sum of the block pairs of a reduction -> sc->sums[out0 + q] for the q in
// qmask: warp w takes q = w, w + nwarps, ... (Neumaier over each lane's
// blocks, then a pair tree across the warp).  mode 1: corrector epilogue
// (norm, mu, renormalisation factor), mode 2: norm only.
EP_DEV void finalize_block(const double* partials, int nblocks, int nq, DevScalars* sc, int out0, int mode,
                           double N, double dxyz, double n4, int renorm, int stats = 1, unsigned qmask = ~0u) {
  const int tid = threadIdx.x + blockDim.x * threadIdx.y;
  const int nth = blockDim.x * blockDim.y;
  const int lane = tid & 31, warp = tid >> 5, nw = (nth + 31) >> 5;
  const double* lo = partials + (long long)nblocks * nq;
  for (int q = warp; q < nq; q += nw) {
    if (!((qmask >> q) & 1u)) continue;
    Acc<double> a;
    double cl = 0.0;
    for (int b = lane; b < nblocks; b += 32) {
      a.add(__ldcg(partials + (long long)b * nq + q));
      cl += __ldcg(lo + (long long)b * nq + q);
    }
    double s = a.s, c = a.c + cl;
    warp_pair_sum(s, c);
    if (lane == 0) sc->sums[out0 + q] = s + c;
  }
  __syncthreads();
  if (tid == 0) {
    bool bad = false;
    for (int q = 0; q < nq; ++q)
      if ((qmask >> q) & 1u) bad |= !isfinite(sc->sums[out0 + q]);
    if (mode == 1) {
      const double norm = sc->sums[out0 + 1] * dxyz;
      sc->norm = norm;
      if (stats) {
        sc->mu = sc->sums[out0 + 2] / sc->sums[out0 + 3];
        sc->errHe = sc->sums[out0] / N;
      }
      sc->scale = (renorm && norm > 0.0) ? sqrt(n4 / norm) : 1.0;
    } else if (mode == 2) {
      const double norm = sc->sums[out0] * dxyz;
      sc->norm = norm;
      sc->scale = norm > 0.0 ? sqrt(n4 / norm) : 1.0;
      bad |= !(norm > 0.0);
    }
    if (bad) atomicOr(&sc->flags, (unsigned)EP_FLAG_NONFINITE);
  }
}
