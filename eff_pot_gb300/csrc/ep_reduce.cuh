// ep_reduce.cuh - compensated reductions shared by the eff_pot kernels.
//
// Every sum the kernels return (norm, errHe, <psi|H|psi>, the energy
// integrals of energy.f90:67-165, the impurity force and moments) is carried
// as an unevaluated pair (hi, lo) from the first addition to the last:
//  * per thread: Neumaier's variant of Kahan-Babuska summation in FP64, or
//    Kahan summation in FP32 for FP32 fields;
//  * across a warp, across the warps of a block and across the blocks:
//    pairs added with Knuth's error-free TwoSum, hi + e into hi, the lows
//    and e into lo;
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

// Per-thread accumulators.
template <class T> struct Acc;
// FP64: Neumaier (the correction of each addition, whichever operand is
// larger in magnitude, goes into c).
template <> struct Acc<double> {
  double s = 0.0, c = 0.0;
  EP_DEV void add(double v) {
    const double t = s + v;
    c += (fabs(s) >= fabs(v)) ? ((s - t) + v) : ((v - t) + s);
    s = t;
  }
  EP_DEV double get() const { return s + c; }
};
// FP32 fields: Kahan in FP32 (c holds minus the lost low part), widened to
// FP64 once per warp.
template <> struct Acc<float> {
  float s = 0.f, c = 0.f;
  EP_DEV void add(float v) {
    const float y = v - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
  }
  EP_DEV double get() const { return (double)s - (double)c; }
};

template <class F>
EP_DEV void warp_pair_sum(F& s, F& c) {
  for (int o = 16; o > 0; o >>= 1) {
    const F s2 = __shfl_down_sync(0xffffffffu, s, o), c2 = __shfl_down_sync(0xffffffffu, c, o);
    pair_add(s, c, s2, c2);
  }
}

// Warp 0 finishes the per-warp pairs red_s/red_c[q][warp] of a block and
// stores the block's pair of every q.
template <int NQ>
EP_DEV void block_pairs_store(double (&red_s)[NQ][32], double (&red_c)[NQ][32], int lane, int warp, int nw,
                              double* __restrict__ partials) {
  if (warp == 0) {
    const long long nb = (long long)gridDim.x * gridDim.y * gridDim.z;
    const long long b = blockIdx.x + (long long)gridDim.x * (blockIdx.y + (long long)gridDim.y * blockIdx.z);
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      double s = lane < nw ? red_s[q][lane] : 0.0, c = lane < nw ? red_c[q][lane] : 0.0;
      warp_pair_sum(s, c);
      if (lane == 0) {
        partials[b * NQ + q] = s;
        partials[nb * NQ + b * NQ + q] = c;
      }
    }
  }
}

// Block reduction of per-thread accumulators into the block's pairs.
template <int NQ>
EP_DEV void block_reduce_store_acc(Acc<double> (&acc)[NQ], double* __restrict__ partials) {
  __shared__ double red_s[NQ][32], red_c[NQ][32];
  const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int nth = blockDim.x * blockDim.y * blockDim.z;
  const int lane = tid & 31, warp = tid >> 5, nw = (nth + 31) >> 5;
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    double s = acc[q].s, c = acc[q].c;
    warp_pair_sum(s, c);
    if (lane == 0) {
      red_s[q][warp] = s;
      red_c[q][warp] = c;
    }
  }
  __syncthreads();
  block_pairs_store<NQ>(red_s, red_c, lane, warp, nw, partials);
}
// FP32 accumulators are summed across the warp as FP32 pairs (only one lane
// per warp widens to FP64: the FP64 pipe is about 1/64 of the FP32 rate).
template <int NQ>
EP_DEV void block_reduce_store_acc(Acc<float> (&acc)[NQ], double* __restrict__ partials) {
  __shared__ double red_s[NQ][32], red_c[NQ][32];
  const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int nth = blockDim.x * blockDim.y * blockDim.z;
  const int lane = tid & 31, warp = tid >> 5, nw = (nth + 31) >> 5;
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    float hi = acc[q].s, lo = -acc[q].c;
    warp_pair_sum(hi, lo);
    if (lane == 0) {
      double s, e;
      two_sum((double)hi, (double)lo, s, e);
      red_s[q][warp] = s;
      red_c[q][warp] = e;
    }
  }
  __syncthreads();
  block_pairs_store<NQ>(red_s, red_c, lane, warp, nw, partials);
}

// Sum of the block pairs of a reduction (Neumaier over each thread's hi
// parts, then pair trees) by one block -> sc->sums[out0 + q]; mode 1:
// corrector epilogue (norm, mu, renormalisation factor), mode 2: norm only.
EP_DEV void finalize_block(const double* partials, int nblocks, int nq, DevScalars* sc, int out0, int mode,
                           double N, double dxyz, double n4, int renorm, int stats = 1) {
  __shared__ double fs[32], fc[32];
  const int tid = threadIdx.x + blockDim.x * threadIdx.y;
  const int nth = blockDim.x * blockDim.y;
  const int lane = tid & 31, warp = tid >> 5, nw = (nth + 31) >> 5;
  const double* lo = partials + (long long)nblocks * nq;
  for (int q = 0; q < nq; ++q) {
    Acc<double> a;
    double cl = 0.0;
    for (int b = tid; b < nblocks; b += nth) {
      a.add(__ldcg(partials + (long long)b * nq + q));
      cl += __ldcg(lo + (long long)b * nq + q);
    }
    double s = a.s, c = a.c + cl;
    warp_pair_sum(s, c);
    if (lane == 0) {
      fs[warp] = s;
      fc[warp] = c;
    }
    __syncthreads();
    if (warp == 0) {
      s = lane < nw ? fs[lane] : 0.0;
      c = lane < nw ? fc[lane] : 0.0;
      warp_pair_sum(s, c);
      if (lane == 0) sc->sums[out0 + q] = s + c;
    }
    __syncthreads();
  }
  if (tid == 0) {
    bool bad = false;
    for (int q = 0; q < nq; ++q) bad |= !isfinite(sc->sums[out0 + q]);
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
