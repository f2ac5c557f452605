// ep_common.cu - launch accounting and the reduction finalize kernel.
#include <cmath>

#include "ep_engine.h"

int Prof::cls(const char* name) {
  for (size_t i = 0; i < names.size(); ++i)
    if (names[i] == name) return (int)i;
  names.emplace_back(name);
  ms.push_back(0.0);
  cnt.push_back(0);
  return (int)names.size() - 1;
}

cudaEvent_t Prof::ev() {
  if (!pool.empty()) {
    cudaEvent_t e = pool.back();
    pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

void Prof::begin(cudaStream_t st, const char* name, cudaEvent_t& a, int& c) {
  ++launches;
  if (!on) return;
  c = cls(name);
  a = ev();
  cudaEventRecord(a, st);
}

void Prof::end(cudaStream_t st, int c, cudaEvent_t a) {
  if (!on || c < 0) return;
  cudaEvent_t b = ev();
  cudaEventRecord(b, st);
  pending.push_back({c, a, b});
}

void Prof::collect() {
  if (pending.empty()) return;
  cudaEventSynchronize(pending.back().b);
  for (auto& r : pending) {
    float t = 0.f;
    if (cudaEventElapsedTime(&t, r.a, r.b) == cudaSuccess) {
      ms[r.cls] += t;
      cnt[r.cls] += 1;
    }
    pool.push_back(r.a);
    pool.push_back(r.b);
  }
  pending.clear();
}

void Prof::release() {
  collect();
  for (cudaEvent_t e : pool) cudaEventDestroy(e);
  pool.clear();
}

// Two-sum accumulation (Neumaier) of the block partials, fixed order:
// thread t takes partials t, t+256, ...; then a fixed pairwise tree.
__device__ __forceinline__ void neu_add(double& s, double& c, double v) {
  const double t = s + v;
  if (fabs(s) >= fabs(v)) c += (s - t) + v; else c += (v - t) + s;
  s = t;
}

__global__ void k_finalize(const double* __restrict__ partials, int nblocks, int nq, DevScalars* sc, int out0,
                           int mode, double N, double dxyz, double n4, int renorm) {
  __shared__ double ss[256], cs[256];
  const int tid = threadIdx.x;
  for (int q = 0; q < nq; ++q) {
    double s = 0.0, c = 0.0;
    for (int b = tid; b < nblocks; b += blockDim.x) neu_add(s, c, partials[(long long)b * nq + q]);
    ss[tid] = s;
    cs[tid] = c;
    __syncthreads();
    for (int off = blockDim.x / 2; off > 0; off >>= 1) {
      if (tid < off) {
        double s1 = ss[tid], c1 = cs[tid] + cs[tid + off];
        neu_add(s1, c1, ss[tid + off]);
        ss[tid] = s1;
        cs[tid] = c1;
      }
      __syncthreads();
    }
    if (tid == 0) sc->sums[out0 + q] = ss[0] + cs[0];
    __syncthreads();
  }
  if (tid == 0) {
    bool bad = false;
    for (int q = 0; q < nq; ++q) bad |= !isfinite(sc->sums[out0 + q]);
    if (mode == 1) {
      const double norm = sc->sums[out0 + 1] * dxyz;
      sc->norm = norm;
      sc->mu = sc->sums[out0 + 2] / sc->sums[out0 + 3];
      sc->errHe = sc->sums[out0] / N;
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
