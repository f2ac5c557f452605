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

__global__ void k_finalize(const double* __restrict__ partials, int nblocks, int nq, DevScalars* sc, int out0,
                           int mode, double N, double dxyz, double n4, int renorm) {
  finalize_block(partials, nblocks, nq, sc, out0, mode, N, dxyz, n4, renorm);
}

__global__ void k_reset_scales(DevScalars* sc) {
  if (threadIdx.x < EP_NSLOTS) {
    sc->bscale[threadIdx.x] = 1.0;
    sc->bscale_f[threadIdx.x] = 1.0f;
  }
  if (threadIdx.x == 0) sc->den_scale = 1.0;
}
