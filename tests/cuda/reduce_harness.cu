// reduce_harness.cu - test harness (not part of the library): the library's
// reduction primitives of ep_reduce.cuh, used by every kernel that returns a
// sum, beside a plain FP64 reduction of the same shape (per-thread running
// sum, warp shuffle tree, block partials, one finalising block).
#include <cuda_runtime.h>

#include "../../eff_pot_gb300/csrc/ep_reduce.cuh"

namespace {

constexpr int kBlocks = 1216, kThreads = 256;

__global__ void k_sum_compensated(const double* __restrict__ x, long long n, double* __restrict__ partials) {
  Acc<double> acc[1];
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    acc[0].add(x[i]);
  block_reduce_store_acc<1>(acc, partials);
}

__global__ void k_finalize_compensated(const double* __restrict__ partials, int nblocks, DevScalars* sc) {
  finalize_block(partials, nblocks, 1, sc, 0, 0, 1.0, 1.0, 1.0, 0);
}

EP_DEV double plain_block_sum(double s) {
  __shared__ double red[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if (lane == 0) red[warp] = s;
  __syncthreads();
  s = 0.0;
  if (warp == 0) {
    s = lane < nw ? red[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  }
  return s;
}

__global__ void k_sum_plain(const double* __restrict__ x, long long n, double* __restrict__ partials) {
  double s = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    s += x[i];
  s = plain_block_sum(s);
  if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

__global__ void k_finalize_plain(const double* __restrict__ partials, int nblocks, double* out) {
  double s = 0.0;
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x) s += partials[b];
  s = plain_block_sum(s);
  if (threadIdx.x == 0) *out = s;
}

}  // namespace

// Sum of n doubles on the GPU: compensated (the library's primitives) or
// plain.  Returns a cudaError_t value (0: success).
extern "C" int harness_sum(const double* hx, long long n, int compensated, double* out) {
  double *dx = nullptr, *partials = nullptr;
  DevScalars* sc = nullptr;
  cudaError_t e = cudaMalloc(&dx, (size_t)n * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&partials, 2 * (size_t)kBlocks * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&sc, sizeof(DevScalars));
  if (e == cudaSuccess) e = cudaMemcpy(dx, hx, (size_t)n * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(sc, 0, sizeof(DevScalars));
  if (e == cudaSuccess) {
    if (compensated) {
      k_sum_compensated<<<kBlocks, kThreads>>>(dx, n, partials);
      k_finalize_compensated<<<1, kThreads>>>(partials, kBlocks, sc);
      e = cudaMemcpy(out, &sc->sums[0], sizeof(double), cudaMemcpyDeviceToHost);
    } else {
      k_sum_plain<<<kBlocks, kThreads>>>(dx, n, partials);
      k_finalize_plain<<<1, kThreads>>>(partials, kBlocks, partials + kBlocks);
      e = cudaMemcpy(out, partials + kBlocks, sizeof(double), cudaMemcpyDeviceToHost);
    }
  }
  if (e == cudaSuccess) e = cudaGetLastError();
  cudaFree(dx);
  cudaFree(partials);
  cudaFree(sc);
  return (int)e;
}
