// Fused multiply-add throughput of this GPU, the denominator of the FP64 ALU
// roofline: every thread runs 8 independent FMA chains (enough to cover the
// pipeline latency), 16 resident 256-thread blocks per SM, one store per
// thread so nothing is dead code.  Prints JSON.
#include <cstdio>
#include <cuda_runtime.h>

template <class T>
__global__ void k_fma(T* out, int iters, T a, T b) {
  T x0 = threadIdx.x * T(1e-3), x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6,
    x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
      x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
    }
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

template <class T>
double tflops(int iters, int nsm) {
  const int nb = nsm * 16, nt = 256;
  T* d = nullptr;
  if (cudaMalloc(&d, sizeof(T) * nb * nt) != cudaSuccess) return -1.0;
  k_fma<T><<<nb, nt>>>(d, 10, T(0.999), T(1e-3));
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(a);
    k_fma<T><<<nb, nt>>>(d, iters, T(0.999), T(1e-3));
    cudaEventRecord(b);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    if (ms < best) best = ms;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(d);
  return 2.0 * 8 * 16 * (double)iters * nb * nt / (best * 1e-3) / 1e12;
}

int main() {
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const double f64 = tflops<double>(200, nsm), f32 = tflops<float>(2000, nsm);
  const cudaError_t e = cudaGetLastError();
  std::printf("{\"fp64_tflops\": %.4f, \"fp32_tflops\": %.4f, \"sms\": %d, \"status\": \"%s\"}\n", f64, f32, nsm,
              cudaGetErrorString(e));
  return e != cudaSuccess;
}
