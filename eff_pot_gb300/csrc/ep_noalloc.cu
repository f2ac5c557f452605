// ep_noalloc.cu - the k-space convolution of poten() for callers that
// cannot allocate device memory.
//
// Some callers can't call cudaMalloc: a Fortran or C host that runs inside
// a framework owning the whole device memory pool (the framework hands out
// buffers, and any allocation behind its back breaks its accounting or
// fails), or code running while a CUDA graph is being captured, where a
// fresh allocation is not allowed.  ep_convolve_noalloc gives them the
// density convolution out = IFFT(FFT(in) * K) / N that poten() applies with
// the coarse-graining, Lennard-Jones and alpha_s kernels, using only the
// buffers the caller passes plus the fixed scratch array below.
//
// The scratch is a file-scope __device__ array: every GPU that loads the
// library holds it (EP_NOALLOC_SCRATCH_BYTES) until the process exits.  In
// host code the array's name is only a host-side stand-in, so its device
// address is looked up once per device with cudaGetSymbolAddress.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/eff_pot.h"
#include "ep_kernels.cuh"

namespace {

// Largest half spectrum: (nx/2+1)*ny*nz <= 33*64*64 (a 64^3 grid); axes of
// at most 320 points.
constexpr long long kMaxHalf = 33LL * 64 * 64;
constexpr int kMaxAxis = 320;
constexpr long long kScratchElems = 2 * kMaxHalf + 3 * kMaxAxis;

static __device__ __align__(256) double2 g_noalloc_scratch[kScratchElems];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
double2* g_scratch_addr[kMaxDevices] = {};

// n >= 2 with no prime factor other than 2, 3 and 5 (any length; the
// scratch limit on the length is checked apart).
bool axis_ok(int n) {
  if (n < 2) return false;
  while (n % 2 == 0) n /= 2;
  while (n % 3 == 0) n /= 3;
  while (n % 5 == 0) n /= 5;
  return n == 1;
}

// Roots exp(-2 pi i k / n), k < n.
__global__ void k_noalloc_twiddles(double2* tw, int n) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    double s, c;
    sincospi(-2.0 * k / n, &s, &c);
    tw[k] = make_double2(c, s);
  }
}

// Backward c2r along x of every line, scaled by 1/N, into a real array.
__global__ void k_noalloc_xinv(Geo g, const double2* __restrict__ spec, double* __restrict__ out,
                               const __grid_constant__ FftPlan p2, const double2* __restrict__ twx, double scale, int nl) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int nx = g.nx;
  XSmem<double> S(smraw, nl, nx, 0);
  const long long nlines = (long long)g.ny * g.nz;
  const long long line0 = (long long)blockIdx.x * nl;
  const int nlv = (int)min((long long)nl, nlines - line0);
  for (int i = threadIdx.x; i < nx; i += blockDim.x) S.tw[i] = twx[i];
  __syncthreads();
  x_inverse<double, 0>(spec, line0, nlv, nl, nx, g.nxh, S, p2, scale, S.R);
  for (int e = threadIdx.x; e < nlv * nx; e += blockDim.x) out[line0 * nx + e] = S.R[e];
}

size_t x_smem_of(int nl, int nx) {
  return 2 * (size_t)nl * (nx / 2 + 1) * sizeof(double2) + (size_t)nx * sizeof(double2) + (size_t)nl * nx * sizeof(double);
}
size_t l_smem_of(int LT, int n, int nbuf) {
  return (size_t)nbuf * LT * (n + 1) * sizeof(double2) + (size_t)n * sizeof(double2) + (size_t)LT * sizeof(long long);
}

// Once per device, with that device current: the device address of the
// scratch array and the shared-memory limits of the kernels used here.
int device_setup(int dev, double2** out) {
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (g_scratch_addr[dev]) {
    *out = g_scratch_addr[dev];
    return EP_OK;
  }
  void* ptr = nullptr;
  if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess || !ptr) {
    cudaGetLastError();
    return EP_ERR_CUDA;
  }
  const int big = 220 * 1024;
  if (cudaFuncSetAttribute(k_x1<double, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, big) != cudaSuccess ||
      cudaFuncSetAttribute(k_c2c<double, -1>, cudaFuncAttributeMaxDynamicSharedMemorySize, big) != cudaSuccess ||
      cudaFuncSetAttribute(k_c2c<double, +1>, cudaFuncAttributeMaxDynamicSharedMemorySize, big) != cudaSuccess ||
      cudaFuncSetAttribute(k_zconv<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, big) != cudaSuccess ||
      cudaFuncSetAttribute(k_noalloc_xinv, cudaFuncAttributeMaxDynamicSharedMemorySize, big) != cudaSuccess) {
    cudaGetLastError();
    return EP_ERR_CUDA;
  }
  g_scratch_addr[dev] = static_cast<double2*>(ptr);
  *out = g_scratch_addr[dev];
  return EP_OK;
}

}  // namespace

extern "C" int ep_convolve_noalloc(const double* d_in, const double* d_kernel, double* d_out, int nx, int ny,
                                   int nz, void* stream) {
  if (!d_in || !d_kernel || !d_out) return EP_ERR_INVALID_ARG;
  if (nx % 2 || !axis_ok(nx) || !axis_ok(ny) || !axis_ok(nz)) return EP_ERR_BAD_GRID;
  const long long half = (long long)(nx / 2 + 1) * ny * nz;
  if (half > kMaxHalf || nx > kMaxAxis || ny > kMaxAxis || nz > kMaxAxis) return EP_ERR_UNSUPPORTED;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return EP_ERR_NO_DEVICE;
  }
  double2* scratch = nullptr;
  int r = device_setup(dev, &scratch);
  if (r) return r;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  double2* S = scratch;
  double2* Tsp = scratch + kMaxHalf;
  double2* twx = scratch + 2 * kMaxHalf;
  double2* twy = twx + kMaxAxis;
  double2* twz = twy + kMaxAxis;
  FftPlan p2{}, pY{}, pZ{};
  make_plan(nx / 2, p2);
  make_plan(ny, pY);
  make_plan(nz, pZ);
  Geo g{nx, ny, nz, nx / 2 + 1, (long long)nx * ny * nz, half};
  k_noalloc_twiddles<<<1, 320, 0, st>>>(twx, nx);
  k_noalloc_twiddles<<<1, 320, 0, st>>>(twy, ny);
  k_noalloc_twiddles<<<1, 320, 0, st>>>(twz, nz);
  const long long nlines = (long long)ny * nz;
  int nl = 16;
  while (nl > 1 && x_smem_of(nl, nx) > 110 * 1024) nl /= 2;
  k_x1<double, 0><<<(unsigned)((nlines + nl - 1) / nl), 256, x_smem_of(nl, nx), st>>>(g, d_in, S, p2, twx, nl);
  Arr8<double> ay{};
  ay.a[0] = S;
  LineSet ly{(long long)g.nxh, (long long)g.nxh * ny, (long long)g.nxh, (long long)g.nxh * nz};
  int LT = 16;
  while (LT > 1 && l_smem_of(LT, ny, 2) > 110 * 1024) LT /= 2;
  k_c2c<double, -1><<<dim3((unsigned)((ly.nlines + LT - 1) / LT), 1), 256, l_smem_of(LT, ny, 2), st>>>(ay, ly, pY, twy, LT);
  ConvSpec<double> cs{};
  cs.in[0] = S;
  cs.out[0][0] = Tsp;
  cs.ker[0][0] = d_kernel;
  cs.nout[0] = 1;
  LineSet lz{(long long)g.nxh * ny, 0, (long long)g.nxh * ny, (long long)g.nxh * ny};
  int LZ = 16;
  while (LZ > 1 && l_smem_of(LZ, nz, 3) > 110 * 1024) LZ /= 2;
  k_zconv<double><<<dim3((unsigned)((lz.nlines + LZ - 1) / LZ), 1), 256, l_smem_of(LZ, nz, 3), st>>>(cs, lz, pZ, twz, LZ);
  ay.a[0] = Tsp;
  k_c2c<double, +1><<<dim3((unsigned)((ly.nlines + LT - 1) / LT), 1), 256, l_smem_of(LT, ny, 2), st>>>(ay, ly, pY, twy, LT);
  k_noalloc_xinv<<<(unsigned)((nlines + nl - 1) / nl), 256, x_smem_of(nl, nx), st>>>(
      g, Tsp, d_out, p2, twx, 1.0 / ((double)nx * ny * nz), nl);
  if (cudaGetLastError() != cudaSuccess) return EP_ERR_CUDA;
  return EP_OK;
}
