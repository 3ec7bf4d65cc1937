// amr_cfl_dt_static: the CFL reduction (main.cpp:209-230) for callers that may
// not allocate device memory.
//
// Some hosts cannot call cudaMalloc at the point where they need the time step:
// code running inside a captured CUDA graph, allocator-free real-time loops,
// or frameworks that own every device allocation and forbid others.  This
// entry point takes the caller's device arrays and keeps its only scratch --
// one partial result per block -- in a fixed array in this file's device
// globals, so it allocates nothing.  Every GPU that loads the library holds
// that array (kCflStaticMaxBlocks doubles, 512 KiB) until the process exits.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>

#include "../../include/amr2d_mhd.h"
#include "stage.cuh"

namespace amr {

constexpr int kCflStaticMaxBlocks = 1 << 16;

// per-block min(dx,dy)/lambda_b of the last call; shared by every call
static __device__ __align__(256) double g_cfl_scratch[kCflStaticMaxBlocks];

// main.cpp:211-228 for one block of the dense array: lambda1 takes |rho| +
// c_f,x (W[..][0], main.cpp:222) and lambda2 |u| + c_f,y (:224) over the
// interior cells
template <int NG>
__global__ void __launch_bounds__(256) k_cfl_static_blocks(const double *U, const double *dxdy, double gamma,
                                                           double *scratch) {
  constexpr int N = Geo<NG>::N, NN = N * N, HI = Geo<NG>::HI;
  __shared__ double red[8];
  const double *u0 = U + static_cast<size_t>(blockIdx.x) * 8 * NN;
  double m = 0.;
  for (int c = threadIdx.x; c < NN; c += blockDim.x) {
    const int i = c % N, j = c / N;
    if (i < NG || i > HI || j < NG || j > HI) continue;
    double u[8], w[8];
#pragma unroll
    for (int k = 0; k < 8; k++) u[k] = u0[k * NN + c];
    cons2prim_cell<double>(u, w, gamma);
    const double v1 = fabs(w[0]) + fast_speed<double>(w, gamma, 5);
    const double v2 = fabs(w[1]) + fast_speed<double>(w, gamma, 6);
    // a NaN speed (e.g. a negative pressure) poisons the block's value
    m = (isnan(v1) || isnan(v2)) ? NAN : smax(smax(m, v1), v2);
  }
  for (int o = 16; o > 0; o >>= 1) {
    const double v = __shfl_xor_sync(0xffffffffu, m, o);
    m = (isnan(v) || isnan(m)) ? NAN : (m < v ? v : m);
  }
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double mm = red[0];
    for (int q = 1; q < static_cast<int>(blockDim.x >> 5); q++)
      mm = (isnan(red[q]) || isnan(mm)) ? NAN : (mm < red[q] ? red[q] : mm);
    scratch[blockIdx.x] = smin(dxdy[2 * blockIdx.x], dxdy[2 * blockIdx.x + 1]) / mm;
  }
}

// lambda = min(1e6, min over blocks) (main.cpp:209,228); a NaN block value
// makes the result NaN, which the caller's invalid-dt check catches
__global__ void k_cfl_static_min(const double *scratch, int n, double *out) {
  __shared__ double red[32];
  double m = 1.E6;
  bool nan = false;
  for (int b = threadIdx.x; b < n; b += blockDim.x) {
    const double v = scratch[b];
    nan |= isnan(v);
    m = v < m ? v : m;
  }
  nan = __syncthreads_or(nan);
  for (int o = 16; o > 0; o >>= 1) {
    const double v = __shfl_xor_sync(0xffffffffu, m, o);
    m = v < m ? v : m;
  }
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double mm = red[0];
    for (int q = 1; q < static_cast<int>(blockDim.x >> 5); q++) mm = red[q] < mm ? red[q] : mm;
    *out = nan ? NAN : mm;
  }
}

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_mu;
double *g_scratch_ptr[kMaxDevices] = {nullptr};

// Set-up of the current device, once per device: the device address of
// g_cfl_scratch (in host code the symbol is only a stand-in, not a device
// address), and every kernel of this entry point loaded now (under lazy
// module loading a kernel first launched inside a stream capture would load
// there).  The cached address belongs to the device's context: after a
// cudaDeviceReset it is stale, so this entry point is not used again in that
// process.
cudaError_t scratch_for_current_device(double **out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_ptr[dev]) {
    cudaFuncAttributes fa;
    if ((e = cudaFuncGetAttributes(&fa, k_cfl_static_blocks<2>)) != cudaSuccess) return e;
    if ((e = cudaFuncGetAttributes(&fa, k_cfl_static_blocks<4>)) != cudaSuccess) return e;
    if ((e = cudaFuncGetAttributes(&fa, k_cfl_static_min)) != cudaSuccess) return e;
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_cfl_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_ptr[dev] = static_cast<double *>(p);
  }
  *out = g_scratch_ptr[dev];
  return cudaSuccess;
}
}  // namespace

}  // namespace amr

extern "C" int amr_cfl_dt_static(const double *U, int32_t nblocks, int32_t nghosts, const double *dxdy,
                                 double gamma, double *dt_per_cfl_out, void *stream) {
  using namespace amr;
  if (!U || !dxdy || !dt_per_cfl_out || nblocks <= 0) return AMR_E_ARG;
  if (nblocks > kCflStaticMaxBlocks) return AMR_E_TOO_LARGE;
  if (nghosts != 2 && nghosts != 4) return AMR_E_CONFIG;
  // an error the caller's own earlier work left pending is theirs: report
  // it without clearing it, and launch nothing
  if (cudaPeekAtLastError() != cudaSuccess) return AMR_E_CUDA;
  double *scratch = nullptr;
  if (scratch_for_current_device(&scratch) != cudaSuccess) return AMR_E_CUDA;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (nghosts == 2) k_cfl_static_blocks<2><<<nblocks, 256, 0, s>>>(U, dxdy, gamma, scratch);
  else k_cfl_static_blocks<4><<<nblocks, 256, 0, s>>>(U, dxdy, gamma, scratch);
  if (cudaGetLastError() != cudaSuccess) return AMR_E_CUDA;
  k_cfl_static_min<<<1, 1024, 0, s>>>(scratch, nblocks, dt_per_cfl_out);
  return cudaGetLastError() == cudaSuccess ? AMR_OK : AMR_E_CUDA;
}
