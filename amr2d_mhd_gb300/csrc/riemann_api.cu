// amr_riemann: riemannS (riemannS.cpp:7-56) on the GPU for independent face
// states, every solver including ROE, with the reference's compile-time
// MAG_field (defs.hpp:32) as an argument.  FP64, compiled without FMA
// contraction like the rest of the FP64 path.
#include <cuda_runtime.h>

#include "../../include/amr2d_mhd.h"
#include "physics.cuh"

namespace amr {

template <int FLUX>
__global__ void k_riemann_pairs(const double *wL, const double *wR, double gamma, int dir_y, int mag_field,
                                double *out, int *status, long long n) {
  const long long q = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (q >= n) return;
  double l[8], r[8], f[8];
#pragma unroll
  for (int k = 0; k < 8; k++) { l[k] = wL[8 * q + k]; r[k] = wR[8 * q + k]; f[k] = 0.0; }
  if (dir_y) {  // riemannS.cpp:12-23: the field components only with MAG_field
    l[1] = wL[8 * q + 2]; l[2] = wL[8 * q + 1]; r[1] = wR[8 * q + 2]; r[2] = wR[8 * q + 1];
    if (mag_field) { l[5] = wL[8 * q + 6]; l[6] = wL[8 * q + 5]; r[5] = wR[8 * q + 6]; r[6] = wR[8 * q + 5]; }
  }
  const int rc = riemann<FLUX, double>(l, r, gamma, f);
  double o[8];
#pragma unroll
  for (int k = 0; k < 8; k++) o[k] = f[k];
  if (dir_y) {  // riemannS.cpp:47-55
    o[1] = f[2]; o[2] = f[1];
    if (mag_field) { o[5] = f[6]; o[6] = f[5]; }
  }
#pragma unroll
  for (int k = 0; k < 8; k++) out[8 * q + k] = rc ? 0.0 : o[k];
  status[q] = rc ? AMR_E_HLLC : AMR_OK;
}

}  // namespace amr

extern "C" int amr_riemann(int32_t flux, int32_t dir_y, int32_t mag_field, double gamma, const double *wL,
                           const double *wR, double *flux_out, int32_t *status, int64_t n) {
  using namespace amr;
  if (!wL || !wR || !flux_out || n < 0) return AMR_E_ARG;
  if (flux < FLX_RUSA || flux > FLX_ROE) return AMR_E_CONFIG;
  if (flux == FLX_ROE && mag_field) return AMR_E_UNSUPPORTED;  // riemannS.cpp:39-40
  if (n == 0) return AMR_OK;
  const size_t bytes = sizeof(double) * 8 * static_cast<size_t>(n);
  double *d = nullptr;
  if (cudaMalloc(&d, 3 * bytes + sizeof(int) * static_cast<size_t>(n)) != cudaSuccess) return AMR_E_OOM;
  double *dL = d, *dR = d + 8 * n, *dO = d + 16 * n;
  int *dS = reinterpret_cast<int *>(d + 24 * n);
  int rc = AMR_OK;
  cudaError_t e = cudaMemcpy(dL, wL, bytes, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dR, wR, bytes, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    const int B = 128;
    const unsigned G = static_cast<unsigned>((n + B - 1) / B);
    const int y = dir_y ? 1 : 0, mf = mag_field ? 1 : 0;
    switch (flux) {
      case FLX_RUSA: k_riemann_pairs<FLX_RUSA><<<G, B>>>(dL, dR, gamma, y, mf, dO, dS, n); break;
      case FLX_HLLE: k_riemann_pairs<FLX_HLLE><<<G, B>>>(dL, dR, gamma, y, mf, dO, dS, n); break;
      case FLX_HLLC: k_riemann_pairs<FLX_HLLC><<<G, B>>>(dL, dR, gamma, y, mf, dO, dS, n); break;
      case FLX_HLLD: k_riemann_pairs<FLX_HLLD><<<G, B>>>(dL, dR, gamma, y, mf, dO, dS, n); break;
      default: k_riemann_pairs<FLX_ROE><<<G, B>>>(dL, dR, gamma, y, mf, dO, dS, n); break;
    }
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(flux_out, dO, bytes, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && status)
    e = cudaMemcpy(status, dS, sizeof(int) * static_cast<size_t>(n), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) rc = AMR_E_CUDA;
  cudaFree(d);
  return rc;
}
