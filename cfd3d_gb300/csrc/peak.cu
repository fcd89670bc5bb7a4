// peak.cu -- the FP64 pipe's throughput on this GPU: the denominator of the FP64 compute
// roofline that the path's kernels are measured against.  Every thread of a full grid
// runs 16 independent fused multiply-add chains on doubles; the grid is timed with CUDA
// events.  Measurement only: nothing of the solver uses it.
#include <cuda_runtime.h>

#include "cfd3d.h"

namespace {

constexpr int CHAINS = 16;

__global__ void __launch_bounds__(256) k_dfma_peak(double* out, int iters, double a, double b) {
  double x[CHAINS];
#pragma unroll
  for (int q = 0; q < CHAINS; ++q) x[q] = 1.0e-9 * threadIdx.x + q;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int q = 0; q < CHAINS; ++q) x[q] = fma(x[q], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int q = 0; q < CHAINS; ++q) s += x[q];
  if (s == -1.0) out[0] = s;   // never true: keeps every chain live
}

}  // namespace

extern "C" int cfd3d_fp64_peak(double seconds, double* tflops) {
  if (!tflops || !(seconds > 0.0) || seconds > 60.0) return CFD3D_ERR_ARG;
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return CFD3D_ERR_NODEVICE;
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return CFD3D_ERR_CUDA;
  double* out = nullptr;
  if (cudaMalloc(&out, sizeof(double)) != cudaSuccess) return CFD3D_ERR_NOMEM;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const unsigned grid = (unsigned)nsm * 8u;
  const double threads = (double)grid * 256.0;
  auto run = [&](int iters, double& ms) -> bool {
    cudaEventRecord(e0);
    k_dfma_peak<<<grid, 256>>>(out, iters, 0.9999999, 1.0e-7);
    cudaEventRecord(e1);
    if (cudaEventSynchronize(e1) != cudaSuccess) return false;
    float f = 0.0f;
    cudaEventElapsedTime(&f, e0, e1);
    ms = f;
    return cudaGetLastError() == cudaSuccess;
  };
  int rc = CFD3D_OK;
  double ms = 0.0;
  int iters = 2000;
  if (!run(iters, ms) || !run(iters, ms)) rc = CFD3D_ERR_CUDA;   // (the first one warms up)
  if (rc == CFD3D_OK) {
    // one launch of about `seconds`, capped so that its iteration count fits an int
    const double scale = seconds * 1e3 / (ms > 1e-3 ? ms : 1e-3);
    iters = (int)(iters * scale < 2.0e9 ? iters * scale : 2.0e9);
    if (iters < 2000) iters = 2000;
    if (!run(iters, ms)) rc = CFD3D_ERR_CUDA;
    else *tflops = 2.0 * CHAINS * (double)iters * threads / (ms * 1e-3) / 1e12;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  return rc;
}
