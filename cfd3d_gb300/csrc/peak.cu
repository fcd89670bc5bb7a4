// peak.cu -- the FP64 pipe's throughput on this GPU: the denominator of the FP64 compute
// roofline that the path's kernels are measured against.  Every thread of a full grid
// runs 16 independent fused multiply-add chains on doubles; the grid is timed with CUDA
// events.  Measurement only: nothing of the solver uses it.
#include <cuda_runtime.h>

#include "cfd3d.h"
#include "df64.cuh"

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

// conversion throughput: each thread converts `reps` values of ordinary magnitude, the
// next one derived from the last by integer operations only; MODE 0 the hardware
// conversion, 1 the integer-pipe one (to_f32 / to_f64)
__global__ void k_fill_ordinary(double* p, long long n) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= n) return;
  unsigned long long z = 99ull + (unsigned long long)t * 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  z ^= z >> 31;
  p[t] = __longlong_as_double((long long)((z & 0x800fffffffffffffull) | ((unsigned long long)(1003 + (int)(z % 40)) << 52)));
}
template <int MODE>
__global__ void k_d2f_rate(const double* in, float* out, long long n, int reps) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= n) return;
  double x = in[t];
  float acc = 0.0f;
  for (int r = 0; r < reps; ++r) {
    acc += MODE ? cfd::to_f32(x) : __double2float_rn(x);
    x = __hiloint2double(__double2hiint(x), __double2loint(x) ^ (r + 1));
  }
  out[t] = acc;
}
template <int MODE>
__global__ void k_f2d_rate(const float* in, double* out, long long n, int reps) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= n) return;
  float x = in[t];
  unsigned acc = 0u;
  for (int r = 0; r < reps; ++r) {
    const double d = MODE ? cfd::to_f64(x) : (double)x;
    acc ^= (unsigned)__double2loint(d) ^ (unsigned)__double2hiint(d);
    x = __uint_as_float(__float_as_uint(x) ^ (unsigned)(r & 7));
  }
  out[t] = (double)acc;
}

}  // namespace

extern "C" int cfd3d_convert_rate(double* rates) {
  if (!rates) return CFD3D_ERR_ARG;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return CFD3D_ERR_NODEVICE;
  const long long n = 1ll << 24;
  const int reps = 64, T = 256;
  const unsigned G = (unsigned)((n + T - 1) / T);
  double *d64 = nullptr, *o64 = nullptr;
  float *f32 = nullptr;
  if (cudaMalloc(&d64, n * 8) != cudaSuccess || cudaMalloc(&o64, n * 8) != cudaSuccess ||
      cudaMalloc(&f32, n * 4) != cudaSuccess) {
    cudaFree(d64); cudaFree(o64); cudaFree(f32);
    return CFD3D_ERR_NOMEM;
  }
  k_fill_ordinary<<<G, T>>>(d64, n);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  int rc = CFD3D_OK;
  auto time = [&](auto launch) -> double {
    launch();   // (warm-up)
    cudaEventRecord(e0);
    launch();
    cudaEventRecord(e1);
    if (cudaEventSynchronize(e1) != cudaSuccess) { rc = CFD3D_ERR_CUDA; return 0.0; }
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    return (double)n * reps / (ms * 1e-3) / 1e9;
  };
  rates[0] = time([&] { k_d2f_rate<0><<<G, T>>>(d64, f32, n, reps); });
  rates[1] = time([&] { k_d2f_rate<1><<<G, T>>>(d64, f32, n, reps); });
  rates[2] = time([&] { k_f2d_rate<0><<<G, T>>>(f32, o64, n, reps); });
  rates[3] = time([&] { k_f2d_rate<1><<<G, T>>>(f32, o64, n, reps); });
  if (cudaGetLastError() != cudaSuccess) rc = CFD3D_ERR_CUDA;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(d64); cudaFree(o64); cudaFree(f32);
  return rc;
}

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
