// Live arithmetic-rate probe: the denominators of the compute roofline
// (FP64 FMA, FP64 divide and FP32 FMA throughput of this GPU), measured with
// CUDA events on independent FMA chains; and an evaluator of the FAST FP64
// reciprocal / square-root forms for their error-bound tests.
#include <cuda_runtime.h>
#include <cstdint>

#include "../../include/weno_gb300.h"
#include "fp64_fast.cuh"

namespace {

template <class T>
__global__ void fma_chains(T* out, int iters, T a, T b) {
  T x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
    x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

__global__ void div_chains(double* out, int iters, double b) {
  double x0 = threadIdx.x + 1.0, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  for (int i = 0; i < iters; ++i) {
    x0 = b / x0 + 1.0; x1 = b / x1 + 1.0; x2 = b / x2 + 1.0; x3 = b / x3 + 1.0;
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3;
}

__global__ void k_fast_math(const double* x, double* out, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double v = x[i];
  out[i] = weno::f64fast::rcp(v);
  out[n + i] = weno::f64fast::rsqrt(v);
  out[2 * n + i] = weno::f64fast::sqrt(v);
  out[3 * n + i] = weno::f64fast::rcp2(v);
}

template <class F>
cudaError_t timed(F launch, cudaStream_t st, float* ms) {
  cudaEvent_t e0, e1;
  cudaError_t e;
  if ((e = cudaEventCreate(&e0))) return e;
  if ((e = cudaEventCreate(&e1))) return e;
  launch();  // warm-up
  cudaEventRecord(e0, st);
  launch();
  cudaEventRecord(e1, st);
  e = cudaEventSynchronize(e1);
  if (!e) e = cudaEventElapsedTime(ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (!e) e = cudaGetLastError();
  return e;
}

}  // namespace

extern "C" int weno_probe_rates(double* fp64_tflops, double* fp64_div_per_s, double* fp32_tflops, void* stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) return WENO_ERR_CUDA;
  const int blocks = sms * 8, threads = 256;
  double* buf = nullptr;
  if (cudaMalloc(&buf, sizeof(double) * blocks * threads)) return WENO_ERR_CUDA;
  float ms = 0.f;
  const double lanes = (double)blocks * threads;
  const int it64 = 1500, itdiv = 200, it32 = 60000;
  cudaError_t e = timed([&] { fma_chains<double><<<blocks, threads, 0, st>>>(buf, it64, 0.999, 1e-3); }, st, &ms);
  if (!e && fp64_tflops) *fp64_tflops = 2.0 * 8 * it64 * lanes / (ms * 1e-3) / 1e12;
  if (!e) e = timed([&] { div_chains<<<blocks, threads, 0, st>>>(buf, itdiv, 3.0); }, st, &ms);
  if (!e && fp64_div_per_s) *fp64_div_per_s = 4.0 * itdiv * lanes / (ms * 1e-3);
  if (!e)
    e = timed([&] { fma_chains<float><<<blocks, threads, 0, st>>>((float*)buf, it32, 0.999f, 1e-3f); }, st, &ms);
  if (!e && fp32_tflops) *fp32_tflops = 2.0 * 8 * it32 * lanes / (ms * 1e-3) / 1e12;
  cudaFree(buf);
  return e ? WENO_ERR_CUDA : WENO_OK;
}

extern "C" int weno_fast_math_eval(const double* x, double* out, int64_t n, void* stream) {
  if (n < 0 || (n > 0 && (!x || !out))) return WENO_ERR_ARG;
  if (n == 0) return WENO_OK;
  const int threads = 256;
  const int64_t blocks = (n + threads - 1) / threads;
  if (blocks > 0x7fffffff) return WENO_ERR_SHAPE;
  k_fast_math<<<(unsigned)blocks, threads, 0, static_cast<cudaStream_t>(stream)>>>(x, out, n);
  return cudaGetLastError() ? WENO_ERR_CUDA : WENO_OK;
}
