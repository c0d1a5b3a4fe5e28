// grx_probe.cu -- FP32 FMA throughput of the device, the denominator of the pair
// kernels' roofline (no measured FP32 figure is supplied with the device peaks).
//
// Every thread runs kChains independent FMA chains (enough instruction-level
// parallelism to cover the FMA latency); the grid fills every SM with 1024 threads.
#include "grx_df.cuh"
#include "grx_host.h"

namespace grx {

constexpr int kChains = 8;

__global__ void __launch_bounds__(256) fma_probe_kernel(float* out, int iters, float b, float c) {
  float a[kChains];
#pragma unroll
  for (int k = 0; k < kChains; ++k) a[k] = 1e-3f * (float)(threadIdx.x + k);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 16; ++u)
#pragma unroll
      for (int k = 0; k < kChains; ++k) a[k] = __fmaf_rn(a[k], b, c);
  }
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < kChains; ++k) s += a[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// The double-float elementary functions of the mixed-precision CBMC stages, one value per
// thread: sin and cos of 2 pi v, and the quaternion rotation of (1, 0.5, -0.25) by the
// Philox words of w (checked against FP64 by the tests).
__global__ void df_functions_probe_kernel(const double* v, const uint32_t* w, int n, double* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  df s, c;
  df_sincos_2pi(df_from(v[i]), s, c);
  double x = 1.0, y = 0.5, z = -0.25;
  df_rotate_quaternion(x, y, z, w[3 * i], w[3 * i + 1], w[3 * i + 2]);
  out[5 * i] = df_to(s);
  out[5 * i + 1] = df_to(c);
  out[5 * i + 2] = x;
  out[5 * i + 3] = y;
  out[5 * i + 4] = z;
}

}  // namespace grx

using namespace grx;

extern "C" grx_status grx_probe_df_functions(const double* v, const uint32_t* words, int64_t n, double* out5) {
  GRX_REQUIRE(v && words && out5 && n >= 1 && n <= (1 << 24), "grx_probe_df_functions: bad argument");
  void* mem = nullptr;
  // each segment starts on a 256-byte boundary (the word segment's length is a multiple of 4 only)
  auto up = [](size_t x) { return (x + 255) & ~(size_t)255; };
  const size_t bv = up(n * sizeof(double)), bw = up(3 * n * sizeof(uint32_t)), bo = 5 * n * sizeof(double);
  GRX_CHECK_CUDA(cudaMalloc(&mem, bv + bw + bo), "probe buffers");
  char* m = (char*)mem;
  cudaError_t e = cudaMemcpy(m, v, n * sizeof(double), cudaMemcpyDefault);
  if (e == cudaSuccess) e = cudaMemcpy(m + bv, words, 3 * n * sizeof(uint32_t), cudaMemcpyDefault);
  if (e == cudaSuccess) {
    df_functions_probe_kernel<<<(int)((n + 127) / 128), 128>>>((const double*)m, (const uint32_t*)(m + bv), (int)n,
                                                              (double*)(m + bv + bw));
    count_launch();
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(out5, m + bv + bw, bo, cudaMemcpyDefault);
  cudaFree(mem);
  GRX_CHECK_CUDA(e, "grx_probe_df_functions");
  return GRX_OK;
}

extern "C" grx_status grx_probe_fp32_fma(int32_t iters, double* tflops, float* ms) {
  GRX_REQUIRE(tflops && iters >= 1, "grx_probe_fp32_fma: bad argument");
  int dev = 0, sms = 0;
  GRX_CHECK_CUDA(cudaGetDevice(&dev), "device");
  GRX_CHECK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count");
  const int blocks = 4 * sms, threads = 256;
  float* out = nullptr;
  GRX_CHECK_CUDA(cudaMalloc(&out, (size_t)blocks * threads * sizeof(float)), "probe buffer");
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  fma_probe_kernel<<<blocks, threads>>>(out, 16, 0.999f, 1e-6f);  // warm-up
  count_launch();
  cudaEventRecord(e0);
  fma_probe_kernel<<<blocks, threads>>>(out, iters, 0.999f, 1e-6f);
  count_launch();
  cudaEventRecord(e1);
  const cudaError_t e = cudaEventSynchronize(e1);
  float t = 0.f;
  cudaEventElapsedTime(&t, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  GRX_CHECK_CUDA(e, "probe run");
  const double flop = 2.0 * kChains * 16.0 * (double)iters * blocks * threads;
  *tflops = flop / (t * 1e-3) / 1e12;
  if (ms) *ms = t;
  return GRX_OK;
}
