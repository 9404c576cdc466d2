// peaks.cu - FP32 and FP64 FMA pipe rates of the current GPU, measured.
//
// The roofline of the kernels that run on the SIMT pipes (the double-float
// residual and escalation, the wide-accumulation trailing update) needs the
// FMA rates of this GPU; the measured HBM and tensor peaks do not cover them.
// Each thread runs 8 independent FMA chains (enough to cover the FMA latency
// at full occupancy) for a fixed number of iterations; the rate is
// 2 flops per FMA over the CUDA-event time of the launch.
#include <cuda_runtime.h>

#include "../../include/fdmgpu.h"

namespace {

template <typename T>
__global__ void __launch_bounds__(256) k_fma_chain(T* out, int iters, T a, T b) {
  T x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
      x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
  }
  const T s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == (T)-1.2345) out[blockIdx.x] = s;  // keeps the chains live; never true for these inputs
}

template <typename T>
double rate(int iters) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = sms * 8;
  T* out = nullptr;
  if (cudaMalloc(&out, blocks * sizeof(T)) != cudaSuccess) return -1.0;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 4; ++rep) {  // the first launch carries module loading
    cudaEventRecord(e0);
    k_fma_chain<T><<<blocks, 256>>>(out, iters, (T)0.999999, (T)1e-7);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (cudaGetLastError() != cudaSuccess) return -1.0;
  const double fmas = (double)blocks * 256 * iters * 16 * 8;
  return 2.0 * fmas / (best * 1e-3) / 1e12;
}

}  // namespace

extern "C" fdmgpu_status fdmgpu_measure_pipe_peaks(double* fp32_tflops, double* fp64_tflops) {
  if (!fp32_tflops || !fp64_tflops) return FDMGPU_ERR_ARG;
  *fp32_tflops = rate<float>(4096);
  *fp64_tflops = rate<double>(256);
  return (*fp32_tflops > 0 && *fp64_tflops > 0) ? FDMGPU_OK : FDMGPU_ERR_CUDA;
}
