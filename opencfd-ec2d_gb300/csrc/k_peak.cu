// k_peak.cu -- measured FP64 FMA throughput of the current GPU, the
// denominator of the FP64 roofline that bounds the residual and sweep kernels
// (every stencil here computes in FP64, and on this part FP64 instructions,
// not HBM bandwidth, set their time).
//
// Every thread runs eight independent FMA chains (a = a b + c, which
// converges to c / (1 - b) = 1 without denormals), so each sub-partition has
// independent FP64 instructions to issue every cycle its FP64 unit accepts one;
// the grid is 8 CTAs of 256 threads per SM.  FLOPs = 2 per FMA.
#include <cuda_runtime.h>

#include <cstdio>

#include "../../include/ec2d_gpu.h"

namespace {

constexpr int CHAINS = 8;

__global__ void __launch_bounds__(256) k_fp64_fma(double *sink, int iters, double b, double c) {
  double a[CHAINS];
#pragma unroll
  for (int k = 0; k < CHAINS; k++) a[k] = 1e-3 * (threadIdx.x + k);
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int k = 0; k < CHAINS; k++) a[k] = fma(a[k], b, c);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < CHAINS; k++) s += a[k];
  if (s == -1.0) sink[blockIdx.x] = s;  // never true; keeps the chains live
}

}  // namespace

extern "C" int ec2d_measure_fp64_peak(double *tflops) {
  if (!tflops) return EC2D_ERR_ARG;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return EC2D_ERR_CUDA;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return EC2D_ERR_CUDA;
  cudaStream_t s = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return EC2D_ERR_CUDA;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int blocks = sms * 8, threads = 256, iters = 2048;
  const double flops = 2.0 * CHAINS * (double)iters * blocks * threads;
  float best = 0.0f;
  for (int rep = 0; rep < 6; rep++) {  // the first launch warms up
    cudaEventRecord(e0, s);
    k_fp64_fma<<<blocks, threads, 0, s>>>(nullptr, iters, 0.999, 0.001);
    cudaEventRecord(e1, s);
    if (cudaEventSynchronize(e1) != cudaSuccess) break;
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && (best == 0.0f || ms < best)) best = ms;
  }
  cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamDestroy(s);
  if (err != cudaSuccess || best <= 0.0f) {
    fprintf(stderr, "ec2d_measure_fp64_peak: %s\n", cudaGetErrorString(err));
    return EC2D_ERR_CUDA;
  }
  *tflops = flops / (best * 1e-3) / 1e12;
  return EC2D_OK;
}
