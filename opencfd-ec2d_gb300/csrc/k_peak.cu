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

#include <algorithm>
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

// The cost model of the latency-bound kernels: one CTA of `warps` warps,
// every thread runs C independent chains of `iters` dependent operations;
// lane 0 of each warp records clock64 cycles per operation and chain.
// OP 0: FP64 fma; 1: FP64 divide; 2: the refined FP64 reciprocal of the face
// and wavefront paths (rcp.approx + one third-order step); 3: FP32 fma.
template <int C, int OP>
__global__ void __launch_bounds__(1024) k_op_cycles(int iters, double *cyc) {
  double a[C];
  float f[C];
#pragma unroll
  for (int k = 0; k < C; k++) {
    a[k] = 1.0 + 1e-3 * (threadIdx.x + k);
    f[k] = 1.0f + 1e-3f * (threadIdx.x + k);
  }
  __syncthreads();
  const long long t0 = clock64();
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int k = 0; k < C; k++) {
      if (OP == 0) a[k] = fma(a[k], 0.999, 0.001);
      if (OP == 1) a[k] = 1.5 / a[k];  // stays between a and 1.5 / a
      if (OP == 2) {
        double r;
        asm volatile("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(a[k]));
        const double e = fma(-a[k], r, 1.0);
        a[k] = 1.5 * fma(r, fma(e, e, e), r);
      }
      if (OP == 3) f[k] = fmaf(f[k], 0.999f, 0.001f);
    }
  }
  const long long t1 = clock64();
  double sum = 0.0;
#pragma unroll
  for (int k = 0; k < C; k++) sum += a[k] + (double)f[k];
  if ((threadIdx.x & 31) == 0) cyc[threadIdx.x >> 5] = (double)(t1 - t0) / ((double)iters * C) + (sum == -1.0);
}

// barriers: OP 4 a CTA barrier per iteration; OP 5 a cluster barrier
// (arrive.release + wait.acquire) per iteration, launched as one cluster
template <int OP>
__global__ void __launch_bounds__(1024) k_barrier_cycles(int iters, double *cyc) {
  __syncthreads();
  const long long t0 = clock64();
  for (int it = 0; it < iters; it++) {
    if (OP == 4) __syncthreads();
    else asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
  }
  const long long t1 = clock64();
  if (threadIdx.x == 0 && blockIdx.x == 0) cyc[0] = (double)(t1 - t0) / iters;
}

// The refined reciprocal against the IEEE quotient on n inputs spread over
// [2^-8, 2^9) by a hash of the index: per block the largest relative error
// of rcp.approx and the largest distance of the refined value in ulps.
__global__ void k_rcp_check(long long n, double *out) {
  __shared__ double s_rel[256], s_ulp[256];
  double rel = 0.0, ulp = 0.0;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    unsigned long long h = (unsigned long long)k * 0x9E3779B97F4A7C15ull;
    h ^= h >> 29;
    h *= 0xBF58476D1CE4E5B9ull;
    h ^= h >> 32;
    const double m = 1.0 + (double)(h >> 12) * 0x1.0p-52;       // [1, 2)
    const double x = ldexp(m, (int)((h >> 4) % 17) - 8);         // [2^-8, 2^9)
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
    const double q = 1.0 / x;  // IEEE quotient
    rel = fmax(rel, fabs(r - q) / q);
    const double e = fma(-x, r, 1.0);
    const double rr = fma(r, fma(e, e, e), r);
    const double u = fabs(rr - q) / (nextafter(q, 2.0 * q) - q);
    ulp = fmax(ulp, u);
  }
  s_rel[threadIdx.x] = rel;
  s_ulp[threadIdx.x] = ulp;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      s_rel[threadIdx.x] = fmax(s_rel[threadIdx.x], s_rel[threadIdx.x + w]);
      s_ulp[threadIdx.x] = fmax(s_ulp[threadIdx.x], s_ulp[threadIdx.x + w]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) { out[2 * blockIdx.x] = s_rel[0]; out[2 * blockIdx.x + 1] = s_ulp[0]; }
}

template <int OP>
void launch_op(int chains, int warps, int iters, double *d) {
  switch (chains) {
    case 1: k_op_cycles<1, OP><<<1, warps * 32>>>(iters, d); break;
    case 2: k_op_cycles<2, OP><<<1, warps * 32>>>(iters, d); break;
    case 4: k_op_cycles<4, OP><<<1, warps * 32>>>(iters, d); break;
    default: k_op_cycles<8, OP><<<1, warps * 32>>>(iters, d); break;
  }
}

}  // namespace

extern "C" int ec2d_measure_op_cycles(int op, int warps, int chains, double *cycles) {
  if (!cycles || op < 0 || op > 5 || warps < 1 || warps > 32 || (chains != 1 && chains != 2 && chains != 4 && chains != 8))
    return EC2D_ERR_ARG;
  double *d = nullptr;
  if (cudaMalloc(&d, 32 * sizeof(double)) != cudaSuccess) return EC2D_ERR_NOMEM;
  const int iters = op == 1 ? 512 : 4096;
  double best = 0.0;
  for (int rep = 0; rep < 3; rep++) {  // the first launch warms up
    if (op == 0) launch_op<0>(chains, warps, iters, d);
    else if (op == 1) launch_op<1>(chains, warps, iters, d);
    else if (op == 2) launch_op<2>(chains, warps, iters, d);
    else if (op == 3) launch_op<3>(chains, warps, iters, d);
    else if (op == 4) k_barrier_cycles<4><<<1, warps * 32>>>(iters, d);
    else {
      // a cluster of `chains` CTAs of `warps` warps each
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(chains);
      cfg.blockDim = dim3(warps * 32);
      cudaLaunchAttribute attr[1];
      attr[0].id = cudaLaunchAttributeClusterDimension;
      attr[0].val.clusterDim.x = chains;
      attr[0].val.clusterDim.y = 1;
      attr[0].val.clusterDim.z = 1;
      cfg.attrs = attr;
      cfg.numAttrs = 1;
      cudaLaunchKernelEx(&cfg, k_barrier_cycles<5>, iters, d);
    }
    const int nw = op >= 4 ? 1 : warps;
    double h[32];
    if (cudaMemcpy(h, d, nw * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess) {
      cudaFree(d);
      return EC2D_ERR_CUDA;
    }
    double mean = 0.0;
    for (int w = 0; w < nw; w++) mean += h[w] / nw;
    if (rep > 0 && (best == 0.0 || mean < best)) best = mean;
  }
  cudaFree(d);
  if (cudaGetLastError() != cudaSuccess) return EC2D_ERR_CUDA;
  *cycles = best;
  return EC2D_OK;
}

extern "C" int ec2d_check_reciprocal(long long n, double *approx_rel, double *refined_ulps) {
  if (n < 1 || !approx_rel || !refined_ulps) return EC2D_ERR_ARG;
  const int blocks = 304, threads = 256;
  double *d = nullptr;
  if (cudaMalloc(&d, 2 * blocks * sizeof(double)) != cudaSuccess) return EC2D_ERR_NOMEM;
  k_rcp_check<<<blocks, threads>>>(n, d);
  double h[2 * 304];
  const cudaError_t err = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (err != cudaSuccess || cudaGetLastError() != cudaSuccess) return EC2D_ERR_CUDA;
  double rel = 0.0, ulp = 0.0;
  for (int b = 0; b < blocks; b++) { rel = std::max(rel, h[2 * b]); ulp = std::max(ulp, h[2 * b + 1]); }
  *approx_rel = rel;
  *refined_ulps = ulp;
  return EC2D_OK;
}

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
