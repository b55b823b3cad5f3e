// probe_latency.cu -- standalone micro-benchmark (not part of libec2d_gpu.so):
// clock64 cycles per operation of a dependent chain (FP64 fma, FP64 mul+add,
// FP64 divide, FP32 fma) for 1, 4 and 8 warps of one CTA, and the cost of
// __syncthreads and of a thread-block-cluster barrier.  These numbers set the
// floor of the per-plane cost of the LU-SGS wavefront sweep, whose critical
// path is a chain of dependent arithmetic plus one barrier per plane.
// Build and run: nvcc -gencode arch=compute_103a,code=sm_103a -O3 -o lat probe_latency.cu && ./lat
#include <cstdio>
#include <cuda_runtime.h>
__global__ void k_dfma(double *out, long long *cyc, double a, double b, int n) {
  double x = a + threadIdx.x;
  long long t0 = clock64();
  for (int k = 0; k < n; k++) {
#pragma unroll
    for (int u = 0; u < 8; u++) x = fma(x, b, a);
  }
  long long t1 = clock64();
  out[threadIdx.x] = x; cyc[threadIdx.x] = t1 - t0;
}
__global__ void k_dadd(double *out, long long *cyc, double a, double b, int n) {
  double x = a + threadIdx.x;
  long long t0 = clock64();
  for (int k = 0; k < n; k++) {
#pragma unroll
    for (int u = 0; u < 8; u++) x = x * b + 0.0;
  }
  long long t1 = clock64();
  out[threadIdx.x] = x; cyc[threadIdx.x] = t1 - t0;
}
__global__ void k_ddiv(double *out, long long *cyc, double a, double b, int n) {
  double x = a + threadIdx.x;
  long long t0 = clock64();
  for (int k = 0; k < n; k++) {
#pragma unroll
    for (int u = 0; u < 8; u++) x = b / x;
  }
  long long t1 = clock64();
  out[threadIdx.x] = x; cyc[threadIdx.x] = t1 - t0;
}
__global__ void k_ffma(double *out, long long *cyc, double a, double b, int n) {
  float x = a + threadIdx.x, fb = b, fa = a;
  long long t0 = clock64();
  for (int k = 0; k < n; k++) {
#pragma unroll
    for (int u = 0; u < 8; u++) x = fmaf(x, fb, fa);
  }
  long long t1 = clock64();
  out[threadIdx.x] = x; cyc[threadIdx.x] = t1 - t0;
}
__global__ void k_sync(double *out, long long *cyc, double a, double b, int n) {
  long long t0 = clock64();
  for (int k = 0; k < n * 8; k++) __syncthreads();
  long long t1 = clock64();
  out[threadIdx.x] = a; cyc[threadIdx.x] = t1 - t0;
}
__global__ void k_cluster(double *out, long long *cyc, double a, double b, int n) {
  long long t0 = clock64();
  for (int k = 0; k < n * 8; k++)
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
  long long t1 = clock64();
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  out[t] = a; cyc[t] = t1 - t0;
}
int main() {
  const int n = 1000, T = 256;
  double *out; long long *cyc; long long h[T];
  cudaMalloc(&out, T * 8 * sizeof(double)); cudaMalloc(&cyc, T * 8 * sizeof(long long));
  const char *names[] = {"dfma", "dmul+add", "ddiv", "ffma"};
  void (*ks[])(double *, long long *, double, double, int) = {k_dfma, k_dadd, k_ddiv, k_ffma};
  for (int q = 0; q < 4; q++)
    for (int warps : {1, 4, 8}) {
      ks[q]<<<1, 32 * warps>>>(out, cyc, 0.5, 0.999, 10);
      ks[q]<<<1, 32 * warps>>>(out, cyc, 0.5, 0.999, n);
      cudaMemcpy(h, cyc, 8 * sizeof(long long), cudaMemcpyDeviceToHost);
      printf("%-9s warps=%d  cycles/op per warp chain = %.2f\n", names[q], warps, h[0] / (8.0 * n));
    }
  for (int warps : {1, 3, 8}) {
    k_sync<<<1, 32 * warps>>>(out, cyc, 0.5, 0.999, n);
    cudaMemcpy(h, cyc, 8 * sizeof(long long), cudaMemcpyDeviceToHost);
    printf("syncthreads warps=%d  cycles each = %.2f\n", warps, h[0] / (8.0 * n));
  }
  for (int cs : {2, 4, 8}) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(cs); cfg.blockDim = dim3(32);
    cudaLaunchAttribute at[1]; at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = cs; at[0].val.clusterDim.y = 1; at[0].val.clusterDim.z = 1;
    cfg.attrs = at; cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, k_cluster, out, cyc, 0.5, 0.999, n);
    cudaDeviceSynchronize();
    cudaMemcpy(h, cyc, 8 * sizeof(long long), cudaMemcpyDeviceToHost);
    printf("cluster barrier cs=%d  cycles each = %.2f\n", cs, h[0] / (8.0 * n));
  }
  cudaError_t e = cudaDeviceSynchronize();
  printf("status %s\n", cudaGetErrorString(e));
  return e != cudaSuccess;
}
