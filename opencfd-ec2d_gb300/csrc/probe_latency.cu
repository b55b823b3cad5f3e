// probe_latency.cu -- standalone micro-benchmark (not part of libec2d_gpu.so):
// clock64 cycles per operation of a dependent chain (FP64 fma, FP64 mul+add,
// FP64 divide, FP32 fma) for 1, 4 and 8 warps of one CTA, and the cost of
// __syncthreads and of a thread-block-cluster barrier.  These numbers set the
// floor of the per-plane cost of the LU-SGS wavefront sweep, whose critical
// path is a chain of dependent arithmetic plus one barrier per plane.
// Build and run: nvcc -gencode arch=compute_103a,code=sm_103a -O3 -o lat probe_latency.cu && ./lat
#include <cmath>
#include <cstdio>
#include <cstring>
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
// ILP independent chains per thread: does one warp overlap independent FP64
// instructions, or does each occupy the sub-partition for its full latency?
template <int ILP>
__global__ void k_dfma_ilp(double *out, long long *cyc, double a, double b, int n) {
  double x[ILP];
#pragma unroll
  for (int q = 0; q < ILP; q++) x[q] = a + threadIdx.x + q;
  long long t0 = clock64();
  for (int k = 0; k < n; k++) {
#pragma unroll
    for (int u = 0; u < 8; u++)
#pragma unroll
      for (int q = 0; q < ILP; q++) x[q] = fma(x[q], b, a);
  }
  long long t1 = clock64();
  double s = 0.0;
#pragma unroll
  for (int q = 0; q < ILP; q++) s += x[q];
  out[threadIdx.x] = s; cyc[threadIdx.x] = t1 - t0;
}
// the same with only `lanes` lanes of each warp active
__global__ void k_dfma_lanes(double *out, long long *cyc, double a, double b, int n, int lanes) {
  double x = a + threadIdx.x;
  long long t0 = clock64();
  if ((threadIdx.x & 31) < lanes)
    for (int k = 0; k < n; k++) {
#pragma unroll
      for (int u = 0; u < 8; u++) x = fma(x, b, a);
    }
  long long t1 = clock64();
  out[threadIdx.x] = x; cyc[threadIdx.x] = t1 - t0;
}
// largest |x * rcp.approx.ftz.f64(x) - 1| over mantissas in [1, 2) (exact
// residual by fma), as the bit pattern of a non-negative double
__global__ void k_rcp_err(unsigned long long *worst, int per_thread) {
  unsigned long long t = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
  double m = 0.0;
  for (int k = 0; k < per_thread; k++) {
    unsigned long long h = (t * per_thread + k) * 0x9E3779B97F4A7C15ull;
    h ^= h >> 29;
    double x = __longlong_as_double((long long)(0x3FF0000000000000ull | (h & 0x000FFFFFFFFFFFFFull)));
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
    double e = fabs(fma(-x, r, 1.0));
    m = e > m ? e : m;
  }
  atomicMax(worst, (unsigned long long)__double_as_longlong(m));
}
// largest distance in ulps between 1/x (IEEE divide) and the reciprocal used
// by the solver kernels (approximate reciprocal + one third-order step), over
// x = mantissa * 2^k, k in [-8, 8]
__global__ void k_rcp3_ulps(unsigned long long *worst, int per_thread) {
  unsigned long long t = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long m = 0;
  for (int k = 0; k < per_thread; k++) {
    unsigned long long h = (t * per_thread + k) * 0xD1B54A32D192ED03ull;
    h ^= h >> 31;
    int ex = (int)((h >> 52) % 17) - 8;
    double x = ldexp(__longlong_as_double((long long)(0x3FF0000000000000ull | (h & 0x000FFFFFFFFFFFFFull))), ex);
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
    const double e = fma(-x, r, 1.0);
    r = fma(r, fma(e, e, e), r);
    long long d = __double_as_longlong(r) - __double_as_longlong(1.0 / x);
    d = d < 0 ? -d : d;
    m = d > m ? d : m;
  }
  atomicMax(worst, (unsigned long long)m);
}
// rsqrt.approx.ftz.f64: largest relative error of y^2 x - 1 (half of it is
// the error of y), and the reciprocal square root refined by one third-order
// step: distance of x * y from the IEEE square root in ulps, and of y from
// 1 / (IEEE square root) in ulps
__global__ void k_rsqrt_err(unsigned long long *worst, int per_thread) {
  unsigned long long t = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
  double m0 = 0.0;
  long long m1 = 0, m2 = 0;
  for (int k = 0; k < per_thread; k++) {
    unsigned long long h = (t * per_thread + k) * 0x9E3779B97F4A7C15ull;
    h ^= h >> 29;
    int ex = (int)((h >> 52) % 17) - 8;
    double x = ldexp(__longlong_as_double((long long)(0x3FF0000000000000ull | (h & 0x000FFFFFFFFFFFFFull))), ex);
    double y;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    double e0 = fabs(fma(-x, y * y, 1.0));
    m0 = e0 > m0 ? e0 : m0;
    const double e = fma(-x, y * y, 1.0);
    const double y3 = fma(y, e * fma(0.375, e, 0.5), y);
    const double sq = __dsqrt_rn(x);
    long long d1 = __double_as_longlong(x * y3) - __double_as_longlong(sq);
    long long d2 = __double_as_longlong(y3) - __double_as_longlong(__ddiv_rn(1.0, sq));
    d1 = d1 < 0 ? -d1 : d1; d2 = d2 < 0 ? -d2 : d2;
    m1 = d1 > m1 ? d1 : m1; m2 = d2 > m2 ? d2 : m2;
  }
  atomicMax(worst, (unsigned long long)__double_as_longlong(m0));
  atomicMax(worst + 1, (unsigned long long)m1);
  atomicMax(worst + 2, (unsigned long long)m2);
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
  for (int warps : {1, 4}) {
    k_dfma_ilp<2><<<1, 32 * warps>>>(out, cyc, 0.5, 0.999, n);
    cudaMemcpy(h, cyc, 8 * sizeof(long long), cudaMemcpyDeviceToHost);
    printf("dfma ILP2 warps=%d  cycles per instruction = %.2f\n", warps, h[0] / (16.0 * n));
    k_dfma_ilp<4><<<1, 32 * warps>>>(out, cyc, 0.5, 0.999, n);
    cudaMemcpy(h, cyc, 8 * sizeof(long long), cudaMemcpyDeviceToHost);
    printf("dfma ILP4 warps=%d  cycles per instruction = %.2f\n", warps, h[0] / (32.0 * n));
    k_dfma_ilp<8><<<1, 32 * warps>>>(out, cyc, 0.5, 0.999, n);
    cudaMemcpy(h, cyc, 8 * sizeof(long long), cudaMemcpyDeviceToHost);
    printf("dfma ILP8 warps=%d  cycles per instruction = %.2f\n", warps, h[0] / (64.0 * n));
  }
  for (int lanes : {1, 8, 16}) {
    k_dfma_lanes<<<1, 32>>>(out, cyc, 0.5, 0.999, n, lanes);
    cudaMemcpy(h, cyc, 8 * sizeof(long long), cudaMemcpyDeviceToHost);
    printf("dfma lanes=%d  cycles/op = %.2f\n", lanes, h[0] / (8.0 * n));
  }
  {
    unsigned long long *w, hw = 0;
    cudaMalloc(&w, sizeof(unsigned long long));
    cudaMemset(w, 0, sizeof(unsigned long long));
    k_rcp_err<<<608, 256>>>(w, 256);  // 40 M mantissas
    cudaMemcpy(&hw, w, sizeof(hw), cudaMemcpyDeviceToHost);
    double e; memcpy(&e, &hw, sizeof(e));
    printf("rcp.approx.ftz.f64 max relative error over 4.0e7 mantissas = %.3e (2^%.2f)\n", e, log2(e));
    cudaFree(w);
  }
  {
    unsigned long long *w, hw = 0;
    cudaMalloc(&w, sizeof(unsigned long long));
    cudaMemset(w, 0, sizeof(unsigned long long));
    k_rcp3_ulps<<<608, 256>>>(w, 256);
    cudaMemcpy(&hw, w, sizeof(hw), cudaMemcpyDeviceToHost);
    printf("third-order reciprocal: max distance from 1/x over 4.0e7 samples = %llu ulp\n", hw);
    cudaFree(w);
  }
  {
    unsigned long long *w, hw[3] = {0, 0, 0};
    cudaMalloc(&w, 3 * sizeof(unsigned long long));
    cudaMemset(w, 0, 3 * sizeof(unsigned long long));
    k_rsqrt_err<<<608, 256>>>(w, 256);
    cudaMemcpy(hw, w, sizeof(hw), cudaMemcpyDeviceToHost);
    double e; memcpy(&e, &hw[0], sizeof(e));
    printf("rsqrt.approx.ftz.f64: max |x y^2 - 1| over 4.0e7 samples = %.3e (2^%.2f)\n", e, log2(e));
    printf("third-order rsqrt: x*y vs sqrt(x) max %llu ulp, y vs 1/sqrt(x) max %llu ulp\n", hw[1], hw[2]);
    cudaFree(w);
  }
  cudaError_t e = cudaDeviceSynchronize();
  printf("status %s\n", cudaGetErrorString(e));
  return e != cudaSuccess;
}
