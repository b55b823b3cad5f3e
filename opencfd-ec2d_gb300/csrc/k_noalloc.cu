// k_noalloc.cu -- residual norms of one block with no device allocation.
//
// Some hosts cannot call cudaMalloc: a Fortran or OpenACC host whose device
// memory is owned by another allocator or framework memory pool, or a host
// that must not allocate once its run has started (fixed memory budget).
// ec2d_residual_norms_noalloc gives them the max / sum-of-squares residual
// norms of a residual array they already hold on the device.  It is the
// two-pass tile reduction of k_norm_partial/k_norm_final, but its tile
// partials live in a file-scope __device__ array instead of context scratch.
//
// Limits and sharing:
//  * at most EC2D_NOALLOC_MAX_CELLS cells per call (8192 tiles of 256 cells);
//    the array holds 8192 x 12 doubles (768 KiB) on every GPU that loads the
//    library, until the process exits;
//  * every call uses the same array; each call first overwrites every
//    partial it later reads, so nothing has to start at zero, but calls
//    that overlap on the GPU (e.g. on two streams) race on the array;
//  * the first call on a device looks up the array's device address
//    (cudaGetSymbolAddress) with that device current; make that first call
//    before any stream capture.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "../../include/ec2d_gpu.h"

namespace {

constexpr int TILE = 256;
constexpr int MAX_TILES = EC2D_NOALLOC_MAX_CELLS / TILE;
constexpr int MAX_DEVICES = 64;

static __device__ __align__(256) double g_norm_scratch[MAX_TILES * 12];

std::mutex g_mu;
double *g_scratch_ptr[MAX_DEVICES] = {nullptr};

// per-tile max |Res| and sum Res^2 of each variable (nvar <= 6)
__global__ void __launch_bounds__(TILE) k_noalloc_partial(const double *res, int nvar, int ncell, double *part) {
  __shared__ double smax[6][TILE / 32], ssum[6][TILE / 32];
  int c = blockIdx.x * TILE + threadIdx.x;
  double vmax[6] = {0, 0, 0, 0, 0, 0}, vsum[6] = {0, 0, 0, 0, 0, 0};
  if (c < ncell) {
    for (int m = 0; m < nvar; m++) {
      double r = res[(size_t)c * nvar + m];
      vmax[m] = fabs(r);
      vsum[m] = r * r;
    }
  }
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int m = 0; m < 6; m++) {
    double a = vmax[m], s = vsum[m];
    for (int o = 16; o > 0; o >>= 1) {
      a = fmax(a, __shfl_down_sync(0xffffffffu, a, o));
      s += __shfl_down_sync(0xffffffffu, s, o);
    }
    if (lane == 0) { smax[m][w] = a; ssum[m][w] = s; }
  }
  __syncthreads();
  if (threadIdx.x < 6) {
    int m = threadIdx.x;
    double a = 0.0, s = 0.0;
    for (int k = 0; k < TILE / 32; k++) { a = fmax(a, smax[m][k]); s += ssum[m][k]; }
    part[(size_t)blockIdx.x * 12 + m] = a;
    part[(size_t)blockIdx.x * 12 + 6 + m] = s;
  }
}

// fixed-order reduction of the tile partials into out[0..5] = max,
// out[6..11] = sum of squares
__global__ void k_noalloc_final(const double *part, int ntiles, double *out) {
  __shared__ double sm[12][32];
  int m = threadIdx.y, lane = threadIdx.x;
  double acc = 0.0;
  for (int t = lane; t < ntiles; t += 32) {
    double v = part[(size_t)t * 12 + m];
    acc = (m < 6) ? fmax(acc, v) : acc + v;
  }
  sm[m][lane] = acc;
  __syncthreads();
  if (lane == 0) {
    double a = 0.0;
    for (int k = 0; k < 32; k++) a = (m < 6) ? fmax(a, sm[m][k]) : a + sm[m][k];
    out[m] = a;
  }
}

// device address of the scratch array on the current device, looked up once
int scratch_for_current_device(double **out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) return EC2D_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_ptr[dev]) {
    double *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress((void **)&p, g_norm_scratch);
    if (e != cudaSuccess || !p) {
      fprintf(stderr, "ec2d_residual_norms_noalloc: cudaGetSymbolAddress failed: %s\n", cudaGetErrorString(e));
      return EC2D_ERR_CUDA;
    }
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return EC2D_OK;
}

}  // namespace

extern "C" int ec2d_residual_norms_noalloc(const double *res, int nvar, int ncell, double *out, void *stream) {
  if (!res || !out || nvar < 1 || nvar > 6 || ncell < 1) return EC2D_ERR_ARG;
  if (ncell > EC2D_NOALLOC_MAX_CELLS) {
    fprintf(stderr, "ec2d_residual_norms_noalloc: %d cells exceed the limit of %d\n", ncell, EC2D_NOALLOC_MAX_CELLS);
    return EC2D_ERR_ARG;
  }
  double *part = nullptr;
  int r = scratch_for_current_device(&part);
  if (r) return r;
  cudaStream_t s = (cudaStream_t)stream;
  int ntiles = (ncell + TILE - 1) / TILE;
  k_noalloc_partial<<<ntiles, TILE, 0, s>>>(res, nvar, ncell, part);
  k_noalloc_final<<<1, dim3(32, 12), 0, s>>>(part, ntiles, out);
  return cudaGetLastError() == cudaSuccess ? EC2D_OK : EC2D_ERR_CUDA;
}
