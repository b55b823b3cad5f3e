// k_noalloc.cu -- residual norms of one block with no device allocation.
//
// Some hosts cannot call cudaMalloc: a Fortran or OpenACC host whose device
// memory is owned by another allocator or framework memory pool, or a host
// that must not allocate once its run has started (fixed memory budget).
// ec2d_residual_norms_noalloc gives them the max / sum-of-squares residual
// norms of a residual array they already hold on the device.  It has the
// two-pass structure of the context path's reduction (tile partials, then a
// per-quantity pass over them; k_residual.cu), with plain warp trees, and its
// tile partials live in a file-scope __device__ array instead of context
// scratch.  As there, the max is taken on the bit patterns
// of |Res| (non-negative doubles order like their bits as integers), so a NaN
// residual gives a NaN max instead of being dropped as fmax would drop it.
//
// Limits and sharing:
//  * at most EC2D_NOALLOC_MAX_CELLS cells per call (8192 tiles of 256 cells);
//    the array holds 8192 x 12 doubles (768 KiB) on every GPU that loads the
//    library, until the process exits;
//  * every call uses the same array; each call first overwrites every
//    partial it later reads, so nothing has to start at zero, but calls
//    that overlap on the GPU (e.g. on two streams) race on the array;
//  * the array's device address is looked up (cudaGetSymbolAddress) with the
//    calling device current on every call made outside stream capture, so a
//    device reset, which reloads the module, never leaves a stale address;
//    a call made during capture uses the address of the last call outside
//    capture on that device, so make the first call on a device before any
//    capture.
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
  __shared__ long long smax[6][TILE / 32];
  __shared__ double ssum[6][TILE / 32];
  int c = blockIdx.x * TILE + threadIdx.x;
  long long vmax[6] = {0, 0, 0, 0, 0, 0};
  double vsum[6] = {0, 0, 0, 0, 0, 0};
  if (c < ncell) {
    for (int m = 0; m < nvar; m++) {
      double r = res[(size_t)c * nvar + m];
      vmax[m] = __double_as_longlong(fabs(r));
      vsum[m] = r * r;
    }
  }
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int m = 0; m < 6; m++) {
    long long a = vmax[m];
    double s = vsum[m];
    for (int o = 16; o > 0; o >>= 1) {
      a = max(a, __shfl_down_sync(0xffffffffu, a, o));
      s += __shfl_down_sync(0xffffffffu, s, o);
    }
    if (lane == 0) { smax[m][w] = a; ssum[m][w] = s; }
  }
  __syncthreads();
  if (threadIdx.x < 6) {
    int m = threadIdx.x;
    long long a = 0;
    double s = 0.0;
    for (int k = 0; k < TILE / 32; k++) { a = max(a, smax[m][k]); s += ssum[m][k]; }
    part[(size_t)blockIdx.x * 12 + m] = __longlong_as_double(a);
    part[(size_t)blockIdx.x * 12 + 6 + m] = s;
  }
}

// fixed-order reduction of the tile partials into out[0..5] = max,
// out[6..11] = sum of squares
// (the maxima again as bit patterns of non-negative doubles)
__global__ void k_noalloc_final(const double *part, int ntiles, double *out) {
  __shared__ double sm[12][32];
  int m = threadIdx.y, lane = threadIdx.x;
  if (m < 6) {
    long long a = 0;
    for (int t = lane; t < ntiles; t += 32) a = max(a, __double_as_longlong(part[(size_t)t * 12 + m]));
    sm[m][lane] = __longlong_as_double(a);
  } else {
    double acc = 0.0;
    for (int t = lane; t < ntiles; t += 32) acc += part[(size_t)t * 12 + m];
    sm[m][lane] = acc;
  }
  __syncthreads();
  if (lane == 0) {
    if (m < 6) {
      long long a = 0;
      for (int k = 0; k < 32; k++) a = max(a, __double_as_longlong(sm[m][k]));
      out[m] = __longlong_as_double(a);
    } else {
      double a = 0.0;
      for (int k = 0; k < 32; k++) a += sm[m][k];
      out[m] = a;
    }
  }
}

// device address of the scratch array on the current device: looked up on
// every call outside stream capture (a device reset reloads the module and
// may move the array), the last such address reused during capture
int scratch_for_current_device(cudaStream_t s, double **out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) return EC2D_ERR_CUDA;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cap) != cudaSuccess) return EC2D_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_mu);
  if (cap == cudaStreamCaptureStatusNone || !g_scratch_ptr[dev]) {
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
  cudaStream_t s = (cudaStream_t)stream;
  double *part = nullptr;
  int r = scratch_for_current_device(s, &part);
  if (r) return r;
  int ntiles = (ncell + TILE - 1) / TILE;
  k_noalloc_partial<<<ntiles, TILE, 0, s>>>(res, nvar, ncell, part);
  k_noalloc_final<<<1, dim3(32, 12), 0, s>>>(part, ntiles, out);
  return cudaGetLastError() == cudaSuccess ? EC2D_OK : EC2D_ERR_CUDA;
}
