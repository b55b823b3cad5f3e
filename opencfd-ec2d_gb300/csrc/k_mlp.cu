// k_mlp.cu -- the learned warm start: a coordinate-conditioned MLP trained and
// evaluated with hand-written kernels.  No counterpart in the reference.
//
// Network: 7 inputs (x, y, log10 wall distance, M, AoA, log10 Re, t/c; padded
// to 64 columns) -> H hidden layers of width W with SiLU -> 5 outputs (rho,
// rho u, rho v, E, log1p(nu_tilde Re)); inputs and outputs standardised with
// the dataset's mean and standard deviation.  Weights and activations are
// BF16, accumulation FP32 (the GEMM kernels), master weights and Adam moments
// FP32.
//
// Every GEMM is C[M x N] = A[M x K] . B[N x K]^T with both operands K-major
// (row-major with K contiguous).  Backward passes materialise the transposes
// they need (dZ^T, H^T, W^T) with a tiled transpose kernel, so one GEMM shape
// serves forward, data-gradient and weight-gradient products; the weight
// gradient splits its long K (the batch) over blockIdx.z into partial tiles
// that a second kernel sums in a fixed order (deterministic training).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "ec2d_dev.cuh"
#include "ec2d_internal.h"
#include "ec2d_mlp.h"

namespace ec2d {
namespace mlp {

// ---------------------------------------------------------------------------
// GEMM (legacy tensor path: mma.sync m16n8k16 BF16 -> FP32)
// Tile 128 x 64 x 32, 8 warps (4 along M x 2 along N, 32 x 32 each), two
// cp.async stages, ldmatrix fragment loads from padded shared rows.
// ---------------------------------------------------------------------------
constexpr int BM = 128, BN = 64, BK = 32, LDS = BK + 8;  // padded row: 80 bytes

__device__ __forceinline__ void cp16(void *dst, const void *src) {
  unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

__device__ __forceinline__ void ldsm4(unsigned &r0, unsigned &r1, unsigned &r2, unsigned &r3, const void *p) {
  unsigned a = (unsigned)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(a));
}
__device__ __forceinline__ void mma16816(float *d, const unsigned *a, const unsigned *b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ float silu(float z) { return z / (1.0f + __expf(-z)); }
__device__ __forceinline__ float dsilu(float z) {
  float s = 1.0f / (1.0f + __expf(-z));
  return s * (1.0f + z * (1.0f - s));
}

// A: [M x K] (lda), B: [N x K] (ldb); K range of this CTA: blockIdx.z
__global__ void __launch_bounds__(256) k_gemm_tn(const __nv_bfloat16 *__restrict__ A, int lda,
                                                 const __nv_bfloat16 *__restrict__ B, int ldb, int K, int ksplit,
                                                 Epi e) {
  __shared__ __align__(16) __nv_bfloat16 sA[2][BM * LDS];
  __shared__ __align__(16) __nv_bfloat16 sB[2][BN * LDS];
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
  const int kc = K / ksplit, kb = blockIdx.z * kc, nk = kc / BK;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int wm = warp & 3, wn = warp >> 2;
  float acc[2][4][4];
#pragma unroll
  for (int a = 0; a < 2; a++)
#pragma unroll
    for (int b = 0; b < 4; b++)
#pragma unroll
      for (int c = 0; c < 4; c++) acc[a][b][c] = 0.0f;

  auto load = [&](int st, int kt) {
    const int k0 = kb + kt * BK;
#pragma unroll
    for (int r = 0; r < 2; r++) {  // A: 128 rows x 4 chunks of 8
      int c = tid + r * 256, row = c >> 2, ch = c & 3;
      cp16(&sA[st][row * LDS + ch * 8], A + (size_t)(m0 + row) * lda + k0 + ch * 8);
    }
    {  // B: 64 rows x 4 chunks
      int row = tid >> 2, ch = tid & 3;
      cp16(&sB[st][row * LDS + ch * 8], B + (size_t)(n0 + row) * ldb + k0 + ch * 8);
    }
    cp_commit();
  };

  load(0, 0);
  for (int kt = 0; kt < nk; kt++) {
    const int st = kt & 1;
    if (kt + 1 < nk) {
      load(st ^ 1, kt + 1);
      cp_wait<1>();
    } else {
      cp_wait<0>();
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; kk += 16) {
      unsigned af[2][4], bfr[4][2];
#pragma unroll
      for (int mi = 0; mi < 2; mi++) {
        const __nv_bfloat16 *p = &sA[st][(wm * 32 + mi * 16 + (lane & 15)) * LDS + kk + (lane >> 4) * 8];
        ldsm4(af[mi][0], af[mi][1], af[mi][2], af[mi][3], p);
      }
#pragma unroll
      for (int nj = 0; nj < 2; nj++) {
        const __nv_bfloat16 *p =
            &sB[st][(wn * 32 + nj * 16 + (lane & 7) + ((lane >> 4) << 3)) * LDS + kk + ((lane >> 3) & 1) * 8];
        ldsm4(bfr[2 * nj][0], bfr[2 * nj][1], bfr[2 * nj + 1][0], bfr[2 * nj + 1][1], p);
      }
#pragma unroll
      for (int mi = 0; mi < 2; mi++)
#pragma unroll
        for (int ni = 0; ni < 4; ni++) mma16816(acc[mi][ni], af[mi], bfr[ni]);
    }
    __syncthreads();
  }

  const int g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int mi = 0; mi < 2; mi++)
#pragma unroll
    for (int ni = 0; ni < 4; ni++)
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const int row = m0 + wm * 32 + mi * 16 + g + h * 8;
        const int col = n0 + wn * 32 + ni * 8 + 2 * t;
        float v0 = acc[mi][ni][2 * h], v1 = acc[mi][ni][2 * h + 1];
        if (e.mode == EPI_F32) {
          float2 *o = reinterpret_cast<float2 *>(e.fout + blockIdx.z * e.split_stride + (size_t)row * e.ldc + col);
          *o = make_float2(v0, v1);
        } else if (e.mode == EPI_BIAS) {
          float2 *o = reinterpret_cast<float2 *>(e.fout + (size_t)row * e.ldc + col);
          *o = make_float2(v0 + e.bias[col], v1 + e.bias[col + 1]);
        } else if (e.mode == EPI_BIAS_SILU) {
          float z0 = v0 + e.bias[col], z1 = v1 + e.bias[col + 1];
          *reinterpret_cast<float2 *>(e.zout + (size_t)row * e.ldz + col) = make_float2(z0, z1);
          *reinterpret_cast<__nv_bfloat162 *>(e.hout + (size_t)row * e.ldc + col) =
              __floats2bfloat162_rn(silu(z0), silu(z1));
        } else if (e.mode == EPI_DSILU) {
          float2 z = *reinterpret_cast<const float2 *>(e.zin + (size_t)row * e.ldz + col);
          *reinterpret_cast<__nv_bfloat162 *>(e.hout + (size_t)row * e.ldc + col) =
              __floats2bfloat162_rn(v0 * dsilu(z.x), v1 * dsilu(z.y));
        } else {
          *reinterpret_cast<__nv_bfloat162 *>(e.hout + (size_t)row * e.ldc + col) = __floats2bfloat162_rn(v0, v1);
        }
      }
}

// out[c][r] = in[r][c], bf16, 32 x 32 tiles
__global__ void k_transpose(const __nv_bfloat16 *__restrict__ in, int rows, int cols, int ldi,
                            __nv_bfloat16 *__restrict__ out, int ldo) {
  __shared__ __nv_bfloat16 t[32][33];
  int c = blockIdx.x * 32 + threadIdx.x, r0 = blockIdx.y * 32;
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    int r = r0 + k;
    if (r < rows && c < cols) t[k][threadIdx.x] = in[(size_t)r * ldi + c];
  }
  __syncthreads();
  int ro = r0 + threadIdx.x;
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    int co = blockIdx.x * 32 + k;
    if (co < cols && ro < rows) out[(size_t)co * ldo + ro] = t[threadIdx.x][k];
  }
}

// sum of the K-split partial tiles in split order
__global__ void k_split_sum(const float *__restrict__ part, int splits, long long n, float *__restrict__ out) {
  long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  float s = 0.0f;
  for (int z = 0; z < splits; z++) s += part[(size_t)z * n + k];
  out[k] = s;
}

// column sums of a bf16 [M x N] matrix (bias gradients): per 256-row chunk
// partials, then a fixed-order sum
__global__ void k_colsum_part(const __nv_bfloat16 *__restrict__ d, int M, int N, int ld, float *__restrict__ part) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= N) return;
  int r0 = blockIdx.y * 256, r1 = min(M, r0 + 256);
  float s = 0.0f;
  for (int r = r0; r < r1; r++) s += __bfloat162float(d[(size_t)r * ld + c]);
  part[(size_t)blockIdx.y * N + c] = s;
}

// MSE over the first `nout` of `ldo` output columns: dOut = 2 (out - y) / (M nout)
__global__ void k_loss(const float *__restrict__ out, int ldo, const float *__restrict__ y, int nout, int M,
                       __nv_bfloat16 *__restrict__ dout, float *__restrict__ lpart) {
  __shared__ float sh[256];
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  float l = 0.0f;
  if (r < M) {
    for (int c = 0; c < ldo; c++) {
      float g = 0.0f;
      if (c < nout) {
        float e = out[(size_t)r * ldo + c] - y[(size_t)r * nout + c];
        l += e * e;
        g = 2.0f * e / (float)(M * nout);
      }
      dout[(size_t)r * ldo + c] = __float2bfloat16_rn(g);
    }
  }
  sh[threadIdx.x] = l;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) lpart[blockIdx.x] = sh[0];
}

__global__ void k_loss_final(const float *__restrict__ lpart, int n, int M, int nout, float *__restrict__ loss) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double s = 0.0;
  for (int k = 0; k < n; k++) s += lpart[k];
  *loss = (float)(s / ((double)M * nout));
}

// Adam on FP32 masters; refreshes the bf16 copy W and its transpose W^T.
// step[0] holds the step count (incremented by k_step_inc before the update).
__global__ void k_adam(float *__restrict__ w, float *__restrict__ m, float *__restrict__ v,
                       const float *__restrict__ g, int rows, int cols, int ldw_true, const int *__restrict__ step,
                       float lr, float b1, float b2, float eps, __nv_bfloat16 *__restrict__ wb, int ldb,
                       __nv_bfloat16 *__restrict__ wt, int ldt) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= rows * cols) return;
  int r = k / cols, c = k % cols;
  float gr = g[k];
  float mk = b1 * m[k] + (1.0f - b1) * gr;
  float vk = b2 * v[k] + (1.0f - b2) * gr * gr;
  m[k] = mk;
  v[k] = vk;
  int t = *step;
  float mh = mk / (1.0f - powf(b1, (float)t)), vh = vk / (1.0f - powf(b2, (float)t));
  float wk = w[k] - lr * mh / (sqrtf(vh) + eps);
  w[k] = wk;
  (void)ldw_true;
  if (wb) {
    __nv_bfloat16 h = __float2bfloat16_rn(wk);
    wb[(size_t)r * ldb + c] = h;
    if (wt) wt[(size_t)c * ldt + r] = h;
  }
}
__global__ void k_step_inc(int *step) {
  if (threadIdx.x == 0 && blockIdx.x == 0) step[0] += 1;
}

// fp32 -> bf16 copy (and transpose) of a weight matrix
__global__ void k_to_bf16(const float *__restrict__ w, int rows, int cols, __nv_bfloat16 *__restrict__ wb, int ldb,
                          __nv_bfloat16 *__restrict__ wt, int ldt) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= rows * cols) return;
  int r = k / cols, c = k % cols;
  __nv_bfloat16 h = __float2bfloat16_rn(w[k]);
  wb[(size_t)r * ldb + c] = h;
  if (wt) wt[(size_t)c * ldt + r] = h;
}

// minibatch gather: rows idx = hash(step, k) mod n; standardised bf16 inputs
// (32 columns, the 7 features then zeros) and standardised fp32 targets
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__global__ void k_gather(const float *__restrict__ feat, const float *__restrict__ targ, long long n, int B,
                         const int *__restrict__ step, unsigned long long seed, const float *__restrict__ nrm,
                         __nv_bfloat16 *__restrict__ X, float *__restrict__ Y) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= B) return;
  unsigned long long h = mix64(seed ^ mix64(((unsigned long long)(*step) << 32) | (unsigned)k));
  long long r = (long long)(h % (unsigned long long)n);
  for (int c = 0; c < NIN_PAD; c++) {
    float x = 0.0f;
    if (c < NIN) x = (feat[r * NIN + c] - nrm[c]) / nrm[NIN + c];
    X[(size_t)k * NIN_PAD + c] = __float2bfloat16_rn(x);
  }
  for (int c = 0; c < NOUT; c++)
    Y[(size_t)k * NOUT + c] = (targ[r * NOUT + c] - nrm[2 * NIN + c]) / nrm[2 * NIN + NOUT + c];
}

// standardise rows [r0, r0+B) of a feature array into X (inference)
__global__ void k_stage_rows(const float *__restrict__ feat, long long r0, int B, long long n,
                             const float *__restrict__ nrm, __nv_bfloat16 *__restrict__ X) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= B) return;
  long long r = r0 + k;
  for (int c = 0; c < NIN_PAD; c++) {
    float x = 0.0f;
    if (c < NIN && r < n) x = (feat[r * NIN + c] - nrm[c]) / nrm[NIN + c];
    X[(size_t)k * NIN_PAD + c] = __float2bfloat16_rn(x);
  }
}

// un-standardise network outputs of rows [r0, r0+B) into pred (n x NOUT)
__global__ void k_unstage_rows(const float *__restrict__ out, int ldo, long long r0, int B, long long n,
                               const float *__restrict__ nrm, float *__restrict__ pred) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  long long r = r0 + k;
  if (k >= B || r >= n) return;
  for (int c = 0; c < NOUT; c++)
    pred[r * NOUT + c] = out[(size_t)k * ldo + c] * nrm[2 * NIN + NOUT + c] + nrm[2 * NIN + c];
}

// per-column mean and standard deviation (double accumulation)
__global__ void k_moments(const float *__restrict__ a, long long n, int cols, double *__restrict__ acc) {
  int c = threadIdx.y;
  double s = 0.0, q = 0.0;
  for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (long long)gridDim.x * blockDim.x) {
    double x = a[r * cols + c];
    s += x;
    q += x * x;
  }
  for (int o = 16; o; o >>= 1) {
    s += __shfl_xor_sync(0xffffffffu, s, o);
    q += __shfl_xor_sync(0xffffffffu, q, o);
  }
  if (threadIdx.x == 0) {
    atomicAdd(&acc[c], s);
    atomicAdd(&acc[cols + c], q);
  }
}

// ---- solver side: features of every fine-level cell, warm-start write ------
__device__ __forceinline__ bool interior_cell(const Lvl &L, int &bk, int &i, int &j) {
  int2 t = L.tiles[blockIdx.x];
  bk = t.x;
  const BlkDev &b = L.blk[bk];
  int W = b.nx + 3, lin = t.y + threadIdx.x;
  if (lin >= W * (b.ny + 3)) return false;
  i = lin % W - 1;
  j = lin / W - 1;
  return i >= 1 && i <= b.nx - 1 && j >= 1 && j <= b.ny - 1;
}

// freestream conservative state of a case (Init_flow, sub_init.f90:383-495)
__device__ __forceinline__ void freestream(const CaseDev &c, double *U) {
  U[0] = 1.0;
  U[1] = c.cosA;
  U[2] = c.sinA;
  U[3] = c.p00 / (c.gamma - 1.0) + 0.5;
}

// one row per interior cell (dense index cell0 + (j-1)(nx-1) + (i-1)):
// features x1, y1, log10(dw), M, AoA [deg], log10 Re, shape; targets (when
// requested) the departure of rho, rho u, rho v, E from the case's
// freestream, and log1p(max(nu_tilde Re, 0)).  Learning the departure makes
// the far field, most of the cells, exact for an untrained output of zero.
__global__ void k_features(Lvl L, const double *__restrict__ shape, float *__restrict__ feat,
                           float *__restrict__ targ) {
  int bk, i, j;
  if (!interior_cell(L, bk, i, j)) return;
  const BlkDev &b = L.blk[bk];
  const CaseDev &c = L.cs[b.cas];
  const long long F = L.F, id = fidx(b, i, j);
  const size_t row = (size_t)b.cell0 + (size_t)(j - 1) * (b.nx - 1) + (i - 1);
  float *f = feat + row * NIN;
  f[0] = (float)L.geo[G_X1 * F + id];
  f[1] = (float)L.geo[G_Y1 * F + id];
  f[2] = (float)log10(fmax(L.geo[G_DW * F + id], 1e-9));
  f[3] = (float)c.Ma;
  f[4] = (float)(atan2(c.sinA, c.cosA) * 57.29577951308232);
  f[5] = (float)log10(c.Re);
  f[6] = (float)shape[b.cas];
  if (targ) {
    float *t = targ + row * NOUT;
    double Ui[4];
    freestream(c, Ui);
    for (int m = 0; m < 4; m++) t[m] = (float)(L.U[m * F + id] - Ui[m]);
    t[4] = L.nvar >= 5 ? (float)log1p(fmax(L.U[4 * F + id] * c.Re, 0.0)) : 0.0f;
  }
}

// predicted state of a cell; false if it is not physical (rho <= 0, p <= 0
// or T < 1e-5, the stop test of sub_Residual.f90:143-146)
__device__ __forceinline__ bool predicted_state(const Lvl &L, const BlkDev &b, int i, int j, const float *pred,
                                                double *U) {
  const CaseDev &c = L.cs[b.cas];
  const size_t row = (size_t)b.cell0 + (size_t)(j - 1) * (b.nx - 1) + (i - 1);
  const float *p = pred + row * NOUT;
  double Ui[4];
  freestream(c, Ui);
  for (int m = 0; m < 4; m++) U[m] = Ui[m] + (double)p[m];
  U[4] = expm1((double)p[4]) / c.Re;
  double d = U[0];
  if (!(d > 0.0)) return false;
  double uu = U[1] / d, v = U[2] / d;
  double T = (U[3] - 0.5 * d * (uu * uu + v * v)) / (c.Cv * d);
  double pr = c.p00 * d * T;
  return pr > 0.0 && T >= 1.0e-5;
}

__global__ void k_warm_check(Lvl L, const float *__restrict__ pred, int *__restrict__ bad) {
  int bk, i, j;
  if (!interior_cell(L, bk, i, j)) return;
  const BlkDev &b = L.blk[bk];
  double U[5];
  if (!predicted_state(L, b, i, j, pred, U)) atomicOr(bad + b.cas, 1);
}

// interior cells of cases whose whole prediction is physical take it (nu_tilde
// clipped at 0 like force_vt_kw); other cases keep the freestream of init
__global__ void k_warm_apply(Lvl L, const float *__restrict__ pred, const int *__restrict__ bad) {
  int bk, i, j;
  if (!interior_cell(L, bk, i, j)) return;
  const BlkDev &b = L.blk[bk];
  if (bad[b.cas]) return;
  double U[5];
  predicted_state(L, b, i, j, pred, U);
  const long long F = L.F, id = fidx(b, i, j);
  for (int m = 0; m < 4; m++) L.U[m * F + id] = U[m];
  if (L.nvar == 5) L.U[4 * F + id] = fmax(U[4], 0.0);
}

}  // namespace mlp

void launch_features(const Lvl &L, const double *shape, float *feat, float *targ, cudaStream_t s) {
  mlp::k_features<<<L.ntiles, EC2D_TILE, 0, s>>>(L, shape, feat, targ);
}
void launch_warm_start(const Lvl &L, const float *pred, int *bad, cudaStream_t s) {
  mlp::k_warm_check<<<L.ntiles, EC2D_TILE, 0, s>>>(L, pred, bad);
  mlp::k_warm_apply<<<L.ntiles, EC2D_TILE, 0, s>>>(L, pred, bad);
}

// ---------------------------------------------------------------------------
// host side of the network
// ---------------------------------------------------------------------------
using namespace mlp;

// tcgen05 kernel when selected and the shape fits its tiles, else mma.sync
void Net::gemm(const __nv_bfloat16 *A, int lda, const __nv_bfloat16 *B, int ldb, int M, int N, int K, int ksplit,
               const Epi &e) {
  if (gemm_kind == 1 && M % 128 == 0 && N % 64 == 0 && (K / ksplit) % 64 == 0) {
    launch_gemm_tc(A, lda, B, ldb, M, N, K, ksplit, e, d_err, stream);
    return;
  }
  dim3 grid(M / BM, N / BN, ksplit);
  k_gemm_tn<<<grid, 256, 0, stream>>>(A, lda, B, ldb, K, ksplit, e);
}

static void transpose(const __nv_bfloat16 *in, int rows, int cols, int ldi, __nv_bfloat16 *out, int ldo,
                      cudaStream_t s) {
  dim3 grid((cols + 31) / 32, (rows + 31) / 32);
  k_transpose<<<grid, dim3(32, 8), 0, s>>>(in, rows, cols, ldi, out, ldo);
}

int Net::layer_in(int l) const { return l == 0 ? NIN_PAD : width; }
int Net::layer_out(int l) const { return l == nlin - 1 ? NOUT_PAD : width; }

template <class T>
static T *dev_alloc(std::vector<void *> &owned, size_t n) {
  void *p = nullptr;
  if (cudaMalloc(&p, n * sizeof(T) + 16) != cudaSuccess) return nullptr;
  cudaMemset(p, 0, n * sizeof(T) + 16);
  owned.push_back(p);
  return (T *)p;
}

int Net::init(int dev, int hidden, int w, unsigned long long seed_) {
  device = dev;
  cudaSetDevice(dev);
  if (hidden < 1 || hidden > MAX_HIDDEN || w < 64 || w % 64 != 0 || w > 1024) return 1;
  width = w;
  nlin = hidden + 1;
  seed = seed_;
  if (cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking) != cudaSuccess) return 2;
  // weights: Kaiming-uniform from a splitmix64 stream, zero biases; padded
  // rows/columns stay zero
  unsigned long long z = seed;
  auto uni = [&]() {
    z += 0x9E3779B97F4A7C15ull;
    unsigned long long x = z;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    x ^= x >> 31;
    return (double)(x >> 11) * (1.0 / 9007199254740992.0);
  };
  for (int l = 0; l < nlin; l++) {
    int ni = layer_in(l), no = layer_out(l);
    int fan_in = l == 0 ? NIN : width, rows_true = l == nlin - 1 ? NOUT : width;
    std::vector<float> hw((size_t)no * ni, 0.0f);
    double a = std::sqrt(6.0 / fan_in) * (l == nlin - 1 ? 0.5 : 1.0);
    for (int r = 0; r < rows_true; r++)
      for (int c = 0; c < fan_in; c++) hw[(size_t)r * ni + c] = (float)((2.0 * uni() - 1.0) * a);
    L[l].w = dev_alloc<float>(owned, hw.size());
    L[l].b = dev_alloc<float>(owned, no);
    L[l].mw = dev_alloc<float>(owned, hw.size());
    L[l].vw = dev_alloc<float>(owned, hw.size());
    L[l].mb = dev_alloc<float>(owned, no);
    L[l].vb = dev_alloc<float>(owned, no);
    L[l].gw = dev_alloc<float>(owned, hw.size());
    L[l].gb = dev_alloc<float>(owned, no);
    L[l].wb = dev_alloc<__nv_bfloat16>(owned, hw.size());
    L[l].wt = dev_alloc<__nv_bfloat16>(owned, hw.size());
    if (!L[l].w || !L[l].wt) return 3;
    cudaMemcpy(L[l].w, hw.data(), hw.size() * sizeof(float), cudaMemcpyHostToDevice);
  }
  nrm = dev_alloc<float>(owned, 2 * NIN + 2 * NOUT);
  std::vector<float> one(2 * NIN + 2 * NOUT, 0.0f);
  for (int c = 0; c < NIN; c++) one[NIN + c] = 1.0f;
  for (int c = 0; c < NOUT; c++) one[2 * NIN + NOUT + c] = 1.0f;
  cudaMemcpy(nrm, one.data(), one.size() * sizeof(float), cudaMemcpyHostToDevice);
  d_step = dev_alloc<int>(owned, 4);
  d_err = dev_alloc<int>(owned, 4);
  d_loss = dev_alloc<float>(owned, 4);
  d_moments = dev_alloc<double>(owned, 2 * (NIN + NOUT));
  refresh_bf16();
  return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

void Net::refresh_bf16() {
  for (int l = 0; l < nlin; l++) {
    int ni = layer_in(l), no = layer_out(l);
    int n = ni * no;
    k_to_bf16<<<(n + 255) / 256, 256, 0, stream>>>(L[l].w, no, ni, L[l].wb, ni, L[l].wt, no);
  }
}

int Net::ensure_batch(int B) {
  if (B <= cap_batch) return 0;
  cap_batch = B;
  const int W = width;
  X = dev_alloc<__nv_bfloat16>(owned, (size_t)B * NIN_PAD);
  Y = dev_alloc<float>(owned, (size_t)B * NOUT);
  for (int l = 0; l < nlin - 1; l++) {
    H[l] = dev_alloc<__nv_bfloat16>(owned, (size_t)B * W);
    Z[l] = dev_alloc<float>(owned, (size_t)B * W);
  }
  out = dev_alloc<float>(owned, (size_t)B * NOUT_PAD);
  dOut = dev_alloc<__nv_bfloat16>(owned, (size_t)B * NOUT_PAD);
  dA = dev_alloc<__nv_bfloat16>(owned, (size_t)B * W);
  dB = dev_alloc<__nv_bfloat16>(owned, (size_t)B * W);
  T1 = dev_alloc<__nv_bfloat16>(owned, (size_t)B * (W > NIN_PAD ? W : NIN_PAD));
  T2 = dev_alloc<__nv_bfloat16>(owned, (size_t)B * W);
  part = dev_alloc<float>(owned, (size_t)KSPLIT * W * W);
  cpart = dev_alloc<float>(owned, (size_t)(B / 256 + 1) * W);
  lpart = dev_alloc<float>(owned, (size_t)(B / 256 + 1));
  return part ? 0 : 1;
}

// forward of B rows staged in X; leaves pre-activations in Z, outputs in out
void Net::forward(int B) {
  const __nv_bfloat16 *in = X;
  int ldin = NIN_PAD;
  for (int l = 0; l < nlin; l++) {
    int no = layer_out(l), ni = layer_in(l);
    Epi e{};
    if (l < nlin - 1) {
      e.mode = EPI_BIAS_SILU; e.bias = L[l].b; e.zout = Z[l]; e.ldz = width; e.hout = H[l]; e.ldc = width;
    } else {
      e.mode = EPI_BIAS; e.bias = L[l].b; e.fout = out; e.ldc = NOUT_PAD;
    }
    gemm(in, ldin, L[l].wb, ni, B, no, ni, 1, e);
    in = H[l < nlin - 1 ? l : 0];
    ldin = width;
  }
}

// loss of the forward outputs against Y, then gradients of every layer
void Net::backward(int B) {
  const int nb = (B + 255) / 256;
  k_loss<<<nb, 256, 0, stream>>>(out, NOUT_PAD, Y, NOUT, B, dOut, lpart);
  k_loss_final<<<1, 32, 0, stream>>>(lpart, nb, B, NOUT, d_loss);
  const __nv_bfloat16 *dz = dOut;  // gradient w.r.t. the pre-activation of layer l's output
  int ldz = NOUT_PAD;
  __nv_bfloat16 *bufs[2] = {dA, dB};
  for (int l = nlin - 1; l >= 0; l--) {
    const int no = layer_out(l), ni = layer_in(l);
    const __nv_bfloat16 *hin = l == 0 ? X : H[l - 1];
    // dW = dz^T . hin : A = dz^T [no x B], B = hin^T [ni x B]
    transpose(dz, B, no, ldz, T2, B, stream);
    transpose(hin, B, ni, l == 0 ? NIN_PAD : width, T1, B, stream);
    Epi e{};
    e.mode = EPI_F32; e.fout = part; e.ldc = ni; e.split_stride = (long long)no * ni;
    int ks = KSPLIT;
    while (ks > 1 && (B / ks) % 64) ks >>= 1;
    gemm(T2, B, T1, B, no, ni, B, ks, e);
    long long n = (long long)no * ni;
    k_split_sum<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(part, ks, n, L[l].gw);
    // db = column sums of dz
    dim3 cg((no + 255) / 256, nb);
    k_colsum_part<<<cg, 256, 0, stream>>>(dz, B, no, ldz, cpart);
    k_split_sum<<<(no + 255) / 256, 256, 0, stream>>>(cpart, nb, no, L[l].gb);
    if (l == 0) break;
    // dH_{l-1} = dz . W_l, times silu'(Z_{l-1}) : A = dz [B x no], B = W_l^T [ni x no]
    Epi d{};
    d.mode = EPI_DSILU; d.zin = Z[l - 1]; d.ldz = width; d.hout = bufs[l & 1]; d.ldc = width;
    gemm(dz, ldz, L[l].wt, no, B, ni, no, 1, d);
    dz = bufs[l & 1];
    ldz = width;
  }
}

void Net::adam(float lr) {
  k_step_inc<<<1, 32, 0, stream>>>(d_step);
  for (int l = 0; l < nlin; l++) {
    int ni = layer_in(l), no = layer_out(l), n = ni * no;
    k_adam<<<(n + 255) / 256, 256, 0, stream>>>(L[l].w, L[l].mw, L[l].vw, L[l].gw, no, ni, ni, d_step, lr, 0.9f,
                                               0.999f, 1e-8f, L[l].wb, ni, L[l].wt, no);
    k_adam<<<(no + 255) / 256, 256, 0, stream>>>(L[l].b, L[l].mb, L[l].vb, L[l].gb, 1, no, no, d_step, lr, 0.9f,
                                                0.999f, 1e-8f, nullptr, 0, nullptr, 0);
  }
}

void Net::gather(int B) {
  k_gather<<<(B + 255) / 256, 256, 0, stream>>>(feat, targ, nsamp, B, d_step, seed, nrm, X, Y);
}

int Net::fit_normalization() {
  if (nsamp < 2) return 1;
  cudaMemsetAsync(d_moments, 0, 2 * (NIN + NOUT) * sizeof(double), stream);
  k_moments<<<256, dim3(32, NIN), 0, stream>>>(feat, nsamp, NIN, d_moments);
  k_moments<<<256, dim3(32, NOUT), 0, stream>>>(targ, nsamp, NOUT, d_moments + 2 * NIN);
  std::vector<double> h(2 * (NIN + NOUT));
  cudaMemcpyAsync(h.data(), d_moments, h.size() * sizeof(double), cudaMemcpyDeviceToHost, stream);
  if (cudaStreamSynchronize(stream) != cudaSuccess) return 2;
  std::vector<float> nv(2 * NIN + 2 * NOUT);
  for (int c = 0; c < NIN; c++) {
    double m = h[c] / nsamp, v = h[NIN + c] / nsamp - m * m;
    nv[c] = (float)m;
    nv[NIN + c] = (float)(v > 1e-12 ? std::sqrt(v) : 1.0);
  }
  for (int c = 0; c < NOUT; c++) {
    double m = h[2 * NIN + c] / nsamp, v = h[2 * NIN + NOUT + c] / nsamp - m * m;
    nv[2 * NIN + c] = (float)m;
    nv[2 * NIN + NOUT + c] = (float)(v > 1e-12 ? std::sqrt(v) : 1.0);
  }
  cudaMemcpyAsync(nrm, nv.data(), nv.size() * sizeof(float), cudaMemcpyHostToDevice, stream);
  return cudaStreamSynchronize(stream) == cudaSuccess ? 0 : 2;
}

int Net::reserve_samples(long long n) {
  if (n <= cap_samp) return 0;
  long long cap = cap_samp ? cap_samp : 1 << 20;
  while (cap < n) cap *= 2;
  float *f = nullptr, *t = nullptr;
  if (cudaMalloc(&f, (size_t)cap * NIN * sizeof(float)) != cudaSuccess) return 1;
  if (cudaMalloc(&t, (size_t)cap * NOUT * sizeof(float)) != cudaSuccess) { cudaFree(f); return 1; }
  if (nsamp) {
    cudaMemcpyAsync(f, feat, (size_t)nsamp * NIN * sizeof(float), cudaMemcpyDeviceToDevice, stream);
    cudaMemcpyAsync(t, targ, (size_t)nsamp * NOUT * sizeof(float), cudaMemcpyDeviceToDevice, stream);
    cudaStreamSynchronize(stream);
  }
  if (feat) cudaFree(feat);
  if (targ) cudaFree(targ);
  feat = f;
  targ = t;
  cap_samp = cap;
  return 0;
}

// predictions for n feature rows (device, n x NIN) into pred (device, n x NOUT)
int Net::predict(const float *f, long long n, float *pred) {
  const int B = 16384;
  if (ensure_batch(B)) return 1;
  for (long long r0 = 0; r0 < n; r0 += B) {
    k_stage_rows<<<B / 256, 256, 0, stream>>>(f, r0, B, n, nrm, X);
    forward(B);
    k_unstage_rows<<<B / 256, 256, 0, stream>>>(out, NOUT_PAD, r0, B, n, nrm, pred);
  }
  return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

int Net::check_err() {
  int h = 0;
  cudaMemcpyAsync(&h, d_err, sizeof(int), cudaMemcpyDeviceToHost, stream);
  cudaMemsetAsync(d_err, 0, sizeof(int), stream);
  cudaStreamSynchronize(stream);
  return h;
}

void Net::destroy() {
  cudaSetDevice(device);
  if (stream) cudaStreamSynchronize(stream);
  if (train_graph) cudaGraphExecDestroy(train_graph);
  for (void *p : owned) cudaFree(p);
  owned.clear();
  if (feat) cudaFree(feat);
  if (targ) cudaFree(targ);
  if (stream) cudaStreamDestroy(stream);
}

}  // namespace ec2d
