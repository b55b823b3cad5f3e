// ec2d_mlp.h -- internal declarations of the warm-start network (k_mlp.cu).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <vector>

namespace ec2d {

constexpr int NIN = 7;        // x, y, log10 dw, M, AoA (deg), log10 Re, t/c
constexpr int NIN_PAD = 64;   // input columns as the GEMMs see them
constexpr int NOUT = 5;       // rho, rho u, rho v, E, log1p(nu_tilde Re)
constexpr int NOUT_PAD = 128; // output rows of the last weight matrix
constexpr int MAX_HIDDEN = 12;
constexpr int KSPLIT = 32;    // K splits of the weight-gradient GEMM

enum { EPI_F32 = 0, EPI_BIAS = 1, EPI_BIAS_SILU = 2, EPI_DSILU = 3, EPI_BF16 = 4 };

// epilogue of C[M x N] = A[M x K] . B[N x K]^T
struct Epi {
  int mode;                 // EPI_*
  const float *bias;        // [N] (bias modes)
  float *zout;              // pre-activation out (EPI_BIAS_SILU), [M x ldz]
  const float *zin;         // pre-activation in (EPI_DSILU), [M x ldz]
  int ldz;
  __nv_bfloat16 *hout;      // bf16 out (EPI_BIAS_SILU, EPI_DSILU, EPI_BF16)
  float *fout;              // fp32 out (EPI_BIAS, EPI_F32)
  int ldc;
  long long split_stride;   // EPI_F32: offset between the K-split partial tiles
};

// tcgen05 (TMEM accumulator) GEMM, k_gemm_tc.cu: M % 128 == 0, N % 64 == 0,
// (K / ksplit) % 64 == 0.  err: device flag set if an mbarrier wait timed out.
void launch_gemm_tc(const __nv_bfloat16 *A, int lda, const __nv_bfloat16 *B, int ldb, int M, int N, int K,
                    int ksplit, const Epi &e, int *err, cudaStream_t s);

struct Layer {
  float *w = nullptr, *b = nullptr;    // FP32 masters [out x in], [out]
  float *mw = nullptr, *vw = nullptr, *mb = nullptr, *vb = nullptr;  // Adam moments
  float *gw = nullptr, *gb = nullptr;  // gradients
  __nv_bfloat16 *wb = nullptr, *wt = nullptr;  // BF16 copy and its transpose
};

struct Net {
  int device = 0, width = 256, nlin = 7;
  unsigned long long seed = 0;
  cudaStream_t stream = nullptr;
  Layer L[MAX_HIDDEN + 1];
  float *nrm = nullptr;  // feature mean[NIN], std[NIN], target mean[NOUT], std[NOUT]
  int *d_step = nullptr;
  int *d_err = nullptr;   // set by a tcgen05 GEMM whose mbarrier wait timed out
  int gemm_kind = 1;      // 1: tcgen05 GEMMs (default), 0: mma.sync GEMMs
  float *d_loss = nullptr;
  double *d_moments = nullptr;
  // batch buffers
  int cap_batch = 0;
  __nv_bfloat16 *X = nullptr, *H[MAX_HIDDEN] = {}, *dOut = nullptr, *dA = nullptr, *dB = nullptr, *T1 = nullptr,
                *T2 = nullptr;
  float *Y = nullptr, *Z[MAX_HIDDEN] = {}, *out = nullptr, *part = nullptr, *cpart = nullptr, *lpart = nullptr;
  // samples (device): features n x NIN, targets n x NOUT
  float *feat = nullptr, *targ = nullptr;
  long long nsamp = 0, cap_samp = 0;
  cudaGraphExec_t train_graph = nullptr;  // one training step (gather, forward, backward, Adam)
  int graph_batch = 0, graph_kind = -1;
  float graph_lr = 0.0f;
  std::vector<void *> owned;

  int init(int dev, int hidden, int width, unsigned long long seed);
  void destroy();
  int layer_in(int l) const;
  int layer_out(int l) const;
  void refresh_bf16();
  void gemm(const __nv_bfloat16 *A, int lda, const __nv_bfloat16 *B, int ldb, int M, int N, int K, int ksplit,
            const Epi &e);
  int ensure_batch(int B);
  void forward(int B);
  void backward(int B);
  void adam(float lr);
  void gather(int B);
  int fit_normalization();
  int reserve_samples(long long n);
  int predict(const float *feat, long long n, float *pred);
  int check_err();  // 0, or 1 if a tcgen05 wait timed out since the last call
};

}  // namespace ec2d
