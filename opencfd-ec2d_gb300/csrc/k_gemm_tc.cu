// k_gemm_tc.cu -- BF16 GEMM on the 5th-generation tensor cores (tcgen05):
// C[M x N] = A[M x K] . B[N x K]^T, both operands K-major, FP32 accumulators
// in tensor memory, the epilogues of the warm-start network (k_mlp.cu).
//
// One CTA of 256 threads computes a 128 x BN tile (BN = 128 or 64):
//  * warp 0 allocates BN TMEM columns (128 lanes x BN x 32 bit: the tile);
//  * all threads stage 64-wide K chunks of A and B into shared memory with
//    16-byte cp.async, in the canonical no-swizzle K-major layout of the MMA
//    operands: 8 x 8 core matrices of 128 contiguous bytes, the 8 K-chunks of
//    a row group adjacent (leading byte offset 128 B), row groups 1024 B apart
//    (stride byte offset);
//  * thread 0 issues four tcgen05.mma (M=128, N=BN, K=16 each) per chunk and
//    commits them to the chunk buffer's mbarrier; a three-buffer ring keeps
//    two chunks loading while the tensor cores work on the third;
//  * after the last commit each warp reads 32 accumulator rows of one column
//    half with tcgen05.ld (32 columns at a time), stages them in shared
//    memory and applies the epilogue row by row with coalesced global
//    accesses (eight warps keep the epilogue's memory latency covered).
// Every mbarrier wait is bounded: on timeout the kernel sets *err, issues no
// further MMA, waits (bounded) for the ones in flight and still frees its
// TMEM.  The timeout decision is made CTA-wide (__syncthreads_and), so all
// threads leave the loop together.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "ec2d_mlp.h"

namespace ec2d {
namespace tc {

constexpr int BM = 128, BK = 64, NS = 3;  // tile rows, K chunk, pipeline stages
constexpr long long WAIT_LIMIT = 1ll << 24;  // try_wait polls before giving up

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void cp16(uint32_t dst, const void *src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

__device__ __forceinline__ void mbar_init(uint32_t a, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(count) : "memory");
}
// true once the phase with the given parity has completed; false on timeout
__device__ __forceinline__ bool mbar_wait(uint32_t a, unsigned parity) {
  for (long long it = 0; it < WAIT_LIMIT; it++) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// shared-memory matrix descriptor: start >> 4, leading / stride byte
// offsets >> 4, the fixed descriptor version 1 at bit 46, no swizzle
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFF) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// instruction descriptor, kind::f16: FP32 accumulate (bit 4), A and B BF16
// (bits 7 and 10), both K-major, N >> 3 at bit 17, M >> 4 at bit 24
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ float silu(float z) { return z / (1.0f + __expf(-z)); }
__device__ __forceinline__ float dsilu(float z) {
  float s = 1.0f / (1.0f + __expf(-z));
  return s * (1.0f + z * (1.0f - s));
}

template <int BN>
__global__ void __launch_bounds__(256) k_gemm_tc(const __nv_bfloat16 *__restrict__ A, int lda,
                                                 const __nv_bfloat16 *__restrict__ B, int ldb, int K, int ksplit,
                                                 Epi e, int *err) {
  constexpr int ABYTES = BM * BK * 2, BBYTES = BN * BK * 2, STAGE = ABYTES + BBYTES;
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ __align__(8) uint64_t mbar[NS];
  __shared__ uint32_t tmem_sh;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
  const int kc = K / ksplit, kb = blockIdx.z * kc, nk = kc / BK;
  const uint32_t s0 = smem_u32(smem);

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_sh)),
                 "r"(BN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int q = 0; q < NS; q++) mbar_init(smem_u32(&mbar[q]), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_sh;

  // piece c of a chunk: row r = (c & 7) + 8 (c >> 6), K piece p = (c >> 3) & 7,
  // placed at core matrix (r / 8, p), row r % 8: byte offset 16 c, so the
  // shared-memory writes of a warp are contiguous
  auto load = [&](int buf, int kt) {
    const int k0 = kb + kt * BK;
    const uint32_t sa = s0 + buf * STAGE, sb = sa + ABYTES;
#pragma unroll
    for (int q = 0; q < BM * 8 / 256; q++) {
      int c = tid + q * 256;
      int r = (c & 7) + ((c >> 6) << 3), p = (c >> 3) & 7;
      cp16(sa + (uint32_t)(((r >> 3) * 8 + p) * 128 + (r & 7) * 16), A + (size_t)(m0 + r) * lda + k0 + p * 8);
    }
#pragma unroll
    for (int q = 0; q < BN * 8 / 256; q++) {
      int c = tid + q * 256;
      int r = (c & 7) + ((c >> 6) << 3), p = (c >> 3) & 7;
      cp16(sb + (uint32_t)(((r >> 3) * 8 + p) * 128 + (r & 7) * 16), B + (size_t)(n0 + r) * ldb + k0 + p * 8);
    }
    cp_commit();
  };

  bool ok = true;
  int last = -1;  // last chunk whose MMAs were committed
  constexpr uint32_t IDESC = idesc_bf16(BM, BN);
  // NS-stage ring: chunk c lives in buffer c % NS; one cp.async group is
  // committed per chunk slot (empty past the end) so that wait_group<NS-1>
  // always means "chunk kt has landed"
#pragma unroll
  for (int c = 0; c < NS - 1; c++) {
    if (c < nk) load(c, c);
    else cp_commit();
  }
  for (int kt = 0; kt < nk; kt++) {
    const int buf = kt % NS, c = kt + NS - 1;
    if (c < nk) {
      // buffer c % NS last held chunk kt-1: free once its MMAs completed
      if (kt >= 1 && ok) ok = mbar_wait(smem_u32(&mbar[(kt - 1) % NS]), ((kt - 1) / NS) & 1);
      load(c % NS, c);
    } else {
      cp_commit();
    }
    cp_wait<NS - 1>();
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    ok = __syncthreads_and(ok) != 0;
    if (!ok) break;
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t sa = s0 + buf * STAGE, sb = sa + ABYTES;
#pragma unroll
      for (int s = 0; s < BK / 16; s++) {
        uint64_t ad = sdesc(sa + s * 256, 128, 1024), bd = sdesc(sb + s * 256, 128, 1024);
        uint32_t acc = (kt > 0 || s > 0) ? 1u : 0u;
        asm volatile(
            "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
            "l"(ad), "l"(bd), "r"(IDESC), "r"(acc)
            : "memory");
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       smem_u32(&mbar[buf]))
                   : "memory");
    }
    last = kt;
  }
  cp_wait<0>();
  // the accumulators are complete (after a timeout: no MMA is in flight any
  // more) once the last committed chunk's barrier completes
  if (last >= 0) {
    bool f = mbar_wait(smem_u32(&mbar[last % NS]), (last / NS) & 1);
    ok = ok && f;
  }
  ok = __syncthreads_and(ok) != 0;
  if (!ok && tid == 0) atomicExch(err, 1);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

  if (ok) {
    // epilogue through shared memory (the operand buffers are free now): each
    // warp stages its 32 accumulator rows x 32 columns, then walks the rows
    // with lane = column, so every global load and store of a warp covers
    // consecutive columns of one row
    // warp w reads TMEM lanes 32 (w % 4) .. +31 (the rows it may access) and
    // the column half w / 4
    float *stage = reinterpret_cast<float *>(smem) + warp * (32 * 33);
    const int wl = warp & 3, half = warp >> 2;
#pragma unroll 1
    for (int c0 = half * (BN / 2); c0 < (half + 1) * (BN / 2); c0 += 32) {
      uint32_t v[32];
      const uint32_t ta = tmem + ((uint32_t)(wl * 32) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
          "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
            "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
            "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
            "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
          : "r"(ta));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
      for (int j = 0; j < 32; j++) stage[lane * 33 + j] = __uint_as_float(v[j]);
      __syncwarp();
      const int col = n0 + c0 + lane;
      const size_t row0 = (size_t)(m0 + wl * 32);
      // the mode is uniform: one fully unrolled row loop per mode, so the 32
      // rows' loads and stores of a lane are all in flight together
      if (e.mode == EPI_F32) {
        float *o = e.fout + blockIdx.z * e.split_stride + row0 * e.ldc + col;
#pragma unroll
        for (int r = 0; r < 32; r++) o[(size_t)r * e.ldc] = stage[r * 33 + lane];
      } else if (e.mode == EPI_BIAS) {
        const float bc = e.bias[col];
        float *o = e.fout + row0 * e.ldc + col;
#pragma unroll
        for (int r = 0; r < 32; r++) o[(size_t)r * e.ldc] = stage[r * 33 + lane] + bc;
      } else if (e.mode == EPI_BIAS_SILU) {
        const float bc = e.bias[col];
        float *zo = e.zout + row0 * e.ldz + col;
        __nv_bfloat16 *ho = e.hout + row0 * e.ldc + col;
#pragma unroll
        for (int r = 0; r < 32; r++) {
          const float z = stage[r * 33 + lane] + bc;
          zo[(size_t)r * e.ldz] = z;
          ho[(size_t)r * e.ldc] = __float2bfloat16_rn(silu(z));
        }
      } else if (e.mode == EPI_DSILU) {
        const float *zi = e.zin + row0 * e.ldz + col;
        float z[32];
#pragma unroll
        for (int r = 0; r < 32; r++) z[r] = zi[(size_t)r * e.ldz];
        __nv_bfloat16 *ho = e.hout + row0 * e.ldc + col;
#pragma unroll
        for (int r = 0; r < 32; r++) ho[(size_t)r * e.ldc] = __float2bfloat16_rn(stage[r * 33 + lane] * dsilu(z[r]));
      } else {
        __nv_bfloat16 *ho = e.hout + row0 * e.ldc + col;
#pragma unroll
        for (int r = 0; r < 32; r++) ho[(size_t)r * e.ldc] = __float2bfloat16_rn(stage[r * 33 + lane]);
      }
      __syncwarp();
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(BN) : "memory");
}

}  // namespace tc

// shared memory: NS stages of A (16 KB) and B (BN x 128 B), 1 KB alignment
// slack; the epilogue reuses the first 17 KB
template <int BN>
static size_t tc_smem() {
  return (size_t)tc::NS * (tc::BM * tc::BK * 2 + BN * tc::BK * 2) + 1024;
}

void launch_gemm_tc(const __nv_bfloat16 *A, int lda, const __nv_bfloat16 *B, int ldb, int M, int N, int K,
                    int ksplit, const Epi &e, int *err, cudaStream_t s) {
  if (N % 128 == 0) {
    size_t sm = tc_smem<128>();
    cudaFuncSetAttribute(tc::k_gemm_tc<128>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    tc::k_gemm_tc<128><<<dim3(M / tc::BM, N / 128, ksplit), 256, sm, s>>>(A, lda, B, ldb, K, ksplit, e, err);
  } else {
    size_t sm = tc_smem<64>();
    cudaFuncSetAttribute(tc::k_gemm_tc<64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    tc::k_gemm_tc<64><<<dim3(M / tc::BM, N / 64, ksplit), 256, sm, s>>>(A, lda, B, ldb, K, ksplit, e, err);
  }
}

}  // namespace ec2d
