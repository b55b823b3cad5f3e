// k_sweep32.cu -- the LU-SGS operator (du_LU_SGS_2D, sub_LU_SGS.f90:4-108) in
// FP32, for the mixed-precision mode in which the sweeps only precondition:
// the residual stays FP64, Res is rounded to float when the records are built,
// U stays FP64 and receives U += (double)dU in a separate all-cells kernel.
//
// Same wavefront as the FP64 sweep (k_sweep.cu): hyperplanes p = i+j in the
// reference's Gauss-Seidel order, one CTA per block, thread j owns row j, the
// next three cells' records are in flight by cp.async, the neighbouring row's
// state comes through a double-buffered shared slot.  One difference in
// arithmetic, not in the operator: the flux difference of comput_DFn
// (sub_LU_SGS.f90:117-138), F_n(U + dU) - F_n(U), is evaluated in the
// algebraically identical increment form
//     du = (d(rho u) - u d(rho)) / (rho + d(rho)),  dv likewise,
//     dp = (gamma-1) (dE - (d(rho u) u' + rho u du + d(rho v) v' + rho v dv) / 2),
//     dF_0 = d(rho) un' + rho dun,        dF_1 = d(rho u) un' + rho u dun + dp n1,
//     dF_2 = d(rho v) un' + rho v dun + dp n2,
//     dF_3 = (dE + dp) un' + (E + p) dun, dF_m = dU_m un' + U_m dun (m >= 4),
// with un' = u' n1 + v' n2 and dun = du n1 + dv n2.  In float, F_n(U + dU)
// - F_n(U) would cancel to zero once |dU| < 6e-8 |U| and stall convergence;
// here every term is an increment times an O(1) state, so the rounding error
// stays relative to dU.  The producer of a state computes du, dv, u', v', dp
// (they do not depend on the face normal) and ships them with dU and its base
// state; the consumer forms un', dun with its own face normal, which already
// carries the factor +-0.5 s of the reference (the flux is linear in n).
#include <algorithm>

#include "ec2d_dev.cuh"
#include "ec2d_internal.h"

namespace ec2d {

namespace {

constexpr int TILE = EC2D_TILE;

constexpr int pad4(int n) { return (n + 3) / 4 * 4; }

// record (floats), identical for both passes:
//  A        Res (forward) or the forward dU (backward)
//  B        base state of the cell: rho, rho u, rho v, E + p, U_5.., then u, v
//  CI, CJ   0.5 Lc_nb (+ Lv_nb when viscous) of the upstream neighbours
//  N1I..N2J face normals of face i / j times the signed 0.5 s of the reference
//  IA, IA5  1/alfa and, for the SA row, 1/(alfa + Lvi + Lvj)
template <int NV>
struct R32 {
  static constexpr int A = 0, B = NV, BU = 2 * NV, BV = 2 * NV + 1, CI = 2 * NV + 2, CJ = CI + 1, N1I = CI + 2,
                       N2I = CI + 3, N1J = CI + 4, N2J = CI + 5, IA = CI + 6, IA5 = CI + 7;
  static constexpr int NF = pad4(CI + 8);
  static constexpr int BYTES = NF * 4;
  static_assert(BYTES % 16 == 0, "records are whole 16-byte units");
};

// shipped state: dU, base (rho, rho u, rho v, E + p, U_5..), u', v', du, dv, dp
template <int NV>
struct S32 {
  static constexpr int D = 0, B = NV, UP = 2 * NV, VP = UP + 1, DU = UP + 2, DV = UP + 3, DP = UP + 4;
  static constexpr int S = pad4(DP + 1);
};

template <int NV>
__global__ void __launch_bounds__(TILE) k_lusgs_prep32(Lvl L, double alfa1, int force) {
  using RC = R32<NV>;
  int bk, i, j;
  if (!core_ij(L, bk, i, j)) return;
  const BlkDev &b = L.blk[bk];
  if (i < 1 || i > b.nx - 1 || j < 1 || j > b.ny - 1) return;
  const CaseDev &c = L.cs[b.cas];
  const long long F = L.F, P = b.P;
  const long long id = fidx(b, i, j);
  const double gm1 = c.gamma - 1.0;
  const double *g = L.geo, *lc = L.lc;
  const bool visc = L.visc != 0;
  const size_t cell = (size_t)b.cell0 + (size_t)(j - 1) * (b.nx - 1) + (i - 1);
  // the two records are assembled in registers and written 16 bytes at a time
  float rf[RC::NF], rb[RC::NF];
#pragma unroll
  for (int k = RC::CI + 8; k < RC::NF; k++) rf[k] = rb[k] = 0.0f;
  double vol = g[G_VOL * F + id];
  double Lv = lc[L_VI * F + id] + lc[L_VJ * F + id];
  double alfa = vol * rcp(lc[L_DT * F + id]) + 1.0 * (lc[L_CI * F + id] + lc[L_CJ * F + id]) + vol * alfa1;
  if (visc) alfa += 2.0 * Lv;
  double ia = rcp(alfa), ia5 = (NV == 5) ? rcp(alfa + Lv) : ia;
  double U[NV];
#pragma unroll
  for (int m = 0; m < NV; m++) U[m] = L.U[m * F + id];
  double r = rcp(U[0]), u = U[1] * r, v = U[2] * r;
  double p = gm1 * (U[3] - 0.5 * (U[1] * u + U[2] * v));
  double ni1 = g[G_NI1 * F + id], ni2 = g[G_NI2 * F + id], nj1 = g[G_NJ1 * F + id], nj2 = g[G_NJ2 * F + id];
#pragma unroll
  for (int m = 0; m < NV; m++) {
    rf[RC::A + m] = (float)((force && m < 4) ? L.res[m * F + id] + L.qf[m * F + id] : L.res[m * F + id]);
    rb[RC::A + m] = 0.0f;
  }
  float *rr[2] = {rf, rb};
#pragma unroll
  for (int pass = 0; pass < 2; pass++) {
    float *q = rr[pass];
    q[RC::B + 0] = (float)U[0];
    q[RC::B + 1] = (float)U[1];
    q[RC::B + 2] = (float)U[2];
    q[RC::B + 3] = (float)(U[3] + p);
#pragma unroll
    for (int m = 4; m < NV; m++) q[RC::B + m] = (float)U[m];
    q[RC::BU] = (float)u;
    q[RC::BV] = (float)v;
    q[RC::IA] = (float)ia;
    q[RC::IA5] = (float)ia5;
#pragma unroll
    for (int dir = 0; dir < 2; dir++) {  // 0: i-neighbour, 1: j-neighbour
      const bool fwd = pass == 0;
      const long long step = dir == 0 ? 1 : P;
      const long long nb = fwd ? id - step : id + step;
      const bool has = dir == 0 ? (fwd ? i > 1 : i < b.nx - 1) : (fwd ? j > 1 : j < b.ny - 1);
      double cc = 0.0, hh = 0.0;
      if (has) {
        cc = 0.5 * lc[(dir == 0 ? L_CI : L_CJ) * F + nb];
        if (visc) cc += lc[(dir == 0 ? L_VI : L_VJ) * F + nb];
        // forward: +0.5 s of this cell's face; backward: -0.5 s of the
        // neighbour's face with this cell's normal (sub_LU_SGS.f90:87-88,95-96)
        hh = 0.5 * g[(dir == 0 ? G_SI : G_SJ) * F + (fwd ? id : nb)];
        if (!fwd) hh = -hh;
      }
      q[dir == 0 ? RC::CI : RC::CJ] = (float)cc;
      q[dir == 0 ? RC::N1I : RC::N1J] = (float)(hh * (dir == 0 ? ni1 : nj1));
      q[dir == 0 ? RC::N2I : RC::N2J] = (float)(hh * (dir == 0 ? ni2 : nj2));
    }
  }
  char *base = reinterpret_cast<char *>(L.rec);
  float4 *wf = reinterpret_cast<float4 *>(base + cell * RC::BYTES);
  float4 *wb = reinterpret_cast<float4 *>(base + ((size_t)L.ncell + cell) * RC::BYTES);
#pragma unroll
  for (int k = 0; k < RC::NF / 4; k++) {
    wf[k] = make_float4(rf[4 * k], rf[4 * k + 1], rf[4 * k + 2], rf[4 * k + 3]);
    wb[k] = make_float4(rb[4 * k], rb[4 * k + 1], rb[4 * k + 2], rb[4 * k + 3]);
  }
}

// acc += dF_n(shipped state, scaled normal) + cc dU_nb
template <int NV>
__device__ __forceinline__ void dflux(const float *s, float n1, float n2, float cc, float *acc) {
  using SL = S32<NV>;
  float unp = s[SL::UP] * n1 + s[SL::VP] * n2;
  float dun = s[SL::DU] * n1 + s[SL::DV] * n2;
  float dp = s[SL::DP];
  acc[0] += s[SL::D + 0] * unp + s[SL::B + 0] * dun + cc * s[SL::D + 0];
  acc[1] += s[SL::D + 1] * unp + s[SL::B + 1] * dun + dp * n1 + cc * s[SL::D + 1];
  acc[2] += s[SL::D + 2] * unp + s[SL::B + 2] * dun + dp * n2 + cc * s[SL::D + 2];
  acc[3] += (s[SL::D + 3] + dp) * unp + s[SL::B + 3] * dun + cc * s[SL::D + 3];
#pragma unroll
  for (int m = 4; m < NV; m++) acc[m] += s[SL::D + m] * unp + s[SL::B + m] * dun + cc * s[SL::D + m];
}

__device__ __forceinline__ void cp16(void *dst, const void *src) {
  unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_wait_ring() { asm volatile("cp.async.wait_group 3;" ::: "memory"); }
// record buffers per thread: the record of the cell three planes ahead is in
// flight while the current one is computed (an FP32 plane is short next to
// the L2 latency)
constexpr int RING32 = 4;
__device__ __forceinline__ void cp_wait0() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

template <int NV>
__device__ __forceinline__ void fetch32(char *dst, const char *src) {
#pragma unroll
  for (int k = 0; k < R32<NV>::BYTES; k += 16) cp16(dst + k, src + k);
}

// One pass of a row, forward (FWD) or backward.
template <int NV, bool fwd>
__device__ __forceinline__ void sweep32_pass(const Lvl &L, float *shf, char *rec, const char *recF, const char *recB,
                                             char *recBw, float *st, const BlkDev &bd, int R, int rl, int j,
                                             bool row_ok, float gm1) {
  using SL = S32<NV>;
  using RC = R32<NV>;
  constexpr int S = SL::S;
  const int nx = bd.nx, ny = bd.ny, rows = ny - 1, ni = nx - 1;
  const char *rsrc = fwd ? recF : recB;
  // record of the k-th visited cell: forward i = 1 + k, backward i = ni - k
  auto src = [&](int k) { return rsrc + (size_t)(fwd ? k : ni - 1 - k) * RC::BYTES; };
  for (int q = 0; q < RING32 - 1; q++) {
    if (row_ok && q < ni) fetch32<NV>(rec + q * RC::BYTES, src(q));
    cp_commit();
  }
  int k = 0;
  for (int pp = 2; pp <= nx + ny - 2; pp++) {
    const int p = fwd ? pp : nx + ny - pp;
    const int i = p - j;
    const int buf = p & 1;
    if (row_ok && i >= 1 && i <= ni) {
      const float4 *cur4 = reinterpret_cast<const float4 *>(rec + (k % RING32) * RC::BYTES);
      if (k + RING32 - 1 < ni) fetch32<NV>(rec + ((k + RING32 - 1) % RING32) * RC::BYTES, src(k + RING32 - 1));
      cp_commit();
      cp_wait_ring();
      // the whole record into registers with 16-byte shared loads at once
      float cur[RC::NF];
#pragma unroll
      for (int q = 0; q < RC::NF / 4; q++) {
        const float4 v = cur4[q];
        cur[4 * q] = v.x; cur[4 * q + 1] = v.y; cur[4 * q + 2] = v.z; cur[4 * q + 3] = v.w;
      }
      float acc[NV];
#pragma unroll
      for (int m = 0; m < NV; m++) acc[m] = fwd ? cur[RC::A + m] : 0.0f;
      if (fwd ? (i > 1) : (i < ni)) dflux<NV>(st, cur[RC::N1I], cur[RC::N2I], cur[RC::CI], acc);
      if (fwd ? (j > 1) : (j < rows)) {
        const float4 *s4 = reinterpret_cast<const float4 *>(shf + ((size_t)(buf ^ 1) * (R + 2) + (fwd ? rl : rl + 2)) * S);
        float sn[S];
#pragma unroll
        for (int m = 0; m < S / 4; m++) {
          float4 v = s4[m];
          sn[4 * m] = v.x; sn[4 * m + 1] = v.y; sn[4 * m + 2] = v.z; sn[4 * m + 3] = v.w;
        }
        dflux<NV>(sn, cur[RC::N1J], cur[RC::N2J], cur[RC::CJ], acc);
      }
      const float ia = cur[RC::IA], ia5 = cur[RC::IA5];
#pragma unroll
      for (int m = 0; m < NV; m++) {
        float inv = (NV == 5 && m == 4) ? ia5 : ia;
        st[SL::D + m] = fwd ? acc[m] * inv : cur[RC::A + m] + acc[m] * inv;
      }
      // state shipped to the two downstream neighbours
#pragma unroll
      for (int m = 0; m < NV; m++) st[SL::B + m] = cur[RC::B + m];
      {
        const float rho = cur[RC::B + 0], m1 = cur[RC::B + 1], m2 = cur[RC::B + 2];
        const float u = cur[RC::BU], v = cur[RC::BV];
        const float dr = st[SL::D + 0], dm1 = st[SL::D + 1], dm2 = st[SL::D + 2], dE = st[SL::D + 3];
        float rr;  // 1 / (rho + d rho): the approximate reciprocal (an FP32 preconditioner)
        asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(rr) : "f"(rho + dr));
        const float du = (dm1 - u * dr) * rr, dv = (dm2 - v * dr) * rr;
        const float up = u + du, vp = v + dv;
        st[SL::UP] = up;
        st[SL::VP] = vp;
        st[SL::DU] = du;
        st[SL::DV] = dv;
        st[SL::DP] = gm1 * (dE - 0.5f * (dm1 * up + m1 * du + dm2 * vp + m2 * dv));
      }
      float4 *own = reinterpret_cast<float4 *>(shf + ((size_t)buf * (R + 2) + rl + 1) * S);
#pragma unroll
      for (int m = 0; m < S / 4; m++) own[m] = make_float4(st[4 * m], st[4 * m + 1], st[4 * m + 2], st[4 * m + 3]);
      // forward: the forward dU becomes the A field of this cell's backward
      // record; backward: the final dU replaces it there, and k_apply32
      // widens it to FP64 afterwards (FP64 instructions hold a warp for
      // about 64 cycles each, so they stay off the wavefront)
      float *w = reinterpret_cast<float *>(recBw + (size_t)(i - 1) * RC::BYTES);
      static_assert(RC::A == 0 && SL::D == 0, "A and D open the record and the slot");
#pragma unroll
      for (int m = 0; m + 3 < NV; m += 4)
        reinterpret_cast<float4 *>(w)[m / 4] = make_float4(st[m], st[m + 1], st[m + 2], st[m + 3]);
#pragma unroll
      for (int m = NV / 4 * 4; m < NV; m++) w[m] = st[m];
      k++;
    }
    __syncthreads();
  }
  cp_wait0();
}

template <int NV>
__global__ void __launch_bounds__(1024) k_lusgs_sweep32(Lvl L) {
  using SL = S32<NV>;
  using RC = R32<NV>;
  constexpr int S = SL::S;
  extern __shared__ __align__(16) float shf[];  // [2][rows+2][S] slots, then [blockDim][RING32] records
  const BlkDev bd = L.blk[blockIdx.x];
  const int rows = bd.ny - 1, ni = bd.nx - 1;
  const int rl = threadIdx.x;
  const int j = rl + 1;
  const int R = blockDim.x;
  const bool row_ok = j <= rows;
  const float gm1 = (float)(L.cs[bd.cas].gamma - 1.0);
  char *rec = reinterpret_cast<char *>(shf + (size_t)2 * (R + 2) * S) + (size_t)threadIdx.x * RING32 * RC::BYTES;
  const char *recF = reinterpret_cast<const char *>(L.rec) + ((size_t)bd.cell0 + (size_t)(j - 1) * ni) * RC::BYTES;
  const char *recB = recF + (size_t)L.ncell * RC::BYTES;
  char *recBw = reinterpret_cast<char *>(L.rec) + ((size_t)L.ncell + bd.cell0 + (size_t)(j - 1) * ni) * RC::BYTES;
  float st[S];
#pragma unroll
  for (int m = 0; m < S; m++) st[m] = 0.0f;
  sweep32_pass<NV, true>(L, shf, rec, recF, recB, recBw, st, bd, R, rl, j, row_ok, gm1);
  sweep32_pass<NV, false>(L, shf, rec, recF, recB, recBw, st, bd, R, rl, j, row_ok, gm1);
}

// dU (FP32, in the backward records) -> U += dU in FP64, or -> L.du
// (NS_Time_advance_LU_SGS, sub_NS_singlegrid.f90:203-211)
template <int NV>
__global__ void __launch_bounds__(TILE) k_apply32(Lvl L, int update) {
  using RC = R32<NV>;
  int2 t = L.tiles[blockIdx.x];
  const BlkDev &b = L.blk[t.x];
  int W = b.nx + 3, lin = t.y + threadIdx.x;
  if (lin >= W * (b.ny + 3)) return;
  int i = lin % W - 1, j = lin / W - 1;
  if (i < 1 || i > b.nx - 1 || j < 1 || j > b.ny - 1) return;
  const long long F = L.F, id = fidx(b, i, j);
  const size_t cell = (size_t)b.cell0 + (size_t)(j - 1) * (b.nx - 1) + (i - 1);
  const float *rb = reinterpret_cast<const float *>(reinterpret_cast<const char *>(L.rec) +
                                                    ((size_t)L.ncell + cell) * RC::BYTES);
  // an updating sweep keeps no DU, as the FP64 sweep (the reference reads DU
  // only inside du_LU_SGS_2D and the update after it)
#pragma unroll
  for (int m = 0; m < NV; m++) {
    double d = (double)rb[RC::A + m];
    if (update) L.U[m * F + id] += d;
    else L.du[m * F + id] = d;
  }
}

template <int NV>
size_t smem32(int rows) {
  int th = ((rows + 31) / 32) * 32;
  return (size_t)2 * (th + 2) * S32<NV>::S * sizeof(float) + (size_t)th * RING32 * R32<NV>::BYTES;
}

template <int NV>
void sweep32_nv(const Lvl &L, double alfa1, int mode, int max_rows, cudaStream_t s) {
  k_lusgs_prep32<NV><<<L.nctiles, TILE, 0, s>>>(L, alfa1, mode & LUSGS_FORCE);
  const int update = mode & LUSGS_UPDATE;
  int th = ((max_rows + 31) / 32) * 32;
  size_t smem = smem32<NV>(max_rows);
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(k_lusgs_sweep32<NV>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k_lusgs_sweep32<NV><<<L.nblk, th, smem, s>>>(L);
  k_apply32<NV><<<L.ntiles, TILE, 0, s>>>(L, update);
}

}  // namespace

size_t lusgs32_smem(int nv, int rows) {
  return nv == 4 ? smem32<4>(rows) : nv == 5 ? smem32<5>(rows) : smem32<6>(rows);
}

void launch_lusgs_fast32(const Lvl &L, double alfa1, int mode, int max_rows, cudaStream_t s) {
  if (L.nvar == 4) sweep32_nv<4>(L, alfa1, mode, max_rows, s);
  else if (L.nvar == 5) sweep32_nv<5>(L, alfa1, mode, max_rows, s);
  else sweep32_nv<6>(L, alfa1, mode, max_rows, s);
}

}  // namespace ec2d
