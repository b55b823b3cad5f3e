// k_sweep.cu -- the LU-SGS operator (du_LU_SGS_2D, sub_LU_SGS.f90:4-108) as a
// latency-optimised wavefront.
//
// The Gauss-Seidel order of the reference is kept exactly: the forward sweep
// visits hyperplanes p = i+j = 2..nx+ny-2, the backward sweep p = nx+ny-2..2,
// and every cell reads only neighbours on plane p-1 (p+1).  The work is split
// so that only the dependency chain sits between two planes:
//   k_lusgs_prep  (all cells in parallel) evaluates everything that does not
//                 depend on the sweep -- 1/alfa, 0.5 Lc + Lv, the face normals
//                 scaled by the reference's +-0.5 s, and the constant half of
//                 the flux difference, -F_n(U_nb, s) of both upstream
//                 neighbours, folded into Res -- and packs them with U into
//                 one 16-byte-aligned record per cell and pass;
//   k_lusgs_sweep (one CTA or one thread-block cluster per block; thread j
//                 owns row j) loads the NEXT cell's record into registers
//                 while it computes the current cell, takes the
//                 own row's previous cell from registers and the neighbouring
//                 row from a double-buffered shared slot, and adds
//                 F_n(U_nb + dU_nb, s) + (0.5 Lc + Lv) (U_nb + dU_nb) to the
//                 record's constant term before the 1/alfa scaling (the same
//                 sum as the reference: F_n is linear in the normal, and the
//                 -(0.5 Lc + Lv) U_nb half of the dissipation term is constant
//                 too, so it sits in the record beside -F_n(U_nb, s)).
// The producer of a state also ships u, v and p of U + dU, so each of its two
// consumers needs no division, and the flux plus dissipation of one neighbour
// folds into seven FMAs: with un = u n1 + v n2 and w = un + cc,
//   rho w,  rho u w + p n1,  rho v w + p n2,  E w + p un  (+ U_m w).
// The FP64 pipe issues one warp instruction per 64 cycles per sub-partition on
// this part, so the operation count per cell, not the dependency depth, sets
// the time per plane.  The backward sweep writes U + dU (the update
// of NS_Time_advance_LU_SGS, sub_NS_singlegrid.f90:203-211): a neighbour needs
// U_old + dU_final of this cell, which is exactly the new U, and F_n(U_old)
// was taken in the pre-pass before any U changed.
#include <algorithm>

#include "ec2d_dev.cuh"
#include "ec2d_internal.h"

namespace ec2d {

constexpr int TILE = EC2D_TILE;

// record layout (doubles), identical for both passes:
//  A    forward: Res + K; backward: the forward dU, or U + dU of the mean
//       flow when the sweep updates U (written by the forward sweep); K =
//       -sum over the upstream neighbours of F_n(U_nb, s) + cc U_nb (mean
//       flow) or F_n(U_nb, s) (turbulence variables)
//  U    U_old of the cell
//  C0   backward only: K of the downstream neighbours
//  CI, CJ  0.5 Lc_nb (+ Lv_nb when viscous)
//  IA, IA5 1/alfa and, for the SA row, 1/(alfa + Lvi + Lvj)
//  N1I..N2J  scaled normals s = +-0.5 (face length) n of face i and face j:
//       the reference multiplies the flux difference by +-0.5 s, and the
//       normal flux is linear in n, so F_n(W, s) = 0.5 s F_n(W, n) and the
//       constant half F_n(U_nb) of the difference moves into the record
template <int NV>
struct Rec {
  static constexpr int A = 0, U = NV, C0 = 2 * NV, CI = 3 * NV, CJ = CI + 1, IA = CI + 2, IA5 = CI + 3,
                       N1I = CI + 4, N2I = CI + 5, N1J = CI + 6, N2J = CI + 7, N = (CI + 8 + 1) / 2 * 2;
  static_assert(N % 2 == 0, "records are whole 16-byte units");
};

// state shipped between neighbours: U2 = U + dU, then u2, v2, p2, then dU of
// the turbulence variables (their dissipation term stays (0.5 Lc + Lv) dU_nb:
// omega and nu~ are large next to their increments, and the folded form
// cc U2 - cc U_nb would round at the scale of cc U)
template <int NV>
struct Slot {
  static constexpr int U = NV, V = NV + 1, P = NV + 2, DT = NV + 3, S = (2 * NV - 1 + 1) / 2 * 2;
  static_assert(S % 2 == 0, "slots are whole 16-byte units");
};

int lusgs_planes(int nv) { return 3 * nv + 10; }  // at least Rec<NV>::N and the FP32 record

// normal flux of the Euler part (+ convected turbulence variables), the F(U)
// half of comput_DFn (sub_LU_SGS.f90:122-137)
template <int NV>
__device__ __forceinline__ void fn(const double *U, double n1, double n2, double gm1, double *Fo) {
  double r = rcp(U[0]);
  double un = (U[1] * n1 + U[2] * n2) * r;
  double p = gm1 * (U[3] - 0.5 * (U[1] * U[1] + U[2] * U[2]) * r);
  Fo[0] = U[0] * un;
  Fo[1] = U[1] * un + p * n1;
  Fo[2] = U[2] * un + p * n2;
  Fo[3] = (U[3] + p) * un;
#pragma unroll
  for (int m = 4; m < NV; m++) Fo[m] = U[m] * un;
}

// acc += F_n(U2, s) + cc U2 (mean flow) or F_n(U2, s) + cc dU (turbulence
// variables) from a shipped state (u, v, p of U2 precomputed by the producer)
template <int NV>
__device__ __forceinline__ void add_shipped(const double *st, double n1, double n2, double cc, double *acc) {
  using SL = Slot<NV>;
  const double p = st[SL::P];
  const double un = fma(st[SL::U], n1, st[SL::V] * n2);
  const double w = un + cc;
  acc[0] = fma(st[0], w, acc[0]);
  acc[1] = fma(st[1], w, fma(p, n1, acc[1]));
  acc[2] = fma(st[2], w, fma(p, n2, acc[2]));
  acc[3] = fma(st[3], w, fma(p, un, acc[3]));
#pragma unroll
  for (int m = 4; m < NV; m++) acc[m] = fma(cc, st[SL::DT + m - 4], fma(st[m], un, acc[m]));
}

template <int NV>
// force: Res + QF in place of Res (the multigrid forcing of a coarse level
// whose residual was evaluated on entry, Add_force_function)
__global__ void __launch_bounds__(TILE) k_lusgs_prep(Lvl L, double alfa1, int force) {
  using RC = Rec<NV>;
  int2 t = L.tiles[blockIdx.x];
  const BlkDev &b = L.blk[t.x];
  int W = b.nx + 3, lin = t.y + threadIdx.x;
  if (lin >= W * (b.ny + 3)) return;
  int i = lin % W - 1, j = lin / W - 1;
  if (i < 1 || i > b.nx - 1 || j < 1 || j > b.ny - 1) return;
  const CaseDev &c = L.cs[b.cas];
  const long long F = L.F, P = b.P;
  const long long id = fidx(b, i, j);
  const double gm1 = c.gamma - 1.0;
  const double *g = L.geo, *lc = L.lc;
  const bool visc = L.visc != 0;
  const size_t cell = (size_t)b.cell0 + (size_t)(j - 1) * (b.nx - 1) + (i - 1);
  // the two records are assembled in registers and written 16 bytes at a time
  double rf[RC::N], rb[RC::N];  // forward and backward record
  double vol = g[G_VOL * F + id];
  double Lv = lc[L_VI * F + id] + lc[L_VJ * F + id];
  double alfa = vol * rcp(lc[L_DT * F + id]) + 1.0 * (lc[L_CI * F + id] + lc[L_CJ * F + id]) + vol * alfa1;
  if (visc) alfa += 2.0 * Lv;
  double ia = rcp(alfa), ia5 = (NV == 5) ? rcp(alfa + Lv) : ia;
  double ni1 = g[G_NI1 * F + id], ni2 = g[G_NI2 * F + id], nj1 = g[G_NJ1 * F + id], nj2 = g[G_NJ2 * F + id];
  double res[NV], K[2][NV];  // K[pass]: -(sum over directions of F_n(U_nb, s))
#pragma unroll
  for (int m = 0; m < NV; m++) {
    double u = L.U[m * F + id];
    res[m] = L.res[m * F + id];
    if (force && m < 4) res[m] = res[m] + L.qf[m * F + id];
    rf[RC::U + m] = u;
    rb[RC::U + m] = u;
    K[0][m] = 0.0;
    K[1][m] = 0.0;
  }
  double *rr[2] = {rf, rb};
#pragma unroll
  for (int pass = 0; pass < 2; pass++) {
    double *r = rr[pass];
    const bool fwd = pass == 0;
    r[RC::IA] = ia; r[RC::IA5] = ia5;
#pragma unroll
    for (int dir = 0; dir < 2; dir++) {  // 0: i-neighbour, 1: j-neighbour
      const long long step = dir == 0 ? 1 : P;
      const long long nb = fwd ? id - step : id + step;
      const bool has = dir == 0 ? (fwd ? i > 1 : i < b.nx - 1) : (fwd ? j > 1 : j < b.ny - 1);
      double cc = 0.0, s1 = 0.0, s2 = 0.0;
      if (has) {
        double Un[NV], Fo[NV];
#pragma unroll
        for (int m = 0; m < NV; m++) Un[m] = L.U[m * F + nb];
        cc = 0.5 * lc[(dir == 0 ? L_CI : L_CJ) * F + nb];
        if (visc) cc += lc[(dir == 0 ? L_VI : L_VJ) * F + nb];
        // forward: +0.5 s of this cell's face; backward: -0.5 s of the
        // neighbour's face with this cell's normal (the reference pairs the
        // normal of face i with the length of face i+1, sub_LU_SGS.f90:87-88,95-96)
        double hh = 0.5 * g[(dir == 0 ? G_SI : G_SJ) * F + (fwd ? id : nb)];
        if (!fwd) hh = -hh;
        s1 = hh * (dir == 0 ? ni1 : nj1);
        s2 = hh * (dir == 0 ? ni2 : nj2);
        fn<NV>(Un, s1, s2, gm1, Fo);
#pragma unroll
        for (int m = 0; m < NV; m++) K[pass][m] -= (m < 4) ? fma(cc, Un[m], Fo[m]) : Fo[m];
      }
      r[dir == 0 ? RC::CI : RC::CJ] = cc;
      r[dir == 0 ? RC::N1I : RC::N1J] = s1;
      r[dir == 0 ? RC::N2I : RC::N2J] = s2;
    }
  }
#pragma unroll
  for (int m = 0; m < NV; m++) {
    rf[RC::A + m] = res[m] + K[0][m];
    rf[RC::C0 + m] = 0.0;
    rb[RC::A + m] = 0.0;
    rb[RC::C0 + m] = K[1][m];
  }
#pragma unroll
  for (int k = RC::CI + 8; k < RC::N; k++) rf[k] = rb[k] = 0.0;
  double2 *wf = reinterpret_cast<double2 *>(L.rec + cell * RC::N);
  double2 *wb = reinterpret_cast<double2 *>(L.rec + ((size_t)L.ncell + cell) * RC::N);
#pragma unroll
  for (int q = 0; q < RC::N / 2; q++) {
    wf[q] = make_double2(rf[2 * q], rf[2 * q + 1]);
    wb[q] = make_double2(rb[2 * q], rb[2 * q + 1]);
  }
}

__device__ __forceinline__ unsigned cluster_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ void cluster_barrier() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
// address of the same shared-memory location in CTA `rank` of the cluster
__device__ __forceinline__ unsigned remote_smem(const void *p, unsigned rank) {
  unsigned local = (unsigned)__cvta_generic_to_shared(p), remote;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(remote) : "r"(local), "r"(rank));
  return remote;
}
__device__ __forceinline__ void st_remote2(unsigned addr, double a, double b) {
  asm volatile("st.shared::cluster.v2.f64 [%0], {%1, %2};" ::"r"(addr), "d"(a), "d"(b) : "memory");
}
// the fields of one record a row needs for its update, held in registers
template <int NV>
struct Cur {
  double a[NV], u[NV], c0[NV];
  double ci, cj, ia, ia5, n1i, n2i, n1j, n2j;
};
// a record as it arrives from memory: the 16-byte pairs one pass needs, loaded
// straight into registers (L2 only: the backward records are written by the
// forward pass of the same kernel)
template <int NV>
struct Raw {
  double2 v[Rec<NV>::N / 2];
};
template <int NV, bool FWD>
__device__ __forceinline__ constexpr bool pair_used(int q) {
  // the forward pass does not read C0
  return !FWD ? true : !(2 * q >= Rec<NV>::C0 && 2 * q + 1 < Rec<NV>::CI);
}
template <int NV, bool FWD>
__device__ __forceinline__ void load_raw(Raw<NV> &r, const double *src) {
  const double2 *s2 = reinterpret_cast<const double2 *>(src);
#pragma unroll
  for (int q = 0; q < Rec<NV>::N / 2; q++)
    if (pair_used<NV, FWD>(q)) r.v[q] = __ldcg(s2 + q);
}
template <int NV>
__device__ __forceinline__ double field(const Raw<NV> &r, int k) { return (k & 1) ? r.v[k >> 1].y : r.v[k >> 1].x; }
template <int NV, bool FWD>
__device__ __forceinline__ void unpack(Cur<NV> &c, const Raw<NV> &r) {
  using RC = Rec<NV>;
#pragma unroll
  for (int m = 0; m < NV; m++) {
    c.a[m] = field(r, RC::A + m);
    c.u[m] = field(r, RC::U + m);
    if (!FWD) c.c0[m] = field(r, RC::C0 + m);
  }
  c.ci = field(r, RC::CI); c.cj = field(r, RC::CJ); c.ia = field(r, RC::IA); c.ia5 = field(r, RC::IA5);
  c.n1i = field(r, RC::N1I); c.n2i = field(r, RC::N2I); c.n1j = field(r, RC::N1J); c.n2j = field(r, RC::N2J);
}

constexpr int SWEEP_MAX_THREADS = 384;

// One pass (forward or backward) of a row.  The record of the next cell the
// row visits is loaded into registers while the current cell is computed,
// so between two barriers only the neighbouring row's state (one
// shared-memory read) sits in front of the FP64 chain.
template <int NV, bool update, bool FWD>
__device__ __forceinline__ void sweep_pass(const Lvl &L, const BlkDev &bd, double *sh, const double *rsrc, double *recBw, double *st, int R, int CS,
                                           unsigned rank, int rl, int j, bool row_ok, double gm1) {
  using SL = Slot<NV>;
  using RC = Rec<NV>;
  constexpr int S = SL::S;
  const int nx = bd.nx, ny = bd.ny, rows = ny - 1, ni = nx - 1;
  const long long F = L.F;
  // record of the k-th visited cell: forward i = 1 + k, backward i = ni - k
  auto src = [&](int k) { return rsrc + (size_t)(FWD ? k : ni - 1 - k) * RC::N; };
  Raw<NV> raw;
  Cur<NV> cur;
  if (row_ok) {
    load_raw<NV, FWD>(raw, src(0));
    unpack<NV, FWD>(cur, raw);
  }
  int k = 0;
  for (int pp = 2; pp <= nx + ny - 2; pp++) {
    const int p = FWD ? pp : nx + ny - pp;
    const int i = p - j;
    const int buf = p & 1;
    if (row_ok && i >= 1 && i <= ni) {
      const bool more = k + 1 < ni;
      if (more) load_raw<NV, FWD>(raw, src(k + 1));
      double acc[NV], dn[NV];
#pragma unroll
      for (int m = 0; m < NV; m++) acc[m] = FWD ? cur.a[m] : cur.c0[m];
      if (FWD ? (i > 1) : (i < ni)) add_shipped<NV>(st, cur.n1i, cur.n2i, cur.ci, acc);
      if (FWD ? (j > 1) : (j < rows)) {
        const double2 *s2 = reinterpret_cast<const double2 *>(sh + ((size_t)(buf ^ 1) * (R + 2) + (FWD ? rl : rl + 2)) * S);
        double sn[S];
#pragma unroll
        for (int m = 0; m < S / 2; m++) { double2 v = s2[m]; sn[2 * m] = v.x; sn[2 * m + 1] = v.y; }
        add_shipped<NV>(sn, cur.n1j, cur.n2j, cur.cj, acc);
      }
#pragma unroll
      for (int m = 0; m < NV; m++) {
        const double inv = (NV == 5 && m == 4) ? cur.ia5 : cur.ia;
        if (update && m < 4) {
          // fused: U + dU* in one fma going forward, carried in the backward
          // record, and U + dU* + dU** in one fma going backward
          st[m] = fma(acc[m], inv, FWD ? cur.u[m] : cur.a[m]);
        } else {
          dn[m] = FWD ? acc[m] * inv : fma(acc[m], inv, cur.a[m]);
          st[m] = cur.u[m] + dn[m];
        }
      }
#pragma unroll
      for (int m = 4; m < NV; m++) st[SL::DT + m - 4] = dn[m];
      const double rd = rcp(st[0]);
      st[SL::U] = st[1] * rd;
      st[SL::V] = st[2] * rd;
      st[SL::P] = gm1 * fma(-0.5, fma(st[2], st[SL::V], st[1] * st[SL::U]), st[3]);
      double2 *own = reinterpret_cast<double2 *>(sh + ((size_t)buf * (R + 2) + rl + 1) * S);
#pragma unroll
      for (int m = 0; m < S / 2; m++) own[m] = make_double2(st[2 * m], st[2 * m + 1]);
      if (CS > 1) {
        if (FWD && rl == R - 1 && (int)rank + 1 < CS) {
          unsigned a = remote_smem(sh + ((size_t)buf * (R + 2) + 0) * S, rank + 1);
#pragma unroll
          for (int m = 0; m < S / 2; m++) st_remote2(a + 16u * m, st[2 * m], st[2 * m + 1]);
        }
        if (!FWD && rl == 0 && rank > 0) {
          unsigned a = remote_smem(sh + ((size_t)buf * (R + 2) + R + 1) * S, rank - 1);
#pragma unroll
          for (int m = 0; m < S / 2; m++) st_remote2(a + 16u * m, st[2 * m], st[2 * m + 1]);
        }
      }
      if (FWD) {
        // the forward result becomes the A field of this cell's backward record
        double *w = recBw + (size_t)(i - 1) * RC::N;
        double val[NV];
#pragma unroll
        for (int m = 0; m < NV; m++) val[m] = (update && m < 4) ? st[m] : dn[m];
#pragma unroll
        for (int m = 0; m + 1 < NV; m += 2) reinterpret_cast<double2 *>(w + RC::A)[m / 2] = make_double2(val[m], val[m + 1]);
        if (NV & 1) w[RC::A + NV - 1] = val[NV - 1];
      } else {
        // an updating sweep writes U only: the reference reads DU nowhere but
        // inside du_LU_SGS_2D and the update that follows it
        const long long id = bd.off + (long long)(j + 2) * bd.P + (i + 2);
#pragma unroll
        for (int m = 0; m < NV; m++) {
          if (update) L.U[m * F + id] = st[m];
          else L.du[m * F + id] = dn[m];
        }
      }
      if (more) unpack<NV, FWD>(cur, raw);
      k++;
    }
    if (CS > 1) cluster_barrier();
    else __syncthreads();
  }
}

// Narrow blocks (the coarse multigrid levels): LPR lanes per row, each lane
// owning some of the row's variables.  An FP64 warp instruction costs the
// same whatever the number of active lanes, so spreading one cell's
// accumulation over 2 or 4 lanes of the same instruction stream shortens the
// chain per plane (21 FP64 operations instead of 31 with four lanes) as long
// as the rows times LPR still fit one warp per SM sub-partition.  Lane q of a row owns
// the variables var(q, k); both neighbours' states come from the shared
// slots (the own row's previous cell included), the mean flow of U + dU is
// gathered across the row's lanes by shuffles, and every lane forms u, v, p.
template <int NV, int LPR>
struct Lanes {
  static constexpr int MV = 4 / LPR;                    // mean-flow variables per lane
  static constexpr int TV = (NV - 4 + LPR - 1) / LPR;   // turbulence variables per lane
  static constexpr int VPL = MV + TV;
  __device__ static int var(int q, int k) { return k < MV ? q * MV + k : 4 + (k - MV) * LPR + q; }
  __host__ __device__ static constexpr int lane_of(int m) { return m < 4 ? m / MV : (m - 4) % LPR; }
  __host__ __device__ static constexpr int reg_of(int m) { return m < 4 ? m % MV : MV + (m - 4) / LPR; }
};
template <int NV, int LPR>
struct CurL {
  double a[Lanes<NV, LPR>::VPL], u[Lanes<NV, LPR>::VPL], c0[Lanes<NV, LPR>::VPL];
  double ci, cj, ia, ia5, n1i, n2i, n1j, n2j;
};

template <int NV, bool update, bool FWD, int LPR>
__device__ __forceinline__ void sweep_pass_lanes(const Lvl &L, const BlkDev &bd, double *sh, const double *rsrc,
                                                 double *recBw, int R, int rl, int q, int gbase, int j, bool row_ok,
                                                 double gm1) {
  using SL = Slot<NV>;
  using RC = Rec<NV>;
  using LN = Lanes<NV, LPR>;
  constexpr int S = SL::S, VPL = LN::VPL;
  const int nx = bd.nx, ny = bd.ny, rows = ny - 1, ni = nx - 1;
  const long long F = L.F;
  int mv[VPL];
  bool ok[VPL];
#pragma unroll
  for (int k = 0; k < VPL; k++) {
    const int m = LN::var(q, k);
    ok[k] = m < NV;
    mv[k] = ok[k] ? m : 0;
  }
  auto src = [&](int k) { return rsrc + (size_t)(FWD ? k : ni - 1 - k) * RC::N; };
  auto load = [&](CurL<NV, LPR> &c, const double *r) {
#pragma unroll
    for (int k = 0; k < VPL; k++) {
      c.a[k] = __ldcg(r + RC::A + mv[k]);
      c.u[k] = __ldcg(r + RC::U + mv[k]);
      if (!FWD) c.c0[k] = __ldcg(r + RC::C0 + mv[k]);
    }
    c.ci = __ldcg(r + RC::CI); c.cj = __ldcg(r + RC::CJ); c.ia = __ldcg(r + RC::IA); c.ia5 = __ldcg(r + RC::IA5);
    c.n1i = __ldcg(r + RC::N1I); c.n2i = __ldcg(r + RC::N2I); c.n1j = __ldcg(r + RC::N1J); c.n2j = __ldcg(r + RC::N2J);
  };
  CurL<NV, LPR> cur, nxt;
  if (row_ok) load(cur, src(0));
  int k = 0;
  for (int pp = 2; pp <= nx + ny - 2; pp++) {
    const int p = FWD ? pp : nx + ny - pp;
    const int i = p - j;
    const int buf = p & 1;
    const bool act = row_ok && i >= 1 && i <= ni;
    const bool more = act && k + 1 < ni;
    double myst[VPL], dn[VPL];
#pragma unroll
    for (int kk = 0; kk < VPL; kk++) myst[kk] = dn[kk] = 0.0;
    if (act) {
      if (more) load(nxt, src(k + 1));
      double acc[VPL];
#pragma unroll
      for (int kk = 0; kk < VPL; kk++) acc[kk] = FWD ? cur.a[kk] : cur.c0[kk];
      // acc += F_n(U2, s) + cc U2 of a neighbour from its shared slot, own variables only
      auto add_nb = [&](const double *sl, double n1, double n2, double cc) {
        const double pn = sl[SL::P];
        const double un = fma(sl[SL::U], n1, sl[SL::V] * n2), w = un + cc;
#pragma unroll
        for (int kk = 0; kk < VPL; kk++) {
          const int m = mv[kk];
          if (kk < LN::MV) {
            const double coef = m == 1 ? n1 : m == 2 ? n2 : m == 3 ? un : 0.0;
            acc[kk] = fma(sl[m], w, fma(pn, coef, acc[kk]));
          } else {
            acc[kk] = fma(cc, sl[SL::DT + m - 4], fma(sl[m], un, acc[kk]));
          }
        }
      };
      if (FWD ? (i > 1) : (i < ni)) add_nb(sh + ((size_t)(buf ^ 1) * (R + 2) + rl + 1) * S, cur.n1i, cur.n2i, cur.ci);
      if (FWD ? (j > 1) : (j < rows))
        add_nb(sh + ((size_t)(buf ^ 1) * (R + 2) + (FWD ? rl : rl + 2)) * S, cur.n1j, cur.n2j, cur.cj);
#pragma unroll
      for (int kk = 0; kk < VPL; kk++) {
        const double inv = (NV == 5 && mv[kk] == 4) ? cur.ia5 : cur.ia;
        if (update && kk < LN::MV) {
          myst[kk] = fma(acc[kk], inv, FWD ? cur.u[kk] : cur.a[kk]);
        } else {
          dn[kk] = FWD ? acc[kk] * inv : fma(acc[kk], inv, cur.a[kk]);
          myst[kk] = cur.u[kk] + dn[kk];
        }
      }
    }
    // every lane of the warp takes part in the gathers
    double s4[4];
#pragma unroll
    for (int m = 0; m < 4; m++) s4[m] = __shfl_sync(0xffffffffu, myst[LN::reg_of(m)], gbase + LN::lane_of(m));
    if (act) {
      const double rd = rcp(s4[0]);
      const double u = s4[1] * rd, v = s4[2] * rd;
      const double pr = gm1 * fma(-0.5, fma(s4[2], v, s4[1] * u), s4[3]);
      double *own = sh + ((size_t)buf * (R + 2) + rl + 1) * S;
#pragma unroll
      for (int kk = 0; kk < VPL; kk++) {
        if (!ok[kk]) continue;
        own[mv[kk]] = myst[kk];
        if (kk >= LN::MV) own[SL::DT + mv[kk] - 4] = dn[kk];
      }
      if (q == 0) { own[SL::U] = u; own[SL::V] = v; own[SL::P] = pr; }
      if (FWD) {
        double *w = recBw + (size_t)(i - 1) * RC::N;
#pragma unroll
        for (int kk = 0; kk < VPL; kk++)
          if (ok[kk]) w[RC::A + mv[kk]] = (update && kk < LN::MV) ? myst[kk] : dn[kk];
      } else {
        const long long id = bd.off + (long long)(j + 2) * bd.P + (i + 2);
#pragma unroll
        for (int kk = 0; kk < VPL; kk++) {
          if (!ok[kk]) continue;
          if (update) L.U[mv[kk] * F + id] = myst[kk];
          else L.du[mv[kk] * F + id] = dn[kk];
        }
      }
      if (more) cur = nxt;
      k++;
    }
    __syncthreads();
  }
}

template <int NV, bool update, int LPR>
__global__ void __launch_bounds__(128) k_lusgs_sweep_lanes(Lvl L, int R) {
  constexpr int S = Slot<NV>::S;
  extern __shared__ __align__(16) double sh[];  // [2][R+2][S] slots
  const BlkDev bd = L.blk[blockIdx.x];
  const int rows = bd.ny - 1, ni = bd.nx - 1;
  const int rl = threadIdx.x / LPR, q = threadIdx.x % LPR;
  const int gbase = (threadIdx.x & 31) / LPR * LPR;
  const int j = rl + 1;
  const bool row_ok = rl < R && j <= rows;
  const double gm1 = L.cs[bd.cas].gamma - 1.0;
  const int jr = row_ok ? j : 1;  // record pointers of idle lanes stay in the array
  const double *recF = L.rec + ((size_t)bd.cell0 + (size_t)(jr - 1) * ni) * Rec<NV>::N;
  const double *recB = recF + (size_t)L.ncell * Rec<NV>::N;
  double *recBw = L.rec + ((size_t)L.ncell + bd.cell0 + (size_t)(jr - 1) * ni) * Rec<NV>::N;
  (void)S;
  sweep_pass_lanes<NV, update, true, LPR>(L, bd, sh, recF, recBw, R, rl, q, gbase, j, row_ok, gm1);
  sweep_pass_lanes<NV, update, false, LPR>(L, bd, sh, recB, recBw, R, rl, q, gbase, j, row_ok, gm1);
}

// lanes per row for a level whose widest block has `rows` rows: 4 when
// rows x 4 fits one warp per sub-partition of one SM (128 lanes).  Two lanes
// per row save 5 of 31 FP64 operations, less than the added loads, shuffles
// and selects cost (2 x 48 x 48 level: 283 us against 276 us for one lane);
// four save 10 (2 x 24 x 24 level: 124 us against 146 us).
int sweep_lanes_per_row(int rows) { return rows * 4 <= 128 ? 4 : 1; }

template <int NV, int LPR>
void launch_lanes(const Lvl &L, int update, int R, cudaStream_t s) {
  const int th = (R * LPR + 31) / 32 * 32;
  const size_t smem = (size_t)2 * (R + 2) * Slot<NV>::S * sizeof(double);
  if (update) k_lusgs_sweep_lanes<NV, true, LPR><<<L.nblk, th, smem, s>>>(L, R);
  else k_lusgs_sweep_lanes<NV, false, LPR><<<L.nblk, th, smem, s>>>(L, R);
}

// CS == 1: one CTA per block, planes separated by __syncthreads.
// CS > 1: a cluster of CS CTAs per block, CTA r owns rows r*R+1..r*R+R; the
// edge rows write into the neighbour CTA's halo slot through distributed
// shared memory and planes are separated by a cluster barrier.
template <int NV, bool update>
__global__ void __launch_bounds__(SWEEP_MAX_THREADS) k_lusgs_sweep(Lvl L, int R, int CS, int RPW) {
  using SL = Slot<NV>;
  using RC = Rec<NV>;
  constexpr int S = SL::S;
  extern __shared__ __align__(16) double sh[];  // [2][R+2][S] slots
  const unsigned rank = CS > 1 ? cluster_rank() : 0u;
  const BlkDev bd = L.blk[blockIdx.x / CS];  // by value: no re-reads after global stores
  const int rows = bd.ny - 1, ni = bd.nx - 1;
  // RPW rows per warp (lanes RPW..31 idle): fewer rows per warp spread a
  // plane's work over more SM sub-partitions
  const int lane_w = threadIdx.x & 31;
  const int rl = lane_w < RPW ? (int)(threadIdx.x >> 5) * RPW + lane_w : R;
  const int j = (int)rank * R + rl + 1;
  const bool row_ok = rl < R && j <= rows;
  const double gm1 = L.cs[bd.cas].gamma - 1.0;
  const double *recF = L.rec + ((size_t)bd.cell0 + (size_t)(j - 1) * ni) * RC::N;   // row j, i = 1
  const double *recB = recF + (size_t)L.ncell * RC::N;
  double *recBw = L.rec + ((size_t)L.ncell + bd.cell0 + (size_t)(j - 1) * ni) * RC::N;
  double st[S];
#pragma unroll
  for (int m = 0; m < S; m++) st[m] = 0.0;
  sweep_pass<NV, update, true>(L, bd, sh, recF, recBw, st, R, CS, rank, rl, j, row_ok, gm1);
  sweep_pass<NV, update, false>(L, bd, sh, recB, recBw, st, R, CS, rank, rl, j, row_ok, gm1);
}

template <int NV>
size_t smem_bytes(int R, int th) {
  (void)th;
  return (size_t)2 * (R + 2) * Slot<NV>::S * sizeof(double);
}

template <int NV>
void sweep_nv(const Lvl &L, double alfa1, int mode, int max_rows, int cs, int rpw, cudaStream_t s) {
  k_lusgs_prep<NV><<<L.ntiles, TILE, 0, s>>>(L, alfa1, mode & LUSGS_FORCE);
  const int update = mode & LUSGS_UPDATE;
  const int lpr = sweep_lanes_per_row(max_rows);
  if (lpr == 4) { launch_lanes<NV, 4>(L, update, max_rows, s); return; }
  int CS = std::max(1, std::min(cs, std::min(8, (max_rows + 7) / 8)));
  int R = (max_rows + CS - 1) / CS;
  if (rpw < 1 || rpw > 32) rpw = 32;
  int th = ((R + rpw - 1) / rpw) * 32;
  size_t smem = smem_bytes<NV>(R, th);
  if (smem > 227 * 1024 || th > SWEEP_MAX_THREADS) {  // fall back to full warps
    rpw = 32;
    th = ((R + 31) / 32) * 32;
    smem = smem_bytes<NV>(R, th);
  }
  auto kern = update ? k_lusgs_sweep<NV, true> : k_lusgs_sweep<NV, false>;
  if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(L.nblk * CS);
  cfg.blockDim = dim3(th);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CS;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, kern, L, R, CS, rpw);
}

// one CTA holding every row of the widest block, or SIZE_MAX when the rows
// exceed the CTA's thread limit
template <int NV>
size_t smem_nv(int rows) {
  int th = ((rows + 31) / 32) * 32;
  if (th > SWEEP_MAX_THREADS) return (size_t)-1;
  return smem_bytes<NV>(rows, th);
}
size_t lusgs_smem(int nv, int rows) { return nv == 4 ? smem_nv<4>(rows) : nv == 5 ? smem_nv<5>(rows) : smem_nv<6>(rows); }

void launch_lusgs_fast(const Lvl &L, double alfa1, int mode, int max_rows, int cs, int rpw, cudaStream_t s) {
  if (L.nvar == 4) sweep_nv<4>(L, alfa1, mode, max_rows, cs, rpw, s);
  else if (L.nvar == 5) sweep_nv<5>(L, alfa1, mode, max_rows, cs, rpw, s);
  else sweep_nv<6>(L, alfa1, mode, max_rows, cs, rpw, s);
}

}  // namespace ec2d
