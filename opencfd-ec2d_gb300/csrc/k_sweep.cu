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
//  G1I..GCJ  (gamma - 1) times n1, n2 and cc of face i and j,
//       the pressure coefficients of the multi-lane sweep, which ships
//       p / (gamma - 1)
template <int NV>
struct Rec {
  static constexpr int A = 0, U = NV, C0 = 2 * NV, CI = 3 * NV, CJ = CI + 1, IA = CI + 2, IA5 = CI + 3,
                       N1I = CI + 4, N2I = CI + 5, N1J = CI + 6, N2J = CI + 7, G1I = CI + 8, G2I = CI + 9,
                       GCI = CI + 10, G1J = CI + 11, G2J = CI + 12, GCJ = CI + 13,
                       N = (CI + 8 + 6 + 1) / 2 * 2;
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

// at least Rec<NV>::N (26, 30, 32 for NV = 4, 5, 6) and the FP32 record
int lusgs_planes(int nv) { return 3 * nv + 15; }
static_assert(Rec<4>::N <= 3 * 4 + 15 && Rec<5>::N <= 3 * 5 + 15 && Rec<6>::N <= 3 * 6 + 15, "record planes");

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
      {
        r[dir == 0 ? RC::G1I : RC::G1J] = gm1 * s1;
        r[dir == 0 ? RC::G2I : RC::G2J] = gm1 * s2;
        r[dir == 0 ? RC::GCI : RC::GCJ] = gm1 * cc;
      }
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
  for (int k = RC::CI + 8 + 6; k < RC::N; k++) rf[k] = rb[k] = 0.0;
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
  // the forward pass does not read C0; the pressure coefficients of the
  // four-lane sweep are not read here
  return 2 * q < Rec<NV>::CI + 8 && (!FWD ? true : !(2 * q >= Rec<NV>::C0 && 2 * q + 1 < Rec<NV>::CI));
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

// ---- mean flow only (NV = 4): four or eight lanes per row, row bands -------
//
// Lane q of a row owns variable q.  A neighbour's state is held as
// X = (rho, rho u, rho v, H = E + p) with u, v and p' = p / (gamma - 1), so
// that its flux plus dissipation in variable q is one pair of FMAs,
// X_q w + p' g_q with w = u n1 + v n2 + cc and g = (gamma - 1) (0, n1, n2,
// -cc) taken from the record (E w + p un = H w - p cc).  With four lanes per
// row a lane adds both neighbours: 18 FP64 operations per cell and lane (2 x
// 4 for the neighbours, one for the update, and rcp(rho), u, v, p', H of the
// new state, formed by every lane of the row after the four variables are
// gathered by shuffles).  With eight, lanes 0-3 add the row's own previous
// cell and lanes 4-7 the neighbouring row on operands selected per lane (one
// FP64 instruction stream for both halves), and a shuffle-add joins them:
// 15 operations.  A CTA holds at most 32 rows of four lanes or 16 of eight
// (up to four warps, one per SM sub-partition); a block with more rows is
// split into bands of R rows on the CTAs of a cluster.  The band edge does
// not wait for a barrier: the edge row of the upstream band writes each new
// state straight into the downstream CTA's inbox (one 64-byte entry and one
// mbarrier per column, through distributed shared memory), and the
// downstream edge row waits for that column's entry only, so the bands run
// as a pipeline a few planes apart.  The per-lane pressure coefficient g_q
// is a record field picked by a per-lane offset and masked or sign-flipped
// with integer operations, so the lanes of a row need no branches or FP64
// selects for it.
constexpr int QROWS = 32;        // rows per CTA
constexpr int QCOLS = 1024;      // cells per row the inboxes hold
constexpr int QWAIT = 1 << 20;   // polls of an inbox mbarrier before the wait gives up (about 20 ms)

struct QRec {
  double a, u, c0, ki, kj;  // ki, kj: the lane's raw coefficient field of face i and j
  double2 c, ia, ni, nj;    // (0.5 Lc + Lv) i / j, 1/alfa, scaled normals of face i and j
  double at[2], ut[2], c0t[2];  // NV = 5, 6: the turbulence rows' A, U and C0
  double ia5;                   // NV = 5: 1/(alfa + Lv) of the SA row
};
// doubles per row of a slot and per inbox entry: rho, rho u, rho v, H (or E),
// u, v, p / (gamma - 1), one spare; then U + dU and dU of each turbulence
// variable (NV = 5: nu~; 6: k, omega)
template <int NV>
constexpr int qslot() { return 8 + 2 * (NV - 4); }
// per-lane record offsets of the pressure coefficient g_q: (gamma - 1) n1
// (q = 1), n2 (q = 2), cc (q = 3, sign flipped below), any field for q = 0
// (zeroed)
struct QLane {
  int offi, offj;
  unsigned keep, sign;
  // eight lanes per row: the half's own face (i for lanes 0-3, j for 4-7)
  int offk, offn, offc;
  bool own;
};
template <int NV = 4>
__device__ __forceinline__ QLane qlane(int q, bool own = true) {
  using RC = Rec<NV>;
  QLane l;
  l.offi = q == 1 ? RC::G1I : q == 2 ? RC::G2I : RC::GCI;
  l.offj = q == 1 ? RC::G1J : q == 2 ? RC::G2J : RC::GCJ;
  l.keep = q == 0 ? 0u : 0xffffffffu;
  l.sign = q == 3 ? 0x80000000u : 0u;
  l.own = own;
  l.offk = own ? l.offi : l.offj;
  l.offn = own ? RC::N1I : RC::N1J;
  l.offc = own ? RC::CI : RC::CJ;
  return l;
}
// g_q from the raw field by integer operations only (zero for q = 0, negated for q = 3)
__device__ __forceinline__ double qcoef(double x, const QLane &l) {
  return __hiloint2double((__double2hiint(x) & (int)l.keep) ^ (int)l.sign, __double2loint(x) & (int)l.keep);
}
// four lanes per row load both faces' fields; eight load their half's face
// only (into ki, ni, c.x) and the fields their half uses
template <bool FWD, bool update, int LPR = 4, int NV = 4>
__device__ __forceinline__ void qload(QRec &r, const double *rec, int q, const QLane &l) {
  using RC = Rec<NV>;
  if (LPR == 8) {
    if (!FWD || l.own) r.a = __ldcg(rec + RC::A + q);
    if (FWD || !update) r.u = __ldcg(rec + RC::U + q);
    if (!FWD && l.own) r.c0 = __ldcg(rec + RC::C0 + q);
    r.ki = __ldcg(rec + l.offk);
    if (NV == 5) {
      // the normals sit at odd offsets of a 5-variable record: two 8-byte loads
      r.ni.x = __ldcg(rec + l.offn);
      r.ni.y = __ldcg(rec + l.offn + 1);
      r.ia5 = __ldcg(rec + RC::IA5);
    } else {
      r.ni = __ldcg(reinterpret_cast<const double2 *>(rec + l.offn));
    }
#pragma unroll
    for (int t = 0; t < NV - 4; t++) {
      r.at[t] = __ldcg(rec + RC::A + 4 + t);
      r.ut[t] = __ldcg(rec + RC::U + 4 + t);
      if (!FWD) r.c0t[t] = __ldcg(rec + RC::C0 + 4 + t);
    }
    r.c.x = __ldcg(rec + l.offc);
    r.ia.x = __ldcg(rec + RC::IA);
    return;
  }
  r.a = __ldcg(rec + RC::A + q);
  if (FWD || !update) r.u = __ldcg(rec + RC::U + q);
  if (!FWD) r.c0 = __ldcg(rec + RC::C0 + q);
  r.ki = __ldcg(rec + l.offi);
  r.kj = __ldcg(rec + l.offj);
  const double2 *p2 = reinterpret_cast<const double2 *>(rec + RC::CI);
  r.c = __ldcg(p2);
  r.ia = __ldcg(p2 + 1);
  r.ni = __ldcg(p2 + 2);
  r.nj = __ldcg(p2 + 3);
}
// Inbox entries arrive by st.async, each 16-byte store counting its bytes on
// the entry's mbarrier in the receiving CTA: no fence on the sending side.
// The receiver arms every entry's mbarrier at start-up (one arrival expecting
// the entry's bytes: 64, or 80 / 96 with the SA / SST rows), so phase 0
// completes when the entry has landed.
__device__ __forceinline__ void qarm(unsigned long long *mb, unsigned bytes) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(mb);
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(1) : "memory");
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(a), "r"(bytes) : "memory");
}
// bounded wait for an inbox entry (phase 0 of its mbarrier); false: gave up
__device__ __forceinline__ bool qwait(const unsigned long long *mb) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(mb);
  for (int n = 0; n < QWAIT; n++) {
    unsigned done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.test_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], 0;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(a)
        : "memory");
    if (done) return true;
  }
  return false;
}
__device__ __forceinline__ void qsend2(unsigned raddr, double x, double y, unsigned rmb) {
  asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v2.f64 [%0], {%1, %2}, [%3];" ::"r"(raddr),
               "d"(x), "d"(y), "r"(rmb)
               : "memory");
}

struct QBand {
  int R, CS, rl, q, j, rows, ni, bk;
  unsigned rank;
  bool row_ok;
};

// One pass of a band.  Records are requested three cells ahead into four
// register sets used in turn by plane number mod 4 (the loop is unrolled by
// four, so no set is ever copied while its loads are in flight): a record
// has three planes to arrive, enough for a read that crosses to the other
// die's L2.  The band-edge state goes to the next band by st.async, its
// bytes counted on the receiving entry's mbarrier (no fence on this side).
// NV = 5, 6 (eight lanes only): every lane also carries the turbulence
// rows, the upstream neighbour of its half adding F_n(X_2) + (0.5 Lc + Lv) dX
// as the one-lane sweep does; lane q = 0 of the leading half stores them.
template <bool update, bool FWD, int LPR, int NV = 4>
__device__ __forceinline__ void qpass(const Lvl &L, const BlkDev &bd, const QBand &B, double *slot, double *inbox,
                                      unsigned long long *mbar, unsigned rbox, unsigned rmbar, const double *rsrc,
                                      double *recBw, double gm1) {
  using RC = Rec<NV>;
  constexpr int QS = qslot<NV>();
  static_assert(NV == 4 || LPR == 8, "the turbulence rows ride on the eight-lane form only");
  constexpr int NT = NV - 4;  // turbulence rows
  const int R = B.R, rl = B.rl, q = B.q, j = B.j, rows = B.rows, ni = B.ni;
  const long long F = L.F;
  const QLane ln = qlane<NV>(q, LPR == 4 || !((threadIdx.x >> 2) & 1));
  // this row's neighbour across the band edge comes through the inbox; the
  // band's edge row feeds the next band's inbox
  const bool from_box = B.row_ok && (FWD ? (rl == 0 && B.rank > 0) : (rl == R - 1 && (int)B.rank + 1 < B.CS && j < rows));
  const bool to_box = B.row_ok && !L.silent_band_edge &&
                      (FWD ? (rl == R - 1 && (int)B.rank + 1 < B.CS && j < rows) : (rl == 0 && B.rank > 0));
  auto src = [&](int k) { return rsrc + (size_t)(FWD ? k : ni - 1 - k) * RC::N; };
  const int j0 = (int)B.rank * R + 1, j1 = min((int)B.rank * R + R, rows);
  const int plo = j0 + 1, phi = j1 + ni;  // planes holding a cell of this band
  // plane p of this pass reads the record in set (pass position of p) mod 4
  auto pos = [&](int p) { return FWD ? p - plo : phi - p; };
  QRec r0, r1, r2, r3;
  if (B.row_ok) {
    // the row's first three cells into the sets of their planes
    const int m0 = pos(FWD ? j + 1 : ni + j) % 4;  // set of the row's first cell
#pragma unroll
    for (int c = 0; c < 3; c++) {
      if (c >= ni) break;
      const int m = (m0 + c) & 3;
      if (m == 0) qload<FWD, update, LPR, NV>(r0, src(c), q, ln);
      else if (m == 1) qload<FWD, update, LPR, NV>(r1, src(c), q, ln);
      else if (m == 2) qload<FWD, update, LPR, NV>(r2, src(c), q, ln);
      else qload<FWD, update, LPR, NV>(r3, src(c), q, ln);
    }
  }
  double wx = 0.0, wu = 0.0, wv = 0.0, wp = 0.0;  // the row's previous cell
  double wt[2] = {0.0, 0.0}, wd[2] = {0.0, 0.0};   // and its turbulence X + dX, dX
  int gave_up = 0;                                 // first column whose inbox wait gave up
  const int gl = (threadIdx.x & 31) & ~(LPR - 1);  // the row's first lane
  // eight lanes per row: lanes 0-3 take the row's own previous cell, lanes
  // 4-7 the neighbouring row; four lanes per row take both
  const bool own_nb = LPR == 4 || !((threadIdx.x >> 2) & 1), row_nb = LPR == 4 || !own_nb;
  const bool lead = LPR == 4 || own_nb;  // stores and sends
  // cur: this plane's record; ahead: the set three planes on (free since the last plane)
  auto plane = [&](int p, const QRec &cur, QRec &ahead) {
    const int i = p - j, buf = p & 1;
    const bool act = B.row_ok && i >= 1 && i <= ni;
    const int k = FWD ? i - 1 : ni - i;
    if (act && k + 3 < ni) qload<FWD, update, LPR, NV>(ahead, src(k + 3), q, ln);
    double acc = 0.0, acct[2] = {0.0, 0.0};
    if (act) {
      if (LPR == 4) {
        acc = FWD ? cur.a : cur.c0;
        if (FWD ? (i > 1) : (i < ni)) {
          const double w = fma(wu, cur.ni.x, fma(wv, cur.ni.y, cur.c.x));
          acc = fma(wx, w, fma(wp, qcoef(cur.ki, ln), acc));
        }
        if (FWD ? (j > 1) : (j < rows)) {
          const double *s;
          if (from_box) {
            // after one wait has given up the row no longer waits (its results
            // are void; the step reports EC2D_ERR_TIMEOUT)
            if (!gave_up && !qwait(mbar + i - 1)) gave_up = i;
            s = inbox + (size_t)(i - 1) * QS;
          } else {
            s = slot + ((size_t)(buf ^ 1) * R + (FWD ? rl - 1 : rl + 1)) * QS;
          }
          const double2 uv = *reinterpret_cast<const double2 *>(s + 4);
          const double sp = s[6], sx = s[q];
          const double w = fma(uv.x, cur.nj.x, fma(uv.y, cur.nj.y, cur.c.y));
          acc = fma(sx, w, fma(sp, qcoef(cur.kj, ln), acc));
        }
      } else {
        // both halves run the same FP64 instructions on their own operands
        const double *s = slot + ((size_t)(buf ^ 1) * R + min(max(FWD ? rl - 1 : rl + 1, 0), R - 1)) * QS;
        if (row_nb && from_box) {
          if (!gave_up && !qwait(mbar + i - 1)) gave_up = i;
          s = inbox + (size_t)(i - 1) * QS;
        }
        const double2 uv = *reinterpret_cast<const double2 *>(s + 4);
        const double sp = s[6], sx = s[q];
        const bool has = own_nb ? (FWD ? (i > 1) : (i < ni)) : (FWD ? (j > 1) : (j < rows));
        const double X = own_nb ? wx : sx, Uu = own_nb ? wu : uv.x, Vv = own_nb ? wv : uv.y, P = own_nb ? wp : sp;
        // the record fields of this half's face (loaded per half)
        acc = own_nb ? (FWD ? cur.a : cur.c0) : 0.0;
#pragma unroll
        for (int t = 0; t < NT; t++) acct[t] = own_nb ? (FWD ? cur.at[t] : cur.c0t[t]) : 0.0;
        if (has) {
          const double w = fma(Uu, cur.ni.x, fma(Vv, cur.ni.y, cur.c.x));
          acc = fma(X, w, fma(P, qcoef(cur.ki, ln), acc));
          if (NT > 0) {
            // F_n(X_2) + (0.5 Lc + Lv) dX: the dissipation on the increment,
            // as the one-lane sweep (add_shipped) forms it
            const double un = fma(Uu, cur.ni.x, Vv * cur.ni.y);
#pragma unroll
            for (int t = 0; t < NT; t++) {
              const double T2 = own_nb ? wt[t] : s[8 + 2 * t], D2 = own_nb ? wd[t] : s[9 + 2 * t];
              acct[t] = fma(cur.c.x, D2, fma(T2, un, acct[t]));
            }
          }
        }
      }
    }
    // eight lanes: the two halves of the row add their neighbours' terms
    const double other = LPR == 8 ? __shfl_xor_sync(0xffffffffu, acc, 4) : 0.0;
    double othert[2] = {0.0, 0.0};
#pragma unroll
    for (int t = 0; t < NT; t++) othert[t] = __shfl_xor_sync(0xffffffffu, acct[t], 4);
    double st = 0.0, dn = 0.0, stt[2] = {0.0, 0.0}, dnt[2] = {0.0, 0.0};
    if (act) {
      if (LPR == 8) acc = acc + other;
#pragma unroll
      for (int t = 0; t < NT; t++) {
        // the turbulence rows never take the fused U update (only the mean
        // flow is carried as U + dU); the SA row has its own 1/alfa
        const double inv = NV == 5 ? cur.ia5 : cur.ia.x;
        const double a = acct[t] + othert[t];
        dnt[t] = FWD ? a * inv : fma(a, inv, cur.at[t]);
        stt[t] = cur.ut[t] + dnt[t];
      }
      if (update) {
        // U + dU* going forward (carried in the backward record), U + dU* + dU** going backward
        st = fma(acc, cur.ia.x, FWD ? cur.u : cur.a);
      } else {
        dn = FWD ? acc * cur.ia.x : fma(acc, cur.ia.x, cur.a);
        st = cur.u + dn;
      }
    }
    const double s0 = __shfl_sync(0xffffffffu, st, gl), s1 = __shfl_sync(0xffffffffu, st, gl + 1);
    const double s2 = __shfl_sync(0xffffffffu, st, gl + 2), s3 = __shfl_sync(0xffffffffu, st, gl + 3);
    if (act) {
      const double rd = rcp(s0);
      const double u = s1 * rd, v = s2 * rd;
      const double pr = fma(-0.5, fma(s2, v, s1 * u), s3);  // p / (gamma - 1)
      const double H = fma(gm1, pr, s3);
      const double x = q == 3 ? H : st;
      if (to_box && lead && q == 0) {
        const unsigned a = rbox + 8u * QS * (unsigned)(i - 1), m = rmbar + 8u * (unsigned)(i - 1);
        qsend2(a, s0, s1, m);
        qsend2(a + 16u, s2, H, m);
        qsend2(a + 32u, u, v, m);
        qsend2(a + 48u, pr, 0.0, m);
#pragma unroll
        for (int t = 0; t < NT; t++) qsend2(a + 64u + 16u * t, stt[t], dnt[t], m);
      }
      double *o = slot + ((size_t)buf * R + rl) * QS;
      if (lead) o[q] = x;
      if (lead && q == 0) *reinterpret_cast<double2 *>(o + 4) = make_double2(u, v);
      if (lead && q == 1) o[6] = pr;
#pragma unroll
      for (int t = 0; t < NT; t++) {
        if (lead && q == 2 + t) *reinterpret_cast<double2 *>(o + 8 + 2 * t) = make_double2(stt[t], dnt[t]);
        wt[t] = stt[t];
        wd[t] = dnt[t];
      }
      wx = x; wu = u; wv = v; wp = pr;
      if (lead) {
        if (FWD) {
          recBw[(size_t)(i - 1) * RC::N + RC::A + q] = update ? st : dn;
#pragma unroll
          for (int t = 0; t < NT; t++)
            if (q == 0) recBw[(size_t)(i - 1) * RC::N + RC::A + 4 + t] = dnt[t];
        } else {
          // an updating sweep writes U only (DU is read nowhere but inside
          // du_LU_SGS_2D and the update that follows it)
          const long long id = bd.off + (long long)(j + 2) * bd.P + (i + 2);
          if (update) L.U[q * F + id] = st;
          else L.du[q * F + id] = dn;
#pragma unroll
          for (int t = 0; t < NT; t++)
            if (q == 0) {
              if (update) L.U[(4 + t) * F + id] = stt[t];
              else L.du[(4 + t) * F + id] = dnt[t];
            }
        }
      }
    }
    __syncthreads();
  };
  const int np = phi - plo + 1;  // planes of the pass; positions past np - 1 hold no cell
  for (int t = 0; t < np; t += 4) {
    plane(FWD ? plo + t : phi - t, r0, r3);
    plane(FWD ? plo + t + 1 : phi - t - 1, r1, r0);
    plane(FWD ? plo + t + 2 : phi - t - 2, r2, r1);
    plane(FWD ? plo + t + 3 : phi - t - 3, r3, r2);
  }
  if (gave_up) set_status(L.status + 4 * bd.cas, 4, B.bk, gave_up, j);
}

template <bool update, int LPR, int NV = 4>
__global__ void __launch_bounds__(4 * QROWS, 1) k_lusgs_sweep_quad(Lvl L, int R, int CS) {
  // [2][R][QS] slots | inbox F [ni][QS] | inbox B | mbarriers F [ni] | B
  extern __shared__ __align__(16) double sh[];
  constexpr int QS = qslot<NV>();
  QBand B;
  B.rank = CS > 1 ? cluster_rank() : 0u;
  B.bk = blockIdx.x / CS;
  const BlkDev bd = L.blk[B.bk];  // by value: no re-reads after global stores
  B.R = R; B.CS = CS;
  B.rows = bd.ny - 1;
  B.ni = bd.nx - 1;
  B.rl = threadIdx.x / LPR;
  B.q = threadIdx.x & 3;
  B.j = (int)B.rank * R + B.rl + 1;
  B.row_ok = B.rl < R && B.j <= B.rows;
  const int ni = B.ni;
  const double gm1 = L.cs[bd.cas].gamma - 1.0;
  double *slot = sh;
  double *inF = sh + (size_t)2 * R * QS, *inB = inF + (size_t)ni * QS;
  unsigned long long *mbF = reinterpret_cast<unsigned long long *>(inB + (size_t)ni * QS), *mbB = mbF + ni;
  unsigned rboxF = 0, rmbF = 0, rboxB = 0, rmbB = 0;
  if (CS > 1) {
    for (int t = threadIdx.x; t < 2 * ni; t += blockDim.x) qarm(mbF + t, 8u * QS);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    if ((int)B.rank + 1 < CS) { rboxF = remote_smem(inF, B.rank + 1); rmbF = remote_smem(mbF, B.rank + 1); }
    if (B.rank > 0) { rboxB = remote_smem(inB, B.rank - 1); rmbB = remote_smem(mbB, B.rank - 1); }
    cluster_barrier();  // every inbox armed before any CTA writes into one
  }
  const int jr = B.row_ok ? B.j : 1;  // record pointers of idle rows stay in the array
  const double *recF = L.rec + ((size_t)bd.cell0 + (size_t)(jr - 1) * ni) * Rec<NV>::N;
  const double *recB = recF + (size_t)L.ncell * Rec<NV>::N;
  double *recBw = L.rec + ((size_t)L.ncell + bd.cell0 + (size_t)(jr - 1) * ni) * Rec<NV>::N;
  qpass<update, true, LPR, NV>(L, bd, B, slot, inF, mbF, rboxF, rmbF, recF, recBw, gm1);
  qpass<update, false, LPR, NV>(L, bd, B, slot, inB, mbB, rboxB, rmbB, recB, recBw, gm1);
  if (CS > 1) cluster_barrier();  // no CTA leaves while a neighbour may still write into it
}

// the four- and eight-lane kernel serves NV = 4 levels (and NV = 5 with eight
// lanes) whose blocks have at most 16 bands of rows and QCOLS cells per row, when every CTA of the launch
// gets an SM of its own (with fewer SMs, one lane per row needs fewer FP64
// instructions) and the device can hold one of its clusters
// rmax: most rows per CTA (4..32); lanes: lanes per row (4 or 8; 0: eight up
// to 16 rows, four above).  Clusters of more than 8 CTAs are non-portable
// sizes, asked for explicitly.
int quad_ctas(int max_rows, int rmax) {
  rmax = std::max(4, std::min(rmax, QROWS));
  return (max_rows + rmax - 1) / rmax;
}
static int quad_lanes(int rmax, int lanes) { return lanes == 4 || lanes == 8 ? lanes : (rmax <= 16 ? 8 : 4); }
static void (*quad_kernel(int lpr, int update, int nv))(Lvl, int, int) {
  if (nv == 5) return update ? k_lusgs_sweep_quad<true, 8, 5> : k_lusgs_sweep_quad<false, 8, 5>;
  if (nv == 6) return update ? k_lusgs_sweep_quad<true, 8, 6> : k_lusgs_sweep_quad<false, 8, 6>;
  return lpr == 8 ? (update ? k_lusgs_sweep_quad<true, 8> : k_lusgs_sweep_quad<false, 8>)
                  : (update ? k_lusgs_sweep_quad<true, 4> : k_lusgs_sweep_quad<false, 4>);
}
struct QuadShape {
  int CS, R, lpr, th, nv;
  size_t smem;
};
static QuadShape quad_shape(int max_rows, int max_cols, int rmax, int lanes, int nv) {
  QuadShape q;
  q.CS = quad_ctas(max_rows, rmax);
  q.R = (max_rows + q.CS - 1) / q.CS;
  q.lpr = nv > 4 ? 8 : quad_lanes(rmax, lanes);
  q.nv = nv;
  q.th = (q.lpr * q.R + 31) / 32 * 32;
  const size_t qs = 8 + 2 * (nv - 4);  // qslot<NV>()
  q.smem = (size_t)2 * q.R * qs * sizeof(double) + (q.CS > 1 ? (size_t)max_cols * 2 * (qs * sizeof(double) + 8) : 0);
  return q;
}
// the kernel's attributes for a launch of this shape (dynamic shared memory
// beyond 48 KiB, cluster sizes beyond 8)
static void quad_attributes(const QuadShape &q) {
  for (int update = 0; update < 2; update++) {
    auto kern = quad_kernel(q.lpr, update, q.nv);
    if (q.smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)q.smem);
    if (q.CS > 8) cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  }
}
bool quad_fits(const Lvl &L, int max_rows, int max_cols, int rmax, int lanes) {
  static int nsm = 0;
  if (!nsm) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  }
  const QuadShape q = quad_shape(max_rows, max_cols, rmax, lanes, L.nvar);
  // NV = 5, 6 ride on eight lanes per row, so at most 16 rows per band
  const bool nv_ok = L.nvar == 4 || (L.nvar <= 6 && std::max(4, std::min(rmax, QROWS)) <= 16 && lanes != 4);
  if (!(nv_ok && max_rows >= 1 && q.CS <= 16 && max_cols <= QCOLS && L.nblk * q.CS <= nsm)) return false;
  if (q.CS <= 8) return true;
  // a non-portable cluster size: launchable only if the device can place one
  quad_attributes(q);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(L.nblk * q.CS);
  cfg.blockDim = dim3(q.th);
  cfg.dynamicSmemBytes = q.smem;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = q.CS;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int nclusters = 0;
  const bool ok = cudaOccupancyMaxActiveClusters(&nclusters, quad_kernel(q.lpr, 1, q.nv), &cfg) == cudaSuccess &&
                  nclusters >= 1;
  cudaGetLastError();  // a refused query leaves no error behind
  return ok;
}

// eight lanes per row: 15 FP64 operations per cell and lane; four: 18
void launch_quad(const Lvl &L, int update, int max_rows, int max_cols, int rmax, int lanes, cudaStream_t s) {
  const QuadShape q = quad_shape(max_rows, max_cols, rmax, lanes, L.nvar);
  quad_attributes(q);
  auto kern = quad_kernel(q.lpr, update, q.nv);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(L.nblk * q.CS);
  cfg.blockDim = dim3(q.th);
  cfg.dynamicSmemBytes = q.smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = q.CS;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, kern, L, q.R, q.CS);
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
void sweep_nv(const Lvl &L, double alfa1, int mode, int max_rows, int max_cols, int cs, int rpw, int lanes,
              cudaStream_t s) {
  if (!(mode & LUSGS_SWEEP_ONLY)) k_lusgs_prep<NV><<<L.nctiles, TILE, 0, s>>>(L, alfa1, mode & LUSGS_FORCE);
  if (mode & LUSGS_PREP_ONLY) return;
  const int update = mode & LUSGS_UPDATE;
  if (cs == 0) {
    // the requested band height and lanes, else four-lane bands of 24 or 32 rows
    for (int r : {rpw, 24, 32}) {
      const int ln = r == rpw ? lanes : 0;
      if (quad_fits(L, max_rows, max_cols, r, ln)) {
        launch_quad(L, update, max_rows, max_cols, r, ln, s);
        return;
      }
    }
    cs = 1;  // one CTA per block, full warps
    rpw = 32;
  }
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

void launch_lusgs_fast(const Lvl &L, double alfa1, int mode, int max_rows, int max_cols, int cs, int rpw, int lanes,
                       cudaStream_t s) {
  if (L.nvar == 4) sweep_nv<4>(L, alfa1, mode, max_rows, max_cols, cs, rpw, lanes, s);
  else if (L.nvar == 5) sweep_nv<5>(L, alfa1, mode, max_rows, max_cols, cs, rpw, lanes, s);
  else sweep_nv<6>(L, alfa1, mode, max_rows, max_cols, cs, rpw, lanes, s);
}

}  // namespace ec2d
