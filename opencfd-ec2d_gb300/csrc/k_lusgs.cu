// k_lusgs.cu -- LU-SGS implicit operator (du_LU_SGS_2D, sub_LU_SGS.f90:4-108)
// and the cell updates of the time-marching and multigrid routines.
//
// The symmetric Gauss-Seidel sweeps keep the reference's dependency order
// exactly: the forward sweep visits the hyperplanes p = i+j = 2..nx+ny-2 and
// every cell of a hyperplane only needs dU of its (i-1,j) and (i,j-1)
// neighbours, which lie on plane p-1; the backward sweep mirrors this.  One
// CTA owns one block; thread t owns rows j = t+1, t+1+blockDim, ... and at
// plane p updates cell (p-j, j).  A CTA barrier separates planes, so every
// cell sees exactly the neighbour values the sequential sweep would see.
// Blocks (and cases of a batch) are independent, as in the reference, whose
// sweeps treat dU outside the block as zero.
#include "ec2d_dev.cuh"
#include "ec2d_internal.h"

namespace ec2d {

// flux difference dF = F_n(U+dU) - F_n(U), comput_DFn (sub_LU_SGS.f90:117-138)
__device__ __forceinline__ void dfn(int nv, double *DF, const double *U, const double *DU, double n1, double n2,
                                    double gm1) {
  double U2[6];
  for (int m = 0; m < nv; m++) U2[m] = U[m] + DU[m];
  double r1 = 1.0 / U[0], r2 = 1.0 / U2[0];
  double un1 = (U[1] * n1 + U[2] * n2) * r1;
  double p1 = gm1 * (U[3] - 0.5 * (U[1] * U[1] + U[2] * U[2]) * r1);
  double un2 = (U2[1] * n1 + U2[2] * n2) * r2;
  double p2 = gm1 * (U2[3] - 0.5 * (U2[1] * U2[1] + U2[2] * U2[2]) * r2);
  DF[0] = U2[0] * un2 - U[0] * un1;
  DF[1] = (U2[1] * un2 + p2 * n1) - (U[1] * un1 + p1 * n1);
  DF[2] = (U2[2] * un2 + p2 * n2) - (U[2] * un1 + p1 * n2);
  DF[3] = (U2[3] + p2) * un2 - (U[3] + p1) * un1;
  for (int m = 4; m < nv; m++) DF[m] = U2[m] * un2 - U[m] * un1;
}

__global__ void __launch_bounds__(128) k_lusgs(Lvl L, double alfa1) {
  const BlkDev &b = L.blk[blockIdx.x];
  const CaseDev &c = L.cs[b.cas];
  const long long F = L.F, P = b.P;
  const int nx = b.nx, ny = b.ny, nv = L.nvar, visc = L.visc;
  const double gm1 = c.gamma - 1.0, w_LU = 1.0;
  const double *geo = L.geo, *lc = L.lc;
  for (int pass = 0; pass < 2; pass++) {
    const bool fwd = (pass == 0);
    for (int pp = 2; pp <= nx + ny - 2; pp++) {
      const int plane = fwd ? pp : nx + ny - pp;
      for (int j = threadIdx.x + 1; j <= ny - 1; j += blockDim.x) {
        int i = plane - j;
        if (i < 1 || i > nx - 1) continue;
        long long id = fidx(b, i, j);
        double vol = geo[G_VOL * F + id];
        double base = vol / lc[L_DT * F + id] + w_LU * (lc[L_CI * F + id] + lc[L_CJ * F + id]) + vol * alfa1;
        double Lv = lc[L_VI * F + id] + lc[L_VJ * F + id];
        if (visc) base += 2.0 * Lv;
        double acc[6] = {0, 0, 0, 0, 0, 0};
        double U0[6], D0[6], DF[6];
        // i-neighbour
        bool hi = fwd ? (i != 1) : (i != nx - 1);
        if (hi) {
          long long nb = fwd ? id - 1 : id + 1;
          for (int m = 0; m < nv; m++) { U0[m] = L.U[m * F + nb]; D0[m] = L.du[m * F + nb]; }
          dfn(nv, DF, U0, D0, geo[G_NI1 * F + id], geo[G_NI2 * F + id], gm1);
          double s = geo[G_SI * F + (fwd ? id : nb)];
          double lcn = lc[L_CI * F + nb], lvn = lc[L_VI * F + nb];
          for (int m = 0; m < nv; m++) {
            double t = fwd ? 0.5 * (DF[m] * s + w_LU * lcn * D0[m]) : -0.5 * (DF[m] * s - w_LU * lcn * D0[m]);
            if (visc) t += lvn * D0[m];
            acc[m] = t;
          }
        }
        // j-neighbour
        bool hj = fwd ? (j != 1) : (j != ny - 1);
        double accj[6] = {0, 0, 0, 0, 0, 0};
        if (hj) {
          long long nb = fwd ? id - P : id + P;
          for (int m = 0; m < nv; m++) { U0[m] = L.U[m * F + nb]; D0[m] = L.du[m * F + nb]; }
          dfn(nv, DF, U0, D0, geo[G_NJ1 * F + id], geo[G_NJ2 * F + id], gm1);
          double s = geo[G_SJ * F + (fwd ? id : nb)];
          double lcn = lc[L_CJ * F + nb], lvn = lc[L_VJ * F + nb];
          for (int m = 0; m < nv; m++) {
            double t = fwd ? 0.5 * (DF[m] * s + w_LU * lcn * D0[m]) : -0.5 * (DF[m] * s - w_LU * lcn * D0[m]);
            if (visc) t += lvn * D0[m];
            accj[m] = t;
          }
        }
        double ia = 1.0 / base;
        double ia5 = (nv == 5) ? 1.0 / (base + Lv) : ia;
        for (int m = 0; m < nv; m++) {
          double inv = (m == 4) ? ia5 : ia;
          if (fwd) L.du[m * F + id] = (L.res[m * F + id] + acc[m] + accj[m]) * inv;
          else L.du[m * F + id] = L.du[m * F + id] + (acc[m] + accj[m]) * inv;
        }
      }
      __syncthreads();
    }
  }
}

// item loop helper over the interior cells of all blocks (tile list)
__device__ __forceinline__ bool tile_cell(const Lvl &L, int &bk, int &i, int &j, int lo, int hi_off) {
  int2 t = L.tiles[blockIdx.x];
  bk = t.x;
  const BlkDev &b = L.blk[bk];
  int W = b.nx + 3, H = b.ny + 3;
  int lin = t.y + threadIdx.x;
  if (lin >= W * H) return false;
  i = lin % W - 1;
  j = lin / W - 1;
  return i >= lo && i <= b.nx - hi_off && j >= lo && j <= b.ny - hi_off;
}

// U += dU (sub_NS_singlegrid.f90:203-211)
__global__ void k_add_du(Lvl L) {
  int bk, i, j;
  if (!tile_cell(L, bk, i, j, 1, 1)) return;
  long long id = fidx(L.blk[bk], i, j);
  for (int m = 0; m < L.nvar; m++) L.U[m * L.F + id] += L.du[m * L.F + id];
}

// explicit Euler update (sub_NS_singlegrid.f90:85-92); forcing added when `force`
__global__ void k_euler(Lvl L, int force) {
  int bk, i, j;
  if (!tile_cell(L, bk, i, j, 1, 1)) return;
  const long long F = L.F;
  long long id = fidx(L.blk[bk], i, j);
  double vol = L.geo[G_VOL * F + id], dt = L.lc[L_DT * F + id];
  for (int m = 0; m < L.nvar; m++) {
    double r = L.res[m * F + id];
    if (force && m < 4) { r = r + L.qf[m * F + id]; L.res[m * F + id] = r; }
    double du = r / vol;
    L.U[m * F + id] = L.U[m * F + id] + dt * du;
  }
}

// one RK3 stage (sub_NS_singlegrid.f90:154-163)
__global__ void k_rk3(Lvl L, int stage, int force) {
  int bk, i, j;
  if (!tile_cell(L, bk, i, j, 1, 1)) return;
  const double Ra[3] = {1.0, 3.0 / 4.0, 1.0 / 3.0}, Rb[3] = {1.0, 1.0 / 4.0, 2.0 / 3.0}, Rg[3] = {0.0, 1.0 / 4.0, 2.0 / 3.0};
  const long long F = L.F;
  long long id = fidx(L.blk[bk], i, j);
  double vol = L.geo[G_VOL * F + id], dt = L.lc[L_DT * F + id];
  for (int m = 0; m < L.nvar; m++) {
    double r = L.res[m * F + id];
    if (force && m < 4) { r = r + L.qf[m * F + id]; L.res[m * F + id] = r; }
    double du = r / vol;
    L.U[m * F + id] = Ra[stage] * L.un[m * F + id] + Rg[stage] * L.U[m * F + id] + dt * Rb[stage] * du;
  }
}

// Res += QF (Add_force_function, sub_NS_multigrid.f90:177-195)
__global__ void k_add_force(Lvl L) {
  int bk, i, j;
  if (!tile_cell(L, bk, i, j, 1, 1)) return;
  long long id = fidx(L.blk[bk], i, j);
  for (int m = 0; m < 4; m++) L.res[m * L.F + id] = L.res[m * L.F + id] + L.qf[m * L.F + id];
}
// QF -= Res (comput_force_function, sub_NS_multigrid.f90:156-173)
__global__ void k_force_fn(Lvl L) {
  int bk, i, j;
  if (!tile_cell(L, bk, i, j, 1, 1)) return;
  long long id = fidx(L.blk[bk], i, j);
  for (int m = 0; m < 4; m++) L.qf[m * L.F + id] = L.qf[m * L.F + id] - L.res[m * L.F + id];
}
// Un = U over 0..nx, 0..ny (Set_Un / RK3 copy, nvar variables)
__global__ void k_set_un(Lvl L, int nv) {
  int bk, i, j;
  if (!tile_cell(L, bk, i, j, 0, 0)) return;
  long long id = fidx(L.blk[bk], i, j);
  for (int m = 0; m < nv; m++) L.un[m * L.F + id] = L.U[m * L.F + id];
}
// restriction fine -> coarse (interpolation2h, sub_NS_multigrid.f90:349-398):
// flag 1 volume-weighted U, flag 2 residual sum into QF, 3 both; with 4 the
// coarse residual already evaluated on the restricted U is subtracted from
// the sum (QF = sum Res_h - Res_2h, comput_force_function,
// sub_NS_multigrid.f90:156-173: the sum is rounded first, as there).  With
// 8 (an extension for turbulent cases) the coarse eddy viscosity over
// 0..nx, 0..ny is the mean of its children's within the finer level's
// 0..nx, 0..ny, summed j-major as the oracle does.  Runs over the coarse
// level's tiles.  Every operand is loaded before the first store: the
// stores may alias the loads as far as the compiler knows, so loads
// interleaved with stores would be issued one variable at a time.
__global__ void k_restrict(Lvl Lf, Lvl Lc, int flag) {
  int bk, i, j;
  if (!tile_cell(Lc, bk, i, j, 0, 0)) return;
  const BlkDev &bc = Lc.blk[bk], &bf = Lf.blk[bk];
  const long long ic = fidx(bc, i, j);
  if (flag & 8) {
    double sum = 0.0;
    int n = 0;
    for (int jj = 2 * j - 1; jj <= 2 * j; jj++)
      for (int ii = 2 * i - 1; ii <= 2 * i; ii++)
        if (ii >= 0 && ii <= bf.nx && jj >= 0 && jj <= bf.ny) {
          sum += Lf.amut[fidx(bf, ii, jj)];
          n++;
        }
    Lc.amut[ic] = sum / (double)n;
  }
  if (i < 1 || i > bc.nx - 1 || j < 1 || j > bc.ny - 1) return;
  const long long f11 = fidx(bf, 2 * i - 1, 2 * j - 1), f12 = fidx(bf, 2 * i - 1, 2 * j);
  const long long f21 = fidx(bf, 2 * i, 2 * j - 1), f22 = fidx(bf, 2 * i, 2 * j);
  const long long FF = Lf.F, FC = Lc.F;
  if (flag & 1) {
    const double *vf = Lf.geo + G_VOL * FF;
    const double w11 = vf[f11], w12 = vf[f12], w21 = vf[f21], w22 = vf[f22];
    // one reciprocal of the coarse volume for the four variables (the
    // reference divides each sum; an IEEE divide costs about a dozen FP64
    // instructions, which bound this kernel on this part)
    const double rvc = 1.0 / Lc.geo[G_VOL * FC + ic];
    double u[4][4];
#pragma unroll
    for (int m = 0; m < 4; m++) {
      const double *q = Lf.U + m * FF;
      u[m][0] = q[f11]; u[m][1] = q[f12]; u[m][2] = q[f21]; u[m][3] = q[f22];
    }
#pragma unroll
    for (int m = 0; m < 4; m++)
      Lc.U[m * FC + ic] = (u[m][0] * w11 + u[m][1] * w12 + u[m][2] * w21 + u[m][3] * w22) * rvc;
  }
  if (flag & 2) {
    double r[4][4], rc[4];
#pragma unroll
    for (int m = 0; m < 4; m++) {
      const double *q = Lf.res + m * FF;
      r[m][0] = q[f11]; r[m][1] = q[f12]; r[m][2] = q[f21]; r[m][3] = q[f22];
      rc[m] = (flag & 4) ? Lc.res[m * FC + ic] : 0.0;
    }
#pragma unroll
    for (int m = 0; m < 4; m++) {
      const double sum = r[m][0] + r[m][1] + r[m][2] + r[m][3];
      Lc.qf[m * FC + ic] = (flag & 4) ? sum - rc[m] : sum;
    }
  }
}

// prolongation coarse -> fine (prolong_U, sub_NS_multigrid.f90:271-343) over
// fine cells 0..nx2, 0..ny2, weights 9/16, 3/16, 3/16, 1/16 on the nearest,
// the two side and the diagonal coarse cells.  flag 1 interpolates U, flag 2
// deltU, flag 3 deltU formed on the fly from the coarse U - Un (comput_delt_U,
// sub_NS_multigrid.f90:199-216, the same subtraction) and then U += deltU on
// the fine interior (comput_new_U, sub_NS_multigrid.f90:240-260), one pass.
// One thread per 2 x 2 fine cells (2k, 2k+1) x (2l, 2l+1), which all take
// their values from the coarse cells k, k+1 x l, l+1: the coarse values (and
// their U - Un) are loaded and formed once for the four.  Runs over the
// coarse level's tiles, k = 0..nxc-1, l = 0..nyc-1 (the fine range 0..nx2 is
// 2 nxc cells wide).
__global__ void k_prolong(Lvl Lc, Lvl Lf, int flag) {
  int bk, k, l;
  if (!tile_cell(Lc, bk, k, l, 0, 1)) return;
  const BlkDev &bc = Lc.blk[bk], &bf = Lf.blk[bk];
  const double a1 = 9.0 / 16.0, a2 = 3.0 / 16.0, a3 = 1.0 / 16.0;
  const long long c00 = fidx(bc, k, l), c10 = fidx(bc, k + 1, l);
  const long long c01 = fidx(bc, k, l + 1), c11 = fidx(bc, k + 1, l + 1);
  const int i0 = 2 * k, j0 = 2 * l;
  const bool has_i1 = i0 + 1 <= bf.nx, has_j1 = j0 + 1 <= bf.ny;
  const long long f00 = fidx(bf, i0, j0), f10 = fidx(bf, i0 + 1, j0);
  const long long f01 = fidx(bf, i0, j0 + 1), f11 = fidx(bf, i0 + 1, j0 + 1);
  // fine interior rows and columns, where flag 3 adds the increment to U
  const bool ai0 = flag == 3 && i0 >= 1 && i0 <= bf.nx - 1, ai1 = flag == 3 && has_i1 && i0 + 1 <= bf.nx - 1;
  const bool aj0 = j0 >= 1 && j0 <= bf.ny - 1, aj1 = has_j1 && j0 + 1 <= bf.ny - 1;
  double s[4][4];
#pragma unroll
  for (int m = 0; m < 4; m++) {
    if (flag == 3) {
      const double *u = Lc.U + m * Lc.F, *un = Lc.un + m * Lc.F;
      s[m][0] = u[c00] - un[c00]; s[m][1] = u[c10] - un[c10];
      s[m][2] = u[c01] - un[c01]; s[m][3] = u[c11] - un[c11];
    } else {
      const double *q = ((flag == 1) ? Lc.U : Lc.deltu) + m * Lc.F;
      s[m][0] = q[c00]; s[m][1] = q[c10]; s[m][2] = q[c01]; s[m][3] = q[c11];
    }
  }
  double uf[4][4];
  if (flag == 3) {
#pragma unroll
    for (int m = 0; m < 4; m++) {
      const double *u = Lf.U + m * Lf.F;
      uf[m][0] = (ai0 && aj0) ? u[f00] : 0.0; uf[m][1] = (ai1 && aj0) ? u[f10] : 0.0;
      uf[m][2] = (ai0 && aj1) ? u[f01] : 0.0; uf[m][3] = (ai1 && aj1) ? u[f11] : 0.0;
    }
  }
  double *dst = (flag == 1) ? Lf.U : Lf.deltu;
#pragma unroll
  for (int m = 0; m < 4; m++) {
    const double s00 = s[m][0], s10 = s[m][1], s01 = s[m][2], s11 = s[m][3];
    // the side pairs of the diagonal cells and of the anti-diagonal ones are
    // the same sums (an IEEE sum does not depend on the operand order)
    const double side_d = s10 + s01, side_a = s00 + s11;
    const double v00 = a1 * s00 + a2 * side_d + a3 * s11;  // fine (2k, 2l)
    const double v10 = a1 * s10 + a2 * side_a + a3 * s01;  // fine (2k+1, 2l)
    const double v01 = a1 * s01 + a2 * side_a + a3 * s10;  // fine (2k, 2l+1)
    const double v11 = a1 * s11 + a2 * side_d + a3 * s00;  // fine (2k+1, 2l+1)
    double *d = dst + m * Lf.F, *u = Lf.U + m * Lf.F;
    d[f00] = v00;
    if (has_i1) d[f10] = v10;
    if (has_j1) d[f01] = v01;
    if (has_i1 && has_j1) d[f11] = v11;
    if (flag == 3) {
      if (ai0 && aj0) u[f00] = uf[m][0] + v00;
      if (ai1 && aj0) u[f10] = uf[m][1] + v10;
      if (ai0 && aj1) u[f01] = uf[m][2] + v01;
      if (ai1 && aj1) u[f11] = uf[m][3] + v11;
    }
  }
}

// freestream in the interior (init_flow_zero, sub_init.f90:461-472) and the
// turbulence start values on the fine mesh (sub_init.f90:433-457)
__global__ void k_freestream(Lvl L, int flow, int turb) {
  int bk, i, j;
  if (!tile_cell(L, bk, i, j, 1, 1)) return;
  const BlkDev &b = L.blk[bk];
  const CaseDev &c = L.cs[b.cas];
  long long id = fidx(b, i, j);
  const long long F = L.F;
  if (flow) {
    double d0 = 1.0, u0 = c.cosA, v0 = c.sinA, p0 = c.p00;
    L.U[id] = d0; L.U[F + id] = d0 * u0; L.U[2 * F + id] = d0 * v0;
    L.U[3 * F + id] = p0 / (c.gamma - 1.0) + 0.5 * d0 * (u0 * u0 + v0 * v0);
  }
  if (turb) {
    if (L.nvar == 5) L.U[4 * F + id] = c.vt_inf / c.Re;
    if (L.nvar == 6) { L.U[4 * F + id] = 10.0 * c.Kt_inf; L.U[5 * F + id] = c.Wt_inf; }
  }
}

constexpr int TILE = EC2D_TILE;
void launch_lusgs(const Lvl &L, double alfa1, cudaStream_t s) { k_lusgs<<<L.nblk, 128, 0, s>>>(L, alfa1); }
void launch_add_du(const Lvl &L, cudaStream_t s) { k_add_du<<<L.ntiles, TILE, 0, s>>>(L); }
void launch_euler(const Lvl &L, int force, cudaStream_t s) { k_euler<<<L.ntiles, TILE, 0, s>>>(L, force); }
void launch_rk3(const Lvl &L, int stage, int force, cudaStream_t s) { k_rk3<<<L.ntiles, TILE, 0, s>>>(L, stage, force); }
void launch_add_force(const Lvl &L, cudaStream_t s) { k_add_force<<<L.ntiles, TILE, 0, s>>>(L); }
void launch_force_fn(const Lvl &L, cudaStream_t s) { k_force_fn<<<L.ntiles, TILE, 0, s>>>(L); }
void launch_set_un(const Lvl &L, int nv, cudaStream_t s) { k_set_un<<<L.ntiles, TILE, 0, s>>>(L, nv); }
void launch_restrict(const Lvl &Lf, const Lvl &Lc, int flag, cudaStream_t s) {
  k_restrict<<<Lc.ntiles, TILE, 0, s>>>(Lf, Lc, flag);
}
void launch_prolong(const Lvl &Lc, const Lvl &Lf, int flag, cudaStream_t s) {
  k_prolong<<<Lc.ntiles, TILE, 0, s>>>(Lc, Lf, flag);
}
void launch_freestream(const Lvl &L, int flow, int turb, cudaStream_t s) {
  k_freestream<<<L.ntiles, TILE, 0, s>>>(L, flow, turb);
}

}  // namespace ec2d
