// k_turb.cu -- turbulence-model residual rows (Spalart-Allmaras,
// sub_turbulence_SA.f90; k-omega SST, sub_turbulence_SST.f90), the ghost
// eddy viscosity at walls (Amut_boundary), the finite-difference WENO5 patch
// (sub_Finite_Difference.f90) and the dual-time source term.
#include "ec2d_dev.cuh"
#include "ec2d_internal.h"

namespace ec2d {

constexpr int TILE = EC2D_TILE;

__device__ __forceinline__ bool tile_xy(const Lvl &L, int &bk, int &i, int &j) {
  int2 t = L.tiles[blockIdx.x];
  bk = t.x;
  const BlkDev &b = L.blk[bk];
  int W = b.nx + 3, H = b.ny + 3;
  int lin = t.y + threadIdx.x;
  if (lin >= W * H) return false;
  i = lin % W - 1;
  j = lin / W - 1;
  return true;
}

// ---- Spalart-Allmaras (sub_turbulence_SA.f90:4-175) -------------------------
namespace sa {
constexpr double sigma = 2.0 / 3.0, Cv1 = 7.1, Cb1 = 0.1355, Cb2 = 0.622, kap = 0.41;
constexpr double Cw2 = 0.3, Cw3 = 2.0, Ct3 = 1.3, Ct4 = 0.5;
}

// eddy viscosity over 0..nx, 0..ny (sub_turbulence_SA.f90:25-32)
__global__ void k_sa_mut(Lvl L) {
  int bk, i, j;
  if (!tile_xy(L, bk, i, j)) return;
  const BlkDev &b = L.blk[bk];
  if (i < 0 || i > b.nx || j < 0 || j > b.ny) return;
  const long long F = L.F;
  long long id = fidx(b, i, j);
  double vt = L.U[4 * F + id], d = L.q[Q_D * F + id];
  double X = d * vt * rcp(L.amu[id]);
  double X3 = X * X * X;
  double fv1 = X3 * rcp(X3 + sa::Cv1 * sa::Cv1 * sa::Cv1);
  L.amut[id] = fv1 * d * vt;
}

// Amut_boundary (sub_turbulence_SA.f90:180-220): mirror the eddy viscosity
// into the first ghost layer of wall subfaces; one CTA per block
__global__ void k_amut_boundary(Lvl L) {
  const BlkDev &b = L.blk[blockIdx.x];
  for (int ks = 0; ks < b.nsub; ks++) {
    const SubDev s = L.sub[b.sub0 + ks];
    if (s.neighb != BC_Wall) continue;
    if (s.face == 1 || s.face == 3) {
      for (int j = s.jst + threadIdx.x; j <= s.jend - 1; j += blockDim.x) {
        if (s.face == 1) L.amut[fidx(b, 0, j)] = -L.amut[fidx(b, 1, j)];
        else L.amut[fidx(b, b.nx, j)] = -L.amut[fidx(b, b.nx - 1, j)];
      }
    } else {
      for (int i = s.ist + threadIdx.x; i <= s.iend - 1; i += blockDim.x) {
        if (s.face == 2) L.amut[fidx(b, i, 0)] = -L.amut[fidx(b, i, 1)];
        else L.amut[fidx(b, i, b.ny)] = -L.amut[fidx(b, i, b.ny - 1)];
      }
    }
    __syncthreads();
  }
}

// nu~ face fluxes: first-order upwind convection and the (1+cb2)/sigma
// diffusion, i faces (sub_turbulence_SA.f90:43-73) and j faces (:87-114);
// planes 4/5 of fi, fj hold Fluxv and fluxv2
__global__ void k_sa_faces(Lvl L) {
  int bk, i, j;
  if (!tile_xy(L, bk, i, j)) return;
  const BlkDev &b = L.blk[bk];
  const long long F = L.F, P = b.P;
  long long id = fidx(b, i, j);
  const double *vt = L.U + 4 * F, *d = L.q + Q_D * F, *uu = L.q + Q_U * F, *vv = L.q + Q_V * F;
  const double *amu = L.amu;
  const double c0 = 0.5 * (1.0 + sa::Cb2) / sa::sigma;
  if (i >= 1 && i <= b.nx && j >= 1 && j <= b.ny - 1) {
    long long w = id - 1, nN = id + P, nS = id - P;
    double s0 = L.geo[G_SI * F + id], n1 = L.geo[G_NI1 * F + id], n2 = L.geo[G_NI2 * F + id];
    double vn1 = uu[w] * n1 + vv[w] * n2, vn2 = uu[id] * n1 + vv[id] * n2;
    double vfi = -0.5 * ((vn1 + fabs(vn1)) * vt[w] + (vn2 - fabs(vn2)) * vt[id]) * s0;
    double v0 = c0 * (vt[id] + amu[id] * rcp(d[id]) + vt[w] + amu[w] * rcp(d[w]));
    // the face's inverse Jacobian, formed at set-up (k_face_metrics)
    const double *gm = L.geo + id;
    double Div = vt[id] - vt[w];
    double Djv = (vt[nN - 1] + vt[nN] - vt[nS - 1] - vt[nS]) * 0.25;
    double vtx = fma(Div, gm[G_VIA * F], -Djv * gm[G_VIB * F]), vty = fma(Djv, gm[G_VID * F], -Div * gm[G_VIC * F]);
    double g = (vtx * n1 + vty * n2) * s0;
    L.fi[4 * F + id] = vfi + v0 * g;
    L.fi[5 * F + id] = g;
  }
  if (i >= 1 && i <= b.nx - 1 && j >= 1 && j <= b.ny) {
    long long s = id - P;
    double s0 = L.geo[G_SJ * F + id], n1 = L.geo[G_NJ1 * F + id], n2 = L.geo[G_NJ2 * F + id];
    double vn1 = uu[s] * n1 + vv[s] * n2, vn2 = uu[id] * n1 + vv[id] * n2;
    double vfi = -0.5 * ((vn1 + fabs(vn1)) * vt[s] + (vn2 - fabs(vn2)) * vt[id]) * s0;
    double v0 = c0 * (vt[id] + amu[id] * rcp(d[id]) + vt[s] + amu[s] * rcp(d[s]));
    const double *gm = L.geo + id;
    double Div = (vt[s + 1] + vt[id + 1] - vt[s - 1] - vt[id - 1]) * 0.25;
    double Djv = vt[id] - vt[s];
    double vtx = fma(Div, gm[G_VJA * F], -Djv * gm[G_VJB * F]), vty = fma(Djv, gm[G_VJD * F], -Div * gm[G_VJC * F]);
    double g = (vtx * n1 + vty * n2) * s0;
    L.fj[4 * F + id] = vfi + v0 * g;
    L.fj[5 * F + id] = g;
  }
}

// Res(5): flux differences with the cb2 cross term and the production /
// destruction source (sub_turbulence_SA.f90:77-82, 118-124, 129-168)
__global__ void k_sa_res(Lvl L) {
  int bk, i, j;
  if (!tile_xy(L, bk, i, j)) return;
  const BlkDev &b = L.blk[bk];
  if (i < 1 || i > b.nx - 1 || j < 1 || j > b.ny - 1) return;
  const long long F = L.F, P = b.P;
  long long id = fidx(b, i, j);
  const double *x1 = L.geo + G_X1 * F, *y1 = L.geo + G_Y1 * F, *uu = L.q + Q_U * F, *vv = L.q + Q_V * F;
  double vt = L.U[4 * F + id], d = L.q[Q_D * F + id], amu = L.amu[id];
  const double ramu = rcp(amu);
  double v0 = (vt + amu * rcp(d)) * (sa::Cb2 / sa::sigma);
  double r = L.fi[4 * F + id + 1] - L.fi[4 * F + id] - v0 * (L.fi[5 * F + id + 1] - L.fi[5 * F + id]);
  r = r + L.fj[4 * F + id + P] - L.fj[4 * F + id] - v0 * (L.fj[5 * F + id + P] - L.fj[5 * F + id]);
  double Dix = (x1[id + 1] - x1[id - 1]) * 0.5, Diy = (y1[id + 1] - y1[id - 1]) * 0.5;
  double Djx = (x1[id + P] - x1[id - P]) * 0.5, Djy = (y1[id + P] - y1[id - P]) * 0.5;
  double Ds = 1.0 / (Dix * Djy - Djx * Diy);
  double Diu = (uu[id + 1] - uu[id - 1]) * 0.5, Div = (vv[id + 1] - vv[id - 1]) * 0.5;
  double Dju = (uu[id + P] - uu[id - P]) * 0.5, Djv = (vv[id + P] - vv[id - P]) * 0.5;
  double vx = (Div * Djy - Djv * Diy) * Ds;
  double uy = (-Diu * Djx + Dju * Dix) * Ds;
  double S = fabs(vx - uy);
  double dw = L.geo[G_DW * F + id];
  double X = d * vt * ramu;
  double X3 = X * X * X;
  double fv1 = X3 * rcp(X3 + sa::Cv1 * sa::Cv1 * sa::Cv1);
  double fv2 = 1.0 - X * rcp(1.0 + X * fv1);
  double kd = sa::kap * dw;
  const double rkd2 = rcp(kd * kd);  // 1 / (kappa d)^2
  double S1 = fmax(S + fv2 * vt * rkd2, (double)0.3f * S);  // 0.3 is a single-precision literal
  double rr = fmin(vt * rcp(S1) * rkd2, 10.0);
  double r2 = rr * rr, r6 = r2 * r2 * r2;
  double g = rr + sa::Cw2 * (r6 - rr);
  double g2 = g * g, g6 = g2 * g2 * g2;
  const double c36 = sa::Cw3 * sa::Cw3 * sa::Cw3 * sa::Cw3 * sa::Cw3 * sa::Cw3;
  // x^(1/6) as cbrt(sqrt(x)): both within an ulp, cheaper than pow
  double fw = g * cbrt(sqrt((1.0 + c36) * rcp(g6 + c36)));
  double ft2 = sa::Ct3 * exp(-sa::Ct4 * X * X);
  const double Cw1 = sa::Cb1 / (sa::kap * sa::kap) + (1.0 + sa::Cb2) / sa::sigma;
  double q = vt * rcp(dw);
  double Q = sa::Cb1 * (1.0 - ft2) * S1 * vt - (Cw1 * fw - sa::Cb1 * ft2 / (sa::kap * sa::kap)) * (q * q);
  L.res[4 * F + id] = r + Q * L.geo[G_VOL * F + id];
}

void launch_sa(const Lvl &L, cudaStream_t s) {
  k_sa_mut<<<L.ntiles, TILE, 0, s>>>(L);
  k_amut_boundary<<<L.nblk, 128, 0, s>>>(L);
  k_sa_faces<<<L.ntiles, TILE, 0, s>>>(L);
  k_sa_res<<<L.ntiles, TILE, 0, s>>>(L);
}
void launch_amut_boundary(const Lvl &L, cudaStream_t s) { k_amut_boundary<<<L.nblk, 128, 0, s>>>(L); }

// ---- k-omega SST (sub_turbulence_SST.f90:6-271) -----------------------------
namespace sst {
constexpr double sk1 = 0.85, sw1 = 0.5, beta1 = 0.075, Cw1 = 0.533;
constexpr double sk2 = 1.0, sw2 = 0.856, beta2 = 0.0828, Cw2 = 0.440;
constexpr double a1 = 0.31, betas = 0.09;
}
// scratch planes in L.tb
enum { T_AMUS = 0, T_AMUTS = 1, T_F1 = 2, T_QK = 3, T_QW = 4 };

// cell pass (sub_turbulence_SST.f90:53-121): eddy viscosity, blending f1 and
// the k/omega sources; Amu is scaled by Re for the model and scaled back
// (x*Re/Re, as the reference does at :85 and :259)
__global__ void k_sst_cell(Lvl L) {
  int bk, i, j;
  if (!tile_xy(L, bk, i, j)) return;
  const BlkDev &b = L.blk[bk];
  if (i < 1 || i > b.nx - 1 || j < 1 || j > b.ny - 1) return;
  const CaseDev &c = L.cs[b.cas];
  const long long F = L.F, P = b.P;
  const double Re = c.Re;
  long long id = fidx(b, i, j);
  const double *x1 = L.geo + G_X1 * F, *y1 = L.geo + G_Y1 * F, *uu = L.q + Q_U * F, *vv = L.q + Q_V * F;
  const double *d = L.q + Q_D * F, *U5 = L.U + 4 * F, *U6 = L.U + 5 * F;
  auto Kt = [&](long long k) { return U5[k] / d[k]; };
  auto Wt = [&](long long k) { return U6[k] / d[k]; };
  double Dix = (x1[id + 1] - x1[id - 1]) * 0.5, Diy = (y1[id + 1] - y1[id - 1]) * 0.5;
  double Djx = (x1[id + P] - x1[id - P]) * 0.5, Djy = (y1[id + P] - y1[id - P]) * 0.5;
  double Ds = 1.0 / (Dix * Djy - Djx * Diy);
  double Diu = (uu[id + 1] - uu[id - 1]) * 0.5, Div = (vv[id + 1] - vv[id - 1]) * 0.5;
  double Dik = (Kt(id + 1) - Kt(id - 1)) * 0.5, Diw = (Wt(id + 1) - Wt(id - 1)) * 0.5;
  double Dju = (uu[id + P] - uu[id - P]) * 0.5, Djv = (vv[id + P] - vv[id - P]) * 0.5;
  double Djk = (Kt(id + P) - Kt(id - P)) * 0.5, Djw = (Wt(id + P) - Wt(id - P)) * 0.5;
  double vx = (Div * Djy - Djv * Diy) * Ds;
  double kx = (Dik * Djy - Djk * Diy) * Ds, wx = (Diw * Djy - Djw * Diy) * Ds;
  double uy = (-Diu * Djx + Dju * Dix) * Ds;
  double ky = (-Dik * Djx + Djk * Dix) * Ds, wy = (-Diw * Djx + Djw * Dix) * Ds;
  double amus = L.amu[id] * Re;
  double omega = vx - uy;
  double dc = d[id], K = Kt(id), W = Wt(id), dw = L.geo[G_DW * F + id];
  const double c009 = (double)0.09f;  // single-precision literal (sub_turbulence_SST.f90:87,96)
  double t2 = 500.0 * amus / (dc * W * (dw * dw) * (Re * Re));
  double arg2 = fmax(2.0 * sqrt(fabs(K)) / (c009 * W * dw * Re), t2);
  double f2 = tanh(arg2 * arg2);
  double amuts = fmin(fmin(dc * K / W, sst::a1 * dc * K * Re / (f2 * fabs(omega))), 100000.0);
  double Kws = 2.0 * (kx * wx + ky * wy) * dc * sst::sw2 / (W + 1.0e-20);
  double CD = fmax(Kws, 1.0e-20);
  double arg3 = fmax(sqrt(fabs(K)) / (c009 * W * dw * Re), t2);
  double arg1 = fmin(arg3, 4.0 * dc * sst::sw2 * K / (CD * (dw * dw)));
  double a1s = arg1 * arg1;
  double f1 = tanh(a1s * a1s);
  double Pk = amuts * omega * omega;
  double Pk0 = fmin(Pk, 20.0 * sst::betas * K * W * (Re * Re));
  double Qk = Pk0 / Re - sst::betas * dc * W * K * Re;
  double Cw = f1 * sst::Cw1 + (1.0 - f1) * sst::Cw2;
  double beta = f1 * sst::beta1 + (1.0 - f1) * sst::beta2;
  double Qw = Cw * dc * omega * omega / Re - beta * dc * (W * W) * Re + (1.0 - f1) * Kws / Re;
  L.tb[T_AMUS * F + id] = amus;
  L.tb[T_AMUTS * F + id] = amuts;
  L.tb[T_F1 * F + id] = f1;
  L.tb[T_QK * F + id] = Qk;
  L.tb[T_QW * F + id] = Qw;
}

// k and omega face fluxes, i faces (sub_turbulence_SST.f90:129-182) and j
// faces (:198-248); planes 4/5 of fi and fj
__global__ void k_sst_faces(Lvl L) {
  int bk, i, j;
  if (!tile_xy(L, bk, i, j)) return;
  const BlkDev &b = L.blk[bk];
  const CaseDev &c = L.cs[b.cas];
  const long long F = L.F, P = b.P;
  const double Re = c.Re;
  long long id = fidx(b, i, j);
  const double *x1 = L.geo + G_X1 * F, *y1 = L.geo + G_Y1 * F, *uu = L.q + Q_U * F, *vv = L.q + Q_V * F;
  const double *d = L.q + Q_D * F, *U5 = L.U + 4 * F, *U6 = L.U + 5 * F;
  const double *amus = L.tb + T_AMUS * F, *amuts = L.tb + T_AMUTS * F;
  auto Kt = [&](long long k) { return U5[k] / d[k]; };
  auto Wt = [&](long long k) { return U6[k] / d[k]; };
  double f1 = L.tb[T_F1 * F + id];
  double sk = f1 * sst::sk1 + (1.0 - f1) * sst::sk2;
  double sw = f1 * sst::sw1 + (1.0 - f1) * sst::sw2;
  if (i >= 1 && i <= b.nx && j >= 1 && j <= b.ny - 1) {
    long long w = id - 1, nN = id + P, nS = id - P;
    double si = L.geo[G_SI * F + id], n1 = L.geo[G_NI1 * F + id], n2 = L.geo[G_NI2 * F + id];
    double un1 = uu[w] * n1 + vv[w] * n2, un2 = uu[id] * n1 + vv[id] * n2;
    double Fk = -0.5 * ((un1 + fabs(un1)) * Kt(w) + (un2 - fabs(un2)) * Kt(id)) * si;
    double Fw = -0.5 * ((un1 + fabs(un1)) * Wt(w) + (un2 - fabs(un2)) * Wt(id)) * si;
    double A1, A2;
    if (i == 1) { A1 = amus[id] + sk * amuts[id]; A2 = amus[id] + sw * amuts[id]; }
    else if (i == b.nx) { A1 = amus[w] + sk * amuts[w]; A2 = amus[w] + sw * amuts[w]; }
    else { A1 = (amus[w] + amus[id] + sk * (amuts[w] + amuts[id])) * 0.5;
           A2 = (amus[w] + amus[id] + sw * (amuts[w] + amuts[id])) * 0.5; }
    double Dix = x1[id] - x1[w], Diy = y1[id] - y1[w];
    double Djx = (x1[nN - 1] + x1[nN] - x1[nS - 1] - x1[nS]) * 0.25;
    double Djy = (y1[nN - 1] + y1[nN] - y1[nS - 1] - y1[nS]) * 0.25;
    double Ds = 1.0 / (Dix * Djy - Djx * Diy);
    double Dik = Kt(id) - Kt(w), Diw = Wt(id) - Wt(w);
    double Djk = (Kt(nN - 1) + Kt(nN) - Kt(nS - 1) - Kt(nS)) * 0.25;
    double Djw = (Wt(nN - 1) + Wt(nN) - Wt(nS - 1) - Wt(nS)) * 0.25;
    double Kx = (Dik * Djy - Djk * Diy) * Ds, Wx = (Diw * Djy - Djw * Diy) * Ds;
    double Ky = (-Dik * Djx + Djk * Dix) * Ds, Wy = (-Diw * Djx + Djw * Dix) * Ds;
    L.fi[4 * F + id] = Fk + A1 * (Kx * n1 + Ky * n2) * si / Re;
    L.fi[5 * F + id] = Fw + A2 * (Wx * n1 + Wy * n2) * si / Re;
  }
  if (i >= 1 && i <= b.nx - 1 && j >= 1 && j <= b.ny) {
    long long s = id - P;
    double sj = L.geo[G_SJ * F + id], n1 = L.geo[G_NJ1 * F + id], n2 = L.geo[G_NJ2 * F + id];
    double un1 = uu[s] * n1 + vv[s] * n2, un2 = uu[id] * n1 + vv[id] * n2;
    double Fk = -0.5 * ((un1 + fabs(un1)) * Kt(s) + (un2 - fabs(un2)) * Kt(id)) * sj;
    double Fw = -0.5 * ((un1 + fabs(un1)) * Wt(s) + (un2 - fabs(un2)) * Wt(id)) * sj;
    double A1, A2;
    if (j == 1) { A1 = amus[id] + sk * amuts[id]; A2 = amus[id] + sw * amuts[id]; }
    else if (j == b.ny) { A1 = amus[s] + sk * amuts[s]; A2 = amus[s] + sw * amuts[s]; }
    else { A1 = (amus[id] + amus[s] + sk * (amuts[id] + amuts[s])) * 0.5;
           A2 = (amus[id] + amus[s] + sw * (amuts[id] + amuts[s])) * 0.5; }
    double Dix = (x1[s + 1] + x1[id + 1] - x1[s - 1] - x1[id - 1]) * 0.25;
    double Diy = (y1[s + 1] + y1[id + 1] - y1[s - 1] - y1[id - 1]) * 0.25;
    double Djx = x1[id] - x1[s], Djy = y1[id] - y1[s];
    double Ds = 1.0 / (Dix * Djy - Djx * Diy);
    double Dik = (Kt(s + 1) + Kt(id + 1) - Kt(s - 1) - Kt(id - 1)) * 0.25;
    double Diw = (Wt(s + 1) + Wt(id + 1) - Wt(s - 1) - Wt(id - 1)) * 0.25;
    double Djk = Kt(id) - Kt(s), Djw = Wt(id) - Wt(s);
    double Kx = (Dik * Djy - Djk * Diy) * Ds, Wx = (Diw * Djy - Djw * Diy) * Ds;
    double Ky = (-Dik * Djx + Djk * Dix) * Ds, Wy = (-Diw * Djx + Djw * Dix) * Ds;
    L.fj[4 * F + id] = Fk + A1 * (Kx * n1 + Ky * n2) * sj / Re;
    L.fj[5 * F + id] = Fw + A2 * (Wx * n1 + Wy * n2) * sj / Re;
  }
}

// Res(5:6) and the rescaled viscosities (sub_turbulence_SST.f90:186-191, 254-262)
__global__ void k_sst_res(Lvl L) {
  int bk, i, j;
  if (!tile_xy(L, bk, i, j)) return;
  const BlkDev &b = L.blk[bk];
  if (i < 1 || i > b.nx - 1 || j < 1 || j > b.ny - 1) return;
  const CaseDev &c = L.cs[b.cas];
  const long long F = L.F, P = b.P;
  long long id = fidx(b, i, j);
  double vol = L.geo[G_VOL * F + id];
  double r5 = L.fi[4 * F + id + 1] - L.fi[4 * F + id];
  double r6 = L.fi[5 * F + id + 1] - L.fi[5 * F + id];
  r5 = r5 + L.fj[4 * F + id + P] - L.fj[4 * F + id] + L.tb[T_QK * F + id] * vol;
  r6 = r6 + L.fj[5 * F + id + P] - L.fj[5 * F + id] + L.tb[T_QW * F + id] * vol;
  L.res[4 * F + id] = r5;
  L.res[5 * F + id] = r6;
  L.amu[id] = L.tb[T_AMUS * F + id] / c.Re;
  L.amut[id] = L.tb[T_AMUTS * F + id] / c.Re;
}

void launch_sst(const Lvl &L, cudaStream_t s) {
  k_sst_cell<<<L.ntiles, TILE, 0, s>>>(L);
  k_sst_faces<<<L.ntiles, TILE, 0, s>>>(L);
  k_sst_res<<<L.ntiles, TILE, 0, s>>>(L);
  k_amut_boundary<<<L.nblk, 128, 0, s>>>(L);
}

// ---- finite-difference patch (sub_Finite_Difference.f90:4-275) --------------
// scratch planes in L.fdm: 0-7 i-direction split fluxes (fp 0-3, fm 4-7),
// 8-15 j-direction, 16-19 i fluxes, 20-23 j fluxes, 24-29 viscous Ev1/Ev2
enum { D_SPI = 0, D_SPJ = 8, D_FI = 16, D_FJ = 20, D_EV1 = 24, D_EV2 = 27 };

// split_Steger_Warming, sub_Finite_Difference.f90:154-202
__device__ __forceinline__ void split_sw(double d, double u, double v, double cc, double A1, double A2,
                                         double gamma, double *fp, double *fm) {
  double tmp1 = 2.0 * (gamma - 1.0), tmp3 = (3.0 - gamma) / (2.0 * (gamma - 1.0));
  double vs = A1 * u + A2 * v, ss = sqrt(A1 * A1 + A2 * A2);
  const double rss = 1.0 / ss;
  double ak1 = A1 * rss, ak2 = A2 * rss;
  double E1 = vs, E2 = vs - cc * ss, E3 = vs + cc * ss;
  double E1P = (E1 + fabs(E1)) * 0.5, E2P = (E2 + fabs(E2)) * 0.5, E3P = (E3 + fabs(E3)) * 0.5;
  double E1M = E1 - E1P, E2M = E2 - E2P, E3M = E3 - E3P;
  double tmp0 = d / (2.0 * gamma);
  double uc1 = u - cc * ak1, uc2 = u + cc * ak1, vc1 = v - cc * ak2, vc2 = v + cc * ak2;
  double vvc1 = (uc1 * uc1 + vc1 * vc1) / 2.0, vvc2 = (uc2 * uc2 + vc2 * vc2) / 2.0;
  double vv = (gamma - 1.0) * (u * u + v * v), W2 = tmp3 * cc * cc;
  fp[0] = tmp0 * (tmp1 * E1P + E2P + E3P);
  fp[1] = tmp0 * (tmp1 * E1P * u + E2P * uc1 + E3P * uc2);
  fp[2] = tmp0 * (tmp1 * E1P * v + E2P * vc1 + E3P * vc2);
  fp[3] = tmp0 * (E1P * vv + E2P * vvc1 + E3P * vvc2 + W2 * (E2P + E3P));
  fm[0] = tmp0 * (tmp1 * E1M + E2M + E3M);
  fm[1] = tmp0 * (tmp1 * E1M * u + E2M * uc1 + E3M * uc2);
  fm[2] = tmp0 * (tmp1 * E1M * v + E2M * vc1 + E3M * vc2);
  fm[3] = tmp0 * (E1M * vv + E2M * vvc1 + E3M * vvc2 + W2 * (E2M + E3M));
}
enum { M_KX = 0, M_KY = 1, M_IX = 2, M_IY = 3, M_JAC = 4 };

__global__ void k_fdm_split(Lvl L) {
  int bk, i, j;
  if (!tile_xy(L, bk, i, j)) return;
  const BlkDev &b = L.blk[bk];
  if (!b.fdm || i < 1 || i > b.nx - 1 || j < 1 || j > b.ny - 1) return;
  const CaseDev &c = L.cs[b.cas];
  const long long F = L.F;
  long long id = fidx(b, i, j);
  double d = L.q[Q_D * F + id], u = L.q[Q_U * F + id], v = L.q[Q_V * F + id], cc = L.q[Q_C * F + id];
  const double rJ = 1.0 / L.met[M_JAC * F + id];  // one divide for the metric quotients
  double fp[4], fm[4];
  // blockIdx.y: 0 the i-direction split, 1 the j-direction split (two threads per cell)
  const int dir = blockIdx.y;
  const int mx = dir == 0 ? M_KX : M_IX, my = dir == 0 ? M_KY : M_IY, out = dir == 0 ? D_SPI : D_SPJ;
  split_sw(d, u, v, cc, L.met[mx * F + id] * rJ, L.met[my * F + id] * rJ, c.gamma, fp, fm);
  for (int m = 0; m < 4; m++) { L.fdm[(out + m) * F + id] = fp[m]; L.fdm[(out + 4 + m) * F + id] = fm[m]; }
}

// fp_weno5 at point k (v[k-2..k+2]) and fm_weno5 producing hj(k-1) from v[k-2..k+2]
// (sub_Finite_Difference.f90:207-275).  The reference forms the weights as
// a_k = C_k / (ep + S_k)^2 and W_k = a_k / sum(a), six divides per
// evaluation; over the common denominator D_0 D_1 D_2 (D_k = (ep + S_k)^2)
// the same weights are W_k = C_k prod_{l != k} D_l / sum_m C_m prod_{l != m} D_l,
// one divide.  The results agree to a few ulps; an IEEE divide costs about a
// dozen FP64 instructions, and the sixteen evaluations per cell made the
// divides most of the kernel's FP64 work.  D_k >= 1e-12, so the numerators
// and the denominator stay above 1e-36, and they overflow only for smoothness
// indicators S_k beyond about 1e50, far from any split flux of this solver.
__device__ __forceinline__ double weno5_mix(double S0, double S1, double S2, double q03, double q13, double q23) {
  const double ep = 1.0e-6, C03 = 3.0 / 10.0, C13 = 3.0 / 5.0, C23 = 1.0 / 10.0;
  const double D0 = (ep + S0) * (ep + S0), D1 = (ep + S1) * (ep + S1), D2 = (ep + S2) * (ep + S2);
  const double n0 = C03 * (D1 * D2), n1 = C13 * (D0 * D2), n2 = C23 * (D0 * D1);
  return (n0 * q03 + n1 * q13 + n2 * q23) / (n0 + n1 + n2);
}
__device__ __forceinline__ double weno5_p(double vm2, double vm1, double v0, double vp1, double vp2) {
  double t0 = v0 - 2.0 * vp1 + vp2, t1 = 3.0 * v0 - 4.0 * vp1 + vp2;
  const double S0 = 13.0 / 12.0 * (t0 * t0) + 1.0 / 4.0 * (t1 * t1);
  t0 = vm1 - 2.0 * v0 + vp1; t1 = vm1 - vp1;
  const double S1 = 13.0 / 12.0 * (t0 * t0) + 1.0 / 4.0 * (t1 * t1);
  t0 = vm2 - 2.0 * vm1 + v0; t1 = vm2 - 4.0 * vm1 + 3.0 * v0;
  const double S2 = 13.0 / 12.0 * (t0 * t0) + 1.0 / 4.0 * (t1 * t1);
  const double q03 = 1.0 / 3.0 * v0 + 5.0 / 6.0 * vp1 - 1.0 / 6.0 * vp2;
  const double q13 = -1.0 / 6.0 * vm1 + 5.0 / 6.0 * v0 + 1.0 / 3.0 * vp1;
  const double q23 = 1.0 / 3.0 * vm2 - 7.0 / 6.0 * vm1 + 11.0 / 6.0 * v0;
  return weno5_mix(S0, S1, S2, q03, q13, q23);
}
__device__ __forceinline__ double weno5_m(double vm2, double vm1, double v0, double vp1, double vp2) {
  double t0 = v0 - 2.0 * vm1 + vm2, t1 = 3.0 * v0 - 4.0 * vm1 + vm2;
  const double S0 = 13.0 / 12.0 * (t0 * t0) + 1.0 / 4.0 * (t1 * t1);
  t0 = vp1 - 2.0 * v0 + vm1; t1 = vp1 - vm1;
  const double S1 = 13.0 / 12.0 * (t0 * t0) + 1.0 / 4.0 * (t1 * t1);
  t0 = vp2 - 2.0 * vp1 + v0; t1 = vp2 - 4.0 * vp1 + 3.0 * v0;
  const double S2 = 13.0 / 12.0 * (t0 * t0) + 1.0 / 4.0 * (t1 * t1);
  const double q03 = 1.0 / 3.0 * v0 + 5.0 / 6.0 * vm1 - 1.0 / 6.0 * vm2;
  const double q13 = -1.0 / 6.0 * vp1 + 5.0 / 6.0 * v0 + 1.0 / 3.0 * vm1;
  const double q23 = 1.0 / 3.0 * vp2 - 7.0 / 6.0 * vp1 + 11.0 / 6.0 * v0;
  return weno5_mix(S0, S1, S2, q03, q13, q23);
}

// WENO5 half-point fluxes (sub_Finite_Difference.f90:37-77) and the central
// viscous tensors Ev1/Ev2 (:87-117); indices are FDM cells = FVM cells.
// blockIdx.y picks the part: 0 the i-direction fluxes, 1 the j-direction
// fluxes, 2 the viscous tensors, so a cell's three independent chains run
// on three threads.
__global__ void k_fdm_flux(Lvl L) {
  const int part = blockIdx.y;
  int bk, i, j;
  if (!tile_xy(L, bk, i, j)) return;
  const BlkDev &b = L.blk[bk];
  int nxF = b.nx - 1, nyF = b.ny - 1;
  if (!b.fdm || i < 1 || i > nxF || j < 1 || j > nyF) return;
  const CaseDev &c = L.cs[b.cas];
  const long long F = L.F, P = b.P;
  long long id = fidx(b, i, j);
  if (part == 0 && j >= LFDM && j <= nyF - LFDM && i >= LFDM && i <= nxF - LFDM) {
    for (int m = 0; m < 4; m++) {
      const double *fp = L.fdm + (D_SPI + m) * F, *fm = L.fdm + (D_SPI + 4 + m) * F;
      double h1 = weno5_p(fp[id - 2], fp[id - 1], fp[id], fp[id + 1], fp[id + 2]);
      double h2 = weno5_m(fm[id - 1], fm[id], fm[id + 1], fm[id + 2], fm[id + 3]);
      L.fdm[(D_FI + m) * F + id] = -(h1 + h2);
    }
  }
  if (part == 1 && i >= LFDM && i <= nxF - LFDM && j >= LFDM && j <= nyF - LFDM) {
    for (int m = 0; m < 4; m++) {
      const double *fp = L.fdm + (D_SPJ + m) * F, *fm = L.fdm + (D_SPJ + 4 + m) * F;
      double h1 = weno5_p(fp[id - 2 * P], fp[id - P], fp[id], fp[id + P], fp[id + 2 * P]);
      double h2 = weno5_m(fm[id - P], fm[id], fm[id + P], fm[id + 2 * P], fm[id + 3 * P]);
      L.fdm[(D_FJ + m) * F + id] = -(h1 + h2);
    }
  }
  if (part == 2 && L.visc && i >= 2 && i <= nxF - 1 && j >= 2 && j <= nyF - 1) {
    const double *uu = L.q + Q_U * F, *vv = L.q + Q_V * F, *TT = L.q + Q_T * F;
    double mu0 = L.amu[id] + L.amut[id];
    double Ak0 = c.Cp * (L.amu[id] / c.Pr + L.amut[id] / PrT);
    double ui = 0.5 * (uu[id + 1] - uu[id - 1]), vi = 0.5 * (vv[id + 1] - vv[id - 1]), Ti = 0.5 * (TT[id + 1] - TT[id - 1]);
    double uj = 0.5 * (uu[id + P] - uu[id - P]), vj = 0.5 * (vv[id + P] - vv[id - P]), Tj = 0.5 * (TT[id + P] - TT[id - P]);
    double Akx = L.met[M_KX * F + id], Aky = L.met[M_KY * F + id], Aix = L.met[M_IX * F + id], Aiy = L.met[M_IY * F + id];
    const double rJ = 1.0 / L.met[M_JAC * F + id];
    double ux = ui * Akx + uj * Aix, vx = vi * Akx + vj * Aix, Tx = Ti * Akx + Tj * Aix;
    double uy = ui * Aky + uj * Aiy, vy = vi * Aky + vj * Aiy, Ty = Ti * Aky + Tj * Aiy;
    double t11 = (4.0 / 3.0 * ux - 2.0 / 3.0 * vy) * mu0, t22 = (4.0 / 3.0 * vy - 2.0 / 3.0 * ux) * mu0;
    double t12 = (uy + vx) * mu0;
    double E1 = uu[id] * t11 + vv[id] * t12 + Ak0 * Tx, E2 = uu[id] * t12 + vv[id] * t22 + Ak0 * Ty;
    L.fdm[(D_EV1 + 0) * F + id] = (Akx * t11 + Aky * t12) * rJ;
    L.fdm[(D_EV1 + 1) * F + id] = (Akx * t12 + Aky * t22) * rJ;
    L.fdm[(D_EV1 + 2) * F + id] = (Akx * E1 + Aky * E2) * rJ;
    L.fdm[(D_EV2 + 0) * F + id] = (Aix * t11 + Aiy * t12) * rJ;
    L.fdm[(D_EV2 + 1) * F + id] = (Aix * t12 + Aiy * t22) * rJ;
    L.fdm[(D_EV2 + 2) * F + id] = (Aix * E1 + Aiy * E2) * rJ;
  }
}

// FDM residual (sub_Finite_Difference.f90:121-145) with the viscous half-point
// averages added to the inviscid fluxes
__global__ void k_fdm_res(Lvl L) {
  int bk, i, j;
  if (!tile_xy(L, bk, i, j)) return;
  const BlkDev &b = L.blk[bk];
  int nxF = b.nx - 1, nyF = b.ny - 1;
  if (!b.fdm || i < LFDM + 1 || i > nxF - LFDM || j < LFDM + 1 || j > nyF - LFDM) return;
  const long long F = L.F, P = b.P;
  long long id = fidx(b, i, j);
  for (int m = 0; m < 4; m++) {
    double fi0 = L.fdm[(D_FI + m) * F + id], fi1 = L.fdm[(D_FI + m) * F + id - 1];
    double fj0 = L.fdm[(D_FJ + m) * F + id], fj1 = L.fdm[(D_FJ + m) * F + id - P];
    if (L.visc && m >= 1) {
      const double *e1 = L.fdm + (D_EV1 + m - 1) * F, *e2 = L.fdm + (D_EV2 + m - 1) * F;
      fi0 = fi0 + 0.5 * (e1[id] + e1[id + 1]);
      fi1 = fi1 + 0.5 * (e1[id - 1] + e1[id]);
      fj0 = fj0 + 0.5 * (e2[id] + e2[id + P]);
      fj1 = fj1 + 0.5 * (e2[id - P] + e2[id]);
    }
    L.res[m * F + id] = (fi0 - fi1 + fj0 - fj1);
  }
}

void launch_fdm(const Lvl &L, cudaStream_t s) {
  k_fdm_split<<<dim3(L.ntiles, 2), TILE, 0, s>>>(L);
  k_fdm_flux<<<dim3(L.ntiles, L.visc ? 3 : 2), TILE, 0, s>>>(L);
  k_fdm_res<<<L.ntiles, TILE, 0, s>>>(L);
}

// dual-time source (sub_Residual.f90:55-65)
__global__ void k_dual(Lvl L, double sfac) {
  int bk, i, j;
  if (!tile_xy(L, bk, i, j)) return;
  const BlkDev &b = L.blk[bk];
  if (i < 1 || i > b.nx - 1 || j < 1 || j > b.ny - 1) return;
  const long long F = L.F;
  long long id = fidx(b, i, j);
  double vol = L.geo[G_VOL * F + id];
  for (int m = 0; m < L.nvar; m++)
    L.res[m * F + id] = L.res[m * F + id] - (3.0 * L.U[m * F + id] - 4.0 * L.un[m * F + id] + L.un1[m * F + id]) * vol * sfac;
}
void launch_dual_term(const Lvl &L, double sfac, cudaStream_t s) { k_dual<<<L.ntiles, TILE, 0, s>>>(L, sfac); }

}  // namespace ec2d
