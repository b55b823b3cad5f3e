// ec2d_oracle.cpp -- CPU oracle: a plain C++ restatement of the OpenCFD-EC2D
// v1.5.4 pseudo-time-marching core (TEST INFRASTRUCTURE ONLY; the product
// library never links this file).
//
// Parity status: UNPINNED by the reference (no tests, no golden vectors, no
// Fortran compiler available).  Each routine below cites the Fortran it
// restates; loop orders, operation order and the reference's precision quirks
// (single-precision literals such as 0.3 and 0.09) are kept.
//
// Build: see oracle/Makefile (-O2 -fno-fast-math -ffp-contract=off).
#include "ec2d_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---- constants, opencfd_ec2d_v1.5.4.f90:39-53 ------------------------------
const double PI = 3.1415926535897932;
enum { Scheme_UD1 = 0, Scheme_NND2 = 1, Scheme_UD3 = 2, Scheme_WENO3 = 3,
       Scheme_MUSCL2 = 4, Scheme_MUSCL3 = 5, Scheme_OMUSCL2 = 6 };
enum { Flux_Steger_Warming = 1, Flux_HLL = 2, Flux_HLLC = 3, Flux_Roe = 4,
       Flux_VanLeer = 5, Flux_Ausm = 6 };
enum { Reconst_Original = 0, Reconst_Conservative = 1, Reconst_Characteristic = 2 };
enum { BC_Wall = -10, BC_Farfield = -20, BC_Symmetry = -30, BC_Inlet = -40, BC_Outlet = -50 };
enum { Time_Euler1 = 1, Time_RK3 = 3, Time_LU_SGS = 0, Time_dual_LU_SGS = -1 };
enum { Turb_NONE = 0, Turb_BL = 1, Turb_SA = 2, Turb_SST = 3 };
const int LAP = 2;
const double PrT = 0.9;
enum { Method_FVM = 0, Method_FDM = 1 };
const int LFDM = 4;

// Fortran-style arrays with arbitrary lower bounds, column-major.
struct A2 {
  std::vector<double> v;
  int i0 = 0, j0 = 0, ni = 0, nj = 0;
  void alloc(int ia, int ib, int ja, int jb, double init = 0.0) {
    i0 = ia; j0 = ja; ni = ib - ia + 1; nj = jb - ja + 1;
    v.assign((size_t)ni * nj, init);
  }
  double &operator()(int i, int j) { return v[(size_t)(i - i0) + (size_t)ni * (j - j0)]; }
  double operator()(int i, int j) const { return v[(size_t)(i - i0) + (size_t)ni * (j - j0)]; }
  bool empty() const { return v.empty(); }
};
struct A3 {
  std::vector<double> v;
  int nm = 0, i0 = 0, j0 = 0, ni = 0, nj = 0;
  void alloc(int m, int ia, int ib, int ja, int jb, double init = 0.0) {
    nm = m; i0 = ia; j0 = ja; ni = ib - ia + 1; nj = jb - ja + 1;
    v.assign((size_t)nm * ni * nj, init);
  }
  // m is 1-based like Fortran
  double &operator()(int m, int i, int j) {
    return v[(size_t)(m - 1) + (size_t)nm * ((size_t)(i - i0) + (size_t)ni * (j - j0))];
  }
  double *col(int i, int j) { return &v[(size_t)nm * ((size_t)(i - i0) + (size_t)ni * (j - j0))]; }
  bool empty() const { return v.empty(); }
};

struct BcMsg { int f_no, face, ist, iend, jst, jend, neighb, subface, orient; };

// Block_TYPE, opencfd_ec2d_v1.5.4.f90:66-83
struct Block {
  int nx = 0, ny = 0, FVM_FDM = Method_FVM;
  A2 x, y, x1, y1, Akx, Aky, Aix, Aiy, Ajac;
  A3 U, Un, Un1, Res, QF, deltU, dU;
  A2 dt, Amu, Amu_t, vol, si, sj, ni1, ni2, nj1, nj2, Lci, Lcj, Lvi, Lvj, dw;
  std::vector<BcMsg> bc;
};
// Mesh_TYPE, opencfd_ec2d_v1.5.4.f90:87-96
struct Mesh {
  int Num_Block = 0, Num_Cell = 0, Kstep = 0, Nvar = 4;
  double Res_max[6] = {0}, Res_rms[6] = {0}, tt = 0;
  std::vector<Block> B;
  int turb = 0, scheme = 0, flux = 0, recon = 0;
};
// Flow_Var temporaries, opencfd_ec2d_v1.5.4.f90:132-135
struct FlowVar {
  A2 d, uu, v, T, p, cc;
  A3 Fluxi, Fluxj;
};

struct Solver {
  orc_params P;
  // Global_Var scalars, opencfd_ec2d_v1.5.4.f90:103-110
  int Num_Mesh = 1, Nvar = 4;
  double Ma, Re, gamma, Pr, AoA, Cp, Cv, p_outlet, T_inf, Twall, vt_inf, Kt_inf, Wt_inf;
  double dt_global, CFL, dtmax, dtmin;
  int If_viscous, Iflag_turbulence_model, Iflag_Scheme, IFlag_flux, Iflag_local_dt,
      IFlag_Reconstruction, Time_Method, Kstep_show;
  std::vector<Mesh> mesh;         // index 1..Num_Mesh (0 unused)
  std::vector<Block> pending;     // blocks added before setup
  std::vector<int> fdm_blocks;
  std::vector<std::vector<double>> dw_in;
  bool setup_done = false;
  int err = 0, err_b = 0, err_i = 0, err_j = 0;
  int dual_iflag1 = 0, dual_iflag = 0;
  // extension, off by default: coarse levels keep an eddy viscosity
  // restricted from the next finer level instead of the reference's zero
  int mg_amut = 0;
};

// ----------------------------------------------------------------------------
// read_parameter derived quantities, opencfd_ec2d_v1.5.4.f90:216-233
void apply_params(Solver &S, const orc_params &p) {
  S.P = p;
  S.Ma = p.Ma; S.Re = p.Re; S.gamma = p.gamma; S.Pr = p.Pr;
  S.If_viscous = p.If_viscous; S.Iflag_turbulence_model = p.Iflag_turbulence_model;
  S.Iflag_local_dt = p.Iflag_local_dt; S.dt_global = p.dt_global; S.CFL = p.CFL;
  S.dtmax = p.dtmax; S.dtmin = p.dtmin; S.Time_Method = p.Time_Method;
  S.p_outlet = p.P_outlet; S.T_inf = p.T_inf; S.vt_inf = p.vt_inf; S.Kt_inf = p.Kt_inf;
  S.Wt_inf = p.Wt_inf; S.Iflag_Scheme = p.Iflag_Scheme; S.IFlag_flux = p.Iflag_flux;
  S.IFlag_Reconstruction = p.IFlag_Reconstruction; S.Kstep_show = p.Kstep_show;
  S.Num_Mesh = p.Num_Mesh;
  if (S.Iflag_turbulence_model == Turb_SST) S.Nvar = 6;
  else if (S.Iflag_turbulence_model == Turb_SA) S.Nvar = 5;
  else S.Nvar = 4;
  S.AoA = p.AoA * PI / 180.0;
  S.Cv = 1.0 / (S.gamma * (S.gamma - 1.0) * S.Ma * S.Ma);
  S.Cp = S.Cv * S.gamma;
  S.Twall = p.Twall / p.T_inf;
}

// ---- geometry of one block: sub_init.f90:176-204 (and 329-353 for coarse) --
void block_geometry(Block &B) {
  int nx = B.nx, ny = B.ny;
  for (int j = 1; j <= ny - 1; j++)
    for (int i = 1; i <= nx - 1; i++)
      B.vol(i, j) = std::fabs((B.x(i, j) - B.x(i + 1, j + 1)) * (B.y(i + 1, j) - B.y(i, j + 1)) -
                              (B.x(i + 1, j) - B.x(i, j + 1)) * (B.y(i, j) - B.y(i + 1, j + 1))) * 0.5;
  for (int j = 1; j <= ny - 1; j++)
    for (int i = 1; i <= nx; i++) {
      double dx = B.x(i, j + 1) - B.x(i, j), dy = B.y(i, j + 1) - B.y(i, j);
      B.si(i, j) = std::sqrt(dx * dx + dy * dy);
      B.ni1(i, j) = dy / B.si(i, j);
      B.ni2(i, j) = -dx / B.si(i, j);
    }
  for (int j = 1; j <= ny; j++)
    for (int i = 1; i <= nx - 1; i++) {
      double dx = B.x(i + 1, j) - B.x(i, j), dy = B.y(i + 1, j) - B.y(i, j);
      B.sj(i, j) = std::sqrt(dx * dx + dy * dy);
      B.nj1(i, j) = -dy / B.sj(i, j);
      B.nj2(i, j) = dx / B.sj(i, j);
    }
}

// allocation + initial values, sub_init.f90:138-174 (fine) / 291-318 (coarse)
void block_alloc(Solver &S, Block &B, int nvar, bool fine) {
  int nx = B.nx, ny = B.ny;
  B.x.alloc(1 - LAP, nx + LAP, 1 - LAP, ny + LAP);
  B.y.alloc(1 - LAP, nx + LAP, 1 - LAP, ny + LAP);
  B.x1.alloc(1 - LAP, nx + LAP - 1, 1 - LAP, ny + LAP - 1);
  B.y1.alloc(1 - LAP, nx + LAP - 1, 1 - LAP, ny + LAP - 1);
  B.U.alloc(nvar, 1 - LAP, nx + LAP - 1, 1 - LAP, ny + LAP - 1);
  B.deltU.alloc(4, 1 - LAP, nx + LAP - 1, 1 - LAP, ny + LAP - 1);
  B.Res.alloc(nvar, 1, nx - 1, 1, ny - 1);
  B.dt.alloc(1, nx - 1, 1, ny - 1);
  B.dU.alloc(nvar, 1, nx, 1, ny);
  B.Amu.alloc(1 - LAP, nx + LAP - 1, 1 - LAP, ny + LAP - 1);
  B.Amu_t.alloc(1 - LAP, nx + LAP - 1, 1 - LAP, ny + LAP - 1);
  A2 *g[] = {&B.vol, &B.si, &B.sj, &B.ni1, &B.ni2, &B.nj1, &B.nj2, &B.Lci, &B.Lcj, &B.Lvi, &B.Lvj};
  for (A2 *a : g) a->alloc(1, nx, 1, ny);
  B.Un.alloc(nvar, 0, nx, 0, ny);
  if (S.Time_Method == Time_dual_LU_SGS) B.Un1.alloc(S.Nvar, 0, nx, 0, ny);
  if (!fine) B.QF.alloc(4, 1, nx - 1, 1, ny - 1);
  // U(1)=1, U(2)=0, U(3)=0, U(4)=1 ; Un(4)=0 on the fine mesh, 1 on coarse
  for (int j = 1 - LAP; j <= ny + LAP - 1; j++)
    for (int i = 1 - LAP; i <= nx + LAP - 1; i++) {
      B.U(1, i, j) = 1.0; B.U(2, i, j) = 0.0; B.U(3, i, j) = 0.0; B.U(4, i, j) = 1.0;
      if (fine && nvar == 5) B.U(5, i, j) = 1.0 / S.Re;
      if (fine && nvar == 6) { B.U(5, i, j) = 0.0; B.U(6, i, j) = 1.0; }
    }
  for (int j = 0; j <= ny; j++)
    for (int i = 0; i <= nx; i++) {
      B.Un(1, i, j) = 1.0; B.Un(2, i, j) = 0.0; B.Un(3, i, j) = 0.0;
      B.Un(4, i, j) = fine ? 0.0 : 1.0;
    }
}

// check_mesh_multigrid, sub_init.f90:39-107
int check_mesh_multigrid(Solver &S) {
  int Km_grid = S.pending[0].nx;
  for (auto &B : S.pending) {
    int Km = 1, NN = 2;
    while ((B.nx - 1) % NN == 0 && (B.nx - 1) / NN >= 2 && (B.ny - 1) % NN == 0 &&
           (B.ny - 1) / NN >= 2) {
      Km++; NN *= 2;
    }
    Km_grid = std::min(Km_grid, Km);
  }
  for (auto &B : S.pending)
    for (auto &c : B.bc) {
      int NN = 1, Km = 1;
      while ((c.ist - 1) % NN == 0 && (c.iend - 1) % NN == 0 && (c.jst - 1) % NN == 0 &&
             (c.jend - 1) % NN == 0) {
        NN *= 2; Km++;
        if (NN > (1 << 20)) break;  // all-ones index ranges would loop forever
      }
      Km_grid = std::min(Km_grid, Km);
    }
  return std::min(3, std::min(Km_grid, S.Num_Mesh));
}

// Creat_Mesh(m1,m2), sub_init.f90:256-380
void creat_mesh(Solver &S, int m1, int m2) {
  Mesh &MP1 = S.mesh[m1], &MP2 = S.mesh[m2];
  MP2.Num_Block = MP1.Num_Block;
  MP2.Num_Cell = 0;
  MP2.B.resize(MP2.Num_Block);
  for (int m = 0; m < MP1.Num_Block; m++) {
    Block &B1 = MP1.B[m], &B2 = MP2.B[m];
    B2.FVM_FDM = Method_FVM;
    B2.nx = (B1.nx - 1) / 2 + 1;
    B2.ny = (B1.ny - 1) / 2 + 1;
    MP2.Num_Cell += (B2.nx - 1) * (B2.ny - 1);
    block_alloc(S, B2, 4, false);
    for (int j = 1; j <= B2.ny; j++)
      for (int i = 1; i <= B2.nx; i++) {
        B2.x(i, j) = B1.x(2 * i - 1, 2 * j - 1);
        B2.y(i, j) = B1.y(2 * i - 1, 2 * j - 1);
      }
    block_geometry(B2);
    B2.bc.resize(B1.bc.size());
    for (size_t k = 0; k < B1.bc.size(); k++) {
      BcMsg c = B1.bc[k];
      c.ist = (c.ist - 1) / 2 + 1; c.iend = (c.iend - 1) / 2 + 1;
      c.jst = (c.jst - 1) / 2 + 1; c.jend = (c.jend - 1) / 2 + 1;
      B2.bc[k] = c;
    }
  }
  MP2.Kstep = 0; MP2.tt = 0.0;
}

// Update_coordinate_buffer_onemesh, sub_boundary.f90:174-282 (file output omitted)
void update_coordinate_buffer_onemesh(Solver &S, int nMesh) {
  Mesh &MP = S.mesh[nMesh];
  for (int mb = 0; mb < MP.Num_Block; mb++) {
    Block &B = MP.B[mb];
    for (auto &Bc : B.bc) {
      int ib2 = Bc.ist, ie2 = Bc.iend, jb2 = Bc.jst, je2 = Bc.jend;
      if (Bc.neighb > 0) {
        int n1 = Bc.iend - Bc.ist + Bc.jend - Bc.jst + 1;
        std::vector<double> Ux(2 * n1 * LAP);
        auto UX = [&](int c, int k, int l) -> double & { return Ux[(c - 1) + 2 * ((k - 1) + n1 * (l - 1))]; };
        Block &B1 = MP.B[Bc.neighb - 1];
        BcMsg &Bc1 = B1.bc[Bc.subface - 1];
        int ib1 = Bc1.ist, ie1 = Bc1.iend, jb1 = Bc1.jst, je1 = Bc1.jend;
        for (int l = 1; l <= LAP; l++) {
          if (Bc1.face == 1) {
            for (int k = 1; k <= je1 - jb1 + 1; k++) { UX(1, k, l) = B1.x(ib1 + l, jb1 + k - 1); UX(2, k, l) = B1.y(ib1 + l, jb1 + k - 1); }
          } else if (Bc1.face == 2) {
            for (int k = 1; k <= ie1 - ib1 + 1; k++) { UX(1, k, l) = B1.x(ib1 + k - 1, jb1 + l); UX(2, k, l) = B1.y(ib1 + k - 1, jb1 + l); }
          } else if (Bc1.face == 3) {
            for (int k = 1; k <= je1 - jb1 + 1; k++) { UX(1, k, l) = B1.x(ie1 - LAP - 1 + l, jb1 + k - 1); UX(2, k, l) = B1.y(ie1 - LAP - 1 + l, jb1 + k - 1); }
          } else {
            for (int k = 1; k <= ie1 - ib1 + 1; k++) { UX(1, k, l) = B1.x(ib1 + k - 1, je1 - LAP - 1 + l); UX(2, k, l) = B1.y(ib1 + k - 1, je1 - LAP - 1 + l); }
          }
        }
        for (int k = 1; k <= n1; k++) {
          int k1 = (Bc.orient == 2) ? k : n1 + 1 - k;
          for (int l = 1; l <= LAP; l++) {
            if (Bc.face == 1) { B.x(ib2 - LAP - 1 + l, jb2 + k - 1) = UX(1, k1, l); B.y(ib2 - LAP - 1 + l, jb2 + k - 1) = UX(2, k1, l); }
            else if (Bc.face == 2) { B.x(ib2 + k - 1, jb2 - LAP - 1 + l) = UX(1, k1, l); B.y(ib2 + k - 1, jb2 - LAP - 1 + l) = UX(2, k1, l); }
            else if (Bc.face == 3) { B.x(ie2 + l, jb2 + k - 1) = UX(1, k1, l); B.y(ie2 + l, jb2 + k - 1) = UX(2, k1, l); }
            else { B.x(ib2 + k - 1, je2 + l) = UX(1, k1, l); B.y(ib2 + k - 1, je2 + l) = UX(2, k1, l); }
          }
        }
      } else {
        for (int l = 1; l <= LAP; l++) {
          if (Bc.face == 1) {
            for (int j = jb2; j <= je2; j++) { B.x(ib2 - l, j) = 2.0 * B.x(ib2, j) - B.x(ib2 + l, j); B.y(ib2 - l, j) = 2.0 * B.y(ib2, j) - B.y(ib2 + l, j); }
          } else if (Bc.face == 2) {
            for (int i = ib2; i <= ie2; i++) { B.x(i, jb2 - l) = 2.0 * B.x(i, jb2) - B.x(i, jb2 + l); B.y(i, jb2 - l) = 2.0 * B.y(i, jb2) - B.y(i, jb2 + l); }
          } else if (Bc.face == 3) {
            for (int j = jb2; j <= je2; j++) { B.x(ie2 + l, j) = 2.0 * B.x(ie2, j) - B.x(ie2 - l, j); B.y(ie2 + l, j) = 2.0 * B.y(ie2, j) - B.y(ie2 - l, j); }
          } else {
            for (int i = ib2; i <= ie2; i++) { B.x(i, je2 + l) = 2.0 * B.x(i, je2) - B.x(i, je2 - l); B.y(i, je2 + l) = 2.0 * B.y(i, je2) - B.y(i, je2 - l); }
          }
        }
      }
    }
    int nx = B.nx, ny = B.ny;
    for (int j = 1; j <= LAP; j++)
      for (int i = 1; i <= LAP; i++) {
        int i1 = 1 - i, j1 = 1 - j, i2 = nx + i, j2 = ny + j;
        B.x(i1, j1) = B.x(i1, 1) + B.x(1, j1) - B.x(1, 1); B.y(i1, j1) = B.y(i1, 1) + B.y(1, j1) - B.y(1, 1);
        B.x(i2, j2) = B.x(i2, ny) + B.x(nx, j2) - B.x(nx, ny); B.y(i2, j2) = B.y(i2, ny) + B.y(nx, j2) - B.y(nx, ny);
        B.x(i1, j2) = B.x(i1, ny) + B.x(1, j2) - B.x(1, ny); B.y(i1, j2) = B.y(i1, ny) + B.y(1, j2) - B.y(1, ny);
        B.x(i2, j1) = B.x(i2, 1) + B.x(nx, j1) - B.x(nx, 1); B.y(i2, j1) = B.y(i2, 1) + B.y(nx, j1) - B.y(nx, 1);
      }
    for (int j = 1 - LAP; j <= ny + LAP - 1; j++)
      for (int i = 1 - LAP; i <= nx + LAP - 1; i++) {
        B.x1(i, j) = (B.x(i, j) + B.x(i + 1, j) + B.x(i, j + 1) + B.x(i + 1, j + 1)) * 0.25;
        B.y1(i, j) = (B.y(i, j) + B.y(i + 1, j) + B.y(i, j + 1) + B.y(i + 1, j + 1)) * 0.25;
      }
  }
}

// dx0/dy0 6th-order metric derivatives, sub_Finite_Difference.f90:387-439
void dx0(const std::vector<double> &f, std::vector<double> &fx, int nx, int ny, double hx) {
  auto F = [&](int i, int j) { return f[(i - 1) + (size_t)nx * (j - 1)]; };
  auto FX = [&](int i, int j) -> double & { return fx[(i - 1) + (size_t)nx * (j - 1)]; };
  double b1 = 8.0 / (12.0 * hx), b2 = 1.0 / (12.0 * hx), a1 = 1.0 / (60.0 * hx),
         a2 = -3.0 / (20.0 * hx), a3 = 3.0 / (4.0 * hx);
  for (int j = 1; j <= ny; j++)
    for (int i = 4; i <= nx - 3; i++)
      FX(i, j) = a1 * (F(i + 3, j) - F(i - 3, j)) + a2 * (F(i + 2, j) - F(i - 2, j)) + a3 * (F(i + 1, j) - F(i - 1, j));
  for (int j = 1; j <= ny; j++) {
    FX(1, j) = (-3.0 * F(1, j) + 4.0 * F(2, j) - F(3, j)) / (2.0 * hx);
    FX(2, j) = (-2.0 * F(1, j) - 3.0 * F(2, j) + 6.0 * F(3, j) - F(4, j)) / (6.0 * hx);
    FX(3, j) = b1 * (F(4, j) - F(2, j)) - b2 * (F(5, j) - F(1, j));
    FX(nx - 2, j) = b1 * (F(nx - 1, j) - F(nx - 3, j)) - b2 * (F(nx, j) - F(nx - 4, j));
    FX(nx - 1, j) = (F(nx - 3, j) - 6.0 * F(nx - 2, j) + 3.0 * F(nx - 1, j) + 2.0 * F(nx, j)) / (6.0 * hx);
    FX(nx, j) = (F(nx - 2, j) - 4.0 * F(nx - 1, j) + 3.0 * F(nx, j)) / (2.0 * hx);
  }
}
void dy0(const std::vector<double> &f, std::vector<double> &fy, int nx, int ny, double hy) {
  auto F = [&](int i, int j) { return f[(i - 1) + (size_t)nx * (j - 1)]; };
  auto FY = [&](int i, int j) -> double & { return fy[(i - 1) + (size_t)nx * (j - 1)]; };
  double b1 = 8.0 / (12.0 * hy), b2 = 1.0 / (12.0 * hy), a1 = 1.0 / (60.0 * hy),
         a2 = -3.0 / (20.0 * hy), a3 = 3.0 / (4.0 * hy);
  for (int j = 4; j <= ny - 3; j++)
    for (int i = 1; i <= nx; i++)
      FY(i, j) = a1 * (F(i, j + 3) - F(i, j - 3)) + a2 * (F(i, j + 2) - F(i, j - 2)) + a3 * (F(i, j + 1) - F(i, j - 1));
  for (int i = 1; i <= nx; i++) {
    FY(i, 1) = (-3.0 * F(i, 1) + 4.0 * F(i, 2) - F(i, 3)) / (2.0 * hy);
    FY(i, 2) = (-2.0 * F(i, 1) - 3.0 * F(i, 2) + 6.0 * F(i, 3) - F(i, 4)) / (6.0 * hy);
    FY(i, 3) = b1 * (F(i, 4) - F(i, 2)) - b2 * (F(i, 5) - F(i, 1));
    FY(i, ny - 2) = b1 * (F(i, ny - 1) - F(i, ny - 3)) - b2 * (F(i, ny) - F(i, ny - 4));
    FY(i, ny - 1) = (F(i, ny - 3) - 6.0 * F(i, ny - 2) + 3.0 * F(i, ny - 1) + 2.0 * F(i, ny)) / (6.0 * hy);
    FY(i, ny) = (F(i, ny - 2) - 4.0 * F(i, ny - 1) + 3.0 * F(i, ny)) / (2.0 * hy);
  }
}

// comput_Jacobian, sub_Finite_Difference.f90:314-382 (file output omitted)
void comput_jacobian(Solver &S) {
  for (auto &B : S.mesh[1].B) {
    if (B.FVM_FDM != Method_FDM) continue;
    int nx = B.nx - 1, ny = B.ny - 1;
    B.Akx.alloc(1, nx, 1, ny); B.Aky.alloc(1, nx, 1, ny); B.Aix.alloc(1, nx, 1, ny);
    B.Aiy.alloc(1, nx, 1, ny); B.Ajac.alloc(1, nx, 1, ny);
    std::vector<double> xx(nx * ny), yy(nx * ny), xk(nx * ny), xi(nx * ny), yk(nx * ny), yi(nx * ny);
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= nx; i++) {
        xx[(i - 1) + nx * (j - 1)] = B.x1(i, j);
        yy[(i - 1) + nx * (j - 1)] = B.y1(i, j);
      }
    dx0(xx, xk, nx, ny, 1.0); dx0(yy, yk, nx, ny, 1.0);
    dy0(xx, xi, nx, ny, 1.0); dy0(yy, yi, nx, ny, 1.0);
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= nx; i++) {
        size_t k = (i - 1) + (size_t)nx * (j - 1);
        double J = xk[k] * yi[k] - xi[k] * yk[k];
        J = 1.0 / J;
        B.Ajac(i, j) = J;
        B.Akx(i, j) = J * yi[k];
        B.Aky(i, j) = -J * xi[k];
        B.Aix(i, j) = -J * yk[k];
        B.Aiy(i, j) = J * xk[k];
      }
  }
}

// comput_dw, sub_turbulence_SST.f90:274-340 (dist_wall.dat cache replaced by orc_set_dw)
void comput_dw(Solver &S) {
  Mesh &MP = S.mesh[1];
  for (auto &B : MP.B) B.dw.alloc(0, B.nx, 0, B.ny, 1.0);
  if (!S.dw_in.empty()) {
    for (int m = 0; m < MP.Num_Block; m++) {
      Block &B = MP.B[m];
      for (int j = 1; j <= B.ny - 1; j++)
        for (int i = 1; i <= B.nx - 1; i++) B.dw(i, j) = S.dw_in[m][(i - 1) + (size_t)(B.nx - 1) * (j - 1)];
    }
    return;
  }
  for (auto &B : MP.B) {
    int nx = B.nx, ny = B.ny;
    A2 dwn; dwn.alloc(1, nx, 1, ny);
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= nx; i++) {
        double best = 1.0e10;
        for (auto &B1 : MP.B)
          for (auto &c : B1.bc) {
            if (c.neighb != BC_Wall) continue;
            for (int j1 = c.jst; j1 <= c.jend; j1++)
              for (int i1 = c.ist; i1 <= c.iend; i1++) {
                double dx = B.x(i, j) - B1.x(i1, j1), dy = B.y(i, j) - B1.y(i1, j1);
                double d1 = std::sqrt(dx * dx + dy * dy);
                if (d1 < best) best = d1;
              }
          }
        dwn(i, j) = best;
      }
    for (int j = 1; j <= ny - 1; j++)
      for (int i = 1; i <= nx - 1; i++)
        B.dw(i, j) = (dwn(i, j) + dwn(i + 1, j) + dwn(i, j + 1) + dwn(i + 1, j + 1)) * 0.25;
  }
}

// ---- boundary conditions: sub_boundary.f90 ---------------------------------
// boundary_wall, sub_boundary.f90:306-386
void boundary_wall(Solver &S, int nMesh, Block &B, const BcMsg &Bc) {
  Mesh &MP = S.mesh[nMesh];
  const double beta1_SST = 0.075;
  double Tsb = 110.4 / S.T_inf;
  double gamma = S.gamma, Ma = S.Ma;
  for (int j = Bc.jst; j <= Bc.jend; j++)
    for (int i = Bc.ist; i <= Bc.iend; i++)
      for (int k = 1; k <= LAP; k++) {
        int i1, j1, i2, j2;
        if (Bc.face == 1) { i1 = i + k - 1; j1 = j; i2 = i - k; j2 = j; }
        else if (Bc.face == 2) { i1 = i; j1 = j + k - 1; i2 = i; j2 = j - k; }
        else if (Bc.face == 3) { i1 = i - k; j1 = j; i2 = i + k - 1; j2 = j; }
        else { i1 = i; j1 = j - k; i2 = i; j2 = j + k - 1; }
        // d1: interior density.  The reference assigns it only on the isothermal
        // branch and reads it in the SST update below on both branches (an
        // uninitialised local on the adiabatic branch); the interior density
        // is the value the SST wall formula intends.
        double d1 = B.U(1, i1, j1), d2 = 0;
        if (S.Twall <= 0) {
          B.U(1, i2, j2) = B.U(1, i1, j1);
          B.U(2, i2, j2) = -B.U(2, i1, j1);
          B.U(3, i2, j2) = -B.U(3, i1, j1);
          B.U(4, i2, j2) = B.U(4, i1, j1);
        } else {
          d1 = B.U(1, i1, j1);
          double u1 = B.U(2, i1, j1) / d1, v1 = B.U(3, i1, j1) / d1;
          double p1 = (B.U(4, i1, j1) - 0.5 * d1 * (u1 * u1 + v1 * v1)) * (gamma - 1.0);
          double T1 = gamma * Ma * Ma * p1 / d1;
          double p2 = p1, T2 = 2.0 * S.Twall - T1, u2 = -u1, v2 = -v1;
          d2 = gamma * Ma * Ma * p2 / T2;
          B.U(1, i2, j2) = d2;
          B.U(2, i2, j2) = d2 * u2;
          B.U(3, i2, j2) = d2 * v2;
          B.U(4, i2, j2) = p2 / (gamma - 1.0) + 0.5 * d2 * (u2 * u2 + v2 * v2);
        }
        if (MP.Nvar == 5) B.U(5, i2, j2) = 0.0;
        if (MP.Nvar == 6) {
          d2 = B.U(1, i2, j2);
          double T2 = (B.U(4, i2, j2) - 0.5 * (B.U(2, i2, j2) * B.U(2, i2, j2) + B.U(3, i2, j2) * B.U(3, i2, j2)) / d2) / (S.Cv * d2);
          double Amu2 = (1.0 + Tsb) * std::sqrt(T2 * T2 * T2) / (Tsb + T2);
          double dwv = B.dw(i1, j1);
          double wt = 60.0 * Amu2 / (d2 * beta1_SST * (dwv * dwv) * S.Re * S.Re);
          B.U(5, i2, j2) = -B.U(5, i1, j1);
          B.U(6, i2, j2) = (d1 + d2) * wt - B.U(6, i1, j1);
        }
      }
}

// Symmetry_or_slidewall, sub_boundary.f90:391-451
void symmetry_or_slidewall(Solver &S, int nMesh, Block &B, const BcMsg &Bc) {
  Mesh &MP = S.mesh[nMesh];
  for (int j = Bc.jst; j <= Bc.jend; j++)
    for (int i = Bc.ist; i <= Bc.iend; i++) {
      double n1, n2;
      if (Bc.face == 1 || Bc.face == 3) {
        double dx = B.x(i, j + 1) - B.x(i, j), dy = B.y(i, j + 1) - B.y(i, j);
        double si = std::sqrt(dx * dx + dy * dy);
        n1 = dy / si; n2 = -dx / si;
      } else {
        double dx = B.x(i + 1, j) - B.x(i, j), dy = B.y(i + 1, j) - B.y(i, j);
        double si = std::sqrt(dx * dx + dy * dy);
        n1 = -dy / si; n2 = dx / si;
      }
      for (int k = 1; k <= LAP; k++) {
        int i1, j1, i2, j2;
        if (Bc.face == 1) { i1 = i + k - 1; j1 = j; i2 = i - k; j2 = j; }
        else if (Bc.face == 2) { i1 = i; j1 = j + k - 1; i2 = i; j2 = j - k; }
        else if (Bc.face == 3) { i1 = i - k; j1 = j; i2 = i + k - 1; j2 = j; }
        else { i1 = i; j1 = j - k; i2 = i; j2 = j + k - 1; }
        double Vn = B.U(2, i1, j1) * n1 + B.U(3, i1, j1) * n2;
        B.U(1, i2, j2) = B.U(1, i1, j1);
        B.U(2, i2, j2) = B.U(2, i1, j1) - 2.0 * Vn * n1;
        B.U(3, i2, j2) = B.U(3, i1, j1) - 2.0 * Vn * n2;
        B.U(4, i2, j2) = B.U(4, i1, j1);
        if (MP.Nvar == 5) B.U(5, i2, j2) = B.U(5, i1, j1);
        else if (MP.Nvar == 6) { B.U(5, i2, j2) = B.U(5, i1, j1); B.U(6, i2, j2) = B.U(6, i1, j1); }
      }
    }
}

// boundary_Farfield_inlet_outlet, sub_boundary.f90:457-581
void boundary_farfield(Solver &S, int nMesh, Block &B, const BcMsg &Bc, int Bctype) {
  Mesh &MP = S.mesh[nMesh];
  double gamma = S.gamma, Ma = S.Ma;
  double d_inf = 1.0, u_inf = 1.0 * std::cos(S.AoA), v_inf = 1.0 * std::sin(S.AoA),
         p_inf = 1.0 / (gamma * Ma * Ma);
  for (int j = Bc.jst; j <= Bc.jend; j++)
    for (int i = Bc.ist; i <= Bc.iend; i++) {
      int i1, j1;
      if (Bc.face == 1) { i1 = i; j1 = j; }
      else if (Bc.face == 2) { i1 = i; j1 = j; }
      else if (Bc.face == 3) { i1 = i - 1; j1 = j; }
      else { i1 = i; j1 = j - 1; }
      double d1 = B.U(1, i1, j1), u1 = B.U(2, i1, j1) / d1, v1 = B.U(3, i1, j1) / d1;
      double p1 = (B.U(4, i1, j1) - 0.5 * d1 * (u1 * u1 + v1 * v1)) * (gamma - 1.0);
      double c1 = std::sqrt(gamma * p1 / d1);
      double n1, n2, dx, dy, s;
      if (Bc.face == 1) {
        dx = B.x(i, j + 1) - B.x(i, j); dy = B.y(i, j + 1) - B.y(i, j); s = std::sqrt(dx * dx + dy * dy);
        n1 = -dy / s; n2 = dx / s;
      } else if (Bc.face == 3) {
        dx = B.x(i, j + 1) - B.x(i, j); dy = B.y(i, j + 1) - B.y(i, j); s = std::sqrt(dx * dx + dy * dy);
        n1 = dy / s; n2 = -dx / s;
      } else if (Bc.face == 2) {
        dx = B.x(i + 1, j) - B.x(i, j); dy = B.y(i + 1, j) - B.y(i, j); s = std::sqrt(dx * dx + dy * dy);
        n1 = dy / s; n2 = -dx / s;
      } else {
        dx = B.x(i + 1, j) - B.x(i, j); dy = B.y(i + 1, j) - B.y(i, j); s = std::sqrt(dx * dx + dy * dy);
        n1 = -dy / s; n2 = dx / s;
      }
      double Ma_n = (u1 * n1 + v1 * n2) / c1;
      for (int k = 1; k <= LAP; k++) {
        int i2, j2;
        if (Bc.face == 1) { i2 = i - k; j2 = j; }
        else if (Bc.face == 2) { i2 = i; j2 = j - k; }
        else if (Bc.face == 3) { i2 = i + k - 1; j2 = j; }
        else { i2 = i; j2 = j + k - 1; }
        if (Bctype == BC_Outlet || (Bctype == BC_Farfield && Ma_n >= 0.0)) {
          if (Ma_n > 1.0 || S.p_outlet < 0 || Bctype == BC_Farfield) {
            for (int m = 1; m <= MP.Nvar; m++) B.U(m, i2, j2) = B.U(m, i1, j1);
          } else {
            double pb = S.p_outlet;
            double db = d1 + (S.p_outlet - p1) / (c1 * c1);
            double ub = u1 + (p1 - S.p_outlet) / (d1 * c1) * n1;
            double vb = v1 + (p1 - S.p_outlet) / (d1 * c1) * n2;
            double p2 = 2.0 * pb - p1, d2 = 2.0 * db - d1, u2 = 2.0 * ub - u1, v2 = 2.0 * vb - v1;
            B.U(1, i2, j2) = d2; B.U(2, i2, j2) = d2 * u2; B.U(3, i2, j2) = d2 * v2;
            B.U(4, i2, j2) = p2 / (gamma - 1.0) + 0.5 * d2 * (u2 * u2 + v2 * v2);
            for (int m = 5; m <= MP.Nvar; m++) B.U(m, i2, j2) = B.U(m, i1, j1);
          }
        } else {
          if (S.p_outlet < 0 || Ma_n <= -1.0) {
            B.U(1, i2, j2) = d_inf; B.U(2, i2, j2) = d_inf * u_inf; B.U(3, i2, j2) = d_inf * v_inf;
            B.U(4, i2, j2) = p_inf / (gamma - 1.0) + 0.5 * d_inf * (u_inf * u_inf + v_inf * v_inf);
          } else {
            double pb = 0.5 * (p1 + p_inf - d1 * c1 * ((u_inf - u1) * n1 + (v_inf - v1) * n2));
            double db = d_inf + (pb - p_inf) / (c1 * c1);
            double ub = u_inf - (p_inf - pb) / (d1 * c1) * n1;
            double vb = v_inf - (p_inf - pb) / (d1 * c1) * n2;
            double p2 = 2.0 * pb - p1, d2 = 2.0 * db - d1, u2 = 2.0 * ub - u1, v2 = 2.0 * vb - v1;
            B.U(1, i2, j2) = d2; B.U(2, i2, j2) = d2 * u2; B.U(3, i2, j2) = d2 * v2;
            B.U(4, i2, j2) = p2 / (gamma - 1.0) + 0.5 * d2 * (u2 * u2 + v2 * v2);
          }
          if (MP.Nvar == 5) B.U(5, i2, j2) = S.vt_inf / S.Re;
          else if (MP.Nvar == 6) { B.U(5, i2, j2) = d_inf * S.Kt_inf; B.U(6, i2, j2) = d_inf * S.Wt_inf; }
        }
      }
    }
}

// Boundary_condition_onemesh, sub_boundary.f90:10-34
void boundary_condition_onemesh(Solver &S, int nMesh) {
  Mesh &MP = S.mesh[nMesh];
  for (auto &B : MP.B)
    for (auto &Bc : B.bc) {
      if (Bc.neighb >= 0) continue;
      if (Bc.neighb == BC_Wall) boundary_wall(S, nMesh, B, Bc);
      else if (Bc.neighb == BC_Farfield || Bc.neighb == BC_Inlet || Bc.neighb == BC_Outlet)
        boundary_farfield(S, nMesh, B, Bc, Bc.neighb);
      else if (Bc.neighb == BC_Symmetry) symmetry_or_slidewall(S, nMesh, B, Bc);
    }
}

// U_average_conner, sub_boundary.f90:595-612
void u_average_conner(int nv, double *U1, double *U2, double *U3, double *U4, double Cv) {
  double d1 = U1[0], uu1 = U1[1] / d1, v1 = U1[2] / d1, T1 = (U1[3] - (uu1 * U1[1] + v1 * U1[2]) * 0.5) / (d1 * Cv);
  double d2 = U2[0], uu2 = U2[1] / d2, v2 = U2[2] / d2, T2 = (U2[3] - (uu2 * U2[1] + v2 * U2[2]) * 0.5) / (d2 * Cv);
  double d3 = U3[0], uu3 = U3[1] / d3, v3 = U3[2] / d3, T3 = (U3[3] - (uu3 * U3[1] + v3 * U3[2]) * 0.5) / (d3 * Cv);
  double d4 = d1 + d3 - d2, uu4 = uu1 + uu3 - uu2, v4 = v1 + v3 - v2, T4 = T1 + T3 - T2;
  U4[0] = d4; U4[1] = d4 * uu4; U4[2] = d4 * v4; U4[3] = d4 * (Cv * T4 + (uu4 * uu4 + v4 * v4) * 0.5);
  if (nv == 5) U4[4] = U1[4] + U3[4] - U2[4];
  if (nv == 6) { U4[4] = U1[4] + U3[4] - U2[4]; U4[5] = U1[5] + U3[5] - U2[5]; }
}

// update_buffer_onemesh, sub_boundary.f90:45-153
void update_buffer_onemesh(Solver &S, int nMesh) {
  Mesh &MP = S.mesh[nMesh];
  int nv = MP.Nvar;
  for (auto &B : MP.B) {
    for (auto &Bc : B.bc) {
      if (Bc.neighb < 0) continue;
      int ib2 = Bc.ist, ie2 = Bc.iend, jb2 = Bc.jst, je2 = Bc.jend;
      int n1 = ie2 - ib2 + je2 - jb2;
      std::vector<double> Ua((size_t)nv * n1 * LAP);
      auto UA = [&](int k, int l) { return &Ua[(size_t)nv * ((k - 1) + (size_t)n1 * (l - 1))]; };
      Block &B1 = MP.B[Bc.neighb - 1];
      BcMsg &Bc1 = B1.bc[Bc.subface - 1];
      int ib1 = Bc1.ist, ie1 = Bc1.iend, jb1 = Bc1.jst, je1 = Bc1.jend;
      if (Bc1.face == 1) {
        for (int j = jb1; j <= je1 - 1; j++)
          for (int l = 1; l <= LAP; l++) std::memcpy(UA(j - jb1 + 1, l), B1.U.col(ib1 + l - 1, j), nv * sizeof(double));
      } else if (Bc1.face == 2) {
        for (int l = 1; l <= LAP; l++)
          for (int i = ib1; i <= ie1 - 1; i++) std::memcpy(UA(i - ib1 + 1, l), B1.U.col(i, jb1 + l - 1), nv * sizeof(double));
      } else if (Bc1.face == 3) {
        for (int j = jb1; j <= je1 - 1; j++)
          for (int l = 1; l <= LAP; l++) std::memcpy(UA(j - jb1 + 1, l), B1.U.col(ie1 - LAP - 1 + l, j), nv * sizeof(double));
      } else {
        for (int l = 1; l <= LAP; l++)
          for (int i = ib1; i <= ie1 - 1; i++) std::memcpy(UA(i - ib1 + 1, l), B1.U.col(i, je1 - LAP - 1 + l), nv * sizeof(double));
      }
      for (int k = 1; k <= n1; k++) {
        int k1 = (Bc.orient == 2) ? k : n1 + 1 - k;
        for (int l = 1; l <= LAP; l++) {
          double *dst;
          if (Bc.face == 1) dst = B.U.col(ib2 - LAP - 1 + l, jb2 + k - 1);
          else if (Bc.face == 2) dst = B.U.col(ib2 + k - 1, jb2 - LAP - 1 + l);
          else if (Bc.face == 3) dst = B.U.col(ie2 + l - 1, jb2 + k - 1);
          else dst = B.U.col(ib2 + k - 1, je2 + l - 1);
          std::memcpy(dst, UA(k1, l), nv * sizeof(double));
        }
      }
    }
    int nx1 = B.nx, ny1 = B.ny;
    u_average_conner(nv, B.U.col(1, 0), B.U.col(1, 1), B.U.col(0, 1), B.U.col(0, 0), S.Cv);
    u_average_conner(nv, B.U.col(1, ny1), B.U.col(1, ny1 - 1), B.U.col(0, ny1 - 1), B.U.col(0, ny1), S.Cv);
    u_average_conner(nv, B.U.col(nx1 - 1, 0), B.U.col(nx1 - 1, 1), B.U.col(nx1, 1), B.U.col(nx1, 0), S.Cv);
    u_average_conner(nv, B.U.col(nx1 - 1, ny1), B.U.col(nx1 - 1, ny1 - 1), B.U.col(nx1, ny1 - 1), B.U.col(nx1, ny1), S.Cv);
  }
}

// ---- reconstruction: sub_Residual.f90:477-659 -----------------------------
inline double minmod(double a, double b) {
  if (a * b <= 0.0) return 0.0;
  if (std::fabs(a) <= std::fabs(b)) return a;
  return b;
}
// scheme_fP, sub_Residual.f90:591-623
double scheme_fP(double u1, double u2, double u3, double u4, int flag) {
  const double k = 1.0, b = 2.0, k3 = 1.0 / 3.0, ep = 1.0e-6;
  double UL = 0.0;
  if (flag == Scheme_UD1) UL = u2;
  else if (flag == Scheme_UD3) UL = (-u1 + 5.0 * u2 + 2.0 * u3) / 6.0;
  else if (flag == Scheme_NND2) UL = u2 + 0.5 * minmod(u2 - u1, u3 - u2);
  else if (flag == Scheme_WENO3) {
    double IS1 = (u2 - u1) * (u2 - u1), IS2 = (u3 - u2) * (u3 - u2);
    double a1 = 1.0 / (3.0 * ((1.0e-6 + IS1) * (1.0e-6 + IS1)));
    double a2 = 2.0 / (3.0 * ((1.0e-6 + IS2) * (1.0e-6 + IS2)));
    double w1 = a1 / (a1 + a2), w2 = a2 / (a1 + a2);
    UL = w1 * (-u1 / 2.0 + 3.0 * u2 / 2.0) + w2 * (u2 / 2.0 + u3 / 2.0);
  } else if (flag == Scheme_MUSCL2) {
    UL = u2 + 0.25 * ((1.0 - k) * minmod(u2 - u1, b * (u3 - u2)) + (1.0 + k) * minmod(u3 - u2, b * (u2 - u1)));
  } else if (flag == Scheme_MUSCL3) {
    double up = u3 - u2, um = u2 - u1;
    double s = (2.0 * up * um + ep) / (up * up + um * um + ep);
    UL = u2 + 0.25 * s * ((1.0 - k3 * s) * um + (1.0 + k3 * s) * up);
  } else if (flag == Scheme_OMUSCL2) {
    double r1 = (u2 - u1 + ep) / (u3 - u2 + ep), r2 = (u3 - u2 + ep) / (u4 - u3 + ep);
    double f1 = 0.8 - 0.175 / r2 + 0.375 * r1;
    double f = std::max(0.0, std::min(std::min(2.0, f1), 2.0 * r1));
    UL = u2 + 0.5 * f * (u3 - u2);
  }
  return UL;
}
// scheme_fm, sub_Residual.f90:626-659
double scheme_fm(double u1, double u2, double u3, double u4, int flag) {
  const double k = 1.0 / 3.0, b = 1.0, k3 = 1.0 / 3.0, ep = 1.0e-6;
  double UR = 0.0;
  if (flag == Scheme_UD1) UR = u3;
  else if (flag == Scheme_UD3) UR = (2.0 * u2 + 5.0 * u3 - u4) / 6.0;
  else if (flag == Scheme_NND2) UR = u3 - 0.5 * minmod(u3 - u2, u4 - u3);
  else if (flag == Scheme_WENO3) {
    double IS1 = (u3 - u4) * (u3 - u4), IS2 = (u2 - u3) * (u2 - u3);
    double a1 = 1.0 / (3.0 * ((1.0e-6 + IS1) * (1.0e-6 + IS1)));
    double a2 = 2.0 / (3.0 * ((1.0e-6 + IS2) * (1.0e-6 + IS2)));
    double w1 = a1 / (a1 + a2), w2 = a2 / (a1 + a2);
    UR = w1 * (-u4 / 2.0 + 3.0 * u3 / 2.0) + w2 * (u3 / 2.0 + u2 / 2.0);
  } else if (flag == Scheme_MUSCL2) {
    UR = u3 - 0.25 * ((1.0 - k) * minmod(u4 - u3, b * (u3 - u2)) + (1.0 + k) * minmod(u3 - u2, b * (u4 - u3)));
  } else if (flag == Scheme_MUSCL3) {
    double up = u4 - u3, um = u3 - u2;
    double s = (2.0 * up * um + ep) / (up * up + um * um + ep);
    UR = u3 - 0.25 * s * ((1.0 - k3 * s) * up + (1.0 + k3 * s) * um);
  } else if (flag == Scheme_OMUSCL2) {
    double r1 = (u4 - u3 + ep) / (u3 - u2 + ep), r2 = (u3 - u2 + ep) / (u2 - u1 + ep);
    double f1 = 0.8 - 0.175 / r2 + 0.375 * r1;
    double f = std::max(0.0, std::min(std::min(2.0, f1), 2.0 * r1));
    UR = u3 - 0.5 * f * (u3 - u2);
  }
  return UR;
}
// U0[k][m]: k = stencil point (i-2,i-1,i,i+1), m = variable
// Reconstuction_original, sub_Residual.f90:505-514
void recon_original(double U0[4][4], double UL[4], double UR[4], int flag) {
  for (int m = 0; m < 4; m++) {
    UL[m] = scheme_fP(U0[0][m], U0[1][m], U0[2][m], U0[3][m], flag);
    UR[m] = scheme_fm(U0[0][m], U0[1][m], U0[2][m], U0[3][m], flag);
  }
}
// Reconstuction_conservative, sub_Residual.f90:517-528
void recon_conservative(double U0[4][4], double UL[4], double UR[4], double gamma, int flag) {
  double QL[4], QR[4];
  for (int m = 0; m < 4; m++) {
    QL[m] = scheme_fP(U0[0][m], U0[1][m], U0[2][m], U0[3][m], flag);
    QR[m] = scheme_fm(U0[0][m], U0[1][m], U0[2][m], U0[3][m], flag);
  }
  UL[0] = QL[0]; UL[1] = QL[1] / UL[0]; UL[2] = QL[2] / UL[0];
  UL[3] = (QL[3] - (UL[1] * QL[1] + UL[2] * QL[2]) * 0.5) * (gamma - 1.0);
  UR[0] = QR[0]; UR[1] = QR[1] / UR[0]; UR[2] = QR[2] / UR[0];
  UR[3] = (QR[3] - (UR[1] * QR[1] + UR[2] * QR[2]) * 0.5) * (gamma - 1.0);
}
// Reconstuction_Characteristic, sub_Residual.f90:531-586
void recon_characteristic(double U0[4][4], double UL[4], double UR[4], double gamma, int flag) {
  double Uh[4];
  for (int m = 0; m < 4; m++) Uh[m] = 0.5 * (U0[1][m] + U0[2][m]);
  double d1 = Uh[0], u1 = Uh[1] / d1, v1 = Uh[2] / d1;
  double p1 = (Uh[3] - (Uh[1] * u1 + Uh[2] * v1) * 0.5) * (gamma - 1.0);
  double c1 = std::sqrt(gamma * p1 / d1);
  double V2 = (u1 * u1 + v1 * v1) * 0.5;
  double tmp1 = (gamma - 1.0) / c1, tmp3 = (gamma - 1.0) / (c1 * c1), tmp5 = 1.0 / (2.0 * c1), tmp0 = 1.0 / tmp3;
  double Sm[4][4] = {{V2 - tmp0, -u1, -v1, 1.0},
                     {-v1, 0.0, 1.0, 0.0},
                     {-u1 - V2 * tmp1, 1.0 + tmp1 * u1, tmp1 * v1, -tmp1},
                     {-u1 + V2 * tmp1, 1.0 - tmp1 * u1, -tmp1 * v1, tmp1}};
  double S1[4][4] = {{-tmp3, 0.0, -tmp5, tmp5},
                     {-tmp3 * u1, 0.0, 0.5 - u1 * tmp5, 0.5 + u1 * tmp5},
                     {-tmp3 * v1, 1.0, -v1 * tmp5, v1 * tmp5},
                     {-tmp3 * V2, v1, (c1 * u1 - V2 - tmp0) * tmp5, (c1 * u1 + V2 + tmp0) * tmp5}};
  double V0[4][4];
  for (int k = 0; k < 4; k++)
    for (int m = 0; m < 4; m++) {
      double s = 0.0;
      for (int j = 0; j < 4; j++) s = s + Sm[m][j] * U0[k][j];
      V0[k][m] = s;
    }
  double VL[4], VR[4], QL[4], QR[4];
  for (int m = 0; m < 4; m++) {
    VL[m] = scheme_fP(V0[0][m], V0[1][m], V0[2][m], V0[3][m], flag);
    VR[m] = scheme_fm(V0[0][m], V0[1][m], V0[2][m], V0[3][m], flag);
  }
  for (int m = 0; m < 4; m++) {
    double a = 0.0, b = 0.0;
    for (int j = 0; j < 4; j++) { a = a + S1[m][j] * VL[j]; b = b + S1[m][j] * VR[j]; }
    QL[m] = a; QR[m] = b;
  }
  UL[0] = QL[0]; UL[1] = QL[1] / UL[0]; UL[2] = QL[2] / UL[0];
  UL[3] = (QL[3] - (UL[1] * QL[1] + UL[2] * QL[2]) * 0.5) * (gamma - 1.0);
  UR[0] = QR[0]; UR[1] = QR[1] / UR[0]; UR[2] = QR[2] / UR[0];
  UR[3] = (QR[3] - (UR[1] * QR[1] + UR[2] * QR[2]) * 0.5) * (gamma - 1.0);
}

// ---- 1-D face fluxes: sub_flux_split.f90 ---------------------------------
// Flux_HLL_HLLC_1D, sub_flux_split.f90:16-93
void flux_hll_hllc(const double *QL, const double *QR, double *Flux, double gamma, int hllc) {
  double dl = QL[0], uul = QL[1], vvl = QL[2], pl = QL[3];
  double dr = QR[0], uur = QR[1], vvr = QR[2], pr = QR[3];
  double UL[4] = {dl, dl * uul, dl * vvl, pl / (gamma - 1.0) + dl * (uul * uul + vvl * vvl) * 0.5};
  double UR[4] = {dr, dr * uur, dr * vvr, pr / (gamma - 1.0) + dr * (uur * uur + vvr * vvr) * 0.5};
  double al = std::sqrt(gamma * pl / dl), ar = std::sqrt(gamma * pr / dr);
  double p_pvrs = 0.5 * (pl + pr) - (uur - uul) * (dl + dr) * (al + ar) * 0.125;
  double p_star = std::max(0.0, p_pvrs);
  double qql, qqr;
  if (p_star <= pl) qql = 1; else qql = std::sqrt(1.0 + ((gamma + 1.0) / (2.0 * gamma)) * (p_star / pl - 1.0));
  if (p_star <= pr) qqr = 1; else qqr = std::sqrt(1.0 + ((gamma + 1.0) / (2.0 * gamma)) * (p_star / pr - 1.0));
  double Sl = uul - al * qql, Sr = uur + ar * qqr;
  double Fl[4] = {UL[1], UL[1] * uul + pl, UL[2] * uul, uul * (UL[3] + pl)};
  double Fr[4] = {UR[1], UR[1] * uur + pr, UR[2] * uur, uur * (UR[3] + pr)};
  if (!hllc) {
    if (Sl >= 0) for (int m = 0; m < 4; m++) Flux[m] = Fl[m];
    else if (Sr <= 0) for (int m = 0; m < 4; m++) Flux[m] = Fr[m];
    else for (int m = 0; m < 4; m++) Flux[m] = (Sr * Fl[m] - Sl * Fr[m] + Sl * Sr * (UR[m] - UL[m])) / (Sr - Sl);
  } else {
    double S_star = (pr - pl + dl * uul * (Sl - uul) - dr * uur * (Sr - uur)) / (dl * (Sl - uul) - dr * (Sr - uur));
    double tmpl = dl * (Sl - uul) / (Sl - S_star), tmpr = dr * (Sr - uur) / (Sr - S_star);
    double Fsl[4], Fsr[4];
    Fsl[0] = Fl[0] + Sl * (tmpl - UL[0]);
    Fsl[1] = Fl[1] + Sl * (tmpl * S_star - UL[1]);
    Fsl[2] = Fl[2] + Sl * (tmpl * vvl - UL[2]);
    double tmp = UL[3] / dl + (S_star - uul) * (S_star + pl / (dl * (Sl - uul)));
    Fsl[3] = Fl[3] + Sl * (tmpl * tmp - UL[3]);
    Fsr[0] = Fr[0] + Sr * (tmpr - UR[0]);
    Fsr[1] = Fr[1] + Sr * (tmpr * S_star - UR[1]);
    Fsr[2] = Fr[2] + Sr * (tmpr * vvr - UR[2]);
    tmp = UR[3] / dr + (S_star - uur) * (S_star + pr / (dr * (Sr - uur)));
    Fsr[3] = Fr[3] + Sr * (tmpr * tmp - UR[3]);
    const double *F = (Sl >= 0) ? Fl : (Sr <= 0) ? Fr : (S_star >= 0) ? Fsl : Fsr;
    for (int m = 0; m < 4; m++) Flux[m] = F[m];
  }
}
// Flux_steger_warming_1Da, sub_flux_split.f90:99-136
void flux_steger_warming(const double *QL, const double *QR, double *Flux, double gamma) {
  double dl = QL[0], uul = QL[1], vvl = QL[2], pl = QL[3];
  double dr = QR[0], uur = QR[1], vvr = QR[2], pr = QR[3];
  double al = std::sqrt(gamma * pl / dl), ar = std::sqrt(gamma * pr / dr);
  double tmp1 = 2.0 * (gamma - 1.0), tmp3 = (3.0 - gamma) / (2.0 * (gamma - 1.0));
  double E1P = (uul + std::fabs(uul)) * 0.5, E2P = (uul - al + std::fabs(uul - al)) * 0.5,
         E3P = (uul + al + std::fabs(uul + al)) * 0.5;
  double tmp0 = dl / (2.0 * gamma);
  double fp[4], fm[4];
  fp[0] = tmp0 * (tmp1 * E1P + E2P + E3P);
  fp[1] = tmp0 * (tmp1 * E1P * uul + E2P * (uul - al) + E3P * (uul + al));
  fp[2] = tmp0 * (tmp1 * E1P * vvl + E2P * vvl + E3P * vvl);
  fp[3] = tmp0 * (E1P * (gamma - 1.0) * (uul * uul + vvl * vvl) + E2P * ((uul - al) * (uul - al) + vvl * vvl) * 0.5 +
                  E3P * ((uul + al) * (uul + al) + vvl * vvl) * 0.5 + tmp3 * al * al * (E2P + E3P));
  double E1M = (uur - std::fabs(uur)) * 0.5, E2M = (uur - ar - std::fabs(uur - ar)) * 0.5,
         E3M = (uur + ar - std::fabs(uur + ar)) * 0.5;
  tmp0 = dr / (2.0 * gamma);
  fm[0] = tmp0 * (tmp1 * E1M + E2M + E3M);
  fm[1] = tmp0 * (tmp1 * E1M * uur + E2M * (uur - ar) + E3M * (uur + ar));
  fm[2] = tmp0 * (tmp1 * E1M * vvr + E2M * vvr + E3M * vvr);
  fm[3] = tmp0 * (E1M * (gamma - 1.0) * (uur * uur + vvr * vvr) + E2M * ((uur - ar) * (uur - ar) + vvr * vvr) * 0.5 +
                  E3M * ((uur + ar) * (uur + ar) + vvr * vvr) * 0.5 + tmp3 * ar * ar * (E2M + E3M));
  for (int m = 0; m < 4; m++) Flux[m] = fp[m] + fm[m];
}
// Flux_Van_Leer_1Da, sub_flux_split.f90:139-189
void flux_van_leer(const double *QL, const double *QR, double *Flux, double gamma) {
  double dl = QL[0], uul = QL[1], vvl = QL[2], pl = QL[3];
  double dr = QR[0], uur = QR[1], vvr = QR[2], pr = QR[3];
  double al = std::sqrt(gamma * pl / dl), ar = std::sqrt(gamma * pr / dr);
  double Ml = uul / al, Mr = uur / ar;
  double fp[4] = {0, 0, 0, 0}, fm[4] = {0, 0, 0, 0};
  if (Ml >= 1.0) {
    fp[0] = dl * uul; fp[1] = dl * uul * uul + pl; fp[2] = dl * uul * vvl;
    fp[3] = uul * (gamma * pl / (gamma - 1.0) + 0.5 * dl * (uul * uul + vvl * vvl));
  } else if (std::fabs(Ml) < 1.0) {
    double Mp = 0.25 * (1.0 + Ml) * (1.0 + Ml);
    double tmp0 = dl * al * Mp;
    fp[0] = tmp0;
    fp[1] = tmp0 * ((gamma - 1.0) * uul + 2.0 * al) / gamma;
    fp[2] = tmp0 * vvl;
    fp[3] = tmp0 * (((gamma - 1.0) * uul + 2.0 * al) * ((gamma - 1.0) * uul + 2.0 * al) * 0.5 / (gamma * gamma - 1.0) + 0.5 * (vvl * vvl));
  }
  if (Mr >= 1.0) {
  } else if (std::fabs(Mr) < 1.0) {
    double Mm = -0.25 * (Mr - 1.0) * (Mr - 1.0);
    double tmp0 = dr * ar * Mm;
    fm[0] = tmp0;
    fm[1] = tmp0 * ((gamma - 1.0) * uur - 2.0 * ar) / gamma;
    fm[2] = tmp0 * vvr;
    fm[3] = tmp0 * (((gamma - 1.0) * uur - 2.0 * ar) * ((gamma - 1.0) * uur - 2.0 * ar) * 0.5 / (gamma * gamma - 1.0) + 0.5 * (vvr * vvr));
  } else if (Mr <= -1.0) {
    fm[0] = dr * uur; fm[1] = dr * uur * uur + pr; fm[2] = dr * uur * vvr;
    fm[3] = uur * (gamma * pr / (gamma - 1.0) + 0.5 * dr * (uur * uur + vvr * vvr));
  }
  for (int m = 0; m < 4; m++) Flux[m] = fp[m] + fm[m];
}
// Flux_Ausm_1Da (AUSM+), sub_flux_split.f90:195-261
void flux_ausm(const double *QL, const double *QR, double *Flux, double gamma) {
  double dl = QL[0], uul = QL[1], vvl = QL[2], pl = QL[3];
  double dr = QR[0], uur = QR[1], vvr = QR[2], pr = QR[3];
  double hl = gamma * pl / ((gamma - 1.0) * dl) + 0.5 * (uul * uul + vvl * vvl);
  double hr = gamma * pr / ((gamma - 1.0) * dr) + 0.5 * (uur * uur + vvr * vvr);
  double al = std::sqrt(gamma * pl / dl), ar = std::sqrt(gamma * pr / dr);
  double a = 0.5 * (al + ar);
  double Ml = uul / a, Mr = uur / a;
  double Mp4, Mm4, Pp5, Pm5;
  if (std::fabs(Ml) >= 1.0) Mp4 = 0.5 * (Ml + std::fabs(Ml));
  else Mp4 = 0.25 * (Ml + 1.0) * (Ml + 1.0) + 0.125 * (Ml * Ml - 1.0) * (Ml * Ml - 1.0);
  if (std::fabs(Mr) >= 1.0) Mm4 = 0.5 * (Mr - std::fabs(Mr));
  else Mm4 = -0.25 * (Mr - 1.0) * (Mr - 1.0) - 0.125 * (Mr * Mr - 1.0) * (Mr * Mr - 1.0);
  double M = Mp4 + Mm4;
  double mp = dl * a * std::max(0.0, M), mm = dr * a * std::min(0.0, M);
  double xm = mp + mm;
  double dm = (M >= 0.0) ? a * std::fabs(M) * dl : a * std::fabs(M) * dr;
  if (std::fabs(Ml) >= 1.0) Pp5 = 0.5 * (Ml + std::fabs(Ml)) / Ml;
  else Pp5 = 0.25 * (Ml + 1.0) * (Ml + 1.0) * (2.0 - Ml) + 3.0 * Ml * (Ml * Ml - 1.0) * (Ml * Ml - 1.0) / 16.0;
  if (std::fabs(Mr) >= 1.0) Pm5 = 0.5 * (Mr - std::fabs(Mr)) / Mr;
  else Pm5 = 0.25 * (Mr - 1.0) * (Mr - 1.0) * (2.0 + Mr) - 3.0 * Mr * (Mr * Mr - 1.0) * (Mr * Mr - 1.0) / 16.0;
  double p = pl * Pp5 + pr * Pm5;
  double fp[4] = {1.0, uul, vvl, hl}, fm[4] = {1.0, uur, vvr, hr};
  Flux[0] = 0.5 * xm * (fp[0] + fm[0]) - 0.5 * dm * (fm[0] - fp[0]);
  Flux[1] = 0.5 * xm * (fp[1] + fm[1]) - 0.5 * dm * (fm[1] - fp[1]) + p;
  Flux[2] = 0.5 * xm * (fp[2] + fm[2]) - 0.5 * dm * (fm[2] - fp[2]);
  Flux[3] = 0.5 * xm * (fp[3] + fm[3]) - 0.5 * dm * (fm[3] - fp[3]);
}
// Flux_Roe_1D, sub_flux_split.f90:265-324
void flux_roe(const double *QL, const double *QR, double *Flux, double gamma) {
  const double delt = 0.1;
  double dl = QL[0], uul = QL[1], vvl = QL[2], pl = QL[3];
  double dr = QR[0], uur = QR[1], vvr = QR[2], pr = QR[3];
  double hl = gamma * pl / ((gamma - 1.0) * dl) + 0.5 * (uul * uul + vvl * vvl);
  double hr = gamma * pr / ((gamma - 1.0) * dr) + 0.5 * (uur * uur + vvr * vvr);
  double Fl[4] = {dl * uul, dl * uul * uul + pl, dl * uul * vvl, uul * dl * hl};
  double Fr[4] = {dr * uur, dr * uur * uur + pr, dr * uur * vvr, uur * dr * hr};
  double tmpp = std::sqrt(dr / dl);
  double avd = 0.25 * dl * (1.0 + tmpp) * (1.0 + tmpp);
  double avu = (uul + tmpp * uur) / (1.0 + tmpp);
  double avv = (vvl + tmpp * vvr) / (1.0 + tmpp);
  double avh = (hl + tmpp * hr) / (1.0 + tmpp);
  double ava = std::sqrt((gamma - 1.0) * (avh - 0.5 * (avu * avu + avv * avv)));
  double lam[4] = {std::fabs(avu - ava), std::fabs(avu), std::fabs(avu), std::fabs(avu + ava)};
  for (int m = 0; m < 4; m++)
    if (lam[m] < delt) lam[m] = (lam[m] * lam[m] + delt * delt) / (2.0 * delt);
  double arr[4];
  arr[0] = (avd * ava * (-uur + uul) + pr - pl) / (2.0 * ava * ava);
  arr[1] = dr - dl - (pr - pl) / (ava * ava);
  arr[2] = avd * (vvr - vvl) / ava;
  arr[3] = (avd * ava * (uur - uul) + pr - pl) / (2.0 * ava * ava);
  Flux[0] = 0.5 * (Fl[0] + Fr[0]) - 0.5 * (lam[0] * arr[0] + lam[1] * arr[1] + lam[3] * arr[3]);
  Flux[1] = 0.5 * (Fl[1] + Fr[1]) - 0.5 * (lam[0] * arr[0] * (avu - ava) + lam[1] * arr[1] * avu + lam[3] * arr[3] * (avu + ava));
  Flux[2] = 0.5 * (Fl[2] + Fr[2]) - 0.5 * (lam[0] * arr[0] * avv + lam[1] * arr[1] * avv + lam[2] * arr[2] + lam[3] * arr[3] * avv);
  Flux[3] = 0.5 * (Fl[3] + Fr[3]) - 0.5 * (lam[0] * arr[0] * (avh - avu * ava) + lam[1] * arr[1] * 0.5 * (avu * avu + avv * avv) +
                                           lam[2] * arr[2] * avv + lam[3] * arr[3] * (avh + avu * ava));
}
void face_flux(int iflux, const double *QL, const double *QR, double *F, double gamma) {
  if (iflux == Flux_Steger_Warming) flux_steger_warming(QL, QR, F, gamma);
  else if (iflux == Flux_HLL) flux_hll_hllc(QL, QR, F, gamma, 0);
  else if (iflux == Flux_HLLC) flux_hll_hllc(QL, QR, F, gamma, 1);
  else if (iflux == Flux_VanLeer) flux_van_leer(QL, QR, F, gamma);
  else if (iflux == Flux_Ausm) flux_ausm(QL, QR, F, gamma);
  else if (iflux == Flux_Roe) flux_roe(QL, QR, F, gamma);
  else { F[0] = F[1] = F[2] = F[3] = 0.0; }
}

// ---- residual pieces ---------------------------------------------------------
// comput_duvtpckw, sub_Residual.f90:114-152 (STOP on T<1e-5 becomes an error code)
int comput_duvtpckw(Solver &S, Block &B, FlowVar &F, int mb) {
  int nx = B.nx, ny = B.ny;
  double p00 = 1.0 / (S.gamma * S.Ma * S.Ma);
#pragma omp parallel for schedule(static)
  for (int j = 1 - LAP; j <= ny + LAP - 1; j++)
    for (int i = 1 - LAP; i <= nx + LAP - 1; i++) {
      F.d(i, j) = B.U(1, i, j);
      F.uu(i, j) = B.U(2, i, j) / F.d(i, j);
      F.v(i, j) = B.U(3, i, j) / F.d(i, j);
      F.T(i, j) = (B.U(4, i, j) - 0.5 * F.d(i, j) * (F.uu(i, j) * F.uu(i, j) + F.v(i, j) * F.v(i, j))) / (S.Cv * F.d(i, j));
      F.p(i, j) = p00 * F.d(i, j) * F.T(i, j);
    }
  for (int j = 1; j <= ny - 1; j++)
    for (int i = 1; i <= nx - 1; i++) {
      if (F.T(i, j) < 1.0e-5) {
        if (!S.err) { S.err = 2; S.err_b = mb + 1; S.err_i = i; S.err_j = j; }
        return 2;
      }
      F.cc(i, j) = std::sqrt(F.T(i, j)) / S.Ma;
    }
  return 0;
}

// get_viscous, sub_Residual.f90:670-689
void get_viscous(Solver &S, Block &B, FlowVar &F) {
  double Tsb = 110.4 / S.T_inf;
  for (int j = 0; j <= B.ny; j++)
    for (int i = 0; i <= B.nx; i++) {
      double T = F.T(i, j);
      B.Amu(i, j) = 1.0 / S.Re * (1.0 + Tsb) * std::sqrt(T * T * T) / (Tsb + T);
    }
}

// Amut_boundary, sub_turbulence_SA.f90:180-220
void amut_boundary(Block &B) {
  int nx = B.nx, ny = B.ny;
  for (auto &Bc : B.bc) {
    if (Bc.neighb != BC_Wall) continue;
    if (Bc.face == 1) for (int j = Bc.jst; j <= Bc.jend - 1; j++) B.Amu_t(0, j) = -B.Amu_t(1, j);
    else if (Bc.face == 3) for (int j = Bc.jst; j <= Bc.jend - 1; j++) B.Amu_t(nx, j) = -B.Amu_t(nx - 1, j);
    else if (Bc.face == 2) for (int i = Bc.ist; i <= Bc.iend - 1; i++) B.Amu_t(i, 0) = -B.Amu_t(i, 1);
    else if (Bc.face == 4) for (int i = Bc.ist; i <= Bc.iend - 1; i++) B.Amu_t(i, ny) = -B.Amu_t(i, ny - 1);
  }
}

// Turbulence_model_SA, sub_turbulence_SA.f90:4-175
void turbulence_sa(Solver &S, Block &B, FlowVar &F) {
  const double SA_sigma = 2.0 / 3.0, Cv1 = 7.1, Cb1 = 0.1355, Cb2 = 0.622, SA_k = 0.41;
  const double Cw1 = Cb1 / (SA_k * SA_k) + (1.0 + Cb2) / SA_sigma, Cw2 = 0.3, Cw3 = 2.0, Ct3 = 1.3, Ct4 = 0.5;
  const double Cv1_3 = Cv1 * Cv1 * Cv1;
  const double Cw3_6 = Cw3 * Cw3 * Cw3 * Cw3 * Cw3 * Cw3;
  const double c03 = (double)0.3f;  // single-precision literal 0.3 (sub_turbulence_SA.f90:159)
  int nx = B.nx, ny = B.ny;
  A2 vt, Fluxv, fluxv2;
  vt.alloc(0, nx, 0, ny); Fluxv.alloc(1, nx, 1, ny); fluxv2.alloc(1, nx, 1, ny);
  for (int j = 0; j <= ny; j++)
    for (int i = 0; i <= nx; i++) {
      vt(i, j) = B.U(5, i, j);
      double X = F.d(i, j) * vt(i, j) / B.Amu(i, j);
      double fv1 = (X * X * X) / (X * X * X + Cv1_3);
      B.Amu_t(i, j) = fv1 * F.d(i, j) * vt(i, j);
    }
  amut_boundary(B);
  for (int j = 1; j <= ny - 1; j++)
    for (int i = 1; i <= nx; i++) {
      double s0 = B.si(i, j), n1 = B.ni1(i, j), n2 = B.ni2(i, j);
      double vn1 = F.uu(i - 1, j) * n1 + F.v(i - 1, j) * n2, vn2 = F.uu(i, j) * n1 + F.v(i, j) * n2;
      double vfi = -0.5 * ((vn1 + std::fabs(vn1)) * vt(i - 1, j) + (vn2 - std::fabs(vn2)) * vt(i, j)) * s0;
      double v0 = 0.5 * (1.0 + Cb2) / SA_sigma * (vt(i, j) + B.Amu(i, j) / F.d(i, j) + vt(i - 1, j) + B.Amu(i - 1, j) / F.d(i - 1, j));
      double Dix = B.x1(i, j) - B.x1(i - 1, j), Diy = B.y1(i, j) - B.y1(i - 1, j);
      double Djx = (B.x1(i - 1, j + 1) + B.x1(i, j + 1) - B.x1(i - 1, j - 1) - B.x1(i, j - 1)) * 0.25;
      double Djy = (B.y1(i - 1, j + 1) + B.y1(i, j + 1) - B.y1(i - 1, j - 1) - B.y1(i, j - 1)) * 0.25;
      double Ds = 1.0 / (Dix * Djy - Djx * Diy);
      double Div = vt(i, j) - vt(i - 1, j);
      double Djv = (vt(i - 1, j + 1) + vt(i, j + 1) - vt(i - 1, j - 1) - vt(i, j - 1)) * 0.25;
      double vtx = (Div * Djy - Djv * Diy) * Ds, vty = (-Div * Djx + Djv * Dix) * Ds;
      Fluxv(i, j) = vfi + v0 * (vtx * n1 + vty * n2) * s0;
      fluxv2(i, j) = (vtx * n1 + vty * n2) * s0;
    }
  for (int j = 1; j <= ny - 1; j++)
    for (int i = 1; i <= nx - 1; i++) {
      double v0 = (vt(i, j) + B.Amu(i, j) / F.d(i, j)) * Cb2 / SA_sigma;
      B.Res(5, i, j) = Fluxv(i + 1, j) - Fluxv(i, j) - v0 * (fluxv2(i + 1, j) - fluxv2(i, j));
    }
  for (int j = 1; j <= ny; j++)
    for (int i = 1; i <= nx - 1; i++) {
      double s0 = B.sj(i, j), n1 = B.nj1(i, j), n2 = B.nj2(i, j);
      double vn1 = F.uu(i, j - 1) * n1 + F.v(i, j - 1) * n2, vn2 = F.uu(i, j) * n1 + F.v(i, j) * n2;
      double vfi = -0.5 * ((vn1 + std::fabs(vn1)) * vt(i, j - 1) + (vn2 - std::fabs(vn2)) * vt(i, j)) * s0;
      double v0 = 0.5 * (1.0 + Cb2) / SA_sigma * (vt(i, j) + B.Amu(i, j) / F.d(i, j) + vt(i, j - 1) + B.Amu(i, j - 1) / F.d(i, j - 1));
      double Dix = (B.x1(i + 1, j - 1) + B.x1(i + 1, j) - B.x1(i - 1, j - 1) - B.x1(i - 1, j)) * 0.25;
      double Diy = (B.y1(i + 1, j - 1) + B.y1(i + 1, j) - B.y1(i - 1, j - 1) - B.y1(i - 1, j)) * 0.25;
      double Djx = B.x1(i, j) - B.x1(i, j - 1), Djy = B.y1(i, j) - B.y1(i, j - 1);
      double Ds = 1.0 / (Dix * Djy - Djx * Diy);
      double Div = (vt(i + 1, j - 1) + vt(i + 1, j) - vt(i - 1, j - 1) - vt(i - 1, j)) * 0.25;
      double Djv = vt(i, j) - vt(i, j - 1);
      double vtx = (Div * Djy - Djv * Diy) * Ds, vty = (-Div * Djx + Djv * Dix) * Ds;
      Fluxv(i, j) = vfi + v0 * (vtx * n1 + vty * n2) * s0;
      fluxv2(i, j) = (vtx * n1 + vty * n2) * s0;
    }
  for (int j = 1; j <= ny - 1; j++)
    for (int i = 1; i <= nx - 1; i++) {
      double v0 = (vt(i, j) + B.Amu(i, j) / F.d(i, j)) * Cb2 / SA_sigma;
      B.Res(5, i, j) = B.Res(5, i, j) + Fluxv(i, j + 1) - Fluxv(i, j) - v0 * (fluxv2(i, j + 1) - fluxv2(i, j));
    }
  for (int j = 1; j <= ny - 1; j++)
    for (int i = 1; i <= nx - 1; i++) {
      double Dix = (B.x1(i + 1, j) - B.x1(i - 1, j)) * 0.5, Diy = (B.y1(i + 1, j) - B.y1(i - 1, j)) * 0.5;
      double Djx = (B.x1(i, j + 1) - B.x1(i, j - 1)) * 0.5, Djy = (B.y1(i, j + 1) - B.y1(i, j - 1)) * 0.5;
      double Ds = 1.0 / (Dix * Djy - Djx * Diy);
      double Diu = (F.uu(i + 1, j) - F.uu(i - 1, j)) * 0.5, Div = (F.v(i + 1, j) - F.v(i - 1, j)) * 0.5;
      double Dju = (F.uu(i, j + 1) - F.uu(i, j - 1)) * 0.5, Djv = (F.v(i, j + 1) - F.v(i, j - 1)) * 0.5;
      double vx = (Div * Djy - Djv * Diy) * Ds;
      double uy = (-Diu * Djx + Dju * Dix) * Ds;
      double Sv = std::fabs(vx - uy);
      double vtc = vt(i, j), dwc = B.dw(i, j);
      double X = F.d(i, j) * vtc / B.Amu(i, j);
      double fv1 = (X * X * X) / (X * X * X + Cv1_3);
      double fv2 = 1.0 - X / (1.0 + X * fv1);
      double kd = SA_k * dwc;
      double S1 = std::max(Sv + fv2 * vtc / (kd * kd), c03 * Sv);
      double r = std::min(vtc / (S1 * SA_k * SA_k * dwc * dwc), 10.0);
      double r2 = r * r, r6 = r2 * r2 * r2;
      double g = r + Cw2 * (r6 - r);
      double g2 = g * g, g6 = g2 * g2 * g2;
      double fw = g * std::pow((1.0 + Cw3_6) / (g6 + Cw3_6), 1.0 / 6.0);
      double ft2 = Ct3 * std::exp(-Ct4 * X * X);
      double q = vtc / dwc;
      double Q_SA = Cb1 * (1.0 - ft2) * S1 * vtc - (Cw1 * fw - Cb1 * ft2 / (SA_k * SA_k)) * (q * q);
      B.Res(5, i, j) = B.Res(5, i, j) + Q_SA * B.vol(i, j);
    }
}

// SST_kw, sub_turbulence_SST.f90:6-271
void turbulence_sst(Solver &S, Block &B, FlowVar &F) {
  const double sigma_k1 = 0.85, sigma_w1 = 0.5, beta1 = 0.075, Cw1 = 0.533;
  const double sigma_k2 = 1.0, sigma_w2 = 0.856, beta2 = 0.0828, Cw2 = 0.440;
  const double a1 = 0.31, betas = 0.09;
  const double c009 = (double)0.09f;   // single-precision literal (sub_turbulence_SST.f90:87,96)
  const double cap = (double)100000.f; // 100000. (exact)
  int nx = B.nx, ny = B.ny;
  double Re = S.Re;
  A2 Kt, Wt, f1, Qk, Qw, Fk, Fw;
  f1.alloc(1, nx, 1, ny, 0.0); Qk.alloc(1, nx, 1, ny); Qw.alloc(1, nx, 1, ny);
  Kt.alloc(1 - LAP, nx + LAP - 1, 1 - LAP, ny + LAP - 1); Wt.alloc(1 - LAP, nx + LAP - 1, 1 - LAP, ny + LAP - 1);
  Fk.alloc(1, nx, 1, ny); Fw.alloc(1, nx, 1, ny);
  for (int j = 1 - LAP; j <= ny + LAP - 1; j++)
    for (int i = 1 - LAP; i <= nx + LAP - 1; i++) {
      Kt(i, j) = B.U(5, i, j) / F.d(i, j);
      Wt(i, j) = B.U(6, i, j) / F.d(i, j);
    }
  for (int j = 1; j <= ny - 1; j++)
    for (int i = 1; i <= nx - 1; i++) {
      double Dix = (B.x1(i + 1, j) - B.x1(i - 1, j)) * 0.5, Diy = (B.y1(i + 1, j) - B.y1(i - 1, j)) * 0.5;
      double Djx = (B.x1(i, j + 1) - B.x1(i, j - 1)) * 0.5, Djy = (B.y1(i, j + 1) - B.y1(i, j - 1)) * 0.5;
      double Ds = 1.0 / (Dix * Djy - Djx * Diy);
      double Diu = (F.uu(i + 1, j) - F.uu(i - 1, j)) * 0.5, Div = (F.v(i + 1, j) - F.v(i - 1, j)) * 0.5;
      double Dik = (Kt(i + 1, j) - Kt(i - 1, j)) * 0.5, Diw = (Wt(i + 1, j) - Wt(i - 1, j)) * 0.5;
      double Dju = (F.uu(i, j + 1) - F.uu(i, j - 1)) * 0.5, Djv = (F.v(i, j + 1) - F.v(i, j - 1)) * 0.5;
      double Djk = (Kt(i, j + 1) - Kt(i, j - 1)) * 0.5, Djw = (Wt(i, j + 1) - Wt(i, j - 1)) * 0.5;
      double ux = (Diu * Djy - Dju * Diy) * Ds, vx = (Div * Djy - Djv * Diy) * Ds;
      double kx = (Dik * Djy - Djk * Diy) * Ds, wx = (Diw * Djy - Djw * Diy) * Ds;
      double uy = (-Diu * Djx + Dju * Dix) * Ds, vy = (-Div * Djx + Djv * Dix) * Ds;
      double ky = (-Dik * Djx + Djk * Dix) * Ds, wy = (-Diw * Djx + Djw * Dix) * Ds;
      (void)ux; (void)vy;
      B.Amu(i, j) = B.Amu(i, j) * Re;
      double omega = vx - uy;
      double dwc = B.dw(i, j), dc = F.d(i, j), K = Kt(i, j), W = Wt(i, j);
      double arg2 = std::max(2.0 * std::sqrt(std::fabs(K)) / (c009 * W * dwc * Re),
                             500.0 * B.Amu(i, j) / (dc * W * (dwc * dwc) * (Re * Re)));
      double f2 = std::tanh(arg2 * arg2);
      B.Amu_t(i, j) = std::min(std::min(dc * K / W, a1 * dc * K * Re / (f2 * std::fabs(omega))), cap);
      double Kws = 2.0 * (kx * wx + ky * wy) * dc * sigma_w2 / (W + 1.0e-20);
      double CD_kw = std::max(Kws, 1.0e-20);
      double arg3 = std::max(std::sqrt(std::fabs(K)) / (c009 * W * dwc * Re),
                             500.0 * B.Amu(i, j) / (dc * W * (dwc * dwc) * (Re * Re)));
      double arg1 = std::min(arg3, 4.0 * dc * sigma_w2 * K / (CD_kw * (dwc * dwc)));
      double a1s = arg1 * arg1;
      f1(i, j) = std::tanh(a1s * a1s);
      double Pk = B.Amu_t(i, j) * omega * omega;
      double Pk0 = std::min(Pk, 20.0 * betas * K * W * (Re * Re));
      Qk(i, j) = Pk0 / Re - betas * dc * W * K * Re;
      double Cw = f1(i, j) * Cw1 + (1.0 - f1(i, j)) * Cw2;
      double beta = f1(i, j) * beta1 + (1.0 - f1(i, j)) * beta2;
      Qw(i, j) = Cw * dc * omega * omega / Re - beta * dc * (W * W) * Re + (1.0 - f1(i, j)) * Kws / Re;
    }
  for (int j = 1; j <= ny - 1; j++)
    for (int i = 1; i <= nx; i++) {
      double si = B.si(i, j), ni1 = B.ni1(i, j), ni2 = B.ni2(i, j);
      double un1 = F.uu(i - 1, j) * ni1 + F.v(i - 1, j) * ni2, un2 = F.uu(i, j) * ni1 + F.v(i, j) * ni2;
      Fk(i, j) = -0.5 * ((un1 + std::fabs(un1)) * Kt(i - 1, j) + (un2 - std::fabs(un2)) * Kt(i, j)) * si;
      Fw(i, j) = -0.5 * ((un1 + std::fabs(un1)) * Wt(i - 1, j) + (un2 - std::fabs(un2)) * Wt(i, j)) * si;
      double sk = f1(i, j) * sigma_k1 + (1.0 - f1(i, j)) * sigma_k2;
      double sw = f1(i, j) * sigma_w1 + (1.0 - f1(i, j)) * sigma_w2;
      double Amu1, Amu2;
      if (i == 1) { Amu1 = B.Amu(i, j) + sk * B.Amu_t(i, j); Amu2 = B.Amu(i, j) + sw * B.Amu_t(i, j); }
      else if (i == nx) { Amu1 = B.Amu(i - 1, j) + sk * B.Amu_t(i - 1, j); Amu2 = B.Amu(i - 1, j) + sw * B.Amu_t(i - 1, j); }
      else {
        Amu1 = (B.Amu(i - 1, j) + B.Amu(i, j) + sk * (B.Amu_t(i - 1, j) + B.Amu_t(i, j))) * 0.5;
        Amu2 = (B.Amu(i - 1, j) + B.Amu(i, j) + sw * (B.Amu_t(i - 1, j) + B.Amu_t(i, j))) * 0.5;
      }
      double Dix = B.x1(i, j) - B.x1(i - 1, j), Diy = B.y1(i, j) - B.y1(i - 1, j);
      double Djx = (B.x1(i - 1, j + 1) + B.x1(i, j + 1) - B.x1(i - 1, j - 1) - B.x1(i, j - 1)) * 0.25;
      double Djy = (B.y1(i - 1, j + 1) + B.y1(i, j + 1) - B.y1(i - 1, j - 1) - B.y1(i, j - 1)) * 0.25;
      double Ds = 1.0 / (Dix * Djy - Djx * Diy);
      double Dik = Kt(i, j) - Kt(i - 1, j), Diw = Wt(i, j) - Wt(i - 1, j);
      double Djk = (Kt(i - 1, j + 1) + Kt(i, j + 1) - Kt(i - 1, j - 1) - Kt(i, j - 1)) * 0.25;
      double Djw = (Wt(i - 1, j + 1) + Wt(i, j + 1) - Wt(i - 1, j - 1) - Wt(i, j - 1)) * 0.25;
      double Kx = (Dik * Djy - Djk * Diy) * Ds, Wx = (Diw * Djy - Djw * Diy) * Ds;
      double Ky = (-Dik * Djx + Djk * Dix) * Ds, Wy = (-Diw * Djx + Djw * Dix) * Ds;
      Fk(i, j) = Fk(i, j) + Amu1 * (Kx * ni1 + Ky * ni2) * si / Re;
      Fw(i, j) = Fw(i, j) + Amu2 * (Wx * ni1 + Wy * ni2) * si / Re;
    }
  for (int j = 1; j <= ny - 1; j++)
    for (int i = 1; i <= nx - 1; i++) {
      B.Res(5, i, j) = Fk(i + 1, j) - Fk(i, j);
      B.Res(6, i, j) = Fw(i + 1, j) - Fw(i, j);
    }
  for (int j = 1; j <= ny; j++)
    for (int i = 1; i <= nx - 1; i++) {
      double sj = B.sj(i, j), nj1 = B.nj1(i, j), nj2 = B.nj2(i, j);
      double un1 = F.uu(i, j - 1) * nj1 + F.v(i, j - 1) * nj2, un2 = F.uu(i, j) * nj1 + F.v(i, j) * nj2;
      Fk(i, j) = -0.5 * ((un1 + std::fabs(un1)) * Kt(i, j - 1) + (un2 - std::fabs(un2)) * Kt(i, j)) * sj;
      Fw(i, j) = -0.5 * ((un1 + std::fabs(un1)) * Wt(i, j - 1) + (un2 - std::fabs(un2)) * Wt(i, j)) * sj;
      double sk = f1(i, j) * sigma_k1 + (1.0 - f1(i, j)) * sigma_k2;
      double sw = f1(i, j) * sigma_w1 + (1.0 - f1(i, j)) * sigma_w2;
      double Amu1, Amu2;
      if (j == 1) { Amu1 = B.Amu(i, j) + sk * B.Amu_t(i, j); Amu2 = B.Amu(i, j) + sw * B.Amu_t(i, j); }
      else if (j == ny) { Amu1 = B.Amu(i, j - 1) + sk * B.Amu_t(i, j - 1); Amu2 = B.Amu(i, j - 1) + sw * B.Amu_t(i, j - 1); }
      else {
        Amu1 = (B.Amu(i, j) + B.Amu(i, j - 1) + sk * (B.Amu_t(i, j) + B.Amu_t(i, j - 1))) * 0.5;
        Amu2 = (B.Amu(i, j) + B.Amu(i, j - 1) + sw * (B.Amu_t(i, j) + B.Amu_t(i, j - 1))) * 0.5;
      }
      double Dix = (B.x1(i + 1, j - 1) + B.x1(i + 1, j) - B.x1(i - 1, j - 1) - B.x1(i - 1, j)) * 0.25;
      double Diy = (B.y1(i + 1, j - 1) + B.y1(i + 1, j) - B.y1(i - 1, j - 1) - B.y1(i - 1, j)) * 0.25;
      double Djx = B.x1(i, j) - B.x1(i, j - 1), Djy = B.y1(i, j) - B.y1(i, j - 1);
      double Ds = 1.0 / (Dix * Djy - Djx * Diy);
      double Dik = (Kt(i + 1, j - 1) + Kt(i + 1, j) - Kt(i - 1, j - 1) - Kt(i - 1, j)) * 0.25;
      double Diw = (Wt(i + 1, j - 1) + Wt(i + 1, j) - Wt(i - 1, j - 1) - Wt(i - 1, j)) * 0.25;
      double Djk = Kt(i, j) - Kt(i, j - 1), Djw = Wt(i, j) - Wt(i, j - 1);
      double Kx = (Dik * Djy - Djk * Diy) * Ds, Wx = (Diw * Djy - Djw * Diy) * Ds;
      double Ky = (-Dik * Djx + Djk * Dix) * Ds, Wy = (-Diw * Djx + Djw * Dix) * Ds;
      Fk(i, j) = Fk(i, j) + Amu1 * (Kx * nj1 + Ky * nj2) * sj / Re;
      Fw(i, j) = Fw(i, j) + Amu2 * (Wx * nj1 + Wy * nj2) * sj / Re;
    }
  for (int j = 1; j <= ny - 1; j++)
    for (int i = 1; i <= nx - 1; i++) {
      B.Res(5, i, j) = B.Res(5, i, j) + Fk(i, j + 1) - Fk(i, j) + Qk(i, j) * B.vol(i, j);
      B.Res(6, i, j) = B.Res(6, i, j) + Fw(i, j + 1) - Fw(i, j) + Qw(i, j) * B.vol(i, j);
      B.Amu(i, j) = B.Amu(i, j) / Re;
      B.Amu_t(i, j) = B.Amu_t(i, j) / Re;
    }
  amut_boundary(B);
}

// BL_model_1d, sub_turbulence_BL.f90:211-273 (1-based arrays of length ny)
void bl_model_1d(int ny, const double *yy, const double *Amu, double *Amu_t, const double *d,
                 const double *u, const double *v, const double *omiga) {
  const double AP = (double)26.f, Ccp = (double)1.6f, Ckleb = (double)0.3f, Cwk = 0.25,
               AKT = (double)0.4f, AK = (double)0.0168f;
  auto Y = [&](int j) { return yy[j - 1]; };
  double Tw = std::fabs(Amu[0] * omiga[0]);
  for (int j = 1; j <= ny - 1; j++)
    if (std::fabs(Amu[j - 1] * omiga[j - 1]) > Tw) Tw = std::fabs(Amu[j - 1] * omiga[j - 1]);
  double Ret = std::sqrt(d[0] * Tw) / Amu[0];
  double Fmax = 0.0, etamax = 0.0, Udif = 0.0;
  int Nb = ny - 1;
  for (int j = 1; j <= Nb; j++) {
    double uu = std::sqrt(u[j - 1] * u[j - 1] + v[j - 1] * v[j - 1]);
    if (uu > Udif) Udif = uu;
    double etap = Y(j) * Ret;
    double FF = Y(j) * std::fabs(omiga[j - 1]) * (1.0 - std::exp(-etap / AP));
    if (FF > Fmax) { Fmax = FF; etamax = Y(j); }
  }
  int Iflag = 0;
  double Fwak = std::min(etamax * Fmax, Cwk * etamax * Udif * Udif / Fmax);
  for (int j = 1; j <= ny - 1; j++) {
    double etap = Ret * Y(j);
    double bl = AKT * Y(j) * (1.0 - std::exp(-etap / AP));
    double visti = d[j - 1] * bl * bl * std::fabs(omiga[j - 1]);
    double r = Ckleb * Y(j) / etamax;
    double r2 = r * r, r6 = r2 * r2 * r2;
    double Fkleb = 1.0 / (1.0 + 5.5 * r6);
    double visto = AK * Ccp * d[j - 1] * Fwak * Fkleb;
    if (std::fabs(visto) < std::fabs(visti)) Iflag = 1;
    Amu_t[j - 1] = (Iflag == 0) ? visti : visto;
  }
}

// turbulence_model_BL, sub_turbulence_BL.f90:6-205
void turbulence_bl(Solver &S, Block &B, FlowVar &F) {
  (void)S;
  int nx1 = B.nx, ny1 = B.ny;
  bool has_wall = false;
  for (auto &c : B.bc) if (c.neighb == BC_Wall) has_wall = true;
  if (!has_wall) return;
  A2 omiga, flag1;
  omiga.alloc(0, nx1, 0, ny1, 0.0); flag1.alloc(0, nx1, 0, ny1, 0.0);
  for (int j = 0; j < (int)B.Amu_t.v.size(); j++) B.Amu_t.v[j] = 0.0;
  for (int j = 1; j <= ny1 - 1; j++)
    for (int i = 1; i <= nx1 - 1; i++) {
      double xi = B.x1(i + 1, j) - B.x1(i - 1, j), yi = B.y1(i + 1, j) - B.y1(i - 1, j);
      double xj = B.x1(i, j + 1) - B.x1(i, j - 1), yj = B.y1(i, j + 1) - B.y1(i, j - 1);
      double Jac = 1.0 / (xi * yj - xj * yi);
      double iy = -Jac * xj, jx = -Jac * yi, ix = Jac * yj, jy = Jac * xi;
      double ui = F.uu(i + 1, j) - F.uu(i - 1, j), vi = F.v(i + 1, j) - F.v(i - 1, j);
      double uj = F.uu(i, j + 1) - F.uu(i, j - 1), vj = F.v(i, j + 1) - F.v(i, j - 1);
      double vx = vi * ix + vj * jx, uy = ui * iy + uj * jy;
      omiga(i, j) = std::fabs(vx - uy);
    }
  for (auto &Bc : B.bc) {
    if (Bc.neighb != BC_Wall) continue;
    if (Bc.face == 1 || Bc.face == 3) {
      std::vector<double> yy(nx1, 0), Amu1d(nx1, 0), Amut1d(nx1, 0), d1d(nx1, 0), u1d(nx1, 0), v1d(nx1, 0), om(nx1, 0);
      for (int j = Bc.jst; j <= Bc.jend - 1; j++) {
        double x0, y0;
        if (Bc.face == 1) { x0 = (B.x1(1, j) + B.x1(0, j)) * 0.5; y0 = (B.y1(1, j) + B.y1(0, j)) * 0.5; }
        else { x0 = (B.x1(nx1 - 1, j) + B.x1(nx1, j)) * 0.5; y0 = (B.y1(nx1 - 1, j) + B.y1(nx1, j)) * 0.5; }
        for (int i = 1; i <= nx1 - 1; i++) {
          int i1 = (Bc.face == 1) ? i : nx1 - i;
          double dx = B.x1(i, j) - x0, dy = B.y1(i, j) - y0;
          yy[i1 - 1] = std::sqrt(dx * dx + dy * dy);
          u1d[i1 - 1] = F.uu(i, j); v1d[i1 - 1] = F.v(i, j); d1d[i1 - 1] = F.d(i, j); om[i1 - 1] = omiga(i, j);
          Amu1d[i1 - 1] = B.Amu(i, j);
        }
        bl_model_1d(nx1, yy.data(), Amu1d.data(), Amut1d.data(), d1d.data(), u1d.data(), v1d.data(), om.data());
        for (int i = 1; i <= nx1 - 1; i++) {
          int i1 = (Bc.face == 1) ? i : nx1 - i;
          if (flag1(i, j) == 0) { flag1(i, j) = 1; B.Amu_t(i, j) = Amut1d[i1 - 1]; }
          else B.Amu_t(i, j) = std::min(B.Amu_t(i, j), Amut1d[i1 - 1]);
        }
      }
      for (int i = 1 - LAP; i <= nx1 + LAP - 1; i++) { B.Amu_t(i, Bc.jst - 1) = B.Amu_t(i, Bc.jst); B.Amu_t(i, Bc.jend) = B.Amu_t(i, Bc.jend - 1); }
      if (Bc.face == 1) {
        for (int j = Bc.jst; j <= Bc.jend; j++) B.Amu_t(nx1, j) = B.Amu_t(nx1 - 1, j);
        for (int j = Bc.jst; j <= Bc.jend; j++) B.Amu_t(0, j) = -B.Amu_t(1, j);
      } else {
        for (int j = Bc.jst; j <= Bc.jend; j++) B.Amu_t(0, j) = B.Amu_t(1, j);
        for (int j = Bc.jst; j <= Bc.jend; j++) B.Amu_t(nx1, j) = -B.Amu_t(nx1 - 1, j);
      }
    } else {
      std::vector<double> yy(ny1, 0), Amu1d(ny1, 0), Amut1d(ny1, 0), d1d(ny1, 0), u1d(ny1, 0), v1d(ny1, 0), om(ny1, 0);
      for (int i = Bc.ist; i <= Bc.iend - 1; i++) {
        double x0, y0;
        if (Bc.face == 2) { x0 = (B.x1(i, 1) + B.x1(i, 0)) * 0.5; y0 = (B.y1(i, 1) + B.y1(i, 0)) * 0.5; }
        else { x0 = (B.x1(i, ny1 - 1) + B.x1(i, ny1)) * 0.5; y0 = (B.y1(i, ny1 - 1) + B.y1(i, ny1)) * 0.5; }
        for (int j = 1; j <= ny1 - 1; j++) {
          int j1 = (Bc.face == 2) ? j : ny1 - j;
          double dx = B.x1(i, j) - x0, dy = B.y1(i, j) - y0;
          yy[j1 - 1] = std::sqrt(dx * dx + dy * dy);
          u1d[j1 - 1] = F.uu(i, j); v1d[j1 - 1] = F.v(i, j); d1d[j1 - 1] = F.d(i, j); om[j1 - 1] = omiga(i, j);
          Amu1d[j1 - 1] = B.Amu(i, j);
        }
        bl_model_1d(ny1, yy.data(), Amu1d.data(), Amut1d.data(), d1d.data(), u1d.data(), v1d.data(), om.data());
        for (int j = 1; j <= ny1 - 1; j++) {
          int j1 = (Bc.face == 2) ? j : ny1 - j;
          if (flag1(i, j) == 0) { flag1(i, j) = 1; B.Amu_t(i, j) = Amut1d[j1 - 1]; }
          else B.Amu_t(i, j) = std::min(B.Amu_t(i, j), Amut1d[j1 - 1]);
        }
      }
      if (Bc.face == 2) {
        for (int i = Bc.ist; i <= Bc.iend; i++) B.Amu_t(i, 0) = -B.Amu_t(i, 1);
        for (int i = Bc.ist; i <= Bc.iend; i++) B.Amu_t(i, ny1) = B.Amu_t(i, ny1 - 1);
      } else {
        for (int i = Bc.ist; i <= Bc.iend; i++) B.Amu_t(i, ny1) = -B.Amu_t(i, ny1 - 1);
        for (int i = Bc.ist; i <= Bc.iend; i++) B.Amu_t(i, 0) = B.Amu_t(i, 1);
      }
      for (int j = 1 - LAP; j <= ny1 + LAP - 1; j++) { B.Amu_t(Bc.ist - 1, j) = B.Amu_t(Bc.ist, j); B.Amu_t(Bc.iend, j) = B.Amu_t(Bc.iend - 1, j); }
    }
  }
}

// viscous stress on a face: shared algebra of sub_Residual.f90:313-343 / 419-450
struct FaceGrad { double Dix, Diy, Djx, Djy, Diu, Div, DiT, Dju, Djv, DjT; };
inline void viscous_face(const FaceGrad &g, double Amu1, double Amk1, double u1, double v1, double n1, double n2,
                         double s, double &F2, double &F3, double &F4) {
  double Ds = 1.0 / (g.Dix * g.Djy - g.Djx * g.Diy);
  double ux = (g.Diu * g.Djy - g.Dju * g.Diy) * Ds, vx = (g.Div * g.Djy - g.Djv * g.Diy) * Ds;
  double Tx = (g.DiT * g.Djy - g.DjT * g.Diy) * Ds;
  double uy = (-g.Diu * g.Djx + g.Dju * g.Dix) * Ds, vy = (-g.Div * g.Djx + g.Djv * g.Dix) * Ds;
  double Ty = (-g.DiT * g.Djx + g.DjT * g.Dix) * Ds;
  double t11 = ((4.0 / 3.0) * ux - (2.0 / 3.0) * vy) * Amu1;
  double t22 = ((4.0 / 3.0) * vy - (2.0 / 3.0) * ux) * Amu1;
  double t12 = (uy + vx) * Amu1;
  double E1 = u1 * t11 + v1 * t12 + Amk1 * Tx, E2 = u1 * t12 + v1 * t22 + Amk1 * Ty;
  F2 = F2 + (t11 * n1 + t12 * n2) * s;
  F3 = F3 + (t12 * n1 + t22 * n2) * s;
  F4 = F4 + (E1 * n1 + E2 * n2) * s;
}

// Residual_FVM, sub_Residual.f90:200-472
void residual_fvm(Solver &S, Mesh &MP, Block &B, FlowVar &F) {
  int nx = B.nx, ny = B.ny;
  int Scheme = MP.scheme, IFlux = MP.flux, Recon = MP.recon;
  double gamma = S.gamma, Cp = S.Cp, Pr = S.Pr;
  bool fdm = B.FVM_FDM == Method_FDM;
  std::fill(F.Fluxi.v.begin(), F.Fluxi.v.end(), 0.0);
  std::fill(F.Fluxj.v.begin(), F.Fluxj.v.end(), 0.0);
#pragma omp parallel for schedule(static)
  for (int j = 1; j <= ny - 1; j++)
    for (int i = 1; i <= nx; i++) {
      if (fdm && (i >= LFDM + 2 && i <= nx - LFDM - 1) && (j >= LFDM + 2 && j <= ny - LFDM - 1)) continue;
      double si = B.si(i, j), ni1 = B.ni1(i, j), ni2 = B.ni2(i, j);
      double U0[4][4], UL[4], UR[4];
      if (Recon == Reconst_Original) {
        for (int k = 0; k < 4; k++) { U0[k][0] = F.d(i - 2 + k, j); U0[k][1] = F.uu(i - 2 + k, j); U0[k][2] = F.v(i - 2 + k, j); U0[k][3] = F.p(i - 2 + k, j); }
        recon_original(U0, UL, UR, Scheme);
      } else {
        for (int k = 0; k < 4; k++) for (int m = 0; m < 4; m++) U0[k][m] = B.U(m + 1, i - 2 + k, j);
        if (Recon == Reconst_Conservative) recon_conservative(U0, UL, UR, gamma, Scheme);
        else recon_characteristic(U0, UL, UR, gamma, Scheme);
      }
      double QL[4] = {UL[0], UL[1] * ni1 + UL[2] * ni2, -UL[1] * ni2 + UL[2] * ni1, UL[3]};
      double QR[4] = {UR[0], UR[1] * ni1 + UR[2] * ni2, -UR[1] * ni2 + UR[2] * ni1, UR[3]};
      double Fl[4];
      face_flux(IFlux, QL, QR, Fl, gamma);
      F.Fluxi(1, i, j) = -Fl[0] * si;
      F.Fluxi(2, i, j) = -(Fl[1] * ni1 - Fl[2] * ni2) * si;
      F.Fluxi(3, i, j) = -(Fl[1] * ni2 + Fl[2] * ni1) * si;
      F.Fluxi(4, i, j) = -Fl[3] * si;
      if (S.If_viscous == 0) continue;
      double Amu1, Amk1;
      if (i == 1) { Amu1 = B.Amu(i, j) + B.Amu_t(i, j); Amk1 = Cp * (B.Amu(i, j) / Pr + B.Amu_t(i, j) / PrT); }
      else if (i == nx) { Amu1 = B.Amu(i - 1, j) + B.Amu_t(i - 1, j); Amk1 = Cp * (B.Amu(i - 1, j) / Pr + B.Amu_t(i - 1, j) / PrT); }
      else {
        Amu1 = (B.Amu(i - 1, j) + B.Amu(i, j) + B.Amu_t(i - 1, j) + B.Amu_t(i, j)) * 0.5;
        Amk1 = Cp * ((B.Amu(i - 1, j) + B.Amu(i, j)) / Pr + (B.Amu_t(i - 1, j) + B.Amu_t(i, j)) / PrT) * 0.5;
      }
      FaceGrad g;
      g.Dix = B.x1(i, j) - B.x1(i - 1, j); g.Diy = B.y1(i, j) - B.y1(i - 1, j);
      g.Djx = (B.x1(i - 1, j + 1) + B.x1(i, j + 1) - B.x1(i - 1, j - 1) - B.x1(i, j - 1)) * 0.25;
      g.Djy = (B.y1(i - 1, j + 1) + B.y1(i, j + 1) - B.y1(i - 1, j - 1) - B.y1(i, j - 1)) * 0.25;
      g.Diu = F.uu(i, j) - F.uu(i - 1, j); g.Div = F.v(i, j) - F.v(i - 1, j); g.DiT = F.T(i, j) - F.T(i - 1, j);
      g.Dju = (F.uu(i - 1, j + 1) + F.uu(i, j + 1) - F.uu(i - 1, j - 1) - F.uu(i, j - 1)) * 0.25;
      g.Djv = (F.v(i - 1, j + 1) + F.v(i, j + 1) - F.v(i - 1, j - 1) - F.v(i, j - 1)) * 0.25;
      g.DjT = (F.T(i - 1, j + 1) + F.T(i, j + 1) - F.T(i - 1, j - 1) - F.T(i, j - 1)) * 0.25;
      double u1 = (F.uu(i, j) + F.uu(i - 1, j)) * 0.5, v1 = (F.v(i, j) + F.v(i - 1, j)) * 0.5;
      viscous_face(g, Amu1, Amk1, u1, v1, ni1, ni2, si, F.Fluxi(2, i, j), F.Fluxi(3, i, j), F.Fluxi(4, i, j));
    }
#pragma omp parallel for schedule(static)
  for (int j = 1; j <= ny; j++)
    for (int i = 1; i <= nx - 1; i++) {
      if (fdm && (i >= LFDM + 2 && i <= nx - LFDM - 1) && (j >= LFDM + 2 && j <= ny - LFDM - 1)) continue;
      double sj = B.sj(i, j), nj1 = B.nj1(i, j), nj2 = B.nj2(i, j);
      double U0[4][4], UL[4], UR[4];
      if (Recon == Reconst_Original) {
        for (int k = 0; k < 4; k++) { U0[k][0] = F.d(i, j - 2 + k); U0[k][1] = F.uu(i, j - 2 + k); U0[k][2] = F.v(i, j - 2 + k); U0[k][3] = F.p(i, j - 2 + k); }
        recon_original(U0, UL, UR, S.Iflag_Scheme);  // global scheme flag (sub_Residual.f90:367)
      } else {
        for (int k = 0; k < 4; k++) for (int m = 0; m < 4; m++) U0[k][m] = B.U(m + 1, i, j - 2 + k);
        if (Recon == Reconst_Conservative) recon_conservative(U0, UL, UR, gamma, Scheme);
        else recon_characteristic(U0, UL, UR, gamma, Scheme);
      }
      double QL[4] = {UL[0], UL[1] * nj1 + UL[2] * nj2, -UL[1] * nj2 + UL[2] * nj1, UL[3]};
      double QR[4] = {UR[0], UR[1] * nj1 + UR[2] * nj2, -UR[1] * nj2 + UR[2] * nj1, UR[3]};
      double Fl[4];
      face_flux(IFlux, QL, QR, Fl, gamma);
      F.Fluxj(1, i, j) = -Fl[0] * sj;
      F.Fluxj(2, i, j) = -(Fl[1] * nj1 - Fl[2] * nj2) * sj;
      F.Fluxj(3, i, j) = -(Fl[1] * nj2 + Fl[2] * nj1) * sj;
      F.Fluxj(4, i, j) = -Fl[3] * sj;
      if (S.If_viscous == 0) continue;
      double Amu1, Amk1;
      if (j == 1) { Amu1 = B.Amu(i, j) + B.Amu_t(i, j); Amk1 = Cp * (B.Amu(i, j) / Pr + B.Amu_t(i, j) / PrT); }
      else if (j == ny) { Amu1 = B.Amu(i, j - 1) + B.Amu_t(i, j - 1); Amk1 = Cp * (B.Amu(i, j - 1) / Pr + B.Amu_t(i, j - 1) / PrT); }
      else {
        Amu1 = (B.Amu(i, j) + B.Amu(i, j - 1) + B.Amu_t(i, j) + B.Amu_t(i, j - 1)) * 0.5;
        Amk1 = Cp * ((B.Amu(i, j - 1) + B.Amu(i, j)) / Pr + (B.Amu_t(i, j - 1) + B.Amu_t(i, j)) / PrT) * 0.5;
      }
      FaceGrad g;
      g.Dix = (B.x1(i + 1, j - 1) + B.x1(i + 1, j) - B.x1(i - 1, j - 1) - B.x1(i - 1, j)) * 0.25;
      g.Diy = (B.y1(i + 1, j - 1) + B.y1(i + 1, j) - B.y1(i - 1, j - 1) - B.y1(i - 1, j)) * 0.25;
      g.Djx = B.x1(i, j) - B.x1(i, j - 1); g.Djy = B.y1(i, j) - B.y1(i, j - 1);
      g.Diu = (F.uu(i + 1, j - 1) + F.uu(i + 1, j) - F.uu(i - 1, j - 1) - F.uu(i - 1, j)) * 0.25;
      g.Div = (F.v(i + 1, j - 1) + F.v(i + 1, j) - F.v(i - 1, j - 1) - F.v(i - 1, j)) * 0.25;
      g.DiT = (F.T(i + 1, j - 1) + F.T(i + 1, j) - F.T(i - 1, j - 1) - F.T(i - 1, j)) * 0.25;
      g.Dju = F.uu(i, j) - F.uu(i, j - 1); g.Djv = F.v(i, j) - F.v(i, j - 1); g.DjT = F.T(i, j) - F.T(i, j - 1);
      double u1 = (F.uu(i, j) + F.uu(i, j - 1)) * 0.5, v1 = (F.v(i, j) + F.v(i, j - 1)) * 0.5;
      viscous_face(g, Amu1, Amk1, u1, v1, nj1, nj2, sj, F.Fluxj(2, i, j), F.Fluxj(3, i, j), F.Fluxj(4, i, j));
    }
  for (int j = 1; j <= ny - 1; j++)
    for (int i = 1; i <= nx - 1; i++) {
      if (fdm && (i >= LFDM + 1 && i <= nx - LFDM - 1) && (j >= LFDM + 1 && j <= ny - LFDM - 1)) continue;
      for (int m = 1; m <= 4; m++)
        B.Res(m, i, j) = F.Fluxi(m, i + 1, j) - F.Fluxi(m, i, j) + F.Fluxj(m, i, j + 1) - F.Fluxj(m, i, j);
    }
}

// split_Steger_Warming, sub_Finite_Difference.f90:154-202
void split_sw(double d, double u, double v, double cc, double *fp, double *fm, double A1, double A2, double gamma) {
  double tmp1 = 2.0 * (gamma - 1.0), tmp3 = (3.0 - gamma) / (2.0 * (gamma - 1.0));
  double vs = A1 * u + A2 * v, ss = std::sqrt(A1 * A1 + A2 * A2);
  double ak1 = A1 / ss, ak2 = A2 / ss;
  double E1 = vs, E2 = vs - cc * ss, E3 = vs + cc * ss;
  double E1P = (E1 + std::fabs(E1)) * 0.5, E2P = (E2 + std::fabs(E2)) * 0.5, E3P = (E3 + std::fabs(E3)) * 0.5;
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
// fp_weno5 / fm_weno5, sub_Finite_Difference.f90:207-275 (1-based v, hj)
void fp_weno5(int nx, const double *v, double *hj) {
  const double ep = 1.0e-6, C03 = 3.0 / 10.0, C13 = 3.0 / 5.0, C23 = 1.0 / 10.0;
  auto V = [&](int k) { return v[k - 1]; };
  for (int k = 3; k <= nx - 2; k++) {
    double t0 = V(k) - 2.0 * V(k + 1) + V(k + 2), t1 = 3.0 * V(k) - 4.0 * V(k + 1) + V(k + 2);
    double S0 = 13.0 / 12.0 * (t0 * t0) + 1.0 / 4.0 * (t1 * t1);
    t0 = V(k - 1) - 2.0 * V(k) + V(k + 1); t1 = V(k - 1) - V(k + 1);
    double S1 = 13.0 / 12.0 * (t0 * t0) + 1.0 / 4.0 * (t1 * t1);
    t0 = V(k - 2) - 2.0 * V(k - 1) + V(k); t1 = V(k - 2) - 4.0 * V(k - 1) + 3.0 * V(k);
    double S2 = 13.0 / 12.0 * (t0 * t0) + 1.0 / 4.0 * (t1 * t1);
    double a0 = C03 / ((ep + S0) * (ep + S0)), a1 = C13 / ((ep + S1) * (ep + S1)), a2 = C23 / ((ep + S2) * (ep + S2));
    double W0 = a0 / (a0 + a1 + a2), W1 = a1 / (a0 + a1 + a2), W2 = a2 / (a0 + a1 + a2);
    double q03 = 1.0 / 3.0 * V(k) + 5.0 / 6.0 * V(k + 1) - 1.0 / 6.0 * V(k + 2);
    double q13 = -1.0 / 6.0 * V(k - 1) + 5.0 / 6.0 * V(k) + 1.0 / 3.0 * V(k + 1);
    double q23 = 1.0 / 3.0 * V(k - 2) - 7.0 / 6.0 * V(k - 1) + 11.0 / 6.0 * V(k);
    hj[k - 1] = W0 * q03 + W1 * q13 + W2 * q23;
  }
}
void fm_weno5(int nx, const double *v, double *hj) {
  const double ep = 1.0e-6, C03 = 3.0 / 10.0, C13 = 3.0 / 5.0, C23 = 1.0 / 10.0;
  auto V = [&](int k) { return v[k - 1]; };
  for (int k = 3; k <= nx - 2; k++) {
    double t0 = V(k) - 2.0 * V(k - 1) + V(k - 2), t1 = 3.0 * V(k) - 4.0 * V(k - 1) + V(k - 2);
    double S0 = 13.0 / 12.0 * (t0 * t0) + 1.0 / 4.0 * (t1 * t1);
    t0 = V(k + 1) - 2.0 * V(k) + V(k - 1); t1 = V(k + 1) - V(k - 1);
    double S1 = 13.0 / 12.0 * (t0 * t0) + 1.0 / 4.0 * (t1 * t1);
    t0 = V(k + 2) - 2.0 * V(k + 1) + V(k); t1 = V(k + 2) - 4.0 * V(k + 1) + 3.0 * V(k);
    double S2 = 13.0 / 12.0 * (t0 * t0) + 1.0 / 4.0 * (t1 * t1);
    double a0 = C03 / ((ep + S0) * (ep + S0)), a1 = C13 / ((ep + S1) * (ep + S1)), a2 = C23 / ((ep + S2) * (ep + S2));
    double W0 = a0 / (a0 + a1 + a2), W1 = a1 / (a0 + a1 + a2), W2 = a2 / (a0 + a1 + a2);
    double q03 = 1.0 / 3.0 * V(k) + 5.0 / 6.0 * V(k - 1) - 1.0 / 6.0 * V(k - 2);
    double q13 = -1.0 / 6.0 * V(k + 1) + 5.0 / 6.0 * V(k) + 1.0 / 3.0 * V(k - 1);
    double q23 = 1.0 / 3.0 * V(k + 2) - 7.0 / 6.0 * V(k + 1) + 11.0 / 6.0 * V(k);
    hj[k - 2] = W0 * q03 + W1 * q13 + W2 * q23;
  }
}

// Residual_FDM, sub_Finite_Difference.f90:4-150
void residual_fdm(Solver &S, Block &B, FlowVar &F) {
  int nx = B.nx - 1, ny = B.ny - 1;
  double gamma = S.gamma, Cp = S.Cp, Pr = S.Pr;
  int NM = std::max(nx, ny);
  std::vector<double> fx1(NM * 4), fx2(NM * 4), hi1(NM), hi2(NM);
  A3 Ev1, Ev2;
  Ev1.alloc(3, 1, nx, 1, ny); Ev2.alloc(3, 1, nx, 1, ny);
  for (int j = LFDM; j <= ny - LFDM; j++) {
    for (int i = 1; i <= nx; i++) {
      double A1 = B.Akx(i, j) / B.Ajac(i, j), A2 = B.Aky(i, j) / B.Ajac(i, j), fp[4], fm[4];
      split_sw(F.d(i, j), F.uu(i, j), F.v(i, j), F.cc(i, j), fp, fm, A1, A2, gamma);
      for (int m = 0; m < 4; m++) { fx1[(i - 1) + NM * m] = fp[m]; fx2[(i - 1) + NM * m] = fm[m]; }
    }
    for (int m = 0; m < 4; m++) {
      fp_weno5(nx, &fx1[NM * m], hi1.data());
      fm_weno5(nx, &fx2[NM * m], hi2.data());
      for (int i = LFDM; i <= nx - LFDM; i++) F.Fluxi(m + 1, i, j) = -(hi1[i - 1] + hi2[i - 1]);
    }
  }
  for (int i = LFDM; i <= nx - LFDM; i++) {
    for (int j = 1; j <= ny; j++) {
      double A1 = B.Aix(i, j) / B.Ajac(i, j), A2 = B.Aiy(i, j) / B.Ajac(i, j), fp[4], fm[4];
      split_sw(F.d(i, j), F.uu(i, j), F.v(i, j), F.cc(i, j), fp, fm, A1, A2, gamma);
      for (int m = 0; m < 4; m++) { fx1[(j - 1) + NM * m] = fp[m]; fx2[(j - 1) + NM * m] = fm[m]; }
    }
    for (int m = 0; m < 4; m++) {
      fp_weno5(ny, &fx1[NM * m], hi1.data());
      fm_weno5(ny, &fx2[NM * m], hi2.data());
      for (int j = LFDM; j <= ny - LFDM; j++) F.Fluxj(m + 1, i, j) = -(hi1[j - 1] + hi2[j - 1]);
    }
  }
  if (S.If_viscous == 1) {
    for (int j = 2; j <= ny - 1; j++)
      for (int i = 2; i <= nx - 1; i++) {
        double mu0 = B.Amu(i, j) + B.Amu_t(i, j);
        double Ak0 = Cp * (B.Amu(i, j) / Pr + B.Amu_t(i, j) / PrT);
        double ui = 0.5 * (F.uu(i + 1, j) - F.uu(i - 1, j)), vi = 0.5 * (F.v(i + 1, j) - F.v(i - 1, j));
        double Ti = 0.5 * (F.T(i + 1, j) - F.T(i - 1, j));
        double uj = 0.5 * (F.uu(i, j + 1) - F.uu(i, j - 1)), vj = 0.5 * (F.v(i, j + 1) - F.v(i, j - 1));
        double Tj = 0.5 * (F.T(i, j + 1) - F.T(i, j - 1));
        double ux = ui * B.Akx(i, j) + uj * B.Aix(i, j), vx = vi * B.Akx(i, j) + vj * B.Aix(i, j);
        double Tx = Ti * B.Akx(i, j) + Tj * B.Aix(i, j);
        double uy = ui * B.Aky(i, j) + uj * B.Aiy(i, j), vy = vi * B.Aky(i, j) + vj * B.Aiy(i, j);
        double Ty = Ti * B.Aky(i, j) + Tj * B.Aiy(i, j);
        double t11 = (4.0 / 3.0 * ux - 2.0 / 3.0 * vy) * mu0, t22 = (4.0 / 3.0 * vy - 2.0 / 3.0 * ux) * mu0;
        double t12 = (uy + vx) * mu0;
        double E1 = F.uu(i, j) * t11 + F.v(i, j) * t12 + Ak0 * Tx, E2 = F.uu(i, j) * t12 + F.v(i, j) * t22 + Ak0 * Ty;
        double J = B.Ajac(i, j);
        Ev1(1, i, j) = (B.Akx(i, j) * t11 + B.Aky(i, j) * t12) / J;
        Ev1(2, i, j) = (B.Akx(i, j) * t12 + B.Aky(i, j) * t22) / J;
        Ev1(3, i, j) = (B.Akx(i, j) * E1 + B.Aky(i, j) * E2) / J;
        Ev2(1, i, j) = (B.Aix(i, j) * t11 + B.Aiy(i, j) * t12) / J;
        Ev2(2, i, j) = (B.Aix(i, j) * t12 + B.Aiy(i, j) * t22) / J;
        Ev2(3, i, j) = (B.Aix(i, j) * E1 + B.Aiy(i, j) * E2) / J;
      }
    for (int j = 3; j <= ny - 2; j++)
      for (int i = 3; i <= nx - 2; i++)
        for (int m = 1; m <= 3; m++) {
          F.Fluxi(m + 1, i, j) = F.Fluxi(m + 1, i, j) + 0.5 * (Ev1(m, i, j) + Ev1(m, i + 1, j));
          F.Fluxj(m + 1, i, j) = F.Fluxj(m + 1, i, j) + 0.5 * (Ev2(m, i, j) + Ev2(m, i, j + 1));
        }
  }
  for (int j = LFDM + 1; j <= ny - LFDM; j++)
    for (int i = LFDM + 1; i <= nx - LFDM; i++)
      for (int m = 1; m <= 4; m++)
        B.Res(m, i, j) = (F.Fluxi(m, i, j) - F.Fluxi(m, i - 1, j) + F.Fluxj(m, i, j) - F.Fluxj(m, i, j - 1));
}

// comput_Lvc, sub_NS_singlegrid.f90:352-388
void comput_lvc(Solver &S, Block &B, FlowVar &F) {
  for (int j = 1; j <= B.ny - 1; j++)
    for (int i = 1; i <= B.nx - 1; i++) {
      double s0 = B.vol(i, j);
      double si = 0.5 * (B.si(i, j) + B.si(i + 1, j));
      double ni1 = 0.5 * (B.ni1(i, j) + B.ni1(i + 1, j)), ni2 = 0.5 * (B.ni2(i, j) + B.ni2(i + 1, j));
      double sj = 0.5 * (B.sj(i, j) + B.sj(i, j + 1));
      double nj1 = 0.5 * (B.nj1(i, j) + B.nj1(i, j + 1)), nj2 = 0.5 * (B.nj2(i, j) + B.nj2(i, j + 1));
      double uni = F.uu(i, j) * ni1 + F.v(i, j) * ni2, unj = F.uu(i, j) * nj1 + F.v(i, j) * nj2;
      B.Lci(i, j) = (std::fabs(uni) + F.cc(i, j)) * si;
      B.Lcj(i, j) = (std::fabs(unj) + F.cc(i, j)) * sj;
      double tmp1 = S.gamma / F.d(i, j) * (B.Amu(i, j) / S.Pr + B.Amu_t(i, j) / PrT);
      B.Lvi(i, j) = tmp1 * si * si / s0;
      B.Lvj(i, j) = tmp1 * sj * sj / s0;
    }
}
// comput_dt, sub_NS_singlegrid.f90:324-348
void comput_dt(Solver &S, Block &B) {
  const double C0 = 1.0;
  for (int j = 1; j <= B.ny - 1; j++)
    for (int i = 1; i <= B.nx - 1; i++) {
      if (S.Iflag_local_dt == 0) B.dt(i, j) = S.dt_global;
      else {
        B.dt(i, j) = S.CFL * B.vol(i, j) / (B.Lci(i, j) + B.Lcj(i, j) + C0 * (B.Lvi(i, j) + B.Lvj(i, j)));
        if (B.dt(i, j) > S.dtmax) B.dt(i, j) = S.dtmax;
        if (B.dt(i, j) < S.dtmin) B.dt(i, j) = S.dtmin;
      }
    }
}

void flowvar_alloc(FlowVar &F, int nx, int ny) {
  F.d.alloc(1 - LAP, nx + LAP - 1, 1 - LAP, ny + LAP - 1);
  F.uu.alloc(1 - LAP, nx + LAP - 1, 1 - LAP, ny + LAP - 1);
  F.v.alloc(1 - LAP, nx + LAP - 1, 1 - LAP, ny + LAP - 1);
  F.T.alloc(1 - LAP, nx + LAP - 1, 1 - LAP, ny + LAP - 1);
  F.p.alloc(1 - LAP, nx + LAP - 1, 1 - LAP, ny + LAP - 1);
  F.cc.alloc(1, nx - 1, 1, ny - 1);
  F.Fluxi.alloc(4, 1, nx, 1, ny);
  F.Fluxj.alloc(4, 1, nx, 1, ny);
}

// Comput_Residual_one_mesh, sub_Residual.f90:13-107 (with Residual 158-191)
int comput_residual_one_mesh(Solver &S, int nMesh) {
  Mesh &MP = S.mesh[nMesh];
  int NV = MP.Nvar;
  for (int m = 0; m < 6; m++) { MP.Res_max[m] = 0.0; MP.Res_rms[m] = 0.0; }
  double Sfac;
  if (S.dual_iflag1 == 0) { S.dual_iflag1 = 1; Sfac = 1.0 / (3.0 * S.dt_global); }
  else Sfac = 1.0 / (2.0 * S.dt_global);
  for (int mb = 0; mb < MP.Num_Block; mb++) {
    Block &B = MP.B[mb];
    FlowVar F;
    flowvar_alloc(F, B.nx, B.ny);
    if (comput_duvtpckw(S, B, F, mb)) return 2;
    // Residual, sub_Residual.f90:158-191
    if (S.If_viscous == 1) {
      get_viscous(S, B, F);
      if (nMesh == 1 || !S.mg_amut) std::fill(B.Amu_t.v.begin(), B.Amu_t.v.end(), 0.0);
      if (MP.turb == Turb_BL) turbulence_bl(S, B, F);
      else if (MP.turb == Turb_SA) turbulence_sa(S, B, F);
      else if (MP.turb == Turb_SST) turbulence_sst(S, B, F);
    }
    residual_fvm(S, MP, B, F);
    if (B.FVM_FDM == Method_FDM) residual_fdm(S, B, F);
    if (S.Time_Method == Time_dual_LU_SGS) {
      for (int j = 1; j <= B.ny - 1; j++)
        for (int i = 1; i <= B.nx - 1; i++)
          for (int m = 1; m <= S.Nvar; m++)
            B.Res(m, i, j) = B.Res(m, i, j) - (3.0 * B.U(m, i, j) - 4.0 * B.Un(m, i, j) + B.Un1(m, i, j)) * B.vol(i, j) * Sfac;
    }
    double rmax[6] = {0}, rrms[6] = {0};
    for (int j = 1; j <= B.ny - 1; j++)
      for (int i = 1; i <= B.nx - 1; i++)
        for (int m = 1; m <= NV; m++) {
          double r = B.Res(m, i, j);
          if (std::fabs(r) > rmax[m - 1]) rmax[m - 1] = std::fabs(r);
          rrms[m - 1] = rrms[m - 1] + r * r;
        }
    for (int m = 0; m < NV; m++) {
      MP.Res_max[m] = std::max(MP.Res_max[m], rmax[m]);
      MP.Res_rms[m] = MP.Res_rms[m] + rrms[m];
    }
    comput_lvc(S, B, F);
    comput_dt(S, B);
  }
  for (int m = 0; m < NV; m++) MP.Res_rms[m] = std::sqrt(MP.Res_rms[m] / (1.0 * MP.Num_Cell));
  return 0;
}

// ---- LU-SGS: sub_LU_SGS.f90 ------------------------------------------------
// comput_DFn, sub_LU_SGS.f90:117-138
void comput_dfn(int NV, double *DF, const double *U, const double *DU, double n1, double n2, double gamma) {
  double U2[6];
  for (int m = 0; m < NV; m++) U2[m] = U[m] + DU[m];
  double un1 = (U[1] * n1 + U[2] * n2) / U[0];
  double p1 = (gamma - 1.0) * (U[3] - 0.5 * (U[1] * U[1] + U[2] * U[2]) / U[0]);
  double un2 = (U2[1] * n1 + U2[2] * n2) / U2[0];
  double p2 = (gamma - 1.0) * (U2[3] - 0.5 * (U2[1] * U2[1] + U2[2] * U2[2]) / U2[0]);
  DF[0] = U2[0] * un2 - U[0] * un1;
  DF[1] = (U2[1] * un2 + p2 * n1) - (U[1] * un1 + p1 * n1);
  DF[2] = (U2[2] * un2 + p2 * n2) - (U[2] * un1 + p1 * n2);
  DF[3] = (U2[3] + p2) * un2 - (U[3] + p1) * un1;
  if (NV == 5) DF[4] = U2[4] * un2 - U[4] * un1;
  else if (NV == 6) { DF[4] = U2[4] * un2 - U[4] * un1; DF[5] = U2[5] * un2 - U[5] * un1; }
}
// du_LU_SGS_2D, sub_LU_SGS.f90:4-108
void du_lu_sgs(Solver &S, int nMesh, int mb, double alfa1) {
  Mesh &MP = S.mesh[nMesh];
  int NV = MP.Nvar;
  Block &B = MP.B[mb];
  int nx = B.nx, ny = B.ny;
  const double w_LU = 1.0;
  double gamma = S.gamma;
  int visc = S.If_viscous;
  for (int plane = 2; plane <= nx + ny - 2; plane++) {
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= ny - 1; j++) {
      int i = plane - j;
      if (i < 1 || i > nx - 1) continue;
      double alfa[6], dui[6] = {0}, duj[6] = {0}, DF[6];
      for (int m = 0; m < NV; m++) alfa[m] = B.vol(i, j) / B.dt(i, j) + w_LU * (B.Lci(i, j) + B.Lcj(i, j)) + B.vol(i, j) * alfa1;
      if (visc == 1) for (int m = 0; m < NV; m++) alfa[m] = alfa[m] + 2.0 * (B.Lvi(i, j) + B.Lvj(i, j));
      if (NV == 5) alfa[4] = alfa[4] + B.Lvi(i, j) + B.Lvj(i, j);
      if (i != 1) {
        comput_dfn(NV, DF, B.U.col(i - 1, j), B.dU.col(i - 1, j), B.ni1(i, j), B.ni2(i, j), gamma);
        for (int m = 0; m < NV; m++) dui[m] = 0.5 * (DF[m] * B.si(i, j) + w_LU * B.Lci(i - 1, j) * B.dU(m + 1, i - 1, j));
        if (visc == 1) for (int m = 0; m < NV; m++) dui[m] = dui[m] + B.Lvi(i - 1, j) * B.dU(m + 1, i - 1, j);
      }
      if (j != 1) {
        comput_dfn(NV, DF, B.U.col(i, j - 1), B.dU.col(i, j - 1), B.nj1(i, j), B.nj2(i, j), gamma);
        for (int m = 0; m < NV; m++) duj[m] = 0.5 * (DF[m] * B.sj(i, j) + w_LU * B.Lcj(i, j - 1) * B.dU(m + 1, i, j - 1));
        if (visc == 1) for (int m = 0; m < NV; m++) duj[m] = duj[m] + B.Lvj(i, j - 1) * B.dU(m + 1, i, j - 1);
      }
      for (int m = 0; m < NV; m++) B.dU(m + 1, i, j) = (B.Res(m + 1, i, j) + dui[m] + duj[m]) / alfa[m];
    }
  }
  for (int plane = nx + ny - 2; plane >= 2; plane--) {
#pragma omp parallel for schedule(static)
    for (int j = ny - 1; j >= 1; j--) {
      int i = plane - j;
      if (i < 1 || i > nx - 1) continue;
      double alfa[6], dui[6] = {0}, duj[6] = {0}, DF[6];
      for (int m = 0; m < NV; m++) alfa[m] = B.vol(i, j) / B.dt(i, j) + w_LU * (B.Lci(i, j) + B.Lcj(i, j)) + B.vol(i, j) * alfa1;
      if (visc == 1) for (int m = 0; m < NV; m++) alfa[m] = alfa[m] + 2.0 * (B.Lvi(i, j) + B.Lvj(i, j));
      if (NV == 5) alfa[4] = alfa[4] + B.Lvi(i, j) + B.Lvj(i, j);
      if (i != nx - 1) {
        comput_dfn(NV, DF, B.U.col(i + 1, j), B.dU.col(i + 1, j), B.ni1(i, j), B.ni2(i, j), gamma);
        for (int m = 0; m < NV; m++) dui[m] = -0.5 * (DF[m] * B.si(i + 1, j) - w_LU * B.Lci(i + 1, j) * B.dU(m + 1, i + 1, j));
        if (visc == 1) for (int m = 0; m < NV; m++) dui[m] = dui[m] + B.Lvi(i + 1, j) * B.dU(m + 1, i + 1, j);
      }
      if (j != ny - 1) {
        comput_dfn(NV, DF, B.U.col(i, j + 1), B.dU.col(i, j + 1), B.nj1(i, j), B.nj2(i, j), gamma);
        for (int m = 0; m < NV; m++) duj[m] = -0.5 * (DF[m] * B.sj(i, j + 1) - w_LU * B.Lcj(i, j + 1) * B.dU(m + 1, i, j + 1));
        if (visc == 1) for (int m = 0; m < NV; m++) duj[m] = duj[m] + B.Lvj(i, j + 1) * B.dU(m + 1, i, j + 1);
      }
      for (int m = 0; m < NV; m++) B.dU(m + 1, i, j) = B.dU(m + 1, i, j) + (dui[m] + duj[m]) / alfa[m];
    }
  }
}

// ---- time advance: sub_NS_singlegrid.f90 and sub_NS_multigrid.f90 ----------
// Add_force_function, sub_NS_multigrid.f90:177-195
void add_force_function(Solver &S, int nMesh) {
  for (auto &B : S.mesh[nMesh].B)
    for (int j = 1; j <= B.ny - 1; j++)
      for (int i = 1; i <= B.nx - 1; i++)
        for (int m = 1; m <= 4; m++) B.Res(m, i, j) = B.Res(m, i, j) + B.QF(m, i, j);
}
// comput_force_function, sub_NS_multigrid.f90:156-173
void comput_force_function(Solver &S, int nMesh) {
  for (auto &B : S.mesh[nMesh].B)
    for (int j = 1; j <= B.ny - 1; j++)
      for (int i = 1; i <= B.nx - 1; i++)
        for (int m = 1; m <= 4; m++) B.QF(m, i, j) = B.QF(m, i, j) - B.Res(m, i, j);
}
// force_vt_kw, sub_NS_singlegrid.f90:30-60
void force_vt_kw(Solver &S, int nMesh) {
  Mesh &MP = S.mesh[nMesh];
  for (auto &B : MP.B)
    for (int j = 1; j <= B.ny - 1; j++)
      for (int i = 1; i <= B.nx - 1; i++) {
        if (MP.Nvar == 5) { if (B.U(5, i, j) < 0) B.U(5, i, j) = 1.0e-10; }
        else if (MP.Nvar == 6) {
          if (B.U(5, i, j) < 0) B.U(5, i, j) = 1.0e-10;
          if (B.U(6, i, j) < 0) B.U(6, i, j) = 1.0e-10;
        }
      }
}
// NS_Time_advance_1Euler, sub_NS_singlegrid.f90:67-106
int time_euler1(Solver &S, int nMesh) {
  Mesh &MP = S.mesh[nMesh];
  if (comput_residual_one_mesh(S, nMesh)) return 2;
  if (nMesh != 1) add_force_function(S, nMesh);
  for (auto &B : MP.B)
    for (int j = 1; j <= B.ny - 1; j++)
      for (int i = 1; i <= B.nx - 1; i++)
        for (int m = 1; m <= MP.Nvar; m++) {
          double du = B.Res(m, i, j) / B.vol(i, j);
          B.U(m, i, j) = B.U(m, i, j) + B.dt(i, j) * du;
        }
  boundary_condition_onemesh(S, nMesh);
  update_buffer_onemesh(S, nMesh);
  MP.tt = MP.tt + S.dt_global;
  MP.Kstep = MP.Kstep + 1;
  return 0;
}
// NS_Time_advance_RK3, sub_NS_singlegrid.f90:115-176
int time_rk3(Solver &S, int nMesh) {
  Mesh &MP = S.mesh[nMesh];
  const double Ralfa[3] = {1.0, 3.0 / 4.0, 1.0 / 3.0}, Rbeta[3] = {1.0, 1.0 / 4.0, 2.0 / 3.0},
               Rgamma[3] = {0.0, 1.0 / 4.0, 2.0 / 3.0};
  for (auto &B : MP.B)
    for (int j = 0; j <= B.ny; j++)
      for (int i = 0; i <= B.nx; i++)
        for (int m = 1; m <= MP.Nvar; m++) B.Un(m, i, j) = B.U(m, i, j);
  for (int KRK = 0; KRK < 3; KRK++) {
    if (comput_residual_one_mesh(S, nMesh)) return 2;
    if (nMesh != 1) add_force_function(S, nMesh);
    for (auto &B : MP.B)
      for (int j = 1; j <= B.ny - 1; j++)
        for (int i = 1; i <= B.nx - 1; i++)
          for (int m = 1; m <= MP.Nvar; m++) {
            double du = B.Res(m, i, j) / B.vol(i, j);
            B.U(m, i, j) = Ralfa[KRK] * B.Un(m, i, j) + Rgamma[KRK] * B.U(m, i, j) + B.dt(i, j) * Rbeta[KRK] * du;
          }
    boundary_condition_onemesh(S, nMesh);
    update_buffer_onemesh(S, nMesh);
  }
  MP.tt = MP.tt + S.dt_global;
  MP.Kstep = MP.Kstep + 1;
  return 0;
}
// NS_Time_advance_LU_SGS, sub_NS_singlegrid.f90:185-224.  On a coarse mesh
// (multigrid with LU-SGS smoothing, an extension) the forcing is added after
// the residual, exactly as the explicit smoothers do at sub_NS_singlegrid.f90:77.
int time_lusgs(Solver &S, int nMesh) {
  Mesh &MP = S.mesh[nMesh];
  if (comput_residual_one_mesh(S, nMesh)) return 2;
  if (nMesh != 1) add_force_function(S, nMesh);
  for (int mb = 0; mb < MP.Num_Block; mb++) {
    du_lu_sgs(S, nMesh, mb, 0.0);
    Block &B = MP.B[mb];
    for (int j = 1; j <= B.ny - 1; j++)
      for (int i = 1; i <= B.nx - 1; i++)
        for (int m = 1; m <= MP.Nvar; m++) B.U(m, i, j) = B.U(m, i, j) + B.dU(m, i, j);
  }
  boundary_condition_onemesh(S, nMesh);
  update_buffer_onemesh(S, nMesh);
  MP.tt = MP.tt + S.dt_global;
  MP.Kstep = MP.Kstep + 1;
  return 0;
}
// Dual_time_LU_SGS, sub_NS_singlegrid.f90:231-310
int time_dual_lusgs(Solver &S) {
  double alfa1;
  if (S.dual_iflag == 0) { S.dual_iflag = 1; alfa1 = 1.0 / S.dt_global; }
  else alfa1 = 3.0 / (2.0 * S.dt_global);
  Mesh &MP = S.mesh[1];
  for (int kt = 1; kt <= S.P.Nstep_Inner_Limit; kt++) {
    if (comput_residual_one_mesh(S, 1)) return 2;
    for (int mb = 0; mb < MP.Num_Block; mb++) {
      du_lu_sgs(S, 1, mb, alfa1);
      Block &B = MP.B[mb];
      for (int j = 1; j <= B.ny - 1; j++)
        for (int i = 1; i <= B.nx - 1; i++)
          for (int m = 1; m <= MP.Nvar; m++) B.U(m, i, j) = B.U(m, i, j) + B.dU(m, i, j);
    }
    boundary_condition_onemesh(S, 1);
    update_buffer_onemesh(S, 1);
    double max_res = MP.Res_rms[0];
    for (int m = 0; m < S.Nvar; m++) max_res = std::max(max_res, MP.Res_rms[m]);
    if (max_res <= S.P.Res_Inner_Limit) break;
  }
  for (auto &B : MP.B)
    for (int j = 1; j <= B.ny - 1; j++)
      for (int i = 1; i <= B.nx - 1; i++)
        for (int m = 1; m <= MP.Nvar; m++) { B.Un1(m, i, j) = B.Un(m, i, j); B.Un(m, i, j) = B.U(m, i, j); }
  MP.tt = MP.tt + S.dt_global;
  MP.Kstep = MP.Kstep + 1;
  return 0;
}
// NS_Time_advance, sub_NS_singlegrid.f90:8-26
int ns_time_advance(Solver &S, int nMesh) {
  int r = 0;
  if (S.Time_Method == Time_Euler1) r = time_euler1(S, nMesh);
  else if (S.Time_Method == Time_RK3) r = time_rk3(S, nMesh);
  else if (S.Time_Method == Time_LU_SGS) r = time_lusgs(S, nMesh);
  else if (S.Time_Method == Time_dual_LU_SGS) r = time_dual_lusgs(S);
  if (r) return r;
  force_vt_kw(S, nMesh);
  return 0;
}

// comput_delt_U, Set_Un, comput_new_U: sub_NS_multigrid.f90:199-260
void comput_delt_u(Solver &S, int nMesh) {
  for (auto &B : S.mesh[nMesh].B)
    for (int j = 0; j <= B.ny; j++)
      for (int i = 0; i <= B.nx; i++)
        for (int m = 1; m <= 4; m++) B.deltU(m, i, j) = B.U(m, i, j) - B.Un(m, i, j);
}
void set_un(Solver &S, int nMesh) {
  for (auto &B : S.mesh[nMesh].B)
    for (int j = 0; j <= B.ny; j++)
      for (int i = 0; i <= B.nx; i++)
        for (int m = 1; m <= 4; m++) B.Un(m, i, j) = B.U(m, i, j);
}
void comput_new_u(Solver &S, int nMesh) {
  for (auto &B : S.mesh[nMesh].B)
    for (int j = 1; j <= B.ny - 1; j++)
      for (int i = 1; i <= B.nx - 1; i++)
        for (int m = 1; m <= 4; m++) B.U(m, i, j) = B.U(m, i, j) + B.deltU(m, i, j);
}
// prolong_U, sub_NS_multigrid.f90:271-343
void prolong_u(Solver &S, int m1, int m2, int flag) {
  const double a1 = 9.0 / 16.0, a2 = 3.0 / 16.0, a3 = 1.0 / 16.0;
  Mesh &MP1 = S.mesh[m1], &MP2 = S.mesh[m2];
  for (int mb = 0; mb < MP1.Num_Block; mb++) {
    Block &B1 = MP1.B[mb], &B2 = MP2.B[mb];
    int nx2 = B2.nx, ny2 = B2.ny;
    std::vector<int> ia1(nx2 + 1), ia2(nx2 + 1), ja1(ny2 + 1), ja2(ny2 + 1);
    for (int i = 0; i <= nx2; i++) {
      if (i % 2 == 0) { ia1[i] = i / 2; ia2[i] = i / 2 + 1; }
      else { ia1[i] = i / 2 + 1; ia2[i] = i / 2; }
    }
    for (int j = 0; j <= ny2; j++) {
      if (j % 2 == 0) { ja1[j] = j / 2; ja2[j] = j / 2 + 1; }
      else { ja1[j] = j / 2 + 1; ja2[j] = j / 2; }
    }
    A3 &src = (flag == 1) ? B1.U : B1.deltU;
    A3 &dst = (flag == 1) ? B2.U : B2.deltU;
    for (int j = 0; j <= ny2; j++)
      for (int i = 0; i <= nx2; i++)
        for (int m = 1; m <= 4; m++)
          dst(m, i, j) = a1 * src(m, ia1[i], ja1[j]) + a2 * (src(m, ia2[i], ja1[j]) + src(m, ia1[i], ja2[j])) +
                         a3 * src(m, ia2[i], ja2[j]);
  }
}
// interpolation2h, sub_NS_multigrid.f90:349-398
void interpolation2h(Solver &S, int m1, int m2, int flag) {
  Mesh &MP1 = S.mesh[m1], &MP2 = S.mesh[m2];
  for (int mb = 0; mb < MP1.Num_Block; mb++) {
    Block &B1 = MP1.B[mb], &B2 = MP2.B[mb];
    for (int j = 1; j <= B2.ny - 1; j++)
      for (int i = 1; i <= B2.nx - 1; i++) {
        int i1 = 2 * i - 1, i2 = 2 * i, j1 = 2 * j - 1, j2 = 2 * j;
        for (int m = 1; m <= 4; m++) {
          if (flag == 1)
            B2.U(m, i, j) = (B1.U(m, i1, j1) * B1.vol(i1, j1) + B1.U(m, i1, j2) * B1.vol(i1, j2) +
                             B1.U(m, i2, j1) * B1.vol(i2, j1) + B1.U(m, i2, j2) * B1.vol(i2, j2)) / B2.vol(i, j);
          else
            B2.QF(m, i, j) = B1.Res(m, i1, j1) + B1.Res(m, i1, j2) + B1.Res(m, i2, j1) + B1.Res(m, i2, j2);
        }
      }
    // extension (mg_amut): the coarse eddy viscosity over 0..nx2, 0..ny2 is
    // the mean of the children's within the finer level's 0..nx, 0..ny
    // (a ghost cell's children are the finer level's ghost cells there)
    if (flag == 1 && S.mg_amut && S.If_viscous == 1 && S.Iflag_turbulence_model != Turb_NONE)
      for (int j = 0; j <= B2.ny; j++)
        for (int i = 0; i <= B2.nx; i++) {
          double sum = 0.0;
          int n = 0;
          for (int jj = 2 * j - 1; jj <= 2 * j; jj++)
            for (int ii = 2 * i - 1; ii <= 2 * i; ii++)
              if (ii >= 0 && ii <= B1.nx && jj >= 0 && jj <= B1.ny) { sum += B1.Amu_t(ii, jj); n++; }
          B2.Amu_t(i, j) = sum / n;
        }
  }
}
// fine/coarse smoother used inside the multigrid cycles (sub_NS_multigrid.f90:23-27,79-83)
int mg_smooth_fine(Solver &S) {
  if (S.Time_Method == Time_Euler1) return time_euler1(S, 1);
  if (S.Time_Method == Time_LU_SGS) { int r = time_lusgs(S, 1); if (!r) force_vt_kw(S, 1); return r; }
  return time_rk3(S, 1);
}
int mg_smooth_coarse(Solver &S, int nMesh) {
  const int Time_step_coarse_mesh = 3;
  if (S.Time_Method == Time_Euler1) {
    set_un(S, nMesh);
    for (int m = 0; m < Time_step_coarse_mesh; m++) if (time_euler1(S, nMesh)) return 2;
    return 0;
  }
  if (S.Time_Method == Time_LU_SGS) { set_un(S, nMesh); return time_lusgs(S, nMesh); }
  return time_rk3(S, nMesh);
}
// NS_2stge_multigrid, sub_NS_multigrid.f90:14-58
int ns_2stage_mg(Solver &S) {
  if (mg_smooth_fine(S)) return 2;
  if (comput_residual_one_mesh(S, 1)) return 2;
  interpolation2h(S, 1, 2, 2);
  interpolation2h(S, 1, 2, 1);
  boundary_condition_onemesh(S, 2);
  update_buffer_onemesh(S, 2);
  if (comput_residual_one_mesh(S, 2)) return 2;
  comput_force_function(S, 2);
  if (mg_smooth_coarse(S, 2)) return 2;
  comput_delt_u(S, 2);
  prolong_u(S, 2, 1, 2);
  comput_new_u(S, 1);
  boundary_condition_onemesh(S, 1);
  update_buffer_onemesh(S, 1);
  return 0;
}
// NS_3stge_multigrid, sub_NS_multigrid.f90:66-142
int ns_3stage_mg(Solver &S) {
  if (mg_smooth_fine(S)) return 2;
  if (comput_residual_one_mesh(S, 1)) return 2;
  interpolation2h(S, 1, 2, 2);
  interpolation2h(S, 1, 2, 1);
  boundary_condition_onemesh(S, 2);
  update_buffer_onemesh(S, 2);
  if (comput_residual_one_mesh(S, 2)) return 2;
  comput_force_function(S, 2);
  if (mg_smooth_coarse(S, 2)) return 2;
  if (comput_residual_one_mesh(S, 2)) return 2;
  add_force_function(S, 2);
  interpolation2h(S, 2, 3, 2);
  interpolation2h(S, 2, 3, 1);
  boundary_condition_onemesh(S, 3);
  update_buffer_onemesh(S, 3);
  if (comput_residual_one_mesh(S, 3)) return 2;
  comput_force_function(S, 3);
  if (mg_smooth_coarse(S, 3)) return 2;
  comput_delt_u(S, 3);
  prolong_u(S, 3, 2, 2);
  comput_new_u(S, 2);
  comput_delt_u(S, 2);
  prolong_u(S, 2, 1, 2);
  comput_new_u(S, 1);
  boundary_condition_onemesh(S, 1);
  update_buffer_onemesh(S, 1);
  return 0;
}
// one iteration of the main loop, opencfd_ec2d_v1.5.4.f90:172-186
int main_loop_step(Solver &S) {
  if (S.Num_Mesh == 1) return ns_time_advance(S, 1);
  if (S.Num_Mesh == 2) return ns_2stage_mg(S);
  return ns_3stage_mg(S);
}

// init_flow_zero, sub_init.f90:423-495
int init_flow_zero(Solver &S) {
  double d0 = 1.0, u0 = 1.0 * std::cos(S.AoA), v0 = 1.0 * std::sin(S.AoA), p0 = 1.0 / (S.gamma * S.Ma * S.Ma);
  // coarse eddy viscosity (kept between residuals only with mg_amut): zero
  // until the first restriction
  for (int m = 2; m <= S.Num_Mesh; m++)
    for (auto &B : S.mesh[m].B) std::fill(B.Amu_t.v.begin(), B.Amu_t.v.end(), 0.0);
  if (S.Nvar == 5)
    for (auto &B : S.mesh[1].B)
      for (int j = 1; j <= B.ny - 1; j++)
        for (int i = 1; i <= B.nx - 1; i++) B.U(5, i, j) = S.vt_inf / S.Re;
  if (S.Nvar == 6)
    for (auto &B : S.mesh[1].B)
      for (int j = 1; j <= B.ny - 1; j++)
        for (int i = 1; i <= B.nx - 1; i++) { B.U(5, i, j) = 10.0 * S.Kt_inf; B.U(6, i, j) = S.Wt_inf; }
  for (auto &B : S.mesh[S.Num_Mesh].B)
    for (int j = 1; j <= B.ny - 1; j++)
      for (int i = 1; i <= B.nx - 1; i++) {
        B.U(1, i, j) = d0; B.U(2, i, j) = d0 * u0; B.U(3, i, j) = d0 * v0;
        B.U(4, i, j) = p0 / (S.gamma - 1.0) + 0.5 * d0 * (u0 * u0 + v0 * v0);
      }
  boundary_condition_onemesh(S, S.Num_Mesh);
  update_buffer_onemesh(S, S.Num_Mesh);
  for (int nMesh = S.Num_Mesh; nMesh >= 1; nMesh--) {
    for (int step = 1; step <= S.P.Pre_Step_Mesh[nMesh - 1]; step++)
      if (ns_time_advance(S, nMesh)) return 2;
    if (nMesh > 1) {
      prolong_u(S, nMesh, nMesh - 1, 1);
      boundary_condition_onemesh(S, nMesh - 1);
      update_buffer_onemesh(S, nMesh - 1);
    }
  }
  return 0;
}

// ---- wall forces (new component; no counterpart in the reference) ----------
// Walks the wall faces like read_flow-1.2.f90:38-51 and integrates pressure and
// viscous stress.  Pressure at the wall face = mean of the two adjacent cells
// (interior and first ghost); stress from the face-gradient formula of
// Residual_FVM (sub_Residual.f90:313-343 / 419-450) with the one-sided
// viscosity used there on block edges.  Normal n points into the fluid.
struct WallFace { double fx, fy, xm, ym, cf; };
void wall_faces(Solver &S, Block &B, const BcMsg &Bc, std::vector<WallFace> &out) {
  int nx = B.nx, ny = B.ny;
  FlowVar F;
  flowvar_alloc(F, nx, ny);
  double p00 = 1.0 / (S.gamma * S.Ma * S.Ma);
  for (int j = 1 - LAP; j <= ny + LAP - 1; j++)
    for (int i = 1 - LAP; i <= nx + LAP - 1; i++) {
      F.d(i, j) = B.U(1, i, j);
      F.uu(i, j) = B.U(2, i, j) / F.d(i, j);
      F.v(i, j) = B.U(3, i, j) / F.d(i, j);
      F.T(i, j) = (B.U(4, i, j) - 0.5 * F.d(i, j) * (F.uu(i, j) * F.uu(i, j) + F.v(i, j) * F.v(i, j))) / (S.Cv * F.d(i, j));
      F.p(i, j) = p00 * F.d(i, j) * F.T(i, j);
    }
  bool ifc = (Bc.face == 1 || Bc.face == 3);
  int kbeg = ifc ? Bc.jst : Bc.ist, kend = ifc ? Bc.jend - 1 : Bc.iend - 1;
  for (int k = kbeg; k <= kend; k++) {
    int fi, fj, ci, cj, gi, gj;  // face index, interior cell, ghost cell
    if (Bc.face == 1) { fi = 1; fj = k; ci = 1; cj = k; gi = 0; gj = k; }
    else if (Bc.face == 3) { fi = nx; fj = k; ci = nx - 1; cj = k; gi = nx; gj = k; }
    else if (Bc.face == 2) { fi = k; fj = 1; ci = k; cj = 1; gi = k; gj = 0; }
    else { fi = k; fj = ny; ci = k; cj = ny - 1; gi = k; gj = ny; }
    double n1, n2, s, xm, ym;
    if (ifc) { n1 = B.ni1(fi, fj); n2 = B.ni2(fi, fj); s = B.si(fi, fj);
      xm = 0.5 * (B.x(fi, fj) + B.x(fi, fj + 1)); ym = 0.5 * (B.y(fi, fj) + B.y(fi, fj + 1)); }
    else { n1 = B.nj1(fi, fj); n2 = B.nj2(fi, fj); s = B.sj(fi, fj);
      xm = 0.5 * (B.x(fi, fj) + B.x(fi + 1, fj)); ym = 0.5 * (B.y(fi, fj) + B.y(fi + 1, fj)); }
    double sgn = ((B.x1(ci, cj) - xm) * n1 + (B.y1(ci, cj) - ym) * n2) >= 0.0 ? 1.0 : -1.0;
    double pw = 0.5 * (F.p(ci, cj) + F.p(gi, gj)) - p00;
    double fx = 0.0, fy = 0.0, f4 = 0.0;
    if (S.If_viscous == 1) {
      double Tsb = 110.4 / S.T_inf, T = 0.5 * (F.T(ci, cj) + F.T(gi, gj));
      double Amu1 = 1.0 / S.Re * (1.0 + Tsb) * std::sqrt(T * T * T) / (Tsb + T);
      FaceGrad g;
      if (ifc) {
        int i = fi, j = fj;
        g.Dix = B.x1(i, j) - B.x1(i - 1, j); g.Diy = B.y1(i, j) - B.y1(i - 1, j);
        g.Djx = (B.x1(i - 1, j + 1) + B.x1(i, j + 1) - B.x1(i - 1, j - 1) - B.x1(i, j - 1)) * 0.25;
        g.Djy = (B.y1(i - 1, j + 1) + B.y1(i, j + 1) - B.y1(i - 1, j - 1) - B.y1(i, j - 1)) * 0.25;
        g.Diu = F.uu(i, j) - F.uu(i - 1, j); g.Div = F.v(i, j) - F.v(i - 1, j); g.DiT = F.T(i, j) - F.T(i - 1, j);
        g.Dju = (F.uu(i - 1, j + 1) + F.uu(i, j + 1) - F.uu(i - 1, j - 1) - F.uu(i, j - 1)) * 0.25;
        g.Djv = (F.v(i - 1, j + 1) + F.v(i, j + 1) - F.v(i - 1, j - 1) - F.v(i, j - 1)) * 0.25;
        g.DjT = (F.T(i - 1, j + 1) + F.T(i, j + 1) - F.T(i - 1, j - 1) - F.T(i, j - 1)) * 0.25;
      } else {
        int i = fi, j = fj;
        g.Dix = (B.x1(i + 1, j - 1) + B.x1(i + 1, j) - B.x1(i - 1, j - 1) - B.x1(i - 1, j)) * 0.25;
        g.Diy = (B.y1(i + 1, j - 1) + B.y1(i + 1, j) - B.y1(i - 1, j - 1) - B.y1(i - 1, j)) * 0.25;
        g.Djx = B.x1(i, j) - B.x1(i, j - 1); g.Djy = B.y1(i, j) - B.y1(i, j - 1);
        g.Diu = (F.uu(i + 1, j - 1) + F.uu(i + 1, j) - F.uu(i - 1, j - 1) - F.uu(i - 1, j)) * 0.25;
        g.Div = (F.v(i + 1, j - 1) + F.v(i + 1, j) - F.v(i - 1, j - 1) - F.v(i - 1, j)) * 0.25;
        g.DiT = (F.T(i + 1, j - 1) + F.T(i + 1, j) - F.T(i - 1, j - 1) - F.T(i - 1, j)) * 0.25;
        g.Dju = F.uu(i, j) - F.uu(i, j - 1); g.Djv = F.v(i, j) - F.v(i, j - 1); g.DjT = F.T(i, j) - F.T(i, j - 1);
      }
      // traction tau.n (n into the fluid) times the face length
      viscous_face(g, Amu1, 0.0, 0.0, 0.0, sgn * n1, sgn * n2, s, fx, fy, f4);
    }
    WallFace w;
    w.fx = -pw * sgn * n1 * s + fx;
    w.fy = -pw * sgn * n2 * s + fy;
    w.xm = xm; w.ym = ym;
    // skin friction: tangential traction / q_inf, tangent along increasing index
    double t1 = ifc ? -n2 : n2, t2 = ifc ? n1 : -n1;
    w.cf = ((fx * t1 + fy * t2) / s) / 0.5;
    out.push_back(w);
  }
}

}  // namespace

// ============================== C API ========================================
extern "C" {

void *orc_new(const orc_params *p) {
  Solver *S = new Solver();
  apply_params(*S, *p);
  return S;
}
void orc_free(void *h) { delete (Solver *)h; }
int orc_set_mg_amut(void *h, int enable) {
  ((Solver *)h)->mg_amut = enable ? 1 : 0;
  return 0;
}
void orc_set_threads(int n) {
#ifdef _OPENMP
  omp_set_num_threads(n);
#else
  (void)n;
#endif
}

int orc_add_block(void *h, int nx, int ny, const double *x, const double *y, int nsub, const int *bc9) {
  Solver &S = *(Solver *)h;
  if (S.setup_done || nx < 3 || ny < 3) return 1;
  Block B;
  B.nx = nx; B.ny = ny;
  B.x.alloc(1 - LAP, nx + LAP, 1 - LAP, ny + LAP);
  B.y.alloc(1 - LAP, nx + LAP, 1 - LAP, ny + LAP);
  for (int j = 1; j <= ny; j++)
    for (int i = 1; i <= nx; i++) { B.x(i, j) = x[(i - 1) + (size_t)nx * (j - 1)]; B.y(i, j) = y[(i - 1) + (size_t)nx * (j - 1)]; }
  for (int k = 0; k < nsub; k++) {
    const int *c = bc9 + 9 * k;
    B.bc.push_back(BcMsg{c[0], c[1], c[2], c[3], c[4], c[5], c[6], c[7], c[8]});
  }
  S.pending.push_back(std::move(B));
  return 0;
}
int orc_set_fdm_block(void *h, int block) { ((Solver *)h)->fdm_blocks.push_back(block); return 0; }
int orc_set_dw(void *h, int block, const double *dw) {
  Solver &S = *(Solver *)h;
  if (block < 1 || block > (int)S.pending.size()) return 1;
  if (S.dw_in.size() < S.pending.size()) S.dw_in.resize(S.pending.size());
  Block &B = S.pending[block - 1];
  S.dw_in[block - 1].assign(dw, dw + (size_t)(B.nx - 1) * (B.ny - 1));
  return 0;
}

// Init + set_control_para + Update_coordinate_buffer + Init_FiniteDifference + comput_dw
// (opencfd_ec2d_v1.5.4.f90:158-164)
int orc_setup(void *h) {
  Solver &S = *(Solver *)h;
  if (S.setup_done || S.pending.empty()) return 1;
  // opencfd_ec2d_v1.5.4.f90:216-221: LU-SGS with multigrid is refused unless the
  // LU-SGS-smoothed multigrid extension is switched on.
  if ((S.Time_Method == Time_LU_SGS && S.Num_Mesh != 1 && !S.P.mg_lusgs) ||
      (S.Time_Method == Time_dual_LU_SGS && S.Num_Mesh != 1))
    return 3;
  S.Num_Mesh = check_mesh_multigrid(S);
  S.mesh.assign(S.Num_Mesh + 1, Mesh());
  Mesh &M1 = S.mesh[1];
  M1.Num_Block = (int)S.pending.size();
  M1.B.resize(M1.Num_Block);
  for (int m = 0; m < M1.Num_Block; m++) {
    Block &Bp = S.pending[m], &B = M1.B[m];
    B.nx = Bp.nx; B.ny = Bp.ny; B.bc = Bp.bc;
    block_alloc(S, B, S.Nvar, true);
    for (int j = 1; j <= B.ny; j++)
      for (int i = 1; i <= B.nx; i++) { B.x(i, j) = Bp.x(i, j); B.y(i, j) = Bp.y(i, j); }
    M1.Num_Cell += (B.nx - 1) * (B.ny - 1);
    block_geometry(B);
  }
  for (int m = 2; m <= S.Num_Mesh; m++) creat_mesh(S, m - 1, m);
  // set_control_para, opencfd_ec2d_v1.5.4.f90:239-260
  M1.turb = S.Iflag_turbulence_model; M1.scheme = S.Iflag_Scheme; M1.flux = S.IFlag_flux;
  M1.recon = S.IFlag_Reconstruction; M1.Nvar = S.Nvar;
  for (int m = 2; m <= S.Num_Mesh; m++) {
    Mesh &MP = S.mesh[m];
    MP.turb = Turb_NONE; MP.scheme = Scheme_UD1; MP.flux = S.IFlag_flux;
    MP.recon = S.IFlag_Reconstruction; MP.Nvar = 4;
  }
  for (int m = 1; m <= S.Num_Mesh; m++) update_coordinate_buffer_onemesh(S, m);
  for (int b : S.fdm_blocks)
    if (b >= 1 && b <= M1.Num_Block) M1.B[b - 1].FVM_FDM = Method_FDM;
  comput_jacobian(S);
  if (S.Iflag_turbulence_model == Turb_SST || S.Iflag_turbulence_model == Turb_SA) comput_dw(S);
  S.pending.clear();
  S.setup_done = true;
  return 0;
}
int orc_num_mesh(void *h) { return ((Solver *)h)->Num_Mesh; }
int orc_nvar(void *h, int mesh) { return ((Solver *)h)->mesh[mesh].Nvar; }
int orc_block_dims(void *h, int mesh, int block, int *nx, int *ny) {
  Solver &S = *(Solver *)h;
  Block &B = S.mesh[mesh].B[block - 1];
  *nx = B.nx; *ny = B.ny;
  return 0;
}
// The start of dual time stepping from the current U: U(n) = U(n-1) = U and
// the first-step flags unset, so the first physical step is the one-step
// form (alfa1 = 1/dt, Sfac = 1/(3 dt), sub_NS_singlegrid.f90:239-245,
// sub_Residual.f90:27-34).  The reference's comment there assumes
// U(n-1) = U(n) on the first step, but its code leaves Un at the allocation
// fill (1,0,0,0) (sub_init.f90:162) and Un1 unset (:155); this sets them as
// the comment says, after a freestream start and after a restart alike.
int orc_dual_time_start(void *h) {
  Solver &S = *(Solver *)h;
  if (S.Time_Method != Time_dual_LU_SGS) return 0;
  for (auto &B : S.mesh[1].B)
    for (int j = 1; j <= B.ny - 1; j++)
      for (int i = 1; i <= B.nx - 1; i++)
        for (int m = 1; m <= S.Nvar; m++) { B.Un(m, i, j) = B.U(m, i, j); B.Un1(m, i, j) = B.U(m, i, j); }
  S.dual_iflag = S.dual_iflag1 = 0;
  return 0;
}
int orc_init_flow(void *h) {
  Solver &S = *(Solver *)h;
  int r = init_flow_zero(S);
  if (!r) orc_dual_time_start(h);
  return r;
}
int orc_get_U(void *h, int mesh, int block, double *U) {
  Solver &S = *(Solver *)h;
  Block &B = S.mesh[mesh].B[block - 1];
  std::memcpy(U, B.U.v.data(), B.U.v.size() * sizeof(double));
  return 0;
}
int orc_set_U(void *h, int mesh, int block, const double *U) {
  Solver &S = *(Solver *)h;
  Block &B = S.mesh[mesh].B[block - 1];
  std::memcpy(B.U.v.data(), U, B.U.v.size() * sizeof(double));
  return 0;
}
static std::vector<double> *field_ptr(Solver &S, int mesh, int block, int field) {
  Block &B = S.mesh[mesh].B[block - 1];
  switch (field) {
    case ORC_F_RES: return &B.Res.v;
    case ORC_F_DT: return &B.dt.v;
    case ORC_F_LCI: return &B.Lci.v;
    case ORC_F_LCJ: return &B.Lcj.v;
    case ORC_F_LVI: return &B.Lvi.v;
    case ORC_F_LVJ: return &B.Lvj.v;
    case ORC_F_DU: return &B.dU.v;
    case ORC_F_AMU: return &B.Amu.v;
    case ORC_F_AMUT: return &B.Amu_t.v;
    case ORC_F_X1: return &B.x1.v;
    case ORC_F_Y1: return &B.y1.v;
    case ORC_F_VOL: return &B.vol.v;
    case ORC_F_SI: return &B.si.v;
    case ORC_F_SJ: return &B.sj.v;
    case ORC_F_NI1: return &B.ni1.v;
    case ORC_F_NI2: return &B.ni2.v;
    case ORC_F_NJ1: return &B.nj1.v;
    case ORC_F_NJ2: return &B.nj2.v;
    case ORC_F_DW: return &B.dw.v;
    case ORC_F_QF: return &B.QF.v;
    case ORC_F_DELTU: return &B.deltU.v;
    case ORC_F_UN: return &B.Un.v;
    case ORC_F_X: return &B.x.v;
    case ORC_F_Y: return &B.y.v;
  }
  return nullptr;
}
int orc_field_size(void *h, int mesh, int block, int field) {
  auto *p = field_ptr(*(Solver *)h, mesh, block, field);
  return p ? (int)p->size() : -1;
}
int orc_get_field(void *h, int mesh, int block, int field, double *out) {
  auto *p = field_ptr(*(Solver *)h, mesh, block, field);
  if (!p) return 1;
  std::memcpy(out, p->data(), p->size() * sizeof(double));
  return 0;
}
int orc_residual(void *h, int mesh) { return comput_residual_one_mesh(*(Solver *)h, mesh); }
int orc_bc(void *h, int mesh) { boundary_condition_onemesh(*(Solver *)h, mesh); return 0; }
int orc_halo(void *h, int mesh) { update_buffer_onemesh(*(Solver *)h, mesh); return 0; }
int orc_lusgs(void *h, int mesh, int block, double alfa1) { du_lu_sgs(*(Solver *)h, mesh, block - 1, alfa1); return 0; }
int orc_time_advance(void *h, int mesh) { return ns_time_advance(*(Solver *)h, mesh); }
int orc_step(void *h, int nsteps) {
  Solver &S = *(Solver *)h;
  for (int k = 0; k < nsteps; k++) { int r = main_loop_step(S); if (r) return r; }
  return 0;
}
int orc_norms(void *h, int mesh, double *res_max6, double *res_rms6, int *kstep, double *tt) {
  Solver &S = *(Solver *)h;
  Mesh &MP = S.mesh[mesh];
  for (int m = 0; m < 6; m++) { res_max6[m] = MP.Res_max[m]; res_rms6[m] = MP.Res_rms[m]; }
  *kstep = MP.Kstep; *tt = MP.tt;
  return 0;
}
int orc_interpolation2h(void *h, int m1, int m2, int flag) { interpolation2h(*(Solver *)h, m1, m2, flag); return 0; }
int orc_prolong(void *h, int m1, int m2, int flag) { prolong_u(*(Solver *)h, m1, m2, flag); return 0; }
int orc_force_function(void *h, int mesh) { comput_force_function(*(Solver *)h, mesh); return 0; }
int orc_set_un(void *h, int mesh) { set_un(*(Solver *)h, mesh); return 0; }
int orc_delt_u(void *h, int mesh) { comput_delt_u(*(Solver *)h, mesh); return 0; }
int orc_new_u(void *h, int mesh) { comput_new_u(*(Solver *)h, mesh); return 0; }
int orc_forces(void *h, double *cl, double *cd, double *cm) {
  Solver &S = *(Solver *)h;
  double Fx = 0, Fy = 0, Mz = 0;
  for (auto &B : S.mesh[1].B)
    for (auto &Bc : B.bc) {
      if (Bc.neighb != BC_Wall) continue;
      std::vector<WallFace> w;
      wall_faces(S, B, Bc, w);
      for (auto &f : w) {
        Fx += f.fx; Fy += f.fy;
        Mz += (f.xm - S.P.xaxis) * f.fy - (f.ym - S.P.yaxis) * f.fx;
      }
    }
  double q = 0.5, ca = std::cos(S.AoA), sa = std::sin(S.AoA);
  *cl = (-Fx * sa + Fy * ca) / q;
  *cd = (Fx * ca + Fy * sa) / q;
  *cm = -Mz / q;
  return 0;
}
int orc_wall_cf(void *h, int block, int sub, double *cf, double *xc, int maxn) {
  Solver &S = *(Solver *)h;
  Block &B = S.mesh[1].B[block - 1];
  std::vector<WallFace> w;
  wall_faces(S, B, B.bc[sub - 1], w);
  int n = std::min((int)w.size(), maxn);
  for (int k = 0; k < n; k++) { cf[k] = w[k].cf; xc[k] = w[k].xm; }
  return (int)w.size();
}
int orc_flux(int iflux, const double *QL, const double *QR, double *F, double gamma) {
  face_flux(iflux, QL, QR, F, gamma);
  return 0;
}
double orc_scheme(int side, double u1, double u2, double u3, double u4, int flag) {
  return side == 0 ? scheme_fP(u1, u2, u3, u4, flag) : scheme_fm(u1, u2, u3, u4, flag);
}
int orc_set_field(void *h, int mesh, int block, int field, const double *in) {
  auto *p = field_ptr(*(Solver *)h, mesh, block, field);
  if (!p) return 1;
  std::memcpy(p->data(), in, p->size() * sizeof(double));
  return 0;
}
int orc_last_error(void *h, int *blk, int *i, int *j) {
  Solver &S = *(Solver *)h;
  *blk = S.err_b; *i = S.err_i; *j = S.err_j;
  return S.err;
}

}  // extern "C"
