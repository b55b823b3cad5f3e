// ec2d_dev.cuh -- device data layout and the pointwise physics of the
// GB300-native OpenCFD-EC2D core.
//
// Layout in HBM (one allocation per field kind and mesh level, all blocks of
// all cases of a context side by side):
//   every 2-D quantity of block b lives in a "frame" of (nx+5) x (ny+5)
//   doubles, row-major with i fastest, origin at (i,j) = (-2,-2):
//       idx(i,j) = off_b + (j+2)*P_b + (i+2),   P_b = nx+5
//   so cell, node and face arrays of the reference (whose index ranges all lie
//   in [-2, nx+2] x [-2, ny+2]) share one index map.  A multi-variable field
//   is NV such planes, plane stride F = total frame size of the level, so the
//   variable index is the slowest (structure of arrays) and warps read
//   consecutive i with unit stride.
#pragma once
#include <cstdint>

namespace ec2d {

constexpr int LAP = 2;
constexpr int LFDM = 4;
constexpr double PrT = 0.9;

enum { Scheme_UD1 = 0, Scheme_NND2 = 1, Scheme_UD3 = 2, Scheme_WENO3 = 3,
       Scheme_MUSCL2 = 4, Scheme_MUSCL3 = 5, Scheme_OMUSCL2 = 6 };
enum { Flux_SW = 1, Flux_HLL = 2, Flux_HLLC = 3, Flux_Roe = 4, Flux_VanLeer = 5, Flux_Ausm = 6 };
enum { Recon_Original = 0, Recon_Conservative = 1, Recon_Characteristic = 2 };
enum { BC_Wall = -10, BC_Farfield = -20, BC_Symmetry = -30, BC_Inlet = -40, BC_Outlet = -50 };
enum { Time_Euler1 = 1, Time_RK3 = 3, Time_LU_SGS = 0, Time_Dual = -1 };
enum { Turb_NONE = 0, Turb_BL = 1, Turb_SA = 2, Turb_SST = 3 };

// primitive planes in Lvl::q
enum { Q_D = 0, Q_U = 1, Q_V = 2, Q_T = 3, Q_P = 4, Q_C = 5, NQ = 6 };
// geometry planes in Lvl::geo
// G_VI*, G_VJ*: the face-local inverse Jacobian of the viscous terms of an i-
// or j-face, (Djy, Diy, Djx, Dix) / (Dix Djy - Djx Diy), formed at set-up
// (k_face_metrics) from the cell centres; G_SIA..G_NJ2A: the cell's face
// length and normal averaged over its two i- (j-) faces, G_VI2 / G_VJ2 their
// squared length over the cell volume (the metric factors of comput_Lvc)
enum { G_VOL = 0, G_SI = 1, G_SJ = 2, G_NI1 = 3, G_NI2 = 4, G_NJ1 = 5, G_NJ2 = 6,
       G_X = 7, G_Y = 8, G_X1 = 9, G_Y1 = 10, G_DW = 11,
       G_VIA = 12, G_VIB = 13, G_VIC = 14, G_VID = 15, G_VJA = 16, G_VJB = 17, G_VJC = 18, G_VJD = 19,
       G_SIA = 20, G_NI1A = 21, G_NI2A = 22, G_SJA = 23, G_NJ1A = 24, G_NJ2A = 25, G_VI2 = 26, G_VJ2 = 27,
       NG = 28 };
// spectral-radius / time-step planes in Lvl::lc
enum { L_CI = 0, L_CJ = 1, L_VI = 2, L_VJ = 3, L_DT = 4, NL = 5 };

struct BlkDev {
  int nx, ny, P, cas;       // node counts, frame pitch, owning case (0-based)
  long long off;            // frame offset in every plane of the level
  int fdm;                  // 1: finite-difference interior (FDM.in)
  int nsub, sub0;           // subfaces [sub0, sub0+nsub) in Lvl::sub
  int tile0;                // first extended-range tile of this block
  int lsub0, lsubn;         // fine-mesh wall faces (forces), unused on coarse levels
  int cell0;                // dense index of cell (1,1) among the level's interior cells
  int nphase;               // barrier phases of the physical boundary conditions
};

struct SubDev {
  int face, ist, iend, jst, jend, neighb, orient;
  int phase, nitem;         // physical BC: barrier phase within the block, work items
  int nbk;                  // level-global index of the neighbour block (-1: physical)
  int nface, nist, niend, njst, njend;  // the neighbour subface it reads
  int nP;                   // the neighbour block's frame pitch and offset (halo copy)
  long long noff;
  int nrm0;                 // far-field / symmetry: first node's entry in Lvl::bcn (-1: none)
};

struct CaseDev {
  double gamma, Ma, Re, Pr, Cv, Cp, cosA, sinA, p00, Tsb, Twall, p_outlet;
  double vt_inf, Kt_inf, Wt_inf, CFL, dtmax, dtmin, dt_global, T_inf;
  double xaxis, yaxis;
  double rPr, rCv, rMa, rRe;  // 1/Pr, 1/Cv, 1/Ma, 1/Re
  double rgm1;                // 1/(gamma - 1)
  double ggm1;                // gamma/(gamma - 1)
  int local_dt, pad;
};

// Everything a kernel needs about one mesh level, passed by value.
struct Lvl {
  int nblk, nvar, scheme, gscheme, flux, recon, visc, turb, level, time_method;
  int ncase, ntiles;
  long long F;              // plane stride (doubles)
  const BlkDev *blk;
  const SubDev *sub;
  const CaseDev *cs;
  const int2 *tiles;        // (block, first linear index) of the extended window's tiles
  const int2 *ctiles;       // the same over the core window (core_ij)
  int nctiles;
  double *U, *q, *amu, *amut, *res, *lc, *du, *geo, *un, *deltu, *qf, *un1;
  double *fi, *fj;          // face-flux scratch, 6 planes each
  double *tb;               // turbulence scratch planes
  double *met;              // FDM metrics Akx,Aky,Aix,Aiy,Ajac
  double *fdm;              // FDM scratch planes
  double *lu;               // LU-SGS pre-pass planes (4 NV + 10)
  double *rec;              // LU-SGS per-cell sweep records: [2 passes][ncell][4 NV + 10]
  double2 *bcn;             // unit normals of the far-field and symmetry boundary nodes
  int ncell;                // interior cells of the level (all blocks of all cases)
  double *npart;            // norm partials: per tile 2*6 doubles
  double *norms;            // per case: max[6], rms[6]
  const int *case_tile0, *case_ntile, *case_ncell;  // per case: first tile, tiles, interior cells
  unsigned *nctr;           // tiles of k_res done (the last one reduces the partials)
  int *status;              // per case: code, block, i, j
  int silent_band_edge;     // test hook: band edges of the four-lane wavefront send nothing
  int keep_amut;            // coarse level: amut is restricted from the finer level, not zeroed
};

// Items (cells, faces or nodes of a block's padded index range) per tile of
// the level's tile list, and threads per CTA of the kernels that walk it.
// Most of those kernels are chains of FP64 operations on this part, so their
// time is the chain length times the warps that share a sub-partition: 128
// gives every warp of the 2 x 48 x 48 and 2 x 24 x 24 multigrid levels its
// own sub-partition, where 256 put two on each.
constexpr int EC2D_TILE = 128;

__host__ __device__ __forceinline__ long long fidx(const BlkDev &b, int i, int j) {
  return b.off + (long long)(j + 2) * b.P + (i + 2);
}

// Tiles of a level come in two windows per block.  The extended window
// (Lvl::tiles, i = -1..nx+1, j = -1..ny+1) reaches the second ghost layer,
// where the primitives and the explicit updates are formed.  The core window
// (Lvl::ctiles, i = 0..nx, j = 0..ny) holds every face, every interior cell
// and the range of Set_Un: the face, residual, norm and record kernels walk
// it.  On two blocks of 97 x 97 nodes the extended window takes 158 tiles and
// the core window 152, so those kernels give no SM of the 152 a second CTA
// (whose warps would share sub-partitions and double the FP64 chain time).
__device__ __forceinline__ bool core_ij(const Lvl &L, int &bk, int &i, int &j) {
  const int2 t = L.ctiles[blockIdx.x];
  bk = t.x;
  const BlkDev &b = L.blk[bk];
  const int W = b.nx + 1, lin = t.y + (int)threadIdx.x;
  if (lin >= W * (b.ny + 1)) return false;
  i = lin % W;
  j = lin / W;
  return true;
}

// Reciprocal on the face and wavefront paths.  FP64: the hardware's
// approximate reciprocal (relative error e below 2^-19.9, measured over 4e7
// mantissas) refined by one third-order step of the series
// 1/x = r / (1 - e) = r (1 + e + e^2 + ...), e = 1 - x r taken exactly by an
// fma; the neglected e^3 is below 2^-59, so the result is within an ulp of
// the quotient in four dependent FP64 operations, against nine times that
// for a divide; a / b becomes a * rcp(b).  FP32: the division.
template <typename T>
__device__ __forceinline__ T rcp(T x);
template <>
__device__ __forceinline__ double rcp<double>(double x) {
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
  const double e = fma(-x, r, 1.0);
  return fma(r, fma(e, e, e), r);
}
template <>
__device__ __forceinline__ float rcp<float>(float x) { return 1.0f / x; }

// 1/sqrt(x), x > 0, FP64: the hardware's approximate reciprocal square root
// (|x y^2 - 1| below 2^-19, measured over 4e7 samples) refined by one
// third-order step of the series (1 - e)^(-1/2) = 1 + e/2 + 3e^2/8 + ...,
// e = 1 - x y^2; within an ulp of 1/sqrt(x), and x times it within two ulps
// of sqrt(x) (measured), in six dependent FP64 operations.
__device__ __forceinline__ double rsqrt_d(double x) {
  double y;
  asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
  const double e = fma(-x, y * y, 1.0);
  return fma(y, e * fma(0.375, e, 0.5), y);
}
// sqrt(x), x > 0, on the face and primitive paths: FP64 x * rsqrt_d(x)
// (within two ulps of the rounded root, seven FP64 operations against about
// ten for the correctly rounded one); FP32 the square root
template <typename T>
__device__ __forceinline__ T sqrt_p(T x);
template <>
__device__ __forceinline__ double sqrt_p<double>(double x) { return x * rsqrt_d(x); }
template <>
__device__ __forceinline__ float sqrt_p<float>(float x) { return sqrtf(x); }

// The face physics below is written once for the arithmetic type T: double
// is the reference's arithmetic (every literal T(x) is then the same double
// constant), float serves the FP32 coarse multigrid levels.

// ---- reconstruction, sub_Residual.f90:477-659 --------------------------------
template <typename T>
__device__ __forceinline__ T minmod(T a, T b) {
  if (a * b <= T(0.0)) return T(0.0);
  return (fabs(a) <= fabs(b)) ? a : b;
}

// scheme_fP (sub_Residual.f90:591-623): left state at the face between u2 and u3
template <typename T>
__device__ __forceinline__ T scheme_fp(T u1, T u2, T u3, T u4, int flag) {
  const T ep = T(1.0e-6), k3 = T(1.0) / T(3.0);
  switch (flag) {
    case Scheme_UD1: return u2;
    case Scheme_UD3: return (-u1 + T(5.0) * u2 + T(2.0) * u3) / T(6.0);
    case Scheme_NND2: return u2 + T(0.5) * minmod(u2 - u1, u3 - u2);
    case Scheme_WENO3: {
      T IS1 = (u2 - u1) * (u2 - u1), IS2 = (u3 - u2) * (u3 - u2);
      T e1 = T(1.0e-6) + IS1, e2 = T(1.0e-6) + IS2;
      T a1 = T(1.0) / (T(3.0) * (e1 * e1)), a2 = T(2.0) / (T(3.0) * (e2 * e2));
      T w1 = a1 / (a1 + a2), w2 = a2 / (a1 + a2);
      return w1 * (-u1 / T(2.0) + T(3.0) * u2 / T(2.0)) + w2 * (u2 / T(2.0) + u3 / T(2.0));
    }
    case Scheme_MUSCL2:  // k=1, b=2
      return u2 + T(0.25) * ((T(1.0) - T(1.0)) * minmod(u2 - u1, T(2.0) * (u3 - u2)) + (T(1.0) + T(1.0)) * minmod(u3 - u2, T(2.0) * (u2 - u1)));
    case Scheme_MUSCL3: {
      T up = u3 - u2, um = u2 - u1;
      T s = (T(2.0) * up * um + ep) * rcp(up * up + um * um + ep);
      return u2 + T(0.25) * s * ((T(1.0) - k3 * s) * um + (T(1.0) + k3 * s) * up);
    }
    case Scheme_OMUSCL2: {
      T r1 = (u2 - u1 + ep) / (u3 - u2 + ep), r2 = (u3 - u2 + ep) / (u4 - u3 + ep);
      T f1 = T(0.8) - T(0.175) / r2 + T(0.375) * r1;
      T f = fmax(T(0.0), fmin(fmin(T(2.0), f1), T(2.0) * r1));
      return u2 + T(0.5) * f * (u3 - u2);
    }
  }
  return T(0.0);
}
// scheme_fm (sub_Residual.f90:626-659): right state at the face between u2 and u3
template <typename T>
__device__ __forceinline__ T scheme_fm(T u1, T u2, T u3, T u4, int flag) {
  const T ep = T(1.0e-6), k3 = T(1.0) / T(3.0);
  switch (flag) {
    case Scheme_UD1: return u3;
    case Scheme_UD3: return (T(2.0) * u2 + T(5.0) * u3 - u4) / T(6.0);
    case Scheme_NND2: return u3 - T(0.5) * minmod(u3 - u2, u4 - u3);
    case Scheme_WENO3: {
      T IS1 = (u3 - u4) * (u3 - u4), IS2 = (u2 - u3) * (u2 - u3);
      T e1 = T(1.0e-6) + IS1, e2 = T(1.0e-6) + IS2;
      T a1 = T(1.0) / (T(3.0) * (e1 * e1)), a2 = T(2.0) / (T(3.0) * (e2 * e2));
      T w1 = a1 / (a1 + a2), w2 = a2 / (a1 + a2);
      return w1 * (-u4 / T(2.0) + T(3.0) * u3 / T(2.0)) + w2 * (u3 / T(2.0) + u2 / T(2.0));
    }
    case Scheme_MUSCL2: {  // k=1/3, b=1
      const T k = T(1.0) / T(3.0);
      return u3 - T(0.25) * ((T(1.0) - k) * minmod(u4 - u3, (u3 - u2)) + (T(1.0) + k) * minmod(u3 - u2, (u4 - u3)));
    }
    case Scheme_MUSCL3: {
      T up = u4 - u3, um = u3 - u2;
      T s = (T(2.0) * up * um + ep) * rcp(up * up + um * um + ep);
      return u3 - T(0.25) * s * ((T(1.0) - k3 * s) * up + (T(1.0) + k3 * s) * um);
    }
    case Scheme_OMUSCL2: {
      T r1 = (u4 - u3 + ep) / (u3 - u2 + ep), r2 = (u3 - u2 + ep) / (u2 - u1 + ep);
      T f1 = T(0.8) - T(0.175) / r2 + T(0.375) * r1;
      T f = fmax(T(0.0), fmin(fmin(T(2.0), f1), T(2.0) * r1));
      return u3 - T(0.5) * f * (u3 - u2);
    }
  }
  return T(0.0);
}

// conservative (rho, rho u, rho v, E) -> primitive (rho, u, v, p), as at the
// end of Reconstuction_conservative/Characteristic (sub_Residual.f90:526-527)
template <typename T>
__device__ __forceinline__ void cons_to_prim(const T Q[4], T W[4], T gm1) {
  W[0] = Q[0];
  W[1] = Q[1] / W[0];
  W[2] = Q[2] / W[0];
  W[3] = (Q[3] - (W[1] * Q[1] + W[2] * Q[2]) * T(0.5)) * gm1;
}

// S0[k][m]: stencil points k = i-2..i+1 (or j-2..j+1), variable m.
// Reconstuction_original/conservative/Characteristic (sub_Residual.f90:505-586)
template <typename T>
__device__ __forceinline__ void reconstruct(int recon, int scheme, T S0[4][4], T gamma,
                                            T UL[4], T UR[4]) {
  if (recon == Recon_Original) {
#pragma unroll
    for (int m = 0; m < 4; m++) {
      UL[m] = scheme_fp(S0[0][m], S0[1][m], S0[2][m], S0[3][m], scheme);
      UR[m] = scheme_fm(S0[0][m], S0[1][m], S0[2][m], S0[3][m], scheme);
    }
    return;
  }
  T gm1 = gamma - T(1.0);
  if (recon == Recon_Conservative) {
    T QL[4], QR[4];
#pragma unroll
    for (int m = 0; m < 4; m++) {
      QL[m] = scheme_fp(S0[0][m], S0[1][m], S0[2][m], S0[3][m], scheme);
      QR[m] = scheme_fm(S0[0][m], S0[1][m], S0[2][m], S0[3][m], scheme);
    }
    cons_to_prim(QL, UL, gm1);
    cons_to_prim(QR, UR, gm1);
    return;
  }
  // characteristic: project on the left eigenvectors at the arithmetic
  // mid-state, limit each characteristic variable, project back
  T Uh[4];
#pragma unroll
  for (int m = 0; m < 4; m++) Uh[m] = T(0.5) * (S0[1][m] + S0[2][m]);
  T d1 = Uh[0], u1 = Uh[1] / d1, v1 = Uh[2] / d1;
  T p1 = (Uh[3] - (Uh[1] * u1 + Uh[2] * v1) * T(0.5)) * gm1;
  T c1 = sqrt(gamma * p1 / d1);
  T V2 = (u1 * u1 + v1 * v1) * T(0.5);
  T tmp1 = gm1 / c1, tmp3 = gm1 / (c1 * c1), tmp5 = T(1.0) / (T(2.0) * c1), tmp0 = T(1.0) / tmp3;
  const T Sm[4][4] = {{V2 - tmp0, -u1, -v1, T(1.0)},
                           {-v1, T(0.0), T(1.0), T(0.0)},
                           {-u1 - V2 * tmp1, T(1.0) + tmp1 * u1, tmp1 * v1, -tmp1},
                           {-u1 + V2 * tmp1, T(1.0) - tmp1 * u1, -tmp1 * v1, tmp1}};
  T V0[4][4];
#pragma unroll
  for (int k = 0; k < 4; k++)
#pragma unroll
    for (int m = 0; m < 4; m++)
      V0[k][m] = Sm[m][0] * S0[k][0] + Sm[m][1] * S0[k][1] + Sm[m][2] * S0[k][2] + Sm[m][3] * S0[k][3];
  T VL[4], VR[4];
#pragma unroll
  for (int m = 0; m < 4; m++) {
    VL[m] = scheme_fp(V0[0][m], V0[1][m], V0[2][m], V0[3][m], scheme);
    VR[m] = scheme_fm(V0[0][m], V0[1][m], V0[2][m], V0[3][m], scheme);
  }
  const T S1[4][4] = {{-tmp3, T(0.0), -tmp5, tmp5},
                           {-tmp3 * u1, T(0.0), T(0.5) - u1 * tmp5, T(0.5) + u1 * tmp5},
                           {-tmp3 * v1, T(1.0), -v1 * tmp5, v1 * tmp5},
                           {-tmp3 * V2, v1, (c1 * u1 - V2 - tmp0) * tmp5, (c1 * u1 + V2 + tmp0) * tmp5}};
  T QL[4], QR[4];
#pragma unroll
  for (int m = 0; m < 4; m++) {
    QL[m] = S1[m][0] * VL[0] + S1[m][1] * VL[1] + S1[m][2] * VL[2] + S1[m][3] * VL[3];
    QR[m] = S1[m][0] * VR[0] + S1[m][1] * VR[1] + S1[m][2] * VR[2] + S1[m][3] * VR[3];
  }
  cons_to_prim(QL, UL, gm1);
  cons_to_prim(QR, UR, gm1);
}

// ---- 1-D face fluxes on rotated primitive states (rho, u_n, u_t, p) ----------
// Flux_Roe_1D, sub_flux_split.f90:265-324 (Harten entropy fix, delta = 0.1)
template <typename T>
__device__ __forceinline__ void flux_roe(const T *QL, const T *QR, T *F, T gamma, T ggm1) {
  const T delt = T(0.1);
  T dl = QL[0], uul = QL[1], vvl = QL[2], pl = QL[3];
  T dr = QR[0], uur = QR[1], vvr = QR[2], pr = QR[3];
  T gm1 = gamma - T(1.0);
  const T rdl = rcp(dl), rdr = rcp(dr);
  T hl = ggm1 * pl * rdl + T(0.5) * (uul * uul + vvl * vvl);
  T hr = ggm1 * pr * rdr + T(0.5) * (uur * uur + vvr * vvr);
  T Fl0 = dl * uul, Fl1 = dl * uul * uul + pl, Fl2 = dl * uul * vvl, Fl3 = uul * dl * hl;
  T Fr0 = dr * uur, Fr1 = dr * uur * uur + pr, Fr2 = dr * uur * vvr, Fr3 = uur * dr * hr;
  T tmpp = sqrt_p(dr * rdl);
  T inv = rcp(T(1.0) + tmpp);
  T avd = T(0.25) * dl * (T(1.0) + tmpp) * (T(1.0) + tmpp);
  T avu = (uul + tmpp * uur) * inv;
  T avv = (vvl + tmpp * vvr) * inv;
  T avh = (hl + tmpp * hr) * inv;
  T ava = sqrt_p(gm1 * (avh - T(0.5) * (avu * avu + avv * avv)));
  T l0 = fabs(avu - ava), l1 = fabs(avu), l3 = fabs(avu + ava);
  const T i2d = T(1.0) / (T(2.0) * delt);
  if (l0 < delt) l0 = (l0 * l0 + delt * delt) * i2d;
  if (l1 < delt) l1 = (l1 * l1 + delt * delt) * i2d;
  T l2 = l1;
  if (l3 < delt) l3 = (l3 * l3 + delt * delt) * i2d;
  T ia = rcp(ava);
  T i2aa = T(0.5) * ia * ia;
  T dp = pr - pl;
  T a0 = (avd * ava * (-uur + uul) + dp) * i2aa;
  T a1 = dr - dl - dp * (ia * ia);
  T a2 = avd * (vvr - vvl) * ia;
  T a3 = (avd * ava * (uur - uul) + dp) * i2aa;
  F[0] = T(0.5) * (Fl0 + Fr0) - T(0.5) * (l0 * a0 + l1 * a1 + l3 * a3);
  F[1] = T(0.5) * (Fl1 + Fr1) - T(0.5) * (l0 * a0 * (avu - ava) + l1 * a1 * avu + l3 * a3 * (avu + ava));
  F[2] = T(0.5) * (Fl2 + Fr2) - T(0.5) * (l0 * a0 * avv + l1 * a1 * avv + l2 * a2 + l3 * a3 * avv);
  F[3] = T(0.5) * (Fl3 + Fr3) - T(0.5) * (l0 * a0 * (avh - avu * ava) + l1 * a1 * T(0.5) * (avu * avu + avv * avv) +
                                    l2 * a2 * avv + l3 * a3 * (avh + avu * ava));
}

// Flux_Ausm_1Da (AUSM+), sub_flux_split.f90:195-261
template <typename T>
__device__ __forceinline__ void flux_ausm(const T *QL, const T *QR, T *F, T gamma, T ggm1) {
  T dl = QL[0], uul = QL[1], vvl = QL[2], pl = QL[3];
  T dr = QR[0], uur = QR[1], vvr = QR[2], pr = QR[3];
  const T rdl = rcp(dl), rdr = rcp(dr);
  const T prl = pl * rdl, prr = pr * rdr;  // p / rho
  T hl = ggm1 * prl + T(0.5) * (uul * uul + vvl * vvl);
  T hr = ggm1 * prr + T(0.5) * (uur * uur + vvr * vvr);
  T al = sqrt_p(gamma * prl), ar = sqrt_p(gamma * prr);
  T a = T(0.5) * (al + ar);
  T ia = rcp(a);
  T Ml = uul * ia, Mr = uur * ia;
  T Mp4, Mm4, Pp5, Pm5;
  T ml2 = Ml * Ml - T(1.0), mr2 = Mr * Mr - T(1.0);
  if (fabs(Ml) >= T(1.0)) { Mp4 = T(0.5) * (Ml + fabs(Ml)); Pp5 = T(0.5) * (Ml + fabs(Ml)) / Ml; }
  else { Mp4 = T(0.25) * (Ml + T(1.0)) * (Ml + T(1.0)) + T(0.125) * ml2 * ml2;
         Pp5 = T(0.25) * (Ml + T(1.0)) * (Ml + T(1.0)) * (T(2.0) - Ml) + T(3.0) * Ml * ml2 * ml2 / T(16.0); }
  if (fabs(Mr) >= T(1.0)) { Mm4 = T(0.5) * (Mr - fabs(Mr)); Pm5 = T(0.5) * (Mr - fabs(Mr)) / Mr; }
  else { Mm4 = -T(0.25) * (Mr - T(1.0)) * (Mr - T(1.0)) - T(0.125) * mr2 * mr2;
         Pm5 = T(0.25) * (Mr - T(1.0)) * (Mr - T(1.0)) * (T(2.0) + Mr) - T(3.0) * Mr * mr2 * mr2 / T(16.0); }
  T M = Mp4 + Mm4;
  T xm = dl * a * fmax(T(0.0), M) + dr * a * fmin(T(0.0), M);
  T dm = (M >= T(0.0)) ? a * fabs(M) * dl : a * fabs(M) * dr;
  T p = pl * Pp5 + pr * Pm5;
  F[0] = xm;  // 0.5 xm (1 + 1) - 0.5 dm (1 - 1): the same value for finite xm, dm
  F[1] = T(0.5) * xm * (uul + uur) - T(0.5) * dm * (uur - uul) + p;
  F[2] = T(0.5) * xm * (vvl + vvr) - T(0.5) * dm * (vvr - vvl);
  F[3] = T(0.5) * xm * (hl + hr) - T(0.5) * dm * (hr - hl);
}

// Flux_Van_Leer_1Da, sub_flux_split.f90:139-189
template <typename T>
__device__ __forceinline__ void flux_vanleer(const T *QL, const T *QR, T *F, T gamma) {
  T dl = QL[0], uul = QL[1], vvl = QL[2], pl = QL[3];
  T dr = QR[0], uur = QR[1], vvr = QR[2], pr = QR[3];
  T gm1 = gamma - T(1.0);
  T al = sqrt(gamma * pl / dl), ar = sqrt(gamma * pr / dr);
  T Ml = uul / al, Mr = uur / ar;
  T fp0 = 0, fp1 = 0, fp2 = 0, fp3 = 0, fm0 = 0, fm1 = 0, fm2 = 0, fm3 = 0;
  if (Ml >= T(1.0)) {
    fp0 = dl * uul; fp1 = dl * uul * uul + pl; fp2 = dl * uul * vvl;
    fp3 = uul * (gamma * pl / gm1 + T(0.5) * dl * (uul * uul + vvl * vvl));
  } else if (fabs(Ml) < T(1.0)) {
    T tmp0 = dl * al * (T(0.25) * (T(1.0) + Ml) * (T(1.0) + Ml));
    T w = gm1 * uul + T(2.0) * al;
    fp0 = tmp0; fp1 = tmp0 * w / gamma; fp2 = tmp0 * vvl;
    fp3 = tmp0 * (w * w * T(0.5) / (gamma * gamma - T(1.0)) + T(0.5) * (vvl * vvl));
  }
  if (Mr >= T(1.0)) {
  } else if (fabs(Mr) < T(1.0)) {
    T tmp0 = dr * ar * (-T(0.25) * (Mr - T(1.0)) * (Mr - T(1.0)));
    T w = gm1 * uur - T(2.0) * ar;
    fm0 = tmp0; fm1 = tmp0 * w / gamma; fm2 = tmp0 * vvr;
    fm3 = tmp0 * (w * w * T(0.5) / (gamma * gamma - T(1.0)) + T(0.5) * (vvr * vvr));
  } else if (Mr <= -T(1.0)) {
    fm0 = dr * uur; fm1 = dr * uur * uur + pr; fm2 = dr * uur * vvr;
    fm3 = uur * (gamma * pr / gm1 + T(0.5) * dr * (uur * uur + vvr * vvr));
  }
  F[0] = fp0 + fm0; F[1] = fp1 + fm1; F[2] = fp2 + fm2; F[3] = fp3 + fm3;
}

// Flux_steger_warming_1Da, sub_flux_split.f90:99-136
template <typename T>
__device__ __forceinline__ void flux_sw(const T *QL, const T *QR, T *F, T gamma) {
  T dl = QL[0], uul = QL[1], vvl = QL[2], pl = QL[3];
  T dr = QR[0], uur = QR[1], vvr = QR[2], pr = QR[3];
  T al = sqrt(gamma * pl / dl), ar = sqrt(gamma * pr / dr);
  T gm1 = gamma - T(1.0);
  T tmp1 = T(2.0) * gm1, tmp3 = (T(3.0) - gamma) / (T(2.0) * gm1);
  T E1P = (uul + fabs(uul)) * T(0.5), E2P = (uul - al + fabs(uul - al)) * T(0.5), E3P = (uul + al + fabs(uul + al)) * T(0.5);
  T t0 = dl / (T(2.0) * gamma);
  T p0 = t0 * (tmp1 * E1P + E2P + E3P);
  T p1 = t0 * (tmp1 * E1P * uul + E2P * (uul - al) + E3P * (uul + al));
  T p2 = t0 * (tmp1 * E1P * vvl + E2P * vvl + E3P * vvl);
  T p3 = t0 * (E1P * gm1 * (uul * uul + vvl * vvl) + E2P * ((uul - al) * (uul - al) + vvl * vvl) * T(0.5) +
                    E3P * ((uul + al) * (uul + al) + vvl * vvl) * T(0.5) + tmp3 * al * al * (E2P + E3P));
  T E1M = (uur - fabs(uur)) * T(0.5), E2M = (uur - ar - fabs(uur - ar)) * T(0.5), E3M = (uur + ar - fabs(uur + ar)) * T(0.5);
  t0 = dr / (T(2.0) * gamma);
  T m0 = t0 * (tmp1 * E1M + E2M + E3M);
  T m1 = t0 * (tmp1 * E1M * uur + E2M * (uur - ar) + E3M * (uur + ar));
  T m2 = t0 * (tmp1 * E1M * vvr + E2M * vvr + E3M * vvr);
  T m3 = t0 * (E1M * gm1 * (uur * uur + vvr * vvr) + E2M * ((uur - ar) * (uur - ar) + vvr * vvr) * T(0.5) +
                    E3M * ((uur + ar) * (uur + ar) + vvr * vvr) * T(0.5) + tmp3 * ar * ar * (E2M + E3M));
  F[0] = p0 + m0; F[1] = p1 + m1; F[2] = p2 + m2; F[3] = p3 + m3;
}

// Flux_HLL_HLLC_1D, sub_flux_split.f90:16-93
template <typename T>
__device__ __forceinline__ void flux_hll(const T *QL, const T *QR, T *F, T gamma, bool hllc) {
  T dl = QL[0], uul = QL[1], vvl = QL[2], pl = QL[3];
  T dr = QR[0], uur = QR[1], vvr = QR[2], pr = QR[3];
  T gm1 = gamma - T(1.0);
  T UL[4] = {dl, dl * uul, dl * vvl, pl / gm1 + dl * (uul * uul + vvl * vvl) * T(0.5)};
  T UR[4] = {dr, dr * uur, dr * vvr, pr / gm1 + dr * (uur * uur + vvr * vvr) * T(0.5)};
  T al = sqrt(gamma * pl / dl), ar = sqrt(gamma * pr / dr);
  T p_pvrs = T(0.5) * (pl + pr) - (uur - uul) * (dl + dr) * (al + ar) * T(0.125);
  T p_star = fmax(T(0.0), p_pvrs);
  T g2 = (gamma + T(1.0)) / (T(2.0) * gamma);
  T qql = (p_star <= pl) ? T(1.0) : sqrt(T(1.0) + g2 * (p_star / pl - T(1.0)));
  T qqr = (p_star <= pr) ? T(1.0) : sqrt(T(1.0) + g2 * (p_star / pr - T(1.0)));
  T Sl = uul - al * qql, Sr = uur + ar * qqr;
  T Fl[4] = {UL[1], UL[1] * uul + pl, UL[2] * uul, uul * (UL[3] + pl)};
  T Fr[4] = {UR[1], UR[1] * uur + pr, UR[2] * uur, uur * (UR[3] + pr)};
  if (!hllc) {
    if (Sl >= 0) { for (int m = 0; m < 4; m++) F[m] = Fl[m]; }
    else if (Sr <= 0) { for (int m = 0; m < 4; m++) F[m] = Fr[m]; }
    else { T inv = T(1.0) / (Sr - Sl);
      for (int m = 0; m < 4; m++) F[m] = (Sr * Fl[m] - Sl * Fr[m] + Sl * Sr * (UR[m] - UL[m])) * inv; }
    return;
  }
  T S_star = (pr - pl + dl * uul * (Sl - uul) - dr * uur * (Sr - uur)) / (dl * (Sl - uul) - dr * (Sr - uur));
  if (Sl >= 0) { for (int m = 0; m < 4; m++) F[m] = Fl[m]; return; }
  if (Sr <= 0) { for (int m = 0; m < 4; m++) F[m] = Fr[m]; return; }
  if (S_star >= 0) {
    T tmpl = dl * (Sl - uul) / (Sl - S_star);
    T tmp = UL[3] / dl + (S_star - uul) * (S_star + pl / (dl * (Sl - uul)));
    F[0] = Fl[0] + Sl * (tmpl - UL[0]);
    F[1] = Fl[1] + Sl * (tmpl * S_star - UL[1]);
    F[2] = Fl[2] + Sl * (tmpl * vvl - UL[2]);
    F[3] = Fl[3] + Sl * (tmpl * tmp - UL[3]);
  } else {
    T tmpr = dr * (Sr - uur) / (Sr - S_star);
    T tmp = UR[3] / dr + (S_star - uur) * (S_star + pr / (dr * (Sr - uur)));
    F[0] = Fr[0] + Sr * (tmpr - UR[0]);
    F[1] = Fr[1] + Sr * (tmpr * S_star - UR[1]);
    F[2] = Fr[2] + Sr * (tmpr * vvr - UR[2]);
    F[3] = Fr[3] + Sr * (tmpr * tmp - UR[3]);
  }
}

template <typename T>
__device__ __forceinline__ void face_flux(int iflux, const T *QL, const T *QR, T *F, T gamma, T ggm1) {
  switch (iflux) {
    case Flux_Roe: flux_roe(QL, QR, F, gamma, ggm1); return;
    case Flux_Ausm: flux_ausm(QL, QR, F, gamma, ggm1); return;
    case Flux_VanLeer: flux_vanleer(QL, QR, F, gamma); return;
    case Flux_SW: flux_sw(QL, QR, F, gamma); return;
    case Flux_HLL: flux_hll(QL, QR, F, gamma, false); return;
    case Flux_HLLC: flux_hll(QL, QR, F, gamma, true); return;
  }
  F[0] = F[1] = F[2] = F[3] = T(0.0);
}

// viscous stress and heat flux through a face from the face-local 2x2
// Jacobian of cell centres, sub_Residual.f90:313-343 / 419-450
template <typename T>
__device__ __forceinline__ void viscous_face(T Dix, T Diy, T Djx, T Djy, T Diu, T Div,
                                             T DiT, T Dju, T Djv, T DjT, T Amu1, T Amk1,
                                             T u1, T v1, T n1, T n2, T s, T &F2,
                                             T &F3, T &F4) {
  T Ds = rcp(Dix * Djy - Djx * Diy);
  T ux = (Diu * Djy - Dju * Diy) * Ds, vx = (Div * Djy - Djv * Diy) * Ds, Tx = (DiT * Djy - DjT * Diy) * Ds;
  T uy = (-Diu * Djx + Dju * Dix) * Ds, vy = (-Div * Djx + Djv * Dix) * Ds, Ty = (-DiT * Djx + DjT * Dix) * Ds;
  T t11 = ((T(4.0) / T(3.0)) * ux - (T(2.0) / T(3.0)) * vy) * Amu1;
  T t22 = ((T(4.0) / T(3.0)) * vy - (T(2.0) / T(3.0)) * ux) * Amu1;
  T t12 = (uy + vx) * Amu1;
  T E1 = u1 * t11 + v1 * t12 + Amk1 * Tx, E2 = u1 * t12 + v1 * t22 + Amk1 * Ty;
  F2 += (t11 * n1 + t12 * n2) * s;
  F3 += (t12 * n1 + t22 * n2) * s;
  F4 += (E1 * n1 + E2 * n2) * s;
}

// the same from the face's precomputed inverse Jacobian (A, B, C, D) =
// (Djy, Diy, Djx, Dix) / (Dix Djy - Djx Diy): u_x = Diu A - Dju B,
// u_y = Dju D - Diu C
template <typename T>
__device__ __forceinline__ void viscous_face_m(T A, T B, T C, T D, T Diu, T Div, T DiT, T Dju, T Djv, T DjT,
                                               T Amu1, T Amk1, T u1, T v1, T n1, T n2, T s, T &F2, T &F3, T &F4) {
  T ux = fma(Diu, A, -Dju * B), vx = fma(Div, A, -Djv * B), Tx = fma(DiT, A, -DjT * B);
  T uy = fma(Dju, D, -Diu * C), vy = fma(Djv, D, -Div * C), Ty = fma(DjT, D, -DiT * C);
  T t11 = ((T(4.0) / T(3.0)) * ux - (T(2.0) / T(3.0)) * vy) * Amu1;
  T t22 = ((T(4.0) / T(3.0)) * vy - (T(2.0) / T(3.0)) * ux) * Amu1;
  T t12 = (uy + vx) * Amu1;
  T E1 = u1 * t11 + v1 * t12 + Amk1 * Tx, E2 = u1 * t12 + v1 * t22 + Amk1 * Ty;
  F2 += (t11 * n1 + t12 * n2) * s;
  F3 += (t12 * n1 + t22 * n2) * s;
  F4 += (E1 * n1 + E2 * n2) * s;
}

// device-side error record (first error of a case wins)
__device__ __forceinline__ void set_status(int *st, int code, int blk, int i, int j) {
  if (atomicCAS(st, 0, code) == 0) { st[1] = blk; st[2] = i; st[3] = j; }
}

}  // namespace ec2d
