// k_residual.cu -- the residual of sub_Residual.f90 on the GPU.
//
// One residual evaluation of a mesh level (Comput_Residual_one_mesh,
// sub_Residual.f90:13-107) is a chain of launches over all blocks of all cases:
//   k_prim      primitives d,u,v,T,p (+c, Sutherland mu)       comput_duvtpckw + get_viscous
//   k_flux_i/j  reconstruction + Riemann flux + viscous stress  Residual_FVM face loops
//   k_res       flux differences, spectral radii, time step    Residual_FVM:460-468, comput_Lvc, comput_dt
//   k_norm_*    max / RMS residual norms, deterministic order  sub_Residual.f90:72-106
// Work is distributed by EC2D_TILE-item tiles of each block's extended index
// range [-1,nx+1] x [-1,ny+1] (k_prim: the primitives of both ghost layers)
// or of its core range [0,nx] x [0,ny] (the face, residual and norm kernels,
// core_ij); a kernel maps the tile item to (i,j) and keeps the items that lie
// in its own index range.
#include "ec2d_dev.cuh"
#include "ec2d_internal.h"

namespace ec2d {

constexpr int TILE = EC2D_TILE;

__device__ __forceinline__ bool tile_ij(const Lvl &L, int &bk, int &i, int &j) {
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

// comput_duvtpckw (sub_Residual.f90:114-152) + get_viscous (:670-689) + Amu_t=0 (:172)
__global__ void __launch_bounds__(TILE) k_prim(Lvl L) {
  int bk, i, j;
  if (!tile_ij(L, bk, i, j)) return;
  const BlkDev &b = L.blk[bk];
  const CaseDev &c = L.cs[b.cas];
  long long id = fidx(b, i, j);
  const long long F = L.F;
  double d = L.U[id], ru = L.U[F + id], rv = L.U[2 * F + id], E = L.U[3 * F + id];
  const double rd = rcp(d);
  double uu = ru * rd, v = rv * rd;
  double T = (E - 0.5 * d * (uu * uu + v * v)) * (rd * c.rCv);
  double p = c.p00 * d * T;
  const double sT = T > 0.0 ? sqrt_p(T) : sqrt(T);  // the reference's sqrt, NaN for T < 0
  L.q[Q_D * F + id] = d;
  L.q[Q_U * F + id] = uu;
  L.q[Q_V * F + id] = v;
  L.q[Q_T * F + id] = T;
  L.q[Q_P * F + id] = p;
  bool interior = (i >= 1 && i <= b.nx - 1 && j >= 1 && j <= b.ny - 1);
  if (interior) {
    if (!(T >= 1.0e-5)) set_status(L.status + 4 * b.cas, 3, bk, i, j);
    L.q[Q_C * F + id] = sT * c.rMa;
  }
  if (L.visc) {
    if (i >= 0 && i <= b.nx && j >= 0 && j <= b.ny)
      L.amu[id] = c.rRe * (1.0 + c.Tsb) * (T * sT) * rcp(c.Tsb + T);  // T^1.5 = T sqrt(T)
    if (!L.keep_amut) L.amut[id] = 0.0;
  }
}

__device__ __forceinline__ bool in_fdm_core(const BlkDev &b, int i, int j) {
  return b.fdm && (i >= LFDM + 2 && i <= b.nx - LFDM - 1) && (j >= LFDM + 2 && j <= b.ny - LFDM - 1);
}

// i-direction face loop of Residual_FVM (sub_Residual.f90:238-346): face (i,j),
// i=1..nx, j=1..ny-1, between cells (i-1,j) and (i,j).
template <typename T>
__global__ void __launch_bounds__(TILE) k_flux_i(Lvl L) {
  int bk, i, j;
  if (!core_ij(L, bk, i, j)) return;
  const BlkDev &b = L.blk[bk];
  if (i < 1 || i > b.nx || j < 1 || j > b.ny - 1) return;
  if (in_fdm_core(b, i, j)) return;
  const CaseDev &c = L.cs[b.cas];
  const long long F = L.F;
  long long id = fidx(b, i, j);
  T si = (T)L.geo[G_SI * F + id], n1 = (T)L.geo[G_NI1 * F + id], n2 = (T)L.geo[G_NI2 * F + id];
  T S0[4][4], UL[4], UR[4];
  if (L.recon == Recon_Original) {
#pragma unroll
    for (int k = 0; k < 4; k++) {
      long long s = id + (k - 2);
      S0[k][0] = (T)L.q[Q_D * F + s]; S0[k][1] = (T)L.q[Q_U * F + s];
      S0[k][2] = (T)L.q[Q_V * F + s]; S0[k][3] = (T)L.q[Q_P * F + s];
    }
  } else {
#pragma unroll
    for (int k = 0; k < 4; k++)
#pragma unroll
      for (int m = 0; m < 4; m++) S0[k][m] = (T)L.U[m * F + id + (k - 2)];
  }
  reconstruct(L.recon, L.scheme, S0, (T)c.gamma, UL, UR);
  T QL[4] = {UL[0], UL[1] * n1 + UL[2] * n2, -UL[1] * n2 + UL[2] * n1, UL[3]};
  T QR[4] = {UR[0], UR[1] * n1 + UR[2] * n2, -UR[1] * n2 + UR[2] * n1, UR[3]};
  T Fl[4];
  face_flux(L.flux, QL, QR, Fl, (T)c.gamma, (T)c.ggm1);
  T F0 = -Fl[0] * si, F1 = -(Fl[1] * n1 - Fl[2] * n2) * si, F2 = -(Fl[1] * n2 + Fl[2] * n1) * si, F3 = -Fl[3] * si;
  if (L.visc) {
    long long w = id - 1, nN = id + b.P, nS = id - b.P;
    T Amu1, Amk1;
    if (i == 1) {
      Amu1 = (T)L.amu[id] + (T)L.amut[id];
      Amk1 = (T)c.Cp * ((T)L.amu[id] * (T)c.rPr + (T)L.amut[id] * (T)(1.0 / PrT));
    } else if (i == b.nx) {
      Amu1 = (T)L.amu[w] + (T)L.amut[w];
      Amk1 = (T)c.Cp * ((T)L.amu[w] * (T)c.rPr + (T)L.amut[w] * (T)(1.0 / PrT));
    } else {
      Amu1 = ((T)L.amu[w] + (T)L.amu[id] + (T)L.amut[w] + (T)L.amut[id]) * T(0.5);
      Amk1 = (T)c.Cp * (((T)L.amu[w] + (T)L.amu[id]) * (T)c.rPr + ((T)L.amut[w] + (T)L.amut[id]) * (T)(1.0 / PrT)) * T(0.5);
    }
    const double *uu = L.q + Q_U * F, *vv = L.q + Q_V * F, *TT = L.q + Q_T * F;
    const double *g = L.geo + id;
    T Diu = (T)uu[id] - (T)uu[w], Div = (T)vv[id] - (T)vv[w], DiT = (T)TT[id] - (T)TT[w];
    T Dju = ((T)uu[nN - 1] + (T)uu[nN] - (T)uu[nS - 1] - (T)uu[nS]) * T(0.25);
    T Djv = ((T)vv[nN - 1] + (T)vv[nN] - (T)vv[nS - 1] - (T)vv[nS]) * T(0.25);
    T DjT = ((T)TT[nN - 1] + (T)TT[nN] - (T)TT[nS - 1] - (T)TT[nS]) * T(0.25);
    T u1 = ((T)uu[id] + (T)uu[w]) * T(0.5), v1 = ((T)vv[id] + (T)vv[w]) * T(0.5);
    viscous_face_m((T)g[G_VIA * F], (T)g[G_VIB * F], (T)g[G_VIC * F], (T)g[G_VID * F], Diu, Div, DiT, Dju, Djv, DjT,
                   Amu1, Amk1, u1, v1, n1, n2, si, F1, F2, F3);
  }
  L.fi[id] = F0; L.fi[F + id] = F1; L.fi[2 * F + id] = F2; L.fi[3 * F + id] = F3;
}

// j-direction face loop of Residual_FVM (sub_Residual.f90:352-455): face (i,j),
// i=1..nx-1, j=1..ny, between cells (i,j-1) and (i,j).
template <typename T>
__global__ void __launch_bounds__(TILE) k_flux_j(Lvl L) {
  int bk, i, j;
  if (!core_ij(L, bk, i, j)) return;
  const BlkDev &b = L.blk[bk];
  if (i < 1 || i > b.nx - 1 || j < 1 || j > b.ny) return;
  if (in_fdm_core(b, i, j)) return;
  const CaseDev &c = L.cs[b.cas];
  const long long F = L.F;
  const long long P = b.P;
  long long id = fidx(b, i, j);
  T sj = (T)L.geo[G_SJ * F + id], n1 = (T)L.geo[G_NJ1 * F + id], n2 = (T)L.geo[G_NJ2 * F + id];
  T S0[4][4], UL[4], UR[4];
  int scheme = L.scheme;
  if (L.recon == Recon_Original) {
    scheme = L.gscheme;  // the reference passes the global Iflag_Scheme here (sub_Residual.f90:367)
#pragma unroll
    for (int k = 0; k < 4; k++) {
      long long s = id + (k - 2) * P;
      S0[k][0] = (T)L.q[Q_D * F + s]; S0[k][1] = (T)L.q[Q_U * F + s];
      S0[k][2] = (T)L.q[Q_V * F + s]; S0[k][3] = (T)L.q[Q_P * F + s];
    }
  } else {
#pragma unroll
    for (int k = 0; k < 4; k++)
#pragma unroll
      for (int m = 0; m < 4; m++) S0[k][m] = (T)L.U[m * F + id + (k - 2) * P];
  }
  reconstruct(L.recon, scheme, S0, (T)c.gamma, UL, UR);
  T QL[4] = {UL[0], UL[1] * n1 + UL[2] * n2, -UL[1] * n2 + UL[2] * n1, UL[3]};
  T QR[4] = {UR[0], UR[1] * n1 + UR[2] * n2, -UR[1] * n2 + UR[2] * n1, UR[3]};
  T Fl[4];
  face_flux(L.flux, QL, QR, Fl, (T)c.gamma, (T)c.ggm1);
  T F0 = -Fl[0] * sj, F1 = -(Fl[1] * n1 - Fl[2] * n2) * sj, F2 = -(Fl[1] * n2 + Fl[2] * n1) * sj, F3 = -Fl[3] * sj;
  if (L.visc) {
    long long s = id - P;
    T Amu1, Amk1;
    if (j == 1) {
      Amu1 = (T)L.amu[id] + (T)L.amut[id];
      Amk1 = (T)c.Cp * ((T)L.amu[id] * (T)c.rPr + (T)L.amut[id] * (T)(1.0 / PrT));
    } else if (j == b.ny) {
      Amu1 = (T)L.amu[s] + (T)L.amut[s];
      Amk1 = (T)c.Cp * ((T)L.amu[s] * (T)c.rPr + (T)L.amut[s] * (T)(1.0 / PrT));
    } else {
      Amu1 = ((T)L.amu[id] + (T)L.amu[s] + (T)L.amut[id] + (T)L.amut[s]) * T(0.5);
      Amk1 = (T)c.Cp * (((T)L.amu[s] + (T)L.amu[id]) * (T)c.rPr + ((T)L.amut[s] + (T)L.amut[id]) * (T)(1.0 / PrT)) * T(0.5);
    }
    const double *uu = L.q + Q_U * F, *vv = L.q + Q_V * F, *TT = L.q + Q_T * F;
    const double *g = L.geo + id;
    T Diu = ((T)uu[s + 1] + (T)uu[id + 1] - (T)uu[s - 1] - (T)uu[id - 1]) * T(0.25);
    T Div = ((T)vv[s + 1] + (T)vv[id + 1] - (T)vv[s - 1] - (T)vv[id - 1]) * T(0.25);
    T DiT = ((T)TT[s + 1] + (T)TT[id + 1] - (T)TT[s - 1] - (T)TT[id - 1]) * T(0.25);
    T Dju = (T)uu[id] - (T)uu[s], Djv = (T)vv[id] - (T)vv[s], DjT = (T)TT[id] - (T)TT[s];
    T u1 = ((T)uu[id] + (T)uu[s]) * T(0.5), v1 = ((T)vv[id] + (T)vv[s]) * T(0.5);
    viscous_face_m((T)g[G_VJA * F], (T)g[G_VJB * F], (T)g[G_VJC * F], (T)g[G_VJD * F], Diu, Div, DiT, Dju, Djv, DjT,
                   Amu1, Amk1, u1, v1, n1, n2, sj, F1, F2, F3);
  }
  L.fj[id] = F0; L.fj[F + id] = F1; L.fj[2 * F + id] = F2; L.fj[3 * F + id] = F3;
}

// Norm reductions.  max |Res| is reduced on the bit patterns: for
// non-negative doubles the order of the patterns as signed 64-bit integers is
// the order of the values, so the maxima run on the integer pipes (an FP64
// warp instruction holds its sub-partition for 64 cycles on this part) and
// are exact in any order.  Sums of Res^2 run in a fixed tree order.
__device__ __forceinline__ long long warp_max_bits(long long a) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) a = max(a, __shfl_xor_sync(0xffffffffu, a, o));
  return a;
}
__device__ __forceinline__ double warp_sum(double q) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) q += __shfl_xor_sync(0xffffffffu, q, o);
  return q;
}

// NV variables (4 or 8) reduced over a warp at once by a transposed
// butterfly: at each of the first log2(NV) exchanges a lane keeps half of the
// variables it carries and combines them with its partner's copies, so one
// instruction serves several variables (four sums take 2 + 1 + 3 FP64 adds per
// lane instead of 4 x 5, eight take 4 + 2 + 1 + 2 instead of 8 x 5).  Lane l
// ends with the warp's value of variable l / (32 / NV); every lane of that
// group holds the same bits (each exchange adds the same two operands on both
// sides), and the order of the operations is fixed.
struct OpMax { __device__ long long operator()(long long a, long long b) const { return max(a, b); } };
struct OpAdd { __device__ double operator()(double a, double b) const { return a + b; } };
template <int NV, typename T, typename Op>
__device__ __forceinline__ T warp_reduce_vars(const T (&v)[NV], Op op) {
  static_assert(NV == 4 || NV == 8, "four or eight variables");
  constexpr int R = NV == 4 ? 2 : 3;  // exchanges that halve the variables
  const int lane = threadIdx.x & 31;
  T c[NV];
#pragma unroll
  for (int k = 0; k < NV; k++) c[k] = v[k];
#pragma unroll
  for (int r = 0; r < R; r++) {
    const int o = 16 >> r, n = NV >> (r + 1);  // lanes o apart; variables kept
    const bool hi = lane & o;
#pragma unroll
    for (int k = 0; k < NV / 2; k++) {
      if (k < n) {
        const T keep = hi ? c[n + k] : c[k], send = hi ? c[k] : c[n + k];
        c[k] = op(keep, __shfl_xor_sync(0xffffffffu, send, o));
      }
    }
  }
#pragma unroll
  for (int o = 32 / NV / 2; o > 0; o >>= 1) c[0] = op(c[0], __shfl_xor_sync(0xffffffffu, c[0], o));
  return c[0];
}

// one warp's max |Res| bits and sum Res^2 of NV variables into the CTA's
// shared arrays (column w)
template <int NV, int NW>
__device__ __forceinline__ void warp_partials(bool act, const double *vres, int nv, long long (*smax)[NW],
                                              double (*ssum)[NW]) {
  long long a[NV];
  double q[NV];
#pragma unroll
  for (int m = 0; m < NV; m++) {
    // variables past the sixth are zero at compile time (no FP64 work)
    const double r = (m < 6 && act && m < nv) ? vres[m < 6 ? m : 0] : 0.0;
    a[m] = __double_as_longlong(fabs(r));
    q[m] = m < 6 ? r * r : 0.0;
  }
  const long long am = warp_reduce_vars<NV>(a, OpMax());
  const double qs = warp_reduce_vars<NV>(q, OpAdd());
  const int lane = threadIdx.x & 31, g = lane / (32 / NV);
  if (lane % (32 / NV) == 0 && g < nv) {
    smax[g][threadIdx.x >> 5] = am;
    ssum[g][threadIdx.x >> 5] = qs;
  }
}

// one CTA's partials: per variable the max |Res| and sum Res^2 of its cells
// (NT threads in the CTA)
template <int NT = TILE>
__device__ __forceinline__ void tile_partials(const Lvl &L, bool act, const double *vres) {
  __shared__ long long smax[6][NT / 32];
  __shared__ double ssum[6][NT / 32];
  const int nv = L.nvar;
  if (nv <= 4) warp_partials<4, NT / 32>(act, vres, nv, smax, ssum);
  else warp_partials<8, NT / 32>(act, vres, nv, smax, ssum);
  __syncthreads();
  if (threadIdx.x < 6) {
    const int m = threadIdx.x;
    long long a = 0;
    double q = 0.0;
    if (m < nv)
      for (int k = 0; k < NT / 32; k++) { a = max(a, smax[m][k]); q += ssum[m][k]; }
    L.npart[(size_t)blockIdx.x * 12 + m] = __longlong_as_double(a);
    L.npart[(size_t)blockIdx.x * 12 + 6 + m] = q;
  }
}

// per case and quantity (max[6], rms[6]) from the tile partials: one warp per
// (case, quantity), lanes over tiles with four loads in flight per lane (four
// accumulators in a fixed order), then the warp tree
__device__ __forceinline__ void final_norm(const Lvl &L, int cs, int m) {
  const int lane = threadIdx.x & 31;
  const int nt = L.case_ntile[cs];
  const double *p = L.npart + (size_t)L.case_tile0[cs] * 12 + m;
  double out = 0.0;
  if (m < 6) {
    long long a[4] = {0, 0, 0, 0};
    for (int t = lane; t < nt; t += 128) {
#pragma unroll
      for (int k = 0; k < 4; k++)
        if (t + 32 * k < nt) a[k] = max(a[k], __double_as_longlong(p[(size_t)(t + 32 * k) * 12]));
    }
    out = __longlong_as_double(warp_max_bits(max(max(a[0], a[1]), max(a[2], a[3]))));
  } else {
    double q[4] = {0.0, 0.0, 0.0, 0.0};
    for (int t = lane; t < nt; t += 128) {
#pragma unroll
      for (int k = 0; k < 4; k++)
        if (t + 32 * k < nt) q[k] += p[(size_t)(t + 32 * k) * 12];
    }
    const double s = warp_sum((q[0] + q[1]) + (q[2] + q[3]));
    out = (m - 6 < L.nvar) ? sqrt(s / (1.0 * L.case_ncell[cs])) : 0.0;
  }
  if (lane == 0) L.norms[cs * 12 + m] = out;
}

// flux differences (sub_Residual.f90:460-468), comput_Lvc (sub_NS_singlegrid.f90:352-388)
// and comput_dt (sub_NS_singlegrid.f90:324-348) for interior cells
// NORM: also the tile's partial norms of Res (the work of k_norm_partial,
// same cells, same reduction tree, so the norms are bit-identical); only when
// no later kernel of the residual stage changes Res (no FDM patch, no
// dual-time term)
// post: RES_ADD_FORCE (Res += QF once the norms are taken), RES_FORCE_FN
// (QF -= Res), RES_SET_UN (Un = U over 0..nx, 0..ny): the multigrid steps
// that follow a residual evaluation, done in the same pass
template <bool NORM, bool FINAL>
__global__ void __launch_bounds__(TILE) k_res(Lvl L, int post) {
  int bk, i, j;
  bool act = core_ij(L, bk, i, j);
  if (act) {
    const BlkDev &b0 = L.blk[bk];
    if ((post & RES_SET_UN) && i >= 0 && i <= b0.nx && j >= 0 && j <= b0.ny) {
      const long long id = fidx(b0, i, j);
#pragma unroll
      for (int m = 0; m < 4; m++) L.un[m * L.F + id] = L.U[m * L.F + id];
    }
    act = i >= 1 && i <= b0.nx - 1 && j >= 1 && j <= b0.ny - 1;
  }
  if (!NORM && !act) return;
  double vres[6] = {0, 0, 0, 0, 0, 0};
  if (act) {
    const BlkDev &b = L.blk[bk];
    const CaseDev &c = L.cs[b.cas];
    const long long F = L.F, P = b.P;
    long long id = fidx(b, i, j);
    bool fdm = b.fdm && (i >= LFDM + 1 && i <= b.nx - LFDM - 1) && (j >= LFDM + 1 && j <= b.ny - LFDM - 1);
    if (!fdm) {
#pragma unroll
      for (int m = 0; m < 4; m++) {
        double r = L.fi[m * F + id + 1] - L.fi[m * F + id] + L.fj[m * F + id + P] - L.fj[m * F + id];
        vres[m] = r;
        if (post & (RES_ADD_FORCE | RES_FORCE_FN)) {
          const double qf = L.qf[m * F + id];
          if (post & RES_FORCE_FN) L.qf[m * F + id] = qf - r;
          if (post & RES_ADD_FORCE) r = r + qf;
        }
        L.res[m * F + id] = r;
      }
    }
    if (NORM)
#pragma unroll
      for (int m = 4; m < 6; m++)
        if (m < L.nvar) vres[m] = L.res[m * F + id];  // constant indices: vres stays in registers
    const double *g = L.geo + id;
    const double s0 = g[G_VOL * F];
    const double si = g[G_SIA * F], ni1 = g[G_NI1A * F], ni2 = g[G_NI2A * F];
    const double sj = g[G_SJA * F], nj1 = g[G_NJ1A * F], nj2 = g[G_NJ2A * F];
    double uu = L.q[Q_U * F + id], vv = L.q[Q_V * F + id], cc = L.q[Q_C * F + id], d = L.q[Q_D * F + id];
    double uni = uu * ni1 + vv * ni2, unj = uu * nj1 + vv * nj2;
    double Lci = (fabs(uni) + cc) * si, Lcj = (fabs(unj) + cc) * sj;
    double amu = L.visc ? L.amu[id] : 0.0, amut = L.visc ? L.amut[id] : 0.0;
    double tmp1 = c.gamma * rcp(d) * (amu * c.rPr + amut * (1.0 / PrT));
    double Lvi = tmp1 * g[G_VI2 * F], Lvj = tmp1 * g[G_VJ2 * F];
    L.lc[L_CI * F + id] = Lci;
    L.lc[L_CJ * F + id] = Lcj;
    L.lc[L_VI * F + id] = Lvi;
    L.lc[L_VJ * F + id] = Lvj;
    double dt;
    if (c.local_dt == 0) dt = c.dt_global;
    else {
      dt = c.CFL * s0 * rcp(Lci + Lcj + 1.0 * (Lvi + Lvj));
      if (dt > c.dtmax) dt = c.dtmax;
      if (dt < c.dtmin) dt = c.dtmin;
    }
    L.lc[L_DT * F + id] = dt;
  }
  if (NORM) {
    tile_partials(L, act, vres);
    if (FINAL) {
      // the last CTA to finish reduces every tile's partials (few cases)
      __shared__ int last;
      __threadfence();
      __syncthreads();
      if (threadIdx.x == 0) last = atomicAdd(L.nctr, 1u) == gridDim.x - 1;
      __syncthreads();
      if (last) {
        __threadfence();
        const int w = threadIdx.x >> 5;
        for (int k = w; k < L.ncase * 12; k += TILE / 32) final_norm(L, k / 12, k % 12);
        if (threadIdx.x == 0) *L.nctr = 0u;
      }
    }
  }
}

// ---- the residual of a level in one kernel --------------------------------
// k_residual_tile does the work of k_prim, k_flux_i, k_flux_j and k_res for a
// 2-D tile of RTX x RTY cells: the primitives (and Sutherland mu) of the tile
// and its two-cell halo go into shared memory, every i- and j-face of the
// tile's cells is reconstructed and fluxed from there (the faces on the
// tile's edges are evaluated by both tiles that share them), and each thread
// forms its cell's residual, spectral radii, time step and norm partials.
// Nothing but U, the geometry and the outputs touches HBM, and one launch
// replaces four.  It serves levels without a turbulence model or a
// finite-difference patch, in FP64; the face, reconstruction and viscous
// arithmetic is the same code as the chain's.
constexpr int RTX = RES_TILE_X, RTY = RES_TILE_Y;  // cells per tile
constexpr int RGX = RTX + 4, RGY = RTY + 4;        // tile + two halo cells on each side
constexpr int RGN = RGX * RGY;
constexpr int RNT = RES_TILE_THREADS;
// one thread per face of the tile, per halo cell and per cell: every FP64
// chain of a phase runs side by side (on the small multigrid levels the
// kernel is as long as one thread's chain)
static_assert((RTX + 1) * RTY + RTX * (RTY + 1) <= RNT && RGN <= RNT && RTX * RTY <= RNT, "a thread per item");

template <bool NORM, bool FINAL>
__global__ void __launch_bounds__(RNT) k_residual_tile(Lvl L, const int4 *rt, int post) {
  __shared__ double sd[RGN], su[RGN], sv[RGN], sp[RGN], sT[RGN], sc[RGN], smu[RGN];
  __shared__ double sU[4][RGN];
  __shared__ double fi[4][RTY][RTX + 1], fj[4][RTY + 1][RTX];
  const int4 t4 = rt[blockIdx.x];
  const int bk = t4.x, i0 = t4.y, j0 = t4.z;
  const BlkDev &b = L.blk[bk];
  const CaseDev &c = L.cs[b.cas];
  const long long F = L.F, P = b.P;
  const int nx = b.nx, ny = b.ny;
  const int i1 = min(i0 + RTX - 1, nx - 1), j1 = min(j0 + RTY - 1, ny - 1);  // last cells of the tile
  auto R = [&](int i, int j) { return (j - j0 + 2) * RGX + (i - i0 + 2); };
  // (1) primitives over the tile and its halo (comput_duvtpckw + get_viscous,
  // as k_prim), within the block's extended range -1..nx+1 x -1..ny+1
  for (int t = threadIdx.x; t < RGN; t += RNT) {
    const int i = i0 - 2 + t % RGX, j = j0 - 2 + t / RGX;
    if (i < -1 || i > nx + 1 || j < -1 || j > ny + 1) continue;
    const long long id = fidx(b, i, j);
    const double d = L.U[id], ru = L.U[F + id], rv = L.U[2 * F + id], E = L.U[3 * F + id];
    const double rd = rcp(d);
    const double uu = ru * rd, v = rv * rd;
    const double T = (E - 0.5 * d * (uu * uu + v * v)) * (rd * c.rCv);
    const double pp = c.p00 * d * T;
    const double st = T > 0.0 ? sqrt_p(T) : sqrt(T);
    sd[t] = d; su[t] = uu; sv[t] = v; sT[t] = T; sp[t] = pp;
    sc[t] = st * c.rMa;
    sU[0][t] = d; sU[1][t] = ru; sU[2][t] = rv; sU[3][t] = E;
    const bool own = i >= i0 && i <= i1 && j >= j0 && j <= j1;
    if (own && !(T >= 1.0e-5)) set_status(L.status + 4 * b.cas, 3, bk, i, j);
    if (L.visc) {
      const double mu = c.rRe * (1.0 + c.Tsb) * (T * st) * rcp(c.Tsb + T);
      smu[t] = mu;
      // Amu over 0..nx x 0..ny as k_prim leaves it: the tile's cells, and the
      // block's ghost lines next to them when the tile is on the block's edge
      const bool wi = (i >= i0 && i <= i1) || (i == 0 && i0 == 1) || (i == nx && i1 == nx - 1);
      const bool wj = (j >= j0 && j <= j1) || (j == 0 && j0 == 1) || (j == ny && j1 == ny - 1);
      if (wi && wj) { L.amu[id] = mu; L.amut[id] = 0.0; }
    }
  }
  __syncthreads();
  // (2) faces: i-faces i0..i1+1 of rows j0..j1, j-faces j0..j1+1 of columns i0..i1
  const int nfi = (i1 - i0 + 2) * (j1 - j0 + 1), nfj = (i1 - i0 + 1) * (j1 - j0 + 2);
  for (int t = threadIdx.x; t < nfi + nfj; t += RNT) {
    const bool ifc = t < nfi;
    int i, j;
    if (ifc) { i = i0 + t % (i1 - i0 + 2); j = j0 + t / (i1 - i0 + 2); }
    else { const int u = t - nfi; i = i0 + u % (i1 - i0 + 1); j = j0 + u / (i1 - i0 + 1); }
    const long long id = fidx(b, i, j);
    const int r = R(i, j), st = ifc ? 1 : RGX;  // stencil stride in the tile's shared arrays
    const double s = L.geo[(ifc ? G_SI : G_SJ) * F + id];
    const double n1 = L.geo[(ifc ? G_NI1 : G_NJ1) * F + id], n2 = L.geo[(ifc ? G_NI2 : G_NJ2) * F + id];
    double S0[4][4], UL[4], UR[4];
    int scheme = L.scheme;
    if (L.recon == Recon_Original) {
      if (!ifc) scheme = L.gscheme;  // the global Iflag_Scheme in the j direction (sub_Residual.f90:367)
#pragma unroll
      for (int k = 0; k < 4; k++) {
        const int q = r + (k - 2) * st;
        S0[k][0] = sd[q]; S0[k][1] = su[q]; S0[k][2] = sv[q]; S0[k][3] = sp[q];
      }
    } else {
#pragma unroll
      for (int k = 0; k < 4; k++)
#pragma unroll
        for (int m = 0; m < 4; m++) S0[k][m] = sU[m][r + (k - 2) * st];
    }
    reconstruct(L.recon, scheme, S0, c.gamma, UL, UR);
    double QL[4] = {UL[0], UL[1] * n1 + UL[2] * n2, -UL[1] * n2 + UL[2] * n1, UL[3]};
    double QR[4] = {UR[0], UR[1] * n1 + UR[2] * n2, -UR[1] * n2 + UR[2] * n1, UR[3]};
    double Fl[4];
    face_flux(L.flux, QL, QR, Fl, c.gamma, c.ggm1);
    double F0 = -Fl[0] * s, F1 = -(Fl[1] * n1 - Fl[2] * n2) * s, F2 = -(Fl[1] * n2 + Fl[2] * n1) * s, F3 = -Fl[3] * s;
    if (L.visc) {
      const double *g = L.geo + id;
      double Amu1, Amk1;
      const int up = r - st;  // the upstream cell of the face
      const bool lo = ifc ? i == 1 : j == 1, hi = ifc ? i == nx : j == ny;
      if (lo) {
        Amu1 = smu[r] + 0.0;
        Amk1 = c.Cp * (smu[r] * c.rPr + 0.0 * (1.0 / PrT));
      } else if (hi) {
        Amu1 = smu[up] + 0.0;
        Amk1 = c.Cp * (smu[up] * c.rPr + 0.0 * (1.0 / PrT));
      } else if (ifc) {
        Amu1 = (smu[up] + smu[r] + 0.0 + 0.0) * 0.5;
        Amk1 = c.Cp * ((smu[up] + smu[r]) * c.rPr + (0.0 + 0.0) * (1.0 / PrT)) * 0.5;
      } else {
        Amu1 = (smu[r] + smu[up] + 0.0 + 0.0) * 0.5;
        Amk1 = c.Cp * ((smu[up] + smu[r]) * c.rPr + (0.0 + 0.0) * (1.0 / PrT)) * 0.5;
      }
      double Diu, Div, DiT, Dju, Djv, DjT, u1, v1;
      if (ifc) {
        const int w = r - 1, nN = r + RGX, nS = r - RGX;
        Diu = su[r] - su[w]; Div = sv[r] - sv[w]; DiT = sT[r] - sT[w];
        Dju = (su[nN - 1] + su[nN] - su[nS - 1] - su[nS]) * 0.25;
        Djv = (sv[nN - 1] + sv[nN] - sv[nS - 1] - sv[nS]) * 0.25;
        DjT = (sT[nN - 1] + sT[nN] - sT[nS - 1] - sT[nS]) * 0.25;
        u1 = (su[r] + su[w]) * 0.5; v1 = (sv[r] + sv[w]) * 0.5;
        viscous_face_m(g[G_VIA * F], g[G_VIB * F], g[G_VIC * F], g[G_VID * F], Diu, Div, DiT, Dju, Djv, DjT, Amu1,
                       Amk1, u1, v1, n1, n2, s, F1, F2, F3);
      } else {
        const int sN = r - RGX;
        Diu = (su[sN + 1] + su[r + 1] - su[sN - 1] - su[r - 1]) * 0.25;
        Div = (sv[sN + 1] + sv[r + 1] - sv[sN - 1] - sv[r - 1]) * 0.25;
        DiT = (sT[sN + 1] + sT[r + 1] - sT[sN - 1] - sT[r - 1]) * 0.25;
        Dju = su[r] - su[sN]; Djv = sv[r] - sv[sN]; DjT = sT[r] - sT[sN];
        u1 = (su[r] + su[sN]) * 0.5; v1 = (sv[r] + sv[sN]) * 0.5;
        viscous_face_m(g[G_VJA * F], g[G_VJB * F], g[G_VJC * F], g[G_VJD * F], Diu, Div, DiT, Dju, Djv, DjT, Amu1,
                       Amk1, u1, v1, n1, n2, s, F1, F2, F3);
      }
    }
    if (ifc) { fi[0][j - j0][i - i0] = F0; fi[1][j - j0][i - i0] = F1; fi[2][j - j0][i - i0] = F2; fi[3][j - j0][i - i0] = F3; }
    else { fj[0][j - j0][i - i0] = F0; fj[1][j - j0][i - i0] = F1; fj[2][j - j0][i - i0] = F2; fj[3][j - j0][i - i0] = F3; }
  }
  __syncthreads();
  // (3) the cell of this thread: flux differences, radii, time step (k_res)
  const int tx = threadIdx.x % RTX, ty = threadIdx.x / RTX;
  const int i = i0 + tx, j = j0 + ty;
  const bool act = threadIdx.x < RTX * RTY && i <= i1 && j <= j1;
  if (post & RES_SET_UN) {
    // Un = U over 0..nx x 0..ny: the tile's cells and the ghost lines at
    // the block's edges next to them
    for (int t = threadIdx.x; t < RGN; t += RNT) {
      const int ii = i0 - 2 + t % RGX, jj = j0 - 2 + t / RGX;
      const bool wi = (ii >= i0 && ii <= i1) || (ii == 0 && i0 == 1) || (ii == nx && i1 == nx - 1);
      const bool wj = (jj >= j0 && jj <= j1) || (jj == 0 && j0 == 1) || (jj == ny && j1 == ny - 1);
      if (wi && wj) {
        const long long id = fidx(b, ii, jj);
#pragma unroll
        for (int m = 0; m < 4; m++) L.un[m * F + id] = sU[m][t];
      }
    }
  }
  double vres[6] = {0, 0, 0, 0, 0, 0};
  if (act) {
    const long long id = fidx(b, i, j);
    const int r = R(i, j);
#pragma unroll
    for (int m = 0; m < 4; m++) {
      double rr = fi[m][ty][tx + 1] - fi[m][ty][tx] + fj[m][ty + 1][tx] - fj[m][ty][tx];
      vres[m] = rr;
      if (post & (RES_ADD_FORCE | RES_FORCE_FN)) {
        const double qf = L.qf[m * F + id];
        if (post & RES_FORCE_FN) L.qf[m * F + id] = qf - rr;
        if (post & RES_ADD_FORCE) rr = rr + qf;
      }
      L.res[m * F + id] = rr;
    }
    const double *g = L.geo + id;
    const double s0 = g[G_VOL * F];
    const double si = g[G_SIA * F], ni1 = g[G_NI1A * F], ni2 = g[G_NI2A * F];
    const double sj = g[G_SJA * F], nj1 = g[G_NJ1A * F], nj2 = g[G_NJ2A * F];
    const double uu = su[r], vv = sv[r], cc = sc[r], d = sd[r];
    const double uni = uu * ni1 + vv * ni2, unj = uu * nj1 + vv * nj2;
    const double Lci = (fabs(uni) + cc) * si, Lcj = (fabs(unj) + cc) * sj;
    const double amu = L.visc ? smu[r] : 0.0, amut = 0.0;
    const double tmp1 = c.gamma * rcp(d) * (amu * c.rPr + amut * (1.0 / PrT));
    const double Lvi = tmp1 * g[G_VI2 * F], Lvj = tmp1 * g[G_VJ2 * F];
    L.lc[L_CI * F + id] = Lci;
    L.lc[L_CJ * F + id] = Lcj;
    L.lc[L_VI * F + id] = Lvi;
    L.lc[L_VJ * F + id] = Lvj;
    double dt;
    if (c.local_dt == 0) dt = c.dt_global;
    else {
      dt = c.CFL * s0 * rcp(Lci + Lcj + 1.0 * (Lvi + Lvj));
      if (dt > c.dtmax) dt = c.dtmax;
      if (dt < c.dtmin) dt = c.dtmin;
    }
    L.lc[L_DT * F + id] = dt;
  }
  if (NORM) {
    tile_partials<RNT>(L, act, vres);
    if (FINAL) {
      __shared__ int last;
      __threadfence();
      __syncthreads();
      if (threadIdx.x == 0) last = atomicAdd(L.nctr, 1u) == gridDim.x - 1;
      __syncthreads();
      if (last) {
        __threadfence();
        const int w = threadIdx.x >> 5;
        for (int k = w; k < L.ncase * 12; k += RNT / 32) final_norm(L, k / 12, k % 12);
        if (threadIdx.x == 0) *L.nctr = 0u;
      }
    }
  }
}

// per-tile partial norms of Res (max |Res| and sum Res^2 per variable)
__global__ void __launch_bounds__(TILE) k_norm_partial(Lvl L) {
  int bk, i, j;
  double vres[6] = {0, 0, 0, 0, 0, 0};
  bool act = false;
  if (core_ij(L, bk, i, j)) {
    const BlkDev &b = L.blk[bk];
    if (i >= 1 && i <= b.nx - 1 && j >= 1 && j <= b.ny - 1) {
      act = true;
      long long id = fidx(b, i, j);
#pragma unroll
      for (int m = 0; m < 6; m++)
        if (m < L.nvar) vres[m] = L.res[m * L.F + id];
    }
  }
  tile_partials(L, act, vres);
}

// per-case reduction of the tile partials (one warp per case and quantity)
__global__ void __launch_bounds__(384) k_norm_final(Lvl L) {
  const int k = blockIdx.x * 12 + (threadIdx.x >> 5);
  final_norm(L, k / 12, k % 12);
}

// set-up: the viscous inverse Jacobians of the i-faces (i = 1..nx, j =
// 1..ny-1) and j-faces (i = 1..nx-1, j = 1..ny) from the cell centres, with the
// stencils of Residual_FVM (sub_Residual.f90:313-330, 419-436), and the cell
// metric factors of the spectral radii
__global__ void __launch_bounds__(TILE) k_face_metrics(Lvl L) {
  int bk, i, j;
  if (!tile_ij(L, bk, i, j)) return;
  const BlkDev &b = L.blk[bk];
  const long long F = L.F, P = b.P, id = fidx(b, i, j);
  const double *x1 = L.geo + G_X1 * F, *y1 = L.geo + G_Y1 * F;
  double *g = L.geo + id;
  if (i >= 1 && i <= b.nx && j >= 1 && j <= b.ny - 1) {
    const long long w = id - 1, nN = id + P, nS = id - P;
    const double Dix = x1[id] - x1[w], Diy = y1[id] - y1[w];
    const double Djx = (x1[nN - 1] + x1[nN] - x1[nS - 1] - x1[nS]) * 0.25;
    const double Djy = (y1[nN - 1] + y1[nN] - y1[nS - 1] - y1[nS]) * 0.25;
    const double Ds = 1.0 / (Dix * Djy - Djx * Diy);
    g[G_VIA * F] = Djy * Ds; g[G_VIB * F] = Diy * Ds; g[G_VIC * F] = Djx * Ds; g[G_VID * F] = Dix * Ds;
  }
  if (i >= 1 && i <= b.nx - 1 && j >= 1 && j <= b.ny) {
    const long long s = id - P;
    const double Dix = (x1[s + 1] + x1[id + 1] - x1[s - 1] - x1[id - 1]) * 0.25;
    const double Diy = (y1[s + 1] + y1[id + 1] - y1[s - 1] - y1[id - 1]) * 0.25;
    const double Djx = x1[id] - x1[s], Djy = y1[id] - y1[s];
    const double Ds = 1.0 / (Dix * Djy - Djx * Diy);
    g[G_VJA * F] = Djy * Ds; g[G_VJB * F] = Diy * Ds; g[G_VJC * F] = Djx * Ds; g[G_VJD * F] = Dix * Ds;
  }
  if (i >= 1 && i <= b.nx - 1 && j >= 1 && j <= b.ny - 1) {
    // comput_Lvc (sub_NS_singlegrid.f90:352-388): face metrics averaged over
    // the cell's two faces of each family
    const double *gg = L.geo;
    const double si = 0.5 * (gg[G_SI * F + id] + gg[G_SI * F + id + 1]);
    const double sj = 0.5 * (gg[G_SJ * F + id] + gg[G_SJ * F + id + P]);
    const double rs0 = 1.0 / gg[G_VOL * F + id];
    g[G_SIA * F] = si;
    g[G_NI1A * F] = 0.5 * (gg[G_NI1 * F + id] + gg[G_NI1 * F + id + 1]);
    g[G_NI2A * F] = 0.5 * (gg[G_NI2 * F + id] + gg[G_NI2 * F + id + 1]);
    g[G_SJA * F] = sj;
    g[G_NJ1A * F] = 0.5 * (gg[G_NJ1 * F + id] + gg[G_NJ1 * F + id + P]);
    g[G_NJ2A * F] = 0.5 * (gg[G_NJ2 * F + id] + gg[G_NJ2 * F + id + P]);
    g[G_VI2 * F] = si * si * rs0;
    g[G_VJ2 * F] = sj * sj * rs0;
  }
}
void launch_face_metrics(const Lvl &L, cudaStream_t s) { k_face_metrics<<<L.ntiles, TILE, 0, s>>>(L); }

void launch_prim(const Lvl &L, cudaStream_t s) { k_prim<<<L.ntiles, TILE, 0, s>>>(L); }
void launch_flux_i(const Lvl &L, bool fp32, cudaStream_t s) {
  if (fp32) k_flux_i<float><<<L.nctiles, TILE, 0, s>>>(L);
  else k_flux_i<double><<<L.nctiles, TILE, 0, s>>>(L);
}
void launch_flux_j(const Lvl &L, bool fp32, cudaStream_t s) {
  if (fp32) k_flux_j<float><<<L.nctiles, TILE, 0, s>>>(L);
  else k_flux_j<double><<<L.nctiles, TILE, 0, s>>>(L);
}
// with_norms: the tile partials inside k_res; with few cases the last CTA of
// k_res also forms the per-case norms (norms_fused_final() tells the caller)
bool norms_fused_final(const Lvl &L) { return L.ncase <= 8; }
void launch_res(const Lvl &L, bool with_norms, int post, cudaStream_t s) {
  if (!with_norms) k_res<false, false><<<L.nctiles, TILE, 0, s>>>(L, post);
  else if (norms_fused_final(L)) k_res<true, true><<<L.nctiles, TILE, 0, s>>>(L, post);
  else k_res<true, false><<<L.nctiles, TILE, 0, s>>>(L, post);
}
// Lr: the level with npart, case_tile0, case_ntile and nctr of the 2-D tile list
void launch_residual_tile(const Lvl &Lr, const int4 *rt, int ntiles, bool with_norms, int post, cudaStream_t s) {
  if (!with_norms) k_residual_tile<false, false><<<ntiles, RNT, 0, s>>>(Lr, rt, post);
  else if (norms_fused_final(Lr)) k_residual_tile<true, true><<<ntiles, RNT, 0, s>>>(Lr, rt, post);
  else k_residual_tile<true, false><<<ntiles, RNT, 0, s>>>(Lr, rt, post);
}
void launch_norms(const Lvl &L, bool partials, cudaStream_t s) {
  if (partials) k_norm_partial<<<L.nctiles, TILE, 0, s>>>(L);
  k_norm_final<<<L.ncase, 384, 0, s>>>(L);
}

}  // namespace ec2d
