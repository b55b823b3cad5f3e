// k_bl.cu -- Baldwin-Lomax algebraic eddy viscosity (turbulence_model_BL and
// BL_model_1d, sub_turbulence_BL.f90:6-273).
//
// The model switches discretely (argmax of F(y), the inner/outer crossover),
// so this file is compiled without FMA contraction (-fmad=false) to round
// every product and sum the way the reference's separate operations do.
//
// Layout: k_bl_omega writes |vx - uy| of every interior cell into plane 0 of
// L.tb.  k_bl runs one CTA per block: the block's wall subfaces in subface
// order, one warp per wall-normal line.  Per line the three passes of
// BL_model_1d become warp reductions: max |mu*omega| (wall shear), max of
// F(y) with the first index on ties (strict '>' in the reference loop), and
// the inner/outer switch, which stays on once triggered, as a ballot prefix.
// flag1 of the reference (first line through a cell sets Amu_t, later lines
// take the minimum) follows from the line ranges of the earlier wall
// subfaces, so it needs no storage.
#include "ec2d_dev.cuh"
#include "ec2d_internal.h"

namespace ec2d {
namespace {

constexpr int TILE = EC2D_TILE;
// single-precision literals of sub_turbulence_BL.f90:215 promoted to double
constexpr double AP = (double)26.f, Ccp = (double)1.6f, Ckleb = (double)0.3f, Cwk = 0.25, AKT = (double)0.4f,
                 AK = (double)0.0168f;

// omiga(i,j) = |vx - uy| at the cell centres, sub_turbulence_BL.f90:35-56
__global__ void __launch_bounds__(TILE) k_bl_omega(Lvl L) {
  int2 t = L.tiles[blockIdx.x];
  const BlkDev b = L.blk[t.x];
  int W = b.nx + 3;
  int k = t.y + threadIdx.x;
  if (k >= W * (b.ny + 3)) return;
  int i = k % W - 1, j = k / W - 1;
  if (i < 1 || i > b.nx - 1 || j < 1 || j > b.ny - 1) return;
  const long long F = L.F;
  const double *x1 = L.geo + G_X1 * F + b.off, *y1 = L.geo + G_Y1 * F + b.off;
  const double *uu = L.q + Q_U * F + b.off, *v = L.q + Q_V * F + b.off;
  int P = b.P;
  auto at = [&](int ii, int jj) { return (jj + 2) * P + (ii + 2); };
  double xi = x1[at(i + 1, j)] - x1[at(i - 1, j)];
  double yi = y1[at(i + 1, j)] - y1[at(i - 1, j)];
  double xj = x1[at(i, j + 1)] - x1[at(i, j - 1)];
  double yj = y1[at(i, j + 1)] - y1[at(i, j - 1)];
  double Jac = 1.0 / (xi * yj - xj * yi);
  double ix = Jac * yj, iy = -Jac * xj, jx = -Jac * yi, jy = Jac * xi;
  double ui = uu[at(i + 1, j)] - uu[at(i - 1, j)];
  double vi = v[at(i + 1, j)] - v[at(i - 1, j)];
  double uj = uu[at(i, j + 1)] - uu[at(i, j - 1)];
  double vj = v[at(i, j + 1)] - v[at(i, j - 1)];
  double vx = vi * ix + vj * jx;
  double uy = ui * iy + uj * jy;
  L.tb[b.off + at(i, j)] = fabs(vx - uy);
}

// cell (i,j) of position k (1-based from the wall) on line t of a wall subface
__device__ __forceinline__ void line_cell(const SubDev &s, const BlkDev &b, int t, int k, int &i, int &j) {
  if (s.face == 1) { i = k; j = t; }
  else if (s.face == 3) { i = b.nx - k; j = t; }
  else if (s.face == 2) { i = t; j = k; }
  else { i = t; j = b.ny - k; }
}

// was cell (i,j) on a line of an earlier wall subface of the block (flag1)
__device__ __forceinline__ bool covered_before(const Lvl &L, const BlkDev &b, int s, int i, int j) {
  for (int r = b.sub0; r < s; r++) {
    const SubDev &q = L.sub[r];
    if (q.neighb != BC_Wall) continue;
    if (q.face == 1 || q.face == 3) {
      if (j >= q.jst && j <= q.jend - 1) return true;
    } else if (i >= q.ist && i <= q.iend - 1) return true;
  }
  return false;
}

__device__ __forceinline__ double wmax(double a) {
  for (int o = 16; o; o >>= 1) a = fmax(a, __shfl_xor_sync(0xffffffffu, a, o));
  return a;
}

__global__ void __launch_bounds__(TILE) k_bl(Lvl L) {
  const BlkDev b = L.blk[blockIdx.x];
  bool wall = false;
  for (int r = b.sub0; r < b.sub0 + b.nsub; r++) wall |= (L.sub[r].neighb == BC_Wall);
  if (!wall) return;
  const long long F = L.F;
  const int P = b.P;
  auto at = [&](int ii, int jj) { return b.off + (long long)(jj + 2) * P + (ii + 2); };
  const double *x1 = L.geo + G_X1 * F, *y1 = L.geo + G_Y1 * F;
  const double *d = L.q + Q_D * F, *uu = L.q + Q_U * F, *v = L.q + Q_V * F;
  const double *om = L.tb;
  double *amut = L.amut;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;

  for (int r = b.sub0; r < b.sub0 + b.nsub; r++) {
    const SubDev s = L.sub[r];
    if (s.neighb != BC_Wall) continue;
    const bool iface = (s.face == 1 || s.face == 3);
    const int t0 = iface ? s.jst : s.ist, t1 = iface ? s.jend - 1 : s.iend - 1;
    const int n = iface ? b.nx : b.ny;  // line arrays of BL_model_1d hold n-1 cells
    for (int t = t0 + warp; t <= t1; t += nwarp) {
      // wall point: midpoint of the first cell centre and its ghost image
      int ia, ja, ig, jg;
      line_cell(s, b, t, 1, ia, ja);
      line_cell(s, b, t, 0, ig, jg);
      double x0 = (x1[at(ia, ja)] + x1[at(ig, jg)]) * 0.5, y0 = (y1[at(ia, ja)] + y1[at(ig, jg)]) * 0.5;
      auto yy = [&](int i, int j) {
        double dx = x1[at(i, j)] - x0, dy = y1[at(i, j)] - y0;
        return sqrt(dx * dx + dy * dy);
      };
      // pass 1: Tw = max |Amu*omiga| over the line
      double tw = 0.0;
      for (int k = 1 + lane; k <= n - 1; k += 32) {
        int i, j;
        line_cell(s, b, t, k, i, j);
        tw = fmax(tw, fabs(L.amu[at(i, j)] * om[at(i, j)]));
      }
      tw = wmax(tw);
      double Ret = sqrt(d[at(ia, ja)] * tw) / L.amu[at(ia, ja)];
      // pass 2: Udif = max |u|, Fmax = max F(y), etamax = y at the first maximum
      double udif = 0.0, fmx = 0.0;
      int kmax = 0x7fffffff;
      for (int k = 1 + lane; k <= n - 1; k += 32) {
        int i, j;
        line_cell(s, b, t, k, i, j);
        double u1 = uu[at(i, j)], v1 = v[at(i, j)];
        udif = fmax(udif, sqrt(u1 * u1 + v1 * v1));
        double y = yy(i, j);
        double etap = y * Ret;
        double FF = y * fabs(om[at(i, j)]) * (1.0 - exp(-etap / AP));
        if (FF > fmx) { fmx = FF; kmax = k; }
      }
      for (int o = 16; o; o >>= 1) {
        double f2 = __shfl_xor_sync(0xffffffffu, fmx, o);
        int k2 = __shfl_xor_sync(0xffffffffu, kmax, o);
        if (f2 > fmx || (f2 == fmx && k2 < kmax)) { fmx = f2; kmax = k2; }
      }
      udif = wmax(udif);
      double etamax = 0.0;
      if (fmx > 0.0) {
        int i, j;
        line_cell(s, b, t, kmax, i, j);
        etamax = yy(i, j);
      }
      double a = etamax * fmx, c = Cwk * etamax * udif * udif / fmx;
      double Fwak = (c < a) ? c : a;
      // pass 3: inner/outer switch; once |visto| < |visti| the outer value stays
      bool on = false;
      for (int k0 = 1; k0 <= n - 1; k0 += 32) {
        int k = k0 + lane;
        bool act = k <= n - 1;
        int i = 0, j = 0;
        double visti = 0.0, visto = 0.0;
        if (act) {
          line_cell(s, b, t, k, i, j);
          double y = yy(i, j);
          double etap = Ret * y;
          double bl = AKT * y * (1.0 - exp(-etap / AP));
          double dd = d[at(i, j)];
          visti = dd * bl * bl * fabs(om[at(i, j)]);
          double q = Ckleb * y / etamax;
          double q2 = q * q, q6 = q2 * q2 * q2;
          double Fkleb = 1.0 / (1.0 + 5.5 * q6);
          visto = AK * Ccp * dd * Fwak * Fkleb;
        }
        unsigned m = __ballot_sync(0xffffffffu, act && fabs(visto) < fabs(visti));
        bool flag = on || (m & (0xffffffffu >> (31 - lane))) != 0;
        on = on || m != 0;
        if (act) {
          double val = flag ? visto : visti;
          long long id = at(i, j);
          if (covered_before(L, b, r, i, j)) {
            double old = amut[id];
            amut[id] = (val < old) ? val : old;
          } else amut[id] = val;
        }
      }
    }
    __syncthreads();
    // ghost rows/columns of the subface, sub_turbulence_BL.f90:84-87,113-116,147-150,181-184
    if (iface) {
      for (int i = -1 + (int)threadIdx.x; i <= b.nx + 1; i += blockDim.x) {
        amut[at(i, s.jst - 1)] = amut[at(i, s.jst)];
        amut[at(i, s.jend)] = amut[at(i, s.jend - 1)];
      }
      __syncthreads();
      double sg0 = (s.face == 1) ? -1.0 : 1.0, sgn = (s.face == 1) ? 1.0 : -1.0;
      for (int j = s.jst + (int)threadIdx.x; j <= s.jend; j += blockDim.x) {
        amut[at(b.nx, j)] = sgn * amut[at(b.nx - 1, j)];
        amut[at(0, j)] = sg0 * amut[at(1, j)];
      }
    } else {
      double sg0 = (s.face == 2) ? -1.0 : 1.0, sgn = (s.face == 2) ? 1.0 : -1.0;
      for (int i = s.ist + (int)threadIdx.x; i <= s.iend; i += blockDim.x) {
        amut[at(i, 0)] = sg0 * amut[at(i, 1)];
        amut[at(i, b.ny)] = sgn * amut[at(i, b.ny - 1)];
      }
      __syncthreads();
      for (int j = -1 + (int)threadIdx.x; j <= b.ny + 1; j += blockDim.x) {
        amut[at(s.ist - 1, j)] = amut[at(s.ist, j)];
        amut[at(s.iend, j)] = amut[at(s.iend - 1, j)];
      }
    }
    __syncthreads();
  }
}

}  // namespace

void launch_bl(const Lvl &L, cudaStream_t s) {
  k_bl_omega<<<L.ntiles, TILE, 0, s>>>(L);
  k_bl<<<L.nblk, TILE, 0, s>>>(L);
}

}  // namespace ec2d
