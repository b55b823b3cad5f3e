// k_bc.cu -- ghost cells: physical boundary conditions (sub_boundary.f90:10-34,
// 306-581), block-interface halo copy and ghost-corner extrapolation
// (update_buffer_onemesh, sub_boundary.f90:45-153), and the nu~/k/omega
// clip (force_vt_kw, sub_NS_singlegrid.f90:30-60).
//
// Write order.  The reference runs every physical subface of every block in
// (block, subface) order, then per block its halo copies followed by its four
// ghost corners.  A physical subface loops over node indices ist..iend,
// jst..jend, so its end points write ghost rows that later subfaces read.
// The write sets of one subface never overlap its read set, halo copies read
// only interior cells, and corners read only the block's own ghosts.  Hence
// one CTA per block reproduces the reference exactly: subfaces of phase 1 in
// order with a barrier between them, all halo items of phase 2 in parallel,
// then the corners.  Physical subfaces whose read and write sets do not meet
// those of any earlier subface of the block share a barrier phase (the
// grouping is computed at set-up from the index rectangles).
#include "ec2d_dev.cuh"
#include "ec2d_internal.h"

namespace ec2d {

__device__ __forceinline__ void ghost_pair(int face, int i, int j, int k, int &i1, int &j1, int &i2, int &j2) {
  if (face == 1) { i1 = i + k - 1; j1 = j; i2 = i - k; j2 = j; }
  else if (face == 2) { i1 = i; j1 = j + k - 1; i2 = i; j2 = j - k; }
  else if (face == 3) { i1 = i - k; j1 = j; i2 = i + k - 1; j2 = j; }
  else { i1 = i; j1 = j - k; i2 = i; j2 = j + k - 1; }
}

// boundary_wall, sub_boundary.f90:306-386
__device__ void bc_wall(const Lvl &L, const BlkDev &b, const CaseDev &c, const SubDev &s, int i, int j, int k) {
  const long long F = L.F;
  int i1, j1, i2, j2;
  ghost_pair(s.face, i, j, k, i1, j1, i2, j2);
  long long a = fidx(b, i1, j1), g = fidx(b, i2, j2);
  double *U = L.U;
  double d1 = U[a];
  if (c.Twall <= 0) {
    U[g] = U[a];
    U[F + g] = -U[F + a];
    U[2 * F + g] = -U[2 * F + a];
    U[3 * F + g] = U[3 * F + a];
  } else {
    double u1 = U[F + a] / d1, v1 = U[2 * F + a] / d1;
    double p1 = (U[3 * F + a] - 0.5 * d1 * (u1 * u1 + v1 * v1)) * (c.gamma - 1.0);
    double T1 = c.gamma * c.Ma * c.Ma * p1 / d1;
    double p2 = p1, T2 = 2.0 * c.Twall - T1, u2 = -u1, v2 = -v1;
    double d2 = c.gamma * c.Ma * c.Ma * p2 / T2;
    U[g] = d2;
    U[F + g] = d2 * u2;
    U[2 * F + g] = d2 * v2;
    U[3 * F + g] = p2 / (c.gamma - 1.0) + 0.5 * d2 * (u2 * u2 + v2 * v2);
  }
  if (L.nvar == 5) U[4 * F + g] = 0.0;
  if (L.nvar == 6) {
    const double beta1 = 0.075;
    double d2 = U[g];
    double r2 = U[F + g], r3 = U[2 * F + g];
    double T2 = (U[3 * F + g] - 0.5 * (r2 * r2 + r3 * r3) / d2) / (c.Cv * d2);
    double Amu2 = (1.0 + c.Tsb) * sqrt(T2 * T2 * T2) / (c.Tsb + T2);
    double dw = L.geo[G_DW * F + a];
    double wt = 60.0 * Amu2 / (d2 * beta1 * (dw * dw) * c.Re * c.Re);
    U[4 * F + g] = -U[4 * F + a];
    U[5 * F + g] = (d1 + d2) * wt - U[5 * F + a];
  }
}

// Symmetry_or_slidewall, sub_boundary.f90:391-451.  The reflection
// U - 2 (U.n) n does not depend on the sign of n, so the far-field edge
// normal serves.
__device__ void bc_symmetry(const Lvl &L, const BlkDev &b, const SubDev &s, int i, int j, int k, double2 nrm) {
  const long long F = L.F;
  const double n1 = nrm.x, n2 = nrm.y;
  int i1, j1, i2, j2;
  ghost_pair(s.face, i, j, k, i1, j1, i2, j2);
  long long a = fidx(b, i1, j1), g = fidx(b, i2, j2);
  double *U = L.U;
  double Vn = U[F + a] * n1 + U[2 * F + a] * n2;
  U[g] = U[a];
  U[F + g] = U[F + a] - 2.0 * Vn * n1;
  U[2 * F + g] = U[2 * F + a] - 2.0 * Vn * n2;
  U[3 * F + g] = U[3 * F + a];
  for (int m = 4; m < L.nvar; m++) U[m * F + g] = U[m * F + a];
}

// Outward unit normal of a boundary node's edge, as boundary_Farfield_inlet_outlet
// (sub_boundary.f90:484-497) and Symmetry_or_slidewall (:400-412) form it: the
// edge from node (i,j) to (i,j+1) on faces 1 and 3, to (i+1,j) on faces 2 and
// 4, rotated by the face's sign.  Geometry only, so it is evaluated once at
// set-up (k_bc_normals), in separately rounded operations: the far-field
// inflow/outflow switch is a sign test on u.n.
__device__ __forceinline__ double2 edge_normal(const Lvl &L, const BlkDev &b, int face, int i, int j) {
  const long long F = L.F;
  const double *x = L.geo + G_X * F, *y = L.geo + G_Y * F;
  const long long p0 = fidx(b, i, j), p1 = (face == 1 || face == 3) ? fidx(b, i, j + 1) : fidx(b, i + 1, j);
  const double dx = __dsub_rn(x[p1], x[p0]), dy = __dsub_rn(y[p1], y[p0]);
  const double sl = __dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
  if (face == 1 || face == 4) return make_double2(__ddiv_rn(-dy, sl), __ddiv_rn(dx, sl));
  return make_double2(__ddiv_rn(dy, sl), __ddiv_rn(-dx, sl));
}

// boundary_Farfield_inlet_outlet, sub_boundary.f90:457-581.  The state is
// formed by reciprocal-multiply and a refined reciprocal square root (each
// within an ulp or two of the reference's divides and square root).  The
// inflow / outflow switch is a comparison of the normal Mach number with 0
// and +-1: where the fast value lies within its error bound of a threshold,
// the switch is decided on the value the reference computes, in separately
// rounded correctly rounded operations, so every cell takes the reference's
// branch.  Every ghost layer takes the same interior state and normal (the
// reference recomputes the same values per layer), so the ghost state is
// formed once and written to all LAP layers.
__device__ void bc_farfield(const Lvl &L, const BlkDev &b, const CaseDev &c, const SubDev &s, int i, int j,
                            double2 nrm) {
  const long long F = L.F;
  double *U = L.U;
  const double gamma = c.gamma, gm1 = gamma - 1.0;
  const double n1 = nrm.x, n2 = nrm.y;
  int i1, j1;
  if (s.face == 1 || s.face == 2) { i1 = i; j1 = j; }
  else if (s.face == 3) { i1 = i - 1; j1 = j; }
  else { i1 = i; j1 = j - 1; }
  long long a = fidx(b, i1, j1);
  const double d1 = U[a], m1 = U[F + a], m2 = U[2 * F + a], E1 = U[3 * F + a];
  const double rd = rcp(d1);
  const double u1 = m1 * rd, v1 = m2 * rd;
  const double p1 = (E1 - 0.5 * d1 * (u1 * u1 + v1 * v1)) * gm1;
  const double c2 = gamma * p1 * rd;
  const double rc = rsqrt_d(c2);  // 1 / c1
  const double c1 = c2 * rc;
  double Ma_n = (u1 * n1 + v1 * n2) * rc;
  // a few ulps of |u| / c bound the fast value's error
  const double tol = 1.0e-12 * (fabs(u1) + fabs(v1)) * rc;
  if (fabs(Ma_n) <= tol || fabs(fabs(Ma_n) - 1.0) <= tol + 1.0e-12) {
    const double ux = __ddiv_rn(m1, d1), vx = __ddiv_rn(m2, d1);
    const double ke = __dmul_rn(__dmul_rn(0.5, d1), __dadd_rn(__dmul_rn(ux, ux), __dmul_rn(vx, vx)));
    const double px = __dmul_rn(__dsub_rn(E1, ke), gm1);
    const double cx = __dsqrt_rn(__ddiv_rn(__dmul_rn(gamma, px), d1));
    Ma_n = __ddiv_rn(__dadd_rn(__dmul_rn(ux, n1), __dmul_rn(vx, n2)), cx);
  }
  double G[6];
  const int type = s.neighb;
  if (type == BC_Outlet || (type == BC_Farfield && Ma_n >= 0.0)) {
    if (Ma_n > 1.0 || c.p_outlet < 0 || type == BC_Farfield) {
      for (int m = 0; m < L.nvar; m++) G[m] = U[m * F + a];
    } else {
      const double pb = c.p_outlet;
      const double db = d1 + (c.p_outlet - p1) * (rc * rc);
      const double t = (p1 - c.p_outlet) * (rd * rc);
      const double ub = u1 + t * n1, vb = v1 + t * n2;
      const double p2 = 2.0 * pb - p1, d2 = 2.0 * db - d1, u2 = 2.0 * ub - u1, v2 = 2.0 * vb - v1;
      G[0] = d2; G[1] = d2 * u2; G[2] = d2 * v2;
      G[3] = p2 * c.rgm1 + 0.5 * d2 * (u2 * u2 + v2 * v2);
      for (int m = 4; m < L.nvar; m++) G[m] = U[m * F + a];
    }
  } else {
    const double d_inf = 1.0, u_inf = c.cosA, v_inf = c.sinA, p_inf = c.p00;
    if (c.p_outlet < 0 || Ma_n <= -1.0) {
      G[0] = d_inf; G[1] = d_inf * u_inf; G[2] = d_inf * v_inf;
      G[3] = p_inf / gm1 + 0.5 * d_inf * (u_inf * u_inf + v_inf * v_inf);
    } else {
      const double pb = 0.5 * (p1 + p_inf - d1 * c1 * ((u_inf - u1) * n1 + (v_inf - v1) * n2));
      const double db = d_inf + (pb - p_inf) * (rc * rc);
      const double t = (p_inf - pb) * (rd * rc);
      const double ub = u_inf - t * n1, vb = v_inf - t * n2;
      const double p2 = 2.0 * pb - p1, d2 = 2.0 * db - d1, u2 = 2.0 * ub - u1, v2 = 2.0 * vb - v1;
      G[0] = d2; G[1] = d2 * u2; G[2] = d2 * v2;
      G[3] = p2 * c.rgm1 + 0.5 * d2 * (u2 * u2 + v2 * v2);
    }
    if (L.nvar == 5) G[4] = c.vt_inf / c.Re;
    else if (L.nvar == 6) { G[4] = d_inf * c.Kt_inf; G[5] = d_inf * c.Wt_inf; }
  }
  for (int k = 1; k <= LAP; k++) {
    int i2, j2;
    if (s.face == 1) { i2 = i - k; j2 = j; }
    else if (s.face == 2) { i2 = i; j2 = j - k; }
    else if (s.face == 3) { i2 = i + k - 1; j2 = j; }
    else { i2 = i; j2 = j + k - 1; }
    const long long g = fidx(b, i2, j2);
    for (int m = 0; m < L.nvar; m++) U[m * F + g] = G[m];
  }
}

// U_average_conner, sub_boundary.f90:595-612: the corner ghost cell i4 takes
// rho, u, v, T extrapolated from its neighbours i1, i3 across the corner of
// i2.  One warp per corner; lanes 0..2 form the primitives of i1, i2, i3 side
// by side (the divisions by rho as reciprocal-multiplies), lane 0 combines.
__device__ void corner(const Lvl &L, const CaseDev &c, long long i1, long long i2, long long i3, long long i4) {
  const long long F = L.F;
  double *U = L.U;
  const int lane = threadIdx.x & 31;
  const long long src = lane == 0 ? i1 : lane == 1 ? i2 : i3;
  double d = 0.0, uu = 0.0, v = 0.0, T = 0.0;
  if (lane < 3) {
    d = U[src];
    const double rd = rcp(d);
    uu = U[F + src] * rd;
    v = U[2 * F + src] * rd;
    T = (U[3 * F + src] - (uu * U[F + src] + v * U[2 * F + src]) * 0.5) * (rd * c.rCv);
  }
  const double d2 = __shfl_sync(0xffffffffu, d, 1), u2 = __shfl_sync(0xffffffffu, uu, 1);
  const double v2 = __shfl_sync(0xffffffffu, v, 1), T2 = __shfl_sync(0xffffffffu, T, 1);
  const double d3 = __shfl_sync(0xffffffffu, d, 2), u3 = __shfl_sync(0xffffffffu, uu, 2);
  const double v3 = __shfl_sync(0xffffffffu, v, 2), T3 = __shfl_sync(0xffffffffu, T, 2);
  if (lane != 0) return;
  const double Cv = c.Cv;
  double d4 = d + d3 - d2, uu4 = uu + u3 - u2, v4 = v + v3 - v2, T4 = T + T3 - T2;
  U[i4] = d4;
  U[F + i4] = d4 * uu4;
  U[2 * F + i4] = d4 * v4;
  U[3 * F + i4] = d4 * (Cv * T4 + (uu4 * uu4 + v4 * v4) * 0.5);
  for (int m = 4; m < L.nvar; m++) U[m * F + i4] = U[m * F + i1] + U[m * F + i3] - U[m * F + i2];
}

// phases: 1 physical BCs, 2 halo copy, 4 corners, 8 nu~/k/omega clip
constexpr int BC_SMEM_SUBS = 32;  // subfaces of a block staged in shared memory
// Threads per block's CTA.  A phase costs the longest chain of its threads
// (a far-field item is some 45 dependent FP64 operations), so a thread that
// takes a second item doubles the phase: 512 threads give one item per
// thread to the phases of blocks up to 2 x 256 boundary items (the flat
// plate's 96-cell blocks have 384 in their single physical phase).
constexpr int BC_THREADS = 512;

__global__ void __launch_bounds__(BC_THREADS, 1) k_bc(Lvl L, int phases) {
  const int bk = blockIdx.x;
  const BlkDev &b = L.blk[bk];
  const CaseDev &c = L.cs[b.cas];
  const long long F = L.F;
  // the block's subface table in shared memory (global beyond 32), read by
  // the physical and the halo phases
  __shared__ SubDev ssub[BC_SMEM_SUBS];
  const int nsub = b.nsub;
  if (phases & 3) {
    for (int ks = threadIdx.x; ks < min(nsub, BC_SMEM_SUBS); ks += blockDim.x) ssub[ks] = L.sub[b.sub0 + ks];
    __syncthreads();
  }
  auto sub = [&](int ks) -> const SubDev & { return ks < BC_SMEM_SUBS ? ssub[ks] : L.sub[b.sub0 + ks]; };
  if (phases & 1) {
    // subfaces of one phase touch disjoint cells (grouped at set-up in
    // subface order): their items are spread over the CTA together
    for (int ph = 0; ph < b.nphase; ph++) {
      int total = 0;
      for (int ks = 0; ks < nsub; ks++) {
        const SubDev &s = sub(ks);
        if (s.neighb < 0 && s.phase == ph) total += s.nitem;
      }
      for (int t = threadIdx.x; t < total; t += blockDim.x) {
        int u = t, ks = 0;
        for (; ks < nsub; ks++) {
          const SubDev &s = sub(ks);
          if (s.neighb >= 0 || s.phase != ph) continue;
          if (u < s.nitem) break;
          u -= s.nitem;
        }
        const SubDev &s = sub(ks);
        int ni = s.iend - s.ist + 1;
        if (s.neighb == BC_Farfield || s.neighb == BC_Inlet || s.neighb == BC_Outlet) {
          bc_farfield(L, b, c, s, s.ist + u % ni, s.jst + u / ni, L.bcn[s.nrm0 + u]);
        } else {
          int k = u % LAP + 1, r = u / LAP;
          int i = s.ist + r % ni, j = s.jst + r / ni;
          if (s.neighb == BC_Wall) bc_wall(L, b, c, s, i, j, k);
          else if (s.neighb == BC_Symmetry) bc_symmetry(L, b, s, i, j, k, L.bcn[s.nrm0 + r]);
        }
      }
      __syncthreads();
    }
  }
  if (phases & 2) {
    for (int ks = 0; ks < nsub; ks++) {
      const SubDev &s = sub(ks);
      if (s.neighb < 0) continue;
      int n1 = s.iend - s.ist + s.jend - s.jst;
      for (int t = threadIdx.x; t < n1 * LAP; t += blockDim.x) {
        int l = t % LAP + 1, k = t / LAP + 1;
        int k1 = (s.orient == 2) ? k : n1 + 1 - k;
        int si, sj;
        if (s.nface == 1) { si = s.nist + l - 1; sj = s.njst + k1 - 1; }
        else if (s.nface == 2) { si = s.nist + k1 - 1; sj = s.njst + l - 1; }
        else if (s.nface == 3) { si = s.niend - LAP - 1 + l; sj = s.njst + k1 - 1; }
        else { si = s.nist + k1 - 1; sj = s.njend - LAP - 1 + l; }
        int di, dj;
        if (s.face == 1) { di = s.ist - LAP - 1 + l; dj = s.jst + k - 1; }
        else if (s.face == 2) { di = s.ist + k - 1; dj = s.jst - LAP - 1 + l; }
        else if (s.face == 3) { di = s.iend + l - 1; dj = s.jst + k - 1; }
        else { di = s.ist + k - 1; dj = s.jend + l - 1; }
        long long src = s.noff + (long long)(sj + 2) * s.nP + (si + 2), dst = fidx(b, di, dj);
        for (int m = 0; m < L.nvar; m++) L.U[m * F + dst] = L.U[m * F + src];
      }
    }
    __syncthreads();
  }
  if (phases & 4) {
    int nx = b.nx, ny = b.ny;
    const int w = threadIdx.x >> 5;
    if (w == 0) corner(L, c, fidx(b, 1, 0), fidx(b, 1, 1), fidx(b, 0, 1), fidx(b, 0, 0));
    else if (w == 1) corner(L, c, fidx(b, 1, ny), fidx(b, 1, ny - 1), fidx(b, 0, ny - 1), fidx(b, 0, ny));
    else if (w == 2) corner(L, c, fidx(b, nx - 1, 0), fidx(b, nx - 1, 1), fidx(b, nx, 1), fidx(b, nx, 0));
    else if (w == 3) corner(L, c, fidx(b, nx - 1, ny), fidx(b, nx - 1, ny - 1), fidx(b, nx, ny - 1), fidx(b, nx, ny));
    __syncthreads();
  }
  if ((phases & 8) && L.nvar >= 5) {
    int nc = (b.nx - 1) * (b.ny - 1);
    for (int t = threadIdx.x; t < nc; t += blockDim.x) {
      int i = t % (b.nx - 1) + 1, j = t / (b.nx - 1) + 1;
      long long id = fidx(b, i, j);
      for (int m = 4; m < L.nvar; m++)
        if (L.U[m * F + id] < 0) L.U[m * F + id] = 1.0e-10;
    }
  }
}

void launch_bc(const Lvl &L, int phases, cudaStream_t s) { k_bc<<<L.nblk, BC_THREADS, 0, s>>>(L, phases); }

// set-up: the edge normals of every far-field and symmetry node (grid y: block)
__global__ void __launch_bounds__(256) k_bc_normals(Lvl L) {
  const BlkDev &b = L.blk[blockIdx.y];
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  for (int ks = 0; ks < b.nsub; ks++) {
    const SubDev &s = L.sub[b.sub0 + ks];
    const int ni = s.iend - s.ist + 1, nn = ni * (s.jend - s.jst + 1);
    if (s.nrm0 < 0 || t >= nn) continue;
    L.bcn[s.nrm0 + t] = edge_normal(L, b, s.face, s.ist + t % ni, s.jst + t / ni);
  }
}
void launch_bc_normals(const Lvl &L, int max_nodes, cudaStream_t s) {
  if (max_nodes > 0) k_bc_normals<<<dim3((max_nodes + 255) / 256, L.nblk), 256, 0, s>>>(L);
}

}  // namespace ec2d
