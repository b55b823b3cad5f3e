// k_misc.cu -- layout conversion at the C-ABI boundary, wall distance and
// wall forces.
#include "ec2d_dev.cuh"
#include "ec2d_internal.h"

namespace ec2d {

// Fortran U(NVAR,-1:nx+1,-1:ny+1) (variable fastest) <-> frame planes
__global__ void k_pack_u(Lvl L, int bk, int nv, const double *aos) {
  const BlkDev &b = L.blk[bk];
  int W = b.nx + 3, H = b.ny + 3;
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= W * H) return;
  int i = t % W - 1, j = t / W - 1;
  long long id = fidx(b, i, j);
  for (int m = 0; m < nv; m++) L.U[m * L.F + id] = aos[(size_t)m + (size_t)nv * t];
}
__global__ void k_unpack_u(Lvl L, int bk, int nv, double *aos) {
  const BlkDev &b = L.blk[bk];
  int W = b.nx + 3, H = b.ny + 3;
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= W * H) return;
  int i = t % W - 1, j = t / W - 1;
  long long id = fidx(b, i, j);
  for (int m = 0; m < nv; m++) aos[(size_t)m + (size_t)nv * t] = L.U[m * L.F + id];
}
void launch_pack_u(const Lvl &L, int bk, int nv, const double *aos, int nitems, cudaStream_t s) {
  k_pack_u<<<(nitems + 255) / 256, 256, 0, s>>>(L, bk, nv, aos);
}
void launch_unpack_u(const Lvl &L, int bk, int nv, double *aos, int nitems, cudaStream_t s) {
  k_unpack_u<<<(nitems + 255) / 256, 256, 0, s>>>(L, bk, nv, aos);
}

// comput_dw (sub_turbulence_SST.f90:310-340): nearest wall node of the case for
// every node, then the cell value as the mean of its four nodes.  Pass 1
// writes node distances into the Q_C plane (free during setup), pass 2 the
// cells.  Wall node coordinates are staged through shared memory.
__global__ void k_dw_nodes(Lvl L, int bk, const double *wxy, int nwall) {
  extern __shared__ double sw[];
  const BlkDev &b = L.blk[bk];
  int n = b.nx * b.ny;
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  int i = t % b.nx + 1, j = t / b.nx + 1;
  double px = 0, py = 0;
  if (t < n) {
    long long id = fidx(b, i, j);
    px = L.geo[G_X * L.F + id];
    py = L.geo[G_Y * L.F + id];
  }
  double best = 1.0e10;
  for (int w0 = 0; w0 < nwall; w0 += 512) {
    int cnt = min(512, nwall - w0);
    __syncthreads();
    for (int k = threadIdx.x; k < cnt; k += blockDim.x) { sw[2 * k] = wxy[2 * (w0 + k)]; sw[2 * k + 1] = wxy[2 * (w0 + k) + 1]; }
    __syncthreads();
    for (int k = 0; k < cnt; k++) {
      double dx = px - sw[2 * k], dy = py - sw[2 * k + 1];
      double d1 = sqrt(dx * dx + dy * dy);
      if (d1 < best) best = d1;
    }
  }
  if (t < n) L.q[Q_C * L.F + fidx(b, i, j)] = best;
}
__global__ void k_dw_cells(Lvl L, int bk) {
  const BlkDev &b = L.blk[bk];
  int W = b.nx + 1, H = b.ny + 1;  // 0..nx, 0..ny
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= W * H) return;
  int i = t % W, j = t / W;
  long long id = fidx(b, i, j);
  double v = 1.0;
  if (i >= 1 && i <= b.nx - 1 && j >= 1 && j <= b.ny - 1) {
    const double *nd = L.q + Q_C * L.F;
    v = (nd[id] + nd[id + 1] + nd[id + b.P] + nd[id + b.P + 1]) * 0.25;
  }
  L.geo[G_DW * L.F + id] = v;
}
void launch_wall_distance(const Lvl &L, int bk, const double *wall_xy, int nwall, int nx, int ny, cudaStream_t s) {
  k_dw_nodes<<<(nx * ny + 255) / 256, 256, 512 * 2 * sizeof(double), s>>>(L, bk, wall_xy, nwall);
  k_dw_cells<<<((nx + 1) * (ny + 1) + 255) / 256, 256, 0, s>>>(L, bk);
}

// Wall forces (no counterpart in the reference; its read_flow-1.2.f90:36-51
// writes wall Cp only).  faces[k] = (block, face, k-index, unused): for each
// wall face, pressure = mean of the interior cell and its first ghost minus
// p_inf, viscous traction from the face-gradient formula of Residual_FVM with
// the laminar viscosity at the mean of the two cell temperatures.  Output per
// face: fx, fy, x_mid, y_mid, cf (normal pointing into the fluid).
__global__ void k_forces(Lvl L, const int4 *faces, int nfaces, double *out) {
  int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nfaces) return;
  int4 fc = faces[f];
  const BlkDev &b = L.blk[fc.x];
  const CaseDev &c = L.cs[b.cas];
  const long long F = L.F, P = b.P;
  int face = fc.y, k = fc.z, nx = b.nx, ny = b.ny;
  bool ifc = (face == 1 || face == 3);
  int fi, fj, ci, cj, gi, gj;
  if (face == 1) { fi = 1; fj = k; ci = 1; cj = k; gi = 0; gj = k; }
  else if (face == 3) { fi = nx; fj = k; ci = nx - 1; cj = k; gi = nx; gj = k; }
  else if (face == 2) { fi = k; fj = 1; ci = k; cj = 1; gi = k; gj = 0; }
  else { fi = k; fj = ny; ci = k; cj = ny - 1; gi = k; gj = ny; }
  long long id = fidx(b, fi, fj), ic = fidx(b, ci, cj), ig = fidx(b, gi, gj);
  const double *x = L.geo + G_X * F, *y = L.geo + G_Y * F, *x1 = L.geo + G_X1 * F, *y1 = L.geo + G_Y1 * F;
  double n1, n2, s, xm, ym;
  if (ifc) { n1 = L.geo[G_NI1 * F + id]; n2 = L.geo[G_NI2 * F + id]; s = L.geo[G_SI * F + id];
             xm = 0.5 * (x[id] + x[id + P]); ym = 0.5 * (y[id] + y[id + P]); }
  else { n1 = L.geo[G_NJ1 * F + id]; n2 = L.geo[G_NJ2 * F + id]; s = L.geo[G_SJ * F + id];
         xm = 0.5 * (x[id] + x[id + 1]); ym = 0.5 * (y[id] + y[id + 1]); }
  double sgn = ((x1[ic] - xm) * n1 + (y1[ic] - ym) * n2) >= 0.0 ? 1.0 : -1.0;
  const double *qp = L.q + Q_P * F, *uu = L.q + Q_U * F, *vv = L.q + Q_V * F, *TT = L.q + Q_T * F;
  double pw = 0.5 * (qp[ic] + qp[ig]) - c.p00;
  double fx = 0.0, fy = 0.0, f4 = 0.0;
  if (L.visc) {
    double T = 0.5 * (TT[ic] + TT[ig]);
    double Amu1 = 1.0 / c.Re * (1.0 + c.Tsb) * sqrt(T * T * T) / (c.Tsb + T);
    double Dix, Diy, Djx, Djy, Diu, Div, DiT, Dju, Djv, DjT;
    if (ifc) {
      long long w = id - 1, nN = id + P, nS = id - P;
      Dix = x1[id] - x1[w]; Diy = y1[id] - y1[w];
      Djx = (x1[nN - 1] + x1[nN] - x1[nS - 1] - x1[nS]) * 0.25;
      Djy = (y1[nN - 1] + y1[nN] - y1[nS - 1] - y1[nS]) * 0.25;
      Diu = uu[id] - uu[w]; Div = vv[id] - vv[w]; DiT = TT[id] - TT[w];
      Dju = (uu[nN - 1] + uu[nN] - uu[nS - 1] - uu[nS]) * 0.25;
      Djv = (vv[nN - 1] + vv[nN] - vv[nS - 1] - vv[nS]) * 0.25;
      DjT = (TT[nN - 1] + TT[nN] - TT[nS - 1] - TT[nS]) * 0.25;
    } else {
      long long sN = id - P;
      Dix = (x1[sN + 1] + x1[id + 1] - x1[sN - 1] - x1[id - 1]) * 0.25;
      Diy = (y1[sN + 1] + y1[id + 1] - y1[sN - 1] - y1[id - 1]) * 0.25;
      Djx = x1[id] - x1[sN]; Djy = y1[id] - y1[sN];
      Diu = (uu[sN + 1] + uu[id + 1] - uu[sN - 1] - uu[id - 1]) * 0.25;
      Div = (vv[sN + 1] + vv[id + 1] - vv[sN - 1] - vv[id - 1]) * 0.25;
      DiT = (TT[sN + 1] + TT[id + 1] - TT[sN - 1] - TT[id - 1]) * 0.25;
      Dju = uu[id] - uu[sN]; Djv = vv[id] - vv[sN]; DjT = TT[id] - TT[sN];
    }
    viscous_face(Dix, Diy, Djx, Djy, Diu, Div, DiT, Dju, Djv, DjT, Amu1, 0.0, 0.0, 0.0, sgn * n1, sgn * n2, s, fx,
                 fy, f4);
  }
  double t1 = ifc ? -n2 : n2, t2 = ifc ? n1 : -n1;
  out[5 * f + 0] = -pw * sgn * n1 * s + fx;
  out[5 * f + 1] = -pw * sgn * n2 * s + fy;
  out[5 * f + 2] = xm;
  out[5 * f + 3] = ym;
  out[5 * f + 4] = ((fx * t1 + fy * t2) / s) / 0.5;
}
void launch_forces(const Lvl &L, const int4 *faces, int nfaces, double *out, cudaStream_t s) {
  if (nfaces > 0) k_forces<<<(nfaces + 127) / 128, 128, 0, s>>>(L, faces, nfaces, out);
}

}  // namespace ec2d
