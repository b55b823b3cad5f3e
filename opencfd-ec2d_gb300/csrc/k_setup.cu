// k_setup.cu -- mesh set-up on the device: coarse meshes by node skipping,
// cell areas, face lengths and normals, ghost node coordinates, cell centres
// and the metric Jacobians of the finite-difference patch.
//
// The host uploads only the fine mesh's node coordinates (Mesh2d.dat); every
// derived geometry plane of every level is formed here once at set-up.  The
// file is compiled without FMA contraction, so each product and sum is
// rounded on its own as in the reference's Fortran, and the planes equal the
// reference's arrays bit for bit.
#include "ec2d_dev.cuh"
#include "ec2d_internal.h"

namespace ec2d {

namespace {

constexpr int SETUP_THREADS = 256;

__device__ __forceinline__ double &GX(const Lvl &L, const BlkDev &b, int i, int j) {
  return L.geo[(size_t)G_X * L.F + fidx(b, i, j)];
}
__device__ __forceinline__ double &GY(const Lvl &L, const BlkDev &b, int i, int j) {
  return L.geo[(size_t)G_Y * L.F + fidx(b, i, j)];
}
__device__ __forceinline__ double &GP(const Lvl &L, int plane, const BlkDev &b, int i, int j) {
  return L.geo[(size_t)plane * L.F + fidx(b, i, j)];
}

// Creat_Mesh (sub_init.f90:276-373): node (i, j) of a coarse block is node
// (2i-1, 2j-1) of the finer block; one CTA per block
__global__ void __launch_bounds__(SETUP_THREADS) k_coarse_nodes(Lvl Lc, Lvl Lf) {
  const BlkDev &bc = Lc.blk[blockIdx.x], &bf = Lf.blk[blockIdx.x];
  const int n = bc.nx * bc.ny;
  for (int t = threadIdx.x; t < n; t += blockDim.x) {
    const int i = 1 + t % bc.nx, j = 1 + t / bc.nx;
    GX(Lc, bc, i, j) = GX(Lf, bf, 2 * i - 1, 2 * j - 1);
    GY(Lc, bc, i, j) = GY(Lf, bf, 2 * i - 1, 2 * j - 1);
  }
}

// One CTA per block, in the reference's order:
//  (a) cell areas and face lengths / unit normals from the block's own nodes
//      (Creat_Mesh1, sub_init.f90:180-204);
//  (b) ghost node coordinates of every subface in bc2d_1.in order
//      (Update_coordinate_buffer_onemesh, sub_boundary.f90:174-282): block
//      interfaces copy the neighbour's first LAP interior node layers,
//      reversed unless orient == 2; physical faces extrapolate linearly.
//      Subfaces that share an end node write the same ghost node, the later
//      one last, hence a barrier between subfaces;
//  (c) the ghost corners from the two edges that meet there;
//  (d) the cell centres over 1-LAP .. n+LAP-1.
// Reads of other blocks touch only their interior nodes, which no CTA
// writes here.
__global__ void __launch_bounds__(SETUP_THREADS) k_setup_geometry(Lvl L) {
  const BlkDev &b = L.blk[blockIdx.x];
  const int nx = b.nx, ny = b.ny;
  // (a) areas and faces
  for (int t = threadIdx.x; t < (nx - 1) * (ny - 1); t += blockDim.x) {
    const int i = 1 + t % (nx - 1), j = 1 + t / (nx - 1);
    const double v = fabs((GX(L, b, i, j) - GX(L, b, i + 1, j + 1)) * (GY(L, b, i + 1, j) - GY(L, b, i, j + 1)) -
                          (GX(L, b, i + 1, j) - GX(L, b, i, j + 1)) * (GY(L, b, i, j) - GY(L, b, i + 1, j + 1))) *
                     0.5;
    GP(L, G_VOL, b, i, j) = v;
  }
  for (int t = threadIdx.x; t < nx * (ny - 1); t += blockDim.x) {
    const int i = 1 + t % nx, j = 1 + t / nx;
    const double dx = GX(L, b, i, j + 1) - GX(L, b, i, j), dy = GY(L, b, i, j + 1) - GY(L, b, i, j);
    const double s = sqrt(dx * dx + dy * dy);
    GP(L, G_SI, b, i, j) = s;
    GP(L, G_NI1, b, i, j) = dy / s;
    GP(L, G_NI2, b, i, j) = -dx / s;
  }
  for (int t = threadIdx.x; t < (nx - 1) * ny; t += blockDim.x) {
    const int i = 1 + t % (nx - 1), j = 1 + t / (nx - 1);
    const double dx = GX(L, b, i + 1, j) - GX(L, b, i, j), dy = GY(L, b, i + 1, j) - GY(L, b, i, j);
    const double s = sqrt(dx * dx + dy * dy);
    GP(L, G_SJ, b, i, j) = s;
    GP(L, G_NJ1, b, i, j) = -dy / s;
    GP(L, G_NJ2, b, i, j) = dx / s;
  }
  // (b) ghost nodes, subface after subface
  for (int s = 0; s < b.nsub; s++) {
    const SubDev &sd = L.sub[b.sub0 + s];
    const int face = sd.face, ib2 = sd.ist, ie2 = sd.iend, jb2 = sd.jst, je2 = sd.jend;
    if (sd.neighb > 0) {
      const BlkDev &b1 = L.blk[sd.nbk];
      const int f1 = sd.nface, ib1 = sd.nist, ie1 = sd.niend, jb1 = sd.njst, je1 = sd.njend;
      const int n1 = ie2 - ib2 + je2 - jb2 + 1;
      for (int t = threadIdx.x; t < n1 * LAP; t += blockDim.x) {
        const int k = 1 + t % n1, l = 1 + t / n1;
        const int k1 = (sd.orient == 2) ? k : n1 + 1 - k;
        int si, sj, di, dj;
        if (f1 == 1) { si = ib1 + l; sj = jb1 + k1 - 1; }
        else if (f1 == 2) { si = ib1 + k1 - 1; sj = jb1 + l; }
        else if (f1 == 3) { si = ie1 - LAP - 1 + l; sj = jb1 + k1 - 1; }
        else { si = ib1 + k1 - 1; sj = je1 - LAP - 1 + l; }
        if (face == 1) { di = ib2 - LAP - 1 + l; dj = jb2 + k - 1; }
        else if (face == 2) { di = ib2 + k - 1; dj = jb2 - LAP - 1 + l; }
        else if (face == 3) { di = ie2 + l; dj = jb2 + k - 1; }
        else { di = ib2 + k - 1; dj = je2 + l; }
        GX(L, b, di, dj) = GX(L, b1, si, sj);
        GY(L, b, di, dj) = GY(L, b1, si, sj);
      }
    } else {
      const int n = (face == 1 || face == 3) ? je2 - jb2 + 1 : ie2 - ib2 + 1;
      for (int t = threadIdx.x; t < n * LAP; t += blockDim.x) {
        const int k = t % n, l = 1 + t / n;
        if (face == 1) {
          const int j = jb2 + k;
          GX(L, b, ib2 - l, j) = 2.0 * GX(L, b, ib2, j) - GX(L, b, ib2 + l, j);
          GY(L, b, ib2 - l, j) = 2.0 * GY(L, b, ib2, j) - GY(L, b, ib2 + l, j);
        } else if (face == 2) {
          const int i = ib2 + k;
          GX(L, b, i, jb2 - l) = 2.0 * GX(L, b, i, jb2) - GX(L, b, i, jb2 + l);
          GY(L, b, i, jb2 - l) = 2.0 * GY(L, b, i, jb2) - GY(L, b, i, jb2 + l);
        } else if (face == 3) {
          const int j = jb2 + k;
          GX(L, b, ie2 + l, j) = 2.0 * GX(L, b, ie2, j) - GX(L, b, ie2 - l, j);
          GY(L, b, ie2 + l, j) = 2.0 * GY(L, b, ie2, j) - GY(L, b, ie2 - l, j);
        } else {
          const int i = ib2 + k;
          GX(L, b, i, je2 + l) = 2.0 * GX(L, b, i, je2) - GX(L, b, i, je2 - l);
          GY(L, b, i, je2 + l) = 2.0 * GY(L, b, i, je2) - GY(L, b, i, je2 - l);
        }
      }
    }
    __syncthreads();
  }
  // (c) corners: each reads only edge ghost nodes and boundary nodes
  if (threadIdx.x < LAP * LAP) {
    const int i = 1 + threadIdx.x % LAP, j = 1 + threadIdx.x / LAP;
    const int i1 = 1 - i, j1 = 1 - j, i2 = nx + i, j2 = ny + j;
    double *P[2] = {L.geo + (size_t)G_X * L.F, L.geo + (size_t)G_Y * L.F};
    for (int q = 0; q < 2; q++) {
      double *A = P[q];
      A[fidx(b, i1, j1)] = A[fidx(b, i1, 1)] + A[fidx(b, 1, j1)] - A[fidx(b, 1, 1)];
      A[fidx(b, i2, j2)] = A[fidx(b, i2, ny)] + A[fidx(b, nx, j2)] - A[fidx(b, nx, ny)];
      A[fidx(b, i1, j2)] = A[fidx(b, i1, ny)] + A[fidx(b, 1, j2)] - A[fidx(b, 1, ny)];
      A[fidx(b, i2, j1)] = A[fidx(b, i2, 1)] + A[fidx(b, nx, j1)] - A[fidx(b, nx, 1)];
    }
  }
  __syncthreads();
  // (d) cell centres
  const int w = nx + 2 * LAP - 1, h = ny + 2 * LAP - 1;
  for (int t = threadIdx.x; t < w * h; t += blockDim.x) {
    const int i = 1 - LAP + t % w, j = 1 - LAP + t / w;
    GP(L, G_X1, b, i, j) = (GX(L, b, i, j) + GX(L, b, i + 1, j) + GX(L, b, i, j + 1) + GX(L, b, i + 1, j + 1)) * 0.25;
    GP(L, G_Y1, b, i, j) = (GY(L, b, i, j) + GY(L, b, i + 1, j) + GY(L, b, i, j + 1) + GY(L, b, i + 1, j + 1)) * 0.25;
  }
}

// dx0 / dy0 (sub_Finite_Difference.f90:387-439): sixth-order central
// differences inside, one-sided and fourth-order ones at the ends, of a
// cell-centre plane along i (di) or j (dj); n = cells in that direction
__device__ __forceinline__ double d_line(const double *f, long long o, long long st, int k, int n) {
  const double b1 = 8.0 / 12.0, b2 = 1.0 / 12.0, a1 = 1.0 / 60.0, a2 = -3.0 / 20.0, a3 = 3.0 / 4.0;
  auto F = [&](int m) { return f[o + (long long)(m - k) * st]; };
  if (k >= 4 && k <= n - 3) return a1 * (F(k + 3) - F(k - 3)) + a2 * (F(k + 2) - F(k - 2)) + a3 * (F(k + 1) - F(k - 1));
  if (k == 1) return (-3.0 * F(1) + 4.0 * F(2) - F(3)) / 2.0;
  if (k == 2) return (-2.0 * F(1) - 3.0 * F(2) + 6.0 * F(3) - F(4)) / 6.0;
  if (k == 3) return b1 * (F(4) - F(2)) - b2 * (F(5) - F(1));
  if (k == n - 2) return b1 * (F(n - 1) - F(n - 3)) - b2 * (F(n) - F(n - 4));
  if (k == n - 1) return (F(n - 3) - 6.0 * F(n - 2) + 3.0 * F(n - 1) + 2.0 * F(n)) / 6.0;
  return (F(n - 2) - 4.0 * F(n - 1) + 3.0 * F(n)) / 2.0;
}

// comput_Jacobian (sub_Finite_Difference.f90:314-382) for the blocks of
// FDM.in: Akx, Aky, Aix, Aiy and the Jacobian at the cell centres; the
// Jacobian plane is 1 over the rest of the block's frame
__global__ void __launch_bounds__(SETUP_THREADS) k_fdm_metrics(Lvl L) {
  const BlkDev &b = L.blk[blockIdx.x];
  if (!b.fdm) return;
  const int nx = b.nx - 1, ny = b.ny - 1;
  const double *x1 = L.geo + (size_t)G_X1 * L.F, *y1 = L.geo + (size_t)G_Y1 * L.F;
  double *akx = L.met, *aky = L.met + L.F, *aix = L.met + 2 * L.F, *aiy = L.met + 3 * L.F, *ajac = L.met + 4 * L.F;
  const int fr = b.P * (b.ny + 5);
  for (int t = threadIdx.x; t < fr; t += blockDim.x) ajac[b.off + t] = 1.0;
  __syncthreads();
  for (int t = threadIdx.x; t < nx * ny; t += blockDim.x) {
    const int i = 1 + t % nx, j = 1 + t / nx;
    const long long o = fidx(b, i, j);
    const double xk = d_line(x1, o, 1, i, nx), yk = d_line(y1, o, 1, i, nx);
    const double xi = d_line(x1, o, b.P, j, ny), yi = d_line(y1, o, b.P, j, ny);
    const double J = 1.0 / (xk * yi - xi * yk);
    ajac[o] = J;
    akx[o] = J * yi;
    aky[o] = -J * xi;
    aix[o] = -J * yk;
    aiy[o] = J * xk;
  }
}

}  // namespace

void launch_setup_geometry(const Lvl &L, const Lvl *finer, bool fdm, cudaStream_t s) {
  if (finer) k_coarse_nodes<<<L.nblk, SETUP_THREADS, 0, s>>>(L, *finer);
  k_setup_geometry<<<L.nblk, SETUP_THREADS, 0, s>>>(L);
  if (fdm) k_fdm_metrics<<<L.nblk, SETUP_THREADS, 0, s>>>(L);
}

}  // namespace ec2d
