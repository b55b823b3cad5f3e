// ec2d_api.cu -- the C-ABI (include/ec2d_gpu.h): context, one-time setup
// (block and subface tables, device layout on the host; the geometry of every
// level, ghost coordinates, coarse meshes and FDM metrics by the set-up
// kernels of k_setup.cu) and the orchestration of the pseudo-time-marching sequences of
// sub_NS_singlegrid.f90 and sub_NS_multigrid.f90 as kernel launches on the
// context's stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <set>
#include <string>
#include <utility>
#include <vector>

#include "../../include/ec2d_gpu.h"
#include "ec2d_dev.cuh"
#include "ec2d_internal.h"
#include "ec2d_mlp.h"

using namespace ec2d;

namespace {

const double PI = 3.1415926535897932;
constexpr int TILE = EC2D_TILE;

struct HBlock {
  int nx = 0, ny = 0;
  std::vector<double> x, y;  // (1:nx,1:ny), i fastest
  std::vector<int> bc;       // 9 per subface
  int nsub = 0;
  bool fdm = false;
  std::vector<double> dw;    // supplied wall distance (1:nx-1,1:ny-1) or empty
};

struct HCase {
  ec2d_params p{};
  std::vector<HBlock> blocks;
  int nvar = 4;
  int kstep[4] = {0, 0, 0, 0};
  double tt[4] = {0, 0, 0, 0};
};

// host-side frame-indexed 2-D array of one block
struct Frame {
  int nx = 0, ny = 0, P = 0;
  std::vector<double> v;
  void init(int nx_, int ny_, double val = 0.0) {
    nx = nx_; ny = ny_; P = nx + 5;
    v.assign((size_t)P * (ny + 5), val);
  }
  double &operator()(int i, int j) { return v[(size_t)(j + 2) * P + (i + 2)]; }
};

struct HLevelBlock {
  int nx, ny, cas, blk;  // blk: 0-based block number within its case
  std::vector<int> bc;   // 9 per subface (level indices)
  int nsub;
  bool fdm;
  Frame x, y;  // fine level: the nodes from Mesh2d.dat (geometry is formed on the device)
};

struct DevBuf {
  void *p = nullptr;
  ~DevBuf() { if (p) cudaFree(p); }
};

struct Level {
  std::vector<HLevelBlock> hb;
  std::vector<BlkDev> blk;
  std::vector<SubDev> sub;
  std::vector<int2> tiles, ctiles;  // extended and core windows (core_ij)
  std::vector<int> case_tile0, case_ntile, case_ncell;  // case ranges of ctiles
  std::vector<int4> wall_faces;          // (block, face, k, 0) for forces
  std::vector<int> case_face0, case_nface;
  long long F = 0;
  int max_rows = 0;   // widest block (ny-1) of the level: LU-SGS threads per CTA
  int max_cols = 0;   // longest row of cells (nx-1) of the level's blocks
  int bc_max_nodes = 0;  // most boundary nodes of one far-field / symmetry subface
  bool fast64 = false, fast32 = false;  // wavefront LU-SGS fits one CTA (FP64 / FP32 records)
  Lvl L{};
  int *d_case_tile0 = nullptr, *d_case_ntile = nullptr, *d_case_ncell = nullptr;
  int4 *d_faces = nullptr;
  double *d_face_out = nullptr;
  // 2-D cell tiles of the one-kernel residual (k_residual_tile): (block, i0,
  // j0), per-case ranges, norm partials and the last-tile counter
  int n_rtiles = 0;
  int4 *d_rtiles = nullptr;
  int *d_rcase_tile0 = nullptr, *d_rcase_ntile = nullptr;
  double *d_rnpart = nullptr;
  unsigned *d_rnctr = nullptr;
  std::vector<std::unique_ptr<DevBuf>> bufs;
};

}  // namespace

struct ec2d_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t side = nullptr;           // second stream for concurrent independent kernels
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  // a second stream pair (and its fork / join events) for the branch of a
  // multigrid transfer that runs beside the fine residual, and the events
  // that open and close that branch
  cudaStream_t stream2 = nullptr, side2 = nullptr;
  cudaEvent_t ev_fork2 = nullptr, ev_join2 = nullptr, ev_b0 = nullptr, ev_b1 = nullptr;
  // the norms branch: inside a step, a residual evaluation's norms (tile
  // partials, per-case reduction) run on their own stream beside the kernels
  // that follow; the next evaluation of the same level, and the end of the
  // step, wait for them (norm_open)
  cudaStream_t nstream = nullptr;
  cudaEvent_t ev_nfork[4] = {}, ev_norm[4] = {};
  bool norm_open[4] = {false, false, false, false};
  bool norm_branch = false;  // set while one_step issues its work
  std::vector<HCase> cases;
  bool setup_done = false;
  int num_mesh = 1;
  int nvar = 4;
  ec2d_params P{};  // method flags (shared by all cases)
  Level lv[4];
  CaseDev *d_cases = nullptr;
  double *d_stage = nullptr;  // staging for U upload/download
  double *d_shape = nullptr;  // per-case shape feature of the warm-start network
  size_t stage_n = 0;
  int dual_iflag1 = 0, dual_iflag = 0;
  int last_err = 0;
  // launch accounting and optional per-kernel event timing
  long long launches = 0;
  int lusgs_cs = 0;  // LU-SGS wavefront shape: 0 four lanes per row where it fits, 1 one CTA per block, >1 a cluster
  bool lusgs_fp32 = false;  // LU-SGS sweeps in FP32 (mixed-precision mode)
  bool concurrent = true;   // i- and j-face flux kernels on two streams
  // test hook (EC2D_TEST_SILENT_BAND_EDGE): the band edges of the four-lane
  // wavefront send nothing, so the downstream waits run out and report
  // EC2D_ERR_TIMEOUT; failure detection is tested without a GPU fault
  bool silent_band_edge = false;
  int lusgs_rpw = 12;       // most rows per CTA of the banded kernel (<= 16: eight lanes per row), or rows per warp of the one-lane one
  int lusgs_lanes = 0;      // lanes per row of the banded kernel: 4 or 8, 0 by the rows (eight up to 16)
  bool coarse_fp32 = false; // face fluxes of multigrid levels >= 2 in FP32
  bool tile_residual = false; // the one-kernel residual where it applies (no turbulence model, no FDM patch, FP64)
  // extension for turbulent multigrid runs: the coarse levels keep the eddy
  // viscosity restricted from the finer level (the reference's are laminar)
  bool mg_amut = false;
  bool timing = false;
  // one pseudo-time step (single grid or V-cycle) captured as a CUDA graph:
  // the replay stands for graph_launches kernel launches and advances the
  // host step counters of level l graph_adv[l] times
  bool use_graphs = true;
  cudaGraphExec_t step_graph = nullptr;
  long long graph_launches = 0;
  int graph_adv[4] = {0, 0, 0, 0};
  struct KRec { const char *name; int level, nk; cudaEvent_t a, b; };
  std::vector<KRec> krec;
  std::vector<cudaEvent_t> evpool;
  // asynchronous snapshot of one case's fine-level U (ec2d_snapshot): the
  // blocks in the reference's layout, packed on the device on the main
  // stream, then copied to pinned host memory on the snapshot stream while
  // the main stream runs on
  cudaStream_t snap_stream = nullptr;
  cudaEvent_t ev_snap = nullptr, ev_snap_done = nullptr;
  double *d_snap = nullptr, *h_snap = nullptr;
  size_t snap_cap = 0;
  int snap_case = 0, snap_kstep = 0;
  double snap_tt = 0.0;
  bool snap_pending = false;
  std::vector<size_t> snap_off;  // per block of the case: offset in the snapshot
};

namespace {

#define CK(x)                                            \
  do {                                                   \
    cudaError_t e_ = (x);                                \
    if (e_ != cudaSuccess) {                             \
      fprintf(stderr, "ec2d: CUDA error %s at %s:%d\n", cudaGetErrorString(e_), __FILE__, __LINE__); \
      return EC2D_ERR_CUDA;                              \
    }                                                    \
  } while (0)

template <class T>
T *dalloc(Level &lv, size_t n) {
  auto b = std::make_unique<DevBuf>();
  if (n == 0) n = 1;
  if (cudaMalloc(&b->p, n * sizeof(T)) != cudaSuccess) return nullptr;
  cudaMemset(b->p, 0, n * sizeof(T));
  T *r = (T *)b->p;
  lv.bufs.push_back(std::move(b));
  return r;
}

bool same_method(const ec2d_params &a, const ec2d_params &b) {
  return a.If_viscous == b.If_viscous && a.Iflag_turbulence_model == b.Iflag_turbulence_model &&
         a.Time_Method == b.Time_Method && a.Iflag_Scheme == b.Iflag_Scheme && a.Iflag_flux == b.Iflag_flux &&
         a.IFlag_Reconstruction == b.IFlag_Reconstruction && a.Num_Mesh == b.Num_Mesh && a.mg_lusgs == b.mg_lusgs;
}

// check_mesh_multigrid (sub_init.f90:39-107)
int mg_depth(const HCase &c) {
  int Km_grid = c.blocks[0].nx;
  for (auto &B : c.blocks) {
    int Km = 1, NN = 2;
    while ((B.nx - 1) % NN == 0 && (B.nx - 1) / NN >= 2 && (B.ny - 1) % NN == 0 && (B.ny - 1) / NN >= 2) { Km++; NN *= 2; }
    Km_grid = std::min(Km_grid, Km);
  }
  for (auto &B : c.blocks)
    for (int k = 0; k < B.nsub; k++) {
      const int *s = &B.bc[9 * k];
      int NN = 1, Km = 1;
      while ((s[2] - 1) % NN == 0 && (s[3] - 1) % NN == 0 && (s[4] - 1) % NN == 0 && (s[5] - 1) % NN == 0) {
        NN *= 2; Km++;
        if (NN > (1 << 20)) break;
      }
      Km_grid = std::min(Km_grid, Km);
    }
  return std::min(3, std::min(Km_grid, c.p.Num_Mesh));
}

CaseDev make_casedev(const ec2d_params &p) {
  CaseDev c{};
  c.gamma = p.gamma; c.Ma = p.Ma; c.Re = p.Re; c.Pr = p.Pr;
  c.rPr = 1.0 / p.Pr;
  c.rMa = 1.0 / p.Ma;
  c.rRe = 1.0 / p.Re;
  c.rgm1 = 1.0 / (p.gamma - 1.0);
  c.ggm1 = p.gamma / (p.gamma - 1.0);
  c.Cv = 1.0 / (p.gamma * (p.gamma - 1.0) * p.Ma * p.Ma);
  c.rCv = p.gamma * (p.gamma - 1.0) * p.Ma * p.Ma;
  c.Cp = c.Cv * p.gamma;
  double aoa = p.AoA * PI / 180.0;
  c.cosA = 1.0 * std::cos(aoa); c.sinA = 1.0 * std::sin(aoa);
  c.p00 = 1.0 / (p.gamma * p.Ma * p.Ma);
  c.Tsb = 110.4 / p.T_inf;
  c.Twall = p.Twall / p.T_inf;
  c.p_outlet = p.P_outlet; c.vt_inf = p.vt_inf; c.Kt_inf = p.Kt_inf; c.Wt_inf = p.Wt_inf;
  c.CFL = p.CFL; c.dtmax = p.dtmax; c.dtmin = p.dtmin; c.dt_global = p.dt_global; c.T_inf = p.T_inf;
  c.xaxis = p.xaxis; c.yaxis = p.yaxis;
  c.local_dt = p.Iflag_local_dt;
  return c;
}

int build_level(ec2d_ctx *ctx, int l) {
  Level &lv = ctx->lv[l];
  const ec2d_params &P = ctx->P;
  int ncase = (int)ctx->cases.size();
  // block tables (and the fine level's nodes)
  if (l == 1) {
    for (int c = 0; c < ncase; c++)
      for (int m = 0; m < (int)ctx->cases[c].blocks.size(); m++) {
        const HBlock &hb = ctx->cases[c].blocks[m];
        HLevelBlock B;
        B.nx = hb.nx; B.ny = hb.ny; B.cas = c; B.blk = m; B.bc = hb.bc; B.nsub = hb.nsub; B.fdm = hb.fdm;
        B.x.init(B.nx, B.ny);
        B.y.init(B.nx, B.ny);
        for (int j = 1; j <= B.ny; j++)
          for (int i = 1; i <= B.nx; i++) {
            B.x(i, j) = hb.x[(i - 1) + (size_t)B.nx * (j - 1)];
            B.y(i, j) = hb.y[(i - 1) + (size_t)B.nx * (j - 1)];
          }
        lv.hb.push_back(std::move(B));
      }
  } else {
    // coarse mesh by node skipping (Creat_Mesh, sub_init.f90:276-373): the
    // block list and subface indices here, the nodes on the device
    for (auto &B1 : ctx->lv[l - 1].hb) {
      HLevelBlock B;
      B.nx = (B1.nx - 1) / 2 + 1; B.ny = (B1.ny - 1) / 2 + 1; B.cas = B1.cas; B.blk = B1.blk;
      B.nsub = B1.nsub; B.fdm = false; B.bc = B1.bc;
      for (int k = 0; k < B.nsub; k++)
        for (int q = 2; q <= 5; q++) B.bc[9 * k + q] = (B1.bc[9 * k + q] - 1) / 2 + 1;
      lv.hb.push_back(std::move(B));
    }
  }
  // device layout
  std::vector<int> case_first_block(ncase, -1);
  long long off = 0;
  int tile = 0, ctile = 0, sub0 = 0;
  lv.case_tile0.assign(ncase, 0); lv.case_ntile.assign(ncase, 0); lv.case_ncell.assign(ncase, 0);
  for (int k = 0; k < (int)lv.hb.size(); k++) {
    auto &B = lv.hb[k];
    if (case_first_block[B.cas] < 0) { case_first_block[B.cas] = k; lv.case_tile0[B.cas] = ctile; }
    BlkDev d{};
    d.nx = B.nx; d.ny = B.ny; d.P = B.nx + 5; d.cas = B.cas; d.off = off; d.fdm = B.fdm ? 1 : 0;
    d.nsub = B.nsub; d.sub0 = sub0; d.tile0 = tile;
    d.cell0 = lv.L.ncell;
    lv.L.ncell += (B.nx - 1) * (B.ny - 1);
    off += ((long long)d.P * (B.ny + 5) + 31) / 32 * 32;
    int items = (B.nx + 3) * (B.ny + 3);
    int nt = (items + TILE - 1) / TILE;
    for (int t = 0; t < nt; t++) lv.tiles.push_back(make_int2(k, t * TILE));
    tile += nt;
    const int nct = ((B.nx + 1) * (B.ny + 1) + TILE - 1) / TILE;
    for (int t = 0; t < nct; t++) lv.ctiles.push_back(make_int2(k, t * TILE));
    ctile += nct;
    lv.case_ntile[B.cas] += nct;
    lv.case_ncell[B.cas] += (B.nx - 1) * (B.ny - 1);
    for (int s = 0; s < B.nsub; s++) {
      const int *c = &B.bc[9 * s];
      SubDev sd{};
      sd.face = c[1]; sd.ist = c[2]; sd.iend = c[3]; sd.jst = c[4]; sd.jend = c[5]; sd.neighb = c[6]; sd.orient = c[8];
      sd.nbk = -1;
      lv.sub.push_back(sd);
    }
    sub0 += B.nsub;
    lv.blk.push_back(d);
  }
  // resolve neighbours to level-global block ids
  for (int k = 0; k < (int)lv.hb.size(); k++) {
    auto &B = lv.hb[k];
    for (int s = 0; s < B.nsub; s++) {
      SubDev &sd = lv.sub[lv.blk[k].sub0 + s];
      if (sd.neighb < 0) continue;
      int nb = case_first_block[B.cas] + sd.neighb - 1;
      if (sd.neighb < 1 || nb >= (int)lv.hb.size() || lv.hb[nb].cas != B.cas) return EC2D_ERR_ARG;
      int msub = B.bc[9 * s + 7];
      if (msub < 1 || msub > lv.hb[nb].nsub) return EC2D_ERR_ARG;
      const int *c1 = &lv.hb[nb].bc[9 * (msub - 1)];
      // the copied strip must have the same cell count on both sides
      if ((sd.iend - sd.ist + sd.jend - sd.jst) != (c1[3] - c1[2] + c1[5] - c1[4])) return EC2D_ERR_ARG;
      sd.nbk = nb; sd.nface = c1[1]; sd.nist = c1[2]; sd.niend = c1[3]; sd.njst = c1[4]; sd.njend = c1[5];
      sd.nP = lv.blk[nb].P; sd.noff = lv.blk[nb].off;
    }
  }
  // physical boundary conditions: a subface joins the earliest barrier phase
  // after every earlier subface of the block whose cells (ghosts written,
  // cells read) meet its own; far-field items cover all ghost layers of a
  // boundary node, wall and symmetry items one layer
  for (int k = 0; k < (int)lv.hb.size(); k++) {
    BlkDev &d = lv.blk[k];
    std::vector<std::set<long long>> rd(d.nsub), wr(d.nsub);
    auto key = [](int i, int j) { return (long long)(i + 8) * 1000003LL + (j + 8); };
    int nph = 0;
    for (int s = 0; s < d.nsub; s++) {
      SubDev &sd = lv.sub[d.sub0 + s];
      sd.phase = -1;
      if (sd.neighb >= 0) continue;
      int ni = sd.iend - sd.ist + 1, nj = sd.jend - sd.jst + 1;
      bool ff = sd.neighb == BC_Farfield || sd.neighb == BC_Inlet || sd.neighb == BC_Outlet;
      sd.nitem = ff ? ni * nj : ni * nj * LAP;
      for (int j = sd.jst; j <= sd.jend; j++)
        for (int i = sd.ist; i <= sd.iend; i++)
          for (int q = 1; q <= LAP; q++) {
            int i1 = i, j1 = j, i2 = i, j2 = j;
            if (sd.face == 1) { i1 = i + q - 1; i2 = i - q; }
            else if (sd.face == 2) { j1 = j + q - 1; j2 = j - q; }
            else if (sd.face == 3) { i1 = i - q; i2 = i + q - 1; }
            else { j1 = j - q; j2 = j + q - 1; }
            rd[s].insert(key(i1, j1));
            wr[s].insert(key(i2, j2));
          }
      auto meet = [](const std::set<long long> &a, const std::set<long long> &b) {
        for (long long v : a) if (b.count(v)) return true;
        return false;
      };
      int ph = 0;
      for (int e = 0; e < s; e++) {
        const SubDev &se = lv.sub[d.sub0 + e];
        if (se.phase < 0) continue;
        if (meet(wr[e], rd[s]) || meet(wr[e], wr[s]) || meet(rd[e], wr[s])) ph = std::max(ph, se.phase + 1);
      }
      sd.phase = ph;
      nph = std::max(nph, ph + 1);
    }
    d.nphase = nph;
  }
  // far-field and symmetry subfaces: one edge normal per boundary node,
  // filled on the device once the coordinates are there
  int nbcn = 0;
  for (auto &sd : lv.sub) {
    sd.nrm0 = -1;
    bool need = sd.neighb == BC_Farfield || sd.neighb == BC_Inlet || sd.neighb == BC_Outlet || sd.neighb == BC_Symmetry;
    if (!need) continue;
    int nn = (sd.iend - sd.ist + 1) * (sd.jend - sd.jst + 1);
    sd.nrm0 = nbcn;
    nbcn += nn;
    lv.bc_max_nodes = std::max(lv.bc_max_nodes, nn);
  }
  // wall faces for forces (fine level only)
  if (l == 1) {
    lv.case_face0.assign(ncase, 0); lv.case_nface.assign(ncase, 0);
    for (int c = 0; c < ncase; c++) {
      lv.case_face0[c] = (int)lv.wall_faces.size();
      for (int k = 0; k < (int)lv.hb.size(); k++) {
        auto &B = lv.hb[k];
        if (B.cas != c) continue;
        lv.blk[k].lsub0 = (int)lv.wall_faces.size();
        for (int s = 0; s < B.nsub; s++) {
          const int *cc = &B.bc[9 * s];
          if (cc[6] != BC_Wall) continue;
          bool ifc = (cc[1] == 1 || cc[1] == 3);
          int kb = ifc ? cc[4] : cc[2], ke = ifc ? cc[5] - 1 : cc[3] - 1;
          for (int q = kb; q <= ke; q++) lv.wall_faces.push_back(make_int4(k, cc[1], q, s));
        }
      }
      lv.case_nface[c] = (int)lv.wall_faces.size() - lv.case_face0[c];
    }
  }
  lv.F = off;
  const long long F = off;
  // allocate device fields
  Lvl &L = lv.L;
  L.nblk = (int)lv.blk.size();
  L.ncase = ncase;
  L.ntiles = (int)lv.tiles.size();
  L.nctiles = (int)lv.ctiles.size();
  L.F = F;
  L.level = l;
  L.nvar = (l == 1) ? ctx->nvar : 4;
  L.scheme = (l == 1) ? P.Iflag_Scheme : Scheme_UD1;
  L.gscheme = P.Iflag_Scheme;
  L.flux = P.Iflag_flux;
  L.recon = P.IFlag_Reconstruction;
  L.visc = P.If_viscous;
  L.turb = (l == 1) ? P.Iflag_turbulence_model : Turb_NONE;
  L.time_method = P.Time_Method;
  int nv = L.nvar;
  BlkDev *dblk = dalloc<BlkDev>(lv, lv.blk.size());
  SubDev *dsub = dalloc<SubDev>(lv, lv.sub.size());
  int2 *dtiles = dalloc<int2>(lv, lv.tiles.size());
  int2 *dctiles = dalloc<int2>(lv, lv.ctiles.size());
  if (!dblk || !dsub || !dtiles || !dctiles) return EC2D_ERR_NOMEM;
  CK(cudaMemcpy(dblk, lv.blk.data(), lv.blk.size() * sizeof(BlkDev), cudaMemcpyHostToDevice));
  if (!lv.sub.empty()) CK(cudaMemcpy(dsub, lv.sub.data(), lv.sub.size() * sizeof(SubDev), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(dtiles, lv.tiles.data(), lv.tiles.size() * sizeof(int2), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(dctiles, lv.ctiles.data(), lv.ctiles.size() * sizeof(int2), cudaMemcpyHostToDevice));
  L.blk = dblk; L.sub = dsub; L.tiles = dtiles; L.ctiles = dctiles; L.cs = ctx->d_cases;
  L.U = dalloc<double>(lv, nv * F);
  L.q = dalloc<double>(lv, NQ * F);
  L.amu = dalloc<double>(lv, F);
  L.amut = dalloc<double>(lv, F);
  L.res = dalloc<double>(lv, nv * F);
  L.lc = dalloc<double>(lv, NL * F);
  L.du = dalloc<double>(lv, nv * F);
  L.geo = dalloc<double>(lv, NG * F);
  L.un = dalloc<double>(lv, nv * F);
  L.deltu = dalloc<double>(lv, 4 * F);
  L.qf = dalloc<double>(lv, 4 * F);
  L.un1 = (P.Time_Method == Time_Dual && l == 1) ? dalloc<double>(lv, nv * F) : nullptr;
  L.fi = dalloc<double>(lv, 6 * F);
  L.fj = dalloc<double>(lv, 6 * F);
  L.tb = (L.turb == Turb_SST) ? dalloc<double>(lv, 5 * F) : (L.turb == Turb_BL) ? dalloc<double>(lv, F) : nullptr;
  bool anyfdm = false;
  for (auto &B : lv.hb) anyfdm |= B.fdm;
  L.met = anyfdm ? dalloc<double>(lv, 5 * F) : nullptr;
  L.fdm = anyfdm ? dalloc<double>(lv, 30 * F) : nullptr;
  for (auto &B : lv.hb) lv.max_rows = std::max(lv.max_rows, B.ny - 1);
  for (auto &B : lv.hb) lv.max_cols = std::max(lv.max_cols, B.nx - 1);
  // wavefront LU-SGS: one thread per row, its shared memory must fit one CTA
  const size_t smem_max = 227 * 1024;
  lv.fast64 = lv.max_rows <= 1024 && lusgs_smem(nv, lv.max_rows) <= smem_max;
  lv.fast32 = lv.max_rows <= 1024 && lusgs32_smem(nv, lv.max_rows) <= smem_max;
  L.rec = (lv.fast64 || lv.fast32) ? dalloc<double>(lv, (size_t)2 * L.ncell * lusgs_planes(nv)) : nullptr;
  {
    size_t nbcn = 0;
    for (auto &sd : lv.sub)
      if (sd.nrm0 >= 0) nbcn = std::max(nbcn, (size_t)sd.nrm0 + (size_t)(sd.iend - sd.ist + 1) * (sd.jend - sd.jst + 1));
    L.bcn = nbcn ? dalloc<double2>(lv, nbcn) : nullptr;
    if (nbcn && !L.bcn) return EC2D_ERR_NOMEM;
  }
  L.npart = dalloc<double>(lv, lv.ctiles.size() * 12);
  L.norms = dalloc<double>(lv, ncase * 12);
  L.status = dalloc<int>(lv, ncase * 4);
  L.silent_band_edge = ctx->silent_band_edge ? 1 : 0;
  if (!L.U || !L.q || !L.amu || !L.amut || !L.res || !L.lc || !L.du || !L.geo || !L.un || !L.deltu || !L.qf ||
      !L.fi || !L.fj || !L.npart || !L.norms || !L.status)
    return EC2D_ERR_NOMEM;
  lv.d_case_tile0 = dalloc<int>(lv, ncase);
  lv.d_case_ntile = dalloc<int>(lv, ncase);
  lv.d_case_ncell = dalloc<int>(lv, ncase);
  CK(cudaMemcpy(lv.d_case_tile0, lv.case_tile0.data(), ncase * sizeof(int), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(lv.d_case_ntile, lv.case_ntile.data(), ncase * sizeof(int), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(lv.d_case_ncell, lv.case_ncell.data(), ncase * sizeof(int), cudaMemcpyHostToDevice));
  L.case_tile0 = lv.d_case_tile0; L.case_ntile = lv.d_case_ntile; L.case_ncell = lv.d_case_ncell;
  L.nctr = dalloc<unsigned>(lv, 1);  // zeroed; the last CTA of k_res resets it
  if (!L.nctr) return EC2D_ERR_NOMEM;
  {
    // 2-D cell tiles of the one-kernel residual, block after block (a case's
    // tiles are contiguous, so its norm partials are too)
    std::vector<int4> rt;
    std::vector<int> rc0(ncase, 0), rcn(ncase, 0);
    for (int k = 0; k < (int)lv.hb.size(); k++) {
      const auto &B = lv.hb[k];
      if (rcn[B.cas] == 0) rc0[B.cas] = (int)rt.size();
      for (int j0 = 1; j0 <= B.ny - 1; j0 += RES_TILE_Y)
        for (int i0 = 1; i0 <= B.nx - 1; i0 += RES_TILE_X) { rt.push_back(make_int4(k, i0, j0, 0)); rcn[B.cas]++; }
    }
    lv.n_rtiles = (int)rt.size();
    lv.d_rtiles = dalloc<int4>(lv, rt.size());
    lv.d_rcase_tile0 = dalloc<int>(lv, ncase);
    lv.d_rcase_ntile = dalloc<int>(lv, ncase);
    lv.d_rnpart = dalloc<double>(lv, rt.size() * 12);
    lv.d_rnctr = dalloc<unsigned>(lv, 1);
    if (!lv.d_rtiles || !lv.d_rcase_tile0 || !lv.d_rcase_ntile || !lv.d_rnpart || !lv.d_rnctr) return EC2D_ERR_NOMEM;
    CK(cudaMemcpy(lv.d_rtiles, rt.data(), rt.size() * sizeof(int4), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(lv.d_rcase_tile0, rc0.data(), ncase * sizeof(int), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(lv.d_rcase_ntile, rcn.data(), ncase * sizeof(int), cudaMemcpyHostToDevice));
  }
  if (!lv.wall_faces.empty()) {
    lv.d_faces = dalloc<int4>(lv, lv.wall_faces.size());
    lv.d_face_out = dalloc<double>(lv, lv.wall_faces.size() * 5);
    CK(cudaMemcpy(lv.d_faces, lv.wall_faces.data(), lv.wall_faces.size() * sizeof(int4), cudaMemcpyHostToDevice));
  }
  // geometry planes and initial values
  {
    // the fine mesh's nodes (the rest of the geometry is formed on the
    // device below), the wall distance plane at 1 until comput_dw fills it
    std::vector<double> g((size_t)NG * F, 0.0);
    std::vector<double> u((size_t)nv * F, 0.0), un((size_t)nv * F, 0.0);
    for (int k = 0; k < (int)lv.hb.size(); k++) {
      auto &B = lv.hb[k];
      long long o = lv.blk[k].off;
      size_t n = (size_t)(B.nx + 5) * (B.ny + 5);
      if (l == 1) {
        std::copy(B.x.v.begin(), B.x.v.end(), g.begin() + (size_t)G_X * F + o);
        std::copy(B.y.v.begin(), B.y.v.end(), g.begin() + (size_t)G_Y * F + o);
      }
      for (size_t t = 0; t < n; t++) g[(size_t)G_DW * F + o + t] = 1.0;
      // B%U(1)=1, U(2)=U(3)=0, U(4)=1 (+ turbulence) ; Un(4)=0 fine, 1 coarse (sub_init.f90:161-174, 311-312)
      for (size_t t = 0; t < n; t++) {
        u[0 * F + o + t] = 1.0; u[3 * F + o + t] = 1.0;
        un[0 * F + o + t] = 1.0; un[3 * F + o + t] = (l == 1) ? 0.0 : 1.0;
        if (l == 1 && nv == 5) u[4 * F + o + t] = 1.0 / ctx->cases[B.cas].p.Re;
        if (l == 1 && nv == 6) { u[4 * F + o + t] = 0.0; u[5 * F + o + t] = 1.0; }
      }
    }
    CK(cudaMemcpy(L.geo, g.data(), g.size() * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(L.U, u.data(), u.size() * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(L.un, un.data(), un.size() * sizeof(double), cudaMemcpyHostToDevice));
  }
  // coarse nodes, areas, faces, ghost nodes, cell centres, FDM metrics
  launch_setup_geometry(L, l > 1 ? &ctx->lv[l - 1].L : nullptr, anyfdm, ctx->stream);
  CK(cudaGetLastError());
  launch_face_metrics(L, ctx->stream);
  CK(cudaGetLastError());
  if (L.bcn) {
    launch_bc_normals(L, lv.bc_max_nodes, ctx->stream);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(ctx->stream));
  }
  return EC2D_OK;
}

int wall_distance(ec2d_ctx *ctx) {
  Level &lv = ctx->lv[1];
  for (int c = 0; c < (int)ctx->cases.size(); c++) {
    std::vector<double> wxy;
    for (auto &B : lv.hb) {
      if (B.cas != c) continue;
      for (int s = 0; s < B.nsub; s++) {
        const int *cc = &B.bc[9 * s];
        if (cc[6] != BC_Wall) continue;
        for (int j = cc[4]; j <= cc[5]; j++)
          for (int i = cc[2]; i <= cc[3]; i++) { wxy.push_back(B.x(i, j)); wxy.push_back(B.y(i, j)); }
      }
    }
    double *dw = nullptr;
    if (!wxy.empty()) {
      CK(cudaMalloc(&dw, wxy.size() * sizeof(double)));
      CK(cudaMemcpy(dw, wxy.data(), wxy.size() * sizeof(double), cudaMemcpyHostToDevice));
    }
    for (int k = 0; k < (int)lv.hb.size(); k++) {
      auto &B = lv.hb[k];
      if (B.cas != c) continue;
      const HBlock &hb = ctx->cases[c].blocks[B.blk];
      if (!hb.dw.empty()) {
        Frame f; f.init(B.nx, B.ny, 1.0);
        for (int j = 1; j <= B.ny - 1; j++)
          for (int i = 1; i <= B.nx - 1; i++) f(i, j) = hb.dw[(i - 1) + (size_t)(B.nx - 1) * (j - 1)];
        CK(cudaMemcpy(lv.L.geo + (size_t)G_DW * lv.F + lv.blk[k].off, f.v.data(), f.v.size() * sizeof(double),
                      cudaMemcpyHostToDevice));
      } else if (dw) {
        launch_wall_distance(lv.L, k, dw, (int)wxy.size() / 2, B.nx, B.ny, ctx->stream);
      }
    }
    CK(cudaStreamSynchronize(ctx->stream));
    if (dw) cudaFree(dw);
  }
  return EC2D_OK;
}

// ---------------- orchestration -------------------------------------------
cudaEvent_t pool_event(ec2d_ctx *ctx) {
  if (!ctx->evpool.empty()) { cudaEvent_t e = ctx->evpool.back(); ctx->evpool.pop_back(); return e; }
  cudaEvent_t e;
  cudaEventCreate(&e);
  return e;
}
// every kernel launch of the time-marching path goes through K(): it counts
// the launches (nk kernels per call) and, when timing is on, brackets them
// with events on the context's stream
template <class Fn>
void K(ec2d_ctx *ctx, const char *name, int level, int nk, Fn fn) {
  ctx->launches += nk;
  if (!ctx->timing) { fn(); return; }
  cudaEvent_t a = pool_event(ctx), b = pool_event(ctx);
  cudaEventRecord(a, ctx->stream);
  fn();
  cudaEventRecord(b, ctx->stream);
  ctx->krec.push_back({name, level, nk, a, b});
}

// Comput_Residual_one_mesh (sub_Residual.f90:13-107) for all blocks of a level
// post: RES_ADD_FORCE / RES_FORCE_FN / RES_SET_UN steps that follow the
// residual in the caller's sequence, done inside k_res when the norms are
// final there, as separate kernels otherwise
// the coarse levels of a turbulent multigrid run keep the eddy viscosity
// restricted from the finer level instead of zero
static void apply_mg_amut(ec2d_ctx *ctx) {
  const bool on = ctx->mg_amut && ctx->P.If_viscous == 1 && ctx->P.Iflag_turbulence_model != Turb_NONE;
  for (int l = 2; l <= ctx->num_mesh; l++) ctx->lv[l].L.keep_amut = on ? 1 : 0;
}
// the stream that issues the next write of level l's Res waits for the norms
// of its previous evaluation
void join_norms(ec2d_ctx *ctx, int l) {
  if (!ctx->norm_open[l]) return;
  cudaStreamWaitEvent(ctx->stream, ctx->ev_norm[l], 0);
  ctx->norm_open[l] = false;
}
void residual(ec2d_ctx *ctx, int l, int post = 0) {
  Level &lv = ctx->lv[l];
  const Lvl &L = lv.L;
  join_norms(ctx, l);
  cudaStream_t s = ctx->stream;
  const bool dual = ctx->P.Time_Method == Time_Dual && l == 1;
  const bool f32 = ctx->coarse_fp32 && l >= 2;
  if (ctx->tile_residual && lv.n_rtiles > 0 && L.turb == Turb_NONE && !L.fdm && !L.keep_amut && !dual && !f32) {
    // the whole residual in one kernel over 2-D tiles (norm partials inside;
    // with few cases the per-case norms and the multigrid post-steps too)
    Lvl Lr = L;
    Lr.npart = lv.d_rnpart;
    Lr.case_tile0 = lv.d_rcase_tile0;
    Lr.case_ntile = lv.d_rcase_ntile;
    Lr.nctr = lv.d_rnctr;
    const int inpass = norms_fused_final(L) ? post : 0;
    K(ctx, "k_residual_tile", l, 1, [&] { launch_residual_tile(Lr, lv.d_rtiles, lv.n_rtiles, true, inpass, s); });
    if (!norms_fused_final(L)) K(ctx, "norms", l, 1, [&] { launch_norms(Lr, false, s); });
    const int rest = post & ~inpass;
    if (rest & RES_ADD_FORCE) K(ctx, "k_add_force", l, 1, [&] { launch_add_force(L, s); });
    if (rest & RES_FORCE_FN) K(ctx, "k_force_fn", l, 1, [&] { launch_force_fn(L, s); });
    if (rest & RES_SET_UN) K(ctx, "k_set_un", l, 1, [&] { launch_set_un(L, 4, s); });
    return;
  }
  K(ctx, "k_prim", l, 1, [&] { launch_prim(L, s); });
  if (L.visc) {
    if (L.turb == Turb_SA) K(ctx, "sa", l, 4, [&] { launch_sa(L, s); });
    else if (L.turb == Turb_SST) K(ctx, "sst", l, 4, [&] { launch_sst(L, s); });
    else if (L.turb == Turb_BL) K(ctx, "bl", l, 2, [&] { launch_bl(L, s); });
  }
  // the i- and j-face kernels read the same primitives and write separate
  // planes: they run concurrently on two streams (graph branches); with
  // kernel timing on they run one after the other
  // face fluxes of a coarse level in FP32 when selected (the coarse levels
  // only smooth the fine-level correction)
  if (!ctx->timing && ctx->concurrent) {
    ctx->launches += 2;
    cudaEventRecord(ctx->ev_fork, s);
    cudaStreamWaitEvent(ctx->side, ctx->ev_fork, 0);
    launch_flux_j(L, f32, ctx->side);
    launch_flux_i(L, f32, s);
    cudaEventRecord(ctx->ev_join, ctx->side);
    cudaStreamWaitEvent(s, ctx->ev_join, 0);
  } else {
    K(ctx, "k_flux_i", l, 1, [&] { launch_flux_i(L, f32, s); });
    K(ctx, "k_flux_j", l, 1, [&] { launch_flux_j(L, f32, s); });
  }
  const bool fused = !L.fdm && !dual;  // Res final after k_res: norm partials fused into it
  // Within a step the norms of an evaluation whose Res stays as k_res
  // leaves it (no forcing added) go to the norms branch: the kernels that
  // follow only read Res, and the norms are read after the step.  k_res without
  // them is about half as long (7 against 14 us per launch on the flat
  // plate's levels); the partials and the reduction are the same kernels
  // as for the FDM patch, so the norms are bit-identical either way.
  if (fused && ctx->norm_branch && ctx->concurrent && !ctx->timing && !(post & RES_ADD_FORCE) &&
      norms_fused_final(L)) {
    K(ctx, "k_res", l, 1, [&] { launch_res(L, false, post, s); });
    ctx->launches += 2;
    cudaEventRecord(ctx->ev_nfork[l], s);
    cudaStreamWaitEvent(ctx->nstream, ctx->ev_nfork[l], 0);
    launch_norms(L, true, ctx->nstream);
    cudaEventRecord(ctx->ev_norm[l], ctx->nstream);
    ctx->norm_open[l] = true;
    return;
  }
  const int inpass = (fused && norms_fused_final(L)) ? post : 0;
  K(ctx, "k_res", l, 1, [&] { launch_res(L, fused, inpass, s); });
  if (L.fdm) K(ctx, "fdm", l, 3, [&] { launch_fdm(L, s); });
  if (dual) {
    double sfac;
    if (ctx->dual_iflag1 == 0) { ctx->dual_iflag1 = 1; sfac = 1.0 / (3.0 * ctx->P.dt_global); }
    else sfac = 1.0 / (2.0 * ctx->P.dt_global);
    K(ctx, "k_dual", l, 1, [&] { launch_dual_term(L, sfac, s); });
  }
  if (!(fused && norms_fused_final(L)))
    K(ctx, "norms", l, fused ? 1 : 2, [&] { launch_norms(L, !fused, s); });
  const int rest = post & ~inpass;
  if (rest & RES_ADD_FORCE) K(ctx, "k_add_force", l, 1, [&] { launch_add_force(L, s); });
  if (rest & RES_FORCE_FN) K(ctx, "k_force_fn", l, 1, [&] { launch_force_fn(L, s); });
  if (rest & RES_SET_UN) K(ctx, "k_set_un", l, 1, [&] { launch_set_un(L, 4, s); });
}

void bc_all(ec2d_ctx *ctx, int l) {
  K(ctx, "k_bc", l, 1, [&] { launch_bc(ctx->lv[l].L, 1 | 2 | 4, ctx->stream); });
}

void advance_counters(ec2d_ctx *ctx, int l) {
  for (auto &c : ctx->cases) { c.tt[l] += c.p.dt_global; c.kstep[l] += 1; }
}

// NS_Time_advance_1Euler (sub_NS_singlegrid.f90:67-106).  fresh: U has not
// changed since the last residual evaluation of this level (the first
// smoothing step after transfer_down), so Res, the spectral radii, dt and the
// norms of that evaluation stand; the reference evaluates them again with the
// same result.
void step_euler(ec2d_ctx *ctx, int l, bool fresh = false) {
  if (!fresh) residual(ctx, l);
  K(ctx, "k_euler", l, 1, [&] { launch_euler(ctx->lv[l].L, l != 1, ctx->stream); });
  bc_all(ctx, l);
  advance_counters(ctx, l);
}
// NS_Time_advance_RK3 (sub_NS_singlegrid.f90:115-176)
void step_rk3(ec2d_ctx *ctx, int l) {
  const Lvl &L = ctx->lv[l].L;
  K(ctx, "k_set_un", l, 1, [&] { launch_set_un(L, L.nvar, ctx->stream); });
  for (int k = 0; k < 3; k++) {
    residual(ctx, l);
    K(ctx, "k_rk3", l, 1, [&] { launch_rk3(L, k, l != 1, ctx->stream); });
    bc_all(ctx, l);
  }
  advance_counters(ctx, l);
}
// du_LU_SGS_2D for every block of the level followed by U += dU
// (sub_NS_singlegrid.f90:196-213): the wavefront kernels fuse the update into
// the backward sweep; blocks wider than 1024 rows take the generic kernel
// force: Res + QF stands for Res (forcing of a coarse level whose residual
// evaluated on entry is reused); the wavefront record builders add it
void lusgs_update(ec2d_ctx *ctx, int l, double alfa1, bool force = false) {
  const Level &lv = ctx->lv[l];
  const Lvl &L = lv.L;
  const int mode = LUSGS_UPDATE | (force ? LUSGS_FORCE : 0);
  if (ctx->lusgs_fp32 && lv.fast32) {
    K(ctx, "k_lusgs32", l, 3, [&] { launch_lusgs_fast32(L, alfa1, mode, lv.max_rows, ctx->stream); });
  } else if (lv.fast64) {
    auto go = [&](int part) {
      launch_lusgs_fast(L, alfa1, mode | part, lv.max_rows, lv.max_cols, ctx->lusgs_cs, ctx->lusgs_rpw,
                        ctx->lusgs_lanes, ctx->stream);
    };
    if (ctx->timing) {  // the record builder and the sweep timed apart (together: the k_lusgs stage)
      K(ctx, "k_lusgs_prep", l, 1, [&] { go(LUSGS_PREP_ONLY); });
      K(ctx, "k_lusgs_sweep", l, 1, [&] { go(LUSGS_SWEEP_ONLY); });
    } else {
      K(ctx, "k_lusgs", l, 2, [&] { go(0); });
    }
  } else {
    if (force) K(ctx, "k_add_force", l, 1, [&] { launch_add_force(L, ctx->stream); });
    K(ctx, "k_lusgs_generic", l, 1, [&] { launch_lusgs(L, alfa1, ctx->stream); });
    K(ctx, "k_add_du", l, 1, [&] { launch_add_du(L, ctx->stream); });
  }
}
// NS_Time_advance_LU_SGS (sub_NS_singlegrid.f90:185-224); on a coarse level of
// an LU-SGS-smoothed multigrid cycle the forcing is added after the residual
// bc: false leaves the boundary conditions after the update to the caller
// (a multigrid transfer issues them after its fork, see transfer_down)
void step_lusgs(ec2d_ctx *ctx, int l, double alfa1 = 0.0, bool fresh = false, bool bc = true) {
  if (!fresh) residual(ctx, l, l != 1 ? RES_ADD_FORCE : 0);
  lusgs_update(ctx, l, alfa1, fresh && l != 1);
  if (bc) bc_all(ctx, l);
  advance_counters(ctx, l);
}
void clip(ec2d_ctx *ctx, int l) {
  if (ctx->lv[l].L.nvar >= 5) K(ctx, "k_clip", l, 1, [&] { launch_bc(ctx->lv[l].L, 8, ctx->stream); });
}
// Dual_time_LU_SGS (sub_NS_singlegrid.f90:231-310).  The inner-loop exit test
// on the RMS residual needs the norms on the host after every inner step.
int step_dual(ec2d_ctx *ctx) {
  double alfa1;
  if (ctx->dual_iflag == 0) { ctx->dual_iflag = 1; alfa1 = 1.0 / ctx->P.dt_global; }
  else alfa1 = 3.0 / (2.0 * ctx->P.dt_global);
  Level &lv = ctx->lv[1];
  const Lvl &L = lv.L;
  for (int kt = 1; kt <= ctx->P.Nstep_Inner_Limit; kt++) {
    residual(ctx, 1);
    lusgs_update(ctx, 1, alfa1);
    bc_all(ctx, 1);
    std::vector<double> nm(12 * L.ncase);
    CK(cudaMemcpyAsync(nm.data(), L.norms, nm.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    bool all_done = true;
    for (int c = 0; c < L.ncase; c++) {
      double mx = nm[12 * c + 6];
      for (int m = 0; m < ctx->nvar; m++) mx = std::max(mx, nm[12 * c + 6 + m]);
      if (!(mx <= ctx->P.Res_Inner_Limit)) all_done = false;
    }
    if (all_done) break;
  }
  // U(n-1) <= U(n), U(n) <= U
  cudaStream_t s = ctx->stream;
  size_t bytes = (size_t)L.nvar * lv.F * sizeof(double);
  CK(cudaMemcpyAsync(L.un1, L.un, bytes, cudaMemcpyDeviceToDevice, s));
  CK(cudaMemcpyAsync(L.un, L.U, bytes, cudaMemcpyDeviceToDevice, s));
  advance_counters(ctx, 1);
  return EC2D_OK;
}
int time_advance(ec2d_ctx *ctx, int l) {
  int tm = ctx->P.Time_Method;
  if (tm == Time_Euler1) step_euler(ctx, l);
  else if (tm == Time_RK3) step_rk3(ctx, l);
  else if (tm == Time_LU_SGS) step_lusgs(ctx, l);
  else if (tm == Time_Dual) { int r = step_dual(ctx); if (r) return r; }
  clip(ctx, l);
  return EC2D_OK;
}
// Returns the work it left to the transfer that follows: SMOOTH_BC, the
// level's boundary conditions after the LU-SGS update, and SMOOTH_CLIP, the
// turbulence clip after them (force_vt_kw)
enum { SMOOTH_BC = 1, SMOOTH_CLIP = 2 };
int mg_smooth_fine(ec2d_ctx *ctx) {
  int tm = ctx->P.Time_Method;
  if (tm == Time_Euler1) step_euler(ctx, 1);
  else if (tm == Time_LU_SGS) {
    step_lusgs(ctx, 1, 0.0, false, false);
    return SMOOTH_BC | SMOOTH_CLIP;
  } else step_rk3(ctx, 1);
  return 0;
}
// Un = U of the coarse level (Euler and LU-SGS smoothing) is taken by the
// residual evaluation just before (RES_SET_UN, see transfer_down), and the
// first smoothing step reuses that evaluation (U is unchanged since)
// defer_bc: a transfer follows and issues the boundary conditions (the
// return value as for mg_smooth_fine)
int mg_smooth_coarse(ec2d_ctx *ctx, int l, bool defer_bc = false) {
  const int Time_step_coarse_mesh = 3;
  int tm = ctx->P.Time_Method;
  if (tm == Time_Euler1) {
    for (int m = 0; m < Time_step_coarse_mesh; m++) step_euler(ctx, l, m == 0);
  } else if (tm == Time_LU_SGS) {
    step_lusgs(ctx, l, 0.0, true, !defer_bc);
    return defer_bc ? SMOOTH_BC : 0;
  } else step_rk3(ctx, l);
  return 0;
}
// the work issued while it is in effect goes to the second stream pair
void swap_branch(ec2d_ctx *ctx) {
  std::swap(ctx->stream, ctx->stream2);
  std::swap(ctx->side, ctx->side2);
  std::swap(ctx->ev_fork, ctx->ev_fork2);
  std::swap(ctx->ev_join, ctx->ev_join2);
}
// Transfer from level f to f + 1 (interpolation2h and comput_force_function,
// sub_NS_multigrid.f90:349-398,156-173): the residual of level f, the
// restriction of U with the coarse boundary conditions, and the coarse
// residual on entry (with Un = U for the smoothing that follows).  The
// residual of level f reads and writes level-f arrays only; the other chain
// reads level-f U and writes level-(f + 1) arrays only, so with concurrent
// kernels it runs on the second stream pair beside the first (graph
// branches); the forcing QF = sum Res_h - R_2h(U_2h) is formed where the two
// join, with the same two roundings as the reference's sum then subtract.
// pending: the smoother's boundary conditions (and clip) of level f, issued
// here on the first chain, after the fork: the restriction of U reads the
// interior mean-flow variables only, which neither of them writes.
void transfer_down(ec2d_ctx *ctx, int f, int fine_post, int pending = 0) {
  const int tm = ctx->P.Time_Method;
  const int cpost = (tm == Time_Euler1 || tm == Time_LU_SGS) ? RES_SET_UN : 0;
  const Lvl &Lf = ctx->lv[f].L, &Lc = ctx->lv[f + 1].L;
  auto finish_smoothing = [&] {
    if (pending & SMOOTH_BC) bc_all(ctx, f);
    if (pending & SMOOTH_CLIP) clip(ctx, f);
  };
  if (Lc.keep_amut) {
    // the coarse eddy viscosity comes from the finer level's after its
    // residual (the oracle's order: residual, then interpolation2h), so
    // this transfer runs in sequence
    finish_smoothing();
    residual(ctx, f, fine_post);
    K(ctx, "k_restrict", f + 1, 1, [&] { launch_restrict(Lf, Lc, 1 | 8, ctx->stream); });
    bc_all(ctx, f + 1);
    residual(ctx, f + 1, cpost);
    K(ctx, "k_restrict", f + 1, 1, [&] { launch_restrict(Lf, Lc, 2 | 4, ctx->stream); });
    return;
  }
  const bool par = !ctx->timing && ctx->concurrent;
  if (par) {
    cudaEventRecord(ctx->ev_b0, ctx->stream);
    cudaStreamWaitEvent(ctx->stream2, ctx->ev_b0, 0);
    swap_branch(ctx);
  } else {
    finish_smoothing();
  }
  K(ctx, "k_restrict", f + 1, 1, [&] { launch_restrict(Lf, Lc, 1, ctx->stream); });
  bc_all(ctx, f + 1);
  residual(ctx, f + 1, cpost);
  if (par) {
    swap_branch(ctx);
    cudaEventRecord(ctx->ev_b1, ctx->stream2);
    finish_smoothing();
  }
  residual(ctx, f, fine_post);
  if (par) cudaStreamWaitEvent(ctx->stream, ctx->ev_b1, 0);
  K(ctx, "k_restrict", f + 1, 1, [&] { launch_restrict(Lf, Lc, 2 | 4, ctx->stream); });
}
// deltU = U - Un on level c, prolonged to level c-1 and added there (one
// kernel: the coarse deltU is formed where it is interpolated)
void correct_from(ec2d_ctx *ctx, int c) {
  const Lvl &Lc = ctx->lv[c].L, &Lf = ctx->lv[c - 1].L;
  K(ctx, "k_prolong", c - 1, 1, [&] { launch_prolong(Lc, Lf, 3, ctx->stream); });
}
// NS_2stge_multigrid (sub_NS_multigrid.f90:14-58)
void mg2(ec2d_ctx *ctx) {
  const int pend = mg_smooth_fine(ctx);
  transfer_down(ctx, 1, 0, pend);
  mg_smooth_coarse(ctx, 2);
  correct_from(ctx, 2);
  bc_all(ctx, 1);
}
// NS_3stge_multigrid (sub_NS_multigrid.f90:66-142)
void mg3(ec2d_ctx *ctx) {
  const int pend1 = mg_smooth_fine(ctx);
  transfer_down(ctx, 1, 0, pend1);
  const int pend2 = mg_smooth_coarse(ctx, 2, true);
  transfer_down(ctx, 2, RES_ADD_FORCE, pend2);
  mg_smooth_coarse(ctx, 3);
  correct_from(ctx, 3);
  correct_from(ctx, 2);
  bc_all(ctx, 1);
}

int one_step(ec2d_ctx *ctx) {
  if (ctx->num_mesh == 1) {
    // dual time stepping reads the norms on the host inside the step
    ctx->norm_branch = ctx->P.Time_Method != Time_Dual;
    const int r = time_advance(ctx, 1);
    ctx->norm_branch = false;
    join_norms(ctx, 1);
    return r;
  }
  ctx->norm_branch = true;
  if (ctx->num_mesh == 2) mg2(ctx);
  else mg3(ctx);
  ctx->norm_branch = false;
  for (int l = 1; l <= 3; l++) join_norms(ctx, l);
  return EC2D_OK;
}

// Records one step into ctx->step_graph.  The orchestration runs once on the
// host with the stream in capture mode, so its host-side effects (launch count,
// step counters) are measured, undone, and re-applied on every replay.  If the
// capture fails the context keeps launching kernels one by one.
int capture_step(ec2d_ctx *ctx) {
  std::vector<std::array<int, 4>> ks(ctx->cases.size());
  std::vector<std::array<double, 4>> ts(ctx->cases.size());
  for (size_t c = 0; c < ctx->cases.size(); c++)
    for (int l = 0; l < 4; l++) { ks[c][l] = ctx->cases[c].kstep[l]; ts[c][l] = ctx->cases[c].tt[l]; }
  long long n0 = ctx->launches;
  CK(cudaGetLastError());
  CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  int r = one_step(ctx);
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
  if (r == EC2D_OK && e == cudaSuccess && g) e = cudaGraphInstantiate(&ctx->step_graph, g, 0);
  if (g) cudaGraphDestroy(g);
  ctx->graph_launches = ctx->launches - n0;
  ctx->launches = n0;
  for (int l = 1; l <= 3; l++) ctx->graph_adv[l] = ctx->cases.empty() ? 0 : ctx->cases[0].kstep[l] - ks[0][l];
  for (size_t c = 0; c < ctx->cases.size(); c++)
    for (int l = 0; l < 4; l++) { ctx->cases[c].kstep[l] = ks[c][l]; ctx->cases[c].tt[l] = ts[c][l]; }
  if (r != EC2D_OK) return r;
  if (e != cudaSuccess || !ctx->step_graph) {
    fprintf(stderr, "ec2d: step capture failed (%s); launching kernels directly\n", cudaGetErrorString(e));
    cudaGetLastError();
    ctx->step_graph = nullptr;
    ctx->use_graphs = false;
  }
  return EC2D_OK;
}

bool valid_case(ec2d_ctx *ctx, int c) { return ctx && c >= 1 && c <= (int)ctx->cases.size(); }

// Fortran extents of the fields of ec2d_get_field
struct FieldShape { int nv, i0, i1, j0, j1, plane_base; double *base; };
bool field_shape(ec2d_ctx *ctx, int l, int field, const BlkDev &b, FieldShape &fs) {
  const Lvl &L = ctx->lv[l].L;
  int nx = b.nx, ny = b.ny;
  fs.plane_base = 0;
  switch (field) {
    case EC2D_F_RES: fs = {L.nvar, 1, nx - 1, 1, ny - 1, 0, L.res}; return true;
    case EC2D_F_DT: fs = {1, 1, nx - 1, 1, ny - 1, 0, L.lc + (size_t)L_DT * L.F}; return true;
    case EC2D_F_LCI: fs = {1, 1, nx, 1, ny, 0, L.lc + (size_t)L_CI * L.F}; return true;
    case EC2D_F_LCJ: fs = {1, 1, nx, 1, ny, 0, L.lc + (size_t)L_CJ * L.F}; return true;
    case EC2D_F_LVI: fs = {1, 1, nx, 1, ny, 0, L.lc + (size_t)L_VI * L.F}; return true;
    case EC2D_F_LVJ: fs = {1, 1, nx, 1, ny, 0, L.lc + (size_t)L_VJ * L.F}; return true;
    case EC2D_F_DU: fs = {L.nvar, 1, nx, 1, ny, 0, L.du}; return true;
    case EC2D_F_AMU: fs = {1, -1, nx + 1, -1, ny + 1, 0, L.amu}; return true;
    case EC2D_F_AMUT: fs = {1, -1, nx + 1, -1, ny + 1, 0, L.amut}; return true;
    case EC2D_F_X1: fs = {1, -1, nx + 1, -1, ny + 1, 0, L.geo + (size_t)G_X1 * L.F}; return true;
    case EC2D_F_Y1: fs = {1, -1, nx + 1, -1, ny + 1, 0, L.geo + (size_t)G_Y1 * L.F}; return true;
    case EC2D_F_VOL: fs = {1, 1, nx, 1, ny, 0, L.geo + (size_t)G_VOL * L.F}; return true;
    case EC2D_F_SI: fs = {1, 1, nx, 1, ny, 0, L.geo + (size_t)G_SI * L.F}; return true;
    case EC2D_F_SJ: fs = {1, 1, nx, 1, ny, 0, L.geo + (size_t)G_SJ * L.F}; return true;
    case EC2D_F_NI1: fs = {1, 1, nx, 1, ny, 0, L.geo + (size_t)G_NI1 * L.F}; return true;
    case EC2D_F_NI2: fs = {1, 1, nx, 1, ny, 0, L.geo + (size_t)G_NI2 * L.F}; return true;
    case EC2D_F_NJ1: fs = {1, 1, nx, 1, ny, 0, L.geo + (size_t)G_NJ1 * L.F}; return true;
    case EC2D_F_NJ2: fs = {1, 1, nx, 1, ny, 0, L.geo + (size_t)G_NJ2 * L.F}; return true;
    case EC2D_F_DW: fs = {1, 0, nx, 0, ny, 0, L.geo + (size_t)G_DW * L.F}; return true;
    case EC2D_F_QF: fs = {4, 1, nx - 1, 1, ny - 1, 0, L.qf}; return true;
    case EC2D_F_DELTU: fs = {4, -1, nx + 1, -1, ny + 1, 0, L.deltu}; return true;
    case EC2D_F_UN: fs = {L.nvar, 0, nx, 0, ny, 0, L.un}; return true;
    case EC2D_F_X: fs = {1, -1, nx + 2, -1, ny + 2, 0, L.geo + (size_t)G_X * L.F}; return true;
    case EC2D_F_Y: fs = {1, -1, nx + 2, -1, ny + 2, 0, L.geo + (size_t)G_Y * L.F}; return true;
  }
  return false;
}

int find_block(ec2d_ctx *ctx, int case_id, int mesh, int block) {
  if (!ctx->setup_done || !valid_case(ctx, case_id) || mesh < 1 || mesh > ctx->num_mesh) return -1;
  Level &lv = ctx->lv[mesh];
  for (int k = 0; k < (int)lv.hb.size(); k++)
    if (lv.hb[k].cas == case_id - 1 && lv.hb[k].blk == block - 1) return k;
  return -1;
}

int check_launch(ec2d_ctx *ctx) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    fprintf(stderr, "ec2d: launch error %s\n", cudaGetErrorString(e));
    return EC2D_ERR_CUDA;
  }
  return EC2D_OK;
}

// the error a case's device status code stands for: 3 the T < 1e-5 stop of
// the primitives, 4 a wavefront wait that gave up
int status_error(int code) {
  return code == 0 ? EC2D_OK : code == EC2D_ERR_TIMEOUT ? EC2D_ERR_TIMEOUT : EC2D_ERR_STATE;
}

}  // namespace

// =============================== C-ABI =====================================
extern "C" {

int ec2d_version(void) { return 10000; }

const char *ec2d_error_string(int code) {
  switch (code) {
    case EC2D_OK: return "ok";
    case EC2D_ERR_ARG: return "invalid argument or call order";
    case EC2D_ERR_CUDA: return "CUDA error";
    case EC2D_ERR_STATE: return "non-physical state (T < 1e-5)";
    case EC2D_ERR_TIMEOUT: return "device wait timed out";
    case EC2D_ERR_UNSUPPORTED: return "option combination not supported";
    case EC2D_ERR_NOMEM: return "out of device memory";
  }
  return "unknown error";
}

int ec2d_create(int device, ec2d_ctx **out) {
  if (!out) return EC2D_ERR_ARG;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) return EC2D_ERR_CUDA;
  CK(cudaSetDevice(device));
  ec2d_ctx *c = new ec2d_ctx();
  c->device = device;
  if (const char *e = getenv("EC2D_LUSGS_CLUSTER")) c->lusgs_cs = std::max(0, std::min(8, atoi(e)));
  if (const char *e = getenv("EC2D_LUSGS_ROWS")) c->lusgs_rpw = std::max(4, std::min(32, atoi(e)));
  if (const char *e = getenv("EC2D_LUSGS_LANES")) {
    const int v = atoi(e);
    c->lusgs_lanes = (v == 4 || v == 8) ? v : 0;
  }
  if (const char *e = getenv("EC2D_TEST_SILENT_BAND_EDGE")) c->silent_band_edge = atoi(e) != 0;
  if (const char *e = getenv("EC2D_CONCURRENT")) c->concurrent = atoi(e) != 0;
  if (const char *e = getenv("EC2D_TILE_RESIDUAL")) c->tile_residual = atoi(e) != 0;
  if (const char *e = getenv("EC2D_MG_EDDY_VISCOSITY")) c->mg_amut = atoi(e) != 0;
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->stream2, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->side2, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->ev_fork2, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->ev_join2, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->ev_b0, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->ev_b1, cudaEventDisableTiming) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->nstream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return EC2D_ERR_CUDA;
  }
  for (int l = 0; l < 4; l++)
    if (cudaEventCreateWithFlags(&c->ev_nfork[l], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_norm[l], cudaEventDisableTiming) != cudaSuccess) {
      delete c;
      return EC2D_ERR_CUDA;
    }
  *out = c;
  return EC2D_OK;
}

void ec2d_destroy(ec2d_ctx *ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  if (ctx->snap_stream) {
    cudaStreamSynchronize(ctx->snap_stream);
    cudaStreamDestroy(ctx->snap_stream);
    cudaEventDestroy(ctx->ev_snap);
    cudaEventDestroy(ctx->ev_snap_done);
  }
  if (ctx->d_snap) cudaFree(ctx->d_snap);
  if (ctx->h_snap) cudaFreeHost(ctx->h_snap);
  for (auto &lv : ctx->lv) lv.bufs.clear();
  for (auto &r : ctx->krec) { cudaEventDestroy(r.a); cudaEventDestroy(r.b); }
  for (auto e : ctx->evpool) cudaEventDestroy(e);
  if (ctx->d_cases) cudaFree(ctx->d_cases);
  if (ctx->d_stage) cudaFree(ctx->d_stage);
  if (ctx->d_shape) cudaFree(ctx->d_shape);
  if (ctx->step_graph) cudaGraphExecDestroy(ctx->step_graph);
  cudaStreamSynchronize(ctx->side);
  cudaStreamSynchronize(ctx->stream2);
  cudaStreamSynchronize(ctx->side2);
  cudaStreamSynchronize(ctx->nstream);
  for (int l = 0; l < 4; l++) { cudaEventDestroy(ctx->ev_nfork[l]); cudaEventDestroy(ctx->ev_norm[l]); }
  cudaStreamDestroy(ctx->nstream);
  cudaEventDestroy(ctx->ev_fork);
  cudaEventDestroy(ctx->ev_join);
  for (cudaEvent_t e : {ctx->ev_fork2, ctx->ev_join2, ctx->ev_b0, ctx->ev_b1}) cudaEventDestroy(e);
  cudaStreamDestroy(ctx->side2);
  cudaStreamDestroy(ctx->stream2);
  cudaStreamDestroy(ctx->side);
  cudaStreamDestroy(ctx->stream);
  delete ctx;
}

int ec2d_add_case(ec2d_ctx *ctx, const ec2d_params *p, int *case_id) {
  if (!ctx || !p || ctx->setup_done) return EC2D_ERR_ARG;
  if (!ctx->cases.empty() && !same_method(ctx->cases[0].p, *p)) return EC2D_ERR_ARG;
  HCase c;
  c.p = *p;
  c.nvar = (p->Iflag_turbulence_model == Turb_SST) ? 6 : (p->Iflag_turbulence_model == Turb_SA) ? 5 : 4;
  ctx->cases.push_back(c);
  if (case_id) *case_id = (int)ctx->cases.size();
  return EC2D_OK;
}

int ec2d_add_block(ec2d_ctx *ctx, int case_id, int nx, int ny, const double *x, const double *y, int nsub,
                   const int *bc9) {
  if (!valid_case(ctx, case_id) || ctx->setup_done || nx < 3 || ny < 3 || !x || !y || nsub < 0 || (nsub && !bc9))
    return EC2D_ERR_ARG;
  HBlock b;
  b.nx = nx; b.ny = ny; b.nsub = nsub;
  b.x.assign(x, x + (size_t)nx * ny);
  b.y.assign(y, y + (size_t)nx * ny);
  b.bc.assign(bc9, bc9 + 9 * nsub);
  // every ghost-cell kernel indexes through these ranges: reject anything
  // that is not a proper block face (face 1: i=1, 3: i=nx, 2: j=1, 4: j=ny)
  for (int k = 0; k < nsub; k++) {
    const int *s = &b.bc[9 * k];
    if (s[1] < 1 || s[1] > 4 || s[2] < 1 || s[3] > nx || s[4] < 1 || s[5] > ny || s[2] > s[3] || s[4] > s[5])
      return EC2D_ERR_ARG;
    if ((s[1] == 1 && (s[2] != 1 || s[3] != 1)) || (s[1] == 3 && (s[2] != nx || s[3] != nx)) ||
        (s[1] == 2 && (s[4] != 1 || s[5] != 1)) || (s[1] == 4 && (s[4] != ny || s[5] != ny)))
      return EC2D_ERR_ARG;
    if ((s[1] == 1 || s[1] == 3) ? (s[4] == s[5]) : (s[2] == s[3])) return EC2D_ERR_ARG;
    if (s[6] >= 0 && s[6] < 1) return EC2D_ERR_ARG;
  }
  ctx->cases[case_id - 1].blocks.push_back(std::move(b));
  return EC2D_OK;
}

int ec2d_set_fdm_block(ec2d_ctx *ctx, int case_id, int block) {
  if (!valid_case(ctx, case_id) || ctx->setup_done) return EC2D_ERR_ARG;
  auto &bl = ctx->cases[case_id - 1].blocks;
  if (block < 1 || block > (int)bl.size()) return EC2D_ERR_ARG;  // "error in 'FDM.in'"
  bl[block - 1].fdm = true;
  return EC2D_OK;
}

int ec2d_set_wall_distance(ec2d_ctx *ctx, int case_id, int block, const double *dw) {
  if (!valid_case(ctx, case_id) || ctx->setup_done || !dw) return EC2D_ERR_ARG;
  auto &bl = ctx->cases[case_id - 1].blocks;
  if (block < 1 || block > (int)bl.size()) return EC2D_ERR_ARG;
  HBlock &b = bl[block - 1];
  b.dw.assign(dw, dw + (size_t)(b.nx - 1) * (b.ny - 1));
  return EC2D_OK;
}

int ec2d_setup(ec2d_ctx *ctx) {
  if (!ctx || ctx->setup_done || ctx->cases.empty()) return EC2D_ERR_ARG;
  CK(cudaSetDevice(ctx->device));
  ctx->P = ctx->cases[0].p;
  const ec2d_params &P = ctx->P;
  for (auto &c : ctx->cases) if (c.blocks.empty()) return EC2D_ERR_ARG;
  // opencfd_ec2d_v1.5.4.f90:216-221 (lifted for LU-SGS when mg_lusgs is set)
  if ((P.Time_Method == Time_LU_SGS && P.Num_Mesh != 1 && !P.mg_lusgs) ||
      (P.Time_Method == Time_Dual && P.Num_Mesh != 1))
    return EC2D_ERR_UNSUPPORTED;
  if (P.Iflag_turbulence_model != Turb_NONE && !P.If_viscous) return EC2D_ERR_UNSUPPORTED;
  int nm = 3;
  for (auto &c : ctx->cases) nm = std::min(nm, mg_depth(c));
  ctx->num_mesh = nm;
  ctx->nvar = ctx->cases[0].nvar;
  std::vector<CaseDev> cd;
  for (auto &c : ctx->cases) cd.push_back(make_casedev(c.p));
  CK(cudaMalloc(&ctx->d_shape, ctx->cases.size() * sizeof(double)));
  CK(cudaMemset(ctx->d_shape, 0, ctx->cases.size() * sizeof(double)));
  CK(cudaMalloc(&ctx->d_cases, cd.size() * sizeof(CaseDev)));
  CK(cudaMemcpy(ctx->d_cases, cd.data(), cd.size() * sizeof(CaseDev), cudaMemcpyHostToDevice));
  for (int l = 1; l <= nm; l++) {
    int r = build_level(ctx, l);
    if (r) return r;
  }
  if (P.Iflag_turbulence_model == Turb_SA || P.Iflag_turbulence_model == Turb_SST) {
    int r = wall_distance(ctx);
    if (r) return r;
  }
  size_t mx = 0;
  for (int l = 1; l <= nm; l++)
    for (auto &b : ctx->lv[l].blk) mx = std::max(mx, (size_t)(b.nx + 3) * (b.ny + 3) * 6);
  CK(cudaMalloc(&ctx->d_stage, mx * sizeof(double)));
  ctx->stage_n = mx;
  CK(cudaDeviceSynchronize());
  ctx->setup_done = true;
  apply_mg_amut(ctx);
  return EC2D_OK;
}

int ec2d_num_mesh(ec2d_ctx *ctx, int *num_mesh) {
  if (!ctx || !ctx->setup_done || !num_mesh) return EC2D_ERR_ARG;
  *num_mesh = ctx->num_mesh;
  return EC2D_OK;
}

int ec2d_block_dims(ec2d_ctx *ctx, int case_id, int mesh, int block, int *nx, int *ny, int *nvar) {
  int k = find_block(ctx, case_id, mesh, block);
  if (k < 0) return EC2D_ERR_ARG;
  const BlkDev &b = ctx->lv[mesh].blk[k];
  if (nx) *nx = b.nx;
  if (ny) *ny = b.ny;
  if (nvar) *nvar = ctx->lv[mesh].L.nvar;
  return EC2D_OK;
}

// init_flow_zero (sub_init.f90:423-495)
int ec2d_clear_status(ec2d_ctx *ctx, int case_id) {
  if (!ctx || !ctx->setup_done || (case_id != 0 && !valid_case(ctx, case_id))) return EC2D_ERR_ARG;
  cudaSetDevice(ctx->device);
  const int c0 = case_id ? case_id - 1 : 0, nc = case_id ? 1 : (int)ctx->cases.size();
  for (int l = 1; l <= ctx->num_mesh; l++)
    CK(cudaMemsetAsync(ctx->lv[l].L.status + 4 * c0, 0, (size_t)4 * nc * sizeof(int), ctx->stream));
  return EC2D_OK;
}

// U(n) = U(n-1) = U on the fine mesh and the first-step flags unset: the
// first physical step after it is the one-step form (alfa1 = 1/dt, Sfac =
// 1/(3 dt), sub_NS_singlegrid.f90:239-245, sub_Residual.f90:27-34), whose
// comment assumes U(n-1) = U(n); the reference's code leaves Un at its
// allocation fill (sub_init.f90:162) and Un1 unset
int ec2d_dual_time_start(ec2d_ctx *ctx) {
  if (!ctx || !ctx->setup_done) return EC2D_ERR_ARG;
  if (ctx->P.Time_Method != Time_Dual) return EC2D_OK;
  cudaSetDevice(ctx->device);
  const Lvl &L = ctx->lv[1].L;
  const size_t bytes = (size_t)L.nvar * ctx->lv[1].F * sizeof(double);
  CK(cudaMemcpyAsync(L.un, L.U, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
  CK(cudaMemcpyAsync(L.un1, L.U, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
  ctx->dual_iflag = ctx->dual_iflag1 = 0;
  return EC2D_OK;
}

int ec2d_init_flow(ec2d_ctx *ctx) {
  if (!ctx || !ctx->setup_done) return EC2D_ERR_ARG;
  cudaSetDevice(ctx->device);
  int rc = ec2d_clear_status(ctx, 0);  // a fresh start: no case carries a stop
  if (rc) return rc;
  int nm = ctx->num_mesh;
  // the reference starts (init_flow_zero) right after the meshes are made,
  // with the coarse forcing QF zero (sub_init.f90:315), which the coarse
  // pre-steps below add (sub_NS_singlegrid.f90:77,146), and with the dual-time
  // first-step flags unset and the step counters at zero: a context that has
  // stepped, or been autotuned, starts here exactly as a new one does
  for (int l = 2; l <= nm; l++)
    CK(cudaMemsetAsync(ctx->lv[l].L.qf, 0, (size_t)4 * ctx->lv[l].F * sizeof(double), ctx->stream));
  ctx->dual_iflag = ctx->dual_iflag1 = 0;
  for (auto &c : ctx->cases)
    for (int l = 0; l < 4; l++) { c.kstep[l] = 0; c.tt[l] = 0.0; }
  // coarse eddy viscosity (kept between residuals only with the multigrid
  // eddy-viscosity extension): zero until the first restriction
  for (int l = 2; l <= nm; l++)
    CK(cudaMemsetAsync(ctx->lv[l].L.amut, 0, (size_t)ctx->lv[l].F * sizeof(double), ctx->stream));
  if (ctx->nvar >= 5) launch_freestream(ctx->lv[1].L, 0, 1, ctx->stream);
  launch_freestream(ctx->lv[nm].L, 1, 0, ctx->stream);
  bc_all(ctx, nm);
  for (int l = nm; l >= 1; l--) {
    int pre = ctx->P.Pre_Step_Mesh[l - 1];
    for (int st = 0; st < pre; st++) {
      int r = time_advance(ctx, l);
      if (r) return r;
    }
    if (l > 1) {
      launch_prolong(ctx->lv[l].L, ctx->lv[l - 1].L, 1, ctx->stream);
      bc_all(ctx, l - 1);
    }
  }
  rc = ec2d_dual_time_start(ctx);
  if (rc) return rc;
  return check_launch(ctx);
}

int ec2d_upload_U(ec2d_ctx *ctx, int case_id, int mesh, int block, const double *U) {
  int k = find_block(ctx, case_id, mesh, block);
  if (k < 0 || !U) return EC2D_ERR_ARG;
  cudaSetDevice(ctx->device);
  const Lvl &L = ctx->lv[mesh].L;
  const BlkDev &b = ctx->lv[mesh].blk[k];
  int items = (b.nx + 3) * (b.ny + 3);
  CK(cudaMemcpyAsync(ctx->d_stage, U, (size_t)items * L.nvar * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  launch_pack_u(L, k, L.nvar, ctx->d_stage, items, ctx->stream);
  return check_launch(ctx);
}

int ec2d_download_U(ec2d_ctx *ctx, int case_id, int mesh, int block, double *U) {
  int k = find_block(ctx, case_id, mesh, block);
  if (k < 0 || !U) return EC2D_ERR_ARG;
  cudaSetDevice(ctx->device);
  const Lvl &L = ctx->lv[mesh].L;
  const BlkDev &b = ctx->lv[mesh].blk[k];
  int items = (b.nx + 3) * (b.ny + 3);
  launch_unpack_u(L, k, L.nvar, ctx->d_stage, items, ctx->stream);
  CK(cudaMemcpyAsync(U, ctx->d_stage, (size_t)items * L.nvar * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return EC2D_OK;
}

int ec2d_snapshot(ec2d_ctx *ctx, int case_id) {
  if (!ctx || !ctx->setup_done || !valid_case(ctx, case_id)) return EC2D_ERR_ARG;
  cudaSetDevice(ctx->device);
  if (!ctx->snap_stream) {
    CK(cudaStreamCreateWithFlags(&ctx->snap_stream, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&ctx->ev_snap, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&ctx->ev_snap_done, cudaEventDisableTiming));
  }
  const Level &lv = ctx->lv[1];
  const Lvl &L = lv.L;
  const HCase &hc = ctx->cases[case_id - 1];
  // per block: U in the layout of ec2d_download_U, then the block's mu_t
  // frame ((nx+5) x (ny+5), origin (-2,-2)) for the Amut column of flow2d.dat
  std::vector<size_t> off;
  size_t n = 0;
  for (int b = 1; b <= (int)hc.blocks.size(); b++) {
    int k = find_block(ctx, case_id, 1, b);
    if (k < 0) return EC2D_ERR_ARG;
    off.push_back(n);
    n += (size_t)(lv.blk[k].nx + 3) * (lv.blk[k].ny + 3) * L.nvar;
    n += (size_t)lv.blk[k].P * (lv.blk[k].ny + 5);
  }
  // the previous snapshot's copy reads the device buffer: the main stream
  // waits for it before packing over it (only when snapshots come faster
  // than their copies)
  if (ctx->snap_pending) CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_snap_done, 0));
  if (n > ctx->snap_cap) {
    CK(cudaStreamSynchronize(ctx->snap_stream));
    if (ctx->d_snap) cudaFree(ctx->d_snap);
    if (ctx->h_snap) cudaFreeHost(ctx->h_snap);
    ctx->d_snap = nullptr;
    ctx->h_snap = nullptr;
    ctx->snap_cap = 0;
    CK(cudaMalloc(&ctx->d_snap, n * sizeof(double)));
    CK(cudaMallocHost(&ctx->h_snap, n * sizeof(double)));
    ctx->snap_cap = n;
  }
  for (int b = 1; b <= (int)hc.blocks.size(); b++) {
    int k = find_block(ctx, case_id, 1, b);
    const BlkDev &bd = lv.blk[k];
    int items = (bd.nx + 3) * (bd.ny + 3);
    launch_unpack_u(L, k, L.nvar, ctx->d_snap + off[b - 1], items, ctx->stream);
    CK(cudaMemcpyAsync(ctx->d_snap + off[b - 1] + (size_t)items * L.nvar, L.amut + bd.off,
                       (size_t)bd.P * (bd.ny + 5) * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
  }
  ctx->launches += (long long)hc.blocks.size();
  CK(cudaEventRecord(ctx->ev_snap, ctx->stream));
  CK(cudaStreamWaitEvent(ctx->snap_stream, ctx->ev_snap, 0));
  CK(cudaMemcpyAsync(ctx->h_snap, ctx->d_snap, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->snap_stream));
  CK(cudaEventRecord(ctx->ev_snap_done, ctx->snap_stream));
  ctx->snap_off = off;
  ctx->snap_case = case_id;
  ctx->snap_kstep = hc.kstep[1];
  ctx->snap_tt = hc.tt[1];
  ctx->snap_pending = true;
  return check_launch(ctx);
}

int ec2d_snapshot_wait(ec2d_ctx *ctx, int *case_id, int *kstep, double *tt) {
  if (!ctx || !ctx->snap_pending) return EC2D_ERR_ARG;
  cudaSetDevice(ctx->device);
  CK(cudaEventSynchronize(ctx->ev_snap_done));
  if (case_id) *case_id = ctx->snap_case;
  if (kstep) *kstep = ctx->snap_kstep;
  if (tt) *tt = ctx->snap_tt;
  return EC2D_OK;
}

int ec2d_snapshot_U(ec2d_ctx *ctx, int block, double *U) {
  if (!ctx || !ctx->snap_pending || !U || block < 1 || block > (int)ctx->snap_off.size()) return EC2D_ERR_ARG;
  int r = ec2d_snapshot_wait(ctx, nullptr, nullptr, nullptr);
  if (r) return r;
  int k = find_block(ctx, ctx->snap_case, 1, block);
  if (k < 0) return EC2D_ERR_ARG;
  const BlkDev &b = ctx->lv[1].blk[k];
  size_t n = (size_t)(b.nx + 3) * (b.ny + 3) * ctx->lv[1].L.nvar;
  memcpy(U, ctx->h_snap + ctx->snap_off[block - 1], n * sizeof(double));
  return EC2D_OK;
}

int ec2d_snapshot_amut(ec2d_ctx *ctx, int block, double *amut) {
  if (!ctx || !ctx->snap_pending || !amut || block < 1 || block > (int)ctx->snap_off.size()) return EC2D_ERR_ARG;
  int r = ec2d_snapshot_wait(ctx, nullptr, nullptr, nullptr);
  if (r) return r;
  int k = find_block(ctx, ctx->snap_case, 1, block);
  if (k < 0) return EC2D_ERR_ARG;
  const BlkDev &b = ctx->lv[1].blk[k];
  const double *fr = ctx->h_snap + ctx->snap_off[block - 1] + (size_t)(b.nx + 3) * (b.ny + 3) * ctx->lv[1].L.nvar;
  for (int j = -1; j <= b.ny + 1; j++)
    for (int i = -1; i <= b.nx + 1; i++)
      amut[(size_t)(i + 1) + (size_t)(b.nx + 3) * (j + 1)] = fr[(size_t)(j + 2) * b.P + (i + 2)];
  return EC2D_OK;
}

int ec2d_step(ec2d_ctx *ctx, int nsteps) {
  if (!ctx || !ctx->setup_done || nsteps < 0) return EC2D_ERR_ARG;
  cudaSetDevice(ctx->device);
  // dual time reads norms on the host inside the step; timing records events
  bool graph = ctx->use_graphs && !ctx->timing && ctx->P.Time_Method != Time_Dual && nsteps > 0;
  if (graph && !ctx->step_graph) {
    int r = capture_step(ctx);
    if (r) return r;
  }
  for (int n = 0; n < nsteps; n++) {
    if (graph && ctx->step_graph) {
      CK(cudaGraphLaunch(ctx->step_graph, ctx->stream));
      ctx->launches += ctx->graph_launches;
      for (int l = 1; l <= 3; l++)
        for (int k = 0; k < ctx->graph_adv[l]; k++) advance_counters(ctx, l);
      continue;
    }
    int r = one_step(ctx);
    if (r) return r;
  }
  return check_launch(ctx);
}

int ec2d_set_graphs(ec2d_ctx *ctx, int enable) {
  if (!ctx) return EC2D_ERR_ARG;
  ctx->use_graphs = enable != 0;
  return EC2D_OK;
}

static void drop_graph(ec2d_ctx *ctx) {
  if (ctx->step_graph) {
    cudaStreamSynchronize(ctx->stream);
    cudaGraphExecDestroy(ctx->step_graph);
    ctx->step_graph = nullptr;
  }
}

int ec2d_autotune(ec2d_ctx *ctx, int trial_steps, int *lusgs_cs, int *rows_per_warp, int *concurrent,
                  double *ms_per_step) {
  if (!ctx || !ctx->setup_done || trial_steps < 1) return EC2D_ERR_ARG;
  cudaSetDevice(ctx->device);
  // snapshot of the state a trial changes: fine-mesh U and the step counters
  // (coarse levels are rebuilt from the fine mesh by every V-cycle), and with
  // dual time stepping the two physical time levels and the first-step flags
  const Level &lv = ctx->lv[1];
  const size_t bytes = (size_t)lv.L.nvar * lv.F * sizeof(double);
  const bool dual = ctx->P.Time_Method == Time_Dual;
  const size_t nelem = bytes / sizeof(double);
  double *snap = nullptr;
  CK(cudaMalloc(&snap, (dual ? 3 : 1) * bytes));
  CK(cudaMemcpyAsync(snap, lv.L.U, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
  if (dual) {
    CK(cudaMemcpyAsync(snap + nelem, lv.L.un, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    CK(cudaMemcpyAsync(snap + 2 * nelem, lv.L.un1, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
  }
  const int dflag = ctx->dual_iflag, dflag1 = ctx->dual_iflag1;
  // the status words of every level (a trial step on a state that trips the
  // T < 1e-5 test must not leave its stop on the restored state)
  const size_t nst = 4 * ctx->cases.size();
  std::vector<std::vector<int>> st(ctx->num_mesh + 1, std::vector<int>(nst));
  for (int l = 1; l <= ctx->num_mesh; l++)
    CK(cudaMemcpyAsync(st[l].data(), ctx->lv[l].L.status, nst * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  std::vector<std::array<int, 4>> ks(ctx->cases.size());
  std::vector<std::array<double, 4>> ts(ctx->cases.size());
  for (size_t c = 0; c < ctx->cases.size(); c++)
    for (int l = 0; l < 4; l++) { ks[c][l] = ctx->cases[c].kstep[l]; ts[c][l] = ctx->cases[c].tt[l]; }
  cudaEvent_t a, b;
  CK(cudaEventCreate(&a));
  CK(cudaEventCreate(&b));
  // candidates: the FP64 wavefront's shape -- bands of 12 or 16 rows with
  // eight lanes per row or of 24 or 32 rows with four (where they fit), one
  // CTA per block with 32, 24 or 16 rows per warp, or a cluster of 2, 4, 8
  // CTAs (the FP32 sweep has one shape) -- x concurrent face kernels
  // (cs, rows, lanes); bands of 6 or 8 rows need 12-16 CTAs per cluster
  // (non-portable sizes, used where the device places them)
  std::vector<std::array<int, 3>> shapes = {{0, 12, 0}};
  if (!ctx->lusgs_fp32 && ctx->P.Time_Method == Time_LU_SGS)
    for (auto sh : std::vector<std::array<int, 3>>{{0, 16, 0}, {0, 24, 0}, {0, 32, 0}, {0, 8, 8}, {0, 8, 4},
                                                   {0, 6, 8}, {0, 6, 4}, {1, 32, 0}, {1, 24, 0}, {1, 16, 0},
                                                   {2, 32, 0}, {4, 32, 0}, {8, 32, 0}})
      shapes.push_back(sh);
  const int old_cs = ctx->lusgs_cs, old_rpw = ctx->lusgs_rpw, old_lanes = ctx->lusgs_lanes;
  const bool old_cc = ctx->concurrent;
  double best = 1e30;
  int best_cs = old_cs, best_rpw = old_rpw, best_lanes = old_lanes, best_cc = old_cc ? 1 : 0, r = EC2D_OK;
  for (auto sh : shapes) {
    for (int cc = 0; cc < 2 && r == EC2D_OK; cc++) {
      ctx->lusgs_cs = sh[0];
      ctx->lusgs_rpw = sh[1];
      ctx->lusgs_lanes = sh[2];
      ctx->concurrent = cc != 0;
      drop_graph(ctx);
      if ((r = ec2d_step(ctx, 1)) != EC2D_OK) break;
      cudaEventRecord(a, ctx->stream);
      if ((r = ec2d_step(ctx, trial_steps)) != EC2D_OK) break;
      cudaEventRecord(b, ctx->stream);
      cudaEventSynchronize(b);
      float ms = 0.0f;
      cudaEventElapsedTime(&ms, a, b);
      if (ms / trial_steps < best) {
        best = ms / trial_steps;
        best_cs = sh[0];
        best_rpw = sh[1];
        best_lanes = sh[2];
        best_cc = cc;
      }
    }
  }
  ctx->lusgs_cs = r == EC2D_OK ? best_cs : old_cs;
  ctx->lusgs_rpw = r == EC2D_OK ? best_rpw : old_rpw;
  ctx->lusgs_lanes = r == EC2D_OK ? best_lanes : old_lanes;
  ctx->concurrent = r == EC2D_OK ? best_cc != 0 : old_cc;
  // then, with that shape, the one-kernel residual against the four-kernel
  // chain (where some level can take it)
  bool tile_applies = false;
  for (int l = 1; l <= ctx->num_mesh; l++)
    tile_applies |= ctx->lv[l].L.turb == Turb_NONE && !ctx->lv[l].L.fdm && !ctx->lv[l].L.keep_amut;
  if (r == EC2D_OK && tile_applies) {
    const bool old_tile = ctx->tile_residual;
    double tbest = 1e30;
    bool tpick = old_tile;
    for (int tile = 0; tile < 2 && r == EC2D_OK; tile++) {
      ctx->tile_residual = tile != 0;
      drop_graph(ctx);
      if ((r = ec2d_step(ctx, 1)) != EC2D_OK) break;
      cudaEventRecord(a, ctx->stream);
      if ((r = ec2d_step(ctx, trial_steps)) != EC2D_OK) break;
      cudaEventRecord(b, ctx->stream);
      cudaEventSynchronize(b);
      float ms = 0.0f;
      cudaEventElapsedTime(&ms, a, b);
      if (ms / trial_steps < tbest) { tbest = ms / trial_steps; tpick = tile != 0; }
    }
    ctx->tile_residual = r == EC2D_OK ? tpick : old_tile;
    if (r == EC2D_OK) best = std::min(best, tbest);
  }
  drop_graph(ctx);
  cudaMemcpyAsync(lv.L.U, snap, bytes, cudaMemcpyDeviceToDevice, ctx->stream);
  if (dual) {
    cudaMemcpyAsync(lv.L.un, snap + nelem, bytes, cudaMemcpyDeviceToDevice, ctx->stream);
    cudaMemcpyAsync(lv.L.un1, snap + 2 * nelem, bytes, cudaMemcpyDeviceToDevice, ctx->stream);
  }
  ctx->dual_iflag = dflag;
  ctx->dual_iflag1 = dflag1;
  for (int l = 1; l <= ctx->num_mesh; l++)
    cudaMemcpyAsync(ctx->lv[l].L.status, st[l].data(), nst * sizeof(int), cudaMemcpyHostToDevice, ctx->stream);
  cudaStreamSynchronize(ctx->stream);
  cudaFree(snap);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  for (size_t c = 0; c < ctx->cases.size(); c++)
    for (int l = 0; l < 4; l++) { ctx->cases[c].kstep[l] = ks[c][l]; ctx->cases[c].tt[l] = ts[c][l]; }
  if (r) return r;
  if (lusgs_cs) *lusgs_cs = ctx->lusgs_cs;
  if (rows_per_warp) *rows_per_warp = ctx->lusgs_rpw;
  if (concurrent) *concurrent = ctx->concurrent ? 1 : 0;
  if (ms_per_step) *ms_per_step = best;
  return check_launch(ctx);
}

int ec2d_lusgs_shape(ec2d_ctx *ctx, int *cs, int *rows, int *lanes) {
  if (!ctx) return EC2D_ERR_ARG;
  if (cs) *cs = ctx->lusgs_cs;
  if (rows) *rows = ctx->lusgs_rpw;
  if (lanes) *lanes = ctx->lusgs_lanes ? ctx->lusgs_lanes : (ctx->lusgs_rpw <= 16 ? 8 : 4);
  return EC2D_OK;
}

int ec2d_tile_residual(ec2d_ctx *ctx, int enable, int *current) {
  if (!ctx || enable < -1 || enable > 1) return EC2D_ERR_ARG;
  if (enable >= 0 && (enable != 0) != ctx->tile_residual) {
    ctx->tile_residual = enable != 0;
    drop_graph(ctx);
  }
  if (current) *current = ctx->tile_residual ? 1 : 0;
  return EC2D_OK;
}

int ec2d_launch_config(ec2d_ctx *ctx, int *lusgs_cs, int *rows, int *lanes, int *concurrent, int *tile_residual) {
  if (!ctx) return EC2D_ERR_ARG;
  if (lusgs_cs) *lusgs_cs = ctx->lusgs_cs;
  if (rows) *rows = ctx->lusgs_rpw;
  if (lanes) *lanes = ctx->lusgs_lanes;
  if (concurrent) *concurrent = ctx->concurrent ? 1 : 0;
  if (tile_residual) *tile_residual = ctx->tile_residual ? 1 : 0;
  return EC2D_OK;
}

// the ranges ec2d_create accepts from EC2D_LUSGS_* (the sweep launcher
// clamps the cluster size and falls back from shapes a level cannot take)
int ec2d_set_launch_config(ec2d_ctx *ctx, int lusgs_cs, int rows, int lanes, int concurrent, int tile_residual) {
  if (!ctx || lusgs_cs < 0 || lusgs_cs > 8 || rows < 4 || rows > 32 || (lanes != 0 && lanes != 4 && lanes != 8) ||
      concurrent < 0 || concurrent > 1 || tile_residual < 0 || tile_residual > 1)
    return EC2D_ERR_ARG;
  if (lusgs_cs != ctx->lusgs_cs || rows != ctx->lusgs_rpw || lanes != ctx->lusgs_lanes ||
      (concurrent != 0) != ctx->concurrent || (tile_residual != 0) != ctx->tile_residual) {
    ctx->lusgs_cs = lusgs_cs;
    ctx->lusgs_rpw = rows;
    ctx->lusgs_lanes = lanes;
    ctx->concurrent = concurrent != 0;
    ctx->tile_residual = tile_residual != 0;
    drop_graph(ctx);
  }
  return EC2D_OK;
}

// digest of the library's sources, written by the build (ec2d_build.py)
extern "C" const char ec2d_internal_build_id[];

int ec2d_launch_signature(ec2d_ctx *ctx, char *buf, int len, int *needed) {
  if (!ctx || !ctx->setup_done || len < 0) return EC2D_ERR_ARG;
  cudaDeviceProp pr;
  CK(cudaGetDeviceProperties(&pr, ctx->device));
  const ec2d_params &P = ctx->P;
  char t[512];
  snprintf(t, sizeof t, "ec2d-launch-1 lib=%d build=%s dev=%s sm=%d%d sms=%d", ec2d_version(),
           ec2d_internal_build_id, pr.name, pr.major, pr.minor, pr.multiProcessorCount);
  std::string s = t;
  snprintf(t, sizeof t,
           " visc=%d turb=%d time=%d local_dt=%d scheme=%d flux=%d recon=%d mesh=%d mg_lusgs=%d lusgs=%d"
           " coarse=%d mg_amut=%d cases=%d",
           P.If_viscous, P.Iflag_turbulence_model, P.Time_Method, P.Iflag_local_dt, P.Iflag_Scheme, P.Iflag_flux,
           P.IFlag_Reconstruction, ctx->num_mesh, P.mg_lusgs, ctx->lusgs_fp32 ? 32 : 64, ctx->coarse_fp32 ? 32 : 64,
           ctx->mg_amut ? 1 : 0, (int)ctx->cases.size());
  s += t;
  // per level: variables, then each block shape (cells, 'f' on finite-
  // difference blocks) with its count, in sorted order
  for (int l = 1; l <= ctx->num_mesh; l++) {
    std::map<std::array<int, 3>, int> shapes;
    for (const HLevelBlock &hb : ctx->lv[l].hb) shapes[{hb.nx - 1, hb.ny - 1, hb.fdm ? 1 : 0}]++;
    snprintf(t, sizeof t, " L%d:nv%d", l, ctx->lv[l].L.nvar);
    s += t;
    for (const auto &kv : shapes) {
      snprintf(t, sizeof t, ",%dx%d%s*%d", kv.first[0], kv.first[1], kv.first[2] ? "f" : "", kv.second);
      s += t;
    }
  }
  const int n = (int)s.size() + 1;
  if (needed) *needed = n;
  if (!buf) return EC2D_OK;
  if (len < n) return EC2D_ERR_ARG;
  memcpy(buf, s.c_str(), (size_t)n);
  return EC2D_OK;
}

int ec2d_mg_eddy_viscosity(ec2d_ctx *ctx, int enable, int *current) {
  if (!ctx || enable < -1 || enable > 1) return EC2D_ERR_ARG;
  if (enable >= 0 && (enable != 0) != ctx->mg_amut) {
    ctx->mg_amut = enable != 0;
    if (ctx->setup_done) apply_mg_amut(ctx);
    drop_graph(ctx);
  }
  if (current) *current = ctx->mg_amut ? 1 : 0;
  return EC2D_OK;
}

int ec2d_set_coarse_precision(ec2d_ctx *ctx, int bits) {
  if (!ctx || (bits != 32 && bits != 64)) return EC2D_ERR_ARG;
  bool fp32 = bits == 32;
  if (fp32 != ctx->coarse_fp32) drop_graph(ctx);
  ctx->coarse_fp32 = fp32;
  return EC2D_OK;
}

int ec2d_set_lusgs_precision(ec2d_ctx *ctx, int bits) {
  if (!ctx || (bits != 32 && bits != 64)) return EC2D_ERR_ARG;
  bool fp32 = bits == 32;
  if (fp32 != ctx->lusgs_fp32 && ctx->step_graph) {
    cudaSetDevice(ctx->device);
    CK(cudaStreamSynchronize(ctx->stream));
    cudaGraphExecDestroy(ctx->step_graph);
    ctx->step_graph = nullptr;
  }
  ctx->lusgs_fp32 = fp32;
  return EC2D_OK;
}

int ec2d_residual(ec2d_ctx *ctx, int case_id, int mesh, double res_max[6], double res_rms[6], int *kstep,
                  double *tt) {
  if (!ctx || !ctx->setup_done || !valid_case(ctx, case_id) || mesh < 1 || mesh > ctx->num_mesh) return EC2D_ERR_ARG;
  cudaSetDevice(ctx->device);
  const Lvl &L = ctx->lv[mesh].L;
  double nm[12];
  int st[4];
  CK(cudaMemcpyAsync(nm, L.norms + 12 * (case_id - 1), sizeof(nm), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(st, L.status + 4 * (case_id - 1), sizeof(st), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (res_max) for (int m = 0; m < 6; m++) res_max[m] = nm[m];
  if (res_rms) for (int m = 0; m < 6; m++) res_rms[m] = nm[6 + m];
  if (kstep) *kstep = ctx->cases[case_id - 1].kstep[mesh];
  if (tt) *tt = ctx->cases[case_id - 1].tt[mesh];
  return status_error(st[0]);
}

int ec2d_run_to_drop(ec2d_ctx *ctx, double drop, const double *r0, int max_steps, double max_seconds,
                     int check_every, int *steps, double *worst_ratio, double *seconds) {
  if (!ctx || !ctx->setup_done || !(drop > 0.0) || max_steps < 1 || check_every < 1) return EC2D_ERR_ARG;
  cudaSetDevice(ctx->device);
  const auto t0 = std::chrono::steady_clock::now();
  auto elapsed = [&] { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); };
  const Lvl &L = ctx->lv[1].L;
  const int nc = L.ncase;
  std::vector<double> nm(12 * (size_t)nc), ref(nc);
  std::vector<int> st(4 * (size_t)nc);
  // Res_rms(1) of every case after the last step; false if a case stopped
  auto read = [&]() -> int {
    CK(cudaMemcpyAsync(nm.data(), L.norms, nm.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(st.data(), L.status, st.size() * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    for (int c = 0; c < nc; c++) if (st[4 * c]) return status_error(st[4 * c]);
    return EC2D_OK;
  };
  int n = 0, r;
  double worst = 1.0;
  if (r0) {
    for (int c = 0; c < nc; c++) ref[c] = r0[c];
  } else {
    if ((r = ec2d_step(ctx, 1)) != EC2D_OK) return r;
    n = 1;
    if ((r = read()) != EC2D_OK) return r;
    for (int c = 0; c < nc; c++) ref[c] = nm[12 * c + 6];
  }
  while (true) {
    if (n > 0) {
      worst = 0.0;
      for (int c = 0; c < nc; c++) worst = std::max(worst, ref[c] > 0.0 ? nm[12 * c + 6] / ref[c] : 0.0);
      if (worst <= drop) break;
    }
    if (n >= max_steps || (max_seconds > 0.0 && elapsed() >= max_seconds)) break;
    int k = std::min(check_every, max_steps - n);
    if ((r = ec2d_step(ctx, k)) != EC2D_OK) return r;
    n += k;
    if ((r = read()) != EC2D_OK) return r;
  }
  if (steps) *steps = n;
  if (worst_ratio) *worst_ratio = worst;
  if (seconds) *seconds = elapsed();
  return EC2D_OK;
}

int ec2d_status(ec2d_ctx *ctx, int case_id, int *code, int *block, int *i, int *j) {
  if (!ctx || !ctx->setup_done || !valid_case(ctx, case_id)) return EC2D_ERR_ARG;
  cudaSetDevice(ctx->device);
  int st[4] = {0, 0, 0, 0};
  for (int l = 1; l <= ctx->num_mesh; l++) {
    CK(cudaMemcpyAsync(st, ctx->lv[l].L.status + 4 * (case_id - 1), sizeof(st), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (st[0]) {
      if (st[1] >= 0 && st[1] < (int)ctx->lv[l].hb.size()) st[1] = ctx->lv[l].hb[st[1]].blk + 1;
      break;
    }
  }
  if (code) *code = st[0];
  if (block) *block = st[1];
  if (i) *i = st[2];
  if (j) *j = st[3];
  return EC2D_OK;
}

static int run_forces(ec2d_ctx *ctx, int case_id, std::vector<double> &out) {
  Level &lv = ctx->lv[1];
  int c = case_id - 1;
  if (lv.wall_faces.empty()) { out.clear(); return EC2D_OK; }
  launch_prim(lv.L, ctx->stream);
  launch_forces(lv.L, lv.d_faces, (int)lv.wall_faces.size(), lv.d_face_out, ctx->stream);
  int n = lv.case_nface[c];
  out.assign((size_t)n * 5, 0.0);
  if (n)
    CK(cudaMemcpyAsync(out.data(), lv.d_face_out + (size_t)5 * lv.case_face0[c], out.size() * sizeof(double),
                       cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return check_launch(ctx);
}

int ec2d_forces(ec2d_ctx *ctx, int case_id, double *cl, double *cd, double *cm) {
  if (!ctx || !ctx->setup_done || !valid_case(ctx, case_id)) return EC2D_ERR_ARG;
  cudaSetDevice(ctx->device);
  std::vector<double> out;
  int r = run_forces(ctx, case_id, out);
  if (r) return r;
  const ec2d_params &p = ctx->cases[case_id - 1].p;
  double Fx = 0, Fy = 0, Mz = 0;
  for (size_t f = 0; f < out.size() / 5; f++) {
    Fx += out[5 * f]; Fy += out[5 * f + 1];
    Mz += (out[5 * f + 2] - p.xaxis) * out[5 * f + 1] - (out[5 * f + 3] - p.yaxis) * out[5 * f];
  }
  double aoa = p.AoA * PI / 180.0, q = 0.5, ca = std::cos(aoa), sa = std::sin(aoa);
  if (cl) *cl = (-Fx * sa + Fy * ca) / q;
  if (cd) *cd = (Fx * ca + Fy * sa) / q;
  if (cm) *cm = -Mz / q;
  return EC2D_OK;
}

int ec2d_wall_cf(ec2d_ctx *ctx, int case_id, int block, int sub, double *cf, double *xc, int maxn, int *n) {
  if (!ctx || !ctx->setup_done || !valid_case(ctx, case_id)) return EC2D_ERR_ARG;
  cudaSetDevice(ctx->device);
  std::vector<double> out;
  int r = run_forces(ctx, case_id, out);
  if (r) return r;
  Level &lv = ctx->lv[1];
  int cnt = 0;
  int f0 = lv.case_face0[case_id - 1];
  for (int f = 0; f < lv.case_nface[case_id - 1]; f++) {
    int4 w = lv.wall_faces[f0 + f];
    if (lv.hb[w.x].blk != block - 1 || w.w != sub - 1) continue;
    if (cnt < maxn) { if (cf) cf[cnt] = out[5 * f + 4]; if (xc) xc[cnt] = out[5 * f + 2]; }
    cnt++;
  }
  if (n) *n = cnt;
  return EC2D_OK;
}

int ec2d_field_size(ec2d_ctx *ctx, int case_id, int mesh, int block, int field, int *n) {
  int k = find_block(ctx, case_id, mesh, block);
  FieldShape fs;
  if (k < 0 || !n || !field_shape(ctx, mesh, field, ctx->lv[mesh].blk[k], fs)) return EC2D_ERR_ARG;
  *n = fs.nv * (fs.i1 - fs.i0 + 1) * (fs.j1 - fs.j0 + 1);
  return EC2D_OK;
}

int ec2d_get_field(ec2d_ctx *ctx, int case_id, int mesh, int block, int field, double *out) {
  int k = find_block(ctx, case_id, mesh, block);
  FieldShape fs;
  if (k < 0 || !out || !field_shape(ctx, mesh, field, ctx->lv[mesh].blk[k], fs)) return EC2D_ERR_ARG;
  cudaSetDevice(ctx->device);
  CK(cudaStreamSynchronize(ctx->stream));
  const BlkDev &b = ctx->lv[mesh].blk[k];
  long long F = ctx->lv[mesh].F;
  size_t fsz = (size_t)b.P * (b.ny + 5);
  std::vector<double> fr(fsz);
  int ni = fs.i1 - fs.i0 + 1, nj = fs.j1 - fs.j0 + 1;
  for (int m = 0; m < fs.nv; m++) {
    CK(cudaMemcpy(fr.data(), fs.base + (size_t)m * F + b.off, fsz * sizeof(double), cudaMemcpyDeviceToHost));
    for (int j = 0; j < nj; j++)
      for (int i = 0; i < ni; i++)
        out[(size_t)m + (size_t)fs.nv * (i + (size_t)ni * j)] = fr[(size_t)(fs.j0 + j + 2) * b.P + (fs.i0 + i + 2)];
  }
  return EC2D_OK;
}

int ec2d_set_field(ec2d_ctx *ctx, int case_id, int mesh, int block, int field, const double *in) {
  int k = find_block(ctx, case_id, mesh, block);
  FieldShape fs;
  if (k < 0 || !in || !field_shape(ctx, mesh, field, ctx->lv[mesh].blk[k], fs)) return EC2D_ERR_ARG;
  cudaSetDevice(ctx->device);
  CK(cudaStreamSynchronize(ctx->stream));
  const BlkDev &b = ctx->lv[mesh].blk[k];
  long long F = ctx->lv[mesh].F;
  size_t fsz = (size_t)b.P * (b.ny + 5);
  std::vector<double> fr(fsz);
  int ni = fs.i1 - fs.i0 + 1, nj = fs.j1 - fs.j0 + 1;
  for (int m = 0; m < fs.nv; m++) {
    double *dst = fs.base + (size_t)m * F + b.off;
    CK(cudaMemcpy(fr.data(), dst, fsz * sizeof(double), cudaMemcpyDeviceToHost));
    for (int j = 0; j < nj; j++)
      for (int i = 0; i < ni; i++)
        fr[(size_t)(fs.j0 + j + 2) * b.P + (fs.i0 + i + 2)] = in[(size_t)m + (size_t)fs.nv * (i + (size_t)ni * j)];
    CK(cudaMemcpy(dst, fr.data(), fsz * sizeof(double), cudaMemcpyHostToDevice));
  }
  return EC2D_OK;
}

int ec2d_comput_residual(ec2d_ctx *ctx, int mesh) {
  if (!ctx || !ctx->setup_done || mesh < 1 || mesh > ctx->num_mesh) return EC2D_ERR_ARG;
  cudaSetDevice(ctx->device);
  residual(ctx, mesh);
  return check_launch(ctx);
}
int ec2d_boundary_condition(ec2d_ctx *ctx, int mesh) {
  if (!ctx || !ctx->setup_done || mesh < 1 || mesh > ctx->num_mesh) return EC2D_ERR_ARG;
  cudaSetDevice(ctx->device);
  launch_bc(ctx->lv[mesh].L, 1, ctx->stream);
  return check_launch(ctx);
}
int ec2d_update_buffer(ec2d_ctx *ctx, int mesh) {
  if (!ctx || !ctx->setup_done || mesh < 1 || mesh > ctx->num_mesh) return EC2D_ERR_ARG;
  cudaSetDevice(ctx->device);
  launch_bc(ctx->lv[mesh].L, 2 | 4, ctx->stream);
  return check_launch(ctx);
}
int ec2d_du_lusgs(ec2d_ctx *ctx, int mesh, double alfa1) {
  if (!ctx || !ctx->setup_done || mesh < 1 || mesh > ctx->num_mesh) return EC2D_ERR_ARG;
  cudaSetDevice(ctx->device);
  const Level &lv = ctx->lv[mesh];
  const Lvl &L = lv.L;
  if (ctx->lusgs_fp32 && lv.fast32) launch_lusgs_fast32(L, alfa1, 0, lv.max_rows, ctx->stream);
  else if (lv.fast64)
    launch_lusgs_fast(L, alfa1, 0, lv.max_rows, lv.max_cols, ctx->lusgs_cs, ctx->lusgs_rpw, ctx->lusgs_lanes,
                      ctx->stream);
  else launch_lusgs(L, alfa1, ctx->stream);
  return check_launch(ctx);
}
int ec2d_time_advance(ec2d_ctx *ctx, int mesh) {
  if (!ctx || !ctx->setup_done || mesh < 1 || mesh > ctx->num_mesh) return EC2D_ERR_ARG;
  cudaSetDevice(ctx->device);
  int r = time_advance(ctx, mesh);
  if (r) return r;
  return check_launch(ctx);
}
int ec2d_interpolation2h(ec2d_ctx *ctx, int m1, int m2, int flag) {
  if (!ctx || !ctx->setup_done || m2 != m1 + 1 || m1 < 1 || m2 > ctx->num_mesh || (flag != 1 && flag != 2 && flag != 6))
    return EC2D_ERR_ARG;
  cudaSetDevice(ctx->device);
  launch_restrict(ctx->lv[m1].L, ctx->lv[m2].L, flag, ctx->stream);
  return check_launch(ctx);
}
int ec2d_prolong(ec2d_ctx *ctx, int m1, int m2, int flag) {
  if (!ctx || !ctx->setup_done || m2 != m1 - 1 || m2 < 1 || m1 > ctx->num_mesh || (flag < 1 || flag > 3))
    return EC2D_ERR_ARG;
  cudaSetDevice(ctx->device);
  launch_prolong(ctx->lv[m1].L, ctx->lv[m2].L, flag, ctx->stream);
  return check_launch(ctx);
}
int ec2d_force_function(ec2d_ctx *ctx, int mesh) {
  if (!ctx || !ctx->setup_done || mesh < 2 || mesh > ctx->num_mesh) return EC2D_ERR_ARG;
  cudaSetDevice(ctx->device);
  launch_force_fn(ctx->lv[mesh].L, ctx->stream);
  return check_launch(ctx);
}
int ec2d_stream(ec2d_ctx *ctx, void **stream) {
  if (!ctx || !stream) return EC2D_ERR_ARG;
  *stream = (void *)ctx->stream;
  return EC2D_OK;
}

int ec2d_launch_count(ec2d_ctx *ctx, long long *n) {
  if (!ctx || !n) return EC2D_ERR_ARG;
  *n = ctx->launches;
  return EC2D_OK;
}

int ec2d_kernel_timing(ec2d_ctx *ctx, int enable) {
  if (!ctx) return EC2D_ERR_ARG;
  ctx->timing = enable != 0;
  return EC2D_OK;
}

int ec2d_kernel_times(ec2d_ctx *ctx, char *buf, int buflen) {
  if (!ctx || !buf || buflen <= 0) return EC2D_ERR_ARG;
  cudaSetDevice(ctx->device);
  CK(cudaStreamSynchronize(ctx->stream));
  struct Acc { std::string name; int level; long long calls, nk; double ms; };
  std::vector<Acc> acc;
  for (auto &r : ctx->krec) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, r.a, r.b);
    ctx->evpool.push_back(r.a);
    ctx->evpool.push_back(r.b);
    bool found = false;
    for (auto &x : acc)
      if (x.name == r.name && x.level == r.level) { x.calls++; x.nk += r.nk; x.ms += ms; found = true; break; }
    if (!found) acc.push_back({r.name, r.level, 1, r.nk, (double)ms});
  }
  ctx->krec.clear();
  std::string out;
  char line[160];
  for (auto &x : acc) {
    snprintf(line, sizeof(line), "%s %d %lld %lld %.6f\n", x.name.c_str(), x.level, x.calls, x.nk, x.ms);
    out += line;
  }
  snprintf(buf, buflen, "%s", out.c_str());
  return (int)out.size() < buflen ? EC2D_OK : EC2D_ERR_ARG;
}

int ec2d_set_case_shape(ec2d_ctx *ctx, int case_id, double shape) {
  if (!ctx || !ctx->setup_done || !valid_case(ctx, case_id)) return EC2D_ERR_ARG;
  cudaSetDevice(ctx->device);
  CK(cudaMemcpyAsync(ctx->d_shape + (case_id - 1), &shape, sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return EC2D_OK;
}

}  // extern "C"

struct ec2d_mlp {
  ec2d::Net net;
};

extern "C" {

int ec2d_mlp_create(int device, int hidden_layers, int width, unsigned long long seed, ec2d_mlp **out) {
  if (!out || width % 128 != 0) return EC2D_ERR_ARG;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) return EC2D_ERR_CUDA;
  ec2d_mlp *m = new ec2d_mlp();
  int r = m->net.init(device, hidden_layers, width, seed);
  if (r) {
    m->net.destroy();
    delete m;
    return r == 1 ? EC2D_ERR_ARG : EC2D_ERR_CUDA;
  }
  *out = m;
  return EC2D_OK;
}

void ec2d_mlp_destroy(ec2d_mlp *m) {
  if (!m) return;
  m->net.destroy();
  delete m;
}

int ec2d_mlp_add_samples(ec2d_mlp *m, ec2d_ctx *ctx) {
  if (!m || !ctx || !ctx->setup_done) return EC2D_ERR_ARG;
  Net &net = m->net;
  if (net.device != ctx->device) return EC2D_ERR_ARG;
  cudaSetDevice(ctx->device);
  const Lvl &L = ctx->lv[1].L;
  long long n0 = net.nsamp, n = L.ncell;
  if (net.reserve_samples(n0 + n)) return EC2D_ERR_NOMEM;
  CK(cudaStreamSynchronize(net.stream));
  launch_features(L, ctx->d_shape, net.feat + n0 * NIN, net.targ + n0 * NOUT, ctx->stream);
  CK(cudaStreamSynchronize(ctx->stream));
  net.nsamp = n0 + n;
  return check_launch(ctx);
}

int ec2d_mlp_num_samples(ec2d_mlp *m, long long *n) {
  if (!m || !n) return EC2D_ERR_ARG;
  *n = m->net.nsamp;
  return EC2D_OK;
}

int ec2d_mlp_clear_samples(ec2d_mlp *m) {
  if (!m) return EC2D_ERR_ARG;
  m->net.nsamp = 0;
  return EC2D_OK;
}

int ec2d_mlp_fit_normalization(ec2d_mlp *m) {
  if (!m || m->net.nsamp < 2) return EC2D_ERR_ARG;
  cudaSetDevice(m->net.device);
  return m->net.fit_normalization() ? EC2D_ERR_CUDA : EC2D_OK;
}

int ec2d_mlp_train(ec2d_mlp *m, int steps, int batch, double lr, double *loss_out) {
  if (!m || steps < 0 || batch < 256 || batch % 256 || !(lr > 0.0) || m->net.nsamp < 1) return EC2D_ERR_ARG;
  Net &net = m->net;
  cudaSetDevice(net.device);
  if (net.ensure_batch(batch)) return EC2D_ERR_NOMEM;
  // one training step as a CUDA graph (its minibatch seed and Adam step count
  // live in device memory), re-recorded when batch, rate or GEMM path change
  if (!net.train_graph || net.graph_batch != batch || net.graph_lr != (float)lr || net.graph_kind != net.gemm_kind) {
    if (net.train_graph) cudaGraphExecDestroy(net.train_graph);
    net.train_graph = nullptr;
    CK(cudaStreamSynchronize(net.stream));
    CK(cudaStreamBeginCapture(net.stream, cudaStreamCaptureModeThreadLocal));
    net.gather(batch);
    net.forward(batch);
    net.backward(batch);
    net.adam((float)lr);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(net.stream, &g);
    if (e == cudaSuccess && g) e = cudaGraphInstantiate(&net.train_graph, g, 0);
    if (g) cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      cudaGetLastError();
      net.train_graph = nullptr;
    }
    net.graph_batch = batch;
    net.graph_lr = (float)lr;
    net.graph_kind = net.gemm_kind;
  }
  for (int k = 0; k < steps; k++) {
    if (net.train_graph) {
      CK(cudaGraphLaunch(net.train_graph, net.stream));
    } else {
      net.gather(batch);
      net.forward(batch);
      net.backward(batch);
      net.adam((float)lr);
    }
  }
  float l = 0.0f;
  CK(cudaMemcpyAsync(&l, net.d_loss, sizeof(float), cudaMemcpyDeviceToHost, net.stream));
  CK(cudaStreamSynchronize(net.stream));
  if (loss_out) *loss_out = l;
  if (cudaGetLastError() != cudaSuccess) return EC2D_ERR_CUDA;
  return net.check_err() ? EC2D_ERR_TIMEOUT : EC2D_OK;
}

int ec2d_mlp_warm_start(ec2d_mlp *m, ec2d_ctx *ctx, int *n_fallback) {
  if (!m || !ctx || !ctx->setup_done || m->net.device != ctx->device) return EC2D_ERR_ARG;
  Net &net = m->net;
  cudaSetDevice(ctx->device);
  int r = ec2d_init_flow(ctx);
  if (r) return r;
  const Level &lv = ctx->lv[1];
  const Lvl &L = lv.L;
  const long long n = L.ncell;
  float *feat = nullptr, *pred = nullptr;
  int *bad = nullptr;
  CK(cudaMalloc(&feat, (size_t)n * NIN * sizeof(float)));
  CK(cudaMalloc(&pred, (size_t)n * NOUT * sizeof(float)));
  CK(cudaMalloc(&bad, ctx->cases.size() * sizeof(int)));
  CK(cudaMemsetAsync(bad, 0, ctx->cases.size() * sizeof(int), ctx->stream));
  launch_features(L, ctx->d_shape, feat, nullptr, ctx->stream);
  CK(cudaStreamSynchronize(ctx->stream));
  r = net.predict(feat, n, pred);
  CK(cudaStreamSynchronize(net.stream));
  if (r == EC2D_OK && net.check_err()) r = EC2D_ERR_TIMEOUT;
  if (r == EC2D_OK) {
    launch_warm_start(L, pred, bad, ctx->stream);
    launch_bc(L, 1 | 2 | 4, ctx->stream);
    if (L.nvar >= 5) launch_bc(L, 8, ctx->stream);
  }
  std::vector<int> hb(ctx->cases.size());
  CK(cudaMemcpyAsync(hb.data(), bad, hb.size() * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  cudaFree(feat);
  cudaFree(pred);
  cudaFree(bad);
  if (r) return r == EC2D_ERR_TIMEOUT ? r : EC2D_ERR_CUDA;
  if (n_fallback) {
    int c = 0;
    for (int v : hb) c += v != 0;
    *n_fallback = c;
  }
  return check_launch(ctx);
}

int ec2d_mlp_num_layers(ec2d_mlp *m, int *nlin) {
  if (!m || !nlin) return EC2D_ERR_ARG;
  *nlin = m->net.nlin;
  return EC2D_OK;
}

int ec2d_mlp_layer_shape(ec2d_mlp *m, int layer, int *rows, int *cols) {
  if (!m || layer < 0 || layer >= m->net.nlin || !rows || !cols) return EC2D_ERR_ARG;
  *rows = m->net.layer_out(layer);
  *cols = m->net.layer_in(layer);
  return EC2D_OK;
}

static int mlp_copy(ec2d_mlp *m, int layer, float *dw, float *db, const float *sw, const float *sb, bool grads) {
  if (!m || layer < 0 || layer >= m->net.nlin) return EC2D_ERR_ARG;
  Net &net = m->net;
  cudaSetDevice(net.device);
  Layer &Ly = net.L[layer];
  size_t nw = (size_t)net.layer_out(layer) * net.layer_in(layer), nb = net.layer_out(layer);
  CK(cudaStreamSynchronize(net.stream));
  if (sw || sb) {
    if (sw) CK(cudaMemcpy(Ly.w, sw, nw * sizeof(float), cudaMemcpyHostToDevice));
    if (sb) CK(cudaMemcpy(Ly.b, sb, nb * sizeof(float), cudaMemcpyHostToDevice));
    net.refresh_bf16();
    CK(cudaStreamSynchronize(net.stream));
  } else {
    if (dw) CK(cudaMemcpy(dw, grads ? Ly.gw : Ly.w, nw * sizeof(float), cudaMemcpyDeviceToHost));
    if (db) CK(cudaMemcpy(db, grads ? Ly.gb : Ly.b, nb * sizeof(float), cudaMemcpyDeviceToHost));
  }
  return EC2D_OK;
}

int ec2d_mlp_get_weights(ec2d_mlp *m, int layer, float *w, float *b) {
  return mlp_copy(m, layer, w, b, nullptr, nullptr, false);
}
int ec2d_mlp_set_weights(ec2d_mlp *m, int layer, const float *w, const float *b) {
  if (!w && !b) return EC2D_ERR_ARG;
  return mlp_copy(m, layer, nullptr, nullptr, w, b, false);
}
int ec2d_mlp_get_grads(ec2d_mlp *m, int layer, float *gw, float *gb) {
  return mlp_copy(m, layer, gw, gb, nullptr, nullptr, true);
}

int ec2d_mlp_get_normalization(ec2d_mlp *m, float *nrm) {
  if (!m || !nrm) return EC2D_ERR_ARG;
  cudaSetDevice(m->net.device);
  CK(cudaStreamSynchronize(m->net.stream));
  CK(cudaMemcpy(nrm, m->net.nrm, (2 * NIN + 2 * NOUT) * sizeof(float), cudaMemcpyDeviceToHost));
  return EC2D_OK;
}
int ec2d_mlp_set_normalization(ec2d_mlp *m, const float *nrm) {
  if (!m || !nrm) return EC2D_ERR_ARG;
  cudaSetDevice(m->net.device);
  CK(cudaStreamSynchronize(m->net.stream));
  CK(cudaMemcpy(m->net.nrm, nrm, (2 * NIN + 2 * NOUT) * sizeof(float), cudaMemcpyHostToDevice));
  return EC2D_OK;
}

int ec2d_mlp_loss_grad(ec2d_mlp *m, const float *x, const float *y, int B, double *loss) {
  if (!m || !x || !y || B < 256 || B % 256) return EC2D_ERR_ARG;
  Net &net = m->net;
  cudaSetDevice(net.device);
  if (net.ensure_batch(B)) return EC2D_ERR_NOMEM;
  std::vector<__nv_bfloat16> xb((size_t)B * NIN_PAD, __float2bfloat16(0.0f));
  for (int r = 0; r < B; r++)
    for (int c = 0; c < NIN; c++) xb[(size_t)r * NIN_PAD + c] = __float2bfloat16(x[(size_t)r * NIN + c]);
  CK(cudaMemcpyAsync(net.X, xb.data(), xb.size() * sizeof(__nv_bfloat16), cudaMemcpyHostToDevice, net.stream));
  CK(cudaMemcpyAsync(net.Y, y, (size_t)B * NOUT * sizeof(float), cudaMemcpyHostToDevice, net.stream));
  net.forward(B);
  net.backward(B);
  float l = 0.0f;
  CK(cudaMemcpyAsync(&l, net.d_loss, sizeof(float), cudaMemcpyDeviceToHost, net.stream));
  CK(cudaStreamSynchronize(net.stream));
  if (loss) *loss = l;
  if (cudaGetLastError() != cudaSuccess) return EC2D_ERR_CUDA;
  return net.check_err() ? EC2D_ERR_TIMEOUT : EC2D_OK;
}

int ec2d_mlp_set_gemm(ec2d_mlp *m, int kind) {
  if (!m || (kind != 0 && kind != 1)) return EC2D_ERR_ARG;
  m->net.gemm_kind = kind;
  return EC2D_OK;
}

int ec2d_mlp_predict(ec2d_mlp *m, const float *feat, long long n, float *pred) {
  if (!m || !feat || !pred || n < 1) return EC2D_ERR_ARG;
  Net &net = m->net;
  cudaSetDevice(net.device);
  float *df = nullptr, *dp = nullptr;
  CK(cudaMalloc(&df, (size_t)n * NIN * sizeof(float)));
  CK(cudaMalloc(&dp, (size_t)n * NOUT * sizeof(float)));
  CK(cudaMemcpy(df, feat, (size_t)n * NIN * sizeof(float), cudaMemcpyHostToDevice));
  int r = net.predict(df, n, dp);
  cudaStreamSynchronize(net.stream);
  if (r == 0) cudaMemcpy(pred, dp, (size_t)n * NOUT * sizeof(float), cudaMemcpyDeviceToHost);
  cudaFree(df);
  cudaFree(dp);
  if (r) return EC2D_ERR_CUDA;
  return net.check_err() ? EC2D_ERR_TIMEOUT : EC2D_OK;
}

int ec2d_sync(ec2d_ctx *ctx) {
  if (!ctx) return EC2D_ERR_ARG;
  cudaSetDevice(ctx->device);
  CK(cudaStreamSynchronize(ctx->stream));
  return EC2D_OK;
}

}  // extern "C"
