// ec2d_internal.h -- launch wrappers shared between the kernel files and the
// C-ABI layer (not part of the public interface).
#pragma once
#include <cuda_runtime.h>

#include "ec2d_dev.cuh"

namespace ec2d {

// k_residual.cu
void launch_prim(const Lvl &L, cudaStream_t s);
void launch_flux_i(const Lvl &L, bool fp32, cudaStream_t s);
void launch_flux_j(const Lvl &L, bool fp32, cudaStream_t s);
// post-residual steps k_res can do in the same pass (bits of `post`)
enum { RES_ADD_FORCE = 1, RES_FORCE_FN = 2, RES_SET_UN = 4 };
// cells per 2-D tile of the one-kernel residual (k_residual_tile) and its
// threads: (16 + 1) x 8 i-faces + 16 x 9 j-faces = 280 faces, 20 x 12 halo
// cells, 128 cells, each a thread of 288 (the 2 x 96 x 96 flat-plate level is
// 144 tiles, one per SM)
constexpr int RES_TILE_X = 16, RES_TILE_Y = 8, RES_TILE_THREADS = 288;
void launch_res(const Lvl &L, bool with_norms, int post, cudaStream_t s);
void launch_face_metrics(const Lvl &L, cudaStream_t s);
void launch_norms(const Lvl &L, bool partials, cudaStream_t s);
void launch_residual_tile(const Lvl &Lr, const int4 *rt, int ntiles, bool with_norms, int post, cudaStream_t s);
bool norms_fused_final(const Lvl &L);
// k_turb.cu
void launch_sa(const Lvl &L, cudaStream_t s);
void launch_sst(const Lvl &L, cudaStream_t s);
void launch_bl(const Lvl &L, cudaStream_t s);
void launch_amut_boundary(const Lvl &L, cudaStream_t s);
void launch_fdm(const Lvl &L, cudaStream_t s);
void launch_dual_term(const Lvl &L, double sfac, cudaStream_t s);
// k_bc.cu
void launch_bc(const Lvl &L, int phases, cudaStream_t s);
void launch_bc_normals(const Lvl &L, int max_nodes, cudaStream_t s);
// k_lusgs.cu
void launch_lusgs(const Lvl &L, double alfa1, cudaStream_t s);
// k_sweep.cu
int lusgs_planes(int nv);
// mode bits of the wavefront launchers: update U in the sweep, and take
// Res + QF for Res (a coarse level's forcing when its residual is reused)
// PREP_ONLY / SWEEP_ONLY launch one of the two kernels of the FP64 wavefront
// (record builder, sweep), so that per-kernel timing can bracket each
enum { LUSGS_UPDATE = 1, LUSGS_FORCE = 2, LUSGS_PREP_ONLY = 4, LUSGS_SWEEP_ONLY = 8 };
// mesh set-up (k_setup.cu): with finer != nullptr the level's nodes by node
// skipping first, then areas, faces, ghost nodes, cell centres and (fdm) the
// finite-difference metrics
void launch_setup_geometry(const Lvl &L, const Lvl *finer, bool fdm, cudaStream_t s);
// cs: 0 the banded multi-lane kernel where it fits, with at most rpw rows per
// CTA and `lanes` lanes per row (4 or 8; 0: eight up to 16 rows, four above),
// else one CTA per block; 1 one CTA per block with rpw rows per warp; 2..8 a
// cluster of cs CTAs with a barrier per plane
void launch_lusgs_fast(const Lvl &L, double alfa1, int mode, int max_rows, int max_cols, int cs, int rpw, int lanes,
                       cudaStream_t s);
size_t lusgs_smem(int nv, int rows);  // dynamic shared memory of the one-CTA FP64 sweep
void launch_lusgs_fast32(const Lvl &L, double alfa1, int mode, int max_rows, cudaStream_t s);
size_t lusgs32_smem(int nv, int rows);
// warm-start network <-> solver level (k_mlp.cu)
void launch_features(const Lvl &L, const double *shape, float *feat, float *targ, cudaStream_t s);
void launch_warm_start(const Lvl &L, const float *pred, int *bad, cudaStream_t s);
void launch_add_du(const Lvl &L, cudaStream_t s);
void launch_euler(const Lvl &L, int force, cudaStream_t s);
void launch_rk3(const Lvl &L, int stage, int force, cudaStream_t s);
void launch_add_force(const Lvl &L, cudaStream_t s);
void launch_force_fn(const Lvl &L, cudaStream_t s);
void launch_set_un(const Lvl &L, int nv, cudaStream_t s);
void launch_restrict(const Lvl &Lf, const Lvl &Lc, int flag, cudaStream_t s);
void launch_prolong(const Lvl &Lc, const Lvl &Lf, int flag, cudaStream_t s);
void launch_freestream(const Lvl &L, int flow, int turb, cudaStream_t s);
// k_misc.cu
void launch_pack_u(const Lvl &L, int bk, int nv, const double *aos, int nitems, cudaStream_t s);
void launch_unpack_u(const Lvl &L, int bk, int nv, double *aos, int nitems, cudaStream_t s);
void launch_wall_distance(const Lvl &L, int bk, const double *wall_xy, int nwall, int nx, int ny, cudaStream_t s);
void launch_forces(const Lvl &L, const int4 *faces, int nfaces, double *out, cudaStream_t s);

}  // namespace ec2d
