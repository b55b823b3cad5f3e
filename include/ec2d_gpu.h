/*
 * ec2d_gpu.h -- C-ABI of libec2d_gpu.so, the GB300-native (sm_103a)
 * pseudo-time-marching core of OpenCFD-EC2D.
 *
 * The reference is one Fortran program whose main loop
 * (opencfd_ec2d_v1.5.4.f90:172-186) calls NS_Time_advance(1),
 * NS_2stge_multigrid or NS_3stge_multigrid.  This library replaces the bodies
 * of those calls: the Fortran host (or any C/C++/Python host) keeps reading
 * control.in, bc2d_1.in and Mesh2d.dat and writing Residual.dat/flow2d.dat,
 * hands the grid and parameters over once, and then calls ec2d_step() per
 * iteration.  The solution, metrics, residuals, turbulence variables and the
 * multigrid levels stay on the GPU for the whole run; only the 12 residual
 * norms (and snapshots on request) come back.
 *
 * Conventions
 *  - Every function returns 0 on success or an EC2D_ERR_* code.
 *  - Arrays crossing the boundary use the reference's Fortran layout
 *    (column-major, variable index fastest), e.g. U(NVAR,-1:nx+1,-1:ny+1).
 *  - Block, mesh and case numbers are 1-based like the Fortran; case ids
 *    returned by ec2d_add_case start at 1.
 *  - One context = one CUDA stream on one device.  A context is not
 *    re-entrant; separate contexts are independent.  Calls are asynchronous
 *    on the context's stream except where they return host data.
 *  - A context may hold several cases (a batch, e.g. a polar sweep).  All
 *    cases of a context share the method flags (scheme, flux,
 *    reconstruction, viscous/turbulence model, time method, multigrid depth)
 *    and advance together in one launch per stage.
 */
#ifndef EC2D_GPU_H
#define EC2D_GPU_H
#ifdef __cplusplus
extern "C" {
#endif

#define EC2D_OK 0
#define EC2D_ERR_ARG 1        /* invalid argument / call order              */
#define EC2D_ERR_CUDA 2       /* CUDA runtime error                         */
#define EC2D_ERR_STATE 3      /* non-physical state (T < 1e-5), see ec2d_status */
#define EC2D_ERR_TIMEOUT 4    /* a device-side wait hit its iteration limit */
#define EC2D_ERR_UNSUPPORTED 5 /* option combination the reference refuses  */
#define EC2D_ERR_NOMEM 6

/* The scalars of control.in (Global_Var, opencfd_ec2d_v1.5.4.f90:103-110),
 * read from lines 2,4,6,8,10 (opencfd_ec2d_v1.5.4.f90:201-211); AoA in
 * degrees and Twall in kelvin as written in control.in.  xaxis/yaxis come
 * from control.in line 12 (moment reference point).  mg_lusgs=1 lifts the
 * reference's refusal of LU-SGS with multigrid (opencfd_ec2d_v1.5.4.f90:216-221)
 * and smooths every multigrid level with LU-SGS. */
typedef struct ec2d_params {
  double Ma, Re, gamma, AoA, Pr, t_end;
  int Kstep_save, If_viscous, Iflag_turbulence_model, Iflag_init;
  int Iflag_local_dt;
  double dt_global, CFL, dtmax, dtmin;
  int Time_Method;
  double P_outlet, T_inf, Twall, vt_inf, Kt_inf, Wt_inf;
  int Iflag_Scheme, Iflag_flux, IFlag_Reconstruction, Kstep_show;
  int Num_Mesh, Num_Threads, Nstep_Inner_Limit;
  double Res_Inner_Limit;
  int Pre_Step_Mesh[3];
  double xaxis, yaxis;
  int mg_lusgs;
} ec2d_params;

typedef struct ec2d_ctx ec2d_ctx;

/* Field ids for ec2d_get_field / ec2d_set_field (Fortran extents):
 *  RES (NVAR,1:nx-1,1:ny-1)  DT (1:nx-1,1:ny-1)  LCI..LVJ (1:nx,1:ny)
 *  DU (NVAR,1:nx,1:ny)  AMU, AMUT, X1, Y1 (-1:nx+1,-1:ny+1)
 *  VOL,SI,SJ,NI1,NI2,NJ1,NJ2 (1:nx,1:ny)  DW (0:nx,0:ny)
 *  QF (4,1:nx-1,1:ny-1)  DELTU (4,-1:nx+1,-1:ny+1)  UN (NVAR,0:nx,0:ny)
 *  X, Y (-1:nx+2,-1:ny+2)
 * DU holds the LU-SGS increment after ec2d_du_lusgs and after steps of
 * levels that take the general LU-SGS kernel; the wavefront sweep of a step
 * adds the increment to U directly and leaves DU as scratch (the reference
 * reads DU only inside du_LU_SGS_2D and the update after it,
 * sub_LU_SGS.f90:44-95, sub_NS_singlegrid.f90:197-211).  Likewise a
 * multigrid cycle fills DELTU of the finer level of each prolongation; the
 * coarse increment U - Un is formed where it is interpolated and not stored. */
enum {
  EC2D_F_RES = 0, EC2D_F_DT = 1, EC2D_F_LCI = 2, EC2D_F_LCJ = 3, EC2D_F_LVI = 4,
  EC2D_F_LVJ = 5, EC2D_F_DU = 6, EC2D_F_AMU = 7, EC2D_F_AMUT = 8, EC2D_F_X1 = 9,
  EC2D_F_Y1 = 10, EC2D_F_VOL = 11, EC2D_F_SI = 12, EC2D_F_SJ = 13, EC2D_F_NI1 = 14,
  EC2D_F_NI2 = 15, EC2D_F_NJ1 = 16, EC2D_F_NJ2 = 17, EC2D_F_DW = 18, EC2D_F_QF = 19,
  EC2D_F_DELTU = 20, EC2D_F_UN = 21, EC2D_F_X = 22, EC2D_F_Y = 23
};

/* Library version (major*10000+minor*100+patch) and error text. */
int ec2d_version(void);
const char *ec2d_error_string(int code);

/* Create an empty context on CUDA device `device` (its own streams).
 * Environment variables read here fix launch choices the autotuner would
 * otherwise make (none changes the arithmetic of a kernel):
 *   EC2D_LUSGS_CLUSTER  FP64 wavefront shape (see ec2d_autotune's lusgs_cs)
 *   EC2D_LUSGS_ROWS     rows per band, or rows per warp of the one-CTA shape
 *   EC2D_LUSGS_LANES    lanes per row of the banded shape (4 or 8)
 *   EC2D_CONCURRENT     0: every kernel on one stream (no concurrent graph
 *                       branches; results are bit-identical either way)
 *   EC2D_TILE_RESIDUAL  1: the residual as one kernel over shared-memory
 *                       tiles (see ec2d_tile_residual)
 *   EC2D_MG_EDDY_VISCOSITY  1: coarse multigrid levels keep the restricted
 *                       eddy viscosity (see ec2d_mg_eddy_viscosity; this one
 *                       changes the iteration, not the converged answer)
 *   EC2D_TEST_SILENT_BAND_EDGE  test hook: band edges of the banded wavefront
 *                       send nothing, so the downstream waits run out and the
 *                       next status read returns EC2D_ERR_TIMEOUT */
int ec2d_create(int device, ec2d_ctx **out);
void ec2d_destroy(ec2d_ctx *ctx);

/* Add one case with its control.in parameters (replaces read_parameter,
 * opencfd_ec2d_v1.5.4.f90:197-235).  *case_id receives the 1-based id. */
int ec2d_add_case(ec2d_ctx *ctx, const ec2d_params *p, int *case_id);

/* Add block `nblocks+1` of a case: node coordinates x(1:nx,1:ny), y(1:nx,1:ny)
 * (column-major, as read from Mesh2d.dat at sub_init.f90:176) and its nsub
 * subfaces, 9 ints each: f_no, face, ist, iend, jst, jend, neighb, subface,
 * orient (bc2d_1.in, sub_init.f90:246).  Replaces Creat_Mesh1 + read_bcin. */
int ec2d_add_block(ec2d_ctx *ctx, int case_id, int nx, int ny, const double *x,
                   const double *y, int nsub, const int *bc9);

/* Mark a block as a finite-difference (WENO5/Steger-Warming) block, as a
 * line of FDM.in does (sub_Finite_Difference.f90:287-308). */
int ec2d_set_fdm_block(ec2d_ctx *ctx, int case_id, int block);

/* Supply the cell wall distance dw(1:nx-1,1:ny-1) of a block, as
 * dist_wall.dat does (sub_turbulence_SST.f90:295-306).  Without it the
 * distance is computed on the GPU (comput_dw, sub_turbulence_SST.f90:310-340). */
int ec2d_set_wall_distance(ec2d_ctx *ctx, int case_id, int block, const double *dw);

/* Build everything on the device: multigrid depth (check_mesh_multigrid,
 * sub_init.f90:39-107), coarse meshes (Creat_Mesh, sub_init.f90:256-380),
 * ghost coordinates (Update_coordinate_buffer, sub_boundary.f90:159-301),
 * metrics, FDM Jacobians and wall distance. */
int ec2d_setup(ec2d_ctx *ctx);

/* Number of multigrid levels in use and the variable count of a level. */
int ec2d_num_mesh(ec2d_ctx *ctx, int *num_mesh);
int ec2d_block_dims(ec2d_ctx *ctx, int case_id, int mesh, int block, int *nx, int *ny, int *nvar);

/* Freestream start including the coarse-to-fine pre-iterations
 * (init_flow_zero, sub_init.f90:423-495) for every case; clears every
 * case's status word.  Like the reference's start, which follows the mesh
 * set-up, it runs with the coarse forcing QF zero, the dual-time first-step
 * flags unset and the step counters and times at zero, so a context that has
 * stepped before (or been autotuned) starts exactly as a new one. */
int ec2d_init_flow(ec2d_ctx *ctx);
/* Dual time stepping (Time_Method -1): start the physical-time history
 * from the current U of every case, U(n) = U(n-1) = U, with the first-step
 * flags unset, so that the next physical step takes the one-step form
 * (Dual_time_LU_SGS, sub_NS_singlegrid.f90:239-245, and the time term of
 * Comput_Residual_one_mesh, sub_Residual.f90:27-34, whose comment assumes
 * U(n-1) = U(n) on the first step).  ec2d_init_flow ends with it; a host
 * calls it after uploading a restart state (init_flow_read), which the
 * reference leaves with U(n) at its allocation fill (sub_init.f90:162) and
 * U(n-1) unset.  Does nothing for the other time methods. */
int ec2d_dual_time_start(ec2d_ctx *ctx);

/* Copy the conservative field of one block in or out, Fortran layout
 * U(NVAR,-1:nx+1,-1:ny+1) (the reference's B%U).  Host pointers may be
 * pageable or pinned. */
int ec2d_upload_U(ec2d_ctx *ctx, int case_id, int mesh, int block, const double *U);
int ec2d_download_U(ec2d_ctx *ctx, int case_id, int mesh, int block, double *U);

/* Asynchronous snapshot of a case's fine-mesh U for `output` at Kstep_save
 * (opencfd_ec2d_v1.5.4.f90:181,284-371), where ec2d_download_U would stall
 * the loop.  ec2d_snapshot enqueues, after the work queued so far, a device
 * copy of every block's U in the layout of ec2d_download_U, and the copy of
 * it to pinned host memory on a stream of its own; it returns at once and
 * later steps run while the copy proceeds (the block's eddy viscosity is
 * copied with it).  ec2d_snapshot_wait waits for
 * that copy and gives the case, Kstep and tt at which it was taken;
 * ec2d_snapshot_U copies one block of it into U(NVAR,-1:nx+1,-1:ny+1)
 * (waiting first).  One snapshot is held at a time: a new one replaces it
 * (the main stream waits only if the previous copy is still running). */
int ec2d_snapshot(ec2d_ctx *ctx, int case_id);
int ec2d_snapshot_wait(ec2d_ctx *ctx, int *case_id, int *kstep, double *tt);
int ec2d_snapshot_U(ec2d_ctx *ctx, int block, double *U);
/* The eddy viscosity Amu_t(-1:nx+1,-1:ny+1) of one block at the snapshot
 * (the Amut column of flow2d.dat is Amu_t * Re). */
int ec2d_snapshot_amut(ec2d_ctx *ctx, int block, double *amut);

/* Advance `nsteps` iterations of the main loop (opencfd_ec2d_v1.5.4.f90:174-180):
 * NS_Time_advance(1) when Num_Mesh==1, else one 2- or 3-level V-cycle. */
int ec2d_step(ec2d_ctx *ctx, int nsteps);

/* Residual norms of the last residual evaluation on `mesh` (MP%Res_max(1:6),
 * MP%Res_rms(1:6), written to Residual.dat at opencfd_ec2d_v1.5.4.f90:276),
 * the step counter and pseudo time.  Synchronises the stream; returns
 * EC2D_ERR_STATE if the case hit the T<1e-5 stop (sub_Residual.f90:143-146). */
int ec2d_residual(ec2d_ctx *ctx, int case_id, int mesh, double res_max[6], double res_rms[6],
                  int *kstep, double *tt);

/* Iterate to a residual drop.  No counterpart in the reference, whose main
 * loop runs to t_end (opencfd_ec2d_v1.5.4.f90:172-186).  Steps until every
 * case's continuity RMS residual MP%Res_rms(1) of the fine mesh is at most
 * `drop` times its reference value, checking every `check_every` steps (one
 * device-to-host read of the norms per check).  r0: per-case reference
 * values (ncase doubles), or NULL to take the residual of the first step of
 * this call.  Stops early after max_steps steps or max_seconds of wall time
 * (<= 0: no limit).  Outputs: steps taken, the worst case's Res_rms(1)/r0,
 * and the wall time in seconds.  Returns EC2D_ERR_STATE if a case hit the
 * T<1e-5 stop. */
int ec2d_run_to_drop(ec2d_ctx *ctx, double drop, const double *r0, int max_steps, double max_seconds,
                     int check_every, int *steps, double *worst_ratio, double *seconds);

/* Status word of a case: code (0 ok, 3 = T<1e-5) and the block/cell. */
int ec2d_status(ec2d_ctx *ctx, int case_id, int *code, int *block, int *i, int *j);
/* Clear the status word of one case (case_id 0: every case), e.g. after the
 * host replaced a failed case's state with ec2d_upload_U; ec2d_init_flow
 * clears every case's.  No counterpart in the reference, which stops. */
int ec2d_clear_status(ec2d_ctx *ctx, int case_id);

/* Lift, drag and moment coefficients (about xaxis, yaxis) from the wall
 * pressure and viscous stress of mesh 1; no counterpart in the reference,
 * whose read_flow-1.2.f90:36-51 writes wall Cp only. */
int ec2d_forces(ec2d_ctx *ctx, int case_id, double *cl, double *cd, double *cm);

/* Skin friction per wall face of subface `sub` of `block` (mesh 1) and the
 * face-centre x; returns the face count in *n (at most maxn written). */
int ec2d_wall_cf(ec2d_ctx *ctx, int case_id, int block, int sub, double *cf, double *xc,
                 int maxn, int *n);

/* Read or overwrite one field of one block (ids above, Fortran layout). */
int ec2d_get_field(ec2d_ctx *ctx, int case_id, int mesh, int block, int field, double *out);
int ec2d_field_size(ec2d_ctx *ctx, int case_id, int mesh, int block, int field, int *n);
int ec2d_set_field(ec2d_ctx *ctx, int case_id, int mesh, int block, int field, const double *in);

/* Finer-grained hooks with the reference's routine names (all blocks of all
 * cases on one mesh level): */
int ec2d_comput_residual(ec2d_ctx *ctx, int mesh);        /* Comput_Residual_one_mesh, sub_Residual.f90:13 */
int ec2d_boundary_condition(ec2d_ctx *ctx, int mesh);     /* Boundary_condition_onemesh, sub_boundary.f90:10 */
int ec2d_update_buffer(ec2d_ctx *ctx, int mesh);          /* update_buffer_onemesh, sub_boundary.f90:45 */
int ec2d_du_lusgs(ec2d_ctx *ctx, int mesh, double alfa1); /* du_LU_SGS_2D, sub_LU_SGS.f90:4 */
int ec2d_time_advance(ec2d_ctx *ctx, int mesh);           /* NS_Time_advance, sub_NS_singlegrid.f90:8 */
/* interpolation2h flags 1 (U) and 2 (residual sum into QF) as in the
 * reference; 6 is the multigrid cycle's form, QF = sum of the four fine Res
 * - the coarse Res (comput_force_function folded in). */
int ec2d_interpolation2h(ec2d_ctx *ctx, int m1, int m2, int flag); /* sub_NS_multigrid.f90:349 */
/* prolong_U flags 1 (U) and 2 (deltU) as in the reference; 3 is the cycle's
 * form: deltU = U - Un of the coarse level (comput_delt_U) prolonged into
 * the fine DELTU and added to the fine interior U (comput_new_U). */
int ec2d_prolong(ec2d_ctx *ctx, int m1, int m2, int flag);         /* prolong_U, sub_NS_multigrid.f90:271 */
int ec2d_force_function(ec2d_ctx *ctx, int mesh);         /* comput_force_function, sub_NS_multigrid.f90:156 */

/* Instrumentation for benchmarks: the context's cudaStream_t (so callers
 * can record CUDA events on it), the number of kernel launches issued so
 * far, and optional per-kernel event timing.  ec2d_kernel_times writes one
 * line "name level calls kernels total_ms" per kernel and level recorded
 * since timing was enabled (or since the last call) and clears the record. */
int ec2d_stream(ec2d_ctx *ctx, void **stream);
int ec2d_launch_count(ec2d_ctx *ctx, long long *n);
int ec2d_kernel_timing(ec2d_ctx *ctx, int enable);
int ec2d_kernel_times(ec2d_ctx *ctx, char *buf, int buflen);

/* Measured FP64 FMA throughput of the current device in TFLOP/s (2 FLOPs per
 * FMA; independent FMA chains on every SM, best of five timed launches).  No
 * counterpart in the reference: it is the denominator of the FP64 roofline
 * that bounds the residual and LU-SGS kernels on this part. */
int ec2d_measure_fp64_peak(double *tflops);

/* The cost model behind the latency-bound kernels: clock64 cycles per
 * operation of a chain of dependent operations, per warp, in one CTA of
 * `warps` warps (1..32) whose threads run `chains` (1, 2, 4, 8) independent
 * chains each.  op 0: FP64 fma; 1: FP64 divide; 2: the refined FP64
 * reciprocal of the face and wavefront paths; 3: FP32 fma; 4: a CTA barrier
 * (cycles per barrier); 5: a cluster barrier among `chains` CTAs.  No
 * counterpart in the reference. */
int ec2d_measure_op_cycles(int op, int warps, int chains, double *cycles);

/* The refined reciprocal of the face and wavefront paths checked on the
 * device on n inputs spread over [2^-8, 2^9): the largest relative error of
 * the hardware approximation and the largest distance of the refined value
 * from the IEEE quotient, in ulps.  No counterpart in the reference. */
int ec2d_check_reciprocal(long long n, double *approx_rel, double *refined_ulps);

/* Residual norms without any device allocation.  No counterpart in the
 * reference: it serves hosts that cannot call cudaMalloc (a Fortran/OpenACC
 * host whose device memory belongs to another allocator or memory pool, or a
 * host that must not allocate after start-up) and already hold a residual
 * array on the device.  res: device pointer to Res(nvar, ncell) (variable
 * fastest, e.g. the reference's Res(NVAR,1:nx-1,1:ny-1) of one block);
 * out: device pointer to 12 doubles, max|Res_m| for m=1..6 then sum Res_m^2
 * for m=1..6 (entries past nvar are 0); stream: a cudaStream_t or NULL.
 * The tile partials live in one file-scope __device__ array of 768 KiB per
 * GPU, so ncell is limited to EC2D_NOALLOC_MAX_CELLS (larger sizes return
 * EC2D_ERR_ARG).  All calls share that array: calls that overlap on the GPU
 * race.  The max is taken on the bit patterns of |Res|, so a NaN residual
 * gives a NaN max, as in ec2d_residual.  The array's device address is looked
 * up on every call made outside stream capture (a device reset therefore
 * leaves no stale address); a call during capture reuses the last address
 * found on that device, so make the first call on a device before any
 * capture. */
#define EC2D_NOALLOC_MAX_CELLS 2097152
int ec2d_residual_norms_noalloc(const double *res, int nvar, int ncell, double *out, void *stream);

/* CUDA graphs for ec2d_step.  No counterpart in the reference.  When enabled
 * (the default), the first ec2d_step records one pseudo-time step (single
 * grid or V-cycle) as a CUDA graph and every step replays it: one launch per
 * step instead of one per kernel, same kernels, same order, same results.
 * Steps with dual time stepping or with kernel timing enabled launch kernels
 * one by one.  enable = 0 switches to one-by-one launches. */
int ec2d_set_graphs(ec2d_ctx *ctx, int enable);

/* Precision of the LU-SGS sweeps (du_LU_SGS_2D) on every level: 64 (the
 * default, the reference's arithmetic) or 32.  No counterpart in the
 * reference.  With 32 the sweeps run in float from records built in FP64
 * (Res, 1/alfa, spectral radii and the state rounded to float, the flux
 * difference in increment form), and U stays FP64 (U += (double)dU); the
 * residual, boundary conditions, multigrid transfers, norms and forces stay
 * FP64, so the converged state is that of the FP64 discretisation. */
int ec2d_set_lusgs_precision(ec2d_ctx *ctx, int bits);

/* ---- Learned warm start (no counterpart in the reference) ----------------
 * A coordinate-conditioned MLP predicts the initial conservative (and SA)
 * field of a case -- its departure from the case's freestream, and
 * log1p(nu_tilde Re) -- from (x, y, log10 wall distance, M, AoA [deg],
 * log10 Re, shape) per cell, where `shape` is a per-case geometry parameter the host
 * supplies (the airfoil's t/c).  Training data are the fields of solved
 * cases; training and inference run in the library's own kernels (BF16
 * weights and activations, FP32 accumulation and Adam).  The freestream start
 * of ec2d_init_flow stays the fallback: a case whose predicted field has any
 * cell with rho <= 0, p <= 0 or T < 1e-5 keeps the freestream. */
typedef struct ec2d_mlp ec2d_mlp;
/* hidden_layers hidden layers of `width` (a multiple of 128) neurons */
int ec2d_mlp_create(int device, int hidden_layers, int width, unsigned long long seed, ec2d_mlp **out);
void ec2d_mlp_destroy(ec2d_mlp *m);
/* per-case shape feature (default 0); call any time after ec2d_setup */
int ec2d_set_case_shape(ec2d_ctx *ctx, int case_id, double shape);
/* append one sample per fine-mesh cell of every case of ctx (its current U) */
int ec2d_mlp_add_samples(ec2d_mlp *m, ec2d_ctx *ctx);
int ec2d_mlp_num_samples(ec2d_mlp *m, long long *n);
int ec2d_mlp_clear_samples(ec2d_mlp *m);
/* standardisation of features and targets from the current samples */
int ec2d_mlp_fit_normalization(ec2d_mlp *m);
/* `steps` Adam steps on minibatches of `batch` (a multiple of 256) random
 * samples; loss_out (may be NULL): the MSE of the last step (standardised) */
int ec2d_mlp_train(ec2d_mlp *m, int steps, int batch, double lr, double *loss_out);
/* predict the fine-mesh field of every case of ctx and write it into U
 * (interior cells, then the boundary conditions and halos); n_fallback: the
 * number of cases that kept the freestream */
int ec2d_mlp_warm_start(ec2d_mlp *m, ec2d_ctx *ctx, int *n_fallback);
/* test and persistence access: layer shapes, FP32 weights, gradients of the
 * last training step or of ec2d_mlp_loss_grad, predictions from host features */
int ec2d_mlp_num_layers(ec2d_mlp *m, int *nlin);
int ec2d_mlp_layer_shape(ec2d_mlp *m, int layer, int *rows, int *cols);
int ec2d_mlp_get_weights(ec2d_mlp *m, int layer, float *w, float *b);
int ec2d_mlp_set_weights(ec2d_mlp *m, int layer, const float *w, const float *b);
int ec2d_mlp_get_grads(ec2d_mlp *m, int layer, float *gw, float *gb);
int ec2d_mlp_get_normalization(ec2d_mlp *m, float *nrm);  /* 2*7 + 2*5 floats */
int ec2d_mlp_set_normalization(ec2d_mlp *m, const float *nrm);
/* loss and gradients for B standardised rows (x: B x 7, y: B x 5, B a multiple
 * of 256) */
int ec2d_mlp_loss_grad(ec2d_mlp *m, const float *x, const float *y, int B, double *loss);
/* GEMM path of the network: 1 = tcgen05 kernels (accumulators in tensor
 * memory; the default), 0 = mma.sync kernels.  A tcgen05 wait that times
 * out makes the call return EC2D_ERR_TIMEOUT. */
int ec2d_mlp_set_gemm(ec2d_mlp *m, int kind);
/* un-standardised predictions (n x 5) for raw features (n x 7), host arrays */
int ec2d_mlp_predict(ec2d_mlp *m, const float *feat, long long n, float *pred);

/* Autotuner.  No counterpart in the reference.  Times `trial_steps` steps of
 * every candidate launch configuration on the context's own cases and keeps
 * the fastest: the shape of the FP64 LU-SGS wavefront (lusgs_cs = 0: row
 * bands of at most rows_per_warp rows on the CTAs of a cluster, eight lanes
 * per row for bands of up to 16 rows and four for taller ones, where the
 * level has 4 variables, at most 8 bands and 1024 cells per row, else as 1;
 * 1: one CTA per block with rows_per_warp (32, 24 or 16) rows per warp; 2, 4,
 * 8: a thread-block cluster of that many CTAs with a barrier per plane) and
 * whether independent kernels run concurrently on two stream pairs (the i-
 * and j-face flux kernels; at a multigrid transfer the fine residual and the
 * restriction + coarse boundary conditions + coarse entry residual).
 * The fine-mesh U, the step counters and every case's status word (with
 * dual time stepping also the two physical time levels and the first-step
 * flags) are restored afterwards; other scratch of the steps (residuals, coarse levels, the
 * coarse forcing) is formed anew before the next step or ec2d_init_flow
 * reads it.  Outputs
 * (may be NULL): the choices and the winner's milliseconds per step.  The
 * default shape, before any autotune, is 0 with 12-row bands; the
 * environment variables EC2D_LUSGS_CLUSTER and EC2D_LUSGS_ROWS read by
 * ec2d_create override it. */
int ec2d_autotune(ec2d_ctx *ctx, int trial_steps, int *lusgs_cs, int *rows_per_warp, int *concurrent,
                  double *ms_per_step);
/* The FP64 wavefront's shape in use: lusgs_cs and rows as above, and the
 * lanes per row of the banded kernel (8 or 4; the autotuner also tries bands
 * of 6 and 8 rows with either, on clusters of up to 16 CTAs, and
 * EC2D_LUSGS_LANES read by ec2d_create fixes the lanes).  No counterpart in
 * the reference. */
int ec2d_lusgs_shape(ec2d_ctx *ctx, int *lusgs_cs, int *rows, int *lanes);

/* The residual of a level as one kernel over 2-D tiles of cells whose
 * primitives and halo sit in shared memory (enable = 1; used on levels with
 * no turbulence model and no finite-difference patch that compute in FP64),
 * or as the chain of four kernels through HBM planes (0, the default); -1
 * only reads the setting into *current (may be NULL).  No counterpart in the
 * reference; both forms evaluate Residual_FVM (sub_Residual.f90:200-472),
 * comput_Lvc and comput_dt with the same face arithmetic.  ec2d_autotune
 * picks the faster; EC2D_TILE_RESIDUAL=1 read by ec2d_create starts with the
 * one-kernel form. */
int ec2d_tile_residual(ec2d_ctx *ctx, int enable, int *current);

/* The launch choices ec2d_autotune makes, read and set directly, so that a
 * host can keep the winners of one autotune and reuse them in later runs of
 * the same cases without timing the candidates again.  No counterpart in the
 * reference.  lusgs_cs and rows as in ec2d_autotune, lanes 4 or 8 (0: by the
 * band height, eight up to 16 rows), concurrent and tile_residual 0 or 1
 * (see ec2d_autotune and ec2d_tile_residual).  ec2d_set_launch_config takes
 * the ranges the EC2D_LUSGS_* variables take (lusgs_cs 0..8, rows 4..32);
 * where a level cannot take a wavefront shape the launcher falls back to one
 * it can, as it does for any shape.  None of the choices changes the
 * discretisation: the wavefront shape changes only the summation order of
 * the sweep's records, the other two nothing.  Setting drops the captured
 * step graph; the next ec2d_step captures the new launches.  Outputs of
 * ec2d_launch_config may be NULL. */
int ec2d_launch_config(ec2d_ctx *ctx, int *lusgs_cs, int *rows, int *lanes, int *concurrent, int *tile_residual);
int ec2d_set_launch_config(ec2d_ctx *ctx, int lusgs_cs, int rows, int lanes, int concurrent, int tile_residual);
/* A one-line description of everything the launch choices depend on, after
 * ec2d_setup: the library version and a digest of its sources, the device
 * (name, compute capability, SM count), the method flags, the LU-SGS and
 * coarse precisions, the coarse eddy-viscosity option, the number of cases,
 * and per multigrid level the variables and every block shape in cells with
 * its count.  Contexts with equal signatures time their candidates alike, so
 * a host keys its cache of ec2d_autotune results by it (ec2d/tuning.py keeps
 * one as a JSON file).  No counterpart in the reference.  *needed (may be
 * NULL) receives the length including the terminating NUL; buf = NULL only
 * queries it; a buf shorter than that returns EC2D_ERR_ARG. */
int ec2d_launch_signature(ec2d_ctx *ctx, char *buf, int len, int *needed);

/* Multigrid with a turbulence model: the coarse levels keep an eddy
 * viscosity restricted from the next finer level (enable = 1; the mean of a
 * coarse cell's children over 0..nx, 0..ny, taken after the finer level's
 * residual, frozen on the coarse level), or are laminar as in the reference
 * (0, the default: Comput_Residual_one_mesh zeroes Amu_t and the coarse
 * levels run no turbulence model, sub_Residual.f90:158-191,
 * opencfd_ec2d_v1.5.4.f90:252-259).  -1 only reads the setting into *current
 * (may be NULL).  The coarse problem changes, its fixed point (the fine
 * discretisation) does not: the option is for stability.  With laminar
 * coarse levels the LU-SGS-smoothed cycle diverges from developed turbulent
 * fields (the oracle likewise), where the frozen eddy viscosity keeps the
 * coarse corrections damped. */
int ec2d_mg_eddy_viscosity(ec2d_ctx *ctx, int enable, int *current);

/* Precision of the face fluxes (reconstruction, Riemann solver, viscous
 * stress) on the coarse multigrid levels: 64 (the default) or 32.  No
 * counterpart in the reference.  The coarse levels only smooth the
 * fine-level correction and their forcing is formed from the same FP32
 * residual, so early convergence follows the FP64 run; the FP32 rounding
 * the forcing carries limits the attainable drop to about 1e-7 of the first
 * residual (measured on the flat plate), so deep convergence wants 64. */
int ec2d_set_coarse_precision(ec2d_ctx *ctx, int bits);

/* Wait for all queued work of the context. */
int ec2d_sync(ec2d_ctx *ctx);

#ifdef __cplusplus
}
#endif
#endif
