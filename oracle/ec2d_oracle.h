/*
 * ec2d_oracle.h -- C API of the CPU oracle (TEST INFRASTRUCTURE ONLY).
 *
 * The oracle is a plain C++ restatement of the OpenCFD-EC2D v1.5.4 Fortran
 * pseudo-time-marching core.  It exists only to check the GPU library: only
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it.
 * The product library (libec2d_gpu.so) never links or calls it.
 *
 * Parity status: UNPINNED by the reference.  The reference ships no tests, no
 * golden vectors and no outputs, and it is Fortran while no Fortran compiler
 * is available here, so the restatement cannot be run against the reference
 * itself.  It is checked instead by known-answer properties derived from the
 * code and from mathematics (flux consistency, freestream preservation,
 * conservation of restriction, symmetry), see tests/test_oracle_*.py.
 *
 * Array layouts at this boundary follow the reference's Fortran arrays
 * (column-major, variable index fastest), e.g. U(NVAR,-1:nx+1,-1:ny+1).
 */
#ifndef EC2D_ORACLE_H
#define EC2D_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

/* Same fields and meaning as control.in lines 2,4,6,8,10 and 12
 * (opencfd_ec2d_v1.5.4.f90:201-211).  AoA in degrees, Twall in K. */
typedef struct orc_params {
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
  double xaxis, yaxis; /* moment reference point (control.in line 12) */
  int mg_lusgs;        /* 1: allow LU-SGS smoothing inside multigrid (extension) */
} orc_params;

void *orc_new(const orc_params *p);
void orc_free(void *h);
int orc_add_block(void *h, int nx, int ny, const double *x, const double *y,
                  int nsub, const int *bc9);
int orc_set_fdm_block(void *h, int block); /* 1-based block id, as in FDM.in */
int orc_set_dw(void *h, int block, const double *dw); /* dist_wall.dat, (1:nx-1,1:ny-1) */
int orc_setup(void *h);
int orc_num_mesh(void *h);
int orc_nvar(void *h, int mesh);
int orc_block_dims(void *h, int mesh, int block, int *nx, int *ny);
int orc_init_flow(void *h);
int orc_dual_time_start(void *h); /* Un = Un1 = U on mesh 1, first-step flags unset */
int orc_get_U(void *h, int mesh, int block, double *U);
int orc_set_U(void *h, int mesh, int block, const double *U);
int orc_get_field(void *h, int mesh, int block, int field, double *out);
int orc_field_size(void *h, int mesh, int block, int field);
int orc_residual(void *h, int mesh);
int orc_bc(void *h, int mesh);
int orc_halo(void *h, int mesh);
int orc_lusgs(void *h, int mesh, int block, double alfa1);
int orc_time_advance(void *h, int mesh);
int orc_step(void *h, int nsteps);
int orc_norms(void *h, int mesh, double *res_max6, double *res_rms6, int *kstep, double *tt);
int orc_interpolation2h(void *h, int m1, int m2, int flag);
int orc_prolong(void *h, int m1, int m2, int flag);
int orc_force_function(void *h, int mesh);
int orc_set_un(void *h, int mesh);
int orc_delt_u(void *h, int mesh);
int orc_new_u(void *h, int mesh);
int orc_forces(void *h, double *cl, double *cd, double *cm);
int orc_wall_cf(void *h, int block, int sub, double *cf, double *xc, int maxn);
int orc_last_error(void *h, int *blk, int *i, int *j);
/* extension: coarse levels take the eddy viscosity restricted from the
 * next finer level (the reference's coarse levels are laminar) */
int orc_set_mg_amut(void *h, int enable);
void orc_set_threads(int n);
/* known-answer hooks: one face flux (sub_flux_split.f90) and one limiter
 * evaluation (scheme_fP side=0 / scheme_fm side=1, sub_Residual.f90:591-659) */
int orc_flux(int iflux, const double *QL, const double *QR, double *F, double gamma);
double orc_scheme(int side, double u1, double u2, double u3, double u4, int flag);
int orc_set_field(void *h, int mesh, int block, int field, const double *in);

/* Field ids for orc_get_field (shared numbering with the GPU library). */
enum {
  ORC_F_RES = 0, ORC_F_DT = 1, ORC_F_LCI = 2, ORC_F_LCJ = 3, ORC_F_LVI = 4,
  ORC_F_LVJ = 5, ORC_F_DU = 6, ORC_F_AMU = 7, ORC_F_AMUT = 8, ORC_F_X1 = 9,
  ORC_F_Y1 = 10, ORC_F_VOL = 11, ORC_F_SI = 12, ORC_F_SJ = 13, ORC_F_NI1 = 14,
  ORC_F_NI2 = 15, ORC_F_NJ1 = 16, ORC_F_NJ2 = 17, ORC_F_DW = 18, ORC_F_QF = 19,
  ORC_F_DELTU = 20, ORC_F_UN = 21, ORC_F_X = 22, ORC_F_Y = 23
};

#ifdef __cplusplus
}
#endif
#endif
