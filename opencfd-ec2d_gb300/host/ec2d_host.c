/*
 * ec2d_host.c -- a C replica of the OpenCFD-EC2D driver over the C-ABI of
 * libec2d_gpu.so: the host a Fortran build would be, for machines without a
 * Fortran compiler.
 *
 * It follows `program main` (opencfd_ec2d_v1.5.4.f90:142-186): read
 * control.in (read_parameter, :197-235), Mesh2d.dat and bc2d_1.in
 * (Creat_Mesh1 + read_bcin, sub_init.f90:111-251) and, when present, FDM.in
 * (Init_FiniteDifference, sub_Finite_Difference.f90:278-311); hand them to
 * the library; then the main loop
 *
 *     do while (tt < t_end)
 *       NS_Time_advance(1) / NS_2stge_multigrid / NS_3stge_multigrid
 *       if (mod(Kstep, Kstep_show) == 0) call output_Res(1)
 *
 * with the step body replaced by ec2d_step, output_Res writing the same
 * Residual.dat record, format (I8,13E24.10) (opencfd_ec2d_v1.5.4.f90:266-279),
 * and output(1) the same flow2d*.dat / SA2d.dat / SST2d.dat files every
 * Kstep_save steps and at the end (:182-186, :284-371).
 * The input files are read in the reference's formats, unchanged.
 *
 *   ec2d_host [case_dir] [--steps N] [--device D] [--fix-nvar-restart]
 *
 * --steps N stops after N steps (the reference stops only on tt >= t_end).
 * SA and SST runs take the wall distance from dist_wall.dat when the case
 * has one, else write it (and dw.dat) from the distances formed on the
 * device, as comput_dw does (sub_turbulence_SST.f90:274-365).
 * Iflag_init = 1 in control.in restarts from flow2d.dat (and SA2d.dat /
 * SST2d.dat) as init_flow_read does (sub_init.f90:499-560); the reference
 * reads the turbulence files under NVAR == 5 for both models (:523, :541),
 * which --fix-nvar-restart corrects (SST2d.dat for NVAR == 6), and without
 * which an SA restart stops with a message where the reference would read
 * SST2d.dat into a 5-variable state.
 * At the end it prints the last step's residual norms and CL, CD, CM.
 * Exit status: 0, or the EC2D_ERR_* code of the failing call (a T < 1e-5
 * state prints the reference's message and stops, as sub_Residual.f90:143-146
 * does).
 */
#include <ctype.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "ec2d_gpu.h"

#define MAXB 64
#define MAXLINE 4096

typedef struct {
  int nx, ny, nsub;
  double *x, *y; /* x(1:nx,1:ny), column-major */
  int *bc9;      /* nsub x 9 */
} host_block;

static char *path_in(const char *dir, const char *name) {
  static char buf[4096];
  snprintf(buf, sizeof(buf), "%s/%s", dir, name);
  return buf;
}

/* Fortran list-directed reals accept d/D exponents */
static double fnum(const char *tok) {
  char t[128];
  size_t n = strlen(tok);
  if (n >= sizeof(t)) n = sizeof(t) - 1;
  for (size_t k = 0; k < n; k++) t[k] = (tok[k] == 'd' || tok[k] == 'D') ? 'e' : tok[k];
  t[n] = 0;
  return strtod(t, NULL);
}

/* the whitespace-separated tokens of one line */
static int split(char *line, char **tok, int maxtok) {
  int n = 0;
  char *s = line;
  while (*s && n < maxtok) {
    while (*s && (isspace((unsigned char)*s) || *s == ',')) s++;
    if (!*s) break;
    tok[n++] = s;
    while (*s && !isspace((unsigned char)*s) && *s != ',') s++;
    if (*s) *s++ = 0;
  }
  return n;
}

static int read_lines(const char *path, char lines[][MAXLINE], int maxl) {
  FILE *f = fopen(path, "r");
  if (!f) return -1;
  int n = 0;
  while (n < maxl && fgets(lines[n], MAXLINE, f)) n++;
  fclose(f);
  return n;
}

/* read_parameter: the data lines 2, 4, 6, 8, 10 (and 12: moment point) */
static int read_control(const char *dir, ec2d_params *p) {
  static char L[16][MAXLINE];
  char *t[32];
  int n = read_lines(path_in(dir, "control.in"), L, 16);
  if (n < 10) return -1;
  memset(p, 0, sizeof(*p));
  if (split(L[1], t, 32) < 10) return -1;
  p->Ma = fnum(t[0]); p->Re = fnum(t[1]); p->gamma = fnum(t[2]); p->AoA = fnum(t[3]);
  p->Pr = fnum(t[4]); p->t_end = fnum(t[5]);
  p->Kstep_save = (int)fnum(t[6]); p->If_viscous = (int)fnum(t[7]);
  p->Iflag_turbulence_model = (int)fnum(t[8]); p->Iflag_init = (int)fnum(t[9]);
  if (split(L[3], t, 32) < 12) return -1;
  p->Iflag_local_dt = (int)fnum(t[0]); p->dt_global = fnum(t[1]); p->CFL = fnum(t[2]);
  p->dtmax = fnum(t[3]); p->dtmin = fnum(t[4]); p->Time_Method = (int)fnum(t[5]);
  p->P_outlet = fnum(t[6]); p->T_inf = fnum(t[7]); p->Twall = fnum(t[8]);
  p->vt_inf = fnum(t[9]); p->Kt_inf = fnum(t[10]); p->Wt_inf = fnum(t[11]);
  if (split(L[5], t, 32) < 4) return -1;
  p->Iflag_Scheme = (int)fnum(t[0]); p->Iflag_flux = (int)fnum(t[1]);
  p->IFlag_Reconstruction = (int)fnum(t[2]); p->Kstep_show = (int)fnum(t[3]);
  if (split(L[7], t, 32) < 4) return -1;
  p->Num_Mesh = (int)fnum(t[0]); p->Num_Threads = (int)fnum(t[1]);
  p->Nstep_Inner_Limit = (int)fnum(t[2]); p->Res_Inner_Limit = fnum(t[3]);
  int k = split(L[9], t, 32);
  for (int m = 0; m < 3; m++) p->Pre_Step_Mesh[m] = (m < k && m < p->Num_Mesh) ? (int)fnum(t[m]) : 0;
  p->xaxis = 0.25;
  p->yaxis = 0.0;
  if (n > 11 && split(L[11], t, 32) >= 2 && (isdigit((unsigned char)t[0][0]) || t[0][0] == '-' || t[0][0] == '.')) {
    p->xaxis = fnum(t[0]);
    p->yaxis = fnum(t[1]);
  }
  /* multigrid levels are smoothed by LU-SGS when the time method is LU-SGS
   * (the reference refuses that combination, opencfd_ec2d_v1.5.4.f90:216-221) */
  p->mg_lusgs = 1;
  if (p->Kstep_show < 1) p->Kstep_show = 1;
  return 0;
}

/* Mesh2d.dat: number of blocks, (nx, ny) per block, then per block x(:,:)
 * and y(:,:) in Fortran order (sub_init.f90:121-127,176) */
static int read_mesh(const char *dir, host_block *B, int *nb) {
  FILE *f = fopen(path_in(dir, "Mesh2d.dat"), "r");
  if (!f) return -1;
  char tok[128];
  if (fscanf(f, "%127s", tok) != 1) { fclose(f); return -1; }
  *nb = (int)fnum(tok);
  if (*nb < 1 || *nb > MAXB) { fclose(f); return -1; }
  for (int m = 0; m < *nb; m++) {
    if (fscanf(f, "%127s", tok) != 1) { fclose(f); return -1; }
    B[m].nx = (int)fnum(tok);
    if (fscanf(f, "%127s", tok) != 1) { fclose(f); return -1; }
    B[m].ny = (int)fnum(tok);
  }
  for (int m = 0; m < *nb; m++) {
    size_t n = (size_t)B[m].nx * B[m].ny;
    B[m].x = (double *)malloc(n * sizeof(double));
    B[m].y = (double *)malloc(n * sizeof(double));
    for (int a = 0; a < 2; a++) {
      double *v = a ? B[m].y : B[m].x;
      for (size_t k = 0; k < n; k++) {
        if (fscanf(f, "%127s", tok) != 1) { fclose(f); return -1; }
        v[k] = fnum(tok);
      }
    }
  }
  fclose(f);
  return 0;
}

/* bc2d_1.in: title, "# Blocks", count; per block "Block n", "Subface",
 * count, a header line and one 9-integer row per subface (sub_init.f90:228-248) */
static int read_bc(const char *dir, host_block *B, int nb) {
  static char L[4096][MAXLINE];
  char *t[32];
  int n = read_lines(path_in(dir, "bc2d_1.in"), L, 4096);
  if (n < 3) return -1;
  int k = 2;
  if (split(L[k++], t, 32) < 1 || (int)fnum(t[0]) != nb) {
    fprintf(stderr, "Block number in bc2d.in is not equal to that in Mesh2d.dat\n");
    return -1;
  }
  for (int m = 0; m < nb; m++) {
    k += 2;
    if (k >= n || split(L[k++], t, 32) < 1) return -1;
    B[m].nsub = (int)fnum(t[0]);
    k++;
    B[m].bc9 = (int *)malloc((size_t)B[m].nsub * 9 * sizeof(int));
    for (int s = 0; s < B[m].nsub; s++) {
      if (k >= n || split(L[k++], t, 32) < 9) return -1;
      for (int q = 0; q < 9; q++) B[m].bc9[s * 9 + q] = (int)fnum(t[q]);
    }
  }
  return 0;
}

/* FDM.in: four comment lines, the block count, one more line, then one
 * block number per line (sub_Finite_Difference.f90:287-308) */
static int read_fdm(const char *dir, int *ids, int nb) {
  static char L[MAXB + 16][MAXLINE];
  char *t[8];
  int n = read_lines(path_in(dir, "FDM.in"), L, MAXB + 16);
  if (n < 0) return 0;
  if (n < 5 || split(L[4], t, 8) < 1) return 0;
  int cnt = (int)fnum(t[0]), got = 0;
  for (int k = 0; k < cnt && 6 + k < n; k++) {
    if (split(L[6 + k], t, 8) < 1) continue;
    int md = (int)fnum(t[0]);
    if (md > nb || md < 1) fprintf(stderr, "error in 'FDM.in'\n");
    else ids[got++] = md;
  }
  return got;
}

/* Fortran E24.10: 0.dddddddddddE+xx right-justified in 24 columns */
static void e24(FILE *f, double v) {
  char m[64], out[64];
  if (v == 0.0) { fprintf(f, "%24s", "0.0000000000E+00"); return; }
  snprintf(m, sizeof(m), "%.9e", v < 0 ? -v : v); /* d.ddddddddde+xx */
  char *e = strchr(m, 'e');
  int ex = atoi(e + 1) + 1;
  char digits[16];
  digits[0] = m[0];
  memcpy(digits + 1, m + 2, 9);
  digits[10] = 0;
  snprintf(out, sizeof(out), "%s0.%sE%c%02d", v < 0 ? "-" : "", digits, ex < 0 ? '-' : '+', ex < 0 ? -ex : ex);
  fprintf(f, "%24s", out);
}

static int fail(const char *what, int r);

/* dist_wall.dat as comput_dw reads it (sub_turbulence_SST.f90:295-306): the
 * block count, the (nx, ny) of every block, then each block's cell distances
 * dw(1:nx-1,1:ny-1), i fastest, as list-directed values (r*c repeats
 * included).  dw[m] receives (nx-1)(ny-1) values (malloc'ed).  0: read;
 * 1: absent; -1: unreadable or written for another mesh. */
static int read_dist_wall(const char *path, const host_block *B, int nb, double **dw) {
  FILE *f = fopen(path, "r");
  if (!f) return 1;
  char tok[128];
  double rep_val = 0.0;
  long rep = 0;
  int bad = 0;
  /* the next value of the stream, with r*c repeats expanded */
#define NEXT(out)                                                     \
  do {                                                                \
    if (rep > 0) { rep--; (out) = rep_val; break; }                   \
    if (fscanf(f, " %127[^ \t\r\n,]%*[ \t\r\n,]", tok) < 1) { bad = 1; (out) = 0; break; } \
    char *star = strchr(tok, '*');                                    \
    if (star) { *star = 0; rep = atol(tok) - 1; rep_val = fnum(star + 1); (out) = rep_val; } \
    else (out) = fnum(tok);                                           \
  } while (0)
  double v;
  NEXT(v);
  if (bad || (int)v != nb) bad = 1;
  for (int m = 0; m < nb && !bad; m++) {
    double a, b;
    NEXT(a);
    NEXT(b);
    if ((int)a != B[m].nx || (int)b != B[m].ny) bad = 1;
  }
  for (int m = 0; m < nb && !bad; m++) {
    size_t n = (size_t)(B[m].nx - 1) * (B[m].ny - 1);
    dw[m] = (double *)malloc(n * sizeof(double));
    if (!dw[m]) { bad = 1; break; }
    for (size_t k = 0; k < n && !bad; k++) NEXT(dw[m][k]);
  }
#undef NEXT
  fclose(f);
  return bad ? -1 : 0;
}

/* dist_wall.dat and dw.dat (sub_turbulence_SST.f90:342-362) from the
 * distances formed on the device, every value with 17 significant digits
 * as list-directed output writes a double (it reads back to the same one). */
static int write_dist_wall(const char *dir, ec2d_ctx *ctx, int cs, const host_block *B, int nb) {
  char path[4096], path2[4096];
  snprintf(path, sizeof(path), "%s/dist_wall.dat", dir);
  snprintf(path2, sizeof(path2), "%s/dw.dat", dir);
  FILE *f = fopen(path, "w"), *g = fopen(path2, "w");
  int r = 0;
  if (!f || !g) { if (f) fclose(f); if (g) fclose(g); return 1; }
  fprintf(f, " %d\n", nb);
  for (int m = 0; m < nb; m++) fprintf(f, " %d %d", B[m].nx, B[m].ny);
  fprintf(f, "\n");
  fprintf(g, " variables=x,y,dw\n");
  for (int m = 0; m < nb && !r; m++) {
    const int nx = B[m].nx, ny = B[m].ny;
    /* DW (0:nx,0:ny); X1, Y1 (-1:nx+1,-1:ny+1) */
    double *dw = (double *)malloc((size_t)(nx + 1) * (ny + 1) * sizeof(double));
    double *x1 = (double *)malloc((size_t)(nx + 3) * (ny + 3) * sizeof(double));
    double *y1 = (double *)malloc((size_t)(nx + 3) * (ny + 3) * sizeof(double));
    if (!dw || !x1 || !y1) r = EC2D_ERR_NOMEM;
    if (!r) r = ec2d_get_field(ctx, cs, 1, m + 1, EC2D_F_DW, dw);
    if (!r) r = ec2d_get_field(ctx, cs, 1, m + 1, EC2D_F_X1, x1);
    if (!r) r = ec2d_get_field(ctx, cs, 1, m + 1, EC2D_F_Y1, y1);
    if (!r) {
      int col = 0;
      fprintf(g, " zone i= %d j= %d\n", nx - 1, ny - 1);
      for (int j = 1; j <= ny - 1; j++)
        for (int i = 1; i <= nx - 1; i++) {
          const double d = dw[(size_t)j * (nx + 1) + i];
          const size_t c = (size_t)(j + 1) * (nx + 3) + (i + 1);
          fprintf(f, " %.17g", d);
          if (++col % 4 == 0) fprintf(f, "\n");
          fprintf(g, " %.17g %.17g %.17g\n", x1[c], y1[c], d);
        }
      if (col % 4) fprintf(f, "\n");
    }
    free(dw); free(x1); free(y1);
  }
  fclose(f);
  fclose(g);
  return r;
}

/* One Tecplot file of `output` (flow2d.dat: x, y, d, u, v, T; SA2d.dat: x, y,
 * nu~; SST2d.dat: x, y, k, omega): a title line, then per block a zone line
 * and (nx+1)(ny+1) records over i = 0..nx fastest, j = 0..ny, as
 * init_flow_read reads them with list-directed reads.  Returns per block the
 * `ncol` columns of every record in `cols[m]` (malloc'ed), or -1. */
static int read_zones(const char *path, const host_block *B, int nb, int ncol, double **cols) {
  FILE *f = fopen(path, "r");
  if (!f) return -1;
  static char line[MAXLINE];
  int ok = fgets(line, sizeof(line), f) != NULL;
  for (int m = 0; m < nb && ok; m++) {
    size_t n = (size_t)(B[m].nx + 1) * (B[m].ny + 1);
    cols[m] = (double *)malloc(n * ncol * sizeof(double));
    if (!cols[m] || !fgets(line, sizeof(line), f)) { ok = 0; break; }
    for (size_t k = 0; k < n && ok; k++) {
      if (!fgets(line, sizeof(line), f)) { ok = 0; break; }
      char *t[8];
      if (split(line, t, 8) < ncol) { ok = 0; break; }
      for (int c = 0; c < ncol; c++) cols[m][k * ncol + c] = fnum(t[c]);
    }
  }
  fclose(f);
  return ok ? 0 : -1;
}

/* init_flow_read (sub_init.f90:499-560) over the library: the freestream start
 * (which leaves the ghost ring and the variables the files do not hold at the
 * freestream), each block's 0..nx x 0..ny from the files, then the boundary
 * conditions and the halo on the fine mesh, and with dual time stepping the
 * physical-time history started from the restart state. */
static int restart(const char *dir, ec2d_ctx *ctx, int cs, const ec2d_params *P, const host_block *B, int nb,
                   int nvar, int fix_nvar) {
  double *flow[MAXB] = {0}, *turb[MAXB] = {0};
  const char *tname = NULL;
  int tcol = 0, r = 1;
  if (nvar == 5) { tname = "SA2d.dat"; tcol = 3; }
  if (nvar == 6 && fix_nvar) { tname = "SST2d.dat"; tcol = 4; }
  if (nvar == 5 && !fix_nvar) {
    fprintf(stderr, "restart: sub_init.f90:541 reads SST2d.dat into U(5:6) of a 5-variable (SA) state as well; "
                    "run with --fix-nvar-restart\n");
    return 1;
  }
  if (read_zones(path_in(dir, "flow2d.dat"), B, nb, 6, flow)) {
    fprintf(stderr, "cannot read %s\n", path_in(dir, "flow2d.dat"));
    goto done;
  }
  if (tname && read_zones(path_in(dir, tname), B, nb, tcol, turb)) {
    fprintf(stderr, "cannot read %s\n", path_in(dir, tname));
    goto done;
  }
  if ((r = ec2d_init_flow(ctx))) { fail("ec2d_init_flow", r); goto done; }
  const double Cv = 1.0 / (P->gamma * (P->gamma - 1.0) * P->Ma * P->Ma);
  for (int m = 0; m < nb; m++) {
    const int nx = B[m].nx, ny = B[m].ny, W = nx + 3;
    double *U = (double *)malloc((size_t)nvar * W * (ny + 3) * sizeof(double));
    if (!U) { r = EC2D_ERR_NOMEM; goto done; }
    if ((r = ec2d_download_U(ctx, cs, 1, m + 1, U))) { free(U); fail("ec2d_download_U", r); goto done; }
    for (int j = 0; j <= ny; j++)
      for (int i = 0; i <= nx; i++) {
        const double *q = flow[m] + ((size_t)j * (nx + 1) + i) * 6;
        const double d0 = q[2], u0 = q[3], v0 = q[4], T0 = q[5];
        double *u = U + (size_t)nvar * ((size_t)(j + 1) * W + (i + 1)); /* U(NVAR,-1:nx+1,-1:ny+1) */
        u[0] = d0;
        u[1] = d0 * u0;
        u[2] = d0 * v0;
        u[3] = d0 * Cv * T0 + 0.5 * d0 * (u0 * u0 + v0 * v0);
        if (turb[m]) {
          const double *w = turb[m] + ((size_t)j * (nx + 1) + i) * tcol;
          for (int c = 2; c < tcol; c++) u[4 + c - 2] = w[c];
        }
      }
    r = ec2d_upload_U(ctx, cs, 1, m + 1, U);
    free(U);
    if (r) { fail("ec2d_upload_U", r); goto done; }
  }
  if ((r = ec2d_boundary_condition(ctx, 1)) || (r = ec2d_update_buffer(ctx, 1)) || (r = ec2d_dual_time_start(ctx)))
    fail("restart", r);
done:
  for (int m = 0; m < nb; m++) { free(flow[m]); free(turb[m]); }
  return r;
}

/* One zone of an `output` file: the header line, then per cell of
 * i = 0..nx (fastest), j = 0..ny the columns in F20.10 */
static void zone(FILE *f, int nx, int ny, const double *const *cols, int ncol) {
  fprintf(f, "  zone i= %11d j= %11d\n", nx + 1, ny + 1);
  for (int j = 0; j <= ny; j++)
    for (int i = 0; i <= nx; i++) {
      const size_t c = (size_t)(j + 1) * (nx + 3) + (i + 1); /* (-1:nx+1,-1:ny+1) */
      for (int k = 0; k < ncol; k++) fprintf(f, "%20.10f", cols[k][c]);
      fprintf(f, "\n");
    }
}

/* output(1) (opencfd_ec2d_v1.5.4.f90:284-371): flow2d-<Kstep>.dat (x, y, d,
 * u, v, T, p), flow2d.dat (the same and Amut Re) and SA2d.dat (x, y, nu~) or
 * SST2d.dat (x, y, k, omega), every block over 0..nx x 0..ny, read from the
 * device with ec2d_download_U and ec2d_get_field */
static int output(const char *dir, ec2d_ctx *ctx, int cs, const ec2d_params *P, const host_block *B, int nb,
                  int nvar, int kstep) {
  char p1[4096], p2[4096], p3[4096];
  snprintf(p1, sizeof(p1), "%s/flow2d-%07d.dat", dir, kstep);
  snprintf(p2, sizeof(p2), "%s/flow2d.dat", dir);
  snprintf(p3, sizeof(p3), "%s/%s", dir, nvar == 5 ? "SA2d.dat" : "SST2d.dat");
  FILE *f1 = fopen(p1, "w"), *f2 = fopen(p2, "w"), *f3 = nvar >= 5 ? fopen(p3, "w") : NULL;
  int r = (!f1 || !f2 || (nvar >= 5 && !f3)) ? 1 : 0;
  if (!r) {
    fprintf(f1, " variables=x,y,d,u,v,T,p\n");
    fprintf(f2, " variables=x,y,d,u,v,T,p,Amut\n");
    if (f3) fprintf(f3, nvar == 5 ? " variables=x,y,vt\n" : " variables=x,y,Kt,Wt\n");
  }
  const double gamma = P->gamma, Ma = P->Ma, Cv = 1.0 / (gamma * (gamma - 1.0) * Ma * Ma);
  for (int m = 0; m < nb && !r; m++) {
    const int nx = B[m].nx, ny = B[m].ny;
    const size_t n = (size_t)(nx + 3) * (ny + 3);
    double *U = (double *)malloc(nvar * n * sizeof(double)), *w = (double *)malloc(8 * n * sizeof(double));
    if (!U || !w) r = EC2D_ERR_NOMEM;
    double *x1 = w, *y1 = w + n, *d = w + 2 * n, *u = w + 3 * n, *v = w + 4 * n, *T = w + 5 * n, *pp = w + 6 * n,
           *amut = w + 7 * n;
    if (!r) r = ec2d_download_U(ctx, cs, 1, m + 1, U);
    if (!r) r = ec2d_get_field(ctx, cs, 1, m + 1, EC2D_F_X1, x1);
    if (!r) r = ec2d_get_field(ctx, cs, 1, m + 1, EC2D_F_Y1, y1);
    if (!r) r = ec2d_get_field(ctx, cs, 1, m + 1, EC2D_F_AMUT, amut);
    if (!r) {
      for (size_t k = 0; k < n; k++) {
        const double *q = U + (size_t)nvar * k; /* U(NVAR,-1:nx+1,-1:ny+1) */
        d[k] = q[0];
        u[k] = q[1] / d[k];
        v[k] = q[2] / d[k];
        T[k] = (q[3] - 0.5 * d[k] * (u[k] * u[k] + v[k] * v[k])) / (Cv * d[k]);
        pp[k] = d[k] * T[k] / (gamma * Ma * Ma);
        amut[k] = amut[k] * P->Re;
      }
      const double *c7[8] = {x1, y1, d, u, v, T, pp, amut};
      zone(f1, nx, ny, c7, 7);
      zone(f2, nx, ny, c7, 8);
      if (f3) {
        /* the turbulence variables, gathered into the free columns */
        for (size_t k = 0; k < n; k++) {
          d[k] = U[(size_t)nvar * k + 4];
          if (nvar == 6) u[k] = U[(size_t)nvar * k + 5];
        }
        const double *ct[4] = {x1, y1, d, u};
        zone(f3, nx, ny, ct, nvar == 5 ? 3 : 4);
      }
    }
    free(U);
    free(w);
  }
  if (f1) fclose(f1);
  if (f2) fclose(f2);
  if (f3) fclose(f3);
  return r;
}

static int fail(const char *what, int r) {
  fprintf(stderr, "%s: %s (%d)\n", what, ec2d_error_string(r), r);
  return r;
}

int main(int argc, char **argv) {
  const char *dir = ".";
  long max_steps = -1;
  int device = 0, fix_nvar = 0;
  for (int a = 1; a < argc; a++) {
    if (!strcmp(argv[a], "--steps") && a + 1 < argc) max_steps = atol(argv[++a]);
    else if (!strcmp(argv[a], "--device") && a + 1 < argc) device = atoi(argv[++a]);
    else if (!strcmp(argv[a], "--fix-nvar-restart")) fix_nvar = 1;
    else dir = argv[a];
  }
  ec2d_params P;
  if (read_control(dir, &P)) { fprintf(stderr, "cannot read %s\n", path_in(dir, "control.in")); return 1; }
  static host_block B[MAXB];
  int nb = 0;
  if (read_mesh(dir, B, &nb)) { fprintf(stderr, "cannot read %s\n", path_in(dir, "Mesh2d.dat")); return 1; }
  if (read_bc(dir, B, nb)) { fprintf(stderr, "cannot read %s\n", path_in(dir, "bc2d_1.in")); return 1; }
  int fdm[MAXB], nfdm = read_fdm(dir, fdm, nb);
  int nvar = P.Iflag_turbulence_model == 3 ? 6 : P.Iflag_turbulence_model == 2 ? 5 : 4;

  ec2d_ctx *ctx = NULL;
  int r, cs = 0;
  if ((r = ec2d_create(device, &ctx))) return fail("ec2d_create", r);
  if ((r = ec2d_add_case(ctx, &P, &cs))) return fail("ec2d_add_case", r);
  for (int m = 0; m < nb; m++)
    if ((r = ec2d_add_block(ctx, cs, B[m].nx, B[m].ny, B[m].x, B[m].y, B[m].nsub, B[m].bc9)))
      return fail("ec2d_add_block", r);
  for (int k = 0; k < nfdm; k++)
    if ((r = ec2d_set_fdm_block(ctx, cs, fdm[k]))) return fail("ec2d_set_fdm_block", r);
  /* comput_dw for SA and SST (opencfd_ec2d_v1.5.4.f90:164): dist_wall.dat
   * when the case has one, else the distances formed on the device, written
   * to dist_wall.dat and dw.dat after the set-up */
  const int turbulent = P.Iflag_turbulence_model == 2 || P.Iflag_turbulence_model == 3;
  int have_dw = 0;
  if (turbulent) {
    double *dw[MAXB] = {0};
    int rd = read_dist_wall(path_in(dir, "dist_wall.dat"), B, nb, dw);
    if (rd < 0) fprintf(stderr, "dist_wall.dat unreadable or for another mesh: distances formed anew\n");
    for (int m = 0; m < nb && rd == 0; m++)
      if ((r = ec2d_set_wall_distance(ctx, cs, m + 1, dw[m]))) return fail("ec2d_set_wall_distance", r);
    have_dw = rd == 0;
    for (int m = 0; m < nb; m++) free(dw[m]);
  }
  if ((r = ec2d_setup(ctx))) return fail("ec2d_setup", r);
  if (turbulent && !have_dw && (r = write_dist_wall(dir, ctx, cs, B, nb))) return fail("dist_wall.dat", r);
  if (P.Iflag_init == 0) {
    if ((r = ec2d_init_flow(ctx))) return fail("ec2d_init_flow", r);
  } else if ((r = restart(dir, ctx, cs, &P, B, nb, nvar, fix_nvar))) {
    ec2d_destroy(ctx);
    return r;
  }
  printf(" Start ......\n");

  double rmax[6] = {0}, rrms[6] = {0}, tt = 0.0;
  int kstep = 0;
  long done = 0;
  char rpath[4096];
  snprintf(rpath, sizeof(rpath), "%s/Residual.dat", dir);
  while (tt < P.t_end && (max_steps < 0 || done < max_steps)) {
    if ((r = ec2d_step(ctx, 1))) return fail("ec2d_step", r);
    done++;
    r = ec2d_residual(ctx, cs, 1, rmax, rrms, &kstep, &tt);
    if (r == EC2D_ERR_STATE) {
      int code, blk, i, j;
      ec2d_status(ctx, cs, &code, &blk, &i, &j);
      printf("T <1.d-5 ! at block %d cell (%d,%d)\n", blk, i, j);
      ec2d_destroy(ctx);
      return r;
    }
    if (r) return fail("ec2d_residual", r);
    /* (a zero Kstep_save or Kstep_show, for which the reference's mod is
     * undefined, writes every step, as the Python driver does) */
    if (kstep % (P.Kstep_save > 0 ? P.Kstep_save : 1) == 0 && (r = output(dir, ctx, cs, &P, B, nb, nvar, kstep)))
      return fail("output", r); /* output(1) */
    if (kstep % (P.Kstep_show > 0 ? P.Kstep_show : 1) == 0) { /* output_Res(1) */
      FILE *f = fopen(rpath, "a");
      if (f) {
        fprintf(f, "%8d", kstep);
        for (int m = 0; m < 6; m++) e24(f, rmax[m]);
        for (int m = 0; m < nvar; m++) e24(f, rrms[m]);
        fprintf(f, "\n");
        fclose(f);
      }
    }
  }
  if ((r = output(dir, ctx, cs, &P, B, nb, nvar, kstep))) return fail("output", r); /* the final output(1) */
  double cl = 0, cd = 0, cm = 0;
  if ((r = ec2d_forces(ctx, cs, &cl, &cd, &cm))) return fail("ec2d_forces", r);
  printf("steps %ld kstep %d tt %.17g\n", done, kstep, tt);
  printf("res_rms");
  for (int m = 0; m < nvar; m++) printf(" %.17g", rrms[m]);
  printf("\nforces %.17g %.17g %.17g\n", cl, cd, cm);
  ec2d_destroy(ctx);
  for (int m = 0; m < nb; m++) { free(B[m].x); free(B[m].y); free(B[m].bc9); }
  return 0;
}
