/*
 * flutas_oracle.h -- CPU FP64 restatement of the FluTAS pressure-projection
 * path (fillps -> updt_rhs_b -> solver_cpu -> boundp -> correc), used ONLY to
 * check the CUDA path against (tests, smoke(), the CPU-baseline leg of
 * bench.py).  Nothing in the product library links or calls this code.
 *
 * Parity status: the reference's own solver_cpu needs gfortran + FFTW 3.3.10
 * (an external, un-vendored dependency) and cannot be built here, and the
 * reference's tests hold no golden vectors for this path.  This restatement
 * is therefore pinned by closed-form discrete-eigenfunction known answers
 * (tests/golden/) and by an independent scipy.fft restatement
 * (oracle/restate_scipy.py), not by a run of the reference itself.
 *
 * Array conventions follow the Fortran code (column-major, x fastest):
 *   p, pold, rho, psi : (0:nx+1, 0:ny+1, 0:nz+1)            halo 1
 *   u, v, w           : (1-nh_u:nx+nh_u, ...)                 halo nh_u
 *   dzc, dzf, dzci... : (1-nh_d:nz+nh_d)                      halo nh_d
 *   lambdaxy          : (nx, ny);  a, b, c : (nz)
 *   rhsbx (ny,nz,0:1), rhsby (nx,nz,0:1), rhsbz (nx,ny,0:1)
 * BC characters are 'P', 'N', 'D'; cbc is cbc(0:1,1:3) in Fortran order
 * (cbc[0]=x-low, cbc[1]=x-high, cbc[2]=y-low, ... ).
 */
#ifndef FLUTAS_ORACLE_H
#define FLUTAS_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

/* FFTW r2r kind numbers (fftw.f90:38-61). */
enum { OR_R2HC = 0, OR_HC2R = 1, OR_REDFT00 = 3, OR_REDFT01 = 4, OR_REDFT10 = 5,
       OR_REDFT11 = 6, OR_RODFT00 = 7, OR_RODFT01 = 8, OR_RODFT10 = 9, OR_RODFT11 = 10 };

/* One r2r transform of a contiguous line, FFTW's unnormalised definitions. */
int  or_r2r(int kind, int n, const double *in, double *out);

/* initsolver.f90:122-186, CPU (natural / halfcomplex) order; not scaled. */
int  or_eigenvalues(int n, char bc0, char bc1, char c_or_f, double *lambda);
/* initsolver.f90:188-246 */
int  or_tridmatrix(char bc0, char bc1, int n, int nh_d, const double *dzci,
                   const double *dzfi, char c_or_f, double *a, double *b, double *c);
/* fft.f90:233-291 */
int  or_find_fft(char bc0, char bc1, char c_or_f, int *kind_fwd, int *kind_bwd, double norm[2]);

/* The oracle's plan: what fftini (fft.f90:24-157) stores in arrplan. */
typedef struct {
  int n[3];
  int kind_fwd[2], kind_bwd[2];   /* x, y */
  int ix, iy;                     /* transform length reduction (DD face) */
} or_plan;

/* initsolver.f90:21-120 (single domain: dims = dims_z = 1). */
int  or_initsolver(const int n[3], const double dli[3], int nh_d, const double *dzci,
                   const double *dzfi, const char cbc[6], const double bc[6],
                   const char c_or_f[3], double *lambdaxy, double *a, double *b,
                   double *c, or_plan *plan, double *normfft, double *rhsbx,
                   double *rhsby, double *rhsbz);

/* solver_cpu.f90:20-115 (+ gaussel 117-145, gaussel_periodic 147-185,
 * dgtsv_homebrewed 187-223).  p has halo 1; its interior is overwritten. */
int  or_solver(const or_plan *plan, double normfft, const double *lambdaxy,
               const double *a, const double *b, const double *c,
               const char bcz[2], const char c_or_f[3], double *p);

/* fillps.f90:16-69 (constant-coefficient: times rho0). */
void or_fillps(int nx, int ny, int nz, int nh_d, int nh_u, double dxi, double dyi,
               double dzi, const double *dzfi, double dti, double rho0,
               const double *u, const double *v, const double *w, double *p);
/* correc.f90:16-81, constant-coefficient branch (57-60). */
void or_correc(int nx, int ny, int nz, int nh_d, int nh_u, double dxi, double dyi,
               double dzi, const double *dzci, double dt, double rho0,
               const double *p, double *u, double *v, double *w);
/* bound.f90:146-225 boundp + set_bc 227-646 (nh_p = 1, single domain). */
void or_boundp(const char cbc[6], const int n[3], const double bc[6], int nh_d,
               const double dl[3], const double *dzc, const double *dzf, double *p);
/* bound.f90:17-144 bounduvw, single domain, no outflow.  cbc, bc are the
 * Fortran cbcvel/bcvel(0:1,1:3,1:3) in memory order. */
void or_bounduvw(const char cbc[18], const int n[3], const double bc[18], int nh_d, int nh_u,
                 const double dl[3], const double *dzc, const double *dzf, double *u, double *v, double *w,
                 const int *isoutflow);
/* bound.f90:829-944 */
void or_updt_rhs_b(int nx, int ny, int nz, const char c_or_f[3], const char cbc[6],
                   const double *rhsbx, const double *rhsby, const double *rhsbz, double *p);
/* chkdiv.f90:18-69 (without the MPI reduction). */
void or_chkdiv(int nx, int ny, int nz, double dxi, double dyi, double dzi, int nh_d,
               int nh_u, const double *dzfi, const double *u, const double *v,
               const double *w, double *divtot, double *divmax);
/* source.f90:247-309, constant-coefficient (Dodd-Ferrante) branch. */
void or_pres_tw_src(int nx, int ny, int nz, double dxi, double dyi, double dzi, int nh_d,
                    int nh_u, const double *dzci, double rho0i, double f_t12,
                    double f_t12_o, const double *p, const double *pold,
                    const double *rho, double *u, double *v, double *w);
/* initgrid.f90:17-97 with gridpoint_cluster_two_end (102-118) or one_end (120-136). */
void or_initgrid(int two_end, int n, double gr, double lz, int nh_d, double *dzc,
                 double *dzf, double *zc, double *zf);
/* vof.f90:240-271 update_property: rho = psi*rho1 + (1-psi)*rho2 on the interior of halo-1 arrays. */
void or_update_property(int nx, int ny, int nz, double rho1, double rho2,
                        const double *psi, double *rho);
/* Residual of the discrete operator the solver inverts: r = f - A p, with the
 * homogeneous ghost rules of tridmatrix/eigenvalues (P copy, N p0=p1, D p0=-p1),
 * cell-centred.  f and p have halo 1; r interior written (halo untouched). */
void or_residual(const int n[3], const char cbc[6], double dxi, double dyi, int nh_d,
                 const double *dzci, const double *dzfi, const double *f,
                 const double *p, double *r);

/* OpenMP threads used by the parallel loops (0 = library default). */
/* momentum predictor (src/mom.f90, src/rk.f90): variant 0 momad_xyz_tw_cen, 1 momad_xyz_tw_fll,
 * 2 momad_xyz_sp (visc_sp = mu_sp/rho_sp; mu, rho unused) */
void or_momad(int variant, int nx, int ny, int nz, double dxi, double dyi, double dzi, int nh_d, int nh_u,
              const double *dzci, const double *dzfi, const double *u, const double *v, const double *w,
              const double *mu, const double *rho, double visc_sp, double *dudt, double *dvdt, double *dwdt);
void or_rk(int variant, double f_t1, double f_t2, int nx, int ny, int nz, double dxi, double dyi, double dzi,
           int nh_d, int nh_u, const double *dzci, const double *dzfi, double *u, double *v, double *w,
           const double *mu, const double *rho, double visc_sp, double *dudtrko, double *dvdtrko,
           double *dwdtrko);
int  or_cmpt_time_factors(const char *time_scheme, int istep, int irk_ss, const double *rkcoeff, double dt,
                          double dto, double *f);
void or_set_threads(int nthreads);
int  or_get_threads(void);

#ifdef __cplusplus
}
#endif
#endif
