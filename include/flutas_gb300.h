/*
 * flutas_gb300.h -- C ABI of the GB300-native FluTAS pressure-projection path.
 *
 * The entry points keep the argument lists of the Fortran routines they
 * replace, so a FluTAS app binds them through iso_c_binding with a one-line
 * `use` swap.  Plain pointers and sizes only.
 *
 * Conventions
 *  - Arrays are Fortran column-major (x fastest) and are passed as the address
 *    of their first element: p(0:nx+1,0:ny+1,0:nz+1) with halo 1; velocities
 *    u,v,w(1-nh_u:nx+nh_u, ...); z spacings dzci,dzfi(1-nh_d:nz+nh_d).
 *  - Field pointers may be device pointers (CUDA device or managed memory:
 *    used in place) or host pointers (pageable or pinned: copied to
 *    library-owned device mirrors and back inside the call).
 *  - BC characters are 'P','N','D'; cbc is the Fortran cbc(0:1,1:3) in
 *    memory order (x-low, x-high, y-low, y-high, z-low, z-high).
 *  - Every call returns FLUTAS_OK (0) or a negative code; the message of the
 *    last failure on the calling thread is available from
 *    flutas_gb300_last_error().  Nothing aborts the process, nothing traps
 *    the device.
 *  - Calls are synchronous (drop-in semantics) unless the plan was switched
 *    to asynchronous mode with flutas_gb300_plan_set_stream().
 */
#ifndef FLUTAS_GB300_H
#define FLUTAS_GB300_H

#include <stddef.h>

#if defined(__GNUC__)
#define FLUTAS_API __attribute__((visibility("default")))
#else
#define FLUTAS_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define FLUTAS_OK 0
#define FLUTAS_EINVAL (-1)       /* bad argument: size, BC character, null pointer */
#define FLUTAS_EUNSUPPORTED (-2) /* combination the GPU path does not implement */
#define FLUTAS_ECUDA (-3)        /* CUDA runtime error */
#define FLUTAS_ENOMEM (-4)       /* device allocation failed or over the HBM budget */
#define FLUTAS_EITER (-5)        /* iterative refinement hit its iteration limit */
#define FLUTAS_ENONFINITE (-6)   /* NaN/Inf found in the input or the result */
#define FLUTAS_EBUSY (-7)        /* serving queue full / request not finished */

/* Replaces initsolver (src/initsolver.f90:21, with fftini src/fft.f90:24-157).
 * Host outputs exactly as the reference: lambdaxy(nx,ny), a,b,c(nz), normfft,
 * rhsbx(ny,nz,0:1), rhsby(nx,nz,0:1), rhsbz(nx,ny,0:1).  arrplan points at the
 * Fortran arrplan(2,2) of type(C_PTR): element (1,1) receives the opaque plan
 * (device-resident eigenvalues, z coefficients, twiddles and scratch); the
 * other three are set to NULL.  dims / dims_z of the reference are 1 (one GPU). */
FLUTAS_API int flutas_gb300_initsolver(const int n[3], const double dli[3], int nh_d, const double *dzci,
                            const double *dzfi, const char cbc[6], const double bc[6],
                            const char c_or_f[3], double *lambdaxy, double *a, double *b,
                            double *c, void **arrplan, double *normfft, double *rhsbx,
                            double *rhsby, double *rhsbz);

/* Replaces initgrid (src/initgrid.f90:17-97, clustering functions 102-135), on
 * the host: the z grid dzc, dzf, zc, zf(1-nh_d:n+nh_d) of n cells on [0,lz],
 * tanh-clustered with factor gr (0: uniform) at both walls, or at the lower
 * wall when inivel is 'hcl' or 'hcp'.  The apps pass 1/dzc, 1/dzf on as dzci,
 * dzfi. */
FLUTAS_API int flutas_gb300_initgrid(const char inivel[3], int n, double gr, double lz, int nh_d, double *dzc,
                                     double *dzf, double *zc, double *zf);

/* Replaces solver_cpu (src/solver_cpu.f90:20) / solver_gpu (src/solver_gpu.f90:31):
 * FP64 fwd x/y r2r transforms, z tridiagonal solve per (kx,ky), inverse
 * transforms, times normfft.  p(0:n+1,...) in place (interior overwritten).
 * lambdaxy/a/b/c may be the host arrays filled by initsolver (the plan's
 * device copies are used) or device arrays. */
FLUTAS_API int flutas_gb300_solver(const int n[3], void *const *arrplan, double normfft,
                        const double *lambdaxy, const double *a, const double *b, const double *c,
                        const char bcz[2], const char c_or_f[3], double *p);

/* Replaces fillps (src/fillps.f90:16): p = rho0 * dti * div(u,v,w). */
FLUTAS_API int flutas_gb300_fillps(int nx, int ny, int nz, int nh_d, int nh_u, double dxi, double dyi,
                        double dzi, const double *dzfi, double dti, double rho0, const double *u,
                        const double *v, const double *w, double *p);

/* Replaces correc (src/correc.f90:16), constant-coefficient branch (57-60):
 * u -= dt*dxi*(p(i+1)-p(i))/rho0, etc.  rho is accepted for signature
 * compatibility and not read (the reference never builds the variable branch). */
FLUTAS_API int flutas_gb300_correc(int nx, int ny, int nz, int nh_d, int nh_u, double dxi, double dyi,
                        double dzi, const double *dzci, double dt, double rho0, const double *p,
                        double *u, double *v, double *w, const double *rho);

/* Replaces boundp (src/bound.f90:146) for a single domain with nh_p = 1:
 * ghost cells of p per set_bc (src/bound.f90:227-646), x then y then z.
 * halo is accepted for signature compatibility (MPI halo types, unused). */
FLUTAS_API int flutas_gb300_boundp(const char cbc[6], const int n[3], const double bc[6], int nh_d, int nh_p,
                        const int halo[3], const double dl[3], const double *dzc,
                        const double *dzf, double *p);

/* Replaces bounduvw (src/bound.f90:17) for a single domain: velocity ghosts per
 * set_bc (src/bound.f90:227-646), the face-normal component non-centred.
 * cbcvel/bcvel are cbcvel/bcvel(0:1,1:3,1:3) in memory order; isoutflow
 * (nullable) is isoutflow(0:1,1:3): flagged faces get the zero-divergence
 * outflow velocity of src/bound.f90:649-773 after the ghosts, bit-identical to
 * the reference expression.  The fused projections take no outflow flags. */
FLUTAS_API int flutas_gb300_bounduvw(const char cbcvel[18], const int n[3], const double bcvel[18],
                                     int nh_d, int nh_u, const int halo[3], const int isoutflow[6],
                                     const double dl[3], const double *dzc, const double *dzf,
                                     double *u, double *v, double *w);

/* Replaces updt_rhs_b (src/bound.f90:829): adds the inhomogeneous-BC terms
 * rhsbx/rhsby/rhsbz (host or device) to the boundary planes of p. */
FLUTAS_API int flutas_gb300_updt_rhs_b(int nx, int ny, int nz, const char c_or_f[3], const char cbc[6],
                            int nh_p, const double *rhsbx, const double *rhsby,
                            const double *rhsbz, double *p);

/* Replaces chkdiv (src/chkdiv.f90:18) on one GPU: total and max |div u|. */
FLUTAS_API int flutas_gb300_chkdiv(int nx, int ny, int nz, double dxi, double dyi, double dzi, int nh_d,
                        int nh_u, const double *dzfi, const double *u, const double *v,
                        const double *w, double *divtot, double *divmax);

/* Replaces pres_tw_src (src/source.f90:247), constant-coefficient
 * (Dodd-Ferrante) branch: adds the explicit pressure terms to u*,v*,w*. */
FLUTAS_API int flutas_gb300_pres_tw_src(int nx, int ny, int nz, double dxi, double dyi, double dzi, int nh_d,
                             int nh_u, const double *dzci, double rho0i, double f_t12,
                             double f_t12_o, const double *p, const double *pold,
                             const double *rho, double *u, double *v, double *w);

/* Replaces rk (src/rk.f90:26-102) of the two-phase apps: the momentum
 * right-hand sides of momad_xyz_tw_cen (space_scheme_mom "cen",
 * src/mom.f90:21-197) or momad_xyz_tw_fll ("fll", src/mom.f90:199-386; needs
 * nh_u >= 2) from the old u,v,w, mu, rho (halo-1 arrays), then
 * u = u + f_t1*dudt + f_t2*dudtrko and dudtrko = dudt on the interior (the
 * halo is left for bounduvw).  dudtrko, dvdtrko, dwdtrko are (nx,ny,nz).
 * FP64, 3-D (the reference's _TWOD build is not covered). */
FLUTAS_API int flutas_gb300_rk(const char space_scheme_mom[3], double f_t1, double f_t2, int nx, int ny, int nz,
                               double dxi, double dyi, double dzi, int nh_d, int nh_u, const double *dzci,
                               const double *dzfi, double *u, double *v, double *w, const double *mu,
                               const double *rho, double *dudtrko, double *dvdtrko, double *dwdtrko);

/* rk of the single-phase build (src/rk.f90:26-102 with momad_xyz_sp,
 * src/mom.f90:388-575): visc_sp = mu_sp/rho_sp of the app's parameters. */
FLUTAS_API int flutas_gb300_rk_sp(double f_t1, double f_t2, int nx, int ny, int nz, double dxi, double dyi,
                                  double dzi, int nh_d, int nh_u, const double *dzci, const double *dzfi,
                                  double visc_sp, double *u, double *v, double *w, double *dudtrko,
                                  double *dvdtrko, double *dwdtrko);

/* Replaces cmpt_time_factors (src/rk.f90:104-135), on the host: f_t1, f_t2,
 * f_t12 of AB2 ("ab2", first-order Euler at istep 1) or of RK3 substep irk_ss
 * ("rk3", rkcoeff(2,3) in memory order). */
FLUTAS_API int flutas_gb300_cmpt_time_factors(const char time_scheme[3], int restart, int istep, int irk_ss,
                                              const double rkcoeff[6], double dt, double dto, double *f_t1,
                                              double *f_t2, double *f_t12);

/* Replaces fftend (src/fft.f90:159-179): frees the plan in arrplan(1,1). */
FLUTAS_API int flutas_gb300_fftend(void **arrplan);

/* Copies the message of the last failure on this thread into buf (NUL-terminated). */
FLUTAS_API int flutas_gb300_last_error(char *buf, int len);

/* ---------------------------------------------------------------------------
 * Extensions beyond the reference interface (no Fortran counterpart).
 * ------------------------------------------------------------------------- */

/* Asynchronous mode: run the plan's work on `stream` (a cudaStream_t, or NULL
 * for the legacy default stream) and return without synchronising. */
FLUTAS_API int flutas_gb300_plan_set_stream(void *plan, void *stream, int synchronous);

/* Mixed-precision solve: FP32 transforms and tridiagonal solves, FP64
 * residual of the 7-point operator and FP64 update, iterated until
 * ||f - A p||_2 / ||f||_2 <= tol or max_iter corrections.  Same in/out as
 * flutas_gb300_solver (p holds the RHS on entry, the solution on exit).
 * relres/iters (nullable) receive the achieved relative residual and the
 * number of FP32 solves.  Returns FLUTAS_EITER if tol was not reached. */
FLUTAS_API int flutas_gb300_solve_mixed(void *plan, double *p, double tol, int max_iter, double *relres,
                             int *iters);

/* Fused projection (one call for the steps of src/apps/<app>/main__<app>.f90: fillps ->
 * updt_rhs_b -> solver -> boundp -> correc -> bounduvw -> p = pold + p -> boundp):
 * on exit u,v,w are projected and p holds pold + phi.  precision: 0 = FP64,
 * 1 = mixed to tol.  dzci/dzfi: (1-nh_d:nz+nh_d).  bcpre = bc(0:1,1:3).
 * cbcvel/bcvel (nullable): velocity BCs; when given, bounduvw is applied
 * after correc.  With page-locked host arrays the mixed form overlaps its
 * copies with its kernels (w copied in z-slabs with the first pass behind
 * it, u copied back while v, w and p are corrected; FLUTAS_GB300_SLABS=0
 * turns the slabs off); the results equal the device-array call bit for bit. */
FLUTAS_API int flutas_gb300_projection(void *plan, int nh_u, double dxi, double dyi, const double *dzci,
                            const double *dzfi, const double bcpre[6], const char *cbcvel,
                            const double *bcvel, double dt, double rho0,
                            double *u, double *v, double *w, double *p, int precision,
                            double tol, int max_iter);

/* Two-phase fused projection: pres_tw_src (src/source.f90:247-309, the
 * Dodd-Ferrante constant-coefficient split: explicit (1/rho - 1/rho0) terms
 * built from p and pold) applied to u*,v*,w*, bounduvw (when cbcvel is
 * given), then the projection above with dt = f_t12.  rho, pold: (0:n+1) halo-1 arrays; p holds p^n on entry and
 * p^n + phi on exit; pold holds p^(n-1) on entry (read by pres_tw_src) and p^n on exit, interior copy
 * then boundp, as the app does between pres_tw_src and fillps
 * (src/apps/two_phase_inc_isot/main__two_phase_inc_isot.f90:624-716, pold = p at 655-674): repeated
 * calls are the app's time steps. */
FLUTAS_API int flutas_gb300_projection_df(void *plan, int nh_u, double dxi, double dyi,
                                          const double *dzci, const double *dzfi,
                                          const double bcpre[6], const char *cbcvel,
                                          const double *bcvel, double f_t12, double f_t12_o,
                                          double rho0, const double *rho, double *pold,
                                          double *u, double *v, double *w, double *p, int precision,
                                          double tol, int max_iter);

/* Relative residual and number of FP32 solves of the plan's last mixed solve. */
FLUTAS_API int flutas_gb300_last_solve(void *plan, double *relres, int *iters);

/* Plan introspection: bytes of device memory held by the plan, and which
 * transform path it uses (0 = separate x/y passes, 1 = fused plane kernel). */
FLUTAS_API int flutas_gb300_plan_info(void *plan, size_t *device_bytes, int *xy_path_fp64, int *xy_path_fp32);

/* Divergence check that allocates nothing (no counterpart in the reference).
 * Same arguments and result as flutas_gb300_chkdiv, for callers that must not
 * allocate device memory at the point of the call: an application that gives
 * the whole device to its own memory pool, or a diagnostic run after an
 * out-of-memory error, when a cudaMalloc would fail.  u, v, w and dzfi must
 * be device memory of the current device, or managed memory (host arrays
 * would need staging buffers; another GPU's arrays are rejected with
 * FLUTAS_EINVAL).  Its scratch is a fixed 1 MiB device array inside the
 * library, one (sum, max) pair per (j,k) row of cells, so ny*nz may not
 * exceed 65536 (FLUTAS_EINVAL otherwise).
 * Set-up: the first call on a device (or the first flutas_gb300_initsolver on
 * it, whichever comes first) loads the check's two kernels and resolves the
 * array's address on that device.  Under CUDA's lazy module loading that
 * first load may itself allocate device memory, so make one call (or create a
 * plan) on each device before relying on the guarantee, and before any
 * stream capture; CUDA_MODULE_LOADING=EAGER loads everything at start-up.
 * All calls share the array and every call rewrites the rows it reads: calls
 * that overlap on the GPU (several host threads, or several streams) race and
 * must be serialised by the caller.  Synchronous: returns after the result is
 * on the host. */
FLUTAS_API int flutas_gb300_chkdiv_noalloc(int nx, int ny, int nz, double dxi, double dyi, double dzi,
                                           int nh_d, int nh_u, const double *dzfi, const double *u,
                                           const double *v, const double *w, double *divtot,
                                           double *divmax);

/* Batched mixed-precision solves of many independent grids (uneven sizes and
 * BCs; no counterpart in the reference, which solves one grid per call).
 * n, dli: 3 per grid; dzci, dzfi: one (1-nh_d:nz+nh_d) host array per grid;
 * cbc: 6 characters per grid.  Each pass of the refinement (x transform, y
 * transform, z solve, inverse transforms, FP64 residual) is one persistent
 * kernel draining a (grid, tile) work queue over all grids; the whole
 * sequence is captured in a CUDA graph and replayed by batch_solve.  With
 * autotune != 0, the radix plan and tile shape of each axis signature are
 * chosen by timing candidates on the device (cached per process).  The batch
 * owns one device halo array per grid (batch_field): the RHS on entry of
 * batch_solve, the solution on exit.  relres/iters (nullable, one per grid)
 * receive the achieved relative residual and the FP32 solves used. */
FLUTAS_API int flutas_gb300_batch_create(int ngrids, const int *n, const double *dli, int nh_d,
                                         const double *const *dzci, const double *const *dzfi,
                                         const char *cbc, int autotune, void **batch);
FLUTAS_API int flutas_gb300_batch_field(void *batch, int grid, double **p);
/* Copy a grid's halo array in (RHS) or out (solution); host or device memory. */
FLUTAS_API int flutas_gb300_batch_set(void *batch, int grid, const double *src);
FLUTAS_API int flutas_gb300_batch_get(void *batch, int grid, double *dst);
FLUTAS_API int flutas_gb300_batch_solve(void *batch, double tol, int max_iter, double *relres, int *iters);
FLUTAS_API int flutas_gb300_batch_report(void *batch, char *buf, int len);
FLUTAS_API int flutas_gb300_batch_destroy(void *batch);

/* ---------------------------------------------------------------------------
 * Serving (no counterpart in the reference): a continuous-batching request
 * loop.  Requests of any size are submitted at any time; `slots` workers, each
 * with its own CUDA stream, admit them in arrival order as soon as a slot is
 * free and the HBM budget covers the request's fields and plan, so admitted
 * requests overlap on the device.  Plans stay resident between requests of
 * the same grid and are evicted least-recently-used when the budget needs
 * room.  The caller's arrays must stay valid until server_wait returns.
 * Fields that already live on the device (device memory of the current
 * device, or managed) are solved in place, with no staging copy and no field
 * memory charged to the budget (a two-phase projection's fields are always
 * staged: its pold is an input the in-place call would overwrite).  Host
 * fields are copied to server-owned device buffers and back.
 * ------------------------------------------------------------------------- */
typedef struct {
  int kind;                    /* 0: Poisson solve rhs -> p; 1: projection of u,v,w,p */
  int n[3];
  double dli[3];
  int nh_d;
  const double *dzci, *dzfi;   /* (1-nh_d:nz+nh_d), host memory */
  char cbc[6];
  const double *bcpre;         /* nullable: homogeneous BC values */
  double tol;                  /* > 0: mixed precision refined to tol; 0: the plain FP64 path */
  int max_iter;
  const double *rhs;           /* kind 0: RHS, halo-1 array */
  double *p;                   /* kind 0: solution out; kind 1: pressure in/out (p^n -> p^n + phi) */
  double *u, *v, *w;           /* kind 1: velocities (halo nh_u), in/out */
  const double *rho, *pold;    /* kind 1: two-phase Dodd-Ferrante split when non-null */
  int nh_u;
  double dt, dt_old, rho0;
  const char *cbcvel;          /* nullable: 18 velocity BC characters (bounduvw) */
  const double *bcvel;         /* 18 values when cbcvel is given */
} flutas_request;

FLUTAS_API int flutas_gb300_server_create(size_t hbm_budget_bytes, int slots, void **server);
FLUTAS_API int flutas_gb300_server_submit(void *server, const flutas_request *req, long long *ticket);
/* Blocks until the request is done; returns its status (FLUTAS_EITER when tol was not reached). */
FLUTAS_API int flutas_gb300_server_wait(void *server, long long ticket, double *relres, int *iters,
                                        double *latency_ms);
/* JSON text: completed, p50_ms, p99_ms (submit-to-result latency), span_s, budget use, and
 * max_device_overlap: the largest number of requests whose work was on the device at one
 * instant (spans from CUDA events on the workers' streams). */
FLUTAS_API int flutas_gb300_server_stats(void *server, char *buf, int len);
FLUTAS_API int flutas_gb300_server_reset_stats(void *server);
/* Waits for every queued request, then stops the workers and frees the plans. */
FLUTAS_API int flutas_gb300_server_destroy(void *server);

/* update_property (src/vof.f90:240-271): prop = vof*prop12[0] + (1-vof)*prop12[1]
 * on the interior of the halo-1 arrays vof and prop (0:n+1 per axis; the halo
 * of prop is left for boundp, as in the apps: main__two_phase_inc_isot.f90:461-462).
 * Rounded as the Fortran expression (bit-identical). */
FLUTAS_API int flutas_gb300_update_property(const int n[3], const double prop12[2], const double *vof,
                                            double *prop);

/* ---------------------------------------------------------------------------
 * Restart-file I/O (src/load.f90).  Fields are raw FP64 files of the global
 * interior, x fastest, no header, exactly 8*n[0]*n[1]*n[2] bytes.
 * ------------------------------------------------------------------------- */
/* load (src/load.f90:21-89): io = 'r' reads `filename` into the interior of
 * fld, io = 'w' writes the interior of fld to it (created or truncated).  fld
 * has nh halo cells on every side (nh = 0: fld is the contiguous interior, as
 * the Fortran explicit-shape dummy argument) and is host or device memory.
 * Reading a missing file or a file of another size returns FLUTAS_EINVAL with
 * the reference's message (where it stops the run). */
FLUTAS_API int flutas_gb300_load(char io, const char *filename, const int n[3], int nh, double *fld);
/* load_scalar (src/load.f90:91-128): time, dto and istep as text; written
 * with the format (2E15.7, 1I9.8), read list-directed. */
FLUTAS_API int flutas_gb300_load_scalar(char io, const char *filename, double *time, int *istep, double *dto);
/* load_ns (src/load.f90:130-214): u, v, w, p and then (time, istep) as two
 * FP64 values in one file (the CaNS restart layout); fields as in load. */
FLUTAS_API int flutas_gb300_load_ns(char io, const char *filename, const int n[3], int nh, double *u, double *v,
                                    double *w, double *p, double *time, double *istep);

/* Number of kernels this library has launched in the process (all plans). */
FLUTAS_API int flutas_gb300_launch_count(unsigned long long *count);

/* Per-kernel timing: when enabled, every launch is bracketed by CUDA events
 * on its own stream.  The report lists "kernel launches total_ms" lines. */
FLUTAS_API int flutas_gb300_profile(int enable);
FLUTAS_API int flutas_gb300_profile_report(char *buf, int len, int reset);

#ifdef __cplusplus
}
#endif
#endif /* FLUTAS_GB300_H */
