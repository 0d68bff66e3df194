/*
 * sfdx.h -- C ABI of the GB300-native SFD_EXCMG forward solver.
 *
 * Plain C types only (double, int, pointers, sizes); complex arrays are
 * interleaved (re, im) doubles, i.e. the memory layout of Fortran
 * complex(8) and C99 double _Complex.  Every entry point returns an SFDX_*
 * status code instead of stopping the process.
 *
 * Mesh conventions are the reference's (sfd_excmg/src/fdfe_main.f90):
 *   nx, ny        cells along x and y
 *   nz            cells along z INCLUDING the nair air layers (z index 1 is
 *                 the top of the air, as in read_input, file_opt.f90:8-95)
 *   a[nx], b[ny], c[nz]   cell sizes; c holds the air layers first
 *   sigma         Fortran sigma(ncell,6) = C [6][ncell], ncell = nx*ny*nz,
 *                 components (xx, yy, zz, xy, xz, yz), cell index
 *                 (k-1)*nx*ny + (j-1)*nx + i  (file_opt.f90:142)
 *   nl            nx(ny+1)(nz+1) + (nx+1)ny(nz+1) + (nx+1)(ny+1)nz edges,
 *                 ordered Ex, Ey, Ez (fdfe_main.f90:261,310,358)
 *   ex            Fortran ex(2*nl, nf) = C [nf][2][nl] complex: the xy
 *                 solution followed by the yx solution of each frequency
 *                 (fwd_solver, fdfe_main.f90:1565-1594)
 */
#ifndef SFDX_H
#define SFDX_H

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define SFDX_OK 0
#define SFDX_ERR_ARG 1         /* invalid argument (null pointer, bad size, bad option)     */
#define SFDX_ERR_MESH 2        /* mesh not divisible by 2^level / level too large            */
#define SFDX_ERR_CUDA 3        /* CUDA runtime error or no device                            */
#define SFDX_ERR_NOCONV 4      /* a system reached its iteration limit before the tolerance  */
#define SFDX_ERR_NAN 5         /* NaN in a right-hand side, guess or residual                */
#define SFDX_ERR_RECEIVER 6    /* receiver outside the interpolation stencil                 */
#define SFDX_ERR_IO 7          /* model/data file missing or malformed                       */
#define SFDX_ERR_UNSUPPORTED 8 /* option combination not implemented                         */
#define SFDX_ERR_TIMEOUT 9     /* a bounded device wait ran out                              */
#define SFDX_ERR_NOMEM 10      /* device allocation failed / size above a fixed limit        */

/* quirk bits: reference behaviours that change intermediate results */
#define SFDX_QUIRK_COARSEN_SHIFT 1   /* mesh_coarsen fine-cell index (fdfe_main.f90:64)          */
#define SFDX_QUIRK_EXCMG_MIDPOINT 2  /* cal_coef along-edge nodes (excmg.f90:685,711,737)         */
#define SFDX_QUIRK_RX_TRANSPOSE 4    /* arho_interp2 rd=2 stencil (fdfe_main.f90:763-768)         */
#define SFDX_QUIRK_TOPO_PLANE 8      /* topography receiver plane one cell deep and c(nair+1) as
                                        its vertical step (fdfe_main.f90:604-616, 627-629)       */
#define SFDX_QUIRKS_REFERENCE 15

/* solver ids (.fwd line 2, read_input file_opt.f90:102).  TFQMR, BiCG and COCR
 * are broken or unreachable in the reference (ptfqmr, pbicg, pcocr); these are
 * the published algorithms (Freund 1993; Fletcher 1976 with A^H; Sogabe & Zhang
 * 2007).  TFQMR and BiCG run in FP64 also in mixed-precision plans. */
#define SFDX_SOLVER_BICGSTAB 1
#define SFDX_SOLVER_TFQMR 2
#define SFDX_SOLVER_GPBICG 3
#define SFDX_SOLVER_BICG 4
#define SFDX_SOLVER_COCR 6

/* most systems (frequency x polarisation, or right-hand sides) in one batch;
 * the reference solves one system at a time, so this has no counterpart there */
#define SFDX_MAX_SYSTEMS 128

/* precision */
#define SFDX_FP64 0   /* complex128 everywhere                                    */
#define SFDX_MIXED 1  /* complex64 operator/smoother/Krylov inside FP64 refinement */

/*
 * Runtime options.  Defaults (sfdx_default_opts) equal the reference's
 * compile-time constants in global_para.f90:5-19 and solvers.f90:14.
 */
typedef struct sfdx_opts {
    int level;          /* EXCMG levels, >= 3 (.fwd line 2; argv 2)                    */
    double eps;         /* finest-level tolerance (.fwd line 2; argv 3)                */
    int solver;         /* SFDX_SOLVER_*                                               */
    int excmg;          /* fwd_acc: 0 single solve from zero guess, 1 EXCMG cascade    */
    int precond;        /* 'S' multi-colour SSOR, 'J' Jacobi (pre_type); 'I' ILU(0) is
                           not built: SFDX_ERR_UNSUPPORTED.  'G' (no counterpart in
                           the reference): edge multigrid V-cycle over the EXCMG
                           mesh levels, multi-colour SSOR + nodal smoother; such
                           plans coarsen the conductivity without the index shift
                           of SFDX_QUIRK_COARSEN_SHIFT and, in mixed precision,
                           run complex128 Krylov iterations preconditioned by a
                           complex64 V-cycle                                     */
    int div_cor;        /* divergence correction (div_cor): 0 off, 1 the reference's
                           (div_correc every corr_intv iterations), 2 consistent
                           gradient-space correction between restart cycles of
                           corr_intv iterations and after the last (no counterpart
                           in the reference: sfdx_grad_correct below)              */
    int corr_intv;      /* iterations between corrections (corr_intv = 200)            */
    double corr_tol;    /* nodal-Poisson PCG tolerance (corr_tol = 1e-3)               */
    double ssor_omega;  /* SSOR relaxation in (0, 2) (ssor_omg = 1)                    */
    double sigma_air;   /* conductivity written into air cells by readers (1e-9)      */
    int maxit_plain;    /* iteration limit of the single solve (5000)                  */
    int maxit_level;    /* iteration limit of each EXCMG level (1000)                  */
    int precision;      /* SFDX_FP64 | SFDX_MIXED                                      */
    int quirks;         /* SFDX_QUIRK_* bits (SFDX_QUIRKS_REFERENCE by default)         */
    double coarse_tol;  /* relative residual of the on-device solve replacing PARDISO */
    int coarse_maxit;   /* iteration limit of that solve                               */
    int reliable_every; /* mixed precision: iterations between FP64 residual updates */
    int batch;          /* must be 0: all 2*nf systems of a plan form one batch; to
                           bound memory, split the frequencies over several plans
                           (sfdx_plan_solve_batch runs them concurrently)           */
    int verbose;        /* 0 silent, 1 per-level summary on stderr                     */
    int use_graphs;     /* replay each 8-iteration check interval of the Krylov solves
                           as a captured CUDA graph (1, default) or launch eagerly (0) */
} sfdx_opts;

/* Fill *o with the reference defaults. */
void sfdx_default_opts(sfdx_opts* o);

/* Human-readable text of a status code (static storage). */
const char* sfdx_strerror(int code);

/* Library version (major*10000 + minor*100 + patch). */
int sfdx_version(void);

/* Number of CUDA kernel launches this library has issued in this process. */
long long sfdx_launch_count(void);

/* ------------------------------------------------------------------------
 * Forward solve.  Replaces fwd_solver(modelname, a, b, c, nair, level, slv,
 * eps, sigma, freq, ex) (fdfe_main.f90:1565-1594, called at
 * sfd_excmg.f90:52).  ex is caller-owned [nf][2][nl] complex.
 * iters (optional, [nf][2][level]): Krylov iterations per level (reference
 * iters(1) semantics: loop index at exit) -- levels 1-2 of the cascade
 * report the on-device coarse solve.  relres (optional, [nf][2]): final
 * relative residual ||b - A x|| / ||b|| on the finest level.
 * ------------------------------------------------------------------------ */
int sfdx_fwd_solve(const sfdx_opts* o, int nx, int ny, int nz, int nair, const double* a, const double* b,
                   const double* c, const double* sigma, int nf, const double* freq, double* ex, int* iters,
                   double* relres);

/* ------------------------------------------------------------------------
 * Reusable plan: device workspace for one mesh and frequency list, so
 * repeated solves (inversion loops, benchmarks) allocate nothing.
 * sigma / ex may be host or device pointers (flag *_on_device).
 * ------------------------------------------------------------------------ */
typedef struct sfdx_plan sfdx_plan;
int sfdx_plan_create(sfdx_plan** plan, const sfdx_opts* o, int nx, int ny, int nz, int nair, const double* a,
                     const double* b, const double* c, int nf, const double* freq);
int sfdx_plan_solve(sfdx_plan* plan, const double* sigma, int sigma_on_device, double* ex, int ex_on_device,
                    int* iters, double* relres);
/* Solve several plans at once (models of different meshes and frequency lists):
 * each plan runs on its own host thread and its own stream (plans must be
 * distinct and should not share a stream), so the GPU overlaps the models.
 * Per plan q: sigma[q], ex[q] (array or entries may be null), iters[q],
 * relres[q] (optional) as sfdx_plan_solve; status[q] its return code.
 * Returns the first error of any plan (SFDX_ERR_NOCONV only if nothing
 * worse).  No counterpart in the reference (it solves one system at a time). */
int sfdx_plan_solve_batch(int nplans, sfdx_plan* const* plans, const double* const* sigma, int sigma_on_device,
                          double* const* ex, int ex_on_device, int* const* iters, double* const* relres, int* status);
/* Re-solve the finest level for a changed conductivity, starting from the
 * fields of the plan's last full solve (no EXCMG cascade): perturbation and
 * continuation studies (finite-difference checks of the misfit gradient), where
 * those fields are a close initial guess and their error cancels in a central
 * difference.  tol > 0: relative residual of A x = b from those fields;
 * tol <= 0: solve the correction equation A d = b - A x0 from zero to a relative
 * reduction |tol| (0: the plan's eps) and return x0 + d.  Outputs as
 * sfdx_plan_solve (iters: the finest-level slot).  No counterpart in the
 * reference. */
int sfdx_plan_resolve(sfdx_plan* plan, const double* sigma, int sigma_on_device, double tol, int* iters,
                      double* relres);
/* Load (and coarsen) the conductivity without solving. */
int sfdx_plan_load(sfdx_plan* plan, const double* sigma, int sigma_on_device);
/* Impedances from the plan's last solution (device resident), see sfdx_impedance. */
int sfdx_plan_impedance(sfdx_plan* plan, int nrec, const double* recv, int out_type, double* out, double* tipper);
/* Gradient of the impedance misfit of the plan's last solution with respect to
 * the cell conductivities, by one adjoint solve per frequency and polarisation
 * (the forward operator with a right-hand side on the receiver planes, solved
 * with the plan's solver, precision and corrections from a zero guess).  No
 * counterpart in the reference (it has no inversion path).
 *   zobs [nf][nrec][4] observed (Re Zxy, Im Zxy, Re Zyx, Im Zyx); wts
 *   [nf][nrec][2] data weights (null: 1); misfit = sum wxy |Zxy - dxy|^2 +
 *   wyx |Zyx - dyx|^2 over frequencies and receivers; zpred (optional)
 *   [nf][nrec][4] the predicted impedances; grad [6][ncell] = d misfit /
 *   d sigma(cell, component) with the Dirichlet data (the 1-D background of
 *   cell column (1,1)) held fixed, on the device if grad_on_device (null:
 *   misfit and zpred only, no adjoint solve); tol the
 *   adjoint solve's relative residual (<= 0: the plan's eps); adj_iters /
 *   adj_relres (optional, [nf][2]) its iterations and FP64 relative residuals.
 * The forward fields stay valid (sfdx_plan_fields, sfdx_plan_impedance). */
int sfdx_plan_misfit_grad(sfdx_plan* plan, int nrec, const double* recv, const double* zobs, const double* wts,
                          double tol, double* misfit, double* zpred, double* grad, int grad_on_device,
                          int* adj_iters, double* adj_relres);
/* Device pointer of the plan's last solution, layout [nf][2][nl] complex (valid until the next solve). */
const double* sfdx_plan_fields(sfdx_plan* plan);
/* Bytes of device memory held by the plan. */
long long sfdx_plan_device_bytes(const sfdx_plan* plan);
/* Issue the plan's work on `stream` (a cudaStream_t; null = the plan's own stream). */
int sfdx_plan_set_stream(sfdx_plan* plan, void* stream);
/* CUDA-event time (ms per launch) of one kernel family on the finest level and its
 * algorithmic HBM bytes: 0 operator c64, 1 operator c128, 2 MC-SSOR c64, 3 MC-SSOR c128 (the
 * multi-colour SSOR whatever opts.precond), 4 one edge-multigrid V-cycle c64 over all levels. */
int sfdx_plan_kernel_time(sfdx_plan* plan, int kernel, int reps, double* ms, double* bytes);
/* Pick the number of systems each thread of the hot kernels handles (4, 2
 * or 1 consecutive systems, complex64 and complex128 separately) by timing, per
 * candidate and `reps` times each on the finest level (conductivity must be
 * loaded): eight complex64 iterations of the plan's Krylov solver (BiCGStab,
 * GPBiCG, COCR; other solvers an operator plus a multi-colour SSOR
 * application), and an operator plus an SSOR application in complex128.  No counterpart in
 * the reference.  The choices are returned in *vs32, *vs64 (optional). */
int sfdx_plan_autotune(sfdx_plan* plan, int reps, int* vs32, int* vs64);
/* Relative residual history of the finest-level solve of the last sfdx_plan_solve,
 * hist[nf*2][maxit] (system 2f + pol), the value at iteration i (0-based, counted
 * over all restart cycles) where the host checked it -- every 8th iteration and at
 * the end -- and 0 elsewhere: the .ccv history of Bicg_stab_p / pgpbicg
 * (solvers.f90:687-704) at the library's check points.  Write it with
 * sfdx_write_ccv, which keeps the non-zero entries. */
int sfdx_plan_history(const sfdx_plan* plan, double* hist, int maxit);
/* Wall time (ms) of each level of the last solve, coarsest first (n >= levels). */
int sfdx_plan_level_times(const sfdx_plan* plan, double* ms, int n);
/* Solution of one of the two levels below the finest from the last EXCMG solve
 * (level = levels-2 or levels-1, 1-based, coarsest = 1), host ex[nf][2][nl_level]
 * complex.  With 3 levels these are the two coarse solves that replace the
 * reference's PARDISO calls (u1u2, fdfe_main.f90:1228-1256), the inputs of the
 * extrapolation of the finest guess (extint_v).  SFDX_ERR_ARG for another
 * level, a plain (fwd_acc = 0) solve, or a conductivity loaded since. */
int sfdx_plan_level_fields(sfdx_plan* plan, int level, double* ex);
void sfdx_plan_destroy(sfdx_plan* plan);

/* ------------------------------------------------------------------------
 * Impedances at the receivers.  Replaces post_process + arho_interp2
 * (fdfe_main.f90:549-790).  recv: Fortran recv(nrec,3) = C [3][nrec].
 * out[nf][nrec][4]: out_type 0/1 -> (Re Zxy, Im Zxy, Re Zyx, Im Zyx),
 * out_type 2 -> (rho_xy, rho_yx, phi_xy, phi_yx); out_type 3 (no counterpart in
 * the reference, which forms Zxy and Zyx only) -> out[nf][nrec][8], the full
 * tensor (Re, Im) of Zxx, Zxy, Zyx, Zyy.  tipper (optional)
 * [nf][nrec][4] = (Re Tx, Im Tx, Re Ty, Im Ty).  The receiver stencil follows
 * SFDX_QUIRK_RX_TRANSPOSE of `quirks`.
 * ------------------------------------------------------------------------ */
int sfdx_impedance(int nx, int ny, int nz, int nair, const double* a, const double* b, const double* c, int nf,
                   const double* freq, const double* ex, int nrec, const double* recv, int out_type, int quirks,
                   double* out, double* tipper);
/* Impedances with topography: the receivers of each surface column sit on that
 * column's earth surface instead of the flat plane nair (the topo branch of
 * post_process, fdfe_main.f90:604-616, which the shipped driver never reaches
 * because it passes no topo).  abr[6] = (i1, i2, j1, j2, k1, k2), 1-based: the
 * column window and the range of cells searched; topo[(i2-i1+1)(j2-j1+1)] the
 * elevation (m, positive up) of each window column, x fastest.  A column's
 * plane is set by the first cell of k1..k2 whose centre lies at or below -topo:
 * with SFDX_QUIRK_TOPO_PLANE (reference) its lower node plane and the vertical
 * step c(nair+1) for every column, without it its upper node plane (the top of
 * the first earth cell) and the cell below that plane.  Columns outside the
 * window, or with no such cell, use nair.  Other arguments and the output as
 * sfdx_impedance. */
int sfdx_impedance_topo(int nx, int ny, int nz, int nair, const double* a, const double* b, const double* c, int nf,
                        const double* freq, const double* ex, int nrec, const double* recv, int out_type, int quirks,
                        const int* abr, const double* topo, double* out, double* tipper);
/* The surface fields at the receivers from which sfdx_impedance forms Z and the
 * tippers (the arho rows of post_process / arho_interp2, fdfe_main.f90:600-700,
 * 718-790): fields[nf][nrec][2][5] complex (interleaved doubles), (Ex, Ey, Hx,
 * Hy, Hz) of the xy and the yx polarisation; E from the edge averages on the
 * receiver plane, H = curl E / (i w mu), both through the 3x3 receiver
 * stencil (quirks: SFDX_QUIRK_RX_TRANSPOSE as for sfdx_impedance). */
int sfdx_receiver_fields(int nx, int ny, int nz, int nair, const double* a, const double* b, const double* c, int nf,
                         const double* freq, const double* ex, int nrec, const double* recv, int quirks,
                         double* fields);

/* ------------------------------------------------------------------------
 * Component entry points (each one replaces one reference routine; all
 * buffers are host memory, the work runs on the GPU unless noted).
 * ------------------------------------------------------------------------ */

/* mt1d_anl (model_selec.f90:266-401), host FP64: conv is Fortran
 * conv(nz,6); edc, hx: 2nz+2 complex; imp: 4 complex. */
/* Impedance misfit of host fields ex[nf][2][nl] (as sfdx_impedance) against
 * zobs [nf][nrec][4] with weights wts [nf][nrec][2] (null: 1), misfit = sum
 * wxy |Zxy - dxy|^2 + wyx |Zyx - dyx|^2, and (grad not null) its derivative
 * with respect to every edge value, grad[nf][2][nl] complex, in the holomorphic
 * sense (d misfit = 2 Re sum grad dx): the right-hand side of an adjoint solve
 * (see sfdx_plan_misfit_grad).  Host FP64, no device use.  No counterpart in
 * the reference. */
int sfdx_impedance_misfit(int nx, int ny, int nz, int nair, const double* a, const double* b, const double* c,
                          int nf, const double* freq, const double* ex, int nrec, const double* recv, int quirks,
                          const double* zobs, const double* wts, double* misfit, double* grad);
int sfdx_mt1d(double freq, int nz, const double* conv, const double* c, double* edc, double* hx, double* imp);

/* fd_assemb + dcfast as a matrix-free operator (fdfe_main.f90:226-546,
 * zamux div_correc.f90:431-449): y = K x for ns systems interleaved
 * ([nl][ns] complex), system s at frequency freqs[s].  precision selects the
 * FP64 or the complex64 kernel. */
int sfdx_apply_operator(int nx, int ny, int nz, const double* a, const double* b, const double* c,
                        const double* sigma, int ns, const double* freqs, int precision, const double* x, double* y);

/* Right-hand sides of dcfast (fdfe_main.f90:470-524): p1 (xy), p2 (yx),
 * from the 1-D field edc (2nz+2 complex, sfdx_mt1d). */
int sfdx_build_rhs(int nx, int ny, int nz, const double* a, const double* b, const double* c, const double* sigma,
                   double freq, const double* edc, double* p1, double* p2);

/* One application of the edge multigrid V-cycle (precond 'G'; no reference
 * counterpart: pre_type offers SSOR, Jacobi and ILU(0) only,
 * global_para.f90:18) on the finest of `levels` 2x-coarsened meshes:
 * x = M^{-1} y for ns systems (y, x: [nl][ns] complex, freqs[ns]).  precision
 * SFDX_FP64 runs the FP64 V-cycle, SFDX_MIXED the complex64 one of mixed
 * plans (whose nodal steps leave out all-air nodes). */
int sfdx_vcycle_apply(int nx, int ny, int nz, int nair, const double* a, const double* b, const double* c,
                      const double* sigma, int ns, const double* freqs, int levels, int precision, const double* y,
                      double* x);

/* One preconditioner application x = M^{-1} y (replaces ssorfac + lusol,
 * div_correc.f90:171-220 / solvers.f90:721-762, with the multi-colour
 * ordering; 'J' replaces diagcsr). */
int sfdx_precond_apply(int nx, int ny, int nz, const double* a, const double* b, const double* c,
                       const double* sigma, int ns, const double* freqs, int precond, int precision, const double* y,
                       double* x);

/* mesh_coarsen (fdfe_main.f90:18-84): k coarsenings (2^k cells merge per
 * axis); quirk = SFDX_QUIRK_COARSEN_SHIFT bit. */
int sfdx_mesh_coarsen(int nx, int ny, int nz, const double* a, const double* b, const double* c, const double* sigma,
                      int k, int quirks, double* a1, double* b1, double* c1, double* sigma1);

/* extint_v (excmg.f90:9-77): EXCMG guess on the fine level (nx,ny,nz,a1,b1,
 * c1,nair) from the 4h solution u0 and the 2h solution u1; ns systems
 * interleaved. */
int sfdx_prolongate(int nx, int ny, int nz, const double* a1, const double* b1, const double* c1, int nair, int ns,
                    const double* u0, const double* u1, double* u, int quirks);

/* One Krylov solve (Bicg_stab_p solvers.f90:522-719 / pgpbicg :137-315 /
 * the other solver ids) of K x = rhs on one mesh for ns interleaved systems,
 * starting from x.  iters[ns], relres[ns] (true residual) are outputs;
 * history (optional, [ns][itmax]) receives the recurrence residual recorded at
 * the top of each iteration (the .ccv history of solvers.f90:687-704). */
int sfdx_krylov_solve(const sfdx_opts* o, int nx, int ny, int nz, const double* a, const double* b, const double* c,
                      const double* sigma, int ns, const double* freqs, const double* rhs, double* x, double tol,
                      int itmax, int* iters, double* relres, double* history);

/* Divergence correction (div_correc.f90:11-147 with fddc_assemb, isotropic
 * scheme, and Jacobi-PCG :343-402): x += grad(phi), P phi = T x, for ns
 * interleaved systems.  Returns PCG iterations of system 0 in *pcg_iters. */
int sfdx_div_correct(int nx, int ny, int nz, const double* a, const double* b, const double* c,
                     const double* sigma, int ns, double* x, double tol, int* pcg_iters);

/* Consistent gradient-space correction.  No counterpart in the reference; it
 * replaces the divergence correction above where the field must stay a
 * solution of the discrete system: x += G phi with
 * (G^T V Ms G) phi = G^T V (rhs - K x) / (-i w mu), G the nodal gradient
 * (interior nodes), V the edge dual volumes, Ms the mass (conductivity) part
 * of K.  The exact solution is a fixed point; the error's gradient component
 * is removed.  Nodal PCG (Jacobi) to relative tolerance tol, at most maxit
 * iterations (*pcg_iters: the most any system took).  rhs, x: [nl][ns]
 * complex, host. */
int sfdx_grad_correct(int nx, int ny, int nz, const double* a, const double* b, const double* c,
                      const double* sigma, int ns, const double* freqs, const double* rhs, double* x, double tol,
                      int maxit, int* pcg_iters);

/* ------------------------------------------------------------------------
 * Residual without any memory allocation.  No counterpart in the reference:
 * it serves callers that cannot call cudaMalloc -- an application whose GPU
 * memory is owned by its own pool or another runtime, or a loop that must not
 * allocate -- and that already hold the model and the vectors on the device.
 *
 * r = rhs - K x for ns interleaved systems ([nl][ns] complex, DEVICE
 * pointers d_sigma, d_rhs, d_x, d_r owned by the caller; a, b, c, freqs and
 * the output relres[ns] = ||r|| / ||rhs|| are host arrays).  Work is issued
 * on `stream` (a cudaStream_t, null = default stream) and the call returns
 * after it completes.  Nothing is allocated: the tables, per-system state and
 * reduction scratch live in one fixed device array of about 4.4 MB that every
 * GPU that ran this entry point holds until the process exits.  Limits: nx,
 * ny, nz <= SFDX_NOALLOC_MAX_N and ns <= SFDX_NOALLOC_MAX_NS, otherwise
 * SFDX_ERR_NOMEM.  Every call looks up the array's device address
 * (cudaGetSymbolAddress).  With CUDA's default lazy module loading the first
 * call on a device loads this entry point's device code and reserves the
 * array there, so that first call must come before any stream capture on the
 * device, and a caller that gives all device memory to its own pool makes it
 * (any small case) before filling the pool, or sets
 * CUDA_MODULE_LOADING=EAGER.  All calls share the array and leave their data in it: calls
 * that overlap on the GPU race and must be serialised by the caller.  The
 * device vectors d_rhs, d_x, d_r must be 16-byte aligned and d_sigma 8-byte
 * aligned (SFDX_ERR_ARG otherwise, before any device work).
 * ------------------------------------------------------------------------ */
#define SFDX_NOALLOC_MAX_N 1024
#define SFDX_NOALLOC_MAX_NS 64
int sfdx_residual_noalloc(int nx, int ny, int nz, const double* a, const double* b, const double* c,
                          const double* d_sigma, int ns, const double* freqs, const double* d_rhs, const double* d_x,
                          double* d_r, double* relres, void* stream);

/* ------------------------------------------------------------------------
 * Reference file formats (file_opt.f90).  sfdx_read_model allocates nothing:
 * call with null arrays to get the sizes, then again with buffers.
 * ------------------------------------------------------------------------ */
int sfdx_read_sizes(const char* model_name, int* nx, int* ny, int* nz, int* nair, int* nf, int* nrec);
int sfdx_read_model(const char* model_name, const sfdx_opts* o, int* level, double* eps, int* solver, int* out_type,
                    double* a, double* b, double* c, double* sigma, double* freq, double* recv, int* abu);
/* Convergence-history file of one solve, as Bicg_stab_p / pgpbicg write it with
 * output_ccv (solvers.f90:687-704): <model>_<freq e9.2>_<polar>_<tag>.ccv with
 * the iteration count, then each non-zero entry of history[n] in e9.2.  polar
 * "xy" or "yx"; tag the solver name, or "excmg" for EXCMG runs.  The history
 * comes from sfdx_krylov_solve. */
int sfdx_write_ccv(const char* model_name, double freq, const char* polar, const char* tag, int iters,
                   const double* history, int n);
/* Result file <model>.res as output_data writes it (file_opt.f90:131-158): one
 * line per frequency and receiver, "x y z f 0 v1 v2 v3 v4" in
 * 4(e12.5,2x),i1,2x,4(e12.5,2x), with out[nf][nrec][4] from sfdx_impedance;
 * recv is [3][nrec].  sfdx_write_res_tipper appends the tipper block
 * tipper[nf][nrec][4] (Re Tx, Im Tx, Re Ty, Im Ty) in the same format, as the
 * reference does with output_tipper; a null tipper writes the impedances only. */
int sfdx_write_res(const char* model_name, int nf, const double* freq, int nrec, const double* recv,
                   const double* out);
int sfdx_write_res_tipper(const char* model_name, int nf, const double* freq, int nrec, const double* recv,
                          const double* out, const double* tipper);

#ifdef __cplusplus
}
#endif
#endif /* SFDX_H */
