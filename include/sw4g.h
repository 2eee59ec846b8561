/*
 * sw4g -- C ABI of the GB300 (sm_103a) elastic-wave time step.
 *
 * Drop-in boundary for the Scheme, Supergrid, BC-phys and Forcing phases of
 * sw4lite's time loop.  Conventions are the reference's:
 *   - inclusive, 1-based (Fortran-style) array bounds ifirst..ilast etc. that
 *     include 2 ghost points per side, i fastest;
 *   - `soa` selects the component layout of 3-component fields: 1 is the
 *     reference's corder=1 layout u[c*npts + p] (the *_rev / *_indrev kernels),
 *     0 the AoS layout u[3*p + c];
 *   - all field pointers are DEVICE pointers owned by the caller unless a
 *     function says otherwise; small tables (wind, bccnd, onesided, sbop) are
 *     host pointers;
 *   - `stream` is a cudaStream_t (NULL = legacy default stream).  The
 *     kernel-level and phase-level calls only enqueue work on it: they never
 *     synchronise the host and never allocate.  The time-loop object
 *     (sw4g_ew_*) allocates its device state when it is created and when a
 *     call sizes it (receivers, sources, the gradient's checkpoint and segment
 *     buffers); the calls that synchronise or allocate say so.
 * Every function returns an sw4g_status (0 = success); none aborts or exits,
 * where the reference would CHECK_ERROR -> exit(0) or MPI_Abort.
 */
#ifndef SW4G_H
#define SW4G_H

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
   SW4G_OK = 0,
   SW4G_BAD_ARGUMENT = 1,
   SW4G_CUDA_ERROR = 2,
   SW4G_NAN_DETECTED = 3,
   SW4G_NOT_SUPPORTED = 4,
   SW4G_TIMEOUT = 5,
   SW4G_IO_ERROR = 6
} sw4g_status;

/* Library version string. */
const char* sw4g_version(void);
/* Human-readable text for a status code. */
const char* sw4g_status_string(int status);

/* SBP operator tables (host arrays), layout of EW::GetStencilCoefficients
 * (src/ew-cfromfort.C:1487): acof[384], ghcof[6], bope[48], sbop[5]. */
int sw4g_stencil_coefficients(double* acof, double* ghcof, double* bope, double* sbop);

/* ---------------------------------------------------------------------------
 * Kernel-level entry points (one reference kernel each)
 * ------------------------------------------------------------------------- */

/* Lu = div(sigma(u)) with supergrid stretching; replaces rhs4sg / rhs4sg_rev
 * (src/EW.C:141-149, src/rhs4sg.C:38, src/rhs4sg_rev.C:44).  The SBP tables
 * acof/bope/ghcof of the reference signature are fixed constants of the scheme
 * and are held on the device by the library.  onesided[6] is a host array;
 * only onesided[4] (top) and onesided[5] (bottom) are used.  Only the interior
 * i,j in [first+2, last-2] and k rows are written, as in the reference. */
int sw4g_rhs4sg(int soa, int ifirst, int ilast, int jfirst, int jlast, int kfirst, int klast,
                int nk, const int* onesided, double* lu, const double* u, const double* mu,
                const double* lambda, double h, const double* strx, const double* stry,
                const double* strz, void* stream);

/* up = 2u - um + dt2/rho (lu + fo) over all points; replaces EW::predfort
 * (src/ew-cfromfort.C:70). */
int sw4g_predfort(int soa, int ib, int ie, int jb, int je, int kb, int ke, double* up,
                  const double* u, const double* um, const double* lu, const double* fo,
                  const double* rho, double dt2, void* stream);

/* up += dt4/(12 rho) (lu + fo); replaces EW::corrfort (src/ew-cfromfort.C:40). */
int sw4g_corrfort(int soa, int ib, int ie, int jb, int je, int kb, int ke, double* up,
                  const double* lu, const double* fo, const double* rho, double dt4, void* stream);

/* u2 = dt2i (up - 2u + um); replaces EW::dpdmtfort (src/ew-cfromfort.C:116). */
int sw4g_dpdmtfort(int ib, int ie, int jb, int je, int kb, int ke, const double* up,
                   const double* u, const double* um, double* u2, double dt2i, void* stream);

/* 4th-order supergrid damping on up; replaces EW::addsgd4fort / addsgd4fort_indrev
 * (src/ew-cfromfort.C:748, :952). */
int sw4g_addsgd4fort(int soa, int ifirst, int ilast, int jfirst, int jlast, int kfirst, int klast,
                     double* up, const double* u, const double* um, const double* rho,
                     const double* dcx, const double* dcy, const double* dcz, const double* strx,
                     const double* stry, const double* strz, const double* cox, const double* coy,
                     const double* coz, double beta, void* stream);

/* 6th-order supergrid damping; replaces EW::addsgd6fort / addsgd6fort_indrev
 * (src/ew-cfromfort.C:852, :1059). */
int sw4g_addsgd6fort(int soa, int ifirst, int ilast, int jfirst, int jlast, int kfirst, int klast,
                     double* up, const double* u, const double* um, const double* rho,
                     const double* dcx, const double* dcy, const double* dcz, const double* strx,
                     const double* stry, const double* strz, const double* cox, const double* coy,
                     const double* coz, double beta, void* stream);

/* Ghost-point closures; replaces EW::bcfortsg / bcfortsg_indrev
 * (src/ew-cfromfort.C:205, :480).  wind[36], bccnd[6] and sbop[5] are host
 * arrays; bforce[s] (6 device pointers, host array of pointers) may hold NULL
 * entries, read as zero boundary data.  The unused (t, om, ph, cv) arguments
 * of the reference signature are dropped. */
int sw4g_bcfortsg(int soa, int ib, int ie, int jb, int je, int kb, int ke, const int* wind,
                  int nx, int ny, int nz, double* u, double h, const int* bccnd, const double* sbop,
                  const double* mu, const double* lambda, const double* const* bforce,
                  const double* strx, const double* stry, void* stream);

/* ---------------------------------------------------------------------------
 * Curvilinear-grid kernels (topography).  met is the 4-component metric in the
 * same layout as u (soa=1: component-major, met[c*npts + p]; soa=0: met[4p + c]).
 * ------------------------------------------------------------------------- */

/* lu = curvilinear divergence of stress over i,j in [first+2, last-2] and
 * k in [kfirst+2, klast-2], with the SBP top rows k=1..6 when onesided[4] == 1
 * (then kfirst <= 0 and klast >= 8 are required); replaces rhs4sgcurv /
 * rhs4sgcurv_rev (src/EW.C:150-160, src/rhs4sgcurv.C:34, src/rhs4sgcurv_rev.C:34).
 * The SBP tables are the library's own (the reference passes acof/bope/ghcof). */
int sw4g_rhs4sgcurv(int soa, int ifirst, int ilast, int jfirst, int jlast, int kfirst, int klast,
                    const int* onesided, double* lu, const double* u, const double* mu,
                    const double* lambda, const double* met, const double* jac, const double* strx,
                    const double* stry, void* stream);

/* Metric and Jacobian from the grid's z over the whole array (x, y are (i-1)h,
 * (j-1)h); replaces EW::metric / metric_rev (src/curvilinear-c.C:53, :175).
 * Synchronises the stream; SW4G_BAD_ARGUMENT if z_r <= 0 somewhere (the
 * reference returns -1). */
int sw4g_metric(int soa, int ib, int ie, int jb, int je, int kb, int ke, double h, const double* z,
                double* met, double* jac, void* stream);

/* z of a curvilinear grid of nz points over a Gaussian hill
 * -amp*exp(-((x-xc)/lx)^2-((y-yc)/ly)^2) down to z = zmax (SoA scalar array);
 * replaces EW::generate_grid with the analytic topography (src/EW.C:6164,
 * grid_mapping :5694, interpolate_topography :5619-5627). */
int sw4g_gaussian_hill_grid(int ib, int ie, int jb, int je, int kb, int ke, int nz, double h,
                            double zmax, double zeta_break, int order, double amp, double xc,
                            double yc, double lx, double ly, double* z, void* stream);

/* Ghost plane k=0 (side 5) or k=nz+1 (side 6) from the traction condition on a
 * curvilinear grid, i,j in [first+2, last-2]; forcing: 3 x ni x nj point-major
 * device array or NULL; sbop: 5 host doubles; replaces EW::freesurfcurvisg /
 * freesurfcurvisg_rev (src/curvilinear-c.C:465, :621). */
int sw4g_freesurfcurvisg(int soa, int ib, int ie, int jb, int je, int kb, int ke, int nz, int side,
                         double* u, const double* mu, const double* lambda, const double* met,
                         const double* sbop, const double* forcing, const double* strx,
                         const double* stry, void* stream);

/* 4th-order supergrid damping in x and y on a curvilinear grid; replaces
 * EW::addsgd4cfort / addsgd4cfort_indrev (src/ew-cfromfort.C:1160, :1323). */
int sw4g_addsgd4cfort(int soa, int ifirst, int ilast, int jfirst, int jlast, int kfirst, int klast,
                      double* up, const double* u, const double* um, const double* rho,
                      const double* dcx, const double* dcy, const double* strx, const double* stry,
                      const double* jac, const double* cox, const double* coy, double beta,
                      void* stream);
/* 6th-order supergrid damping in x and y on a curvilinear grid; replaces
 * EW::addsgd6cfort / addsgd6cfort_indrev (src/ew-cfromfort.C:1241, :1405). */
int sw4g_addsgd6cfort(int soa, int ifirst, int ilast, int jfirst, int jlast, int kfirst, int klast,
                      double* up, const double* u, const double* um, const double* rho,
                      const double* dcx, const double* dcy, const double* strx, const double* stry,
                      const double* jac, const double* cox, const double* coy, double beta,
                      void* stream);

/* dt = cfl / sqrt(max over the grid of -lambda_min(A)/(4 rho)), the curvilinear
 * limit of EW::computeDT (src/EW.C:5066-5125).  The reference gets lambda_min from
 * LAPACK dspev; here it is the closed form for a symmetric 3x3 matrix.
 * Synchronises the stream. */
int sw4g_curvilinear_time_step(int soa, int ib, int ie, int jb, int je, int kb, int ke,
                               const double* rho, const double* mu, const double* lambda,
                               const double* met, const double* jac, double cfl, double* dt,
                               void* stream);

/* ---------------------------------------------------------------------------
 * Phase-level entry points for the one-sided SBP rows (SoA fields only)
 * ------------------------------------------------------------------------- */

/* Size in doubles of the scratch sw4g_corr_rows needs: the corrector's stage
 * field on 10 planes of the array, 3 components. */
long long sw4g_corr_rows_scratch_len(int ifirst, int ilast, int jfirst, int jlast);

/* Predictor on the 6 one-sided rows next to a free surface, fused with the
 * operator: out = 2u - um + dt^2/rho L(u) at k=1..6 (side 0, top) or nz-5..nz
 * (side 1, bottom), i,j in [first+2, last-2]; forcing is added separately.
 * Replaces rhs4_lowk_pred_gpu / rhs4_highk_pred_gpu (src/device-routines.h:337,
 * :344).  The array must hold planes 0..8 (top) or nz-7..nz+1 (bottom). */
int sw4g_pred_rows(int ifirst, int ilast, int jfirst, int jlast, int kfirst, int klast, int nz,
                   int side, double* out, const double* u, const double* um, const double* mu,
                   const double* lambda, const double* rho, const double* strx, const double* stry,
                   const double* strz, double h, double dt, void* stream);

/* Corrector with 4th-order supergrid damping on the 6 one-sided rows:
 *   out = up + dt^4/(12 rho) L((up - 2u + um)/dt^2) - beta/rho SG(u - um)
 * Replaces rhs4_lowk_corr_gpu / rhs4_highk_corr_gpu (src/device-routines.h:351,
 * :358) together with evalDpDmInTimeCU (src/EW_cuda.C:267) and the supergrid
 * damping of those rows (addSuperGridDampingCU_upper_boundary,
 * src/EW_cuda.C:1420-1466).  `scratch` is a caller-owned device buffer of at
 * least sw4g_corr_rows_scratch_len(...) doubles, overwritten by the call. */
int sw4g_corr_rows(int ifirst, int ilast, int jfirst, int jlast, int kfirst, int klast, int nz,
                   int side, double* out, const double* up, const double* u, const double* um,
                   const double* mu, const double* lambda, const double* rho, const double* strx,
                   const double* stry, const double* strz, const double* dcx, const double* dcy,
                   const double* dcz, const double* cox, const double* coy, const double* coz,
                   double h, double dt, double beta, double* scratch, long long scratch_len,
                   void* stream);

/* sw4g_corr_rows for callers that cannot allocate device memory (no counterpart
 * in the reference).  Some callers may not call cudaMalloc: code holding a host
 * allocator lock, launch-interception tools, frameworks that forbid allocation
 * after start-up.  They cannot hand sw4g_corr_rows its scratch slab, so this
 * entry point keeps the slab in a 64 MiB array of device memory owned by the
 * library (held by every GPU that loads it, until exit) and allocates nothing.
 * Limit: (ilast-ifirst+1)*(jlast-jfirst+1) <= 279,620 points per plane; larger
 * planes return SW4G_BAD_ARGUMENT without device work.  All calls on a device
 * share the array, so calls that overlap on the GPU race; serialise them on
 * one stream.  Every scratch element the call reads it writes first, so the
 * array carries no state between calls.  Every call looks up the array's
 * address (cudaGetSymbolAddress) with the current device, so a device reset
 * between calls does no harm; the first call on a device also loads the
 * library's device code there, so make it before capturing a stream into a
 * CUDA graph. */
int sw4g_corr_rows_noalloc(int ifirst, int ilast, int jfirst, int jlast, int kfirst, int klast,
                           int nz, int side, double* out, const double* up, const double* u,
                           const double* um, const double* mu, const double* lambda,
                           const double* rho, const double* strx, const double* stry,
                           const double* strz, const double* dcx, const double* dcy,
                           const double* dcz, const double* cox, const double* coy,
                           const double* coz, double h, double dt, double beta, void* stream);

/* ---------------------------------------------------------------------------
 * Host-side set-up helpers (no device work)
 * ------------------------------------------------------------------------- */

/* Grid description: one Cartesian grid, 2 ghost points per side. */
typedef struct {
   int nx, ny, nz;    /* interior points per axis */
   double h;          /* grid spacing */
   double zmin;       /* z of the first interior plane */
   int bc[6];         /* per side: 0 free surface, 1 Dirichlet, 2 supergrid, 3 periodic */
   int sg_gp;         /* supergrid layer width in grid points (reference default 20) */
   double sg_damping; /* supergrid damping coefficient (reference default 0.02) */
   int sg_order;      /* damping order, 4 or 6 */
   int soa;           /* must be 1 for the time loop */
   int precision;     /* 0: FP64 throughout.  1: FP32-mixed form -- FP32 fields-in-
                         stencil and material, double-float (FP32 compensated)
                         time-level accumulation, FP64 one-sided SBP rows,
                         free-surface solve and forcing */
} sw4g_grid;

/* Supergrid profiles along one axis of g (0 x, 1 y, 2 z) over the array index
 * range; replaces SuperGrid::dampingCoeff/stretching/cornerTaper sampled as in
 * EW::assign_supergrid_damping_arrays (src/SuperGrid.C:108-198,
 * src/EW.C:4671-4803).  Arrays have n+4 entries for an axis with n points. */
int sw4g_supergrid_profile(const sw4g_grid* g, int axis, double* dc, double* str, double* corner);

/* Boundary windows and point counts; replaces EW::setup_boundary_arrays
 * (src/EW.C:3347). */
int sw4g_boundary_windows(const sw4g_grid* g, int* wind, int* npts);

/* A point source: force (moment == 0) or moment tensor.  kind selects the time
 * function: 0 Gaussian, 1 C6SmoothBump, 2 Ricker, 3 VerySmoothBump. */
typedef struct {
   double x, y, z;
   int moment;
   double fx, fy, fz;
   double mxx, mxy, mxz, myy, myz, mzz;
   double freq, t0;
   int kind;
} sw4g_source;

/* Grid-point sources of one source; replaces Source::set_grid_point_sources4
 * (src/Source.C:1074) for a Cartesian grid.  Writes at most `cap` entries and
 * returns the count through *n (the full count even when it exceeds cap). */
int sw4g_discretize_source(const sw4g_grid* g, const sw4g_source* s, int cap, int* ijk,
                           double* amp, int* n);

/* ---------------------------------------------------------------------------
 * Phase-level driver: the EW time loop on one grid (src/EW.C:2339-2930)
 * ------------------------------------------------------------------------- */
typedef struct sw4g_ew sw4g_ew;

/* mode for sw4g_ew_step */
#define SW4G_MODE_PHASES 0 /* reference phase order, dense Lu/F/Uacc arrays */
#define SW4G_MODE_FUSED 1  /* fused predictor / corrector stage kernels */

int sw4g_ew_create(const sw4g_grid* g, void* stream, sw4g_ew** out);
int sw4g_ew_destroy(sw4g_ew* ew);
/* number of array points (ghosts included) */
long long sw4g_ew_npts(const sw4g_ew* ew);
/* material over the full array: host (on_device=0) or device pointers */
int sw4g_ew_set_material(sw4g_ew* ew, const double* rho, const double* mu, const double* lambda,
                         int on_device);
int sw4g_ew_add_source(sw4g_ew* ew, const sw4g_source* s);
int sw4g_ew_add_grid_point_sources(sw4g_ew* ew, int n, const int* ijk, const double* amp,
                                   const double* freq, const double* t0, const int* kind);
int sw4g_ew_clear_sources(sw4g_ew* ew);
int sw4g_ew_num_grid_point_sources(const sw4g_ew* ew);
/* Where sw4g_ew_add_source computes the grid-point sources (the host loop of
 * Source::set_grid_point_sources4, src/Source.C:1074-1990): on the host (0, the
 * default), or on the device (1), one CTA per source for the whole batch before the
 * next step, grouped by grid point on the device; the same bits either way on a
 * Cartesian grid, the last bits of exp/pow with topography.  SW4G_NOT_SUPPORTED with
 * sources from sw4g_ew_add_grid_point_sources or on a subdomain. */
int sw4g_ew_set_source_discretization(sw4g_ew* ew, int on_device);
int sw4g_ew_set_time_step(sw4g_ew* ew, double dt, double t0);
/* dt from the CFL number, adjusted to end at tmax (EW::computeDT, src/EW.C:5041) */
int sw4g_ew_compute_time_step(sw4g_ew* ew, double cfl, double tmax, double* dt, int* nsteps);
double sw4g_ew_time(const sw4g_ew* ew);
/* CUDA graphs for the fused time loop and the gradient (on != 0): sw4g_ew_step and
   sw4g_ew_gradient then replay captured chunks of steps, bit-identical to direct
   launches; the forcing time and record row are kept in device memory.  Needs an
   explicit (non-default) stream.  No reference counterpart: the reference launches
   each kernel of timesteploop directly (src/EW.C:2537-2756). */
int sw4g_ew_set_graphs(sw4g_ew* ew, int on);
/* current (u) and previous (um) levels, 3*npts each, host or device */
int sw4g_ew_set_fields(sw4g_ew* ew, const double* u, const double* um, int on_device);
int sw4g_ew_get_fields(const sw4g_ew* ew, double* u, double* um, int on_device);
/* device pointer of the current (which=0) or previous (which=1) level */
double* sw4g_ew_field(const sw4g_ew* ew, int which);
/* advance nsteps time steps */
int sw4g_ew_step(sw4g_ew* ew, int nsteps, int mode);
/* Non-finite check of the time loop; replaces the reference's checkfornan option
 * (src/EW.C:1333) with EW::check_for_nan_GPU / check_nan_dev (src/EW_cuda.C:652,
 * src/device-routines.C:8279) after the phases of timesteploop (src/EW.C:2544-2759).
 * every > 0: after every `every`-th step, and after the last step of each
 * sw4g_ew_step call, the new level of every grid is scanned on the device for NaN
 * and infinite values; sw4g_ew_step then synchronises the stream and returns
 * SW4G_NAN_DETECTED after the first checked step that holds one, with the object at
 * that step (the reference prints and goes on).  every = 0 (the default) turns the
 * check off; the time loop then never synchronises. */
int sw4g_ew_set_nan_check(sw4g_ew* ew, int every);
/* The last detection: grid (0 Cartesian, 1 curvilinear, -1 none), the first offending
 * entry in storage order as component c (0-based) and point (i, j, k) in the grid's
 * 1-based bounds, the number of non-finite entries, and the time of that level. */
int sw4g_ew_nan_report(const sw4g_ew* ew, int* grid, int* c, int* i, int* j, int* k,
                       long long* count, double* t);
/* Synchronises the object's stream and returns SW4G_TIMEOUT if one of its kernels
 * gave up a bounded wait since the last call (the FP32-mixed tensor-copy stage
 * kernels wait at most one second for each plane's data; their CTAs then stop and
 * the level they write is incomplete), else SW4G_OK.  sw4g_ew_step with the
 * non-finite check on and sw4g_ew_gradient in the FP32-mixed form report it too. */
int sw4g_ew_status(sw4g_ew* ew);

/* Discrete adjoint (no reference counterpart: sw4lite computes source-parameter
 * gradients only, src/GridPointSource.C:659-760).  Runs nsteps fused FP64 steps
 * from the current levels, recording the receivers (all SW4G_REC_DISPLACEMENT,
 * capacity >= nsteps+1; rows are rewritten from row 0), and returns the misfit
 * J = 1/2 sum_{n=0..nsteps} sum_r |rec^n_r - obs^n_r|^2 (obs: (nsteps+1) x nvals,
 * the record layout) and dJ/drho, dJ/dmu, dJ/dlambda at every array point (npts
 * each), by the exact transpose of the step with checkpoints every
 * checkpoint_every steps.  Device memory: (2*ceil(nsteps/C) + 2*C + 19) levels of
 * 3*npts doubles, plus the segments kept from the forward run (below).  Requires
 * Dirichlet or supergrid sides (zero ghost data) or free-surface z sides (with the z
 * stretching 1 and no z damping on the ten planes next to them, nz >= 22), 4th- or
 * 6th-order damping, no topography.  Receivers may share a grid point.
 * The object ends at the end of the forward run.  It keeps that device memory for its
 * next gradient of the same nsteps, checkpoint interval and receivers; a failed call,
 * sw4g_ew_set_gradient_memory and sw4g_ew_destroy release it. */
int sw4g_ew_gradient(sw4g_ew* ew, int nsteps, int checkpoint_every, const double* observed,
                     int obs_on_device, double* misfit, double* grad_rho, double* grad_mu,
                     double* grad_lambda, int grad_on_device);
/* The forward run of sw4g_ew_gradient keeps every level of its last segment, and of
 * as many segments before it as max_bytes allows (2C+2 levels each), so the backward
 * sweep recomputes only the others from their checkpoints.  max_bytes < 0 (the
 * default): all free device memory but a reserve of max(4 GiB, 1/32 of the device);
 * 0: only the last segment.  Releases the device memory kept from an earlier gradient. */
int sw4g_ew_set_gradient_memory(sw4g_ew* ew, long long max_bytes);

/* Restart files in the reference's checkpoint format (CheckPoint::write_checkpoint,
 * src/CheckPoint.C:251-370, and read_checkpoint, :373-470): precision 8, the number of
 * grids, the current level's time, the cycle, per grid {1, nx, 1, ny, 1, nz}, then per
 * grid the previous and the current level at the interior points, components
 * fastest.  Reading checks the grids, sets both levels, fills their ghost points from
 * the boundary conditions (as src/EW.C:2403-2415) and the time; a restarted run
 * continues bit for bit.  SW4G_IO_ERROR on a file error. */
int sw4g_ew_write_checkpoint(sw4g_ew* ew, const char* path, int cycle);
int sw4g_ew_read_checkpoint(sw4g_ew* ew, const char* path, int* cycle);

/* ---------------------------------------------------------------------------
 * Domain decomposition: subdomains and halo exchange
 * ------------------------------------------------------------------------- */

/* Elements (doubles) of one side's halo of a 3-component FP64 field along axis 0 (x)
 * or 1 (y): the 2 planes next to the side over the full extent of the other two
 * axes, ghosts included; -1 for bad bounds.  With sw4g_halo_pack / _unpack, replaces
 * the reference's halo packing (EW::pack_HaloArrayCU_X/Y and unpack_HaloArrayCU_X/Y,
 * src/EW_cuda.C:1515-1698) for one side: pack copies the two interior planes next
 * to side (0 low, 1 high) into buf, unpack copies buf into that side's two ghost
 * planes (the neighbour's interior planes across the shared side). */
long long sw4g_halo_len(int ifirst, int ilast, int jfirst, int jlast, int kfirst, int klast, int axis);
int sw4g_halo_pack(int soa, int ifirst, int ilast, int jfirst, int jlast, int kfirst, int klast,
                   int axis, int side, const double* u, double* buf, void* stream);
int sw4g_halo_unpack(int soa, int ifirst, int ilast, int jfirst, int jlast, int kfirst, int klast,
                     int axis, int side, const double* buf, double* u, void* stream);

/* The EW object of the subdomain of the global grid g whose interior points are
 * i0..i1 x j0..j1 (1-based, global; all nz planes), on the current device: the
 * reference's per-rank grid of its 2-D (i, j) decomposition (src/EW.C:1921-1949).
 * Sides shared with a neighbour get no boundary closure (bProcessor); the supergrid
 * profiles are the global grid's, and sources are discretised on the global grid
 * and kept on this subdomain's interior points, so the subdomains of a grid
 * reproduce the undivided run.  Material, levels and receivers are the
 * subdomain's own arrays (nx = i1-i0+1, ny = j1-j0+1, 2 ghost points per side, the
 * ghost planes at shared sides holding the neighbours' values).  Periodic axes
 * cannot be divided (SW4G_NOT_SUPPORTED). */
int sw4g_ew_create_subdomain(const sw4g_grid* g, int i0, int i1, int j0, int j1, void* stream,
                             sw4g_ew** out);
/* One fused step of a subdomain in three parts; after part 0 and after part 1 the
 * caller exchanges the halos of the level the part left (the reference's exchange
 * points after the predictor and after the corrector, src/EW.C:2596-2616,
 * 2728-2744): x sides first, then y sides.  Parts run in the order 0, 1, 2. */
int sw4g_ew_step_part(sw4g_ew* ew, int part);
/* Bytes of one side's halo along axis in the object's level format (FP64 or the
 * FP32-mixed form's double-float pairs); pack / unpack that side of the level to
 * exchange to / from a device buffer of that size on the object's stream. */
long long sw4g_ew_halo_bytes(const sw4g_ew* ew, int axis);
int sw4g_ew_halo_pack(sw4g_ew* ew, int axis, int side, void* buf);
int sw4g_ew_halo_unpack(sw4g_ew* ew, int axis, int side, const void* buf);
/* nsteps steps of n subdomains in lockstep inside one process, with the halo
 * exchanges between them: neighbors[4 s + q] is the subdomain across side q (x-low,
 * x-high, y-low, y-high) of subdomain s, or -1 for a physical side.  The subdomains
 * may sit on different GPUs: halos travel by device-to-device copies into the
 * receiving GPU's own memory, ordered by events on the objects' streams (the
 * reference's MPI Sendrecv of packed halos, src/EW_cuda.C:1699-1900). */
int sw4g_ew_step_group(sw4g_ew* const* subs, int n, const int* neighbors, int nsteps);

/* Topography (replaces the reference's topography + curvilinear grid set-up,
 * src/EW.C:540-720 (deck), 2018-2046 (dimensions), 6164 (generate_grid), 6229
 * (setup_metric), and the curvilinear grid's share of every phase of the time
 * loop).  A Gaussian hill z_s = -amp exp(-((x-xc)/lx)^2 - ((y-yc)/ly)^2) is
 * meshed by a curvilinear grid from z_s down to the Cartesian grid's zmin (the
 * reference's topography zmax); zeta_break and order as the reference's
 * topography options (defaults 0.95 and 4). */
typedef struct sw4g_topography {
   double amp, xc, yc, lx, ly;
   double zeta_break;
   int order;
} sw4g_topography;
/* An EW object with a curvilinear grid (grid 1) over topography t on top of the
 * Cartesian grid g (grid 0), whose bc[4] must be SW4G_BC_INTERFACE.  The
 * curvilinear grid has g's nx, ny and nz = 1 + round((zmin - z_avg)/h) points,
 * z_avg the midpoint of the topography's z range (src/EW.C:2039-2044).  FP64,
 * 4th-order damping; sources anywhere below the topography.  SW4G_BAD_ARGUMENT
 * if the grid folds (topography too steep for h). */
#define SW4G_BC_INTERFACE 4
int sw4g_ew_create_topo(const sw4g_grid* g, const sw4g_topography* t, void* stream, sw4g_ew** out);
/* Grid-point sources of one source on the two grids of g and t (the curvilinear grid:
 * nzc planes, Jacobian jac over its array with 2 ghost points per side, host), as
 * Source::set_grid_point_sources4 with the curvilinear branches (src/Source.C:1074-1990):
 * at or above the interface the source goes to the curvilinear grid, below it to the
 * Cartesian grid, and a stencil that reaches across the interface is split.  Up to
 * cap entries per grid; the counts come back in *ncart, *ncurv.  SW4G_BAD_ARGUMENT
 * for a source above the topography. */
int sw4g_discretize_source_topo(const sw4g_grid* g, const sw4g_topography* t, int nzc,
                                const double* jac, const sw4g_source* s, int cap, int* cart_ijk,
                                double* cart_amp, int* ncart, int* curv_ijk, double* curv_amp,
                                int* ncurv);
/* The grid-point sources an EW object holds for grid 0 or 1 (host copy, up to cap). */
int sw4g_ew_grid_point_sources(const sw4g_ew* ew, int grid, int cap, int* ijk, double* amp, int* n);
/* 1, or 2 with topography */
int sw4g_ew_num_grids(const sw4g_ew* ew);
int sw4g_ew_grid_dims(const sw4g_ew* ew, int grid, int* nx, int* ny, int* nz, long long* npts);
int sw4g_ew_set_material_grid(sw4g_ew* ew, int grid, const double* rho, const double* mu,
                              const double* lambda, int on_device);
int sw4g_ew_set_fields_grid(sw4g_ew* ew, int grid, const double* u, const double* um,
                            int on_device);
int sw4g_ew_get_fields_grid(const sw4g_ew* ew, int grid, double* u, double* um, int on_device);
/* z (npts), metric (4 x npts, component-major) and Jacobian (npts) of grid 1 */
int sw4g_ew_curvilinear_arrays(const sw4g_ew* ew, double* z, double* met, double* jac,
                               int on_device);

/* Receivers (replace TimeSeries + EW::extractRecordData, src/EW.C:5854-6072, and the
 * per-step recording in the time loop, src/EW.C:2485-2500 and 2797-2835).
 * Record modes are numbered as TimeSeries::receiverMode (src/TimeSeries.h:52);
 * values per receiver and step: */
#define SW4G_REC_DISPLACEMENT 0 /* 3: ux, uy, uz */
#define SW4G_REC_DIV 1          /* 1 */
#define SW4G_REC_CURL 2         /* 3 */
#define SW4G_REC_STRAINS 3      /* 6: xx, yy, zz, xy, xz, yz */
#define SW4G_REC_VELOCITY 4     /* 3: (u^{n+1} - u^{n-1}) / (2 dt) */
#define SW4G_REC_GRADIENT 5     /* 9: du_c/dx_a, c-major */
/* Nearest grid point of (x, y, z) on one Cartesian grid, as
 * EW::computeNearestGridPoint (src/EW.C:5149).  ijk receives 1-based indices;
 * SW4G_BAD_ARGUMENT if the point is outside the interior. */
int sw4g_nearest_grid_point(const sw4g_grid* g, double x, double y, double z, int* ijk);
/* Sets n receivers at grid points ijk[3n] with modes mode[n] and allocates a device
 * record array of `capacity` rows.  The first step after this call first writes the
 * initial data (velocity entries of that row are 0: the reference records no
 * velocity for it), then every step appends one row of all receivers' values in
 * receiver order.  A step that would overflow the array returns SW4G_BAD_ARGUMENT
 * before doing anything.  n = 0 removes the receivers. */
int sw4g_ew_set_receivers(sw4g_ew* ew, int n, const int* ijk, const int* mode, int capacity);
/* As sw4g_ew_set_receivers, each receiver on grid grid[r]: 0 the Cartesian grid, 1 the
 * curvilinear grid of an object with topography (grid may be NULL: all on grid 0).
 * On the curvilinear grid the derivative modes use the metric at the receiver's
 * point as the reference's curvilinear branches of EW::extractRecordData
 * (src/EW.C:5882-6068). */
int sw4g_ew_set_receivers_grid(sw4g_ew* ew, int n, const int* ijk, const int* mode, const int* grid,
                               int capacity);
/* The grid point (ijk, 1-based) and grid of a receiver at (x, y, z) on this object's
 * grids: EW::computeNearestGridPoint (src/EW.C:5149-5213) with TimeSeries' placement on
 * the curvilinear grid (src/TimeSeries.C:139-168, :307-329): (i, j) nearest, a point
 * half-way going to the lower index; below the interface (z > zmin) the Cartesian k;
 * at or above it the curvilinear k = round(s) of the inverted grid mapping, limited to
 * 1..nz, or 1 where the mapping cannot be inverted.  SW4G_BAD_ARGUMENT above the
 * topography (allowance 1e-9) or outside the grids; SW4G_NOT_SUPPORTED on a
 * subdomain object. */
int sw4g_ew_nearest_grid_point(const sw4g_ew* ew, double x, double y, double z, int* ijk, int* grid);
/* z of the topography surface at (x, y), 0 without topography: a receiver or source
 * given by its depth below the surface lies at z = depth + this (the reference's
 * topodepth, src/TimeSeries.C:145-150; EW::find_topo_zcoord_owner, src/EW.C:6311). */
int sw4g_ew_topography_z(const sw4g_ew* ew, double x, double y, double* z);
/* rows written so far and values per row */
int sw4g_ew_record_shape(const sw4g_ew* ew, int* rows, int* nvals);
/* copies rows x nvals doubles (row-major) to host (on_device=0) or device memory */
int sw4g_ew_get_records(const sw4g_ew* ew, double* out, int on_device);
/* Receiver files.  The grid's geographic mapping: the members of EW that
 * EW::computeGeographicCoord reads (src/EW.C:5794-5816; defaults src/EW.C:192-197). */
typedef struct {
   double lon_origin, lat_origin; /* degrees, at x = y = 0 */
   double az;                     /* grid azimuth, degrees (mGeoAz) */
   double meters_per_degree;
   double meters_per_longitude;   /* used when const_meters_per_longitude != 0 */
   int const_meters_per_longitude;
} sw4g_geo;
/* The reference's defaults: lon -118, lat 37, az 0, 111319.5 m per degree,
 * 87721 m per degree of longitude (not constant). */
int sw4g_geo_default(sw4g_geo* geo);
/* longitude and latitude of grid point (x, y); replaces EW::computeGeographicCoord
 * (src/EW.C:5794) for the spheroidal mapping (no proj4 projection). */
int sw4g_geographic_coord(const sw4g_geo* geo, double x, double y, double* lon, double* lat);
/* One receiver's file: what a TimeSeries holds besides its records. */
typedef struct {
   const char* station; /* written as "# Station:" (TimeSeries::m_fileName) */
   double x, y;         /* requested location, m */
   double gp_x, gp_y;   /* location of the grid point that records, m */
   int utc[7];          /* year, month, day, hour, minute, second, millisecond */
   int mode;            /* SW4G_REC_*: the columns */
   int xyz;             /* 1: grid components; 0: east-west, north-south, up-down */
   double t_shift, dt;  /* row r is at time t_shift + r dt */
} sw4g_usgs_station;
/* Writes `rows` record rows of one receiver in the USGS text format of
 * TimeSeries::write_usgs_format (src/TimeSeries.C:924-1056), byte for byte: the
 * header, then per row the time and the mode's values.  rec points at the
 * receiver's first value of row 0; its values are consecutive and rows are
 * row_stride doubles apart (the record array of sw4g_ew_get_records on the host:
 * row_stride = nvals, rec offset by the values of the receivers before it).  With
 * xyz = 0, displacement and velocity are rotated to east-west, north-south and
 * up-down as the reference does; for the other modes (curl, strains, gradient) the
 * reference writes the header alone, and so does this function, returning
 * SW4G_NOT_SUPPORTED.  SW4G_IO_ERROR if the file cannot be written. */
int sw4g_write_usgs(const char* path, const sw4g_geo* geo, const sw4g_usgs_station* st,
                    const double* rec, long long rows, long long row_stride);
/* The event a SAC header names (EVLA, EVLO, EVDP, O). */
typedef struct {
   double lat, lon;    /* degrees */
   double depth;       /* m (written in km) */
   double time_offset; /* s */
} sw4g_sac_event;
/* Writes one receiver's records as binary SAC files, one per value of the mode,
 * named prefix + the reference's suffix (x y z, e n u, xv yv zv, ev nv uv, div,
 * curlx.., xx yy zz xy xz yz, duxdx..duzdz); replaces the SAC branch of
 * TimeSeries::writeFile (src/TimeSeries.C:416-822) with write_sac_format (:826) and
 * its SAC header library (src/sacsubc.C: newhdr, scmxmn, bwsac).  The values are
 * written as FP32 (the reference's mRecordedFloats), the header holds their
 * extrema and mean, the time axis (t_shift, dt), the UTC fields with the day of
 * the year, the station's latitude and longitude, the event, the component's name,
 * inclination and azimuth, and KSTNM = st->station.  With xyz = 0 displacement,
 * velocity and curl are rotated as in the USGS writer.  flush_subnormals = 1 writes
 * samples that round to an FP32 subnormal as signed zeros, as builds with
 * flush-to-zero arithmetic do (the reference's stored LOH.1 h=100 traces); 0 keeps
 * IEEE rounding (its stored LOH.2 traces, a default gcc build).  Little-endian
 * words, as the reference's fwrite of its header struct on x86_64 and aarch64. */
int sw4g_write_sac(const char* prefix, const sw4g_geo* geo, const sw4g_usgs_station* st,
                   const sw4g_sac_event* ev, const double* rec, long long rows, long long row_stride,
                   int flush_subnormals);
/* boundary conditions of this grid on a caller's 3-component device array */
int sw4g_ew_enforce_bc(sw4g_ew* ew, double* u);
/* kernel launches one step enqueues */
int sw4g_ew_launches_per_step(const sw4g_ew* ew, int mode);
#ifdef __cplusplus
}
#endif
#endif
