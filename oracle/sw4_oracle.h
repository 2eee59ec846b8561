/*
 * CPU oracle for the sw4lite elastic time step -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's CPU kernels for the hot path, used by
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the checker.
 * The product (sw4lite_gb300/) never links, loads or calls it.
 *
 * Parity pin: tests/test_oracle_pin.py compares every function here with the
 * reference's own kernels compiled from the reference sources into
 * oracle/_ref/libsw4ref.so (built by `make -C oracle ref` where the reference tree
 * exists), and tests/golden/ holds fixtures generated from that library so the pin
 * also travels to machines without the reference tree.
 *
 * Conventions follow the reference: inclusive, 1-based (Fortran-style) bounds
 * [ib,ie]x[jb,je]x[kb,ke] that include 2 ghost points per side; i fastest.
 * `soa` selects the component layout: soa=1 is the reference's "_rev/_indrev"
 * layout u[c*npts + p] (src/rhs4sg_rev.C:60-62), soa=0 the AoS layout u[3*p + c]
 * (src/rhs4sg.C:53).  All arithmetic is IEEE double.
 */
#ifndef SW4G_ORACLE_H
#define SW4G_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* SBP coefficient tables, layout as src/ew-cfromfort.C:1487-1944. */
void sw4o_stencil_coefficients(double acof[384], double ghcof[6], double bope[48], double sbop[5]);

/* Lu = div(sigma(u)) / rho-less, 4th-order SBP (src/rhs4sg_rev.C:44, src/rhs4sg.C:38). */
void sw4o_rhs4sg(int soa, int ifirst, int ilast, int jfirst, int jlast, int kfirst, int klast,
                 int nk, const int onesided[6], const double* acof, const double* bope,
                 const double* ghcof, double* lu, const double* u, const double* mu,
                 const double* la, double h, const double* strx, const double* stry,
                 const double* strz);

/* Pointwise time-level updates (src/ew-cfromfort.C:40-142). */
void sw4o_predfort(int soa, int ib, int ie, int jb, int je, int kb, int ke, double* up,
                   const double* u, const double* um, const double* lu, const double* fo,
                   const double* rho, double dt2);
void sw4o_corrfort(int soa, int ib, int ie, int jb, int je, int kb, int ke, double* up,
                   const double* lu, const double* fo, const double* rho, double dt4);
void sw4o_dpdmtfort(int ib, int ie, int jb, int je, int kb, int ke, const double* up,
                    const double* u, const double* um, double* u2, double dt2i);

/* Supergrid damping, 4th and 6th order (src/ew-cfromfort.C:748-1158). */
void sw4o_addsgd4(int soa, int ifirst, int ilast, int jfirst, int jlast, int kfirst, int klast,
                  double* up, const double* u, const double* um, const double* rho,
                  const double* dcx, const double* dcy, const double* dcz, const double* strx,
                  const double* stry, const double* strz, const double* cox, const double* coy,
                  const double* coz, double beta);
void sw4o_addsgd6(int soa, int ifirst, int ilast, int jfirst, int jlast, int kfirst, int klast,
                  double* up, const double* u, const double* um, const double* rho,
                  const double* dcx, const double* dcy, const double* dcz, const double* strx,
                  const double* stry, const double* strz, const double* cox, const double* coy,
                  const double* coz, double beta);

/* Ghost-point closures (src/ew-cfromfort.C:205-746).  bccnd values are the
 * reference's boundaryConditionType (0 free surface, 1 Dirichlet, 2 supergrid,
 * 3 periodic, others: no-op).  bforce[s] may be NULL when side s has no forcing. */
void sw4o_bcfortsg(int soa, int ib, int ie, int jb, int je, int kb, int ke, const int wind[36],
                   int nx, int ny, int nz, double* u, double h, const int bccnd[6],
                   const double sbop[5], const double* mu, const double* la,
                   double* const bforce[6], const double* strx, const double* stry);

/* Boundary windows (src/EW.C:3347-3444) for one grid with bounds and global sizes;
 * writes wind[36] and npts[6]. */
void sw4o_boundary_windows(int ib, int ie, int jb, int je, int kb, int ke, int nx, int ny,
                           int nz, const int bccnd[6], int wind[36], int npts[6]);

/* Supergrid 1-D profiles along one axis (src/SuperGrid.C:52-198 and the
 * assignment loop src/EW.C:4745-4781): for index q in [first,last],
 * x = (q-1)*h + xmin.  width = gp*h. */
void sw4o_supergrid_profile(int first, int last, double h, double xmin, int left, int right,
                            double x0, double x1, double width, double* dc, double* str,
                            double* corner);

/* Time functions used by grid-point sources (src/time_functions.C:284-319, :1637-1700). */
double sw4o_timefunc(int kind, double freq, double t);     /* kind: 0 Gaussian, 1 C6SmoothBump */
double sw4o_timefunc_tt(int kind, double freq, double t);

/* Forcing: zero F then accumulate every grid-point source (src/EW.C:3085-3124). */
void sw4o_force(int soa, int ib, int ie, int jb, int je, int kb, int ke, double* f, int nsrc,
                const int* src_ijk, const double* src_amp, const double* src_freq,
                const double* src_t0, const int* src_kind, double t, int tt);

/* One full time step for one Cartesian grid, in the reference CPU phase order
 * (src/EW.C:2537-2756): Force, evalRHS, evalPredictor, enforceBC, Force_tt,
 * evalDpDmInTime, evalRHS, evalCorrector, addSuperGridDamping, enforceBC.
 * up receives the new level.  lu, f, uacc are caller-provided work arrays of
 * 3*npts doubles.  Boundary forcing arrays are zero (no point-source-test
 * Dirichlet data). */
typedef struct {
   int ib, ie, jb, je, kb, ke;
   int nx, ny, nz;
   double h, dt;
   int onesided[6];
   int bccnd[6];
   int wind[36];
   double sg_beta; /* supergrid damping coefficient; 0 disables damping */
   int sg_order;   /* 4 or 6 */
   const double *mu, *la, *rho;
   const double *strx, *stry, *strz, *dcx, *dcy, *dcz, *cox, *coy, *coz;
   int nsrc;
   const int* src_ijk;
   const double* src_amp;
   const double* src_freq;
   const double* src_t0;
   const int* src_kind;
} sw4o_problem;

void sw4o_step(const sw4o_problem* p, int soa, double t, double* up, const double* u,
               const double* um, double* lu, double* f, double* uacc);

/* ---- curvilinear grid (sw4_oracle_curv.c) ---- */
/* Curvilinear operator, rhs4sgcurv_rev.C:34 (soa=1) / rhs4sgcurv.C:34 (soa=0);
 * met is 4 components (SoA or AoS as u).  Only onesided[4] (top) is used. */
void sw4o_rhs4sgcurv(int soa, int ib, int ie, int jb, int je, int kb, int ke, const double* u,
                     const double* mu, const double* la, const double* met, const double* jac,
                     double* lu, const int* onesided, const double* strx, const double* stry);
/* Numerical metric from z (EW::metric_rev, curvilinear-c.C:175); -1 if z_r <= 0. */
int sw4o_metric(int soa, int ib, int ie, int jb, int je, int kb, int ke, double h, const double* z,
                double* met, double* jac);
/* z of a curvilinear grid over a Gaussian hill (EW::grid_mapping, EW.C:5694). */
void sw4o_gaussian_hill_z(int ib, int ie, int jb, int je, int kb, int ke, int nz, double h,
                          double zmax, double zeta_break, int order, double amp, double xc,
                          double yc, double lx, double ly, double* z);
/* Curvilinear free-surface ghost plane (EW::freesurfcurvisg_rev, curvilinear-c.C:621). */
void sw4o_freesurfcurvisg(int soa, int ib, int ie, int jb, int je, int kb, int ke, int nz, int side,
                          double* u, const double* mu, const double* la, const double* met,
                          const double* sbop, const double* forcing, const double* strx,
                          const double* stry);
/* Sixth-order curvilinear supergrid damping (EW::addsgd6cfort(_indrev),
 * ew-cfromfort.C:1241, :1405). */
void sw4o_addsgd6c(int soa, int ib, int ie, int jb, int je, int kb, int ke, double* up,
                   const double* u, const double* um, const double* rho, const double* dcx,
                   const double* dcy, const double* strx, const double* stry, const double* jac,
                   const double* cox, const double* coy, double beta);
/* Curvilinear supergrid damping (EW::addsgd4cfort_indrev, ew-cfromfort.C:1323). */
void sw4o_addsgd4c(int soa, int ib, int ie, int jb, int je, int kb, int ke, double* up,
                   const double* u, const double* um, const double* rho, const double* dcx,
                   const double* dcy, const double* strx, const double* stry, const double* jac,
                   const double* cox, const double* coy, double beta);
/* Smallest eigenvalue of a symmetric 3x3 matrix [a00 a01 a02 a11 a12 a22]. */
double sw4o_sym3_min_eig(const double a[6]);
/* Curvilinear time-step limit cfl / sqrt(max eig) (EW::computeDT, EW.C:5066-5125). */
double sw4o_curv_dt(int soa, int ib, int ie, int jb, int je, int kb, int ke, const double* rho,
                    const double* mu, const double* la, const double* met, const double* jac,
                    double cfl);

/* Two-grid step over topography: a curvilinear grid on top of the Cartesian grid
 * of `cart` (whose top side, bccnd[4] = 4, is the interface).  The reference's
 * time loop order for both grids (EW.C:2537-2756) with the curvilinear operator,
 * free surface, damping and the interface copy enforceCartTopo (EW.C:3504). */
typedef struct {
   int ib, ie, jb, je, kb, ke;
   int nx, ny, nz;
   double h;
   int bccnd[6]; /* sides 0-3 as the Cartesian grid, 4 free surface (0), 5 interface (4) */
   int wind[36];
   const double *rho, *mu, *la, *met, *jac;
   const double *strx, *stry, *dcx, *dcy, *cox, *coy;
   /* grid-point sources of the curvilinear grid (as sw4o_problem's) */
   int nsrc;
   const int* src_ijk;
   const double *src_amp, *src_freq, *src_t0;
   const int* src_kind;
} sw4o_curv;

/* cart: arrays up, u, um, lu, f, uacc of the Cartesian grid; c*: the curvilinear
 * grid's (its forcing is zero: sources lie in the Cartesian grid). */
void sw4o_step_topo(const sw4o_problem* cart, const sw4o_curv* cv, double t, double* up,
                    const double* u, const double* um, double* lu, double* f, double* uacc,
                    double* cup, const double* cu, const double* cum, double* clu, double* cf,
                    double* cuacc);
/* enforceCartTopo (EW.C:3504): Cartesian k=-1,0 from curvilinear k=nz-2,nz-1;
 * curvilinear k=nz..nz+2 from Cartesian k=1..3 (SoA, same i,j bounds). */
void sw4o_cart_topo(const sw4o_problem* cart, const sw4o_curv* cv, double* ucart, double* ucurv);

/* ---- discrete adjoint (sw4_oracle_adj.c): grids with zero ghost points ---- */
void sw4o_apply_lt(int ib, int ie, int jb, int je, int kb, int ke, int nz, const double* y,
                   const double* mu, const double* la, double h, const double* strx,
                   const double* stry, const double* strz, double* lt);
void sw4o_sg_adjoint(int ib, int ie, int jb, int je, int kb, int ke, const double* y,
                     const double* rho, const double* dcx, const double* dcy, const double* dcz,
                     const double* strx, const double* stry, const double* strz, const double* cox,
                     const double* coy, const double* coz, double* z);
void sw4o_coef_gradient(int ib, int ie, int jb, int je, int kb, int ke, const double* v,
                        const double* w, double h, const double* strx, const double* stry,
                        const double* strz, double* gmu, double* gla);
/* Free-surface z sides (onesided[4], onesided[5]): G(v, w) including the one-sided
 * rows, and L^T y = D L D^-1 y with D = H W (H the SBP norm weights). */
void sw4o_coef_gradient_fs(int ib, int ie, int jb, int je, int kb, int ke, int nz, const int onesided[6],
                           const double* v, const double* w, double h, const double* strx,
                           const double* stry, const double* strz, double* gmu, double* gla);
void sw4o_apply_lt_fs(int ib, int ie, int jb, int je, int kb, int ke, int nx, int ny, int nz,
                      const int onesided[6], const double* y, const double* mu, const double* la,
                      double h, const double* strx, const double* stry, const double* strz, double* lt);
/* Sixth-order damping: z = SG6^T (y / rho) on I, and its rho gradient term. */
void sw4o_sg6_adjoint(int ib, int ie, int jb, int je, int kb, int ke, const double* y,
                      const double* rho, const double* dcx, const double* dcy, const double* dcz,
                      const double* strx, const double* stry, const double* strz, const double* cox,
                      const double* coy, const double* coz, double* z);
void sw4o_sg6_rho_gradient(int ib, int ie, int jb, int je, int kb, int ke, const double* a1,
                           const double* d, const double* rho, const double* dcx, const double* dcy,
                           const double* dcz, const double* strx, const double* stry,
                           const double* strz, const double* cox, const double* coy,
                           const double* coz, double beta, double* grho);
void sw4o_sg_rho_gradient(int ib, int ie, int jb, int je, int kb, int ke, const double* a1,
                          const double* d, const double* rho, const double* dcx, const double* dcy,
                          const double* dcz, const double* strx, const double* stry,
                          const double* strz, const double* cox, const double* coy,
                          const double* coz, double beta, double* grho);
/* sw4o_step that also returns the predicted level (after its boundary pass) in pred */
void sw4o_step_pred(const sw4o_problem* p, int soa, double t, double* up, const double* u,
                    const double* um, double* lu, double* f, double* uacc, double* pred);

/* Analytic whole-space displacement of one point source in a homogeneous medium
 * (rho, cp, cs) at time t, written SoA over the array [ib,ie]x[jb,je]x[kb,ke]
 * with x=(i-1)h, y=(j-1)h, z=zmin+(k-1)h: the field the reference compares
 * its point-source test against (EW::get_exact_point_source, src/EW.C:3899).
 * moment=0: force (f[0..2]); moment=1: moment tensor m[] = mxx,mxy,mxz,myy,myz,mzz.
 * kind: 0 Gaussian, 1 C6SmoothBump, 3 VerySmoothBump (as sw4o_timefunc).
 * Points closer than 1e-3 h to the source get 0, as in the reference. */
void sw4o_exact_point_source(int ib, int ie, int jb, int je, int kb, int ke, double h, double zmin,
                             double rho, double cp, double cs, double x0, double y0, double z0,
                             int moment, const double* f, const double* m, int kind, double freq,
                             double t0, double t, double* u);

/* Error norms of u against uex (SoA) over [imin,imax]x[jmin,jmax]x[kmin,kmax],
 * skipping points within `radius` of (x0,y0,z0) (radius < 0: skip none):
 * li = max |u - uex|, l2 = sqrt(sum h^3 (u - uex)^2), xli = max(0, max uex)
 * (EW::solerr3fort, src/ew-cfromfort.C:144, and the square root taken in
 * EW::normOfDifference, src/EW.C:4537-4600). */
void sw4o_solerr3(int ib, int ie, int jb, int je, int kb, int ke, double h, double zmin,
                  const double* uex, const double* u, double x0, double y0, double z0,
                  double radius, int imin, int imax, int jmin, int jmax, int kmin, int kmax,
                  double* li, double* l2, double* xli);

/* Source discretisation on a Cartesian grid (sw4_oracle_src.c; restates the
 * Cartesian branch of Source::set_grid_point_sources4, src/Source.C:1074-1930, and
 * the weights of src/Source.C:553-679).  which: 0 delta, 1 delta', 2 and 3 their
 * five-point free-surface variants.  Returns the number of grid-point sources
 * written (ijk[3n] 1-based, amp[3n]), or -1 if more than cap. */
void sw4o_source_weights(int which, double a, double w[6]);
int sw4o_discretize_source(int nx, int ny, int nz, double h, double zmin, int top_onesided,
                           int bot_onesided, double x, double y, double z, int is_moment,
                           const double f[3], const double m[6], int cap, int* ijk, double* amp);

#ifdef __cplusplus
}
#endif
#endif
