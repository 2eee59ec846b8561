// Host-side launchers of the sm_103a kernels.  Every launcher enqueues on the
// given stream, allocates nothing and returns a Status code (common.cuh).
#pragma once

#include <cuda_runtime.h>

#include "common.cuh"

namespace sw4g {

// Precomputed second-difference weights: slot axis*4 + type*2 + n, with type 0
// for mu*s and 1 for (2mu+lambda)*s, n 0 for W1 and 1 for W2 (stage_fused.cu).
constexpr int kWeightArrays = 12;
// s[ax*2 + t] = W1(p) + W2(p) + W2(p+o) + W1(p+2o), the sum of the four weights a
// point's second difference along ax applies (t: 0 mu s, 1 (2mu+la) s)
constexpr int kWeightSums = 6;
struct WeightPtrs {
   double* p[kWeightArrays];
   double* s[kWeightSums];
};

// One fused stage launch over the centred rows [k1,k2] of a SoA grid.
struct FusedStage {
   Box b;
   int k1 = 0, k2 = -1;
   int corrector = 0;  // 0 predictor, 1 corrector, 2 adjoint stage (stage_fused.cu)
   int kchunk = 0;  // planes per CTA; 0 picks one
   const double* u = nullptr;
   const double* um = nullptr;
   const double* up = nullptr;
   double* out = nullptr;
   const double* mu = nullptr;
   const double* la = nullptr;
   const double* rho = nullptr;
   const double* irho = nullptr;
   WeightPtrs w{};
   const double* st[3] = {nullptr, nullptr, nullptr};
   const double* dc[3] = {nullptr, nullptr, nullptr};
   const double* co[3] = {nullptr, nullptr, nullptr};
   double h = 1, dt = 0, beta = 0;
   double coef = 0;  // > 0: the L(.) coefficient instead of dt^2 (dt^2/12 corrector)
   int* emax = nullptr;  // corrector: atomicMax of the exponent fields of the level written
};

// (hi, lo) pairs interleaved: one 8-byte load per coefficient
struct WeightPtrsDF {
   float2* p[kWeightArrays];
};

// One mixed-form stage launch (stage_mixed.cu): double-float levels (hi at
// [c*npts+p], lo 3*npts further), FP32 material and profiles.
struct MixedStage {
   Box b;
   int k1 = 0, k2 = -1;
   int corrector = 0;
   const float* u = nullptr;
   const float* um = nullptr;
   const float* up = nullptr;
   float* out = nullptr;
   const float2* mu2 = nullptr;  // interleaved (hi, lo) pairs of mu, lambda and 1/rho
   const float2* la2 = nullptr;
   const float2* ir2 = nullptr;
   const float* rho = nullptr;
   const float2* w2[kWeightArrays] = {};
   const float* st[3] = {nullptr, nullptr, nullptr};
   const float* dc[3] = {nullptr, nullptr, nullptr};
   const float* co[3] = {nullptr, nullptr, nullptr};
   double h = 1, dt = 0, beta = 0;
   // corrector 0 predictor, 1 corrector, 2 adjoint form (stage_mixed.cu); coef != 0
   // replaces the stage's dt^2 (predictor, adjoint) or dt^2/12 (corrector)
   double coef = 0;
   // device status word: the tensor-copy kernels or in 1 << kTimeout when an
   // mbarrier wait gives up (may be null)
   int* status = nullptr;
};

// Device-resident grid-point sources grouped by grid point: the sources of point
// r are [start[r], start[r+1]); all share ijk[3*start[r] .. +2].
struct SourceSet {
   int npoints = 0;
   int nsources = 0;
   const int* start = nullptr;   // npoints+1
   const int* ijk = nullptr;     // 3*nsources
   const double* amp = nullptr;  // 3*nsources
   const double* freq = nullptr; // nsources
   const double* t0 = nullptr;   // nsources
   const int* kind = nullptr;    // nsources
};

__host__ __device__ double timefunc(int kind, double freq, double t, bool tt);

// Receiver record modes, numbered as the reference's TimeSeries::receiverMode
// (src/TimeSeries.h:52).
enum RecMode : int {
   kRecDisplacement = 0,
   kRecDiv = 1,
   kRecCurl = 2,
   kRecStrains = 3,
   kRecVelocity = 4,
   kRecGradient = 5,
};

// Device-resident receivers: grid point and mode of each, and the offset of its
// values within one record row.
struct ReceiverSet {
   int n = 0;
   const int* ijk = nullptr;   // 3*n
   const int* mode = nullptr;  // n
   const int* off = nullptr;   // n
   const int* grid = nullptr;  // n: 0 Cartesian, 1 curvilinear; null: all Cartesian
};

// The curvilinear grid's arrays for receivers on it: its box, the two levels (FP64,
// or (hi, lo) FP32 pairs in the mixed form), the metric (4 x npts) and Jacobian.
struct RecCurv {
   Box b{};
   const void* up = nullptr;
   const void* um = nullptr;
   const double* met = nullptr;
   const double* jac = nullptr;
};

// A curvilinear grid's arrays for the curvilinear kernels (curv.cu): 3-component
// field u and 4-component metric met in the same layout (soa: component-major).
struct CurvSpec {
   int soa = 1;
   int ib = 0, ie = 0, jb = 0, je = 0, kb = 0, ke = 0;
   const double* u = nullptr;
   const double* mu = nullptr;
   const double* la = nullptr;
   const double* met = nullptr;
   const double* jac = nullptr;
   const double* strx = nullptr;
   const double* stry = nullptr;
};

int launch_rhs4sgcurv(const CurvSpec& s, const int onesided[6], double* lu, cudaStream_t st);
// only the SBP top rows k = 1..6 of the curvilinear operator
int launch_rhs4sgcurv_top(const CurvSpec& s, double* lu, cudaStream_t st);

// Time-invariant coefficients of the fused curvilinear stage (curv_stage.cu):
// 20 second-difference weight arrays, 8 cross-term products, K = sx sy/(J rho),
// rho J and 1/(rho J).
struct CurvCoef {
   double* w[20];
   double* prod[8];
   double* K;
   double* rj;
   double* irj;
   double* topw;  // acof-contracted r-r coefficients of the top rows, per column
};
long long curv_coef_doubles(long long npts, long long ncol);
int curv_coef_setup(const Box& b, const double* mu, const double* la, const double* rho,
                    const double* met, const double* jac, const double* sx, const double* sy,
                    double* store, CurvCoef* c, cudaStream_t s);
// One fused curvilinear stage: rows 7..nz, the SBP top rows k = 1..6 and the
// ghost shell.
struct CurvStage {
   Box b;
   int nz = 0;
   int corrector = 0;
   const double* u = nullptr;
   const double* um = nullptr;
   const double* up = nullptr;
   double* out = nullptr;
   CurvCoef cc{};
   const double *sx = nullptr, *sy = nullptr, *dcx = nullptr, *dcy = nullptr, *cox = nullptr,
                *coy = nullptr;
   // the stage field of the top rows: the grid's u (predictor) or a slab of
   // up - 2u + um over planes kb..8 (corrector), and its array box
   const double* f = nullptr;
   Box fbox;
   // work array of the top rows: 36 x (columns of the grid) doubles
   double* scratch = nullptr;
   double dt = 0, beta = 0;
};
// part 0: the whole stage; 1: the ghost shell and the SBP top rows k = 1..6 alone (with
// ctas > 0 the top rows as a persistent grid of that many CTAs); 2: the stage kernel
// of rows 7..nz alone.  Parts 1 and 2 write disjoint points from the same inputs.
int launch_curv_stage(const CurvStage& st, cudaStream_t s, int part = 0, int ctas = 0);

// The curvilinear coefficients of the FP32-mixed stage as (hi, lo) FP32 pairs:
// products 0..7 as CurvCoef::prod, 8 = (2mu+la) m2 m1, 9 = (2mu+la) m3 m1; the
// twenty second-difference weights x144; K/144; 1/(rho J); rho J in FP32.
struct CurvCoefDF {
   float* ph[10];
   float* pl[10];
   float* wh[20];
   float* wl[20];
   float *Kh, *Kl, *irh, *irl, *rj;
};
long long curv_coef_df_floats(long long npts);
int curv_coef_df_setup(long long npts, const CurvCoef& c, float* store, CurvCoefDF* d, cudaStream_t s);

// One fused curvilinear stage of the FP32-mixed form over double-float levels:
// FP32 interior rows 7..nz, FP64 SBP top rows and the ghost shell.
struct CurvStageDF {
   Box b;
   int nz = 0;
   int corrector = 0;
   const float* u = nullptr;  // double-float levels: hi at [c*npts + p], lo at 3*npts further
   const float* um = nullptr;
   const float* up = nullptr;
   float* out = nullptr;
   CurvCoef cc{};    // FP64 coefficients (top rows)
   CurvCoefDF cd{};  // (hi, lo) coefficients (interior)
   const double *sx = nullptr, *sy = nullptr, *dcx = nullptr, *dcy = nullptr, *cox = nullptr,
                *coy = nullptr;
   const float *sx32 = nullptr, *sy32 = nullptr, *dcx32 = nullptr, *dcy32 = nullptr,
               *cox32 = nullptr, *coy32 = nullptr;
   // FP64 work slabs over planes kb..8 (3 x columns x (9 - kb) doubles each): the top
   // rows' stage field (u, or up - 2u + um) and the corrector's u - um; f, fbox and dd
   // are set by launch_curv_stage_df
   double* work1 = nullptr;
   double* work2 = nullptr;
   const double* f = nullptr;
   const double* dd = nullptr;
   Box fbox;
   // work array of the top rows: 36 x (columns of the grid) doubles
   double* scratch = nullptr;
   double dt = 0, beta = 0;
};
int launch_curv_stage_df(const CurvStageDF& st, cudaStream_t s, int part = 0, int ctas = 0);
int launch_curv_top_df(const CurvStageDF& st, cudaStream_t s, int ctas = 0);
int launch_freesurfcurvisg_df(const CurvSpec& s, int nz, int side, const double* sbop, float* uh,
                              cudaStream_t st);
int launch_cart_topo_df(const Box& cart, const Box& curv, int nzc, float* ucart, float* ucurv,
                        cudaStream_t st);
int launch_metric(int soa, int ib, int ie, int jb, int je, int kb, int ke, double h, const double* z,
                  double* met, double* jac, int* bad_flag, cudaStream_t st);
int launch_gaussian_hill_z(int ib, int ie, int jb, int je, int kb, int ke, int nz, double h,
                           double zmax, double zeta_break, int order, double amp, double xc,
                           double yc, double lx, double ly, double* z, cudaStream_t st);
int launch_freesurfcurvisg(const CurvSpec& s, int nz, int side, const double* sbop,
                           const double* forcing, double* u, cudaStream_t st);
int launch_addsgd4c(int soa, int ib, int ie, int jb, int je, int kb, int ke, double* up,
                    const double* u, const double* um, const double* rho, const double* dcx,
                    const double* dcy, const double* strx, const double* stry, const double* jac,
                    const double* cox, const double* coy, double beta, cudaStream_t st);
int launch_cart_topo(const Box& cart, const Box& curv, int nzc, double* ucart, double* ucurv,
                     cudaStream_t st);
int launch_curv_eig(int soa, long long n, const double* rho, const double* mu, const double* la,
                    const double* met, const double* jac, double* blockmax, int nblocks,
                    cudaStream_t st);

int receiver_values(int mode);  // values one receiver records per step (0: bad mode)
// cv: the curvilinear grid's arrays when a receiver lies on it (else null)
int launch_record(const Box& b, const double* up, const double* um, const ReceiverSet& r,
                  double* row, double dt, double h, int initial, cudaStream_t s,
                  const double* clk = nullptr, int nvals = 0, const RecCurv* cv = nullptr);
int launch_record_df(const Box& b, const float* up, const float* um, const ReceiverSet& r,
                     double* row, double dt, double h, int initial, cudaStream_t s,
                     const double* clk = nullptr, int nvals = 0, const RecCurv* cv = nullptr);

int upload_sbp_tables_direct();

int launch_rhs4sg_direct(int soa, int ifirst, int ilast, int jfirst, int jlast, int kfirst,
                         int klast, int nk, const int onesided[6], double* lu, const double* u,
                         const double* mu, const double* la, double h, const double* strx,
                         const double* stry, const double* strz, cudaStream_t stream);

int launch_predfort(int soa, int ib, int ie, int jb, int je, int kb, int ke, double* up,
                    const double* u, const double* um, const double* lu, const double* fo,
                    const double* rho, double dt2, cudaStream_t s);
int launch_corrfort(int soa, int ib, int ie, int jb, int je, int kb, int ke, double* up,
                    const double* lu, const double* fo, const double* rho, double dt4,
                    cudaStream_t s);
int launch_dpdmtfort(int ib, int ie, int jb, int je, int kb, int ke, const double* up,
                     const double* u, const double* um, double* u2, double dt2i, cudaStream_t s);
int launch_addsgd(int order, int soa, int ifirst, int ilast, int jfirst, int jlast, int kfirst,
                  int klast, double* up, const double* u, const double* um, const double* rho,
                  const double* dcx, const double* dcy, const double* dcz, const double* strx,
                  const double* stry, const double* strz, const double* cox, const double* coy,
                  const double* coz, double beta, cudaStream_t s);

int launch_ghost_shell(const Box& b, int corrector, double* out, const double* u,
                       const double* um, const double* up, cudaStream_t s);

int launch_bcfortsg(int soa, int ib, int ie, int jb, int je, int kb, int ke, const int wind[36],
                    int nx, int ny, int nz, double* u, double h, const int bccnd[6],
                    const double sbop[5], const double* mu, const double* la,
                    const double* const bforce[6], const double* strx, const double* stry,
                    cudaStream_t s);

// The ghost plane of one free-surface z side (4 top, 5 bottom) from the homogeneous
// traction condition, on an FP64 level or a double-float level (df).
int launch_free_surface_ghosts(const Box& b, int nz, int side, bool df, void* u, const double* mu,
                               const double* la, const double* strx, const double* stry, double h,
                               const double sbop[5], cudaStream_t s);

int launch_force_dense(int soa, int ib, int ie, int jb, int je, int kb, int ke, double* f,
                       const SourceSet& src, double t, int tt, cudaStream_t s);
// clk (optional): the device clock of a captured time loop, [0] the forcing time,
// [1] the record row, [2] the adjoint residual row (launch_clock_advance adds to each)
int launch_clock_advance(double* clk, double dt, double drow, double dres, cudaStream_t s);
int launch_force_update(int soa, int ib, int ie, int jb, int je, int kb, int ke, double* up,
                        const double* rho, const SourceSet& src, double t, int tt, double coef,
                        cudaStream_t s,
                  const double* clk = nullptr);
int launch_force_update_f32(int soa, int ib, int ie, int jb, int je, int kb, int ke, float* up,
                            const double* rho, const SourceSet& src, double t, int tt,
                            double coef, cudaStream_t s);

int launch_mixed_stage(const MixedStage& st, cudaStream_t stream);
// Sixth-order supergrid damping (damping6.cu): curvilinear FP64 (addsgd6cfort), and
// on double-float levels in FP32 arithmetic for the mixed form, naxes 3 (Cartesian,
// e = rho) or 2 (curvilinear, e = rho J); rho J as FP32 for the latter.
int launch_addsgd6c(const Box& b, double* up, const double* u, const double* um, const double* rho,
                    const double* dcx, const double* dcy, const double* strx, const double* stry,
                    const double* jac, const double* cox, const double* coy, double beta,
                    cudaStream_t s);
int launch_addsgd6_df(int naxes, const Box& b, float* out, const float* u, const float* um,
                      const float* e, const float* const dc[3], const float* const st[3],
                      const float* const co[3], double beta, cudaStream_t s, int adj = 0);
// The transpose of the Cartesian sixth-order damping on the interior points (the
// adjoint's scaled recursion): every point two from the array edges, u - um taken as
// zero outside the points three from every edge; FP64.  The double-float form is
// launch_addsgd6_df with adj = 1.
int launch_addsgd6_adj(const Box& b, double* up, const double* u, const double* um, const double* rho,
                       const double* const dc[3], const double* const st[3], const double* const co[3],
                       double beta, cudaStream_t s);
int launch_rho_jac_f32(long long n, const double* rho, const double* jac, float* e, cudaStream_t s);

// Halo planes of a decomposed grid (halo.cu): the first of the two planes a side
// sends (pack: the interior planes next to it) or receives (the ghost planes), the
// elements of one side's halo, and the pack / unpack of those planes of a field of
// ncomp components of float or double.
int halo_first_plane(const Box& b, int axis, int side, bool pack);
long long halo_len(const Box& b, int axis, int ncomp);
int launch_halo_copy(const Box& b, int axis, int side, bool pack, bool is_float, int ncomp,
                     void* field, void* buf, cudaStream_t s);

// Status block of an EW object (device, 4 words): [0] flags (bit kTimeout: an
// mbarrier wait gave up), [1] non-finite values found by the scans, [2] the
// smallest offending storage offset, tagged with its grid above kScanGridShift.
constexpr int kScanGridShift = 48;
// Counts non-finite entries of x[0..n) (double, or float when is_float) into block.
int launch_nonfinite_scan(const void* x, long long n, bool is_float, int grid,
                          unsigned long long* block, cudaStream_t s);

// The predictor and corrector forms fed by tensor copies (stage_mixed_tma.cu), where
// the strides and addresses allow them; launch_mixed_stage picks this path by itself.
bool mixed_stage_tma_ok(const MixedStage& st);
int launch_mixed_stage_tma(const MixedStage& st, cudaStream_t stream);
// 0 keeps launch_mixed_stage on the synchronous kernels (for comparisons), 1 the default
void set_mixed_tma(int on);
int mixed_tma_enabled();
// 1 (the default): the one-sided rows of a stage run on a second stream beside the
// stage kernel; 0: after it, on the object's stream
void set_rows_overlap(int on);
int rows_overlap_enabled();
// 1 (the default): the gradient's backward sweep recomputes the next segment beside
// the current segment's adjoint steps where two or more segments are kept; 0: after it
void set_adjoint_pipeline(int on);
int adjoint_pipeline_enabled();
int launch_df_from_f64(long long n, const double* x, float* h, float* l, cudaStream_t s);
// FP64 -> interleaved (hi, lo) FP32 pairs
int launch_df2_from_f64(long long n, const double* x, float2* hl, cudaStream_t s);
int launch_df_to_f64(long long n, const float* h, const float* l, double* x, cudaStream_t s);
int launch_to_f32(long long n, const double* x, float* y, cudaStream_t s);
int launch_weights_df(const Box& b, const double* mu, const double* la, const double* sx,
                      const double* sy, const double* sz, WeightPtrsDF w, cudaStream_t s);
int launch_force_update_df(int ib, int ie, int jb, int je, int kb, int ke, float* uph,
                           const double* rho, const SourceSet& src, double t, int tt, double coef,
                           cudaStream_t s,
                  const double* clk = nullptr);
int launch_ghost_shell_df(const Box& b, int corrector, float* out, const float* u, const float* um,
                          const float* up, cudaStream_t s);
// out = a (- bsub) in FP64 over planes k0..k1 of double-float levels of box b
int launch_df_slab(const Box& b, int k0, int k1, const float* a, const float* bsub, double* out,
                   cudaStream_t s);
int launch_uacc_slab_df(const Box& b, int k0, int k1, const float* up, const float* u,
                        const float* um, double* out, cudaStream_t s);
int launch_bcfortsg_df(int ib, int ie, int jb, int je, int kb, int ke, const int wind[36], int nx,
                       int ny, int nz, float* uh, double h, const int bccnd[6], const double sbop[5],
                       const double* mu, const double* la, const double* strx, const double* stry,
                       cudaStream_t s);
int launch_stage_rows_df(int corrector, bool top, const Box& b, int nz, const double* field_f64,
                         const float* field_df, const Box& field_box, const double* mu,
                         const double* la, double h, const double* strx, const double* stry,
                         const double* strz, const float* u, const float* um, const float* up,
                         float* out, const double* rho, const double* irho, double coef,
                         double beta, const double* const dc[3], const double* const st[3],
                         const double* const co[3], const double* zc, cudaStream_t stream,
                         const double* dd = nullptr, double* rscr = nullptr, int ctas = 0);

int launch_weights(const Box& b, const double* mu, const double* la, const double* sx,
                   const double* sy, const double* sz, double h, WeightPtrs w, cudaStream_t s);
int launch_inverse(long long n, const double* x, double* y, cudaStream_t s);
int launch_uacc_slab(const Box& b, int k0, int k1, const double* up, const double* u,
                     const double* um, double* out, cudaStream_t s);
int launch_fused_stage(const FusedStage& st, cudaStream_t stream);
int launch_stage_rows(int corrector, bool top, const Box& b, int nk, const double* field,
                      const Box& field_box, const double* mu, const double* la, double h,
                      const double* strx, const double* stry, const double* strz,
                      const double* u, const double* um, const double* up, double* out,
                      const double* rho, const double* irho, double coef, double beta,
                      const double* const dc[3], const double* const st[3],
                      const double* const co[3], const double* zc, cudaStream_t stream,
                      double* rscr = nullptr, int ctas = 0);
// rscr (optional): work array of 42 x (columns of b) doubles for the rows' per-column terms;
// ctas > 0: a persistent grid of that many CTAs strides over the rows' blocks
long long zcoef_len(const Box& b);
int launch_zcoef(const Box& b, int nk, bool top, const double* mu, const double* la, double* zc,
                 cudaStream_t s);

// Material gradient of one adjoint step (adj_grad.cu): the FP64 form in double-float
// arithmetic (pairs (hi, lo) as float2, 3 components at [c*npts + p]; adjoint levels
// scaled by 2^-sA and forward levels by 2^-sF, sA/sF = emax[0/1] - 1023 +
// marg_a/marg_f; per-point sums flushed per segment), or the FP32-mixed form in FP32
// (floats, from the double-float levels lb1 .. lun with lo halves lo further; each
// step added to gm64, gl64, gr64 with kmu).
struct GradDF {
   Box b;
   const double *b1 = nullptr, *mt = nullptr, *up = nullptr, *u = nullptr, *um = nullptr,
                *un = nullptr;
   const float *lb1 = nullptr, *lmt = nullptr, *lup = nullptr, *lu = nullptr, *lum = nullptr,
               *lun = nullptr;
   long long lo = 0;
   // the step's levels in the kernels' number type: float2 pairs or floats
   void *db1 = nullptr, *dmt = nullptr, *dw1 = nullptr, *du = nullptr, *dum = nullptr;
   const float2* st24[3] = {};  // 24 st, 1/st, co/st, beta dc per axis
   const float2* ist[3] = {};
   const float2* cist[3] = {};
   const float2* bdc[3] = {};
   void *am = nullptr, *al = nullptr, *ar = nullptr;  // per-point sums (mu, lambda, rho), pairs
   void* ed = nullptr;  // edge sums, 12 x npts
   const int* emax = nullptr;
   int marg_a = 0, marg_f = 0;
   double *gm64 = nullptr, *gl64 = nullptr, *gr64 = nullptr;  // FP32 form: the gradients
   double kmu = 0;
   // free-surface z sides: the one-sided rows' planes k <= zlo, k >= zhi, whose adjoint
   // values the z-involving terms skip (grad_rows covers them)
   int zlo = -(1 << 29), zhi = 1 << 29;
   int sg6 = 0;  // sixth-order damping: its rho term from third differences at half points
};
// The z-involving gradient terms of the six one-sided rows next to a free-surface z
// side (top: rows 1..6, bottom: nz-5..nz), FP64, added to the FP64 gradients gm, gl:
// pairs (c1 H W b1, up - 2u + um) and (c2 H W mt, u); levels FP64 or, with the lb1..lum
// pointers, double-float (hi at q, lo at q + lo).
struct GradRows {
   Box b;
   int nz = 0, top = 1;
   const double *b1 = nullptr, *mt = nullptr, *up = nullptr, *u = nullptr, *um = nullptr;
   const float *lb1 = nullptr, *lmt = nullptr, *lup = nullptr, *lu = nullptr, *lum = nullptr;
   long long lo = 0;
   const double *sx = nullptr, *sy = nullptr, *sz = nullptr, *hz = nullptr;
   double c1 = 0, c2 = 0, h = 0;
   double *gm = nullptr, *gl = nullptr;
};
int launch_grad_rows(const GradRows& g, cudaStream_t s);
struct GradDFProfiles {
   int n[3];
   const double *st[3], *co[3], *dc[3];
   double beta;
   float2 *st24[3], *ist[3], *cist[3], *bdc[3];
   const double* hz = nullptr;  // SBP norm weights of the z planes (free-surface sides)
};
int launch_grad_df_profiles(const GradDFProfiles& p, cudaStream_t s);
int launch_exp_max(const double* x, long long n, int* out, cudaStream_t s);
int launch_inj_exp(const Box& b, const double* const st[3], int nrec, const int* ijk, const double* res,
                   long long rows, int nval, const double* rho, const double* hz, int* out, cudaStream_t s);
int launch_grad_df_step(const GradDF& g, cudaStream_t s);
// The grid-point sources of nsrc sources on the Cartesian grid (srcdisc.cu): one
// device block *mem (freed and replaced) holding the grouped SourceSet.  Synchronises
// the stream (the point count sizes the forcing launches).
struct GridSpec;
struct SourceSpec;
struct CurvSourceGrid;
int launch_discretize_sources(const GridSpec& g, const int onesided[6], int nsrc, const SourceSpec* host_specs,
                              SourceSet* out, void** mem, cudaStream_t s);
// Two grids: the Cartesian and curvilinear grid-point sources (cv.jac in device memory).
int launch_discretize_sources_topo(const GridSpec& g, const int onesided[6], const CurvSourceGrid& cv,
                                   int nsrc, const SourceSpec* host_specs, SourceSet* cart, void** cart_mem,
                                   SourceSet* curv, void** curv_mem, cudaStream_t s);
int launch_grad_f1_step(const GradDF& g, cudaStream_t s);
// gm += kmu 2^(sA+sF) am, gl likewise, gr += 2^(sA+sF) ar; the sums are zeroed
int launch_grad_df_flush(const GradDF& g, double kmu, double* gm, double* gl, double* gr, cudaStream_t s);

}  // namespace sw4g
