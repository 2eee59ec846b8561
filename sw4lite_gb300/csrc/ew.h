// Host-side driver of the elastic time step for one Cartesian grid on one GPU:
// the GB300 counterpart of the reference's EW time loop (src/EW.C:2339-2930)
// for the Forcing, Scheme, BC-phys and Supergrid phases.
//
// Ownership: the EW object owns its device arrays (material, 1-D profiles,
// precomputed weights, four rotating time levels and source lists).  Stepping
// enqueues kernels on the stream given at creation and never synchronises the
// host; no allocation happens after set-up, so a step sequence can be captured
// into a CUDA graph.
#pragma once

#include <cuda_runtime.h>

#include <functional>
#include <memory>
#include <vector>

#include "kernels.h"
#include "setup.h"

namespace sw4g {

// Topography over this Cartesian grid: a Gaussian hill
// z_s = -amp exp(-((x-xc)/lx)^2 - ((y-yc)/ly)^2), mapped onto a curvilinear grid
// from z_s down to the Cartesian grid's zmin as the reference's grid_mapping does
// (src/EW.C:5694, zeta_break and order are its m_zetaBreak and
// m_grid_interpolation_order, defaults src/EW.C:180-181).
struct TopoSpec {
   double amp = 0, xc = 0, yc = 0, lx = 1, ly = 1;
   double zeta_break = 0.95;
   int order = 4;
};

// The curvilinear grid on top of the Cartesian grid (ew_topo.cu).
struct CurvGrid {
   TopoSpec topo;
   int nz = 0;
   Bounds b{};
   long long npts = 0;
   int bc[6] = {}, wind[36] = {}, bcpts[6] = {};
   double *z = nullptr, *met = nullptr, *jac = nullptr;
   double *rho = nullptr, *mu = nullptr, *la = nullptr;
   double* lev[4] = {};
   double *lu = nullptr, *uacc = nullptr, *fzero = nullptr;
   double* coef = nullptr;  // fused-stage coefficients (curv_stage.cu)
   CurvCoef cc{};
   float* coefdf = nullptr;  // the mixed form's (hi, lo) coefficients (curv_mixed.cu)
   double* topscr = nullptr;  // work array of the SBP top rows, 36 doubles per column
   std::vector<double> hjac;  // host copy of the Jacobian (source discretisation)
   CurvCoefDF cd{};
   float* rhoj32 = nullptr;  // rho J in FP32: the mixed form's 6th-order damping
   bool rhoj32_ok = false;
   bool material = false;
   ~CurvGrid();
};

enum StepMode : int {
   kModePhases = 0,  // reference phase order with dense Lu / F / Uacc arrays
   kModeFused = 1,   // fused predictor and corrector stage kernels
};

class EW {
 public:
   // topo != nullptr: a curvilinear grid over that topography on top of this grid,
   // whose top side must then be the interface (bc[4] == kInterface).
   EW(const GridSpec& g, cudaStream_t stream, const TopoSpec* topo = nullptr);
   ~EW();
   EW(const EW&) = delete;
   EW& operator=(const EW&) = delete;

   // Makes this object the subdomain of `global` whose interior points are the global
   // points i = ioff + 1 .. ioff + nx, j = joff + 1 .. joff + ny of this object's grid
   // (sides shared with a neighbour are kProcessor).  Call before init().
   int set_subdomain(const GridSpec& global, int ioff, int joff);
   int init();  // allocates device memory; returns a Status
   const GridSpec& grid() const { return g_; }
   const Bounds& bounds() const { return b_; }
   long long npts() const { return npts_; }
   cudaStream_t stream() const { return stream_; }

   // Material (rho, mu, lambda) over the full array (ghosts included), host or device.
   int set_material(const double* rho, const double* mu, const double* la, bool on_device);
   // Sources: discretised on the host, uploaded before the next step.
   int add_source(const SourceSpec& s);
   int add_grid_point_sources(int n, const int* ijk, const double* amp, const double* freq,
                              const double* t0, const int* kind);
   int clear_sources();
   // Where add_source's grid-point sources are computed: on the host (the default)
   // or on the device, the whole batch at the next step (srcdisc.cu; the same bits).
   // The device path takes the Cartesian grid alone and no raw grid-point sources.
   int set_source_discretization(bool on_device);
   int num_grid_point_sources() const;
   // the discretised grid-point sources of grid 0 (Cartesian) or 1 (curvilinear)
   int grid_point_sources(int grid, std::vector<GridPointSource>* out) const;
   // Time step: explicit dt, or computed from the CFL number and an end time.
   int set_time_step(double dt, double t0);
   int compute_time_step(double cfl, double tmax, double* dt, int* nsteps);
   double time() const { return t_; }
   double dt() const { return dt_; }

   // Solution levels U (current) and Um (previous), 3*npts doubles each.
   int set_fields(const double* u, const double* um, bool on_device);
   int get_fields(double* u, double* um, bool on_device) const;
   double* field_u() const { return lev_[iu_]; }
   double* field_um() const { return lev_[ium_]; }

   int step(int nsteps, int mode);
   // A subdomain's fused step in three parts, with a halo exchange of the level the
   // part leaves after parts 0 and 1 (the reference's exchange points after the
   // predictor and after the corrector, src/EW.C:2596-2616, 2728-2744): part 0 the
   // predictor stage, its one-sided rows and forcing; part 1 the predictor's boundary
   // closures, the corrector stage, rows, damping and forcing; part 2 the corrector's
   // boundary closures, receivers, level rotation and time.  Parts run in order.
   int step_part(int part);
   bool is_subdomain() const { return sub_; }
   int device() const { return dev_; }
   // bytes of one side's halo along axis (0 x, 1 y) in the level's storage format
   long long halo_bytes(int axis) const;
   // pack the two interior planes next to side (0 low, 1 high) of the level to
   // exchange into buf, or unpack buf into that side's two ghost planes (halo.cu)
   int halo_pack(int axis, int side, void* buf) { return halo_copy(axis, side, true, buf); }
   int halo_unpack(int axis, int side, const void* buf)
   {
      return halo_copy(axis, side, false, const_cast<void*>(buf));
   }
   // the object's own exchange buffers (device memory of its GPU), halo_bytes each
   void* send_buffer(int axis, int side) const { return xbuf_[2 * axis + side]; }
   void* recv_buffer(int axis, int side) const { return xbuf_[4 + 2 * axis + side]; }
   // Non-finite check of the time loop (the reference's checkfornan, src/EW.C:1333,
   // 2544-2759): every `every` steps (and after the last step of a step() call) the
   // new level of every grid is scanned; step() then synchronises and returns
   // kNanDetected after the first checked step that holds a NaN or an infinity, with
   // the object at that step.  0 turns the check off (the default).
   int set_nan_check(int every);
   struct NanReport {
      int grid = -1, c = 0, i = 0, j = 0, k = 0;
      long long count = 0;
      double t = 0;
   };
   const NanReport& nan_report() const { return nan_; }
   // Synchronises the object's stream and returns kTimeout if a kernel's bounded wait
   // gave up since the last call (clearing the flag), else kOk.
   int status();
   // CUDA graphs for the fused time loop: when on, step() replays captured chunks of
   // kGraphSteps steps (a multiple of the level rotation's period 3) and gradient()
   // replays its forward chunks, recompute segments and adjoint segments; the forcing
   // time and the record row then live in a device clock.  Results are bit-identical
   // to direct launches.
   int set_graphs(bool on);
   static constexpr int kGraphSteps = 30;

   // Misfit J = 1/2 sum_{n=0..nsteps} |rec^n - obs^n|^2 of the receivers (all in
   // displacement mode) over nsteps fused steps from the current levels, and its
   // gradient with respect to rho, mu, lambda at every array point, by the
   // discrete adjoint (adjoint.cu) with checkpoints every ckpt steps.  FP64,
   // Dirichlet / supergrid sides only.  The object ends after the forward run.
   int gradient(int nsteps, int ckpt, const double* obs, bool obs_on_device, double* misfit,
                double* g_rho, double* g_mu, double* g_la, bool grad_on_device);
   // Restart files in the reference's checkpoint format (checkpoint.cu); read sets
   // both levels, their ghost points and the time.
   int write_checkpoint(const char* path, int cycle);
   int read_checkpoint(const char* path, int* cycle);
   // Device memory gradient() may add for segments kept from its forward run (whose
   // recompute the backward sweep then skips): < 0 all free memory but a reserve
   // (the default), 0 none beyond the last segment, else at most this many bytes.
   // gradient() keeps its device buffers for the next call of the same shape; this
   // call releases them.
   int set_gradient_memory(long long bytes)
   {
      drop_grad_cache();
      grad_store_bytes_ = bytes;
      return kOk;
   }

   // Grids: 0 the Cartesian grid, 1 the curvilinear grid (with topography).
   int num_grids() const { return cv_ ? 2 : 1; }
   int grid_dims(int grid, int* nx, int* ny, int* nz, long long* npts) const;
   int set_material_grid(int grid, const double* rho, const double* mu, const double* la,
                         bool on_device);
   int set_fields_grid(int grid, const double* u, const double* um, bool on_device);
   int get_fields_grid(int grid, double* u, double* um, bool on_device) const;
   // z, metric (4 x npts, SoA) and Jacobian of the curvilinear grid; any may be null
   int curvilinear_arrays(double* z, double* met, double* jac, bool on_device) const;

   // Receivers at grid points (i,j,k) with record modes (kernels.h RecMode).  Each
   // step appends one row of values (all receivers, in order) to a device record
   // array of `capacity` rows; the first row holds the initial data and is written
   // by the first step after this call.  A step that would overflow the array is
   // refused before it starts.  grid[n] (may be null: all on grid 0) puts a receiver
   // on the Cartesian grid (0) or the curvilinear grid (1, with topography).
   int set_receivers(int n, const int* ijk, const int* mode, int capacity, const int* grid = nullptr);
   // The grid point and grid of a receiver at (x, y, z) (EW::computeNearestGridPoint,
   // src/EW.C:5149-5213, with TimeSeries' placement on the curvilinear grid,
   // src/TimeSeries.C:139-168 and :307-329): nearest (i, j); below the interface the
   // Cartesian k, at or above it k = round(s) of the inverted grid mapping, limited
   // to 1..nz (the surface if the mapping cannot be inverted).  kBadArgument for a
   // point above the topography or outside the grids.
   int nearest_grid_point(double x, double y, double z, int ijk[3], int* grid) const;
   // z of the topography surface at (x, y) (EW::find_topo_zcoord_owner,
   // src/EW.C:6311, with the analytic Gaussian hill); 0 without topography
   double topography_z(double x, double y) const;
   int record_shape(int* rows, int* nvals) const;
   int get_records(double* out, bool on_device) const;
   // Boundary conditions on an arbitrary 3-component device array of this grid.
   int enforce_bc(double* u);

   // Device pointers of set-up arrays (tests / bench)
   const double* profile(int which, int axis) const;  // which: 0 dc, 1 str, 2 co
   const double* weights(int slot) const { return w_.p[slot]; }
   int launches_per_step(int mode) const;
   // Average device time (ms, CUDA events on the EW stream) of each piece of a
   // fused step, each launched nrep times on the current levels without advancing
   // time: [0] predictor stage kernel, [1] corrector stage kernel, [2] one-sided
   // rows of both stages, [3] boundary conditions + forcing of both stages.
   int profile_kernels(int nrep, double ms[4]);

 private:
   int upload_sources();
   int halo_copy(int axis, int side, bool pack, void* buf);
   // discretise one source into hsrc_ (on the global grid for a subdomain, keeping
   // the entries on this subdomain's interior points)
   void discretize_into(const SourceSpec& s, std::vector<GridPointSource>& out) const;
   int scan_levels();                 // non-finite scans of the current levels, then the outcome
   int read_status(unsigned long long out[4]);
   int record(int iup, int ium, int initial);  // levels by index (both grids)
   int step_phases();
   int step_fused();
   int fused_piece(int piece, int ip, int iq);
   int mixed_piece(int piece, int ip, int iq);
   int piece(int which, int ip, int iq) { return mixed_ ? mixed_piece(which, ip, iq) : fused_piece(which, ip, iq); }
   // pieces 2 and 5 split at a subdomain's exchange points: forcing, then closures
   static constexpr int kForcePred = 6, kBcPred = 7, kForceCorr = 8, kBcCorr = 9;
   int ensure_staging();
   int init_topo();
   int curv_pred(int ip);
   int curv_corr(int ip, int iq);
   int curv_bc(double* ucart, double* ucurv);
   int curv_time_step(double cfl, double* dt);
   int curv_launches(int mode) const;
   int curv_force(double* lev, int tt, double coef);
   CurvSourceGrid curv_source_grid(bool device) const;
   int ensure_phase_arrays();
   // graphs
   int sync_clock(double res_row = 0);
   int run_graphed(int nsteps);
   void drop_graphs();
   // records what body() enqueues on the stream as a graph and instantiates it (the
   // host-side effects of body happen once, at capture)
   int capture(const std::function<int()>& body, cudaGraphExec_t* exec);

   GridSpec g_;
   Bounds b_{};
   cudaStream_t stream_ = nullptr;
   long long npts_ = 0;
   bool ready_ = false, material_ = false;
   int wind_[36] = {}, bcpts_[6] = {}, onesided_[6] = {};
   double sbop_[5] = {};
   SupergridProfiles prof_;

   bool mixed_ = false;
   float* rho32_ = nullptr;  // mixed form: FP32 rho and profiles, (hi, lo) pairs of
   float* mu32_ = nullptr;   // mu, lambda, 1/rho (2*npts floats each) and of the
   float* la32_ = nullptr;   // second-difference weights
   float* irho32_ = nullptr;
   float* wdf_ = nullptr;
   WeightPtrsDF wd_{};
   float* prof32_[9] = {};
   double* staging_ = nullptr;  // FP64 buffer for converting the mixed form's levels
   double* rho_ = nullptr;
   double* mu_ = nullptr;
   double* la_ = nullptr;
   double* irho_ = nullptr;
   double* dprof_[9] = {};  // dc x,y,z ; str x,y,z ; co x,y,z
   WeightPtrs w_{};
   double* wstore_ = nullptr;
   double* lev_[4] = {};
   int iu_ = 0, ium_ = 1;
   double* lu_ = nullptr;   // phase mode work arrays
   double* f_ = nullptr;
   double* uacc_ = nullptr;
   double* zc_[2] = {nullptr, nullptr};  // SBP z coefficients of the top / bottom rows
   double* slab_ = nullptr; // corrector stage field on the one-sided rows
   double* rscr_ = nullptr; // per-column terms of the one-sided rows (42 x columns)
   long long slab_len_ = 0;

   std::vector<GridPointSource> hsrc_;
   std::vector<SourceSpec> specs_;  // the sources added, in order
   int raw_src_ = 0;                // grid-point sources added directly
   bool dev_src_ = false;           // discretise on the device
   std::vector<GridPointSource> hsrc_curv_;  // sources of the curvilinear grid
   SourceSet dsrc_curv_{};
   void* dsrc_curv_mem_ = nullptr;
   bool src_dirty_ = true;
   SourceSet dsrc_{};
   void* dsrc_mem_ = nullptr;

   ReceiverSet drec_{};
   void* drec_mem_ = nullptr;
   double* records_ = nullptr;
   int rec_cap_ = 0, rec_rows_ = 0, rec_nvals_ = 0;
   bool rec_initial_ = false;  // the initial-data row is still to be written
   bool rec_curv_ = false;     // a receiver lies on the curvilinear grid

   std::unique_ptr<CurvGrid> cv_;
   long long grad_store_bytes_ = -1;  // gradient(): budget for kept segments
   // gradient()'s device buffers, kept for the next call of the same shape (freeing
   // ~100 GB takes tens of milliseconds; a multi-shot inversion calls it once per shot)
   struct GradCache {
      long long npts = 0, budget = 0;
      int nsteps = 0, ckpt = 0, nval = 0, mixed = -1, host_grad = -1;
      std::vector<void*> mem;  // every allocation
      double *ck = nullptr, *seg = nullptr, *pred = nullptr, *work = nullptr, *resd = nullptr,
             *dfw = nullptr, *dfp = nullptr, *dfe = nullptr, *gtmp = nullptr, *hz = nullptr,
             *rgrp = nullptr;  // rgrp: receivers grouped by grid point (ints)
      std::vector<double*> xbuf;  // segments kept from the forward run
   } gcache_;
   void drop_grad_cache();
   int* stage_emax_ = nullptr;        // gradient(): exponent maximum of the corrector's levels

   double t_ = 0, dt_ = 0;
   // subdomain of a decomposed grid
   bool sub_ = false;
   GridSpec global_{};
   int ioff_ = 0, joff_ = 0, dev_ = 0;
   int part_ = 0, split_ip_ = 0, split_iq_ = 0;  // step_part state
   void* xbuf_[8] = {};                           // send (4) and receive (4) halo buffers
   unsigned long long* dstat_ = nullptr;  // status block (kernels.h): flags, count, first offset
   int nan_every_ = 0;
   NanReport nan_{};

   bool graphs_ = false, clocked_ = false, warm_ = false;
   // the one-sided rows beside the stage kernels: a second stream forked from and
   // joined to stream_ by events (made on first use)
   cudaStream_t side_ = nullptr;
   cudaEvent_t ev_fork_ = nullptr, ev_join_ = nullptr;
   int sms_ = 0;        // the device's SM count
   int rows_ctas_ = 0;  // > 0 while the rows run beside a stage: a persistent grid
   int side_stream();
   int curv_pred_part(int ip, int part, cudaStream_t s, int ctas);
   int curv_corr_part(int ip, int iq, int part, cudaStream_t s, int ctas);
   double* dclock_ = nullptr;  // [0] forcing time, [1] record row, [2] adjoint residual row
   struct GraphKey {
      int iu, ium, rec;
      cudaGraphExec_t exec;
   };
   std::vector<GraphKey> graph_cache_;
};

// Steps subdomain objects in lockstep with halo exchanges between them (halo.cu);
// nb[4 s + q] is the neighbour of subdomain s across side q (x-low, x-high, y-low,
// y-high) or -1.
int step_group(EW* const* subs, int n, const int* nb, int nsteps);

}  // namespace sw4g
