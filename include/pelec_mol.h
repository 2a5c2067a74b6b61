/*
 * pelec_mol.h — C ABI of the GB300-native method-of-lines right-hand side.
 *
 * This library replaces the per-box body of PeleC's MOL operator,
 *   void PeleC::getMOLSrcTerm(const MultiFab& S, MultiFab& MOLSrcTerm,
 *                             Real time, Real dt, Real flux_factor)
 * (Source/PeleC.H:523-528, Source/Diffusion.cpp:4-681, regular-box branch),
 * for one AMR level without embedded boundaries.  The caller keeps its
 * MultiFabs, its MFIter loop and its ghost fill; it describes each box with a
 * pc_box_desc (an AMReX Array4 restated as plain pointers and strides) and
 * calls pc_mol_rhs_level once per level.
 *
 * Conventions
 *   - All arrays are FP64, Array4 layout: element (i,j,k,n) lives at
 *     p[(i-begin[0]) + (j-begin[1])*jstride + (k-begin[2])*kstride + n*nstride]
 *     (i fastest, component slowest), as amrex::Array4 (AMReX_Array4.H).
 *   - Conserved components follow Source/IndexDefines.H:6-13,60:
 *     URHO=0, UMX=1, UMY=2, UMZ=3, UEDEN=4, UEINT=5, UTEMP=6, UFS=7..7+nspec-1,
 *     NVAR = 7 + nspec (NUM_ADV = NUM_AUX = NUM_LIN = 0).
 *   - Device pointers are CUDA device addresses on the current device.
 *     Streams are passed as void* (a cudaStream_t; NULL = legacy default).
 *   - Every entry point returns a pc_status_code; device code never traps.
 *     Per-call diagnostic counters are read with pc_mol_last_status.
 *   - A handle may be used by one host thread at a time.  Calls are
 *     asynchronous on the given stream unless stated otherwise.
 */
#ifndef PELEC_MOL_H
#define PELEC_MOL_H

#ifdef __cplusplus
extern "C" {
#endif

#define PC_MOL_ABI_VERSION 2
#define PC_MAX_SPECIES 21

/* Return codes. */
typedef enum pc_status_code {
  PC_OK = 0,
  PC_ERR_INVALID_ARGUMENT = 1, /* bad pointer, box, stride or flag value   */
  PC_ERR_UNSUPPORTED = 2,      /* configuration with no compiled kernel     */
  PC_ERR_CUDA = 3,             /* a CUDA runtime call failed                */
  PC_ERR_OUT_OF_MEMORY = 4,    /* scratch allocation failed                 */
  PC_ERR_NO_DEVICE = 5,        /* no CUDA device visible                    */
  PC_ERR_TOO_LARGE = 6         /* request exceeds a fixed-size limit        */
} pc_status_code;

/* Equation of state (PelePhysics EosType selected at compile time in the
 * reference, Exec/Make.PeleC:74-115). */
typedef enum pc_eos_kind {
  PC_EOS_GAMMA_LAW = 0, /* calorically perfect gas, p = (gamma-1) rho e     */
  PC_EOS_IDEAL_MIX = 1  /* ideal-gas mixture with NASA-7 species thermo     */
} pc_eos_kind;

/* Transport model (PelePhysics transport(), called from
 * Source/TransCoeff.H:30-33). */
typedef enum pc_transport_kind {
  PC_TRANSPORT_CONSTANT = 0, /* mu, xi, lambda, rhoD fixed                  */
  PC_TRANSPORT_SIMPLE = 1    /* mixture-averaged, Docs Algorithms.rst:510-566 */
} pc_transport_kind;

/* Arithmetic of the right-hand side. */
typedef enum pc_precision {
  PC_PRECISION_FP64 = 0,    /* every operation in FP64, each quotient
                               correctly rounded                           */
  PC_PRECISION_MIXED = 1,   /* FP32 reconstruction, Riemann and diffusion
                               fluxes; the EOS Newton solve, the cell
                               mass fractions, the Godunov energy and the
                               flux-divergence accumulation in double-float
                               arithmetic (~48 bits on the FP32 pipe)      */
  PC_PRECISION_FP64_RCP = 2,/* every operation in FP64; a quotient by a
                               divisor shared by several numerators (Y_k =
                               rhoY_k / rho, the slopes' 1/c, the face-state
                               renormalisation, the Riemann weights, 1/V) is
                               the product with the divisor's correctly
                               rounded reciprocal, within one ulp of the
                               PC_PRECISION_FP64 quotient: about 1.1x faster,
                               and different from PC_PRECISION_FP64 by
                               rounding (as a build with multiply-add
                               contraction would be), about 1e-15 of each
                               component's flux scale |F|/V               */
  PC_PRECISION_MIXED_FP64 = 3 /* PC_PRECISION_MIXED with the EOS Newton
                                 solve, the cell mass fractions and the
                                 flux-divergence accumulation in FP64     */
} pc_precision;

/* Species data.  Thermodynamics is NASA-7 per species:
 *   cp/R = a0 + a1 T + a2 T^2 + a3 T^3 + a4 T^4
 *   h/(R T) = a0 + a1 T/2 + a2 T^2/3 + a3 T^3/4 + a4 T^4/5 + a5/T
 * with the low set for T < tmid and the high set otherwise.
 * Transport fits are ln(q) = c0 + c1 L + c2 L^2 + c3 L^3, L = ln T, for the
 * pure-species viscosity (g/cm/s), conductivity (erg/cm/s/K) and the binary
 * diffusion coefficient (cm^2/s) at pressure diff_pref (dyn/cm^2). */
typedef struct pc_mechanism {
  int nspec;
  int pad_;
  double mw[PC_MAX_SPECIES];       /* molecular weights, g/mol              */
  double gamma;                    /* GammaLaw ratio of specific heats      */
  double nasa_tmid[PC_MAX_SPECIES];
  double nasa_lo[PC_MAX_SPECIES][7];
  double nasa_hi[PC_MAX_SPECIES][7];
  double visc_fit[PC_MAX_SPECIES][4];
  double cond_fit[PC_MAX_SPECIES][4];
  double diff_fit[PC_MAX_SPECIES][PC_MAX_SPECIES][4];
  double bulk_ratio[PC_MAX_SPECIES]; /* xi = sum_k X_k bulk_ratio_k mu_k    */
  double diff_pref;
  /* Constant transport (Source/TransCoeff.H with Constant transport):     */
  double const_mu, const_xi, const_lambda, const_rhoD;
} pc_mechanism;

/* Operator configuration: the static PeleC flags that shape
 * getMOLSrcTerm (Source/Params/_cpp_parameters; defaults in
 * Source/Params/param_includes/pelec_defaults.H:32-57). */
typedef struct pc_mol_config {
  int nspec;                   /* NUM_SPECIES: 1 (GammaLaw, constant
                                  transport), 9 or 21 (ideal mixture,
                                  mixture-averaged transport)                */
  int eos;                     /* pc_eos_kind                                */
  int transport;               /* pc_transport_kind                          */
  int precision;               /* pc_precision                               */
  int do_hydro;                /* pelec.do_hydro (do_mol is implied)         */
  int diffuse_vel;             /* pelec.diffuse_vel                          */
  int diffuse_temp;            /* pelec.diffuse_temp                         */
  int diffuse_spec;            /* pelec.diffuse_spec                         */
  int diffuse_enth;            /* pelec.diffuse_enth                         */
  int plm_iorder;              /* slopes are on unless == 1: getMOLSrcTerm
                                  passes plm_iorder as mol_iorder
                                  (Diffusion.cpp:366-368, MOL.cpp:56)        */
  int use_laxf_flux;           /* pelec.use_laxf_flux                        */
  int transport_harmonic_mean; /* pelec.transport_harmonic_mean              */
  int check_output;            /* count non-finite RHS entries               */
  int newton_max_iter;         /* cap on the EOS temperature Newton (0: 50)  */
  int time_passes;             /* record CUDA events around each pass        */
  int pad_;
  double mixed_p_ref;          /* PC_PRECISION_MIXED: reference pressure the
                                  FP32 flux arithmetic is offset by, dyn/cm^2
                                  (<= 0: 1 atm); set it near the ambient p   */
  pc_mechanism mech;
} pc_mol_config;

/* An amrex::Array4<Real> restated. */
typedef struct pc_array4 {
  double* p;           /* address of element (begin, comp 0)                 */
  long long jstride;   /* elements between j and j+1                         */
  long long kstride;   /* elements between k and k+1                         */
  long long nstride;   /* elements between components                        */
  int begin[3];        /* smallEnd of the array's box                        */
  int end[3];          /* bigEnd + 1                                         */
  int ncomp;
  int pad_;
} pc_array4;

/* One box of the level: its valid region (an MFIter tilebox), the state
 * with ghost cells (at least 2 ghost layers must be filled; PeleC fills
 * numGrow()=4, Source/PeleC.H:877-900) and the output on the valid region. */
typedef struct pc_box_desc {
  int lo[3];           /* valid box smallEnd                                 */
  int hi[3];           /* valid box bigEnd                                   */
  pc_array4 state;     /* S, NVAR components, read only                      */
  pc_array4 rhs;       /* MOLSrcTerm, NVAR components, written on [lo,hi]    */
} pc_box_desc;

/* Diagnostic counters accumulated over the last pc_mol_rhs_level call. */
typedef struct pc_mol_status {
  long long cells;                 /* valid cells evaluated                  */
  long long newton_nonconverged;   /* cells whose T solve hit the cap        */
  long long nonpositive_state;     /* cells with rho, p or T <= 0 or NaN     */
  long long nonfinite_output;      /* RHS entries that are NaN or Inf        */
  int last_error;                  /* pc_status_code of the last call        */
  int pad_;
  long long exact_recomputes;      /* lanes of the FP64 passes whose quotient
                                      operands needed an IEEE division (the
                                      pass was then evaluated again with
                                      IEEE quotients): subnormal, infinite or
                                      NaN operands, or a quotient next to a
                                      power of two                           */
} pc_mol_status;

/* Physical boundary conditions of a domain face (PCPhysBCType, PeleC.H, and
 * the BCType maps of Source/Setup.cpp:34-56).  A direction is periodic when
 * both of its faces are PC_BC_INTERIOR. */
typedef enum pc_phys_bc {
  PC_BC_INTERIOR = 0,   /* periodic (int_dir)                                */
  PC_BC_OUTFLOW = 1,    /* foextrap: copy of the nearest interior cell       */
  PC_BC_SYMMETRY = 2,   /* reflect_even; normal momentum reflect_odd         */
  PC_BC_SLIPWALL = 3,   /* as symmetry                                       */
  PC_BC_NOSLIPWALL = 4  /* reflect_even; all momenta reflect_odd             */
} pc_phys_bc;

/* Index-space domain of the level (geom.Domain()) and its face BCs. */
typedef struct pc_geometry {
  int domain_lo[3];
  int domain_hi[3];
  int bc_lo[3];        /* pc_phys_bc of the low face of each direction       */
  int bc_hi[3];        /* pc_phys_bc of the high face                        */
} pc_geometry;

typedef struct pc_mol_handle pc_mol_handle;

/* ABI version of the loaded library (PC_MOL_ABI_VERSION). */
int pc_mol_abi_version(void);

/* Human-readable text for a pc_status_code. */
const char* pc_mol_error_string(int code);

/* Create an operator for one configuration.  Validates the flags, builds
 * the device-side species tables and allocates the diagnostic counters on
 * the current device.  Replaces the static setup that getMOLSrcTerm reads
 * (trans_parms, the EOS functor, PeleC static flags). */
int pc_mol_create(pc_mol_handle** out, const pc_mol_config* cfg);

/* Release the handle, its scratch and its counters. */
void pc_mol_destroy(pc_mol_handle* h);

/* MOL right-hand side of every box of one level:
 *   rhs = -(1/V) sum_d (F_d(hi face) - F_d(lo face)),
 * F = diffusion flux + hyperbolic flux, extensive (times face area).
 * Replaces the MFIter loop body of getMOLSrcTerm (Diffusion.cpp:85-679,
 * regular boxes).  dx is geom.CellSize().  The caller owns all arrays; the
 * handle owns the scratch it grows on demand.  Asynchronous on stream. */
int pc_mol_rhs_level(pc_mol_handle* h, const pc_box_desc* boxes, int nboxes,
                     const double dx[3], void* stream);

/* Same result as pc_mol_rhs_level computed with one kernel launch per box
 * and per pass (the per-box launch baseline). */
int pc_mol_rhs_level_per_box(pc_mol_handle* h, const pc_box_desc* boxes,
                             int nboxes, const double dx[3], void* stream);

/* pc_mol_rhs_level that also writes the face fluxes — the hyperbolic plus
 * diffusion flux times the face area, all NVAR components — that
 * getMOLSrcTerm hands to the flux registers for refluxing on multi-level
 * runs (Diffusion.cpp:652-670).  fluxes[3*b + d] covers
 * surroundingNodes(valid_b, d); the RHS is the same as without the export.
 * Every precision; with the mixed forms the fluxes are their FP32 face
 * fluxes (the energy fluxes double-float; the normal-momentum flux with the
 * reference pressure mixed_p_ref added back) times the area, in FP64, so that
 * -sum_d (F(hi) - F(lo)) / V reproduces their RHS.  Asynchronous on stream. */
int pc_mol_rhs_level_fluxes(pc_mol_handle* h, const pc_box_desc* boxes, int nboxes, const double dx[3],
                            const pc_array4* fluxes, void* stream);

/* Synchronize the handle's last stream and copy the diagnostic counters of
 * the last rhs call into *st. */
int pc_mol_last_status(pc_mol_handle* h, pc_mol_status* st);

/* With cfg.time_passes set: synchronize and return the device time in
 * milliseconds of each pass of the last pc_mol_rhs_level call, measured with
 * CUDA events on the call's stream: ms[0] = cell pass (primitives, EOS,
 * transport), ms[1] = flux pass (faces and divergence).  n >= 2. */
int pc_mol_pass_times(pc_mol_handle* h, double* ms, int n);

/* Launch configurations of the flux pass: a tile shape (one thread per cell
 * of a tile; every shape gives bit-identical FP64 results), launched with one
 * CTA per tile, or the same shape + PC_LAUNCH_PERSISTENT, launched with as many
 * CTAs as are resident on the GPU at once, each striding over the tile list
 * (same results again).  The reference's counterpart is the MFIter tile size
 * and the launch shape of its GPU loops (hydro_tile_size,
 * Diffusion.cpp:81-86; amrex::ParallelFor block size), which are fixed. */
#define PC_NUM_TILES 4
#define PC_LAUNCH_PERSISTENT PC_NUM_TILES
#define PC_NUM_LAUNCH_CONFIGS (2 * PC_NUM_TILES)
enum {
  PC_TILE_8x8x4 = 0,   /* 256 threads, 2 CTAs/SM (default)                   */
  PC_TILE_8x8x8 = 1,   /* 512 threads, 1 CTA/SM                               */
  PC_TILE_16x8x4 = 2,  /* 512 threads, 1 CTA/SM                               */
  PC_TILE_8x4x4 = 3    /* 128 threads, 4 CTAs/SM                              */
};

/* shape[0..3] = tile extents x, y, z and threads per CTA of launch
 * configuration t (0 <= t < PC_NUM_LAUNCH_CONFIGS). */
int pc_mol_tile_shape(int t, int shape[4]);

/* Force launch configuration t for the following calls, or t = -1 to return
 * to the automatic choice (the autotune cache entry of the BoxArray's
 * box-size histogram, else PC_TILE_8x8x4).  PC_ERR_UNSUPPORTED when the flux
 * pass of configuration t needs more shared memory per CTA than the device
 * allows at the handle's species count and precision (FP64 with 21 species:
 * the 8x8x8 and 16x8x4 tiles). */
int pc_mol_set_tile(pc_mol_handle* h, int t);

/* The launch configuration that the last rhs call used. */
int pc_mol_current_tile(pc_mol_handle* h, int* t);

/* Autotuner: time pc_mol_rhs_level on this BoxArray at every launch
 * configuration (one warm-up, then reps timed calls each, CUDA events on
 * stream), keep the fastest in the handle's cache under the BoxArray's
 * box-size histogram (the species count and precision are the handle's) and
 * return it in *best.  ms[t] receives the mean time per call of
 * configuration t when ms is not NULL and n_ms >= PC_NUM_LAUNCH_CONFIGS, or
 * -1 for a configuration that does not fit the device (pc_mol_set_tile) and
 * is not timed.
 * Writes the RHS into the boxes' rhs arrays (every configuration gives the
 * same values).  Synchronous; not to be called during a stream capture. */
int pc_mol_autotune(pc_mol_handle* h, const pc_box_desc* boxes, int nboxes, const double dx[3], int reps,
                    int* best, double* ms, int n_ms, void* stream);

/* Fill ngrow ghost layers of every box's state array on one level that
 * covers its domain: each ghost cell takes the value of the valid cell it
 * maps to — periodic images wrap, PC_BC_OUTFLOW clamps to the nearest
 * interior cell, reflecting faces mirror (momentum components negated as
 * the face type says).  Replaces FillPatcherFill / FillBoundary with the
 * physical BC fill at a single level (Source/Advance.cpp:98,132;
 * Source/BCfill.cpp; Source/Setup.cpp:34-56).  The boxes' states must cover
 * grow(valid, ngrow) and the valid boxes must tile the domain. */
int pc_mol_fill_ghosts(pc_mol_handle* h, const pc_box_desc* boxes, int nboxes, const pc_geometry* geom, int ngrow,
                       void* stream);

/* dst = a*x + b*y on the valid cells of each box, all NVAR components
 * (MultiFab::LinComb / Saxpy of the MOL advance, Advance.cpp:117,148-151).
 * lohi holds 6 ints per box (valid lo, hi); dst may alias x or y. */
int pc_mol_lincomb(pc_mol_handle* h, int nboxes, const int* lohi, const pc_array4* dst, double a,
                   const pc_array4* x, double b, const pc_array4* y, void* stream);

/* PeleC::computeTemp on the valid cells (PeleC.cpp:2254-2271): with the
 * default allow_small_energy = allow_negative_energy = true,
 * reset_internal_energy sets rho e = rho E - rho |u|^2/2 (Utilities.H:219-236)
 * and pc_cmpTemp solves the EOS for T from U(UTEMP) (Utilities.H:67-84). */
int pc_mol_compute_temp(pc_mol_handle* h, int nboxes, const int* lohi, const pc_array4* state, void* stream);

/* Transposes of the two level operations above, for the adjoint of a
 * trajectory (no counterpart in the reference).
 * pc_mol_fill_ghosts_adjoint: boxes[b].state holds cotangents; the cotangent
 * of every ghost cell of grow(valid, ngrow) is added (with the fill's sign
 * flips) to the valid cell the fill copies it from, and the ghost is set to
 * 0.  FP64 atomics: the sum order, and so the last bit, may vary between
 * runs.
 * pc_mol_compute_temp_adjoint: state[b] is the state after computeTemp,
 * state_bar[b] its cotangent (valid cells), overwritten with the cotangent
 * of the state before computeTemp (UEINT and UTEMP entries become 0). */
int pc_mol_fill_ghosts_adjoint(pc_mol_handle* h, const pc_box_desc* boxes, int nboxes, const pc_geometry* geom,
                               int ngrow, void* stream);
int pc_mol_compute_temp_adjoint(pc_mol_handle* h, int nboxes, const int* lohi, const pc_array4* state,
                                pc_array4* state_bar, void* stream);

/* A CUDA graph of one level's RHS, optionally preceded by its ghost fill
 * (FillPatcherFill + getMOLSrcTerm of Advance.cpp:98-100), captured once and
 * replayed with one launch.  The layout (boxes, array pointers, dx, fill
 * geometry when not NULL, tile shape) is fixed at creation; each replay
 * reads the arrays' current contents.  The graph owns a private copy of h
 * (configuration, tile choice and autotune cache as they are at creation)
 * with its own scratch and counters, so later calls through h do not
 * disturb it; pc_mol_graph_status reads the counters of the last replay.
 * Creation runs the sequence once uncaptured on an internal stream (uploads,
 * scratch) and synchronizes. */
typedef struct pc_mol_graph pc_mol_graph;
int pc_mol_graph_create(pc_mol_handle* h, const pc_box_desc* boxes, int nboxes, const double dx[3],
                        const pc_geometry* fill_geom, int ngrow, pc_mol_graph** out);
int pc_mol_graph_launch(pc_mol_graph* g, void* stream);
int pc_mol_graph_status(pc_mol_graph* g, pc_mol_status* st);
void pc_mol_graph_destroy(pc_mol_graph* g);

/* One SSP-RK2 step of a level per CUDA-graph replay: PeleC's do_mol_advance
 * without sources (Source/Advance.cpp:98-168), i.e. the ghost fill
 * (FillPatcherFill, :98, :132), getMOLSrcTerm (:100, :134), MultiFab::LinComb
 * (:117), computeTemp (:125), LinComb and Saxpy (:148-151), computeTemp (:168):
 *   fill(S_old); R = RHS(S_old); S_new = S_old + dt R; computeTemp(S_new);
 *   fill(S_new); R = RHS(S_new); S_new = 0.5 S_new + 0.5 S_old;
 *   S_new += 0.5 dt R; computeTemp(S_new)
 * with each operation's arithmetic that of the separate entry points (the
 * replayed step equals the sequence of calls bit for bit).  a[b] gives box
 * b's valid region, its state S_a (ngrow >= 2 filled-ghost layers, the
 * layers the fill writes) and the RHS array R; state_b[b] is the second
 * state S_b, with the same array geometry.  Creation captures both
 * directions, S_a -> S_b and S_b -> S_a, so a trajectory alternates them
 * without copies; like pc_mol_graph it owns a private copy of h with its own
 * scratch and counters, and runs the RHS of both states once, uncaptured,
 * writing R, then synchronizes.  geom: the level's domain and face BCs, as
 * for pc_mol_fill_ghosts.  Launch: dt is written to a device scalar ahead of
 * the replay (reverse = 0: S_a -> S_b, 1: S_b -> S_a); asynchronous on
 * stream.  No counterpart in the reference, which issues these as separate
 * launches from the host. */
typedef struct pc_mol_step_graph pc_mol_step_graph;
int pc_mol_step_graph_create(pc_mol_handle* h, const pc_box_desc* a, const pc_array4* state_b, int nboxes,
                             const double dx[3], const pc_geometry* geom, int ngrow, pc_mol_step_graph** out);
int pc_mol_step_graph_launch(pc_mol_step_graph* g, double dt, int reverse, void* stream);
int pc_mol_step_graph_status(pc_mol_step_graph* g, pc_mol_status* st);
void pc_mol_step_graph_destroy(pc_mol_step_graph* g);

/* Vector-Jacobian product of the RHS (reverse mode, hand-written):
 *   state_bar = (d rhs / d state)^T rhs_bar
 * for PC_PRECISION_FP64 with the Riemann solver of riemann() (use_laxf_flux
 * = 0).  boxes as for pc_mol_rhs_level (their rhs arrays are not touched);
 * rhs_bar[b] covers the valid box, state_bar[b] covers grow(valid, 2) and
 * receives the cotangent of every state entry the RHS reads there (the
 * ghost entries included; UEINT and UTEMP get 0: the RHS does not read
 * UEINT, and UTEMP only as the Newton guess).  The EOS temperature solve is
 * differentiated by the implicit-function theorem; at the kinks of the
 * limiters and Riemann switches the derivative of the branch the forward
 * pass took is used.  The reference has no adjoint; this is the entry point
 * a differentiable getMOLSrcTerm would bind.  Asynchronous on stream. */
int pc_mol_rhs_vjp(pc_mol_handle* h, const pc_box_desc* boxes, int nboxes, const double dx[3],
                   const pc_array4* rhs_bar, pc_array4* state_bar, void* stream);

/* Jacobian-vector product of the RHS (forward mode, dual numbers):
 *   rhs_dot = (d rhs / d state) state_dot,
 * and the RHS itself into boxes[b].rhs (bit for bit the pc_mol_rhs_level
 * result).  PC_PRECISION_FP64 only.  state_dot[b] covers grow(valid, 2)
 * (UEINT and UTEMP entries are ignored), rhs_dot[b] the valid box.  Uses
 * the derivative of the branch the forward takes and the implicit-function
 * theorem for the EOS temperature solve, like pc_mol_rhs_vjp, so
 * <rhs_bar, JVP(v)> = <VJP(rhs_bar), v> to round-off.  No counterpart in the
 * reference.  Asynchronous on stream. */
int pc_mol_rhs_jvp(pc_mol_handle* h, const pc_box_desc* boxes, int nboxes, const double dx[3],
                   const pc_array4* state_dot, pc_array4* rhs_dot, void* stream);

/* PeleC::estTimeStep (PeleC.cpp:839-972, Timestep.H): min over valid cells
 * of dx/(c+|u|) (do_hydro) and the viscous, thermal and enthalpy diffusion
 * limits (diffuse_vel/temp/enth), times cfl, capped by max_dt.  Synchronous:
 * returns the time step in *dt. */
int pc_mol_est_dt(pc_mol_handle* h, const pc_box_desc* boxes, int nboxes, const double dx[3], double cfl,
                  double max_dt, double* dt, void* stream);

/* Diagnostic: q[i] = a[i] / b[i] (device arrays of n doubles) through the
 * exact shared-divisor quotient of the FP64 kernels (the product with the
 * IEEE reciprocal of b, corrected to the correctly rounded quotient in
 * integer arithmetic).  No counterpart in the reference; it lets a test
 * compare that routine with IEEE division on arbitrary operands.
 * Asynchronous on stream. */
int pc_mol_check_quotients(const double* a, const double* b, double* q, long long n, void* stream);

/* Right-hand side of ONE box without allocating any device memory.  This
 * entry point has no counterpart in the reference: it exists for callers
 * that cannot call cudaMalloc while they run (code running under an external
 * memory pool that forbids other allocations, applications that reserve all
 * device memory at start-up).
 * There is no handle: cfg is read on every call.  The caller passes the box
 * (state with at least 2 ghost layers, output on the valid region) as for
 * pc_mol_rhs_level and gets the same result.  The per-cell scratch, launch
 * lists and counters live in one fixed 48 MiB device array that each GPU
 * reserves when the library is loaded and keeps until the process exits; a
 * box that does not fit (larger than about 46^3 valid cells with 9 species,
 * 67^3 with one, 36^3 with 21) returns PC_ERR_TOO_LARGE before anything is
 * launched.  The first call
 * on each device, and per precision, does the one-time set-up — it looks up
 * that array's device address and raises the flux kernels' shared-memory
 * limit — so make that first call before any stream capture.  Every call
 * reuses the same array: calls whose work overlaps on the GPU (other
 * streams, other host threads) race and must be serialised by the caller.
 * PC_PRECISION_FP64, PC_PRECISION_MIXED and PC_PRECISION_MIXED_FP64 (the
 * mixed records fit the same array); PC_PRECISION_FP64_RCP returns
 * PC_ERR_UNSUPPORTED.  Asynchronous on stream; no diagnostic counters are
 * returned. */
int pc_mol_rhs_box_static(const pc_mol_config* cfg, const pc_box_desc* box, const double dx[3], void* stream);

#ifdef __cplusplus
}
#endif

#endif /* PELEC_MOL_H */
