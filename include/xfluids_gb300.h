/*
 * xfluids_gb300.h - C ABI of the GB300-native convective right-hand side of XFluids.
 *
 * The reference host code (class XFLUIDS, src/XFLUIDS.cpp) drives one fluid through the methods of
 * class Fluid (src/global_class.h:14-55, implemented in src/Fluids.cpp). Every entry point below
 * replaces one of those methods, or the block function underneath it, for the path
 *
 *     BoundaryCondition -> UpdateFluidStates -> ComputeFluidLU -> UpdateFluidURK3   (per RK stage)
 *     GetFluidDt                                                                    (per step)
 *
 * The signatures use plain C types only: parameter blocks mirror the reference's POD structs
 * (Block/MeshSize/Thermal, src/include/global_setup.h:162-208) and the compile-time macros that
 * select the scheme (SCHEME_ORDER, Artificial_type, COP, NUM_SPECIES, GhostSpecies, Thermo,
 * NCOP_Gamma) become run-time fields of xfg_scheme.
 *
 * Conventions
 *  - Cell index id = Xmax*Ymax*k + Xmax*j + i (x fastest), as in the reference.
 *  - Arrays crossing the ABI use the reference's layouts: conserved state AoS U[Emax*id + n],
 *    primitives SoA of length Xmax*Ymax*Zmax, mass fractions AoS y[NUM_SPECIES*id + s].
 *    Pointers may be host or device memory (the copies use unified addressing).
 *  - Inside the handle the state is stored SoA (U[n*pitch + id]) in device memory.
 *  - Every function returns an int status: 0 ok, >0 a numerical error code in the reference's
 *    encoding (10000 negative density, 1100/1200 NaN/Inf state, 21/22 NaN/Inf right-hand side,
 *    src/Fluids.cpp:1024-1029), <0 a CUDA or argument error (message in xfg_last_error()).
 *    No function calls exit().
 */
#ifndef XFLUIDS_GB300_H
#define XFLUIDS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define XFG_MAX_SPECIES 9   /* largest NUM_SPECIES built into the kernels */
#define XFG_MAX_EQ (XFG_MAX_SPECIES + 4)

/* Boundary condition ids, src/include/global_setup.h:96-105 (enum BConditions). */
enum xfg_bc { XFG_INFLOW = 0, XFG_OUTFLOW = 1, XFG_SYMMETRY = 2, XFG_PERIODIC = 3,
              XFG_NSLIPWALL = 4, XFG_VISCWALL = 5, XFG_SLIPWALL = 6, XFG_INNERBLOCK = 7 };

/* Mesh block, the fields of Block/MeshSize the path reads (global_setup.h:162-200, filled by
 * Setup::init, src/read_ini/src/iniset.cpp:290-369). Absent dimensions have inner=1, Bwidth=0. */
typedef struct xfg_block {
    int Xmax, Ymax, Zmax;
    int X_inner, Y_inner, Z_inner;
    int Bwidth_X, Bwidth_Y, Bwidth_Z;
    int DimX, DimY, DimZ;
    double dx, dy, dz;
    double _dx, _dy, _dz;
    double CFLnumber;
    int Boundarys[6];          /* XMIN, XMAX, YMIN, YMAX, ZMIN, ZMAX (Setup::Boundarys) */
} xfg_block;

/* Thermo tables as Setup::ReadThermal leaves them (src/read_ini/src/thermal.cpp:36-178):
 * Hia[n*21 + coeff*3 + range], Hib[n*6 + k*3 + range], Wi in kg/mol, Ri = Ru/Wi, _Wi = 1/Wi. */
typedef struct xfg_thermal {
    int num_species;
    double Wi[XFG_MAX_SPECIES];
    double _Wi[XFG_MAX_SPECIES];
    double Ri[XFG_MAX_SPECIES];
    double Hia[XFG_MAX_SPECIES * 21];
    double Hib[XFG_MAX_SPECIES * 6];
} xfg_thermal;

/* Scheme selection: the reference's compile-time switches (cmake/init_options.cmake:23-90,
 * cmake/init_sample.cmake:216-282) as run-time values. */
enum xfg_artificial { XFG_ROE = 1, XFG_LLF = 2, XFG_GLF = 3 };  /* Artificial_type */
/* XFG_FP64: FP64 path; single-gas kernels use fused multiply-add, mixture kernels are compiled
 *           without contraction (their characteristic system amplifies rounding differences).
 * XFG_MIXED: FP32 reconstruction / splitting / WENO with the FP64 state and RK stage sum.
 * XFG_FP64_STRICT: FP64 without contraction anywhere: the operation sequence of the reference's
 *           CPU build, bit-identical to it where the math library calls agree. */
enum xfg_precision { XFG_FP64 = 0, XFG_MIXED = 1, XFG_FP64_STRICT = 2 };

typedef struct xfg_scheme {
    int cop;               /* COP: multi-component (Emax = NUM_SPECIES + 4) or single gas (Emax = 5) */
    int num_species;       /* NUM_SPECIES (1 without COP) */
    int scheme_order;      /* SCHEME_ORDER: 5 (WENO5-JS) or 7 (WENO7) */
    int artificial_type;   /* Artificial_type: 1 Roe, 2 local LF, 3 global LF */
    int thermo;            /* Thermo: 1 NASA-9, 0 JANAF / NASA-7 */
    int ghost_species;     /* GhostSpecies: renormalise Y and write it back into U */
    double ncop_gamma;     /* NCOP_Gamma, ratio of specific heats without COP */
    int precision;         /* xfg_precision */
    int positivity;        /* PositivityPreserving (src/read_ini/settings/read_json.cpp:68): the flux
                              limiter of FDM_Method/positive-definite_eigen/PositivityPreserving_kernels.hpp
                              after each face sweep (ConVenction_block.hpp:328-410); 0 = off */
    int viscous;           /* Visc | Visc_Heat << 1 | Visc_Diffu << 2 (cmake/init_options.cmake:81-91):
                              fourth-order viscous, heat-conduction and diffusion fluxes subtracted
                              from the face fluxes (ConVenction_block.hpp:419-566); mixtures only,
                              needs xfg_set_transport */
} xfg_scheme;

/* Transport data of a viscous run: the fitted coefficients Setup::GetFitCoefficient computes
 * (src/read_ini/src/viscfit.cpp:148-200) and the species characteristics of transport_data.dat,
 * as Thermal holds them (src/include/global_setup.h:202-208), plus the two diffusion limiters of
 * Block (src/read_ini/src/iniset.cpp:358-359). */
#define XFG_FIT_ORDER 4      /* order_polynominal_fitted */
#define XFG_SPCH 9           /* SPCH_Sz: geo, epsilon_kB, d, mue, alpha, Zrot_298, Wi, Vis, SID */
typedef struct xfg_transport {
    int num_species;
    double visc[XFG_MAX_SPECIES * XFG_FIT_ORDER];                     /* ln(mu) in powers of ln(T) */
    double therm[XFG_MAX_SPECIES * XFG_FIT_ORDER];                    /* ln(kappa) in powers of ln(T) */
    double dkj[XFG_MAX_SPECIES * XFG_MAX_SPECIES * XFG_FIT_ORDER];    /* ln(p D_kj), k-major */
    double species_chara[XFG_MAX_SPECIES * XFG_SPCH];
    double yil_limiter, dim_limiter;                                  /* Block::Yil_limiter, Dim_limiter */
} xfg_transport;

/* Arrays a caller can read back (xfg_get_array). */
enum xfg_array {
    XFG_U = 0, XFG_U1 = 1, XFG_LU = 2,                /* AoS, Emax per cell */
    XFG_RHO = 3, XFG_P = 4, XFG_U_VEL = 5, XFG_V_VEL = 6, XFG_W_VEL = 7,
    XFG_C = 8, XFG_H = 9, XFG_T = 10, XFG_GAMMA = 11, XFG_E = 12, XFG_CP = 13, XFG_R = 14,
    XFG_Y = 15,                                       /* AoS, NUM_SPECIES per cell */
    XFG_FWX = 16, XFG_FWY = 17, XFG_FWZ = 18          /* face fluxes Fwall, AoS Emax per cell */
};

typedef struct xfg_handle xfg_handle;

/* Text of the last error raised on this host thread. */
const char *xfg_last_error(void);

/* Library build information: kernel instantiations, architecture. */
const char *xfg_build_info(void);

/* Create the device state of one fluid block: replaces Fluid::Fluid + Fluid::AllocateFluidMemory
 * (src/Fluids.cpp:90-100, :270-583) and Setup::CpyToGPU (src/read_ini/src/gpucopy.cpp:5-36).
 * device: CUDA ordinal. All device memory of the handle is allocated here. */
int xfg_create(const xfg_block *block, const xfg_scheme *scheme, const xfg_thermal *thermal,
               int device, xfg_handle **out);

/* Free the handle: replaces Fluid::~Fluid (src/Fluids.cpp:103-252). */
int xfg_destroy(xfg_handle *h);

/* Load the conserved state U (AoS, Emax*Xmax*Ymax*Zmax doubles) and, for COP, the temperature
 * that warm-starts the Newton iteration (Xmax*Ymax*Zmax doubles, may be NULL: keeps the stored T).
 * Replaces the U/T writes of Fluid::InitialU and XFLUIDS::Read_Ubak (src/XFLUIDS.cpp:689-724).
 * Also copies U into U1, as InitialUFKernel does (sample ini_sample.hpp). */
int xfg_set_state(xfg_handle *h, const double *U_aos, const double *T);

/* Copy one array out (host or device pointer): replaces the q.memcpy reads of Fluid's public
 * buffers in XFLUIDS::Output / CopyDataFromDevice (src/XFLUIDS.cpp:644-656, :726-828). */
int xfg_get_array(xfg_handle *h, int which, double *out);

/* Copy one array in (host or device pointer), for which = XFG_U, XFG_U1 (AoS) or XFG_T: the
 * writes a caller makes into Fluid's public device buffers d_U / d_U1 / d_fstate.T (e.g. the
 * memcpy of XFLUIDS::Read_Ubak, src/XFLUIDS.cpp:689-724). T is the warm start of the next
 * temperature Newton iteration. */
int xfg_set_array(xfg_handle *h, int which, const double *in);

/* Ghost-cell fill of U (flag 0) or U1 (flag != 0): replaces Fluid::BoundaryCondition
 * (src/Fluids.cpp:922-933) -> FluidBoundaryCondition (src/solver_BCs/BCs_block.cpp:4-218). */
int xfg_boundary(xfg_handle *h, int flag);

/* Primitive recovery and physical fluxes on all cells of U (flag 0) or U1: replaces
 * Fluid::UpdateFluidStates (src/Fluids.cpp:935-944) -> UpdateFluidStateFlux
 * (src/solver_UpdateStates/UpdateStates_block.cpp:7-191). *error receives the reference's
 * "error captured" flag; timers4 (may be NULL) gets the 4 timers the reference returns. */
int xfg_update_states(xfg_handle *h, int flag, int *error, float *timers4);

/* Convective right-hand side LU of U (flag 0) or U1: replaces Fluid::ComputeFluidLU
 * (src/Fluids.cpp:951-961) -> GetLU (src/solver_Reconstruction/FDM_Method/ConVenction_block.hpp:10-617).
 * timers23 (may be NULL) gets the 23 timers the reference returns (unused ones are 0). */
int xfg_compute_lu(xfg_handle *h, int flag, float *timers23);

/* SSP-RK3 stage combination: replaces Fluid::UpdateFluidURK3 (src/Fluids.cpp:946-949) ->
 * UpdateURK3rd (src/solver_UpdateStates/UpdateStates_block.cpp:193-211). */
int xfg_update_rk3(xfg_handle *h, int flag, double dt);

/* CFL time step from the primitives of the last xfg_update_states: replaces Fluid::GetFluidDt
 * (src/Fluids.cpp:897-920) -> GetDt (src/solver_GetDt/GlobalDt_block.hpp:6-114). */
int xfg_get_dt(xfg_handle *h, double *dt);

/* NaN / Inf / negative-density check of the stage state and LU: replaces Fluid::EstimateFluidNAN
 * (src/Fluids.cpp:963-1040). *error = 1 when captured; error_pos (may be NULL) receives
 * Emax+4 ints in the reference's layout (per-component codes, then i, j, k). */
int xfg_estimate_nan(xfg_handle *h, int flag, int *error, int *error_pos);

/* One full time step as XFLUIDS::Evolution runs it (src/XFLUIDS.cpp:196-214 and
 * SinglePhaseSolverRK3rd :377-411): dt from the primitives left by the previous stage-3
 * UpdateStates, clipped to target_t, then three RK stages, fused into few kernels. On return *t
 * is the new time and *dt the step taken. Call xfg_update_states once before the first step, as
 * main.cpp:45-47 does. */
int xfg_step(xfg_handle *h, double target_t, double *t, double *dt);

/* Advance up to nsteps steps toward target_t with the step sequence of xfg_step, dt kept on the
 * device and the launches replayed from a captured CUDA graph. Stops early once target_t is
 * reached. *t and *steps_done report the result; the call synchronises once at the end. */
int xfg_advance(xfg_handle *h, int nsteps, double target_t, double *t, int *steps_done);

/* xfg_advance with the device time of the replayed steps (CUDA events on the handle's stream
 * around the graph launches) written to *device_ms. */
int xfg_advance_timed(xfg_handle *h, int nsteps, double target_t, double *t, int *steps_done, float *device_ms);

/* Number of kernel launches of one fused step (xfg_step / one xfg_advance replay). */
int xfg_launches_per_step(xfg_handle *h, int *n);

/* Page-locked host buffers for callers that stream states to and from the device. */
int xfg_pinned_alloc(size_t bytes, void **ptr);
int xfg_pinned_free(void *ptr);

/* One fused step like xfg_step with CUDA events between the launches: ms_out[7] receives the
 * device time of each phase summed over the three stages: [0] dt, [1] boundary, [2] primitive
 * recovery, [3..5] face fluxes x/y/z, [6] divergence + RK update. Advances the state. A handle that
 * runs the fused mixed stage (2D single gas, XFG_MIXED, WENO5, LLF or Roe, no positivity limiter:
 * primitive recovery, both face sweeps, divergence and RK update in one kernel per stage) reports
 * that kernel in [3] and [2], [4..6] are 0; [1] then includes the ghost cells' dt maxima. */
int xfg_time_phases(xfg_handle *h, double target_t, float *ms_out);

/* Current simulated time of the handle (set by xfg_step / xfg_advance, reset by xfg_set_time). */
int xfg_set_time(xfg_handle *h, double t);
int xfg_get_time(xfg_handle *h, double *t);

/* Wait for all work of the handle's stream. */
int xfg_synchronize(xfg_handle *h);

/* Device pointer of a handle array (SoA inside the handle) and its pitch in elements, for callers
 * that keep their own device-side post-processing. */
int xfg_device_array(xfg_handle *h, int which, double **ptr, size_t *pitch);

/* Measure this GPU's FP64 and FP32 FMA throughput (FLOP/s, FMA = 2) with a register-resident
 * FMA chain; used as the roofline denominator of the compute-bound kernels. out[0] = FP64,
 * out[1] = FP32, out[2] = SM clock (MHz) reported by the driver during the run (0 if unknown). */
int xfg_measure_pipe_peaks(int device, double *out);

/* Transport data of a viscous scheme (xfg_scheme.viscous != 0); required before the first
 * xfg_compute_lu / xfg_step of such a handle. The drop-in copies Setup::h_thermal's fitted
 * coefficients and species characteristics. */
int xfg_set_transport(xfg_handle *h, const xfg_transport *tr);

/* Checkpoint files in the reference's format (XFLUIDS::Output_Ubak / Read_Ubak,
 * src/XFLUIDS.cpp:658-724): int Step, double Time, float duration, then U in the reference layout
 * (Emax doubles per cell, ghosts included), packed. Read loads U (and U1 = U) and sets the
 * handle's time; like Read_Ubak it restores no temperature (mixtures warm-start the Newton
 * iteration from the T already in the handle). Follow with xfg_boundary + xfg_update_states. */
int xfg_checkpoint_write(xfg_handle *h, const char *path, int step, double time, float duration);
int xfg_checkpoint_read(xfg_handle *h, const char *path, int *step, double *time, float *duration);

/* ------------------------------------------------------------------------------------------
 * Ensemble of independent grids (batched ensemble, request serving).
 * No single counterpart in the reference, which advances one block per process: the members are
 * XFLUIDS runs of the same scheme (each member's step is XFLUIDS::Evolution's loop body with its
 * own dt and target time, src/XFLUIDS.cpp:172-214), advanced together by batched kernels.
 * ------------------------------------------------------------------------------------------ */
typedef struct xfg_ensemble xfg_ensemble;

/* Create an ensemble with `capacity` member slots and a device pool of pool_bytes from which the
 * members are sub-allocated (admission by HBM budget). scheme: single gas (cop = 0) or a mixture of
 * 5 species (cop = 1, num_species = 5, thermal holding its tables; GhostSpecies and NASA-9 / JANAF
 * as the single-grid path; inviscid, or viscous stress / heat conduction with the transport data
 * of xfg_ensemble_set_transport), ROE, LLF or GLF (running maxima per member), WENO5 / WENO-CU6 /
 * WENO7, positivity limiter on or off, precision XFG_FP64 or XFG_MIXED. The batched kernels of
 * each gas model and form are compiled with the contraction flags of the single-grid kernels, so a
 * member advances as the same block alone in a handle would. */
int xfg_ensemble_create(int capacity, size_t pool_bytes, const xfg_scheme *scheme, const xfg_thermal *thermal,
                        int device, xfg_ensemble **out);
int xfg_ensemble_destroy(xfg_ensemble *e);

/* Device bytes one single-gas member of this block takes from the pool; _for: a member of this
 * block under the given scheme (single gas or mixture). */
size_t xfg_ensemble_member_bytes(const xfg_block *block, int precision);
size_t xfg_ensemble_member_bytes_for(const xfg_block *block, const xfg_scheme *scheme);

/* Viscous mixture ensembles: the fitted transport data of the species, shared by every member
 * (as xfg_set_transport for one handle); required before the first xfg_ensemble_advance. */
int xfg_ensemble_set_transport(xfg_ensemble *e, const xfg_transport *tr);

/* Admit a member: state U (AoS, host or device), target time; runs BoundaryCondition(U) and
 * UpdateStates(U) for it (main.cpp:45-47). Returns 0 and *slot, 1 when no slot is free, 2 when the
 * pool has no room (the caller retries after members leave). */
int xfg_ensemble_add(xfg_ensemble *e, const xfg_block *block, const double *U_aos, double target_t, int *slot);
/* xfg_ensemble_add with the member's temperature (Xmax*Ymax*Zmax doubles, host or device), the warm
 * start of its temperature Newton iteration; required for a mixture, may be NULL for a single gas.
 * A mixture member cannot come from xfg_ensemble_add_checkpoint (the file holds no temperature). */
int xfg_ensemble_add_t(xfg_ensemble *e, const xfg_block *block, const double *U_aos, const double *T,
                       double target_t, int *slot);

/* Release a member's slot and pool memory. */
int xfg_ensemble_remove(xfg_ensemble *e, int slot);

/* nsteps fused steps of every active member (members past their target time do nothing),
 * replayed from a CUDA graph when use_graph (the graph is re-captured after membership changes).
 * A member whose step produced an error (the codes of xfg_step) stops at that step; the others go
 * on. Synchronises once; *device_ms (may be NULL) receives the device time of the steps. Returns
 * 0, or the worst error code among the active members (10000 state NaN / negative density, 1
 * primitive error), or < 0 on a CUDA or argument error. */
int xfg_ensemble_advance(xfg_ensemble *e, int nsteps, int use_graph, float *device_ms);

/* Time, step count and done flag (also set for a member stopped by an error) of a member as of
 * the last advance; returns its error code (0, 1 or 10000 as xfg_step). */
int xfg_ensemble_status(xfg_ensemble *e, int slot, double *t, int *steps, int *done);

/* Copy a member's state U out (AoS, host or device pointer). */
int xfg_ensemble_get_state(xfg_ensemble *e, int slot, double *U_aos);

/* A member as a checkpoint file of the reference's format (see xfg_checkpoint_write), with its
 * step count and time; and a member admitted from such a file (U, time and step count restored,
 * then BoundaryCondition + UpdateStates as xfg_ensemble_add; returns 1 / 2 like it). The file
 * holds no dt: lam_out (3 doubles, may be NULL) receives the GetDt maxima the member's next step
 * would use, and lam_in (may be NULL) restores them, so that a resumed member takes the steps the
 * saved one would have taken; without it the next dt comes from the restored U, as after the
 * reference's Read_Ubak. */
int xfg_ensemble_checkpoint_write(xfg_ensemble *e, int slot, const char *path, float duration, double *lam_out);
int xfg_ensemble_add_checkpoint(xfg_ensemble *e, const xfg_block *block, const char *path, double target_t,
                                const double *lam_in, int *slot);

/* Launch schedule of the batched step (the autotuner's knobs). None changes the operations of a
 * step: FP64 results are bit-identical under every schedule, mixed-precision results agree to FP32
 * rounding (FMA contraction of FP32 expressions may differ between kernel forms).
 *   XFG_ENS_LARGEST_FIRST  members in the launch tables largest first (1, default) or by slot (0)
 *   XFG_ENS_FUSED_FACES    all face sweeps of a stage in one launch (1) or one launch each (0, default)
 *   XFG_ENS_GRAPH_STEPS    fused steps per captured CUDA graph, 1..64 (default 1)
 *   XFG_ENS_TILE_1D..3D    face tile of a size class (1D; 2D below 384 cells per side; 2D from 384;
 *                          3D): log2 of its x extent, 3..7, the tile being 2^v x 128/2^v faces
 *                          (defaults 7, 5, 5, 5) */
enum {
    XFG_ENS_LARGEST_FIRST = 0,
    XFG_ENS_FUSED_FACES = 1,
    XFG_ENS_GRAPH_STEPS = 2,
    XFG_ENS_TILE_1D = 3,
    XFG_ENS_TILE_2D_SMALL = 4,
    XFG_ENS_TILE_2D_LARGE = 5,
    XFG_ENS_TILE_3D = 6
};
int xfg_ensemble_set_option(xfg_ensemble *e, int option, int value);
int xfg_ensemble_get_option(xfg_ensemble *e, int option, int *value);

size_t xfg_ensemble_free_bytes(xfg_ensemble *e);
int xfg_ensemble_active(xfg_ensemble *e);

/* Right-hand side of one state without any device allocation.
 *
 * No counterpart in the reference. For callers that cannot allocate device memory (a host
 * application or plugin host that owns every allocation or forbids the driver allocator, a
 * real-time loop where an allocation and its implicit synchronisation are not allowed): the caller
 * passes device pointers to the state U (reference AoS layout, all cells), to the temperature T
 * (Newton warm start, Xmax*Ymax*Zmax doubles; required for a mixture, may be NULL otherwise) and to
 * the output LU (AoS, Emax per cell; inner cells are written, ghost cells are 0). The function
 * applies the boundary conditions to its own copy of U, recovers the primitives and computes LU
 * as xfg_boundary + xfg_update_states + xfg_compute_lu do, on `stream` (a cudaStream_t, 0 = legacy
 * default stream), without synchronising. FP64 forms only (precision XFG_FP64 or XFG_FP64_STRICT).
 * Unlike xfg_update_states, the call reports no non-physical state (negative or NaN density,
 * pressure or temperature in an inner cell): it returns 0 once the launches are queued, and such a
 * state leaves NaN or Inf in LU, which the caller checks.
 *
 * The scratch holds 8 Mi doubles; a block needs (arrays) x (cells rounded up to 64) of them, with
 * 37 arrays for a 1D single gas (about 226 k cells at most), 50 for a 2D single gas (about 167 k
 * cells), 63 for a 3D single gas (about 133 k cells) and more for mixtures (96 for a 3D 5-species
 * mixture, about 87 k cells).
 *
 * Every intermediate array lives in one file-scope device array of XFG_NOALLOC_MAX_SCRATCH_BYTES,
 * which every GPU that loads the library holds until the process exits; blocks that need more are
 * rejected with a status < 0 and a message in xfg_last_error(). The first call on a device looks
 * up the array's device address (cudaGetSymbolAddress) with that device current: make it before
 * any stream capture. All calls share the array, which keeps the previous call's contents (the
 * words that must start at zero are cleared by each call): calls that overlap on the GPU, on
 * different streams or from different host threads, race and must be serialised by the caller. */
#define XFG_NOALLOC_MAX_SCRATCH_BYTES (64u << 20)
int xfg_compute_lu_noalloc(const xfg_block *block, const xfg_scheme *scheme, const xfg_thermal *thermal,
                           const double *U_aos, const double *T, double *LU_aos, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* XFLUIDS_GB300_H */
