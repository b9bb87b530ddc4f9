/*
 * astg.h -- C ABI of the GB300 octree smoke-step library (libastgrid_gpu.so).
 *
 * Drop-in boundary for the AST-modified octree smoke step of YuweiXiao/AST-Grid
 * (OctreeOmniGridSolver3 / OmniBoundarySolver3 / PCGSolver).  Host callers pass plain pointers
 * and sizes; all device memory belongs to the handle; every call returns an astg_status and no
 * C++ exception crosses the boundary.  One CUDA stream per handle; a handle is
 * thread-compatible, not thread-safe.  Different handles may be driven from different host threads
 * at the same time: their work runs side by side on the device (a step keeps one 16-SM cluster
 * busy for most of its time), and each handle's results are the same as when it runs alone.
 * Arrays exchanged through astg_get / astg_set are in the
 * reference's storage order (level-major, then the reference's layout index: non-ghost cells in
 * raster z-y-x order followed by ghosts in discovery order), so they can be compared with the
 * reference's own grids element by element.
 */
#ifndef ASTG_H
#define ASTG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum astg_status {
    ASTG_OK = 0,
    ASTG_BAD_ARG = 1,
    ASTG_CUDA_ERROR = 2,
    ASTG_NOT_CONVERGED = 3,
    ASTG_DEVICE_WAIT_TIMEOUT = 4,
    ASTG_NAN_DETECTED = 5,
    ASTG_LAYOUT_ERROR = 6,
    ASTG_NO_DEVICE = 7
} astg_status;

typedef enum astg_precision {
    ASTG_FP64 = 0,  /* all-FP64 PCG, the drop-in form */
    ASTG_MIXED = 1  /* FP32 SpMV / preconditioner / axpy inside FP64 defect correction */
} astg_precision;

/* Solver and scene parameters.  Defaults (astg_default_params) are the benchmark scene:
 * unit cube, walls closed except z+, sphere source r = 0.06 at (0.5, 0.5, 0.12), buoyancy -0.1
 * (density) and +1.0 (temperature), no decay, rho = 2, MIC(0) omega 0.97 / min diagonal ratio
 * 0.25, PCG tolerance 1e-6 relative to |b|_inf, at most 3000 iterations. */
typedef struct astg_params {
    int coarsest;         /* cells per axis on the coarsest level */
    int levels;           /* numOctreeLayer: level 0 is the finest, res = coarsest << (levels-1) */
    double tol;           /* PCG tolerance factor (set_solver_parameters) */
    int max_iter;
    double omega;         /* MIC(0) modification parameter */
    double min_diag;      /* MIC(0) minimum diagonal ratio */
    double rho;           /* fluid density (setRho) */
    double buoy_density;  /* _buoyancySmokeDensityFactor */
    double buoy_temp;     /* _buoyancyTemperatureFactor */
    double decay;         /* _smokeDecayFactor and _temperatureDecayFactor */
    int closed_mask;      /* walls closed: bit 0 x+, 1 x-, 2 y+, 3 y-, 4 z+, 5 z- */
    int tilt_adaptivity;  /* enableTiltAdaptivity */
    double src_x, src_y, src_z, src_r;  /* sphere source re-injected every step (r <= 0: none) */
    double noise;         /* amplitude of the initial divergence-free curl noise */
    uint64_t seed;        /* seed of the curl noise */
    int precision;        /* astg_precision of astg_step's projection */
    int device;           /* CUDA device ordinal */
} astg_params;

typedef struct astg_handle astg_handle;

typedef struct astg_solve_stats {
    int iterations;       /* PCG iterations (inner iterations for ASTG_MIXED) */
    int outer;            /* defect-correction cycles (ASTG_MIXED), 0 for FP64 */
    int converged;
    int n;                /* system size */
    long long nnz;
    double residual;      /* final |r|_inf */
    double tolerance;     /* tol * |b|_inf */
    double ms;            /* device time of the solve (CUDA events) */
} astg_solve_stats;

typedef struct astg_step_stats {
    astg_solve_stats solve;
    double ms_total;      /* device time of the whole step */
    double ms_force;      /* device time of addForce and the wall / ghost constraint after it */
    double ms_project;    /* the projection's PCG solve (its astg_solve_stats.ms) */
    double ms_advect;     /* tilt adaptivity, the advection of scalars and velocity, the decay */
} astg_step_stats;

/* refineSplitMapByObstacleSdf (include/octree_util.h:17-47), a host-side utility for building the
 * split_map that astg_create takes: every block of 2^level finest cells whose split value is `level`
 * and whose SDF, sampled at the block centre, lies in [lo, hi] is set to level - 1.  split_map and
 * sdf are res^3 arrays (index (z * res + y) * res + x; sdf at the finest cell centres, inside the
 * obstacle negative).  ASTG_BAD_ARG when res is not divisible by 2^level.  Needs no device. */
astg_status astg_refine_split_map(int32_t* split_map, int res, int level, const double* sdf, double lo, double hi);
/* The same on device memory of the current device (split_map and sdf device pointers), one thread
 * per block on `stream` (a cudaStream_t; NULL: the default stream), asynchronous; the result equals
 * astg_refine_split_map's.  ASTG_BAD_ARG for host pointers or bad sizes, ASTG_CUDA_ERROR when the
 * launch fails. */
astg_status astg_refine_split_map_device(int32_t* split_map, int res, int level, const double* sdf, double lo,
                                         double hi, void* stream);

/* Fills p with the benchmark defaults for a given coarsest resolution and level count. */
void astg_default_params(astg_params* p, int coarsest, int levels);

/* OctreeOmniGridSolver3(res, spac, name) + initialize() (src/octree_omnigrid_solver3.cpp:45-149):
 * builds the octree from split_map (res^3 level ids, index (z*res + y)*res + x; NULL = the
 * benchmark scene's refinement around the source), constrains the tilted cells, sets the cut-cell
 * weights, uploads everything and initialises the velocity with the curl noise. */
astg_status astg_create(const astg_params* p, const int32_t* split_map, astg_handle** out);
void astg_destroy(astg_handle* h);
const char* astg_last_error(const astg_handle* h);

/* Solver::update(dt) with useFixedTimeStep (src/solver.cpp:8-46) ->
 * OctreeOmniGridSolver3::onUpdate (src/octree_omnigrid_solver3.cpp:222-249). */
astg_status astg_step(astg_handle* h, double dt, astg_step_stats* stats);

/* Solver::update(dt) with useFixedTimeStep = false (src/solver.cpp:21-41), the reference's default:
 * the frame is split into sub-steps of remaining / k, k = numberOfSubTimeSteps(remaining) =
 * max(1, ceil(cfl(remaining) / maxCfl)) recomputed from the current velocity before each sub-step,
 * until at most EPSILON remains (src/octree_omnigrid_solver3.cpp:1060-1063).  *substeps (may be
 * NULL) receives the number of sub-steps; stats are the last sub-step's, with the times summed over
 * the frame.  ASTG_NOT_CONVERGED when any sub-step's solve did not converge. */
astg_status astg_update(astg_handle* h, double dt, int* substeps, astg_step_stats* stats);

/* OmniBoundarySolver3::updateCollider (src/omni_boundary_solver3.cpp:17-32) with a Sphere3 collider
 * of radius `radius` centred at (cx, cy, cz), as OctreeOmniGridSolver3::initObstacle builds the stock
 * one ((0.5, 0.5, 0.45), 0.1; src/octree_omnigrid_solver3.cpp:150-158): the SDF grid is computed on
 * the device at the finest cell centres, then the cut-cell weights and solid masks as for astg_set
 * "collider_sdf".  radius <= 0 removes the collider.  The inside-solid projection keeps taking its
 * normals from "collider_centre" (the reference hard-codes it, whatever the collider). */
astg_status astg_set_collider_sphere(astg_handle* h, double cx, double cy, double cz, double radius);

/* setMaxCfl (include/octree_omnigrid_solver3.h:29); the default is the reference's 3. */
astg_status astg_set_max_cfl(astg_handle* h, double max_cfl);

/* OctreeOmniGridSolver3::cfl(dt) (src/octree_omnigrid_solver3.cpp:1066-1122: dt times the largest
 * MAC face value, counted from 0, over the finest spacing, truncated to int) and
 * numberOfSubTimeSteps(dt) for the current velocity; either pointer may be NULL. */
astg_status astg_cfl(astg_handle* h, double dt, int* cfl, int* substeps);

/* One stage of onUpdate: 0 scene setup (source), 1 addForce, 2 wall constraint + velocity ghosts,
 * 3 project (:350-679), 4 constraint + ghosts + dual grid, 5 advect (:850-914). */
astg_status astg_stage(astg_handle* h, int stage, double dt);

/* PCGSolver::set_solver_parameters (include/pcgsolver/pcg_solver.h:267-274). */
astg_status astg_set_solver_parameters(astg_handle* h, double tol, int max_iter, double omega, double min_diag);
astg_status astg_set_precision(astg_handle* h, astg_precision prec);

/* Order of the floating-point reductions of the FP64 solve and of addForce's mean temperature.
 * ASTG_ORDER_LIBRARY (the default, the fast path): one fixed reduction tree for every dot product
 * and sum, one fused multiply-add for every product the PCG accumulates (sweep updates, matrix
 * rows, dot terms, vector updates); results are reproducible, and match the reference to the PCG
 * tolerance.  ASTG_ORDER_REFERENCE: the reference's own arithmetic, so the
 * solve reproduces it bit for bit: dot products in Eigen 3.3.7's SSE2 order (BLAS::dot,
 * include/pcgsolver/blas_wrapper.h:112-115), the MIC(0) sweep updates, matrix rows and vector
 * updates as a multiply and an addition or subtraction (include/pcgsolver/pcg_solver.h:211-253),
 * and the mean temperature as BLAS::sum's
 * per-worker slice sums (blas_wrapper.h:101-110, include/thread_pool.h:319-348) over `workers`
 * workers, the reference's thread-pool size (its hardware concurrency: the slices depend on it),
 * 1..256.  The reference order runs the dot products and sums as serial chains: it is a parity
 * mode, much slower than the library order.  It applies to the FP64 form (ASTG_FP64). */
typedef enum astg_order {
    ASTG_ORDER_LIBRARY = 0,
    ASTG_ORDER_REFERENCE = 1
} astg_order;
astg_status astg_set_reduction_order(astg_handle* h, astg_order order, int workers);

/* CUDA-event timing of the PCG's main kernels (forward and backward MIC(0) sweeps, SpMV + dot,
 * factorisation), read back as astg_get(h, "kernel_ms", ...).  No counterpart in the reference:
 * it replaces the BENCHMARK_SCOPED_TIMER_SECTION probes (include/global_benchmark.h:33-43). */
astg_status astg_set_profiling(astg_handle* h, int on);

/* Statistics of the last projection. */
astg_status astg_last_solve(const astg_handle* h, astg_solve_stats* out);

/* Sizes: 0 slots, 1 levels, 2 finest resolution, 3 DOFs of the last projection,
 * 4 half tilts, 5 non-zeros of the last matrix, 6 kernels launched by the library so far,
 * 7 form of the MIC(0) preconditioner: 100 + cluster size when both sweeps run fused in one
 * cluster launch, the cluster size of the global-memory cluster sweeps, or 0 for the sync-free
 * sweeps. */
long long astg_size(const astg_handle* h, int what);

/* Copy a state array out of / into the handle.  Names (element type):
 *   density_oct density_tilt heat_oct heat_tilt tilt_e (f64, slots)  mac (f64, 3 x slots)
 *   tilt_vel (f64, slots x 8)  dual_oct dual_tilt (f64, slots x 3)
 *   tilt_flags (i32, slots x 2: bit 0 largest, 1 closed, 2 fixed, 3 T-joint, 4 closed by T-joint,
 *   5 half tilt; half direction)  tilt_open (u8, slots: bit 0 open, bit 1 fixed)
 *   source_density_oct source_density_tilt (f64, slots: density the source sets, default 1)
 *   prefix "t_" = the swap-partner buffer of the reference's double-buffered grids;
 * collider_sdf (f64, res^3 at the finest cell centres, index (z * res + y) * res + x:
 *   OmniBoundarySolver3::updateCollider's SDF grid, inside negative; 0 bytes without a collider;
 *   set: 0 bytes removes the collider, else the cut-cell weights are recomputed);
 * write only: collider_centre (f64 x 3: the centre the inside-solid
 *   projection takes its normals from, the reference's hard-coded (0.5, 0.5, 0.45) by default);
 * read only: slot_coords (i32, slots x 4: x y z flags) level_sizes (i32, levels x 3)
 *   half_tilts t_joints closed_by_half_tilt (i64 packed level coordinates) split_map (i32)
 *   w_mac w_tilt dual_tables (f64) pindex_oct pindex_tilt (i32) A_rowptr A_col (i32) A_val b p
 *   (f64) pcg_iters (i32 x 2) ambT (f64).
 * bytes must equal the array's size (astg_get with dst = NULL returns ASTG_BAD_ARG and stores
 * the size in *bytes_needed when that pointer is not NULL). */
astg_status astg_get(astg_handle* h, const char* name, void* dst, size_t bytes, size_t* bytes_needed);
astg_status astg_set(astg_handle* h, const char* name, const void* src, size_t bytes);

/* Stand-alone PCGSolver::solve(A, b, x) on a CSR matrix held in host memory
 * (include/pcgsolver/pcg_solver.h:366-426): MIC(0) preconditioner, stop when
 * |r|_inf <= rel_tol * |b|_inf.  Rows must be sorted by column and the pattern symmetric. */
astg_status astg_solve(astg_handle* h, int n, const int32_t* rowptr, const int32_t* col, const double* val,
                       const double* b, double* x, double rel_tol, int max_iter, astg_precision prec,
                       astg_solve_stats* stats);

/* astg_solve for nrhs right-hand sides of one matrix (b and x: nrhs rows of n values).  The
 * factorisation is computed once; the solves run side by side (each keeps one cluster of the
 * preconditioner busy, and up to 8 clusters fit on the device), each returning the result astg_solve
 * returns for its right-hand side, bit for bit.  stats (nrhs entries), wall_ms (host time of the whole
 * call, copies included) and lanes (solves run side by side) may be NULL.  No counterpart in the
 * reference, which solves one right-hand side per PCGSolver::solve call. */
astg_status astg_solve_batch(astg_handle* h, int n, const int32_t* rowptr, const int32_t* col, const double* val,
                             int nrhs, const double* b, double* x, double rel_tol, int max_iter, astg_precision prec,
                             astg_solve_stats* stats, double* wall_ms, int* lanes);

/* Largest MAC face value over all faces, starting from 0 (signed, as the reference's max(v)),
 * the quantity OctreeOmniGridSolver3::cfl divides by the finest spacing
 * (src/octree_omnigrid_solver3.cpp:1066-1122). */
astg_status astg_max_velocity(astg_handle* h, double* out);

/* OctreeOmniGridSolver3::restart (src/octree_omnigrid_solver3.cpp:1015-1057) from the reference's
 * binary dumps (src/viewer/grid_dump.cpp:280-615, the files saveResult writes with saveStatus):
 * tilt-E, density, heat and velocity go into both buffers, then the velocity ghosts, the dual grid
 * and its ghosts are recomputed.  layout_file (may be NULL) must describe the handle's own octree
 * (same nodes, order and flags), else ASTG_LAYOUT_ERROR; the octree is not rebuilt.  boundary_file
 * is not read and frame is not kept, as in the reference.  A file that cannot be read, is
 * truncated or has other sizes returns ASTG_BAD_ARG and leaves the state unchanged. */
astg_status astg_restart(astg_handle* h, int frame, const char* layout_file, const char* boundary_file,
                         const char* tilt_file, const char* density_file, const char* heat_file,
                         const char* velocity_file);

/* The dumps saveResult writes with saveStatus (src/octree_omnigrid_solver3.cpp:148, 996-1007;
 * dumpOctreeLayout3dBinary, dumpOctreeOmniTiltE3dBinary, dumpOctreeOmniScalar3dBinary,
 * dumpOctreeOmniFaceCentered3dBinary in src/viewer/grid_dump.cpp) of the current state, readable
 * by the reference's restart; NULL skips a file; parent directories are created. */
astg_status astg_save_checkpoint(astg_handle* h, const char* layout_file, const char* tilt_file,
                                 const char* density_file, const char* heat_file, const char* velocity_file);

typedef struct astg_extrap_stats {
    long long assigned;   /* nodes given an extrapolated value */
    int passes;           /* parallel passes (dependency rounds) used */
    double ms;            /* device time (CUDA events) */
} astg_extrap_stats;

/* FmmLevelSetSolver3::extrapolate (include/jet/fmm_levelset_solver3.h:84-408) with no cached
 * marker, in place on the scalar omni field `field` ("density" or "heat": octagon and tilt values
 * of the current state).  sdf is a signed distance grid of sdf_res^3 cell-centred values on the
 * unit cube (index (z*res + y)*res + x), sampled trilinearly like CellCenteredGrid::sample.  Nodes
 * whose sample v satisfies v < -valid_offset * d are known (d: dx_l*sqrt(3)/2 for octagons, the
 * tilt size e for tilts, dx_l for half tilts); the others are filled outward in increasing SDF
 * order with the mean of their known neighbours, up to max_distance_factor * dx_0 (the finest
 * spacing).  Ghost values are left as they are, as in the reference. */
astg_status astg_extrapolate(astg_handle* h, const char* field, const double* sdf, int sdf_res, double valid_offset,
                             double max_distance_factor, astg_extrap_stats* stats);

/* Mean temperature ambT of addForce (src/octree_omnigrid_solver3.cpp:922-929) over an octagon heat
 * array the caller keeps in its own device memory.  It is the reduction astg_step runs in its force
 * stage, with the same fixed summation tree, so the result equals astg_get(h, "ambT") bit for bit
 * for the same heat.  No counterpart in the reference: it exists for callers that must not
 * allocate, such as a framework whose caching allocator has reserved most of the device's memory,
 * or a per-step loop on a shared device that cannot take the device-wide synchronisation of
 * cudaMalloc / cudaFree.  It takes no handle and allocates nothing: its scratch (the chunk partials)
 * is one static 64 KiB device array per device.
 *   d_heat_oct   device pointer: the heat of all levels in "heat_oct" order (level-major, then the
 *                reference's layout index, ghosts included)
 *   level_slots  host array of `levels` counts: slots (cells + ghosts) per level, column 2 of
 *                astg_get(h, "level_sizes")
 *   d_amb        device pointer receiving one double
 *   stream       the cudaStream_t to run on (NULL: the legacy default stream); the call returns once
 *                the work is queued, and d_amb is valid when the stream reaches it
 *   err, errlen  optional buffer for the reason of a failed call
 * Limits: 1 <= levels <= 6; at most 2048 * 2048 slots per level; the sum over levels of
 * ceil(slots / 2048) at most 8192.  Larger inputs return ASTG_BAD_ARG and say which limit failed.
 * Nothing in the scratch needs to start at zero: each call writes every partial it reads.
 * The first call with each device current looks up the scratch's address (cudaGetSymbolAddress),
 * which may load this library's device code onto that device; make that first call before any
 * stream capture begins.  The address is kept with the context it was taken in: after the
 * device's context is destroyed and created again (cudaDeviceReset), the next call looks it up
 * anew, and should again come before any capture.  ASTG_CUDA_ERROR reports only the failure of this
 * call's own launches; an error another call left pending on the host thread is neither reported
 * nor cleared.  All calls on one device share the scratch: calls whose kernels may
 * overlap in time (different streams, or host threads without ordering between them) race on it
 * and must be serialised by the caller. */
astg_status astg_mean_temperature_noalloc(const double* d_heat_oct, const int64_t* level_slots, int levels,
                                          double* d_amb, void* stream, char* err, size_t errlen);

/* ---------------------------------------------------------------- reverse mode (adjoint)
 * No counterpart in the reference, which has no gradients: the transposes of the step's stages for a
 * window of steps with the octree topology frozen (astg_params.tilt_adaptivity = 0, so the tilt-E
 * state, the DOF map and the pressure matrix stay fixed).  The advection transpose is the transposed
 * octree interpolation (scattered with atomics) plus the chain through the RK2 back-trace; the
 * projection transpose is one solve with the same SPD matrix (MIC(0)-PCG, the precision and
 * tolerance of astg_set_precision / astg_set_solver_parameters).
 * Cotangents are exchanged through astg_get / astg_set under the names
 *   adj_density_oct adj_density_tilt adj_heat_oct adj_heat_tilt adj_mac adj_tilt_vel adj_dual_oct
 *   adj_dual_tilt (f64, the shapes of the state arrays) and adj_source_density_oct /
 *   adj_source_density_tilt (f64, slots: gradients of the per-slot source densities
 *   "source_density_oct" / "source_density_tilt", which default to 1). */
typedef struct astg_adjoint_stats {
    int steps;              /* taped steps differentiated */
    int checkpoints;        /* checkpoints held (0 when every step's advection input was kept) */
    int recomputed_steps;   /* forward steps re-run from checkpoints during the pass */
    int solves;             /* adjoint pressure solves */
    long long pcg_iterations;  /* their PCG iterations (inner iterations for ASTG_MIXED) */
    double ms;              /* device time of the whole reverse pass (CUDA events) */
    double ms_recompute;    /* of which re-running forward steps */
    long long tape_bytes;   /* device memory held by the tape */
} astg_adjoint_stats;

/* enableTiltAdaptivity (include/octree_omnigrid_solver3.h:23-57, read in advect,
 * src/octree_omnigrid_solver3.cpp:852).  Turning it off also copies the current tilt-E state into the
 * swap-partner buffer, so the octree topology stays frozen from here on (the reference swaps the two
 * tilt-E buffers every step, which with the flag cleared mid-run would alternate between them). */
astg_status astg_set_tilt_adaptivity(astg_handle* h, int on);

/* Starts recording the astg_step calls that follow (any earlier tape is dropped).  checkpoint_every
 * = 0 keeps each step's advection input (13 doubles per slot per step); k > 0 keeps the whole state
 * every k steps (42 doubles per slot) and re-runs the steps of each segment during astg_backward.
 * ASTG_BAD_ARG when tilt adaptivity is on.  astg_stage is refused while recording. */
astg_status astg_tape_start(astg_handle* h, int checkpoint_every);
astg_status astg_tape_stop(astg_handle* h);  /* frees the tape */

/* Zeroes every cotangent array, source gradients included. */
astg_status astg_adjoint_reset(astg_handle* h);

/* Reverse pass over all taped steps.  On entry the adj_* state arrays hold the cotangent of the
 * final state (e.g. d loss / d density_oct); on return they hold the cotangent of the state at
 * astg_tape_start, and adj_source_density_* has the source gradients added.  The forward state is
 * left at the final state; the tape stays, so the pass can be repeated with another cotangent. */
astg_status astg_backward(astg_handle* h, astg_adjoint_stats* stats);

/* Vector-Jacobian product of one step (astg_step_vjp) or one stage (astg_stage_vjp, stages as in
 * astg_stage) at the current state, which is left unchanged: the adj_* arrays go from the cotangent
 * of the output to that of the input. */
astg_status astg_step_vjp(astg_handle* h, double dt);
astg_status astg_stage_vjp(astg_handle* h, int stage, double dt);

/* The samplers' weight enumeration used by the transposes, at n positions (xyz, host or device
 * memory) of the current state: what 0 -> per point {scalar sample of density, the same from the
 * weights, its gradient (3)}; what 1 -> {velocity sample (3), from the weights (3), Jacobian (9,
 * row c = d v_c / d p)}. */
astg_status astg_adjoint_probe(astg_handle* h, int what, int n, const double* pos, double* out);

#ifdef __cplusplus
}
#endif

#endif /* ASTG_H */
