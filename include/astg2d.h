/*
 * astg2d.h -- C ABI of the uniform 2-D AST smoke solver in libastgrid_gpu.so.
 *
 * Drop-in for the reference's ASTSolver<2> (include/ast_solver.h), the class its Python module
 * binds as ASTSolver2 (python_bindings/ast_solver.cc:43-54): constructor (resolution, dx,
 * adaptive_dofs), initialize(), update(dt) and getDensity().  The scene is the reference's
 * sphereSource2DSetup (source of radius 0.03 at (0.5, 0.04), buoyancy 0.5 on the heat, closed x
 * walls, open top and bottom), the projection its MIC(0)-PCG with absolute tolerance 1e-5,
 * omega 0.97 and minimum diagonal ratio 0.95, the time step Solver::update's CFL sub-stepping.
 *
 * Arrays exchanged through astg2_get / astg2_set are in the reference's storage order, x fastest:
 *   density_cell, heat_cell       nx * ny                 doubles
 *   density_vert, heat_vert       (nx + 1) * (ny + 1)     doubles (tilted cells at the vertices)
 *   mac_x                         (nx + 1) * ny           doubles
 *   mac_y                         nx * (ny + 1)           doubles
 *   tilt_vel                      4 * (nx + 1) * (ny + 1) doubles (tilted faces, per vertex)
 *   dual_vert                     2 * (nx + 1) * (ny + 1) doubles (set by each advection, open tilts)
 *   tilt_open                     (nx + 1) * (ny + 1)     uint8 (1 = open; boundary tilts stay closed)
 *   pindex_cell, pindex_vert      nx * ny, (nx+1)(ny+1)   int32 (unknown of each cell / tilt, -1 closed)
 *   A_rowptr, A_col, A_val, b, p  the last projection's CSR system, right-hand side and pressure
 *   sub_dt                        every sub-step length taken so far (host record)
 * Only the state fields (the first seven and tilt_open) can be set.  Values of closed tilts are
 * never read by the solver.
 *
 * The status codes are those of astg.h.  One CUDA stream per handle; thread-compatible.
 */
#ifndef ASTG2D_H
#define ASTG2D_H

#include <stddef.h>
#include <stdint.h>

#include "astg.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct astg2_handle astg2_handle;

typedef struct astg2_stats {
    int substeps;         /* sub-steps of the last astg2_update */
    int unknowns;         /* rows of the last projection (cells + open tilts) */
    int pcg_iterations;   /* its PCG iterations */
    int pcg_converged;
    long long nnz;
    double pcg_residual;  /* final |r|_inf */
    double ms;            /* device time of the last astg2_update or astg2_stage (CUDA events) */
    long long substeps_total;
} astg2_stats;

/* ASTSolver<2>(Size2(nx, ny), dx, adaptive_dofs) followed by initialize()
 * (include/ast_solver.h:28-50).  nx, ny >= 2, nx * ny + (nx + 1) * (ny + 1) <= 4,194,304 (the
 * reduction tree folds at most 2048 x 2048 partial sums).  On failure *out may still hold a handle
 * with the message; destroy it. */
astg_status astg2_create(int nx, int ny, double dx, int adaptive_dofs, int device, astg2_handle** out);
void astg2_destroy(astg2_handle* h);
const char* astg2_last_error(const astg2_handle* h);

/* Solver::update(dt) (src/solver.cpp:8-46): CFL sub-steps of source, force, project, advect.
 * ASTG_NAN_DETECTED when the CFL number is not finite or asks for more than 100,000 sub-steps in
 * one call (a diverged velocity field; the reference would keep stepping). */
astg_status astg2_update(astg2_handle* h, double dt);
/* one stage of a sub-step: 0 sphereSource2DSetup, 1 addForce, 2 project, 3 advect, 4 all four */
astg_status astg2_stage(astg2_handle* h, int stage, double dt);
/* getDensity() (include/ast_solver.h:72): the cell densities, nx * ny doubles */
astg_status astg2_get_density(astg2_handle* h, double* out, long long count);

/* element count and kind (0 double, 1 uint8, 2 int32) of a named array; -1 if unknown */
long long astg2_count(const astg2_handle* h, const char* name, int* kind);
/* copy a named array to / from host memory; count must equal astg2_count */
astg_status astg2_get(astg2_handle* h, const char* name, void* dst, long long count);
astg_status astg2_set(astg2_handle* h, const char* name, const void* src, long long count);

/* PCG settings (defaults: tol 1e-5 absolute, 5000 iterations, omega 0.97, min diagonal 0.95,
 * ASTG_FP64) */
astg_status astg2_set_solver(astg2_handle* h, double tol, int max_iter, double omega, double min_diag,
                             int precision);
astg_status astg2_last_stats(const astg2_handle* h, astg2_stats* out);

#ifdef __cplusplus
}
#endif

#endif /* ASTG2D_H */
