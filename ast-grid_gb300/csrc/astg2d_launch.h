// Device data of the uniform 2-D AST solver (astg2d.cu) and its kernel launchers.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include <vector>

#include "astg_launch.h"

namespace astg {

// grid constants and the device status word
struct Grid2 {
    int nx, ny;
    double dx, hdx, tiltOctDx, rho;
    int* status;
};

// one time level of the state (reference storage order, x fastest)
struct Fields2 {
    double* dC;     // density on cells, nx * ny
    double* dV;     // density on vertices (tilted cells), (nx + 1) * (ny + 1)
    double* hC;     // heat
    double* hV;
    double* mx;     // x faces, (nx + 1) * ny
    double* my;     // y faces, nx * (ny + 1)
    double* tv;     // 4 tilted-face velocities per vertex
    uint8_t* open;  // tilt layout, one byte per vertex
};

// sphereSource2DSetup
void launch2_source(const Grid2& g, const Fields2& F, cudaStream_t st);
// addForce (buoyancy 0.5 on the upward components) and constrainVelocity
void launch2_force(const Grid2& g, const Fields2& F, double dt, cudaStream_t st);
// updateIndex: vIdx[v] = nx * ny + rank of v among the open tilts, -1 when closed; *nDof
void launch2_numbering(const Grid2& g, const Fields2& F, int* cnt, int* vIdx, int* bsum, int* total, int* nDof,
                       cudaStream_t st);
// the system of project: padded rows, then CSR with b scaled by rho / dt
void launch2_assemble(const Grid2& g, const Dev& d, const Fields2& F, const int* vIdx, Proj& P, double dt,
                      cudaStream_t st);
// correctVelocityByPressure and constrainVelocity
void launch2_correct(const Grid2& g, const Fields2& F, const int* vIdx, const double* p, double dt, cudaStream_t st);
// updateDualGrid (open tilts)
void launch2_dual(const Grid2& g, const Fields2& F, double* dual, cudaStream_t st);
// adjustLayout (when adaptive) and the three semi-Lagrangian advections, cur -> nxt
void launch2_advect(const Grid2& g, const Fields2& cur, const Fields2& nxt, const double* dual, const uint8_t* fixedT,
                    bool adaptive, double dt, cudaStream_t st);
// the wavefront preconditioner's records from the factorised system (Proj::wave fields set);
// whether the wavefront kernel takes grids nx columns wide
void launch2_wave_gather(const Proj& P, const int* vIdx, int rows, cudaStream_t st);
bool wave_supported(int nx, int ny);
// max over cells of mx(x, y)^2 + my(x, y)^2 (ASTSolver::cfl) as the bit pattern of a double
void launch2_cfl(const Grid2& g, const Fields2& F, unsigned long long* out, cudaStream_t st);

}  // namespace astg
