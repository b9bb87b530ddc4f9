// Uniform 2-D AST smoke solver on the GPU: the reference's ASTSolver<2> (include/ast_solver.h), the
// solver behind its Python module's ASTSolver2.  Storage follows the reference's grids (x fastest):
// cells x + y*nx, vertices (tilted cells) x + y*(nx+1), x faces x + y*(nx+1), y faces x + y*nx, four
// tilted-face velocities per vertex.  The reference is configured with CORRECTION_MAC and
// LAYOUT_ADJUST_DENSITY on and EDGE_NODE_ADAPTIVITY off (include/ast_general.h:9-13), so edge nodes
// never open and the degrees of freedom are the cells and the open tilts.
//
// Every floating-point expression keeps the reference's operand order and the library is built
// with FMA contraction off, so each stage reproduces the CPU restatement bit for bit.  One change
// of evaluation, not of arithmetic: ASTFaceGrid<double, 2>::sample's correction term
// (include/ast_face_grid.h:59-63) is an `auto` Eigen expression that refers to a temporary destroyed
// before it is read, so the reference's own build reads a dead stack slot there; this code
// evaluates the difference the expression spells out.
//
// Kernels per sub-step: source, force (+ x walls), numbering (scan of the open tilts), assembly of
// padded rows -> CSR (shared with the octree path), MIC(0) factorisation and PCG (shared; the
// preconditioner is the wavefront kernel below), pressure correction (+ x walls), dual velocities,
// and one fused advection kernel (layout adjustment, density, heat, tilted faces and MAC faces;
// density and heat share each back-trace).
#include <cstdint>
#include <cuda_runtime.h>

#include "astg_launch.h"
#include "astg2d_launch.h"

namespace astg {
namespace g2 {

constexpr double SQRT2 = 1.4142135623730951;   // include/macro.h:16
constexpr double INV_SQRT2 = 1.0 / SQRT2;       // include/macro.h:19 (value of the macro)
constexpr double EPS2 = 2.220446049250313e-16;  // include/general.h:48
constexpr int TB2 = 256;

// include/ast_constant.h:24-26 and include/constants.h:36-39 (the same values)
__constant__ double TILT_OFF[4][2] = {{INV_SQRT2, INV_SQRT2}, {INV_SQRT2, -INV_SQRT2},
                                      {-INV_SQRT2, -INV_SQRT2}, {-INV_SQRT2, INV_SQRT2}};
// include/ast_constant.h:39-44 (mac_direction: 0 x+, 1 x-, 2 y+, 3 y-)
__constant__ int TILT_MAC[4][2] = {{0, 2}, {0, 3}, {1, 3}, {1, 2}};
// include/constants.h:71-77
__constant__ int OCT_NB_TILT[4][2] = {{1, 1}, {1, 0}, {0, 0}, {0, 1}};
__constant__ int TILT_NB_OCT[4][2] = {{0, 0}, {0, -1}, {-1, -1}, {-1, 0}};

struct P2 {
    double x, y;
};

static inline int nblk2(long long n) { return (int)((n + TB2 - 1) / TB2); }
__device__ inline double dmin2(double a, double b) { return (b < a) ? b : a; }  // std::min
__device__ inline double lerp2(double a, double b, double f) { return a * (1 - f) + b * f; }
// include/util.h:172-176
__device__ inline double bilerp2(double v00, double v01, double v11, double v10, double fx, double fy) {
    return lerp2(lerp2(v00, v10, fx), lerp2(v01, v11, fx), fy);
}
// include/util.h:243-256, one component: truncating cast, index clamped to [0, high - 1], fraction
// clamped to [0, 1]
__device__ inline void bary2(double x, int high, int* i, double* f) {
    int c = (int)x;
    c = c < 0 ? 0 : c;
    c = c > high - 1 ? high - 1 : c;
    *i = c;
    double t = x - c;
    t = t < 0.0 ? 0.0 : t;
    *f = t > 1.0 ? 1.0 : t;
}

__device__ inline int ci(const Grid2& g, int x, int y) { return x + y * g.nx; }
__device__ inline int vi(const Grid2& g, int x, int y) { return x + y * (g.nx + 1); }
__device__ inline int mxi(const Grid2& g, int x, int y) { return x + y * (g.nx + 1); }
__device__ inline int myi(const Grid2& g, int x, int y) { return x + y * g.nx; }
// CellCenteredGrid::position, VertexCenteredGrid::position, FaceCenteredGrid::position
__device__ inline P2 cellPos(const Grid2& g, int x, int y) { return P2{(x + 0.5) * g.dx, (y + 0.5) * g.dx}; }
__device__ inline P2 vertPos(const Grid2& g, int x, int y) { return P2{x * g.dx, y * g.dx}; }
__device__ inline P2 macPos(const Grid2& g, int a, int x, int y) {
    return a == 0 ? P2{(x + 0.0) * g.dx, (y + 0.5) * g.dx} : P2{(x + 0.5) * g.dx, (y + 0.0) * g.dx};
}
__device__ inline bool inSphere(P2 p) {
    double ax = p.x - 0.5, ay = p.y - 0.04;  // sphereSource2DSetup: centre (0.5, 0.04), radius 0.03
    return sqrt(ax * ax + ay * ay) < 0.03;
}

// CellCenteredGrid<T, 2>::sample (include/cell_centered_grid.h:40-55)
__device__ inline double cellSample(const Grid2& g, const double* c, P2 pos) {
    int ix, iy;
    double fx, fy;
    bary2(pos.x / g.dx - 0.5, g.nx - 1, &ix, &fx);
    bary2(pos.y / g.dx - 0.5, g.ny - 1, &iy, &fy);
    int x1 = min(ix + 1, g.nx - 1), y1 = min(iy + 1, g.ny - 1);
    return bilerp2(c[ci(g, ix, iy)], c[ci(g, ix, y1)], c[ci(g, x1, y1)], c[ci(g, x1, iy)], fx, fy);
}
// ASTGrid<T, 2>::sample2D (include/ast_grid.h:62-96) with the edge nodes closed
__device__ inline double scalarSample(const Grid2& g, const double* c, const double* v, const uint8_t* open, P2 pos) {
    int cx, cy;
    double fx, fy;
    bary2(pos.x / g.hdx, g.nx * 2, &cx, &fx);
    bary2(pos.y / g.hdx, g.ny * 2, &cy, &fy);
    cx = cx < 1 ? 1 : cx;
    cy = cy < 1 ? 1 : cy;
    int bx = (cx - 1) / 2, by = (cy - 1) / 2;
    int tx = bx + 1, ty = by + 1;
    if (!open[vi(g, tx, ty)]) return cellSample(g, c, pos);
    int ox = min(bx * 2 + 1 - cx, 0), oy = min(by * 2 + 1 - cy, 0);
    fx = fx / 2.0 - 0.5 * (double)ox;
    fy = fy / 2.0 - 0.5 * (double)oy;
    int b1x = min(tx, g.nx - 1), b1y = min(ty, g.ny - 1);
    double v0 = c[ci(g, bx, by)], v1 = c[ci(g, bx, b1y)], v2 = c[ci(g, b1x, b1y)], v3 = c[ci(g, b1x, by)];
    double val = bilerp2(v0, v1, v2, v3, fx, fy);
    double delta = v[vi(g, tx, ty)] - 0.25 * (v0 + v1 + v2 + v3);
    return val + 2 * delta * dmin2(dmin2(fx, fy), dmin2(1 - fx, 1 - fy));
}
// FaceCenteredGrid<Real, 2>::sampleComponent (include/face_centered_grid.h:43-60)
__device__ inline double macAxis(const Grid2& g, const double* mx, const double* my, int a, P2 pos) {
    double rx = pos.x / g.dx, ry = pos.y / g.dx;
    if (a == 0) ry = ry - 0.5;
    else rx = rx - 0.5;
    int lx = g.nx - 1 + (a == 0), ly = g.ny - 1 + (a == 1);
    int ix, iy;
    double fx, fy;
    bary2(rx, lx, &ix, &fx);
    bary2(ry, ly, &iy, &fy);
    int x1 = min(ix + 1, lx), y1 = min(iy + 1, ly);
    if (a == 0)
        return bilerp2(mx[mxi(g, ix, iy)], mx[mxi(g, ix, y1)], mx[mxi(g, x1, y1)], mx[mxi(g, x1, iy)], fx, fy);
    return bilerp2(my[myi(g, ix, iy)], my[myi(g, ix, y1)], my[myi(g, x1, y1)], my[myi(g, x1, iy)], fx, fy);
}
// ASTFaceGrid<Real, 2>::sample with CORRECTION_MAC (include/ast_face_grid.h:52-66), the correction
// term evaluated
__device__ inline P2 velSample(const Grid2& g, const Fields2& F, const double* dual, P2 pos) {
    int ix, iy;
    double fx, fy;
    bary2(pos.x / g.dx - 0.5, g.nx - 1, &ix, &fx);
    bary2(pos.y / g.dx - 0.5, g.ny - 1, &iy, &fy);
    P2 ret{macAxis(g, F.mx, F.my, 0, pos), macAxis(g, F.mx, F.my, 1, pos)};
    int v = vi(g, ix + 1, iy + 1);
    if (!F.open[v]) return ret;
    P2 vp{(ix + 1) * g.dx, (iy + 1) * g.dx};
    double ddx = dual[2 * v] - macAxis(g, F.mx, F.my, 0, vp);
    double ddy = dual[2 * v + 1] - macAxis(g, F.mx, F.my, 1, vp);
    double m = dmin2(dmin2(fx, fy), dmin2(1 - fx, 1 - fy));
    return P2{ret.x + 2 * ddx * m, ret.y + 2 * ddy * m};
}
// backTrace (include/ast_advection.h:11-16)
__device__ inline P2 backTrace(const Grid2& g, const Fields2& F, const double* dual, P2 p, double dt) {
    P2 v = velSample(g, F, dual, p);
    P2 mid{p.x - v.x * dt * 0.5, p.y - v.y * dt * 0.5};
    P2 w = velSample(g, F, dual, mid);
    return P2{p.x - w.x * dt, p.y - w.y * dt};
}

// ------------------------------------------------------------------ source, force
// sphereSource2DSetup (include/ast_solver.h:148-205): density and heat 1 on every cell and vertex
// inside the sphere, the open tilts inside it take (1, -1, 1, -1) / sqrt(2), the y faces 1
__global__ void k2_source(Grid2 g, Fields2 F) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int nc = g.nx * g.ny, nv = (g.nx + 1) * (g.ny + 1), nmy = g.nx * (g.ny + 1);
    if (i < nc && inSphere(cellPos(g, i % g.nx, i / g.nx))) {
        F.dC[i] = 1;
        F.hC[i] = 1;
    }
    if (i < nv && inSphere(vertPos(g, i % (g.nx + 1), i / (g.nx + 1)))) {
        F.dV[i] = 1;
        F.hV[i] = 1;
        if (F.open[i]) {
            F.tv[4 * i + 0] = INV_SQRT2 * 1.0;
            F.tv[4 * i + 1] = -INV_SQRT2 * 1.0;
            F.tv[4 * i + 2] = INV_SQRT2 * 1.0;
            F.tv[4 * i + 3] = -INV_SQRT2 * 1.0;
        }
    }
    if (i < nmy && inSphere(macPos(g, 1, i % g.nx, i / g.nx))) F.my[i] = 1.0;
}
// addForce (include/ast_solver.h:246-281) with constrainVelocity (:609-616): the open tilts take
// beta dt times the heat sampled half a cell out along each tilted normal, projected on the
// upward axis; the y faces take beta dt times the heat at the face; the x walls are closed
__global__ void k2_force(Grid2 g, Fields2 F, double dt) {
    const double beta = 0.5;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int nv = (g.nx + 1) * (g.ny + 1), nmy = g.nx * (g.ny + 1);
    if (i < nv && F.open[i]) {
        P2 pc = vertPos(g, i % (g.nx + 1), i / (g.nx + 1));
        double f[4];
        for (int k = 0; k < 4; ++k) {
            P2 p{pc.x + TILT_OFF[k][0] * g.hdx, pc.y + TILT_OFF[k][1] * g.hdx};
            f[k] = scalarSample(g, F.hC, F.hV, F.open, p) * ((k & 1) ? -INV_SQRT2 : INV_SQRT2);
        }
        for (int k = 0; k < 4; ++k) F.tv[4 * i + k] += f[k] * beta * dt;
    }
    if (i < nmy) F.my[i] += scalarSample(g, F.hC, F.hV, F.open, macPos(g, 1, i % g.nx, i / g.nx)) * beta * dt;
    if (i < g.ny) {
        F.mx[mxi(g, 0, i)] = 0;
        F.mx[mxi(g, g.nx, i)] = 0;
    }
}

// ------------------------------------------------------------------ numbering
// updateIndex (include/ast_solver.h:585-607): cells keep 0 .. nc-1, the open tilts follow in
// vertex order
__global__ void k2_count(Grid2 g, const uint8_t* open, int* cnt) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < (g.nx + 1) * (g.ny + 1)) cnt[i] = open[i] ? 1 : 0;
}
__global__ void k2_assign(Grid2 g, const uint8_t* open, const int* base, const int* total, int* vIdx, int* nDof) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int nc = g.nx * g.ny;
    if (i < (g.nx + 1) * (g.ny + 1)) vIdx[i] = open[i] ? nc + base[i] : -1;
    if (i == 0) *nDof = nc + *total;
}

// ------------------------------------------------------------------ assembly
// project's system (include/ast_solver.h:326-469).  Cell rows: the open tilts at the cell's corners
// (coefficient 1, the tilt's face takes half of each of the two MAC faces it cuts), then the MAC
// faces with what is left of their area (Neumann x walls, Dirichlet top and bottom); the centre and
// the right-hand side accumulate in the reference's order, the entries are written sorted by
// column (cells below, the diagonal, cells above, then the tilts, whose indices follow the cells').
__global__ void k2_asm_cell(Grid2 g, Dev d, Fields2 F, const int* vIdx, Proj P) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    const int nx = g.nx, ny = g.ny;
    if (c >= nx * ny) return;
    const int x = c % nx, y = c / nx;
    bool ok[4], fent[4] = {false, false, false, false};
    int tIdx[4] = {0, 0, 0, 0};
    double tcoef[4] = {0, 0, 0, 0}, fcoef[4] = {0, 0, 0, 0};
    double fa[4] = {0, 0, 0, 0}, center = 0, tb = 0;
    for (int k = 0; k < 4; ++k) {
        const int v = vi(g, x + OCT_NB_TILT[k][0], y + OCT_NB_TILT[k][1]);
        ok[k] = F.open[v] != 0;
        if (!ok[k]) continue;
        for (int i = 0; i < 2; ++i) fa[TILT_MAC[k][i]] -= g.hdx;
        tIdx[k] = vIdx[v];
        if (tIdx[k] < 0) report(d, DS_MISSING_NODE);
        double area = g.hdx * SQRT2 * (1.0 - 0.5 * 0.0);
        double coeff = area / g.tiltOctDx;
        tcoef[k] = -coeff;
        center += coeff;
        int sign = k <= 1 ? -1 : 1;
        tb += sign * area * F.tv[4 * v + (k + 2) % 4];
    }
    for (int k = 0; k < 4; ++k) {
        fa[k] += g.dx;
        if (!(fa[k] > EPS2)) continue;
        const int axis = k / 2;
        int nbx = x, nby = y;
        if (axis == 0) nbx += (k & 1) ? -1 : 1;
        else nby += (k & 1) ? -1 : 1;
        const int fx = x + (axis == 0 && !(k & 1)), fy = y + (axis == 1 && !(k & 1));
        const double u = axis == 0 ? F.mx[mxi(g, fx, fy)] : F.my[myi(g, fx, fy)];
        const bool valid = nbx >= 0 && nby >= 0 && nbx < nx && nby < ny;
        if (valid || axis == 1) {
            double coeff = fa[k] / g.dx;
            if (valid) {
                fent[k] = true;
                fcoef[k] = -coeff;
            }
            center += coeff;
            tb += ((k & 1) ? 1 : -1) * fa[k] * u;
        }
    }
    if (center < EPS2) center = 1;
    const size_t o = (size_t)c * ROW_W;
    int n = 0;
    auto put = [&](int col, double v) {
        P.padCol[o + n] = col;
        P.padVal[o + n] = v;
        ++n;
    };
    if (fent[3]) put(c - nx, fcoef[3]);
    if (fent[1]) put(c - 1, fcoef[1]);
    put(c, center);
    if (fent[0]) put(c + 1, fcoef[0]);
    if (fent[2]) put(c + nx, fcoef[2]);
    const int korder[4] = {2, 1, 3, 0};  // corners (x, y), (x+1, y), (x, y+1), (x+1, y+1)
    for (int j = 0; j < 4; ++j)
        if (ok[korder[j]]) put(tIdx[korder[j]], tcoef[korder[j]]);
    P.rowCnt[c] = n;
    P.bRaw[c] = tb;
}
// tilt rows: the four cells around the vertex, each through a full tilted face
__global__ void k2_asm_tilt(Grid2 g, Dev d, Fields2 F, const int* vIdx, Proj P) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    const int nx = g.nx, ny = g.ny;
    if (v >= (nx + 1) * (ny + 1) || !F.open[v]) return;
    const int x = v % (nx + 1), y = v / (nx + 1);
    const int r = vIdx[v];
    if (r < 0 || x < 1 || y < 1 || x >= nx || y >= ny) {  // boundary tilts are fixed closed
        report(d, DS_MISSING_NODE);
        return;
    }
    double fa[4] = {0, 0, 0, 0}, center = 0, tb = 0, coef[4];
    for (int k = 0; k < 4; ++k) {
        fa[k] += g.hdx * SQRT2;
        double coeff = fa[k] / g.tiltOctDx;
        coef[k] = -coeff;
        center += coeff;
        int sign = k <= 1 ? -1 : 1;
        tb += sign * fa[k] * F.tv[4 * v + k];
    }
    const size_t o = (size_t)r * ROW_W;
    // cells (x-1, y-1), (x, y-1), (x-1, y), (x, y): k = 2, 1, 3, 0; the diagonal last
    const int korder[4] = {2, 1, 3, 0};
    for (int j = 0; j < 4; ++j) {
        int k = korder[j];
        P.padCol[o + j] = ci(g, x + TILT_NB_OCT[k][0], y + TILT_NB_OCT[k][1]);
        P.padVal[o + j] = coef[k];
    }
    P.padCol[o + 4] = r;
    P.padVal[o + 4] = center;
    P.rowCnt[r] = 5;
    P.bRaw[r] = tb;
}
__global__ void k2_zero_rows(Proj P, int rows) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < rows) {
        P.rowCnt[r] = 0;
        P.bRaw[r] = 0;
    }
}

// ------------------------------------------------------------------ pressure correction, dual
// correctVelocityByPressure (include/ast_solver.h:283-324) and constrainVelocity: pressure outside
// the domain is 0 on the y faces; the x walls end closed
__global__ void k2_correct(Grid2 g, Fields2 F, const int* vIdx, const double* p, double dt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int nx = g.nx, ny = g.ny;
    const int nv = (nx + 1) * (ny + 1), nmx = (nx + 1) * ny, nmy = nx * (ny + 1);
    if (i < nv && F.open[i]) {
        const int c = vIdx[i];
        const int x = i % (nx + 1), y = i / (nx + 1);
        if (c >= 0 && x >= 1 && y >= 1 && x < nx && y < ny)
            for (int k = 0; k < 4; ++k) {
                int t = ci(g, x + TILT_NB_OCT[k][0], y + TILT_NB_OCT[k][1]);
                F.tv[4 * i + k] += ((k < 2) ? -1 : 1) * dt / g.rho * (p[t] - p[c]) / g.tiltOctDx;
            }
    }
    if (i < nmx) {
        const int x = i % (nx + 1), y = i / (nx + 1);
        double p1 = x < nx ? p[ci(g, x, y)] : 0.0, p0 = x > 0 ? p[ci(g, x - 1, y)] : 0.0;
        double u = F.mx[i] - dt / g.rho * (p1 - p0) / g.dx;
        F.mx[i] = (x == 0 || x == nx) ? 0.0 : u;
    }
    if (i < nmy) {
        const int x = i % nx, y = i / nx;
        double p1 = y < ny ? p[ci(g, x, y)] : 0.0, p0 = y > 0 ? p[ci(g, x, y - 1)] : 0.0;
        F.my[i] -= dt / g.rho * (p1 - p0) / g.dx;
    }
}
// ASTFaceGrid::updateDualGrid with CORRECTION_MAC (include/ast_face_grid.h:69-150): the velocity
// of an open tilt is half the sum of its opposite faces along the two diagonal directions
__global__ void k2_dual(Grid2 g, const uint8_t* open, const double* tv, double* dual) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= (g.nx + 1) * (g.ny + 1) || !open[v]) return;
    const double* u = tv + 4 * v;
    double s02 = u[0] + u[2], s13 = u[1] + u[3];
    double ux = INV_SQRT2 * s02 + INV_SQRT2 * s13;
    double uy = INV_SQRT2 * s02 + -INV_SQRT2 * s13;
    dual[2 * v] = ux * 0.5;
    dual[2 * v + 1] = uy * 0.5;
}

// ------------------------------------------------------------------ advection
// advect (include/ast_solver.h:533-553) in one pass over cells, vertices, x faces and y faces.
// adjustLayout (:471-531) opens a tilt where the back-traced density lies in (0.005, 0.7) and the
// tilt is not fixed; semiLagrangianAST (include/ast_advection.h:18-29) fills the cells and the
// tilts open in the new layout; semiLagrangianASTVector (:31-68) projects the sampled velocity on
// TILT_UNIT_DIR[k % 2] for the tilted faces and takes the face's own component on the MAC faces.
// All reads come from `cur` (and its layout), all writes go to `nxt`.  The density of a vertex in
// the new layout is the value the layout test sampled (same position, same back-trace).
__global__ void k2_advect(Grid2 g, Fields2 cur, Fields2 nxt, const double* dual, const uint8_t* fixedT, int adaptive,
                          double dt) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int nx = g.nx, ny = g.ny;
    const long long nc = (long long)nx * ny, nv = (long long)(nx + 1) * (ny + 1), nmx = (long long)(nx + 1) * ny,
                    nmy = (long long)nx * (ny + 1);
    if (i < nc) {
        const int x = (int)(i % nx), y = (int)(i / nx);
        P2 old = backTrace(g, cur, dual, cellPos(g, x, y), dt);
        nxt.dC[i] = scalarSample(g, cur.dC, cur.dV, cur.open, old);
        nxt.hC[i] = scalarSample(g, cur.hC, cur.hV, cur.open, old);
        return;
    }
    i -= nc;
    if (i < nv) {
        const int x = (int)(i % (nx + 1)), y = (int)(i / (nx + 1));
        const P2 pc = vertPos(g, x, y);
        P2 old{0, 0};
        double dens = 0;
        bool sampled = false, o;
        if (adaptive) {
            old = backTrace(g, cur, dual, pc, dt);
            dens = scalarSample(g, cur.dC, cur.dV, cur.open, old);
            sampled = true;
            o = dens > 0.005 && dens < 0.7 && !fixedT[i];
            nxt.open[i] = o ? 1 : 0;
        } else {
            o = nxt.open[i] != 0;
        }
        if (!o) return;
        if (!sampled) {
            old = backTrace(g, cur, dual, pc, dt);
            dens = scalarSample(g, cur.dC, cur.dV, cur.open, old);
        }
        nxt.dV[i] = dens;
        nxt.hV[i] = scalarSample(g, cur.hC, cur.hV, cur.open, old);
        for (int k = 0; k < 4; ++k) {
            P2 p{pc.x + TILT_OFF[k][0] * g.hdx, pc.y + TILT_OFF[k][1] * g.hdx};
            P2 s = velSample(g, cur, dual, backTrace(g, cur, dual, p, dt));
            const double* up = TILT_OFF[k % 2];  // TILT_UNIT_DIR[k % 2], the same values
            nxt.tv[4 * i + k] = s.x * up[0] + s.y * up[1];
        }
        return;
    }
    i -= nv;
    if (i < nmx) {
        const int x = (int)(i % (nx + 1)), y = (int)(i / (nx + 1));
        nxt.mx[i] = velSample(g, cur, dual, backTrace(g, cur, dual, macPos(g, 0, x, y), dt)).x;
        return;
    }
    i -= nmx;
    if (i < nmy) {
        const int x = (int)(i % nx), y = (int)(i / nx);
        nxt.my[i] = velSample(g, cur, dual, backTrace(g, cur, dual, macPos(g, 1, x, y), dt)).y;
    }
}

// ASTSolver::cfl (include/ast_solver.h:55-70): the lower x and y faces of every cell
__global__ void k2_cfl(Grid2 g, const double* mx, const double* my, unsigned long long* out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    double v = 0;
    if (c < g.nx * g.ny) {
        const int x = c % g.nx, y = c / g.nx;
        double vx = mx[mxi(g, x, y)], vy = my[myi(g, x, y)];
        v = vx * vx + vy * vy;
    }
    for (int o = 16; o > 0; o >>= 1) {
        double w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w > v ? w : v;
    }
    if ((threadIdx.x & 31) == 0 && v > 0) atomicMax(out, (unsigned long long)__double_as_longlong(v));
}

// ------------------------------------------------------------------ wavefront MIC(0) sweeps
// The system's cells come first in raster order, so a cell's lower neighbours are the cells below
// and to the left (one anti-diagonal earlier) and its upper ones the cells to the right and above
// and its open corner tilts; a tilt row's lower neighbours are its four cells and it has no upper
// ones.  The forward sweep is therefore one anti-diagonal per step (the cells of a diagonal are
// independent), then the tilt rows in one pass; the backward sweep the tilt rows, then the
// diagonals in reverse.  Every row applies its updates in ascending column order with one fused
// multiply-subtract each and multiplies by its pivot reciprocal last -- the generic sweeps'
// arithmetic (and the oracle's in reduce mode 1), so the result is bit-identical.
//
// One CTA, one thread per column (column x = lane x % 32 of warp x / 32), one block barrier per
// diagonal.  A column's own previous result is the neighbour below (forward) or above (backward)
// and stays in a register; the neighbour to the left / right is the adjacent lane's previous
// result (a warp shuffle), across a warp boundary a shared-memory slot per warp and step parity.
// The per-cell records, the residual and the results are stored diagonal-major (cell (x, y) at
// x + (x + y) * nx), so every step's accesses are contiguous across a warp; they are loaded WAVE_PF
// steps ahead.  A second kernel returns the cells' result to the system's order.  Each step's
// critical path is three dependent FP64 operations (~60 cycles each on this GPU) plus a shuffle
// and the barrier.  (A barrier-free form with per-warp progress counters measured 1.5x slower:
// its per-step handshake and fences cost more than the barrier.)
constexpr int WAVE_PF = 4;
constexpr int WAVE_MAX_NX = 512;
constexpr int WAVE_MAX_W = WAVE_MAX_NX / 32;

// records of the factorised system for the wavefront kernel (one thread per row)
__global__ void k2_wave_gather(Proj P, const int* vIdx) {
    const int nx = P.wnx, ny = P.wny, nc = nx * ny;
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= *P.nDof) return;
    const int q0 = P.rowPtr[r], q1 = P.rowPtr[r + 1];
    if (r >= nc) {  // tilt row: its cells (all columns below r), ascending
        const int t = r - nc;
        int k = 0;
        for (int q = q0; q < q1 && k < 4; ++q) {
            int col = P.col[q];
            if (col >= r) break;
            P.wTc[4 * t + k] = col;
            P.wTv[4 * t + k] = P.Lv[P.tpos[q]];
            ++k;
        }
        for (; k < 4; ++k) {  // an interior tilt always has four cells
            P.wTc[4 * t + k] = -1;
            P.wTv[4 * t + k] = 0;
        }
        return;
    }
    const int x = r % nx, y = r / nx, j = x + (x + y) * nx;  // diagonal-major slot
    const int corner[4] = {vIdx[x + y * (nx + 1)], vIdx[x + 1 + y * (nx + 1)], vIdx[x + (y + 1) * (nx + 1)],
                           vIdx[x + 1 + (y + 1) * (nx + 1)]};
    double lb = 0, ll = 0, lr = 0, la = 0;
    unsigned f = 0;
    for (int k = 0; k < 4; ++k) {
        P.wTt[4 * j + k] = -1;
        P.wTl[4 * j + k] = 0;
    }
    for (int q = q0; q < q1; ++q) {
        const int col = P.col[q];
        if (col == r - nx) { lb = P.Lv[P.tpos[q]]; f |= 1; }
        else if (col == r - 1) { ll = P.Lv[P.tpos[q]]; f |= 2; }
        else if (col == r + 1) { lr = P.Lv[q]; f |= 4; }
        else if (col == r + nx) { la = P.Lv[q]; f |= 8; }
        else if (col >= nc) {
            for (int k = 0; k < 4; ++k)
                if (corner[k] == col) {
                    P.wTt[4 * j + k] = col;
                    P.wTl[4 * j + k] = P.Lv[q];
                    f |= 16u << k;
                }
        }
    }
    const double inv = P.invdiag[r], fb = __longlong_as_double((long long)f);
    P.wRecF[2 * j] = make_double2(lb, ll);
    P.wRecF[2 * j + 1] = make_double2(inv, fb);
    P.wRecB[2 * j] = make_double2(lr, la);
    P.wRecB[2 * j + 1] = make_double2(inv, fb);
}

constexpr unsigned WAVE_NONE = 0x80000000u;  // no cell in this column on this diagonal
struct WStep {
    double v, l0, l1, inv;
    unsigned f;
};
// one slot's record; WAVE_NONE when the column has no cell on the diagonal (then nothing is
// computed: a warp with no cell on a diagonal issues no FP64 work there)
__device__ __forceinline__ void wload(const double2* rec, const double* val, int j, bool on, WStep& s) {
    if (!on) {
        s.f = WAVE_NONE;
        return;
    }
    const double2 a = rec[2 * j], b = rec[2 * j + 1];
    s.v = val[j];
    s.l0 = a.x;
    s.l1 = a.y;
    s.inv = b.x;
    s.f = (unsigned)__double_as_longlong(b.y);
}

// the cells' result from diagonal-major order to the system's
__global__ void k2_wave_unskew(Proj P, double* z) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int nx = P.wnx;
    if (*P.done || i >= nx * P.wny) return;
    const int x = i % nx;
    z[i] = P.wZ[x + (x + i / nx) * nx];
}

__global__ void __launch_bounds__(WAVE_MAX_NX) k2_precond_wave(Proj P, const double* r, double* z) {
    __shared__ double edge[2][WAVE_MAX_W];  // per step parity: each warp's boundary value
    if (*P.done) return;
    const int nx = P.wnx, ny = P.wny, nc = nx * ny, n = *P.nDof;
    const int D = nx + ny - 1;
    const int x = threadIdx.x, lane = x & 31, w = x >> 5, W = blockDim.x >> 5;
    const bool mine = x < nx;  // lanes past the last column only take part in the exchanges
    const unsigned FULL = 0xffffffffu;
    WStep A[WAVE_PF], B[WAVE_PF];

    // ---- forward over the cells: step d visits slot x + d * nx, the cell (x, d - x).  The update
    // from the cell below (this column's previous result) is applied before the barrier that ends
    // the previous step; the one from the left needs the neighbouring column's previous result
    // (shuffle, or the boundary slot of the warp to the left for lane 0).
    double zb = 0;  // this column's last result
    double t = 0;   // the current slot's accumulator after the update from below
    auto fload = [&](WStep* S, int d0) {
#pragma unroll
        for (int s = 0; s < WAVE_PF; ++s) {
            const int d = d0 + s, y = d - x;
            wload(P.wRecF, P.wR, x + d * nx, mine && y >= 0 && y < ny, S[s]);
        }
    };
    auto below = [&](const WStep& c) {  // (x, y - 1)
        return (!(c.f & WAVE_NONE) && (c.f & 1)) ? fma(-c.l0, zb, c.v) : c.v;
    };
    auto fstep = [&](const WStep& c, const WStep& nxt, int d) {
        const int cur = d & 1, prv = cur ^ 1;
        double zl = __shfl_up_sync(FULL, zb, 1);
        const double ze = edge[prv][w > 0 ? w - 1 : 0];
        if (lane == 0) zl = ze;
        if (!(c.f & WAVE_NONE)) {
            double acc = (c.f & 2) ? fma(-c.l1, zl, t) : t;  // (x - 1, y)
            acc = acc * c.inv;
            P.wZ[x + d * nx] = acc;
            zb = acc;
        }
        if (lane == 31) edge[cur][w] = zb;
        t = below(nxt);
        __syncthreads();
    };
    fload(A, 0);
    t = below(A[0]);
    for (int g = 0; g < D; g += 2 * WAVE_PF) {
        fload(B, g + WAVE_PF);
#pragma unroll
        for (int s = 0; s < WAVE_PF; ++s)
            if (g + s < D) fstep(A[s], s + 1 < WAVE_PF ? A[s + 1] : B[0], g + s);
        fload(A, g + 2 * WAVE_PF);
#pragma unroll
        for (int s = 0; s < WAVE_PF; ++s)
            if (g + WAVE_PF + s < D) fstep(B[s], s + 1 < WAVE_PF ? B[s + 1] : A[0], g + WAVE_PF + s);
    }

    // ---- tilt rows: forward (their four cells), then their backward step (no upper entries)
    for (int tr = nc + x; tr < n; tr += blockDim.x) {
        const int i = tr - nc;
        double acc = r[tr];
        for (int k = 0; k < 4; ++k) {
            const int c = P.wTc[4 * i + k];
            if (c >= 0) acc = fma(-P.wTv[4 * i + k], P.wZ[c % nx + (c % nx + c / nx) * nx], acc);
        }
        const double inv = P.invdiag[tr];
        acc = acc * inv;
        z[tr] = acc * inv;
    }
    __syncthreads();

    // ---- backward over the cells: step s visits diagonal D - 1 - s; the update from the right
    // (neighbouring column, shuffle or boundary slot) comes first, then the one from above (this
    // column's previous result), then the corner tilts
    double za = 0;
    auto bload = [&](WStep* S, int s0) {
#pragma unroll
        for (int s = 0; s < WAVE_PF; ++s) {
            const int d = D - 1 - (s0 + s), y = d - x;
            wload(P.wRecB, P.wZ, x + d * nx, mine && y >= 0 && y < ny, S[s]);
        }
    };
    auto bstep = [&](const WStep& c, int st) {
        const int cur = st & 1, prv = cur ^ 1;
        double zr = __shfl_down_sync(FULL, za, 1);
        const double ze = edge[prv][w + 1 < W ? w + 1 : w];
        if (lane == 31) zr = ze;
        if (!(c.f & WAVE_NONE)) {
            double acc = c.v;
            if (c.f & 4) acc = fma(-c.l0, zr, acc);  // (x + 1, y)
            if (c.f & 8) acc = fma(-c.l1, za, acc);  // (x, y + 1)
            const int j = x + (D - 1 - st) * nx;
            if (c.f & 0xf0u) {
#pragma unroll
                for (int k = 0; k < 4; ++k)
                    if (c.f & (16u << k)) acc = fma(-P.wTl[4 * j + k], z[P.wTt[4 * j + k]], acc);
            }
            acc = acc * c.inv;
            P.wZ[j] = acc;  // in place: this slot's forward value was loaded steps ago
            za = acc;
        }
        if (lane == 0) edge[cur][w] = za;
        __syncthreads();
    };
    bload(A, 0);
    for (int g = 0; g < D; g += 2 * WAVE_PF) {
        bload(B, g + WAVE_PF);
#pragma unroll
        for (int s = 0; s < WAVE_PF; ++s)
            if (g + s < D) bstep(A[s], g + s);
        bload(A, g + 2 * WAVE_PF);
#pragma unroll
        for (int s = 0; s < WAVE_PF; ++s)
            if (g + WAVE_PF + s < D) bstep(B[s], g + WAVE_PF + s);
    }
}

}  // namespace g2

using namespace g2;
void launch2_source(const Grid2& g, const Fields2& F, cudaStream_t st) {
    long long n = (long long)(g.nx + 1) * (g.ny + 1);
    ASTG_LAUNCH(k2_source<<<nblk2(n), TB2, 0, st>>>(g, F));
}
void launch2_force(const Grid2& g, const Fields2& F, double dt, cudaStream_t st) {
    long long n = (long long)(g.nx + 1) * (g.ny + 1);
    ASTG_LAUNCH(k2_force<<<nblk2(n), TB2, 0, st>>>(g, F, dt));
}
void launch2_numbering(const Grid2& g, const Fields2& F, int* cnt, int* vIdx, int* bsum, int* total, int* nDof,
                       cudaStream_t st) {
    long long nv = (long long)(g.nx + 1) * (g.ny + 1);
    ASTG_LAUNCH(k2_count<<<nblk2(nv), TB2, 0, st>>>(g, F.open, cnt));
    launch_exclusive_scan(cnt, vIdx, bsum, total, nv, st);
    // vIdx holds the scan; k2_assign reads it through `base` before overwriting the same entry
    ASTG_LAUNCH(k2_assign<<<nblk2(nv), TB2, 0, st>>>(g, F.open, vIdx, total, vIdx, nDof));
}
void launch2_assemble(const Grid2& g, const Dev& d, const Fields2& F, const int* vIdx, Proj& P, double dt,
                      cudaStream_t st) {
    const long long nc = (long long)g.nx * g.ny, nv = (long long)(g.nx + 1) * (g.ny + 1);
    const int rows = (int)(nc + nv);
    ASTG_LAUNCH(k2_zero_rows<<<nblk2(rows), TB2, 0, st>>>(P, rows));
    ASTG_LAUNCH(k2_asm_cell<<<nblk2(nc), TB2, 0, st>>>(g, d, F, vIdx, P));
    ASTG_LAUNCH(k2_asm_tilt<<<nblk2(nv), TB2, 0, st>>>(g, d, F, vIdx, P));
    launch_rows_to_csr(d, P, rows, g.rho / dt, st);
}
void launch2_correct(const Grid2& g, const Fields2& F, const int* vIdx, const double* p, double dt, cudaStream_t st) {
    const long long n = (long long)(g.nx + 1) * (g.ny + 1);
    ASTG_LAUNCH(k2_correct<<<nblk2(n), TB2, 0, st>>>(g, F, vIdx, p, dt));
}
void launch2_dual(const Grid2& g, const Fields2& F, double* dual, cudaStream_t st) {
    const long long n = (long long)(g.nx + 1) * (g.ny + 1);
    ASTG_LAUNCH(k2_dual<<<nblk2(n), TB2, 0, st>>>(g, F.open, F.tv, dual));
}
void launch2_advect(const Grid2& g, const Fields2& cur, const Fields2& nxt, const double* dual, const uint8_t* fixedT,
                    bool adaptive, double dt, cudaStream_t st) {
    const long long n = (long long)g.nx * g.ny + (long long)(g.nx + 1) * (g.ny + 1) + (long long)(g.nx + 1) * g.ny +
                        (long long)g.nx * (g.ny + 1);
    ASTG_LAUNCH(k2_advect<<<nblk2(n), TB2, 0, st>>>(g, cur, nxt, dual, fixedT, adaptive ? 1 : 0, dt));
}
void launch2_cfl(const Grid2& g, const Fields2& F, unsigned long long* out, cudaStream_t st) {
    cudaMemsetAsync(out, 0, sizeof(unsigned long long), st);
    ASTG_LAUNCH(k2_cfl<<<nblk2((long long)g.nx * g.ny), TB2, 0, st>>>(g, F.mx, F.my, out));
}

void launch2_wave_gather(const Proj& P, const int* vIdx, int rows, cudaStream_t st) {
    ASTG_LAUNCH(k2_wave_gather<<<nblk2(rows), TB2, 0, st>>>(P, vIdx));
}
void launch_precond_wave(const Proj& P, const double* r, double* z, cudaStream_t st) {
    const int threads = (P.wnx + 31) / 32 * 32;
    ASTG_LAUNCH(k2_precond_wave<<<1, threads, 0, st>>>(P, r, z));
    ASTG_LAUNCH(k2_wave_unskew<<<nblk2((long long)P.wnx * P.wny), TB2, 0, st>>>(P, z));
}
// the wavefront kernel takes up to WAVE_MAX_NX columns; its diagonal-major slots use 32-bit indices
bool wave_supported(int nx, int ny) {
    return nx >= 2 && nx <= WAVE_MAX_NX && (long long)nx * (nx + ny - 1) * 4 < (1LL << 31);
}

}  // namespace astg
