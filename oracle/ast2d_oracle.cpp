// CPU restatement of the reference's uniform 2-D AST smoke solver, ASTSolver<2>
// (include/ast_solver.h), the solver behind the reference's pybind ASTSolver2 (test
// infrastructure only: the tests and the smoke check use it as the checker of the GPU
// library's 2-D solver; nothing in the product loads it).
//
// The reference is configured by include/ast_general.h: CORRECTION_MAC on, LAYOUT_ADJUST_DENSITY
// on, EDGE_NODE_ADAPTIVITY off -- so the 2-D edge nodes never open and every edge-node branch of
// the solver is dead; the degrees of freedom are the cells and the open tilted cells at the
// vertices.  Storage order follows the reference's grids (x fastest): cells x + y*nx, vertices
// x + y*(nx+1), x faces x + y*(nx+1), y faces x + y*nx, four tilted-face velocities per vertex.
//
// Two reduction modes, as in oracle/smoke_oracle.cpp: 0 = the reference's own order (the PCG's
// dot products summed in the per-worker slices of ThreadPool::parallelForTFWithCoreID, then the
// slice sums in order, include/pcgsolver/blas_wrapper.h:17-38 with USE_TASKFLOW), 1 = the CUDA
// library's (its fixed reduction tree, and one fused multiply-add for every product it accumulates:
// MIC(0) sweep updates, CSR rows, dot-product lanes and the PCG's vector updates).
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

namespace ast2o {

static const double SQRT2 = 1.4142135623730951;  // include/macro.h:16
static const double INV_SQRT2 = 1.0 / SQRT2;       // include/macro.h:19
static const double EPS = DBL_EPSILON;            // include/general.h:48

// include/ast_constant.h, include/constants.h
static const double TILT_POS_OFFSET[4][2] = {{INV_SQRT2, INV_SQRT2}, {INV_SQRT2, -INV_SQRT2},
                                             {-INV_SQRT2, -INV_SQRT2}, {-INV_SQRT2, INV_SQRT2}};
static const double TILT_UNIT_DIR[4][2] = {{INV_SQRT2, INV_SQRT2}, {INV_SQRT2, -INV_SQRT2},
                                           {-INV_SQRT2, -INV_SQRT2}, {-INV_SQRT2, INV_SQRT2}};
static const int TILT_DIRECTION_NEIGHBOR_MAC2[4][2] = {{0, 2}, {0, 3}, {1, 3}, {1, 2}};
static const int OCT_NB_TILT_DXDY[4][2] = {{1, 1}, {1, 0}, {0, 0}, {0, 1}};
static const int TILT_NB_OCT_DXDY[4][2] = {{0, 0}, {0, -1}, {-1, -1}, {-1, 0}};

struct P2 {
    double x, y;
};

// include/util.h:165-176
static double lerp(double a, double b, double f) { return a * (1 - f) + b * f; }
static double bilerp(double v00, double v01, double v11, double v10, double fx, double fy) {
    return lerp(lerp(v00, v10, fx), lerp(v01, v11, fx), fy);
}
// include/util.h:243-256 (one component): truncating cast, clamped index, clamped fraction
static void bary(double x, int high, int* i, double* f) {
    int c = (int)x;
    c = std::max(c, 0);
    c = std::min(c, high - 1);
    *i = c;
    double t = x - c;
    *f = std::min(std::max(t, 0.0), 1.0);
}

// fixed reduction tree of the CUDA library
static const int RED_LANES = 256, RED_PER_LANE = 8, RED_CHUNK = RED_LANES * RED_PER_LANE;
template <class F>
static double treeReduce(size_t n, const F& step) {
    size_t chunks = (n + RED_CHUNK - 1) / RED_CHUNK;
    std::vector<double> part(chunks);
    std::vector<double> lane(RED_LANES);
    auto fold = [&]() {
        for (int st = RED_LANES / 2; st >= 1; st >>= 1)
            for (int t = 0; t < st; ++t) lane[t] = lane[t] + lane[t + st];
        return lane[0];
    };
    for (size_t c = 0; c < chunks; ++c) {
        for (int t = 0; t < RED_LANES; ++t) {
            double acc = 0.0;
            for (int k = 0; k < RED_PER_LANE; ++k) {
                size_t i = c * RED_CHUNK + t + (size_t)RED_LANES * k;
                if (i < n) acc = step(acc, i);
            }
            lane[t] = acc;
        }
        part[c] = fold();
    }
    while (part.size() > 1) {
        size_t m = part.size(), next = (m + RED_CHUNK - 1) / RED_CHUNK;
        std::vector<double> np(next);
        for (size_t c = 0; c < next; ++c) {
            for (int t = 0; t < RED_LANES; ++t) {
                double acc = 0.0;
                for (int k = 0; k < RED_PER_LANE; ++k) {
                    size_t i = c * RED_CHUNK + t + (size_t)RED_LANES * k;
                    if (i < m) acc = acc + part[i];
                }
                lane[t] = acc;
            }
            np[c] = fold();
        }
        part.swap(np);
    }
    return part.empty() ? 0.0 : part[0];
}
// BLAS::dot with USE_TASKFLOW (include/pcgsolver/blas_wrapper.h:17-38) over
// ThreadPool::parallelForTFWithCoreID's slices (include/thread_pool.h:391-425)
static double workerDot(const std::vector<double>& x, const std::vector<double>& y, int workers) {
    std::vector<double> sums(workers + 1, 0.0);
    long long start = 0, end = (long long)x.size();
    long long n = end - start + 1;
    long long slice = (long long)std::round(n / (double)workers);
    slice = std::max(slice, 1LL);
    long long i1 = start, i2 = std::min(start + slice, end);
    int i = 0;
    for (; i + 1 < workers && i1 < end; i++) {
        for (long long k = i1; k < i2; ++k) sums[i] += x[k] * y[k];
        i1 = i2;
        i2 = std::min(i2 + slice, end);
    }
    if (i1 < end)
        for (long long k = i1; k < end; ++k) sums[i] += x[k] * y[k];
    double acc = 0.0;
    for (double s : sums) acc = acc + s;
    return acc;
}

// PCG::SparseMatrix (include/pcgsolver/sparse_matrix.h:14-103): rows of sorted columns
struct RowMatrix {
    int n = 0;
    std::vector<std::vector<int>> idx;
    std::vector<std::vector<double>> val;
    void reset(int n_) {
        n = n_;
        idx.assign(n, {});
        val.assign(n, {});
    }
    void set(int i, int j, double v) {
        auto& I = idx[i];
        auto& V = val[i];
        size_t k = 0;
        for (; k < I.size(); ++k) {
            if (I[k] == j) { V[k] = v; return; }
            if (I[k] > j) { I.insert(I.begin() + k, j); V.insert(V.begin() + k, v); return; }
        }
        I.push_back(j);
        V.push_back(v);
    }
};

// PCGSolver::solve for std::vector (include/pcgsolver/pcg_solver.h:302-362): x = 0, r = b, stop
// when |r|_inf <= tolerance_factor (absolute), MIC(0) preconditioner (:89-190, 197-237)
struct Pcg {
    double tol = 1e-5, omega = 0.97, minDiag = 0.95;
    int maxIter = 5000, reduceMode = 0, workers = 8;
    int iters = 0;
    bool ok = true;
    struct Factor {
        int n = 0;
        std::vector<double> invdiag, value, adiag;
        std::vector<int> rowindex, colstart;
    } F;
    void factor(const RowMatrix& A) {
        int n = A.n;
        F.n = n;
        F.invdiag.assign(n, 0);
        F.adiag.assign(n, 0);
        F.value.clear();
        F.rowindex.clear();
        F.colstart.assign(n + 1, 0);
        for (int i = 0; i < n; ++i) {
            F.colstart[i] = F.rowindex.size();
            for (size_t j = 0; j < A.idx[i].size(); ++j) {
                if (A.idx[i][j] > i) { F.rowindex.push_back(A.idx[i][j]); F.value.push_back(A.val[i][j]); }
                else if (A.idx[i][j] == i) F.invdiag[i] = F.adiag[i] = A.val[i][j];
            }
        }
        F.colstart[n] = F.rowindex.size();
        for (int k = 0; k < n; ++k) {
            if (F.adiag[k] == 0) continue;
            if (F.invdiag[k] < minDiag * F.adiag[k]) F.invdiag[k] = 1 / std::sqrt(F.adiag[k]);
            else F.invdiag[k] = 1 / std::sqrt(F.invdiag[k]);
            for (int q = F.colstart[k]; q < F.colstart[k + 1]; ++q) F.value[q] *= F.invdiag[k];
            for (int q = F.colstart[k]; q < F.colstart[k + 1]; ++q) {
                int j = F.rowindex[q];
                double mult = F.value[q];
                double missing = 0;
                int a = F.colstart[k];
                size_t bq = 0;
                while (a < F.colstart[k + 1] && F.rowindex[a] < j) {
                    while (bq < A.idx[j].size()) {
                        if (A.idx[j][bq] < F.rowindex[a]) ++bq;
                        else if (A.idx[j][bq] == F.rowindex[a]) break;
                        else { missing += F.value[a]; break; }
                    }
                    ++a;
                }
                if (a < F.colstart[k + 1] && F.rowindex[a] == j) F.invdiag[j] -= mult * F.value[a];
                ++a;
                int bb = F.colstart[j];
                while (a < F.colstart[k + 1] && bb < F.colstart[j + 1]) {
                    if (F.rowindex[bb] < F.rowindex[a]) ++bb;
                    else if (F.rowindex[bb] == F.rowindex[a]) { F.value[bb] -= mult * F.value[a]; ++a; ++bb; }
                    else { missing += F.value[a]; ++a; }
                }
                while (a < F.colstart[k + 1]) { missing += F.value[a]; ++a; }
                F.invdiag[j] -= omega * mult * missing;
            }
        }
    }
    void precond(const std::vector<double>& r, std::vector<double>& z) const {
        z = r;
        const bool fused = reduceMode != 0;
        for (int i = 0; i < F.n; ++i) {
            z[i] *= F.invdiag[i];
            for (int j = F.colstart[i]; j < F.colstart[i + 1]; ++j) {
                double& t = z[F.rowindex[j]];
                t = fused ? std::fma(-F.value[j], z[i], t) : t - F.value[j] * z[i];
            }
        }
        for (int i = F.n - 1; i >= 0; --i) {
            for (int j = F.colstart[i]; j < F.colstart[i + 1]; ++j)
                z[i] = fused ? std::fma(-F.value[j], z[F.rowindex[j]], z[i]) : z[i] - F.value[j] * z[F.rowindex[j]];
            z[i] *= F.invdiag[i];
        }
    }
    // acc + a * b: one fused multiply-add in the library's order, a product then an addition in the
    // reference's (r -= alpha z is r + (-alpha) z there, the same number)
    double fmadd(double acc, double a, double b) const {
        if (reduceMode != 0) return std::fma(a, b, acc);
        double prod = a * b;
        return acc + prod;
    }
    double dot(const std::vector<double>& a, const std::vector<double>& b) const {
        if (reduceMode == 0) return workerDot(a, b, workers);
        return treeReduce(a.size(), [&](double acc, size_t i) { return std::fma(a[i], b[i], acc); });
    }
    static double absmax(const std::vector<double>& a) {
        double m = 0;
        for (double v : a) m = std::max(m, std::fabs(v));
        return m;
    }
    void solve(const RowMatrix& A, const std::vector<double>& b, std::vector<double>& x) {
        int n = A.n;
        x.assign(n, 0.0);
        std::vector<double> r = b, z(n), s(n);
        double resid = absmax(r);
        iters = 0;
        ok = true;
        if (resid == 0) return;
        factor(A);
        precond(r, z);
        double rho = dot(z, r);
        if (rho == 0 || rho != rho) { ok = false; return; }
        s = z;
        int it;
        for (it = 0; it < maxIter; ++it) {
            for (int i = 0; i < n; ++i) {
                double t = 0;
                for (size_t j = 0; j < A.idx[i].size(); ++j) t = fmadd(t, A.val[i][j], s[A.idx[i][j]]);
                z[i] = t;
            }
            double alpha = rho / dot(s, z);
            for (int i = 0; i < n; ++i) {
                x[i] = fmadd(x[i], alpha, s[i]);
                r[i] = fmadd(r[i], -alpha, z[i]);
            }
            resid = absmax(r);
            if (resid <= tol) { iters = it + 1; return; }
            precond(r, z);
            double rn = dot(z, r);
            double beta = rn / rho;
            for (int i = 0; i < n; ++i) z[i] = fmadd(z[i], beta, s[i]);
            s.swap(z);
            rho = rn;
        }
        iters = it;
        ok = false;
    }
};

}  // namespace ast2o

namespace ast2o {

// ASTSolver<2> (include/ast_solver.h): state, samplers and stages
class Solver2 {
public:
    int nx, ny;
    double dx, hdx, qdx, tiltOctDx;
    bool adaptive;
    double rho = 2.0;
    int maxCfl = 2;
    Pcg pcg;
    // fields (reference storage order)
    std::vector<double> dC, dV, hC, hV;  // density / heat at cells and vertices
    std::vector<double> mx, my;          // MAC faces
    std::vector<double> tv;              // 4 tilted-face velocities per vertex
    std::vector<double> dual;            // dual velocity at vertices (x, y)
    std::vector<uint8_t> open, openTmp, fixedT;  // tilt layout, its double buffer, fixed nodes
    std::vector<uint8_t> cellTilt;       // per cell: status of its 4 tilts (bit k), from the layout
    std::vector<int> pIdx;               // cells then vertices
    int nIndex = 0;
    RowMatrix A;
    std::vector<double> b, p;
    int substeps = 0;
    std::vector<double> subDt;

    Solver2(int nx_, int ny_, double dx_, bool adaptive_) : nx(nx_), ny(ny_), dx(dx_), adaptive(adaptive_) {
        hdx = dx / 2.0;
        qdx = dx / 4.0;
        tiltOctDx = hdx * SQRT2;
        int nc = nx * ny, nv = (nx + 1) * (ny + 1);
        dC.assign(nc, 0); hC.assign(nc, 0);
        dV.assign(nv, 0); hV.assign(nv, 0);
        mx.assign((size_t)(nx + 1) * ny, 0);
        my.assign((size_t)nx * (ny + 1), 0);
        tv.assign((size_t)nv * 4, 0);
        dual.assign((size_t)nv * 2, 0);
        open.assign(nv, 0); openTmp.assign(nv, 0); fixedT.assign(nv, 0);
        cellTilt.assign(nc, 0);
        pIdx.assign(nc + nv, -1);
        pcg.tol = 1e-5;  // SOLVER_ACCURACY (include/macro.h:21), set in initialize()
        pcg.maxIter = 5000;
        pcg.omega = 0.97;
        pcg.minDiag = 0.95;
    }
    int ci(int x, int y) const { return x + y * nx; }
    int vi(int x, int y) const { return x + y * (nx + 1); }
    int mxi(int x, int y) const { return x + y * (nx + 1); }
    int myi(int x, int y) const { return x + y * nx; }
    bool cellValid(int x, int y) const { return x >= 0 && y >= 0 && x < nx && y < ny; }

    // initialize() / initData() (:36-98): boundary tilts fixed closed, cells numbered once
    void initialize() {
        for (int y = 0; y <= ny; ++y)
            for (int x = 0; x <= nx; ++x)
                if (x == 0 || y == 0 || x == nx || y == ny) fixedT[vi(x, y)] = 1;
        int c = 0;
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) pIdx[ci(x, y)] = c++;
        nIndex = c;
    }

    // ---- samplers
    // CellCenteredGrid<T, 2>::sample (include/cell_centered_grid.h:40-55)
    double cellSample(const std::vector<double>& c, P2 pos) const {
        int ix, iy;
        double fx, fy;
        bary(pos.x / dx - 0.5, nx - 1, &ix, &fx);
        bary(pos.y / dx - 0.5, ny - 1, &iy, &fy);
        int x1 = std::min(ix + 1, nx - 1), y1 = std::min(iy + 1, ny - 1);
        return bilerp(c[ci(ix, iy)], c[ci(ix, y1)], c[ci(x1, y1)], c[ci(x1, iy)], fx, fy);
    }
    // ASTGrid<T, 2>::sample2D (include/ast_grid.h:62-96), edge nodes never open
    double scalarSample(const std::vector<double>& c, const std::vector<double>& v, const std::vector<uint8_t>& lay,
                        P2 pos) const {
        int cx, cy;
        double fx, fy;
        bary(pos.x / hdx, nx * 2, &cx, &fx);
        bary(pos.y / hdx, ny * 2, &cy, &fy);
        cx = std::max(cx, 1);
        cy = std::max(cy, 1);
        int bx = (cx - 1) / 2, by = (cy - 1) / 2;
        int tx = bx + 1, ty = by + 1;
        if (!lay[vi(tx, ty)]) return cellSample(c, pos);
        int ox = std::min(bx * 2 + 1 - cx, 0), oy = std::min(by * 2 + 1 - cy, 0);
        fx = fx / 2.0 - 0.5 * (double)ox;
        fy = fy / 2.0 - 0.5 * (double)oy;
        int b1x = std::min(tx, nx - 1), b1y = std::min(ty, ny - 1);
        double v0 = c[ci(bx, by)], v1 = c[ci(bx, b1y)], v2 = c[ci(b1x, b1y)], v3 = c[ci(b1x, by)];
        double val = bilerp(v0, v1, v2, v3, fx, fy);
        double delta = v[vi(tx, ty)] - 0.25 * (v0 + v1 + v2 + v3);
        return val + 2 * delta * std::min(std::min(fx, fy), std::min(1 - fx, 1 - fy));
    }
    // FaceCenteredGrid<Real, 2>::sampleComponent (include/face_centered_grid.h:43-60)
    double macAxis(int a, P2 pos) const {
        double rx = pos.x / dx, ry = pos.y / dx;
        if (a == 0) ry = ry - 0.5; else rx = rx - 0.5;
        int lx = nx - 1 + (a == 0), ly = ny - 1 + (a == 1);
        int ix, iy;
        double fx, fy;
        bary(rx, lx, &ix, &fx);
        bary(ry, ly, &iy, &fy);
        int x1 = std::min(ix + 1, lx), y1 = std::min(iy + 1, ly);
        auto g = [&](int x, int y) { return a == 0 ? mx[mxi(x, y)] : my[myi(x, y)]; };
        return bilerp(g(ix, iy), g(ix, y1), g(x1, y1), g(x1, iy), fx, fy);
    }
    P2 macSample(P2 pos) const { return P2{macAxis(0, pos), macAxis(1, pos)}; }
    // ASTFaceGrid::sample with CORRECTION_MAC (include/ast_face_grid.h:52-66)
    P2 velSample(P2 pos) const {
        int ix, iy;
        double fx, fy;
        bary(pos.x / dx - 0.5, nx - 1, &ix, &fx);
        bary(pos.y / dx - 0.5, ny - 1, &iy, &fy);
        P2 ret = macSample(pos);
        int v = vi(ix + 1, iy + 1);
        if (!open[v]) return ret;
        P2 vm = macSample(P2{(ix + 1) * dx, (iy + 1) * dx});
        double ddx = dual[2 * v] - vm.x, ddy = dual[2 * v + 1] - vm.y;
        double m = std::min(std::min(fx, fy), std::min(1 - fx, 1 - fy));
        return P2{ret.x + 2 * ddx * m, ret.y + 2 * ddy * m};
    }
    // backTrace (include/ast_advection.h:11-16)
    P2 backTrace(P2 p, double dt) const {
        P2 v = velSample(p);
        P2 mid{p.x - v.x * dt * 0.5, p.y - v.y * dt * 0.5};
        P2 w = velSample(mid);
        return P2{p.x - w.x * dt, p.y - w.y * dt};
    }
    P2 cellPos(int x, int y) const { return P2{(x + 0.5) * dx, (y + 0.5) * dx}; }
    P2 vertPos(int x, int y) const { return P2{x * dx, y * dx}; }
    P2 macPos(int a, int x, int y) const {
        return a == 0 ? P2{(x + 0.0) * dx, (y + 0.5) * dx} : P2{(x + 0.5) * dx, (y + 0.0) * dx};
    }
    static bool inSphere(P2 p, double cx, double cy, double r) {
        double ax = p.x - cx, ay = p.y - cy;
        return std::sqrt(ax * ax + ay * ay) < r;
    }

    // ---- layout
    // ASTGridLayout::propogateNodeInfo (include/ast_grid_layout.h:166-190), cell half: bit k is
    // the open state of the tilt at cell + OCT_NB_TILT_DXDY[k]
    void propagate() {
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) {
                uint8_t bits = 0;
                for (int k = 0; k < 4; ++k)
                    if (open[vi(x + OCT_NB_TILT_DXDY[k][0], y + OCT_NB_TILT_DXDY[k][1])]) bits |= (uint8_t)(1 << k);
                cellTilt[ci(x, y)] = bits;
            }
    }
    // updateIndex (include/ast_solver.h:585-607): cells keep 0..nc-1, open tilts follow in
    // vertex order, closed tilts get -1
    void updateIndex() {
        int c = nx * ny;
        for (int y = 0; y <= ny; ++y)
            for (int x = 0; x <= nx; ++x) pIdx[nx * ny + vi(x, y)] = open[vi(x, y)] ? c++ : -1;
        nIndex = c;
    }

    // ---- stages
    // sphereSource2DSetup (include/ast_solver.h:148-205)
    void source() {
        const double scx = 0.5, scy = 0.04, r = 0.03;
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x)
                if (inSphere(cellPos(x, y), scx, scy, r)) { dC[ci(x, y)] = 1; hC[ci(x, y)] = 1; }
        for (int y = 0; y <= ny; ++y)
            for (int x = 0; x <= nx; ++x)
                if (inSphere(vertPos(x, y), scx, scy, r)) { dV[vi(x, y)] = 1; hV[vi(x, y)] = 1; }
        const double tiv[4] = {INV_SQRT2, -INV_SQRT2, INV_SQRT2, -INV_SQRT2};
        for (int y = 0; y <= ny; ++y)
            for (int x = 0; x <= nx; ++x) {
                int v = vi(x, y);
                if (!open[v] || !inSphere(vertPos(x, y), scx, scy, r)) continue;
                for (int k = 0; k < 4; ++k) tv[4 * v + k] = tiv[k] * 1.0;
            }
        for (int y = 0; y <= ny; ++y)
            for (int x = 0; x < nx; ++x)
                if (inSphere(macPos(1, x, y), scx, scy, r)) my[myi(x, y)] = 1.0;
    }
    // constrainVelocity (include/ast_solver.h:609-616): closed x walls
    void constrain() {
        for (int y = 0; y < ny; ++y) {
            mx[mxi(0, y)] = 0;
            mx[mxi(nx, y)] = 0;
        }
    }
    // addForce (include/ast_solver.h:246-281), buoyancy beta = 0.5 on the upward components
    void force(double dt) {
        const double beta = 0.5;
        for (int y = 0; y <= ny; ++y)
            for (int x = 0; x <= nx; ++x) {
                int v = vi(x, y);
                if (!open[v]) continue;
                P2 pc = vertPos(x, y);
                double f[4];
                for (int k = 0; k < 4; ++k) {
                    P2 p{pc.x + TILT_POS_OFFSET[k][0] * hdx, pc.y + TILT_POS_OFFSET[k][1] * hdx};
                    f[k] = scalarSample(hC, hV, open, p) * ((k & 1) ? -INV_SQRT2 : INV_SQRT2);
                }
                for (int k = 0; k < 4; ++k) tv[4 * v + k] += f[k] * beta * dt;
            }
        for (int y = 0; y <= ny; ++y)
            for (int x = 0; x < nx; ++x) my[myi(x, y)] += scalarSample(hC, hV, open, macPos(1, x, y)) * beta * dt;
        constrain();
    }
    double macAt(int axis, int x, int y) const { return axis == 0 ? mx[mxi(x, y)] : my[myi(x, y)]; }
    // project (include/ast_solver.h:326-469): system assembly, b scaled by rho/dt, MIC(0)-PCG
    void assemble(double dt) {
        updateIndex();
        const int nc = nx * ny;
        A.reset(nIndex);
        b.assign(nIndex, 0.0);
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) {
                int c = pIdx[ci(x, y)];
                double center = 0, tb = 0, fa[4] = {0, 0, 0, 0};
                uint8_t bits = cellTilt[ci(x, y)];
                for (int k = 0; k < 4; ++k) {
                    if (!((bits >> k) & 1)) continue;
                    for (int i = 0; i < 2; ++i) fa[TILT_DIRECTION_NEIGHBOR_MAC2[k][i]] -= hdx;
                    int vx = x + OCT_NB_TILT_DXDY[k][0], vy = y + OCT_NB_TILT_DXDY[k][1];
                    int t = pIdx[nc + vi(vx, vy)];
                    double area = hdx * SQRT2 * (1.0 - 0.5 * 0.0);
                    double coeff = area / tiltOctDx;
                    A.set(c, t, -coeff);
                    center += coeff;
                    int sign = k <= 1 ? -1 : 1;
                    tb += sign * area * tv[4 * vi(vx, vy) + (k + 2) % 4];
                }
                for (int k = 0; k < 4; ++k) {
                    fa[k] += dx;
                    int axis = k / 2;
                    if (!(fa[k] > EPS)) continue;
                    int nbx = x, nby = y;
                    (axis == 0 ? nbx : nby) += (k & 1) ? -1 : 1;
                    int fx = x + (axis == 0 && !(k & 1)), fy = y + (axis == 1 && !(k & 1));
                    if (cellValid(nbx, nby)) {
                        int t = pIdx[ci(nbx, nby)];
                        double coeff = fa[k] / dx;
                        A.set(c, t, -coeff);
                        center += coeff;
                        tb += ((k & 1) ? 1 : -1) * fa[k] * macAt(axis, fx, fy);
                    } else if (axis == 1) {
                        double coeff = fa[k] / dx;
                        center += coeff;
                        tb += ((k & 1) ? 1 : -1) * fa[k] * macAt(axis, fx, fy);
                    }
                }
                if (center < EPS) center = 1;
                b[c] = tb;
                A.set(c, c, center);
            }
        for (int y = 0; y <= ny; ++y)
            for (int x = 0; x <= nx; ++x) {
                int v = vi(x, y);
                if (!open[v]) continue;
                int c = pIdx[nc + v];
                double center = 0, tb = 0, fa[4] = {0, 0, 0, 0};
                for (int k = 0; k < 4; ++k) {
                    fa[k] += hdx * SQRT2;
                    if (fa[k] < EPS) continue;
                    int t = pIdx[ci(x + TILT_NB_OCT_DXDY[k][0], y + TILT_NB_OCT_DXDY[k][1])];
                    double coeff = fa[k] / tiltOctDx;
                    A.set(c, t, -coeff);
                    center += coeff;
                    int sign = k <= 1 ? -1 : 1;
                    tb += sign * fa[k] * tv[4 * v + k];
                }
                A.set(c, c, center);
                b[c] = tb;
            }
        const double s = rho / dt;
        for (double& e : b) e *= s;
    }
    // correctVelocityByPressure (include/ast_solver.h:283-324)
    void correct(double dt) {
        const int nc = nx * ny;
        for (int y = 0; y <= ny; ++y)
            for (int x = 0; x <= nx; ++x) {
                int v = vi(x, y);
                if (!open[v]) continue;
                int c = pIdx[nc + v];
                if (c < 0) continue;
                for (int k = 0; k < 4; ++k) {
                    int t = pIdx[ci(x + TILT_NB_OCT_DXDY[k][0], y + TILT_NB_OCT_DXDY[k][1])];
                    tv[4 * v + k] += ((k < 2) ? -1 : 1) * dt / rho * (p[t] - p[c]) / tiltOctDx;
                }
            }
        auto pAt = [&](int x, int y) { return cellValid(x, y) ? p[pIdx[ci(x, y)]] : 0.0; };
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x <= nx; ++x) mx[mxi(x, y)] -= dt / rho * (pAt(x, y) - pAt(x - 1, y)) / dx;
        for (int y = 0; y <= ny; ++y)
            for (int x = 0; x < nx; ++x) my[myi(x, y)] -= dt / rho * (pAt(x, y) - pAt(x, y - 1)) / dx;
    }
    void project(double dt) {
        assemble(dt);
        pcg.solve(A, b, p);
        correct(dt);
        constrain();
    }

    // ASTFaceGrid::updateDualGrid with CORRECTION_MAC (include/ast_face_grid.h:69-150), open tilts
    void updateDual() {
        for (int y = 0; y <= ny; ++y)
            for (int x = 0; x <= nx; ++x) {
                int v = vi(x, y);
                if (!open[v]) continue;
                const double* u = &tv[4 * v];
                double s02 = u[0] + u[2], s13 = u[1] + u[3];
                double ux = TILT_UNIT_DIR[0][0] * s02 + TILT_UNIT_DIR[1][0] * s13;
                double uy = TILT_UNIT_DIR[0][1] * s02 + TILT_UNIT_DIR[1][1] * s13;
                dual[2 * v] = ux * 0.5;
                dual[2 * v + 1] = uy * 0.5;
            }
    }
    // adjustLayout with LAYOUT_ADJUST_DENSITY (include/ast_solver.h:471-531): a tilt opens where
    // the back-traced density lies in (0.005, 0.7); fixed tilts stay closed
    void adjustLayout(double dt) {
        for (int y = 0; y <= ny; ++y)
            for (int x = 0; x <= nx; ++x) {
                int v = vi(x, y);
                openTmp[v] = 0;
                P2 old = backTrace(vertPos(x, y), dt);
                double t = scalarSample(dC, dV, open, old);
                if (t > 0.005 && t < 0.7) openTmp[v] = 1;
            }
        for (size_t v = 0; v < fixedT.size(); ++v)
            if (fixedT[v]) openTmp[v] = 0;
    }
    // semiLagrangianAST (include/ast_advection.h:18-29) into the new layout
    void advectScalar(std::vector<double>& c, std::vector<double>& v, double dt) {
        std::vector<double> nc = c, nv = v;
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) nc[ci(x, y)] = scalarSample(c, v, open, backTrace(cellPos(x, y), dt));
        for (int y = 0; y <= ny; ++y)
            for (int x = 0; x <= nx; ++x)
                if (openTmp[vi(x, y)]) nv[vi(x, y)] = scalarSample(c, v, open, backTrace(vertPos(x, y), dt));
        c.swap(nc);
        v.swap(nv);
    }
    // semiLagrangianASTVector (include/ast_advection.h:31-68): tilted faces project the sampled
    // velocity on TILT_UNIT_DIR[k % 2], MAC faces take their own component
    void advectVelocity(double dt) {
        std::vector<double> ntv = tv, nmx = mx, nmy = my;
        for (int y = 0; y <= ny; ++y)
            for (int x = 0; x <= nx; ++x) {
                int v = vi(x, y);
                if (!openTmp[v]) continue;
                P2 pc = vertPos(x, y);
                for (int k = 0; k < 4; ++k) {
                    P2 p{pc.x + TILT_POS_OFFSET[k][0] * hdx, pc.y + TILT_POS_OFFSET[k][1] * hdx};
                    P2 s = velSample(backTrace(p, dt));
                    const double* up = TILT_UNIT_DIR[k % 2];
                    ntv[4 * v + k] = s.x * up[0] + s.y * up[1];
                }
            }
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x <= nx; ++x) nmx[mxi(x, y)] = velSample(backTrace(macPos(0, x, y), dt)).x;
        for (int y = 0; y <= ny; ++y)
            for (int x = 0; x < nx; ++x) nmy[myi(x, y)] = velSample(backTrace(macPos(1, x, y), dt)).y;
        tv.swap(ntv);
        mx.swap(nmx);
        my.swap(nmy);
    }
    // advect (include/ast_solver.h:533-553)
    void advect(double dt) {
        updateDual();
        if (adaptive) adjustLayout(dt);
        advectScalar(dC, dV, dt);
        advectScalar(hC, hV, dt);
        advectVelocity(dt);
        open.swap(openTmp);
        propagate();
    }
    // ASTSolver::cfl / numberOfSubTimeSteps (include/ast_solver.h:50-70): the lower x and y
    // faces of every cell, an integer CFL number, max_cfl 2 in integer division
    int numberOfSubTimeSteps(double dt) const {
        double m = 0;
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) {
                double vx = mx[mxi(x, y)], vy = my[myi(x, y)];
                m = std::max(m, vx * vx + vy * vy);
            }
        double c = dt * std::sqrt(m) / dx;
        if (!(c < 2147483647.0)) throw std::runtime_error("2-D oracle: CFL number out of int range");
        int cfl = (int)c;
        int step = (int)std::ceil(cfl / maxCfl);
        return step > 1 ? step : 1;
    }
    // onUpdate (include/ast_solver.h:100-108) without the images
    void substep(double dt) {
        subDt.push_back(dt);
        source();
        force(dt);
        project(dt);
        advect(dt);
    }
    // Solver::update without a fixed time step (src/solver.cpp:8-46)
    void update(double dt) {
        double remaining = dt;
        substeps = 0;
        while (remaining > EPS) {
            int n = numberOfSubTimeSteps(remaining);
            double actual = remaining / (double)n;
            substep(actual);
            ++substeps;
            remaining -= actual;
        }
    }
};

}  // namespace ast2o

// ---- C interface for the Python wrapper (oracle/oracle.py)
using ast2o::Solver2;

static thread_local std::string g_err;

template <class F>
static int guarded(F f) {
    try {
        f();
        return 0;
    } catch (const std::exception& e) {
        g_err = e.what();
        return -1;
    }
}

struct Field2 {
    int kind;  // 0 f64, 1 u8, 2 i32
    void* ptr;
    long n;
};

static thread_local std::vector<double> g_vals;

static bool field(Solver2* s, const char* name, Field2* f, std::vector<int>& scratch) {
    const std::string n(name);
    const int nc = s->nx * s->ny;
    auto f64 = [&](std::vector<double>& v) { *f = Field2{0, v.data(), (long)v.size()}; return true; };
    if (n == "density_cell") return f64(s->dC);
    if (n == "density_vert") return f64(s->dV);
    if (n == "heat_cell") return f64(s->hC);
    if (n == "heat_vert") return f64(s->hV);
    if (n == "mac_x") return f64(s->mx);
    if (n == "mac_y") return f64(s->my);
    if (n == "tilt_vel") return f64(s->tv);
    if (n == "dual_vert") return f64(s->dual);
    if (n == "b") return f64(s->b);
    if (n == "p") return f64(s->p);
    if (n == "sub_dt") return f64(s->subDt);
    if (n == "tilt_open") { *f = Field2{1, s->open.data(), (long)s->open.size()}; return true; }
    if (n == "pindex_cell") { *f = Field2{2, s->pIdx.data(), (long)nc}; return true; }
    if (n == "pindex_vert") { *f = Field2{2, s->pIdx.data() + nc, (long)(s->pIdx.size() - nc)}; return true; }
    if (n == "A_val") {
        g_vals.clear();
        for (int i = 0; i < s->A.n; ++i) g_vals.insert(g_vals.end(), s->A.val[i].begin(), s->A.val[i].end());
        *f = Field2{0, g_vals.data(), (long)g_vals.size()};
        return true;
    }
    if (n == "A_rowptr" || n == "A_col") {
        scratch.clear();
        if (n == "A_rowptr") {
            scratch.push_back(0);
            for (int i = 0; i < s->A.n; ++i) scratch.push_back(scratch.back() + (int)s->A.idx[i].size());
        } else {
            for (int i = 0; i < s->A.n; ++i) scratch.insert(scratch.end(), s->A.idx[i].begin(), s->A.idx[i].end());
        }
        *f = Field2{2, scratch.data(), (long)scratch.size()};
        return true;
    }
    return false;
}

extern "C" {

const char* ast2o_error() { return g_err.c_str(); }

// workers: the reference's taskflow worker count (its default is the host's hardware threads,
// src/util.cpp:10), which sets the slices of its dot products in reduce mode 0
void* ast2o_create(int nx, int ny, double dx, int adaptive, int reduceMode, int workers) {
    if (nx < 2 || ny < 2 || !(dx > 0) || workers < 1) {
        g_err = "2-D oracle: resolution must be at least 2x2, dx positive, workers at least 1";
        return nullptr;
    }
    Solver2* s = new Solver2(nx, ny, dx, adaptive != 0);
    s->pcg.reduceMode = reduceMode;
    s->pcg.workers = workers;
    s->initialize();
    return s;
}

void ast2o_destroy(void* h) { delete (Solver2*)h; }

// one frame: Solver::update's CFL sub-stepping over dt
int ast2o_update(void* h, double dt) { return guarded([&] { ((Solver2*)h)->update(dt); }); }

// one stage of a sub-step: 0 source, 1 force, 2 project, 3 advect, 4 the whole sub-step
int ast2o_stage(void* h, int which, double dt) {
    Solver2* s = (Solver2*)h;
    return guarded([&] {
        switch (which) {
            case 0: s->source(); break;
            case 1: s->force(dt); break;
            case 2: s->project(dt); break;
            case 3: s->advect(dt); break;
            case 4: s->substep(dt); break;
            default: throw std::runtime_error("2-D oracle: unknown stage");
        }
    });
}

// element count and kind (0 f64, 1 u8, 2 i32) of a named field, -1 when unknown
long ast2o_count(void* h, const char* name, int* kind) {
    std::vector<int> scratch;
    Field2 f;
    if (!field((Solver2*)h, name, &f, scratch)) return -1;
    if (kind) *kind = f.kind;
    return f.n;
}

int ast2o_get(void* h, const char* name, void* out, long n) {
    std::vector<int> scratch;
    Field2 f;
    if (!field((Solver2*)h, name, &f, scratch) || n != f.n) {
        g_err = std::string("2-D oracle: bad field or size: ") + name;
        return -1;
    }
    size_t es = f.kind == 0 ? 8 : (f.kind == 1 ? 1 : 4);
    if (f.n) std::memcpy(out, f.ptr, es * f.n);
    return 0;
}

// writes a state field (doubles or tilt_open); tilt_open also refreshes the cells' tilt states
int ast2o_set(void* h, const char* name, const void* in, long n) {
    Solver2* s = (Solver2*)h;
    std::vector<int> scratch;
    Field2 f;
    std::string nm(name);
    bool state = nm != "b" && nm != "p" && nm != "sub_dt" && nm.rfind("pindex", 0) != 0 && nm.rfind("A_", 0) != 0;
    if (!state || !field(s, name, &f, scratch) || n != f.n) {
        g_err = std::string("2-D oracle: field not settable or bad size: ") + name;
        return -1;
    }
    size_t es = f.kind == 0 ? 8 : 1;
    if (f.n) std::memcpy(f.ptr, in, es * f.n);
    if (nm == "tilt_open") s->propagate();
    return 0;
}

// [sub-steps of the last frame, unknowns, PCG iterations, PCG converged, nonzeros, sub-steps taken]
int ast2o_info(void* h, long* out) {
    Solver2* s = (Solver2*)h;
    long nnz = 0;
    for (int i = 0; i < s->A.n; ++i) nnz += (long)s->A.idx[i].size();
    out[0] = s->substeps;
    out[1] = s->nIndex;
    out[2] = s->pcg.iters;
    out[3] = s->pcg.ok ? 1 : 0;
    out[4] = nnz;
    out[5] = (long)s->subDt.size();
    return 0;
}

}  // extern "C"
