// ORACLE — test infrastructure only.
//
// A plain C++ restatement of the reference's octree smoke step
// (YuweiXiao/AST-Grid, OctreeOmniGridSolver3).  It is the checker for the CUDA library: the
// tests, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it; the library never
// does.  Each function cites the reference file:line it restates.  It is pinned against the
// reference itself through the fixtures in tests/golden/ (made by oracle/ref/ref_harness.cpp
// from the reference's own sources).
//
// Data model: "slots".  Level l (0 = finest) stores N_l non-ghost nodes followed by G_l ghost
// nodes in the reference's layout index order (src/octree_layer3.cpp:14-85); the levels are
// concatenated finest first, so slot = level_offset[l] + layout index.  A dense index brick per
// level replaces the reference's hash map (include/octree_layer3.h:24-80).  Every per-node
// field (octagon value, tilt value, MAC faces, 8 tilt slots, dual vectors, tilt-E state) is a
// flat array over slots, double-buffered where the reference swaps grid objects
// (src/octree_omnigrid_solver3.cpp:898-909).
//
// Scope: the benchmark scene has no collider (the collider SDF is the constant +1 of
// src/omni_boundary_solver3.cpp:13-17), so every SDF test of the reference evaluates to
// "outside the solid" and the cut-cell weights are the constants that
// initCuttingCellWeights (src/octree_omnigrid_solver3.cpp:1169-1238) produces for it.
//
// Built with FP contraction off so the arithmetic follows the reference's IEEE order.  The
// optional OpenMP build parallelises only loops whose iterations are independent (one slot or one
// row each), so its results are bit-identical to the serial build.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <limits>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <queue>
#include <tuple>
#include <stdexcept>
#include <string>
#include <vector>

#include "scene.h"

namespace oracle {

static const double SQRT3 = 1.7320508075688772;     // include/macro.h:17
static const double INV_SQRT3 = 1.0 / SQRT3;         // include/macro.h:20
static const double EPS = DBL_EPSILON;               // include/general.h:48

// include/octree_layer.h:3-7
enum { F_VALID = 1, F_GHOST = 2, F_FROM_COARSE = 4 };

// include/constants.h:85-88  (+x, -x, +y, -y, +z, -z)
static const int OCT_NB[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
// include/constants.h:90-93
static const int OCT_NB_TILT[8][3] = {{1, 1, 1}, {0, 1, 1}, {0, 0, 1}, {1, 0, 1},
                                      {1, 1, 0}, {0, 1, 0}, {0, 0, 0}, {1, 0, 0}};
// include/constants.h:96-99
static const int OCT_NB_FACE[6][3] = {{1, 0, 0}, {0, 0, 0}, {0, 1, 0}, {0, 0, 0}, {0, 0, 1}, {0, 0, 0}};
// include/constants.h:102-105
static const int TILT_NB_OCT[8][3] = {{0, 0, 0},  {-1, 0, 0},  {-1, -1, 0},  {0, -1, 0},
                                      {0, 0, -1}, {-1, 0, -1}, {-1, -1, -1}, {0, -1, -1}};
// include/constants.h:111-118
static const int HALF_SLOT[6][5] = {{0, 3, 4, 7, 1}, {0, 1, 4, 5, 2}, {0, 1, 2, 3, 5},
                                    {1, 2, 5, 6, 0}, {2, 3, 6, 7, 4}, {4, 5, 6, 7, 3}};
// include/constants.h:127-130 (indexed by the 5th HALF_SLOT entry)
static const double HALF_DIR_POS[6][3] = {{1, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {0, 1, 0}, {0, 0, 1}};
// include/constants.h:55-60 (components are +-INV_SQRT3)
static const int TILT_UP_SIGN[8][3] = {{1, 1, 1},   {-1, 1, 1}, {-1, -1, 1}, {1, -1, 1},
                                       {-1, -1, 1}, {1, -1, 1}, {1, 1, 1},   {-1, 1, 1}};
// include/constants.h:146-155, XYZ_MARKER codes (0x1000 = VOIDAXIS)
static const int SAMPLE_MARKER[8][8] = {
    {0x1000, 0x011, 0x001, 0x101, 0x110, 0x010, 0x1000, 0x100},
    {0x011, 0x1000, 0x201, 0x001, 0x010, 0x210, 0x200, 0x1000},
    {0x001, 0x201, 0x1000, 0x021, 0x1000, 0x200, 0x220, 0x020},
    {0x101, 0x001, 0x021, 0x1000, 0x100, 0x1000, 0x020, 0x120},
    {0x110, 0x010, 0x1000, 0x100, 0x1000, 0x012, 0x002, 0x102},
    {0x010, 0x210, 0x200, 0x1000, 0x012, 0x1000, 0x202, 0x002},
    {0x1000, 0x200, 0x220, 0x020, 0x002, 0x202, 0x1000, 0x022},
    {0x100, 0x1000, 0x020, 0x120, 0x102, 0x002, 0x022, 0x1000}};

static double tilt_up(int k, int c) { return TILT_UP_SIGN[k][c] * INV_SQRT3; }

struct V3 {
    double x, y, z;
    double& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    double operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
static V3 v3(double a, double b, double c) { return V3{a, b, c}; }
static V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
static V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
static V3 operator*(V3 a, double s) { return v3(a.x * s, a.y * s, a.z * s); }
static V3 operator/(V3 a, double s) { return v3(a.x / s, a.y / s, a.z / s); }
static double dot3(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// include/util.h:164-187
template <class T> static T lerp(const T& a, const T& b, double f) { return a * (1 - f) + b * f; }
template <class T> static T trilerp(const T& f000, const T& f100, const T& f010, const T& f110, const T& f001,
                                    const T& f101, const T& f011, const T& f111, double tx, double ty, double tz) {
    T a = lerp(lerp(f000, f100, tx), lerp(f010, f110, tx), ty);
    T b = lerp(lerp(f001, f101, tx), lerp(f011, f111, tx), ty);
    return lerp(a, b, tz);
}
// include/util.h:258-282
static void bary(double x, int iLow, int iHigh, int* i, double* f) {
    double s = std::floor(x);
    *i = (int)s;
    int off = -iLow;
    iLow += off;
    iHigh += off;
    if (iLow == iHigh) { *i = iLow; *f = 0; }
    else if (*i < iLow) { *i = iLow; *f = 0; }
    else if (*i > iHigh - 1) { *i = iHigh - 1; *f = 1; }
    else *f = x - s;
    *i -= off;
}
// include/util.h:243-256 (Eigen vector form: truncating cast, clamped)
static void bary_vec(double x, int high, int* i, double* f) {
    int c = (int)x;
    if (c < 0) c = 0;
    if (c > high - 1) c = high - 1;
    *i = c;
    double t = x - c;
    *f = t < 0 ? 0 : (t > 1 ? 1 : t);
}

// tilt-E node, include/tilt_e_node.h:15-56
struct TiltE {
    double e = 0;
    bool largest = false, closed = true, fixed = false, tjoint = false, closedByT = false, half = false;
    int dir = 0;
    void setE(double ne, double maxE = -1) {
        if (fixed) return;
        if (ne <= 0) { closed = true; largest = false; ne = 0; }
        else if (maxE > 0 && ne >= maxE) { closed = false; largest = true; ne = maxE; }
        else { closed = false; largest = false; }
        e = ne;
    }
};

struct Params {
    double tol = 1e-6, buoyD = -0.1, buoyT = 1.0, decay = 1.0, rho = 2.0, noise = 1e-3;
    double omega = 0.97, minDiag = 0.25;
    uint64_t seed = 0;
    int maxIter = 3000;
    bool tiltAdaptivity = true;
    astg_scene::Sphere src = astg_scene::default_source();
    int closedMask = 1 | 2 | 4 | 8 | 32;  // bits: x+, x-, y+, y-, z+, z- (OCT_NB order); z+ open
    // Order of the floating-point reductions (dot products, the mean temperature):
    //  0 = the reference's own order: Eigen 3.3.7's SSE2 dot (two packets of two lanes,
    //      Eigen/src/Core/Redux.h) and BLAS::sum's per-worker partial sums
    //      (include/pcgsolver/blas_wrapper.h:101-110 over ThreadPool::parallelForPlainTF,
    //      include/thread_pool.h:319-348) with refWorkers workers;
    //  1 = the fixed reduction tree of the CUDA library (chunks of 2048, 256 lanes x 8
    //      strided elements, binary tree over the lanes, chunk partials reduced the same way),
    //      and one fused multiply-add for every product the PCG accumulates: each MIC(0) sweep
    //      update, each CSR row term, each dot-product lane term and the vector updates.
    int reduceMode = 0;
    int refWorkers = 8;
};

// ---------------------------------------------------------------- reductions
// Eigen 3.3.7 LinearVectorizedTraversal redux of a*b with 16-byte aligned data and packets of
// two doubles: four running lanes over groups of four, folded pairwise, then the scalar tail.
static double eigenDot(const double* a, const double* b, size_t n) {
    size_t asz2 = (n / 4) * 4, asz = (n / 2) * 2;
    if (asz == 0) {
        double s = 0;
        for (size_t i = 0; i < n; ++i) s += a[i] * b[i];
        return s;
    }
    double l0 = a[0] * b[0], l1 = a[1] * b[1];
    if (asz > 2) {
        double l2 = a[2] * b[2], l3 = a[3] * b[3];
        for (size_t i = 4; i < asz2; i += 4) {
            l0 += a[i] * b[i];
            l1 += a[i + 1] * b[i + 1];
            l2 += a[i + 2] * b[i + 2];
            l3 += a[i + 3] * b[i + 3];
        }
        l0 = l0 + l2;
        l1 = l1 + l3;
        if (asz > asz2) {
            l0 += a[asz2] * b[asz2];
            l1 += a[asz2 + 1] * b[asz2 + 1];
        }
    }
    double r = l0 + l1;
    for (size_t i = asz; i < n; ++i) r += a[i] * b[i];
    return r;
}

// The CUDA library's fixed reduction tree.  Element i belongs to chunk i / 2048 and lane
// (i % 2048) % 256; a lane accumulates its (up to) eight elements in index order starting from 0
// with step(acc, i) (a sum adds the element; a dot is one fused multiply-add per element), the 256
// lanes are folded by halving strides (lane t += lane t + s for s = 128 ... 1), and the chunk
// partials are added by the same rule until one value is left.
static const int RED_LANES = 256, RED_PER_LANE = 8, RED_CHUNK = RED_LANES * RED_PER_LANE;
template <class F>
static double treeReduce(size_t n, const F& step) {
    if (n == 0) return 0.0;
    std::vector<double> part((n + RED_CHUNK - 1) / RED_CHUNK);
    double lane[RED_LANES];
    for (size_t c = 0; c < part.size(); ++c) {
        size_t base = c * RED_CHUNK;
        for (int t = 0; t < RED_LANES; ++t) {
            double acc = 0.0;
            for (int k = 0; k < RED_PER_LANE; ++k) {
                size_t i = base + t + (size_t)RED_LANES * k;
                if (i < n) acc = step(acc, i);
            }
            lane[t] = acc;
        }
        for (int st = RED_LANES / 2; st >= 1; st >>= 1)
            for (int t = 0; t < st; ++t) lane[t] = lane[t] + lane[t + st];
        part[c] = lane[0];
    }
    while (part.size() > 1) {
        std::vector<double> q = part;
        part = std::vector<double>((q.size() + RED_CHUNK - 1) / RED_CHUNK);
        for (size_t c = 0; c < part.size(); ++c) {
            size_t base = c * RED_CHUNK;
            for (int t = 0; t < RED_LANES; ++t) {
                double acc = 0.0;
                for (int k = 0; k < RED_PER_LANE; ++k) {
                    size_t i = base + t + (size_t)RED_LANES * k;
                    if (i < q.size()) acc = acc + q[i];
                }
                lane[t] = acc;
            }
            for (int st = RED_LANES / 2; st >= 1; st >>= 1)
                for (int t = 0; t < st; ++t) lane[t] = lane[t] + lane[t + st];
            part[c] = lane[0];
        }
    }
    return part[0];
}

// BLAS::sum: per-worker partial sums over parallelForPlainTF's slices, added in worker order
static double refSum(const double* v, size_t size, int workers) {
    std::vector<double> sums(workers, 0.0);
    long long start = 0, end = (long long)size;
    long long n = end - start + 1;
    long long slice = (long long)std::round(n / (double)workers);
    slice = std::max(slice, 1LL);
    long long i1 = start, i2 = std::min(start + slice, end);
    int i = 0;
    auto run = [&](long long a, long long b2, int w) {
        double t = 0;
        for (long long k = a; k < b2; ++k) t += v[k];
        sums[w] = t;
    };
    for (; i + 1 < workers && i1 < end; i++) {
        run(i1, i2, i);
        i1 = i2;
        i2 = std::min(i2 + slice, end);
    }
    if (i1 < end) run(i1, end, i);
    double acc = 0.0;
    for (double x : sums) acc += x;
    return acc;
}

// Row-list sparse matrix with sorted columns, include/pcgsolver/sparse_matrix.h:14-103
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
    void add(int i, int j, double v) {
        auto& I = idx[i];
        auto& V = val[i];
        size_t k = 0;
        for (; k < I.size(); ++k) {
            if (I[k] == j) { V[k] += v; return; }
            if (I[k] > j) { I.insert(I.begin() + k, j); V.insert(V.begin() + k, v); return; }
        }
        I.push_back(j);
        V.push_back(v);
    }
};

class Solver {
public:
    // ---------------------------------------------------------------- topology
    int res = 0, L = 0;
    double dx = 0;
    Params P;
    std::vector<int> lres, loff, lN, lG;  // per level
    std::vector<double> ldh;
    std::vector<std::vector<int>> brick;  // per level dense index, -1 = absent
    std::vector<int> sx, sy, sz, slev, sflag;
    int S = 0;
    std::vector<int32_t> split;
    std::vector<int> halfTilts, tJoints, closedByHalf;  // slots
    std::vector<double> wMac[3];
    std::vector<double> wTilt;  // S*8
    // Collider: OmniBoundarySolver3's SDF grid (res^3 finest cells, spacing dx, index
    // (z*res + y)*res + x; src/omni_boundary_solver3.cpp:11-32); empty = no collider (the reference's
    // grid filled with 1, on which every test below is false).  colCentre is the centre the
    // inside-solid projection takes its normals from, hard-coded (0.5, 0.5, 0.45) in the reference
    // (include/omni_boundary_solver3.h:27,57,77).
    std::vector<double> colSdf;
    V3 colCentre{0.5, 0.5, 0.45};
    double M37[128][3][7];      // OCTREE_OMNI_DUAL_GRAPH_EIGEN_MATRIX3, bits x y z n0 n1 n2 n3
    int anomalies = 0;          // lookups the reference would have inserted into its hash map

    // ---------------------------------------------------------------- state
    int cur = 0;
    std::vector<TiltE> tiltE[2];
    std::vector<uint8_t> tOpen, tFixed;  // tilt_layout (OctreeOmniGridLayout)
    std::vector<double> dO[2], dT[2], hO[2], hT[2];
    std::vector<double> mac[2][3];
    std::vector<double> tv[2];  // S*8
    std::vector<double> dual[2][2];  // [buf][0 oct,1 tilt] S*3
    std::vector<int> pO, pT;          // pIndex octagon / tilt
    int nDof = 0;
    RowMatrix A;
    std::vector<double> b, p;
    int pcgIters = 0;
    double pcgErr = 0, ambT = 0;
    bool pcgOk = false, firstSource = true;
    // CSR copy of the last system (for the tests)
    std::vector<int> csrPtr, csrCol;
    std::vector<double> csrVal;

    // ---------------------------------------------------------------- lookups
    int get(int l, int x, int y, int z) const {  // layout->get (ghosts included)
        if (l < 0 || l >= L) return -1;
        int r = lres[l];
        if (x < 0 || y < 0 || z < 0 || x >= r || y >= r || z >= r) return -1;
        return brick[l][((size_t)z * r + y) * r + x];
    }
    int slotOf(int l, int x, int y, int z) const {
        int i = get(l, x, y, z);
        return i < 0 ? -1 : loff[l] + i;
    }
    int slotReq(int l, int x, int y, int z) {
        int s = slotOf(l, x, y, z);
        if (s < 0) {
            char m[160];
            snprintf(m, sizeof m, "oracle: missing layout node l=%d (%d,%d,%d)", l, x, y, z);
            throw std::runtime_error(m);
        }
        return s;
    }
    bool isGhostNode(int l, int x, int y, int z) {  // layout->node(...).flag & IS_GHOST
        int s = slotOf(l, x, y, z);
        if (s < 0) {
#pragma omp atomic
            ++anomalies;
            return false;
        }
        return sflag[s] & F_GHOST;
    }
    double dh(int l) const { return ldh[l]; }
    bool octValid(int l, int x, int y, int z) const {  // include/octree_cell_centered_grid3.h:35
        int r = lres[l] - 1;
        return x >= 0 && y >= 0 && z >= 0 && x < r && y < r && z < r;
    }
    bool layValid(int l, int x, int y, int z) const {  // OctreeGridLayout3::isValid
        int r = lres[l];
        return x >= 0 && y >= 0 && z >= 0 && x < r && y < r && z < r;
    }
    bool macValid(int a, int l, int x, int y, int z) const {  // include/octree_face_centered_grid3.h:29-31
        int r = lres[l];
        int c[3] = {x, y, z};
        for (int k = 0; k < 3; ++k) {
            int hi = (k == a) ? r : r - 1;
            if (c[k] < 0 || c[k] >= hi) return false;
        }
        return true;
    }
    // src/octree_grid_layout3.cpp:51-69
    int getUntil(int l, int x, int y, int z, bool toFinest) {
        int r = lres[l];
        if (x < 0 || y < 0 || z < 0 || x >= r || y >= r || z >= r) return -1;
        for (;;) {
            int s = slotOf(l, x, y, z);
            if (s >= 0 && !(sflag[s] & F_GHOST)) return s;
            if (toFinest) { x <<= 1; y <<= 1; z <<= 1; l -= 1; }
            else { x >>= 1; y >>= 1; z >>= 1; l += 1; }
            if (l < 0 || l >= L) return -1;
        }
    }
    // src/octree_grid_layout3.cpp:16-41: finest non-ghost cell containing pos
    int levelCoordinate(double px, double py, double pz) {
        int xi, yi, zi;
        double f;
        bary(px / dx, 0, res, &xi, &f);
        bary(py / dx, 0, res, &yi, &f);
        bary(pz / dx, 0, res, &zi, &f);
        for (int l = 0; l < L; ++l) {
            int s = slotOf(l, xi, yi, zi);
            if (s >= 0 && !(sflag[s] & F_GHOST)) return l;
            xi >>= 1; yi >>= 1; zi >>= 1;
        }
        throw std::runtime_error("oracle: levelCoordinate found no cell");
    }

    // ---------------------------------------------------------------- construction
    // src/octree_layer3.cpp:7-88 for every level, src/octree_grid_layout3.cpp:6-13
    void buildLayout() {
        lres.resize(L); loff.resize(L); lN.resize(L); lG.resize(L); ldh.resize(L);
        brick.assign(L, {});
        sx.clear(); sy.clear(); sz.clear(); slev.clear(); sflag.clear();
        int off = 0;
        for (int l = 0; l < L; ++l) {
            int r = res >> l;
            lres[l] = r;
            ldh[l] = dx * (1 << l);
            loff[l] = off;
            brick[l].assign((size_t)r * r * r, -1);
            std::vector<int> nodes;
            auto sp = [&](int x, int y, int z) { return split[((size_t)(z << l) * res + (y << l)) * res + (x << l)]; };
            for (int z = 0; z < r; ++z)
                for (int y = 0; y < r; ++y)
                    for (int x = 0; x < r; ++x)
                        if (sp(x, y, z) == l) {
                            brick[l][((size_t)z * r + y) * r + x] = (int)nodes.size() / 3;
                            nodes.push_back(x); nodes.push_back(y); nodes.push_back(z);
                        }
            int n = nodes.size() / 3;
            lN[l] = n;
            for (int i = 0; i < n; ++i) {
                sx.push_back(nodes[3 * i]); sy.push_back(nodes[3 * i + 1]); sz.push_back(nodes[3 * i + 2]);
                slev.push_back(l); sflag.push_back(F_VALID);
            }
            int cIdx = n;
            for (int i = 0; i < n; ++i) {
                for (int a = -1; a <= 1; ++a)
                    for (int bb = -1; bb <= 1; ++bb)
                        for (int c = -1; c <= 1; ++c) {
                            if (a == 0 && bb == 0 && c == 0) continue;
                            int nx = nodes[3 * i] + a, ny = nodes[3 * i + 1] + bb, nz = nodes[3 * i + 2] + c;
                            if (nx < 0 || ny < 0 || nz < 0 || nx >= r || ny >= r || nz >= r) continue;
                            int tv = sp(nx, ny, nz);
                            int& bk = brick[l][((size_t)nz * r + ny) * r + nx];
                            if (bk >= 0) continue;
                            if (tv == l - 1 || tv == l + 1) {
                                bk = cIdx++;
                                sx.push_back(nx); sy.push_back(ny); sz.push_back(nz); slev.push_back(l);
                                sflag.push_back(F_VALID | F_GHOST | (tv == l + 1 ? F_FROM_COARSE : 0));
                            }
                        }
            }
            lG[l] = cIdx - n;
            off += cIdx;
        }
        S = off;
    }

    // OctreeVertexCenteredGrid3<TiltENode>::updateGhost, src/octree_vertex_centered_grid3.cpp:6-24
    template <class T>
    void vertexCopyGhost(std::vector<T>& g) {
        for (int l = 0; l < L; ++l)
            for (int i = lN[l]; i < lN[l] + lG[l]; ++i) {
                int s = loff[l] + i;
                int x = sx[s], y = sy[s], z = sz[s];
                if (sflag[s] & F_FROM_COARSE) {
                    if ((x & 1) || (y & 1) || (z & 1)) continue;
                    g[s] = g[slotReq(l + 1, x >> 1, y >> 1, z >> 1)];
                } else {
                    g[s] = g[slotReq(l - 1, x << 1, y << 1, z << 1)];
                }
            }
    }

    // src/octree_util.cpp:38-169
    void constrainTiltE(std::vector<TiltE>& te, bool record) {
        // T-joints
        for (int s = 0; s < S; ++s) {
            if (sflag[s] & F_GHOST) continue;
            int l = slev[s], x = sx[s], y = sy[s], z = sz[s];
            TiltE n = te[s];
            int minL = l, maxL = l;
            for (int i = -1; i <= 0; ++i)
                for (int j = -1; j <= 0; ++j)
                    for (int k = -1; k <= 0; ++k) {
                        int c = getUntil(l, x + i, y + j, z + k, true);
                        if (c < 0) c = getUntil(l, x + i, y + j, z + k, false);
                        // the reference tests the packed coordinate c > 0, which excludes the
                        // finest-level node (0,0,0)
                        if (c >= 0 && !(slev[c] == 0 && sx[c] == 0 && sy[c] == 0 && sz[c] == 0)) {
                            minL = std::min(minL, slev[c]);
                            maxL = std::max(maxL, slev[c]);
                        }
                    }
            if (minL < l || (maxL > l && !(x & 1) && !(y & 1) && !(z & 1))) {
                n.tjoint = true;
                n.e = dh(minL);
                n.fixed = true;
                n.closed = false;
                if (record) tJoints.push_back(s);
            }
            te[s] = n;
        }
        // tilts closed by T-joints
        for (int s = 0; s < S; ++s) {
            if (sflag[s] & F_GHOST) continue;
            if (!te[s].tjoint) continue;
            int l = slev[s];
            int ix = sx[s], iy = sy[s], iz = sz[s];
            int tl = l;
            if (te[s].e < dh(l)) { tl -= 1; ix *= 2; iy *= 2; iz *= 2; }
            for (int i = 0; i < 6; ++i) {
                int t = slotOf(tl, ix + OCT_NB[i][0], iy + OCT_NB[i][1], iz + OCT_NB[i][2]);
                if (t >= 0) {
                    TiltE n = te[t];
                    n.setE(0);
                    n.fixed = true;
                    n.closedByT = true;
                    te[t] = n;
                }
            }
        }
        vertexCopyGhost(te);
        // half tilts
        for (int s = 0; s < S; ++s) {
            if (sflag[s] & F_GHOST) continue;
            TiltE tn = te[s];
            if (!tn.tjoint) continue;
            int l = slev[s];
            bool coarse = tn.e < dh(l);
            int ci[3];
            if (coarse) { ci[0] = sx[s]; ci[1] = sy[s]; ci[2] = sz[s]; }
            else { ci[0] = sx[s] >> 1; ci[1] = sy[s] >> 1; ci[2] = sz[s] >> 1; }
            int lc = l + (!coarse);
            for (int axis = 0; axis < 3; ++axis) {
                if (ci[axis] == 0 || ci[axis] == lres[l - coarse] - 1) continue;
                bool flag = true;
                for (int i = 0; i <= 1 && flag; ++i)
                    for (int j = 0; j <= 1 && flag; ++j) {
                        if (i == 0 && j == 0) continue;
                        int id[3] = {ci[0], ci[1], ci[2]};
                        id[(axis + 1) % 3] += i;
                        id[(axis + 2) % 3] += j;
                        int c = (lc < L) ? getUntil(lc, id[0], id[1], id[2], true) : -1;
                        if (c < 0 && lc < L) c = getUntil(lc, id[0], id[1], id[2], false);
                        if (c >= 0) { if (!te[c].tjoint) flag = false; }
                        else flag = false;
                    }
                if (flag) {
                    int nb[3] = {ci[0], ci[1], ci[2]};
                    nb[axis] -= 1;
                    int c = (lc < L) ? getUntil(lc, ci[0], ci[1], ci[2], true) : -1;
                    int c1 = (lc < L) ? getUntil(lc, nb[0], nb[1], nb[2], true) : -1;
                    // UNPACK_LEVEL3(-1) reads 15 in the reference
                    int lvc = c >= 0 ? slev[c] : 15;
                    if (c1 < 0 || lvc == slev[c1]) flag = false;
                }
                if (flag) {
                    int id[3] = {ci[0] * 2, ci[1] * 2, ci[2] * 2};
                    id[(axis + 1) % 3] += 1;
                    id[(axis + 2) % 3] += 1;
                    int hl = l - coarse;
                    int hs = slotOf(hl, id[0], id[1], id[2]);
                    if (hs >= 0) {
                        TiltE n = te[hs];
                        n.closed = true;
                        n.half = true;
                        n.fixed = true;
                        n.dir = axis + (coarse ? 3 : 0);
                        n.e = dh(hl);
                        te[hs] = n;
                        if (record) halfTilts.push_back(hs);
                        int t[3] = {id[0], id[1], id[2]};
                        t[axis] += n.dir < 3 ? 1 : -1;
                        int ts = slotReq(hl, t[0], t[1], t[2]);
                        if (record && std::find(closedByHalf.begin(), closedByHalf.end(), ts) == closedByHalf.end())
                            closedByHalf.push_back(ts);
                        TiltE m = te[ts];
                        m.setE(0);
                        m.closedByT = true;
                        m.dir = -1;
                        m.fixed = true;
                        te[ts] = m;
                    }
                }
            }
        }
    }

    // Constants::init, src/constants.cpp:170-256: least-squares recovery matrices
    void buildDualTables() {
        memset(M37, 0, sizeof M37);
        const double s = INV_SQRT3;
        const double rows[7][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {s, s, s}, {-s, s, s}, {-s, -s, s}, {s, -s, s}};
        for (int bits = 0; bits < 128; ++bits) {
            int use[7], cnt = 0;
            for (int k = 0; k < 7; ++k) {
                use[k] = (bits >> (6 - k)) & 1;
                cnt += use[k];
            }
            if (cnt <= 1) continue;
            // G = m^T m (3x3)
            double G[3][3] = {{0}};
            for (int r = 0; r < 7; ++r)
                if (use[r])
                    for (int i = 0; i < 3; ++i)
                        for (int j = 0; j < 3; ++j) G[i][j] += rows[r][i] * rows[r][j];
            // inverse through a partial-pivoting LU as Eigen's MatrixXd::inverse() computes it
            // (row pivot = first largest magnitude; column-oriented unit-lower forward
            // substitution; backward substitution multiplying by the pivot's reciprocal)
            double lu[3][3];
            memcpy(lu, G, sizeof lu);
            int tr[3];
            for (int k = 0; k < 3; ++k) {
                int piv = k;
                double best = std::fabs(lu[k][k]);
                for (int i = k + 1; i < 3; ++i)
                    if (std::fabs(lu[i][k]) > best) { best = std::fabs(lu[i][k]); piv = i; }
                tr[k] = piv;
                if (best != 0) {
                    if (piv != k)
                        for (int j = 0; j < 3; ++j) std::swap(lu[k][j], lu[piv][j]);
                    for (int i = k + 1; i < 3; ++i) lu[i][k] /= lu[k][k];
                }
                for (int i = k + 1; i < 3; ++i)
                    for (int j = k + 1; j < 3; ++j) lu[i][j] -= lu[i][k] * lu[k][j];
            }
            double inv[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
            for (int k = 0; k < 3; ++k)
                if (tr[k] != k)
                    for (int j = 0; j < 3; ++j) std::swap(inv[k][j], inv[tr[k]][j]);
            for (int i = 0; i < 3; ++i)
                for (int r2 = i + 1; r2 < 3; ++r2)
                    for (int j = 0; j < 3; ++j) inv[r2][j] -= inv[i][j] * lu[r2][i];
            for (int i = 2; i >= 0; --i) {
                double rcp = 1.0 / lu[i][i];
                for (int j = 0; j < 3; ++j) inv[i][j] *= rcp;
                for (int r2 = 0; r2 < i; ++r2)
                    for (int j = 0; j < 3; ++j) inv[r2][j] -= inv[i][j] * lu[r2][i];
            }
            for (int k = 0; k < 3; ++k)
                for (int r = 0; r < 7; ++r) {
                    if (!use[r]) continue;
                    M37[bits][k][r] = inv[k][0] * rows[r][0] + inv[k][1] * rows[r][1] + inv[k][2] * rows[r][2];
                }
        }
    }
    static int dualBits(int x, int y, int z, int n0, int n1, int n2, int n3) {
        return (x << 6) | (y << 5) | (z << 4) | (n0 << 3) | (n1 << 2) | (n2 << 1) | n3;
    }
    // Matrix37d * Vector7d as Eigen 3.3.7 evaluates it into a Vector3d: rows 0-1 as one SSE2
    // packet (products accumulated in column order), row 2 as a scalar unrolled redux
    // ((a0 + (a1 + a2)) + ((a3 + a4) + (a5 + a6))).
    V3 applyM37(int bits, const double v[7]) const {
        double o[3];
        for (int k = 0; k < 2; ++k) {
            double acc = M37[bits][k][0] * v[0];
            for (int r = 1; r < 7; ++r) acc = acc + M37[bits][k][r] * v[r];
            o[k] = acc;
        }
        double a[7];
        for (int r = 0; r < 7; ++r) a[r] = M37[bits][2][r] * v[r];
        o[2] = (a[0] + (a[1] + a[2])) + ((a[3] + a[4]) + (a[5] + a[6]));
        return v3(o[0], o[1], o[2]);
    }

    // src/octree_omnigrid_solver3.cpp:60-149 + 152-219 + 1169-1238 (no collider)
    void init(int coarsest, int levels, const Params& prm) {
        P = prm;
        L = levels;
        res = coarsest << (levels - 1);
        dx = 1.0 / res;
        split = astg_scene::split_map(res, L, P.src);
        buildLayout();
        buildDualTables();
        for (int b2 = 0; b2 < 2; ++b2) {
            tiltE[b2].assign(S, TiltE());
            dO[b2].assign(S, 0); dT[b2].assign(S, 0); hO[b2].assign(S, 0); hT[b2].assign(S, 0);
            for (int a = 0; a < 3; ++a) mac[b2][a].assign(S, 0);
            tv[b2].assign((size_t)S * 8, 0);
            dual[b2][0].assign((size_t)S * 3, 0);
            dual[b2][1].assign((size_t)S * 3, 0);
        }
        tOpen.assign(S, 0);
        tFixed.assign(S, 0);
        pO.assign(S, -1);
        pT.assign(S, -1);
        halfTilts.clear(); tJoints.clear(); closedByHalf.clear();
        constrainTiltE(tiltE[0], true);
        vertexCopyGhost(tiltE[0]);
        constrainTiltE(tiltE[1], false);
        vertexCopyGhost(tiltE[1]);
        // fixed and outermost tilts, :128-145
        for (int s = 0; s < S; ++s) {
            if (sflag[s] & F_GHOST) continue;
            TiltE n = tiltE[0][s];
            if (n.tjoint || n.fixed) {
                tOpen[s] = !n.closed;
                tFixed[s] = 1;
                continue;
            }
            int l = slev[s], r = lres[l];
            if (sx[s] == 0 || sy[s] == 0 || sz[s] == 0 || sx[s] == r - 1 || sy[s] == r - 1 || sz[s] == r - 1) {
                n.setE(0);
                n.fixed = true;
                tOpen[s] = !n.closed;
                tFixed[s] = 1;
                tiltE[0][s] = n;
                tiltE[1][s] = n;
            }
        }
        cuttingCellWeights();
        cur = 0;
        firstSource = true;
    }

    // ---------------------------------------------------------------- collider
    // boundarySdf->sample(p): CellCenteredGrid<REAL,3>::sample of the collider grid, or the
    // reference's constant 1 without a collider
    double bsdf(const V3& p) const { return colSdf.empty() ? 1.0 : sdfSample(colSdf, res, p); }
    // fractionInside, include/util.h:340-349
    static double fractionInside(double l, double r) {
        if (l < 0 && r < 0) return 1;
        if (l < 0 && r >= 0) return l / (l - r);
        if (l >= 0 && r < 0) return r / (r - l);
        return 0;
    }
    // isInsideSdf, include/util.h:324
    static bool insideSdf(double phi) { return phi <= 0; }
    V3 octPosL(int l, int x, int y, int z) const {
        double h = dh(l);
        return v3(x * h + 0.5 * h, y * h + 0.5 * h, z * h + 0.5 * h);
    }
    // initCuttingCellWeights, src/octree_omnigrid_solver3.cpp:1169-1238 (weightsCC->setAll(1) first,
    // :83): MAC faces and tilt slots of non-ghost nodes get 1 - fractionInside of the SDF at the two
    // octagon centres (tilt centre and octagon centre) when the neighbouring octagon is valid; a half
    // tilt starts from zero and fills its big-octagon slot and its four same-level slots.  Two
    // quirks are kept: the big octagon's position is taken at the half tilt's own level with the
    // coarse index, and the same-level slots sample the SDF at the last position computed (the big
    // octagon's when it was valid, else the half tilt's centre), not at their own octagon.
    void cuttingCellWeights() {
        for (int a = 0; a < 3; ++a) wMac[a].assign(S, 1.0);
        wTilt.assign((size_t)S * 8, 1.0);
        for (int s = 0; s < S; ++s) {
            if (sflag[s] & F_GHOST) continue;
            int l = slev[s], x = sx[s], y = sy[s], z = sz[s];
            double current = bsdf(octPosL(l, x, y, z));
            for (int a = 0; a < 3; ++a) {
                int id[3] = {x, y, z};
                id[a] -= 1;
                if (macValid(a, l, x, y, z) && octValid(l, id[0], id[1], id[2]))
                    wMac[a][s] = 1 - fractionInside(bsdf(octPosL(l, id[0], id[1], id[2])), current);
            }
        }
        for (int s = 0; s < S; ++s) {
            if (sflag[s] & F_GHOST) continue;
            int l = slev[s];
            double current = bsdf(vertPos(s));
            for (int i = 0; i < 8; ++i) {
                int nx = sx[s] + TILT_NB_OCT[i][0], ny = sy[s] + TILT_NB_OCT[i][1], nz = sz[s] + TILT_NB_OCT[i][2];
                if (octValid(l, nx, ny, nz))
                    wTilt[(size_t)s * 8 + i] = 1 - fractionInside(current, bsdf(octPosL(l, nx, ny, nz)));
            }
        }
        for (int hs : halfTilts) {
            double w[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            const TiltE& n = tiltE[0][hs];
            int l = slev[hs];
            V3 pos = vertPos(hs);
            double current = bsdf(pos);
            int id[3] = {sx[hs] >> 1, sy[hs] >> 1, sz[hs] >> 1};
            id[n.dir % 3] -= n.dir < 3 ? 1 : 0;
            if (l + 1 < L && octValid(l + 1, id[0], id[1], id[2])) {
                pos = octPosL(l, id[0], id[1], id[2]);
                w[HALF_SLOT[n.dir][4]] = 1 - fractionInside(current, bsdf(pos));
            }
            for (int i = 0; i < 4; ++i) {
                int k = HALF_SLOT[n.dir][i];
                if (octValid(l, sx[hs] + TILT_NB_OCT[k][0], sy[hs] + TILT_NB_OCT[k][1], sz[hs] + TILT_NB_OCT[k][2]))
                    w[k] = 1 - fractionInside(current, bsdf(pos));
            }
            for (int k = 0; k < 8; ++k) wTilt[(size_t)hs * 8 + k] = w[k];
        }
    }
    // wipeBoundary, src/octree_omnigrid_solver3.cpp:1240-1293 (EXTRAPOLATE_DENSITY undefined): density
    // and heat of non-ghost octagons and tilts and of half tilts whose position has SDF < 0 become
    // 0 / EPSILON = 0
    void wipeBoundary() {
        if (colSdf.empty()) return;
        int c = cur;
        for (int s = 0; s < S; ++s) {
            if (sflag[s] & F_GHOST) continue;
            if (bsdf(cellPos(s)) < 0) { dO[c][s] = 0.0 / DBL_EPSILON; hO[c][s] = 0.0 / DBL_EPSILON; }
        }
        for (int s = 0; s < S; ++s) {
            if (sflag[s] & F_GHOST) continue;
            if (bsdf(vertPos(s)) < 0) { dT[c][s] = 0.0 / DBL_EPSILON; hT[c][s] = 0.0 / DBL_EPSILON; }
        }
        for (int hs : halfTilts)
            if (bsdf(vertPos(hs)) < 0) { dT[c][hs] = 0; hT[c][hs] = 0; }
    }
    // Eigen 3.3.7 on 3-vectors (no packet access: the unrolled redux splits the range in halves,
    // Eigen/src/Core/Redux.h:91-105, so a sum of three terms is t0 + (t1 + t2)): the norm, and the
    // tangential part v - (v . n) n with n normalised by normalize() (division by sqrt of the squared
    // norm when it is positive, Eigen/src/Core/Dot.h:145-151)
    static double sq3(const V3& n) { return n.x * n.x + (n.y * n.y + n.z * n.z); }
    static double norm3(const V3& n) { return std::sqrt(sq3(n)); }
    // OmniBoundarySolver3::updateCollider (src/omni_boundary_solver3.cpp:17-32) for a Sphere3 in
    // ShapeToImplicit3: signedDistanceLocal (include/geometry/shape_to_implicit3.h:41-46) at each
    // cell centre (i + 0.5) * dx of the finest grid.  Sphere3::closestNormalLocal
    // (include/geometry/sphere3.h:24-26) is (1, 0, 0) below epsilon, else normalized(); the
    // transforms' identity orientations leave translations only.  These norms and the dot product
    // are on plain 3-vectors, which Eigen reduces with one SSE2 packet for the first two terms and
    // the third added after, (t0 + t1) + t2 (Eigen/src/Core/Redux.h:306-329).
    static double sq3p(const V3& n) { return (n.x * n.x + n.y * n.y) + n.z * n.z; }
    void sphereSdf(const V3& c, double r) {
        if (!(r > 0)) {
            colSdf.clear();
            return;
        }
        const double dx = 1.0 / res;
        colSdf.assign((size_t)res * res * res, 0.0);
        for (int z = 0; z < res; ++z)
            for (int y = 0; y < res; ++y)
                for (int x = 0; x < res; ++x) {
                    V3 p = v3((x + 0.5) * dx, (y + 0.5) * dx, (z + 0.5) * dx);
                    V3 q = p - c;
                    V3 nl = v3(1, 0, 0);
                    if (!(std::sqrt(sq3p(q)) < DBL_EPSILON)) {
                        double zz = sq3p(q);
                        nl = q;
                        if (zz > 0) {
                            double k = std::sqrt(zz);
                            nl = v3(q.x / k, q.y / k, q.z / k);
                        }
                    }
                    V3 xc = v3(nl.x * r, nl.y * r, nl.z * r) + c;
                    V3 off = p - xc;
                    double dot = (nl.x * off.x + nl.y * off.y) + nl.z * off.z;
                    double len = std::sqrt(sq3p(xc - p));
                    colSdf[((size_t)z * res + y) * res + x] = dot < 0.0 ? -len : len;
                }
    }
    static V3 tangential(const V3& v, V3 n) {
        double z = sq3(n);
        if (z > 0) {
            double q = std::sqrt(z);
            n = v3(n.x / q, n.y / q, n.z / q);
        }
        double d = v.x * n.x + (v.y * n.y + v.z * n.z);
        return v3(v.x - d * n.x, v.y - d * n.y, v.z - d * n.z);
    }
    // OmniBoundarySolver3::constrainVelocity(MAC grid), include/omni_boundary_solver3.h:74-92: each valid
    // face of a non-ghost node inside the solid (SDF <= 0) becomes the matching component of the
    // tangential part of the MAC velocity sampled there, or 0 at the centre itself.  The reference's
    // loop writes the grid it samples from one task per worker, each over a contiguous run of nodes,
    // all at once: where the solid's faces span two runs, what a sample reads depends on thread
    // timing.  Restated with a defined order: every sample reads the velocity as it was before this
    // loop (it agrees with the reference wherever no sample reads another solid face).
    void colliderMac() {
        if (colSdf.empty()) return;
        int c = cur;
        std::vector<double> before[3] = {mac[c][0], mac[c][1], mac[c][2]};
        for (int s = 0; s < S; ++s) {
            if (sflag[s] & F_GHOST) continue;
            for (int a = 0; a < 3; ++a) {
                if (!macValid(a, slev[s], sx[s], sy[s], sz[s])) continue;
                V3 pos = macPos(a, s);
                if (!insideSdf(bsdf(pos))) continue;
                V3 n = pos - colCentre;
                if (norm3(n) < DBL_EPSILON) {
                    mac[c][a][s] = 0;
                } else {
                    V3 t = tangential(macSample(pos, before), n);
                    mac[c][a][s] = t[a];
                }
            }
        }
    }
    // constrainVelocity(tilt grid, MAC grid), include/omni_boundary_solver3.h:26-52: for open tilts of
    // non-ghost nodes with SDF(centre) - dx <= 0, slot k at centre + e/3 (e = dx/2) inside the solid.
    // The reference's projected value is written into a shadowing local Vector3f, not into the tilt,
    // so only the degenerate case (slot position at the centre itself: v[k] = 0) changes the tilt.
    void colliderTilt() {
        if (colSdf.empty()) return;
        int c = cur;
        for (int s = 0; s < S; ++s) {
            if (sflag[s] & F_GHOST) continue;
            if (tiltE[c][s].closed) continue;
            V3 centre = vertPos(s);
            double h = dh(slev[s]);
            if (!insideSdf(bsdf(centre) - h)) continue;
            double e = h * 0.5;
            for (int k = 0; k < 8; ++k) {
                V3 p1 = tiltPos(centre, k, e);
                if (insideSdf(bsdf(p1)) && norm3(p1 - colCentre) < DBL_EPSILON) tv[c][(size_t)s * 8 + k] = 0;
            }
        }
    }
    // constrainVelocity(OctreeOmniVector3Grid3), include/omni_boundary_solver3.h:55-71: the dual vectors
    // at non-ghost tilt positions inside the solid lose their normal part (0 at the centre itself)
    void colliderDual() {
        if (colSdf.empty()) return;
        int c = cur;
        std::vector<double>& DT = dual[c][1];
        for (int s = 0; s < S; ++s) {
            if (sflag[s] & F_GHOST) continue;
            V3 pos = vertPos(s);
            if (!insideSdf(bsdf(pos))) continue;
            V3 n = pos - colCentre;
            V3 v = v3(DT[3 * s], DT[3 * s + 1], DT[3 * s + 2]);
            V3 t = norm3(n) < DBL_EPSILON ? v3(0, 0, 0) : tangential(v, n);
            DT[3 * s] = t.x;
            DT[3 * s + 1] = t.y;
            DT[3 * s + 2] = t.z;
        }
    }

    // ---------------------------------------------------------------- positions
    V3 cellPos(int s) const { double h = dh(slev[s]); return v3(sx[s] * h + 0.5 * h, sy[s] * h + 0.5 * h, sz[s] * h + 0.5 * h); }
    V3 vertPos(int s) const { double h = dh(slev[s]); return v3(sx[s] * h, sy[s] * h, sz[s] * h); }
    V3 macPos(int a, int s) const {
        double h = dh(slev[s]);
        V3 p = v3(sx[s] * h + 0.5 * h, sy[s] * h + 0.5 * h, sz[s] * h + 0.5 * h);
        p[a] = (a == 0 ? sx[s] : (a == 1 ? sy[s] : sz[s])) * h + 0.0 * h;
        return p;
    }
    // include/octree_omni_tilt_grid3.h:35-42
    static V3 tiltPos(V3 c, int dir, double e) {
        int m = dir & 3;
        double tz = (dir < 4 ? 1 : -1) * e / 3.0;
        double ty = (m < 2 ? 1 : -1) * e / 3.0;
        double tx = ((m == 0 || m == 3) ? 1 : -1) * e / 3.0;
        return v3(c.x + tx, c.y + ty, c.z + tz);
    }

    // ---------------------------------------------------------------- sampling
    // cell-centred trilinear sample, include/octree_cell_centered_grid3.h:97-123
    template <class T, class G>
    T cellSample(const G& get, V3 p) {
        int l = levelCoordinate(p.x, p.y, p.z);
        double h = dh(l);
        int r = lres[l];
        int xi, yi, zi;
        double fx, fy, fz;
        bary(p.x / h - 0.5, 0, r - 2, &xi, &fx);
        bary(p.y / h - 0.5, 0, r - 2, &yi, &fy);
        bary(p.z / h - 0.5, 0, r - 2, &zi, &fz);
        int x1 = std::min(xi + 1, r - 2), y1 = std::min(yi + 1, r - 2), z1 = std::min(zi + 1, r - 2);
        return trilerp(get(slotReq(l, xi, yi, zi)), get(slotReq(l, x1, yi, zi)), get(slotReq(l, xi, y1, zi)),
                       get(slotReq(l, x1, y1, zi)), get(slotReq(l, xi, yi, z1)), get(slotReq(l, x1, yi, z1)),
                       get(slotReq(l, xi, y1, z1)), get(slotReq(l, x1, y1, z1)), fx, fy, fz);
    }

    // include/octree_util.h:117-185
    template <class T, class GO, class GT>
    void neighborCube(int l, int xi, int yi, int zi, int dir, T* v, const GO& oct, const GT& til,
                      const std::vector<TiltE>& te, bool tj) {
        int reDir = ((dir & 1) ? 8 : 6) - dir;
        T c = oct(slotReq(l, xi, yi, zi));
        v[reDir] = c;
        for (int i = 0; i < 8; ++i) {
            int mk = SAMPLE_MARKER[dir][i];
            if (mk == 0x1000) continue;
            T t = c;
            double count = 1;
            int m[3] = {(mk >> 8) & 0xf, (mk >> 4) & 0xf, mk & 0xf};
            if (tj && l > 0) {
                bool flag = false;
                for (int k = 0; k < 3; ++k) {
                    if (m[k] != 0 && m[(k + 1) % 3] == 0 && m[(k + 2) % 3] == 0) {
                        int id[3] = {xi, yi, zi};
                        id[k] += (m[k] == 1);
                        id[0] *= 2; id[1] *= 2; id[2] *= 2;
                        id[(k + 1) % 3] += 1;
                        id[(k + 2) % 3] += 1;
                        int s = slotOf(l - 1, id[0], id[1], id[2]);
                        if (s >= 0 && te[s].half) { v[i] = til(s); flag = true; }
                    }
                    if (m[k] == 0 && m[(k + 1) % 3] != 0 && m[(k + 2) % 3] != 0) {
                        int id[3] = {(xi << 1) + (dir == 0 || dir == 3 || dir == 4 || dir == 7), (yi << 1) + ((dir % 4) < 2),
                                     (zi << 1) + (dir < 4)};
                        int tx = id[0] + OCT_NB_TILT[i][0], ty = id[1] + OCT_NB_TILT[i][1], tz = id[2] + OCT_NB_TILT[i][2];
                        int s = slotOf(l - 1, tx, ty, tz);
                        if (s >= 0 && !(sflag[s] & F_GHOST)) {
                            if (te[s].closedByT) { v[i] = til(s); flag = true; }
                        }
                    }
                }
                if (flag) continue;
            }
            int r2 = lres[l] - 2;
            for (int x = -(m[0] == 2); x <= (m[0] == 1); ++x)
                for (int y = -(m[1] == 2); y <= (m[1] == 1); ++y)
                    for (int z = -(m[2] == 2); z <= (m[2] == 1); ++z) {
                        if (x == 0 && y == 0 && z == 0) continue;
                        int cx = std::min(std::max(0, xi + x), r2), cy = std::min(std::max(0, yi + y), r2),
                            cz = std::min(std::max(0, zi + z), r2);
                        t = t + oct(slotReq(l, cx, cy, cz));
                        count += 1;
                    }
            v[i] = t / count;
        }
    }

    // include/octree_omni_grid3.h:243-286
    template <class T, class GO, class GT>
    T omniSampleSub(V3 p, const GO& oct, const GT& til, const std::vector<TiltE>& te) {
        int l = levelCoordinate(p.x, p.y, p.z);
        double h = dh(l);
        int r = lres[l];
        double rx = p.x / h, ry = p.y / h, rz = p.z / h;
        int xi, yi, zi;
        double fx, fy, fz;
        bary(rx, 0, r - 1, &xi, &fx);
        bary(ry, 0, r - 1, &yi, &fy);
        bary(rz, 0, r - 1, &zi, &fz);
        int dir = fz >= 0.5 ? 0 : 4;
        dir += (fx >= 0.5) ? (fy >= 0.5 ? 0 : 3) : (fy >= 0.5 ? 1 : 2);
        int ts = slotReq(l, xi + OCT_NB_TILT[dir][0], yi + OCT_NB_TILT[dir][1], zi + OCT_NB_TILT[dir][2]);
        const TiltE& tn = te[ts];
        if (!tn.half && !tn.closedByT && tn.closed) {
            // sampleGivenRelativePosition, include/octree_cell_centered_grid3.h:158-179
            int a, bb, c;
            double ga, gb, gc;
            bary(rx - 0.5, 0, r - 2, &a, &ga);
            bary(ry - 0.5, 0, r - 2, &bb, &gb);
            bary(rz - 0.5, 0, r - 2, &c, &gc);
            int a1 = std::min(a + 1, r - 2), b1 = std::min(bb + 1, r - 2), c1 = std::min(c + 1, r - 2);
            return trilerp(oct(slotReq(l, a, bb, c)), oct(slotReq(l, a1, bb, c)), oct(slotReq(l, a, b1, c)),
                           oct(slotReq(l, a1, b1, c)), oct(slotReq(l, a, bb, c1)), oct(slotReq(l, a1, bb, c1)),
                           oct(slotReq(l, a, b1, c1)), oct(slotReq(l, a1, b1, c1)), ga, gb, gc);
        }
        T v[8];
        v[dir] = til(ts);
        neighborCube<T>(l, xi, yi, zi, dir, v, oct, til, te, tn.tjoint);
        switch (dir) {
            case 0: fx -= 0.5, fy -= 0.5, fz -= 0.5; break;
            case 1: fy -= 0.5, fz -= 0.5; break;
            case 2: fz -= 0.5; break;
            case 3: fx -= 0.5, fz -= 0.5; break;
            case 4: fx -= 0.5, fy -= 0.5; break;
            case 5: fy -= 0.5; break;
            case 6: break;
            case 7: fx -= 0.5; break;
        }
        fx *= 2; fy *= 2; fz *= 2;
        return trilerp(v[6], v[7], v[5], v[4], v[2], v[3], v[1], v[0], fx, fy, fz);
    }

    // the level-transition test shared by the scalar and velocity samplers
    // (include/octree_omni_grid3.h:172-175, include/octree_omni_face_centered_grid3.h:61-64)
    bool nearTransition(int l, int xi, int yi, int zi) {
        if (isGhostNode(l, xi, yi, zi)) return true;
        if (l == 0 && get(1, xi >> 1, yi >> 1, zi >> 1) >= 0) return true;
        if (l == 1 && get(0, (xi << 1) + 1, (yi << 1) + 1, (zi << 1) + 1) >= 0) return true;
        if (l == 1 && get(0, xi << 1, yi << 1, zi << 1) >= 0) return true;
        return false;
    }

    // include/octree_omni_grid3.h:147-187 (OCTREE_CORRECTION_BASED)
    double scalarSample(V3 p, const std::vector<double>& oct, const std::vector<double>& til, const std::vector<TiltE>& te) {
        int l = levelCoordinate(p.x, p.y, p.z);
        double h = dh(l);
        int r = lres[l];
        int xi, yi, zi;
        double fx, fy, fz;
        bary(p.x / h - 0.5, 0, r - 2, &xi, &fx);
        bary(p.y / h - 0.5, 0, r - 2, &yi, &fy);
        bary(p.z / h - 0.5, 0, r - 2, &zi, &fz);
        int x1 = std::min(xi + 1, r - 2), y1 = std::min(yi + 1, r - 2), z1 = std::min(zi + 1, r - 2);
        double o000 = oct[slotReq(l, xi, yi, zi)], o100 = oct[slotReq(l, x1, yi, zi)], o010 = oct[slotReq(l, xi, y1, zi)],
               o110 = oct[slotReq(l, x1, y1, zi)], o001 = oct[slotReq(l, xi, yi, z1)], o101 = oct[slotReq(l, x1, yi, z1)],
               o011 = oct[slotReq(l, xi, y1, z1)], o111 = oct[slotReq(l, x1, y1, z1)];
        double ret = trilerp(o000, o100, o010, o110, o001, o101, o011, o111, fx, fy, fz);
        int ts = slotReq(l, xi + 1, yi + 1, zi + 1);
        if (nearTransition(l, xi, yi, zi)) {
            auto go = [&](int s) { return oct[s]; };
            auto gt = [&](int s) { return til[s]; };
            return omniSampleSub<double>(p, go, gt, te);
        }
        const TiltE& tn = te[ts];
        if (tn.closed && !tn.half) return ret;
        double diff = til[ts] - (1 / 8.0) * (o000 + o100 + o010 + o110 + o001 + o101 + o011 + o111);
        double mn = std::min(std::min(std::min(fx, fy), fz), std::min(std::min(1 - fx, 1 - fy), 1 - fz));
        return ret + diff * 2.0 * mn;
    }

    // include/octree_face_centered_grid3.h / src/octree_face_centered_grid3.cpp:36-121
    double macSampleAxis(int a, int l, double rx, double ry, double rz, const std::vector<double>& u) {
        int r = lres[l];
        double q[3] = {rx, ry, rz};
        int id[3], id1[3];
        double f[3];
        for (int k = 0; k < 3; ++k) {
            if (k == a) {
                bary(q[k], 0, r - 1, &id[k], &f[k]);
                id1[k] = std::min(id[k] + 1, r - 1);
            } else {
                bary(q[k] - 0.5, 0, r - 2, &id[k], &f[k]);
                id1[k] = std::min(id[k] + 1, r - 2);
            }
        }
        auto g = [&](int x, int y, int z) { return u[slotReq(l, x, y, z)]; };
        return trilerp(g(id[0], id[1], id[2]), g(id1[0], id[1], id[2]), g(id[0], id1[1], id[2]), g(id1[0], id1[1], id[2]),
                       g(id[0], id[1], id1[2]), g(id1[0], id[1], id1[2]), g(id[0], id1[1], id1[2]),
                       g(id1[0], id1[1], id1[2]), f[0], f[1], f[2]);
    }
    V3 macSample(V3 p, std::vector<double>* U) {
        int l = levelCoordinate(p.x, p.y, p.z);
        double h = dh(l);
        double rx = p.x / h, ry = p.y / h, rz = p.z / h;
        return v3(macSampleAxis(0, l, rx, ry, rz, U[0]), macSampleAxis(1, l, rx, ry, rz, U[1]),
                  macSampleAxis(2, l, rx, ry, rz, U[2]));
    }
    double macSampleOne(int a, V3 p, std::vector<double>* U) {
        int l = levelCoordinate(p.x, p.y, p.z);
        double h = dh(l);
        return macSampleAxis(a, l, p.x / h, p.y / h, p.z / h, U[a]);
    }

    // include/octree_omni_face_centered_grid3.h:37-80 (velocity of buffer b)
    V3 velSample(V3 p, int bf) {
        const std::vector<TiltE>& te = tiltE[bf];
        int l = levelCoordinate(p.x, p.y, p.z);
        double h = dh(l);
        int r = lres[l];
        int id[3];
        double f[3];
        bary_vec(p.x / h - 0.5, r - 1, &id[0], &f[0]);
        bary_vec(p.y / h - 0.5, r - 1, &id[1], &f[1]);
        bary_vec(p.z / h - 0.5, r - 1, &id[2], &f[2]);
        int ts = slotReq(l, id[0] + 1, id[1] + 1, id[2] + 1);
        if (nearTransition(l, id[0], id[1], id[2])) {
            const std::vector<double>& DO = dual[bf][0];
            const std::vector<double>& DT = dual[bf][1];
            auto go = [&](int s) { return v3(DO[3 * s], DO[3 * s + 1], DO[3 * s + 2]); };
            auto gt = [&](int s) { return v3(DT[3 * s], DT[3 * s + 1], DT[3 * s + 2]); };
            return omniSampleSub<V3>(p, go, gt, te);
        }
        V3 v = macSample(p, mac[bf]);
        const TiltE& tn = te[ts];
        if (!tn.half && tn.closed) return v;
        const std::vector<double>& DT = dual[bf][1];
        V3 dt = v3(DT[3 * ts], DT[3 * ts + 1], DT[3 * ts + 2]);
        V3 diff = dt - macSample(vertPos(ts), mac[bf]);
        double mn = std::min(std::min(std::min(f[0], f[1]), f[2]), std::min(std::min(1 - f[0], 1 - f[1]), 1 - f[2]));
        return v + diff * 2 * mn;
    }

    // include/advection.h:49-62: RK2 midpoint, then the boundary clamp: when the SDF changes sign
    // between p and the traced point, the point moves back toward p by |phi1| / (|phi0| + |phi1|)
    V3 backTrace(V3 p, double dt, int bf) {
        V3 mid = p - velSample(p, bf) * dt * 0.5;
        V3 ret = p - velSample(mid, bf) * dt;
        double phi0 = bsdf(p), phi1 = bsdf(ret);
        if (phi0 * phi1 < 0.0) {
            double w = std::fabs(phi1) / (std::fabs(phi0) + std::fabs(phi1));
            return v3(w * p.x + (1.0 - w) * ret.x, w * p.y + (1.0 - w) * ret.y, w * p.z + (1.0 - w) * ret.z);
        }
        return ret;
    }

    // ---------------------------------------------------------------- ghost updates
    // OctreeCellCenteredGrid3<T>::updateGhost, include/octree_cell_centered_grid3.h:184-208
    template <class T, class GO, class SO>
    void cellGhost(const GO& get_, const SO& set_) {
        for (int l = 0; l < L; ++l)
            for (int i = lN[l]; i < lN[l] + lG[l]; ++i) {
                int s = loff[l] + i;
                if (sflag[s] & F_FROM_COARSE) continue;
                int x = sx[s] << 1, y = sy[s] << 1, z = sz[s] << 1;
                T v{};
                for (int a = 0; a <= 1; ++a)
                    for (int bb = 0; bb <= 1; ++bb)
                        for (int c = 0; c <= 1; ++c) v = v + get_(slotReq(l - 1, x + a, y + bb, z + c));
                set_(s, v * (1 / 8.0));
            }
        for (int l = 0; l < L; ++l)
            for (int i = lN[l]; i < lN[l] + lG[l]; ++i) {
                int s = loff[l] + i;
                if (!(sflag[s] & F_FROM_COARSE)) continue;
                set_(s, cellSample<T>(get_, cellPos(s)));
            }
    }

    // OctreeVertexCenteredGrid3<T>::updateGhost, include/octree_vertex_centered_grid3.h:129-153,
    // skipping half tilts (update_ghost_exclude_half_tilt, include/base_octree_omni_grid.h:20-28)
    template <class T, class GT, class ST>
    void vertexGhost(const GT& get_, const ST& set_, const std::vector<TiltE>& te) {
        for (int l = 0; l < L; ++l)
            for (int i = lN[l]; i < lN[l] + lG[l]; ++i) {
                int s = loff[l] + i;
                // half-tilt slots keep their value (saved and restored around the pass)
                if (isHalfTiltSlot(s)) continue;
                int x = sx[s], y = sy[s], z = sz[s];
                if (sflag[s] & F_FROM_COARSE) {
                    T v{};
                    int count = 0;
                    for (int a = 0; a <= (x & 1); ++a)
                        for (int bb = 0; bb <= (y & 1); ++bb)
                            for (int c = 0; c <= (z & 1); ++c) {
                                int t = getUntil(l + 1, (x >> 1) + a, (y >> 1) + bb, (z >> 1) + c, true);
                                if (t >= 0) { v = v + get_(t); count += 1; }
                            }
                    set_(s, v * (1.0 / (count + EPS)));
                } else {
                    int t = getUntil(l - 1, x << 1, y << 1, z << 1, true);
                    if (t < 0) throw std::runtime_error("oracle: vertex ghost without source");
                    set_(s, get_(t));
                }
            }
    }
    std::vector<uint8_t> halfMark;
    bool isHalfTiltSlot(int s) const { return halfMark[s]; }

    // getTiltFromOctagonNeighbor3, include/octree_util.h:103-121
    template <class T, class GO>
    T tiltFromOct(int l, int x, int y, int z, const GO& get_) {
        T v = get_(slotReq(l, x, y, z));
        double count = 1;
        for (int m = -1; m <= 0; ++m)
            for (int n = -1; n <= 0; ++n)
                for (int k = -1; k <= 0; ++k) {
                    if (m == 0 && n == 0 && k == 0) continue;
                    if (octValid(l, x + m, y + n, z + k) && get(l, x + m, y + n, z + k) >= 0) {
                        v = v + get_(slotOf(l, x + m, y + n, z + k));
                        count += 1;
                    }
                }
        return v / count;
    }

    // OctreeOmniGrid3<T>::updateGhost, include/octree_omni_grid3.h:136-143 and :289-337
    template <class T, class GO, class SO, class GT, class ST>
    void omniGhost(const GO& go, const SO& so, const GT& gt, const ST& st, const std::vector<TiltE>& te) {
        cellGhost<T>(go, so);
        vertexGhost<T>(gt, st, te);
        // updateCellGhost
        for (int l = 0; l < L; ++l)
            for (int i = lN[l]; i < lN[l] + lG[l]; ++i) {
                int s = loff[l] + i;
                if (!octValid(l, sx[s], sy[s], sz[s])) continue;
                if (!(sflag[s] & F_FROM_COARSE)) continue;
                int x = sx[s], y = sy[s], z = sz[s];
                int dp = slotReq(l, x + (x & 1), y + (y & 1), z + (z & 1));
                so(s, (gt(dp) + go(slotReq(l + 1, x >> 1, y >> 1, z >> 1))) * 0.5);
            }
        // interpolateClosedJoint
        for (int tj : tJoints) {
            int l = slev[tj], x = sx[tj], y = sy[tj], z = sz[tj];
            if (te[tj].e < dh(l)) { l -= 1; x <<= 1; y <<= 1; z <<= 1; }
            for (int i = 0; i < 6; ++i) {
                int tx = x + OCT_NB[i][0], ty = y + OCT_NB[i][1], tz = z + OCT_NB[i][2];
                int t = slotOf(l, tx, ty, tz);
                if (t >= 0) st(t, tiltFromOct<T>(l, tx, ty, tz, go));
            }
        }
        for (int cs : closedByHalf) {
            if (te[cs].closed && te[cs].dir == -1) st(cs, tiltFromOct<T>(slev[cs], sx[cs], sy[cs], sz[cs], go));
        }
    }

    void scalarGhost(std::vector<double>& oct, std::vector<double>& til, const std::vector<TiltE>& te) {
        auto go = [&](int s) { return oct[s]; };
        auto so = [&](int s, double v) { oct[s] = v; };
        auto gt = [&](int s) { return til[s]; };
        auto st = [&](int s, double v) { til[s] = v; };
        omniGhost<double>(go, so, gt, st, te);
    }
    void dualGhost(int bf) {
        std::vector<double>& DO = dual[bf][0];
        std::vector<double>& DT = dual[bf][1];
        auto go = [&](int s) { return v3(DO[3 * s], DO[3 * s + 1], DO[3 * s + 2]); };
        auto so = [&](int s, V3 v) { DO[3 * s] = v.x; DO[3 * s + 1] = v.y; DO[3 * s + 2] = v.z; };
        auto gt = [&](int s) { return v3(DT[3 * s], DT[3 * s + 1], DT[3 * s + 2]); };
        auto st = [&](int s, V3 v) { DT[3 * s] = v.x; DT[3 * s + 1] = v.y; DT[3 * s + 2] = v.z; };
        omniGhost<V3>(go, so, gt, st, tiltE[bf]);
    }

    // OctreeOmniFaceCenteredGrid3::updateGhost, include/octree_omni_face_centered_grid3.h:97-120
    void velocityGhost(int bf) {
        std::vector<double>* U = mac[bf];
        for (int s = 0; s < S; ++s)
            if (sflag[s] & F_GHOST) U[0][s] = U[1][s] = U[2][s] = 0;
        for (int l = 0; l < L; ++l)
            for (int i = lN[l]; i < lN[l] + lG[l]; ++i) {
                int s = loff[l] + i;
                if (sflag[s] & F_FROM_COARSE) continue;
                for (int a = 0; a < 3; ++a) U[a][s] = macSampleOne(a, macPos(a, s), U);
            }
        // updateGhostFromHalfTilt, src/octree_omni_face_centered_grid3.cpp:162-173
        for (int hs : halfTilts) {
            const TiltE& n = tiltE[bf][hs];
            int a = n.dir % 3;
            int t = slotReq(slev[hs] + 1, sx[hs] >> 1, sy[hs] >> 1, sz[hs] >> 1);
            U[a][t] = tv[bf][(size_t)hs * 8 + HALF_SLOT[n.dir][4]];
        }
        for (int l = 0; l < L; ++l)
            for (int i = lN[l]; i < lN[l] + lG[l]; ++i) {
                int s = loff[l] + i;
                if (!(sflag[s] & F_FROM_COARSE)) continue;
                for (int a = 0; a < 3; ++a) U[a][s] = macSampleOne(a, macPos(a, s), U);
            }
        // OctreeOmniTiltGrid3::updateGhost, include/octree_omni_tilt_grid3.h:56-74
        std::vector<double>& T8 = tv[bf];
        for (int l = 0; l < L; ++l)
            for (int i = lN[l]; i < lN[l] + lG[l]; ++i) {
                int s = loff[l] + i;
                if (tiltE[bf][s].half) continue;
                int x = sx[s], y = sy[s], z = sz[s];
                int src = -1;
                if (sflag[s] & F_FROM_COARSE) {
                    if ((x & 1) || (y & 1) || (z & 1)) {
                        for (int k = 0; k < 8; ++k) T8[(size_t)s * 8 + k] = 0;
                        continue;
                    }
                    src = slotReq(l + 1, x >> 1, y >> 1, z >> 1);
                } else {
                    src = slotReq(l - 1, x << 1, y << 1, z << 1);
                }
                for (int k = 0; k < 8; ++k) T8[(size_t)s * 8 + k] = T8[(size_t)src * 8 + k];
            }
    }

    // ---------------------------------------------------------------- step stages
    bool inSrc(V3 p) const { return astg_scene::inside(P.src, p.x, p.y, p.z); }

    // sphere source as in example/octree_smoke_3d/main.cpp:23-86 (density = heat = 1, w = 1)
    void source() {
        const double initV = 1.0;
        int c = cur;
        for (int s = 0; s < S; ++s) {
            if (sflag[s] & F_GHOST) continue;
            if (inSrc(cellPos(s))) { dO[c][s] = 1; hO[c][s] = 1; }
        }
        for (int s = 0; s < S; ++s) {
            if (sflag[s] & F_GHOST) continue;
            if (inSrc(vertPos(s))) { dT[c][s] = 1; hT[c][s] = 1; }
        }
        for (int hs : halfTilts)
            if (inSrc(vertPos(hs))) { dT[c][hs] = 1; hT[c][hs] = 1; }
        for (int s = 0; s < S; ++s) {
            if (sflag[s] & F_GHOST) continue;
            if (inSrc(macPos(2, s))) mac[c][2][s] = initV;
            if (inSrc(vertPos(s)))
                for (int k = 0; k < 8; ++k) tv[c][(size_t)s * 8 + k] = initV * INV_SQRT3;
        }
        for (int hs : halfTilts) {
            if (!inSrc(vertPos(hs))) continue;
            double nv[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            const TiltE& n = tiltE[cur][hs];
            for (int i = 0; i < 4; ++i) nv[HALF_SLOT[n.dir][i]] = initV * INV_SQRT3;
            if (n.dir % 3 == 2) nv[HALF_SLOT[n.dir][4]] = initV;
            for (int k = 0; k < 8; ++k) tv[c][(size_t)hs * 8 + k] = nv[k];
        }
        if (firstSource) {
            scalarGhost(dO[c], dT[c], tiltE[c]);
            scalarGhost(hO[c], hT[c], tiltE[c]);
            firstSource = false;
        }
    }

    // initial curl noise (same definition as the fixture harness)
    void initNoise() {
        astg_scene::CurlNoise cn(P.seed, P.noise);
        int c = cur;
        for (int s = 0; s < S; ++s) {
            if (sflag[s] & F_GHOST) continue;
            for (int a = 0; a < 3; ++a) {
                if (!macValid(a, slev[s], sx[s], sy[s], sz[s])) continue;
                V3 p = macPos(a, s);
                double pp[3] = {p.x, p.y, p.z}, u[3];
                cn.velocity(pp, u);
                mac[c][a][s] = u[a];
            }
            if (tOpen[s]) {
                for (int k = 0; k < 8; ++k) {
                    V3 p = tiltPos(vertPos(s), k, tiltE[c][s].e);
                    double pp[3] = {p.x, p.y, p.z}, u[3];
                    cn.velocity(pp, u);
                    tv[c][(size_t)s * 8 + k] = dot3(v3(u[0], u[1], u[2]), v3(tilt_up(k, 0), tilt_up(k, 1), tilt_up(k, 2)));
                }
            }
        }
        for (int hs : halfTilts) {
            double nv[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            const TiltE& n = tiltE[c][hs];
            for (int i = 0; i < 5; ++i) {
                int k = HALF_SLOT[n.dir][i];
                V3 p = (i == 4) ? vertPos(hs) : tiltPos(vertPos(hs), k, n.e);
                double pp[3] = {p.x, p.y, p.z}, u[3];
                cn.velocity(pp, u);
                V3 d = (i == 4) ? v3(HALF_DIR_POS[k][0], HALF_DIR_POS[k][1], HALF_DIR_POS[k][2])
                                : v3(tilt_up(k, 0), tilt_up(k, 1), tilt_up(k, 2));
                nv[k] = dot3(v3(u[0], u[1], u[2]), d);
            }
            for (int k = 0; k < 8; ++k) tv[c][(size_t)hs * 8 + k] = nv[k];
        }
    }

    // src/octree_omnigrid_solver3.cpp:917-972
    void addForce(double dt) {
        int c = cur;
        double amb = 0;
        long long count = 0;
        for (int l = 0; l < L; ++l) {
            const double* h = &hO[c][loff[l]];
            size_t nl = lN[l] + lG[l];
            double sum = P.reduceMode == 0 ? refSum(h, nl, P.refWorkers) : treeReduce(nl, [&](double acc, size_t i) { return acc + h[i]; });
            amb += sum * (l == 0 ? 1 : 8);
            count += (long long)(lN[l] + lG[l]) * (l == 0 ? 1 : 8);
        }
        amb /= (double)count;
        ambT = amb;
        const std::vector<TiltE>& te = tiltE[c];
        auto force = [&](V3 p) {
            return P.buoyD * scalarSample(p, dO[c], dT[c], te) + P.buoyT * (scalarSample(p, hO[c], hT[c], te) - amb);
        };
#pragma omp parallel for schedule(dynamic, 256)
        for (int s = 0; s < S; ++s) {
            if (sflag[s] & F_GHOST) continue;
            if (macValid(2, slev[s], sx[s], sy[s], sz[s])) mac[c][2][s] = mac[c][2][s] + dt * force(macPos(2, s));
        }
#pragma omp parallel for schedule(dynamic, 256)
        for (int s = 0; s < S; ++s) {
            if (sflag[s] & F_GHOST) continue;
            if (!tOpen[s]) continue;
            double nf[8];
            for (int k = 0; k < 8; ++k) nf[k] = tilt_up(k, 2) * force(tiltPos(vertPos(s), k, te[s].e));
            for (int k = 0; k < 8; ++k) tv[c][(size_t)s * 8 + k] = tv[c][(size_t)s * 8 + k] + dt * nf[k];
        }
        for (int hs : halfTilts) {
            double nf[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            const TiltE& n = te[hs];
            for (int i = 0; i < 5; ++i) {
                int k = HALF_SLOT[n.dir][i];
                V3 p = (i == 4) ? vertPos(hs) : tiltPos(vertPos(hs), k, n.e);
                double tf = force(p);
                V3 d = (i == 4) ? v3(HALF_DIR_POS[k][0], HALF_DIR_POS[k][1], HALF_DIR_POS[k][2])
                                : v3(tilt_up(k, 0), tilt_up(k, 1), tilt_up(k, 2));
                nf[k] = dot3(v3(0, 0, tf), d);
            }
            for (int k = 0; k < 8; ++k) tv[c][(size_t)hs * 8 + k] = tv[c][(size_t)hs * 8 + k] + dt * nf[k];
        }
    }

    // OmniBoundarySolver3::constrainVelocity(MAC), include/omni_boundary_solver3.h:73-162: the
    // collider part never triggers; walls zero the normal faces on every level (ghosts too)
    void constrainWalls() {
        int c = cur;
        for (int s = 0; s < S; ++s) {
            int l = slev[s], r = lres[l];
            if ((P.closedMask & 1) && sx[s] == r - 1) mac[c][0][s] = 0;
            if ((P.closedMask & 2) && sx[s] == 0) mac[c][0][s] = 0;
            if ((P.closedMask & 4) && sy[s] == r - 1) mac[c][1][s] = 0;
            if ((P.closedMask & 8) && sy[s] == 0) mac[c][1][s] = 0;
            if ((P.closedMask & 16) && sz[s] == r - 1) mac[c][2][s] = 0;
            if ((P.closedMask & 32) && sz[s] == 0) mac[c][2][s] = 0;
        }
    }
    bool closedDomain(int i) const { return (P.closedMask >> i) & 1; }

    // src/octree_omnigrid_solver3.cpp:292-347 (sequential numbering in iterator order)
    void updateIndex() {
        int n = 0;
        // a DOF only where the SDF at its position exceeds -3 dx_l (:297-309, threshold 3)
        auto fluid = [&](int s, const V3& p) { return bsdf(p) > -dh(slev[s]) * 3.0; };
        for (int s = 0; s < S; ++s) {
            if (sflag[s] & F_GHOST) continue;
            pO[s] = octValid(slev[s], sx[s], sy[s], sz[s]) && fluid(s, cellPos(s)) ? n++ : -1;
            pT[s] = tOpen[s] && fluid(s, vertPos(s)) ? n++ : -1;
        }
        for (int s = 0; s < S; ++s)
            if (sflag[s] & F_GHOST) { pO[s] = -1; pT[s] = -1; }
        for (int hs : halfTilts) pT[hs] = fluid(hs, vertPos(hs)) ? n++ : -1;
        // OctreeVertexCenteredGrid3<int>::updateGhost, src/octree_vertex_centered_grid3.cpp:47-64
        for (int l = 0; l < L; ++l)
            for (int i = lN[l]; i < lN[l] + lG[l]; ++i) {
                int s = loff[l] + i;
                int x = sx[s], y = sy[s], z = sz[s];
                if (sflag[s] & F_FROM_COARSE) {
                    if ((x & 1) || (y & 1) || (z & 1)) continue;
                    pT[s] = pT[slotReq(l + 1, x >> 1, y >> 1, z >> 1)];
                } else {
                    pT[s] = pT[slotReq(l - 1, x << 1, y << 1, z << 1)];
                }
            }
        nDof = n;
    }

    // tiltNeighborOctagon3, src/octree_util.cpp:172-194.  The reference returns a packed level
    // coordinate (or -1); the coordinate may name a cell that is not in the layout when it is
    // outside the octagon-valid range, so the coordinate itself is returned here.
    struct NbOct {
        bool some;
        int l, x, y, z;
    };
    void tiltNbOct(int l, int x, int y, int z, NbOct out[8]) {
        for (int i = 0; i < 8; ++i) {
            out[i].some = false;
            int nx = x + TILT_NB_OCT[i][0], ny = y + TILT_NB_OCT[i][1], nz = z + TILT_NB_OCT[i][2];
            if (!layValid(l, nx, ny, nz)) continue;
            int c = getUntil(l, nx, ny, nz, true);
            if (c < 0) c = getUntil(l, nx, ny, nz, false);
            if (c < 0) continue;
            int tl = slev[c], tx = sx[c], ty = sy[c], tz = sz[c];
            if (tl < l) {
                int m = i % 4;
                tz += i >= 4 ? 1 : 0;
                ty += m >= 2 ? 1 : 0;
                tx += (m == 1 || m == 2) ? 1 : 0;
            }
            out[i] = NbOct{true, tl, tx, ty, tz};
        }
    }

    int pOctAt(int l, int x, int y, int z) {  // pIndex->getOctagon(l, x, y, z)
        int s = slotOf(l, x, y, z);
        if (s < 0) throw std::runtime_error("oracle: pIndex lookup outside the layout");
        return pO[s];
    }

    // src/octree_omnigrid_solver3.cpp:350-653
    void assemble(double dt) {
        int c = cur;
        const std::vector<TiltE>& te = tiltE[c];
        A.reset(nDof);
        b.assign(nDof, 0.0);
#pragma omp parallel for schedule(dynamic, 256)
        for (int s = 0; s < S; ++s) {
            if (sflag[s] & F_GHOST) continue;
            int ci = pO[s];
            int l = slev[s], x = sx[s], y = sy[s], z = sz[s];
            if (ci < 0 || !octValid(l, x, y, z)) continue;
            double h = dh(l);
            double center = 0, tb = 0, tC = 0, tK = 0;
            for (int i = 0; i < 6; ++i) {
                int axis = i / 2;
                int nx = x + OCT_NB[i][0], ny = y + OCT_NB[i][1], nz = z + OCT_NB[i][2];
                if (octValid(l, nx, ny, nz) && isGhostNode(l, nx, ny, nz)) continue;
                double area = h * h;
                for (int m = 0; m <= 1; ++m)
                    for (int n = 0; n <= 1; ++n) {
                        int t[3] = {x, y, z};
                        t[axis] += (i & 1) ? 0 : 1;
                        t[(axis + 1) % 3] += m;
                        t[(axis + 2) % 3] += n;
                        const TiltE& tn = te[slotReq(l, t[0], t[1], t[2])];
                        area -= tn.e * tn.e * 0.5;
                    }
                int fs = slotReq(l, x + OCT_NB_FACE[i][0], y + OCT_NB_FACE[i][1], z + OCT_NB_FACE[i][2]);
                if (octValid(l, nx, ny, nz)) {
                    double term = wMac[axis][fs];
                    int ti = pOctAt(l, nx, ny, nz);
                    if (ti >= 0) {
                        tC = term * area / h;
                        tK = area * term;
                        A.set(ci, ti, -tC);
                    } else { tC = 0; tK = 0; }
                } else if (closedDomain(i)) {
                    tC = 0; tK = 0;
                } else {
                    tK = area;
                    tC = tK / h;
                }
                center += tC;
                tb += ((i & 1) ? 1 : -1) * tK * mac[c][axis][fs];
            }
            for (int i = 0; i < 8; ++i) {
                int ns = slotReq(l, x + OCT_NB_TILT[i][0], y + OCT_NB_TILT[i][1], z + OCT_NB_TILT[i][2]);
                const TiltE& e = te[ns];
                int re = ((i & 1) ? 8 : 6) - i;
                if (!e.closed || e.half) {
                    double area = e.e * e.e * SQRT3 * 0.5;
                    double term = wTilt[(size_t)ns * 8 + re];
                    int ti = pT[ns];
                    if (ti >= 0) {
                        tC = term * area / (h * SQRT3 * 0.5);
                        tK = area * term;
                        A.add(ci, ti, -tC);
                    } else { tC = 0; tK = 0; }
                    center += tC;
                    tb += (i < 4 ? -1 : 1) * tK * tv[c][(size_t)ns * 8 + re];
                }
            }
            if (std::fabs(center) < EPS) { center = 1; tb = 0; }
            A.set(ci, ci, center);
            b[ci] = tb;
        }
#pragma omp parallel for schedule(dynamic, 256)
        for (int s = 0; s < S; ++s) {
            if (sflag[s] & F_GHOST) continue;
            int ci = pT[s];
            if (!tOpen[s] || ci < 0) continue;
            int l = slev[s], x = sx[s], y = sy[s], z = sz[s];
            const TiltE& e = te[s];
            double center = 0, tb = 0, tC = 0, tK = 0;
            const double* u = &tv[c][(size_t)s * 8];
            const double* tw = &wTilt[(size_t)s * 8];
            NbOct nb[8];
            tiltNbOct(l, x, y, z, nb);
            double area = e.e * e.e * SQRT3 * 0.5;
            for (int i = 0; i < 8; ++i) {
                if (!nb[i].some) {
                    if (!octValid(l, x + TILT_NB_OCT[i][0], y + TILT_NB_OCT[i][1], z + TILT_NB_OCT[i][2])) {
                        tC = area / (dh(l) * SQRT3 / 3.0);
                        tK = area;
                        center += tC;
                        tb += (i < 4 ? -1 : 1) * tK * u[i];
                    }
                    continue;
                }
                int nl = nb[i].l;
                if (octValid(nl, nb[i].x, nb[i].y, nb[i].z)) {
                    double h2 = dh(nl);
                    int ti = pOctAt(nl, nb[i].x, nb[i].y, nb[i].z);
                    if (ti >= 0) {
                        tC = tw[i] * area / (h2 * SQRT3 * 0.5);
                        tK = area * tw[i];
                        A.set(ci, ti, -tC);
                    } else { tC = 0; tK = 0; }
                } else {
                    tC = area / (dh(l) * SQRT3 / 3.0);
                    tK = area;
                }
                center += tC;
                tb += (i < 4 ? -1 : 1) * tK * u[i];
            }
            if (std::fabs(center) < EPS) center = 1;
            A.set(ci, ci, center);
            b[ci] = tb;
        }
        for (int hs : halfTilts) {
            int l = slev[hs];
            int ci = pT[hs];
            const TiltE& tn = te[hs];
            double area = tn.e * tn.e * 2;
            double h = dh(l);
            double center = 0, tb = 0, tC = 0, tK = 0;
            const double* u = &tv[c][(size_t)hs * 8];
            const double* tw = &wTilt[(size_t)hs * 8];
            int id[3] = {sx[hs] >> 1, sy[hs] >> 1, sz[hs] >> 1};
            id[tn.dir % 3] -= tn.dir < 3 ? 1 : 0;
            int oi = HALF_SLOT[tn.dir][4];
            if (l + 1 < L && octValid(l + 1, id[0], id[1], id[2])) {
                int ti = pOctAt(l + 1, id[0], id[1], id[2]);
                if (ti >= 0) {
                    if (ci >= 0) {
                        A.add(ti, ti, tw[oi] * area / h);
                        center += tw[oi] * area / h;
                        A.add(ti, ci, -tw[oi] * area / h);
                        A.add(ci, ti, -tw[oi] * area / h);
                        b[ti] += (tn.dir < 3 ? -1 : 1) * u[oi] * tw[oi] * area;
                        tb += (tn.dir < 3 ? 1 : -1) * u[oi] * tw[oi] * area;
                    }
                }
            } else if (ci >= 0) {
                int axis = (tn.dir % 3) * 2 + (tn.dir >= 3);
                if (closedDomain(axis)) { tC = 0; tK = area; }
                else { tC = 1000; tK = area; }
                center += tC;
                tb += (tn.dir < 3 ? 1 : -1) * u[oi] * area;
            }
            if (ci < 0) continue;
            area = tn.e * tn.e * SQRT3 * 0.5;
            for (int i = 0; i < 8; ++i) {
                bool listed = false;
                for (int q = 0; q < 4; ++q) listed |= HALF_SLOT[tn.dir][q] == i;
                if (!listed) continue;
                int nx = sx[hs] + TILT_NB_OCT[i][0], ny = sy[hs] + TILT_NB_OCT[i][1], nz = sz[hs] + TILT_NB_OCT[i][2];
                if (octValid(l, nx, ny, nz)) {
                    int ti = pOctAt(l, nx, ny, nz);
                    if (ti >= 0) {
                        tC = area * tw[i] / (h * SQRT3 * 0.5);
                        tK = area * tw[i];
                        A.set(ci, ti, -tC);
                    } else { tC = 0; tK = 0; }
                } else {
                    throw std::runtime_error("oracle: half tilt next to the domain edge");
                }
                center += tC;
                tb += (i < 4 ? -1 : 1) * tK * u[i];
            }
            A.add(ci, ci, center);
            b[ci] = tb;
        }
        double sc = P.rho / dt;
        for (auto& v : b) v *= sc;
    }

    // ---------------------------------------------------------------- PCG with MIC(0)
    // include/pcgsolver/pcg_solver.h:89-190
    struct Factor {
        int n = 0;
        std::vector<double> invdiag, value, adiag;
        std::vector<int> rowindex, colstart;
    } F;
    void factorMIC() {
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
            if (F.invdiag[k] < P.minDiag * F.adiag[k]) F.invdiag[k] = 1 / std::sqrt(F.adiag[k]);
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
                F.invdiag[j] -= P.omega * mult * missing;
            }
        }
    }
    // :211-253.  reduce_mode 0: the reference's multiply-then-subtract; reduce_mode 1 (the GPU
    // library's order): each update as one fused multiply-subtract, std::fma(-L, z, acc), in the
    // same order (correctly rounded, the same operation as the GPU's FP64 fma)
    void applyPrecond(const std::vector<double>& r, std::vector<double>& z) {
        z = r;
        const bool fused = P.reduceMode != 0;
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
    // acc + a * b: in the library's order one fused multiply-add (CSR rows, dots, vector updates), in
    // the reference's a product, then an addition
    double fmadd(double acc, double a, double b) const {
        if (P.reduceMode != 0) return std::fma(a, b, acc);
        double prod = a * b;
        return acc + prod;
    }
    double dotv(const std::vector<double>& a, const std::vector<double>& b) const {
        if (P.reduceMode == 0) return eigenDot(a.data(), b.data(), a.size());
        return treeReduce(a.size(), [&](double acc, size_t i) { return std::fma(a[i], b[i], acc); });
    }
    static double absmax(const std::vector<double>& a) {
        double m = 0;
        for (double v : a) m = std::max(m, std::fabs(v));
        return m;
    }
    void buildCSR() {
        csrPtr.assign(A.n + 1, 0);
        for (int i = 0; i < A.n; ++i) csrPtr[i + 1] = csrPtr[i] + A.idx[i].size();
        csrCol.resize(csrPtr[A.n]);
        csrVal.resize(csrPtr[A.n]);
        for (int i = 0; i < A.n; ++i)
            for (size_t k = 0; k < A.idx[i].size(); ++k) {
                csrCol[csrPtr[i] + k] = A.idx[i][k];
                csrVal[csrPtr[i] + k] = A.val[i][k];
            }
    }
    // :366-426
    void pcg() {
        int n = A.n;
        p.assign(n, 0.0);
        std::vector<double> r = b, z(n), s(n);
        double resid = absmax(r);
        buildCSR();
        if (resid == 0) { pcgIters = 0; pcgErr = 0; pcgOk = true; return; }
        double tol = P.tol * resid;
        factorMIC();
        applyPrecond(r, z);
        double rho = dotv(z, r);
        if (rho == 0 || rho != rho) { pcgIters = 0; pcgErr = resid; pcgOk = false; return; }
        s = z;
        int it;
        for (it = 0; it < P.maxIter; ++it) {
    #pragma omp parallel for schedule(dynamic, 256)
            for (int i = 0; i < n; ++i) {
                double t = 0;
                for (int j = csrPtr[i]; j < csrPtr[i + 1]; ++j) t = fmadd(t, csrVal[j], s[csrCol[j]]);
                z[i] = t;
            }
            double alpha = rho / dotv(s, z);
            for (int i = 0; i < n; ++i) { p[i] = fmadd(p[i], alpha, s[i]); r[i] = fmadd(r[i], -alpha, z[i]); }
            resid = absmax(r);
            if (resid <= tol) { pcgIters = it + 1; pcgErr = resid; pcgOk = true; return; }
            applyPrecond(r, z);
            double rn = dotv(z, r);
            double beta = rn / rho;
            for (int i = 0; i < n; ++i) z[i] = fmadd(z[i], beta, s[i]);
            s.swap(z);
            rho = rn;
        }
        pcgIters = it;
        pcgErr = resid;
        pcgOk = false;
    }

    // src/octree_omnigrid_solver3.cpp:682-847
    void pressureUpdate(double dt) {
        int c = cur;
        const std::vector<TiltE>& te = tiltE[c];
        const double k0 = dt / P.rho;
#pragma omp parallel for schedule(dynamic, 256)
        for (int s = 0; s < S; ++s) {
            if (sflag[s] & F_GHOST) continue;
            int l = slev[s], x = sx[s], y = sy[s], z = sz[s];
            double h = dh(l);
            double p0 = 0;
            if (octValid(l, x, y, z) && pO[s] >= 0) p0 = p[pO[s]];
            for (int a = 0; a < 3; ++a) {
                if (!macValid(a, l, x, y, z)) continue;
                if (wMac[a][s] <= 0) { mac[c][a][s] = 0; continue; }
                int id[3] = {x, y, z};
                id[a] -= 1;
                double p1 = 0;
                if (octValid(l, id[0], id[1], id[2])) {
                    int ti = pOctAt(l, id[0], id[1], id[2]);
                    if (ti >= 0) p1 = p[ti];
                }
                mac[c][a][s] = mac[c][a][s] - k0 * (p0 - p1) / h;
            }
        }
#pragma omp parallel for schedule(dynamic, 256)
        for (int s = 0; s < S; ++s) {
            if (sflag[s] & F_GHOST) continue;
            if (!tOpen[s]) continue;
            int ci = pT[s];
            double p0 = ci >= 0 ? p[ci] : 0;
            double* nv = &tv[c][(size_t)s * 8];
            const double* tw = &wTilt[(size_t)s * 8];
            NbOct nb[8];
            tiltNbOct(slev[s], sx[s], sy[s], sz[s], nb);
            double out[8];
            for (int k = 0; k < 8; ++k) {
                if (tw[k] > 0 && nb[k].some) {
                    double h2 = dh(nb[k].l);
                    double p1 = 0;
                    if (octValid(nb[k].l, nb[k].x, nb[k].y, nb[k].z)) {
                        int ti = pOctAt(nb[k].l, nb[k].x, nb[k].y, nb[k].z);
                        if (ti >= 0) p1 = p[ti];
                    }
                    out[k] = nv[k] - k0 * (k < 4 ? 1 : -1) / (h2 * SQRT3 * 0.5) * (p1 - p0);
                } else out[k] = 0;
            }
            for (int k = 0; k < 8; ++k) nv[k] = out[k];
        }
        for (int hs : halfTilts) {
            const TiltE& tn = te[hs];
            int ci = pT[hs];
            int l = slev[hs];
            double p0 = ci >= 0 ? p[ci] : 0;
            double nv[8];
            for (int k = 0; k < 8; ++k) nv[k] = tv[c][(size_t)hs * 8 + k];
            const double* tw = &wTilt[(size_t)hs * 8];
            int id[3] = {sx[hs] >> 1, sy[hs] >> 1, sz[hs] >> 1};
            id[tn.dir % 3] -= tn.dir < 3 ? 1 : 0;
            int fsl = HALF_SLOT[tn.dir][4];
            if (tw[fsl] > 0) {
                int ti = pOctAt(l + 1, id[0], id[1], id[2]);
                double p1 = ti >= 0 ? p[ti] : 0;
                nv[fsl] -= k0 * (tn.dir < 3 ? 1 : -1) / dh(l) * (p0 - p1);
            } else nv[fsl] = 0;
            for (int k = 0; k < 8; ++k) {
                bool listed = false;
                for (int q = 0; q < 4; ++q) listed |= HALF_SLOT[tn.dir][q] == k;
                if (tw[k] > 0 && listed) {
                    int nx = sx[hs] + TILT_NB_OCT[k][0], ny = sy[hs] + TILT_NB_OCT[k][1], nz = sz[hs] + TILT_NB_OCT[k][2];
                    double p1 = 0;
                    if (octValid(l, nx, ny, nz)) {
                        int ti = pOctAt(l, nx, ny, nz);
                        if (ti >= 0) p1 = p[ti];
                    }
                    nv[k] = nv[k] - k0 * (k < 4 ? 1 : -1) / (dh(l) * SQRT3 * 0.5) * (p1 - p0);
                } else if (k != fsl) nv[k] = 0;
            }
            for (int k = 0; k < 8; ++k) tv[c][(size_t)hs * 8 + k] = nv[k];
        }
    }

    // src/octree_omni_face_centered_grid3.cpp:32-159
    void updateDual() {
        int c = cur;
        const std::vector<TiltE>& te = tiltE[c];
        std::vector<double>& DO = dual[c][0];
        std::vector<double>& DT = dual[c][1];
        const double s3 = INV_SQRT3 * (3.0 / 4.0);
#pragma omp parallel for schedule(dynamic, 256)
        for (int s = 0; s < S; ++s) {
            if (sflag[s] & F_GHOST) continue;
            if (te[s].closed) { DT[3 * s] = DT[3 * s + 1] = DT[3 * s + 2] = 0; continue; }
            const double* g = &tv[c][(size_t)s * 8];
            double v4[4] = {(g[0] + g[6]) * 0.5, (g[1] + g[7]) * 0.5, (g[2] + g[4]) * 0.5, (g[3] + g[5]) * 0.5};
            const double M[3][4] = {{s3, -s3, -s3, s3}, {s3, s3, -s3, -s3}, {s3, s3, s3, s3}};
            // Matrix34d * Vector4d, same evaluation scheme as applyM37
            for (int k = 0; k < 2; ++k) DT[3 * s + k] = ((M[k][0] * v4[0] + M[k][1] * v4[1]) + M[k][2] * v4[2]) + M[k][3] * v4[3];
            DT[3 * s + 2] = (M[2][0] * v4[0] + M[2][1] * v4[1]) + (M[2][2] * v4[2] + M[2][3] * v4[3]);
        }
#pragma omp parallel for schedule(dynamic, 256)
        for (int s = 0; s < S; ++s) {
            if (sflag[s] & F_GHOST) continue;
            int l = slev[s], x = sx[s], y = sy[s], z = sz[s];
            if (!octValid(l, x, y, z)) { DO[3 * s] = DO[3 * s + 1] = DO[3 * s + 2] = 0; continue; }
            double h = dh(l);
            double sq = SQRT3 * h, hsq = sq * 0.5;
            int nj[8];
            int ts[8];
            for (int i = 0; i < 8; ++i) {
                ts[i] = slotReq(l, x + OCT_NB_TILT[i][0], y + OCT_NB_TILT[i][1], z + OCT_NB_TILT[i][2]);
                const TiltE& n = te[ts[i]];
                nj[i] = (n.tjoint && std::fabs(n.e - h) < EPS) || n.half;
            }
            double v[7] = {0, 0, 0, 0, 0, 0, 0};
            int cnt[7] = {0, 0, 0, 0, 0, 0, 0};
            if (!((nj[1] && nj[6]) || (nj[2] && nj[5]))) { v[0] += mac[c][0][s]; cnt[0]++; }
            if (!((nj[0] && nj[7]) || (nj[3] && nj[4]))) { v[0] += mac[c][0][slotReq(l, x + 1, y, z)]; cnt[0]++; }
            if (!((nj[2] && nj[7]) || (nj[3] && nj[6]))) { v[1] += mac[c][1][s]; cnt[1]++; }
            if (!((nj[0] && nj[5]) || (nj[1] && nj[4]))) { v[1] += mac[c][1][slotReq(l, x, y + 1, z)]; cnt[1]++; }
            if (!((nj[4] && nj[6]) || (nj[5] && nj[7]))) { v[2] += mac[c][2][s]; cnt[2]++; }
            if (!((nj[0] && nj[2]) || (nj[1] && nj[3]))) { v[2] += mac[c][2][slotReq(l, x, y, z + 1)]; cnt[2]++; }
            for (int i = 0; i < 4; ++i) {
                int slot = i, re = ((i & 1) ? 8 : 6) - i, vs = i + 3;
                const TiltE& n = te[ts[slot]];
                const TiltE& rn = te[ts[re]];
                if (!n.closed || n.half) { v[vs] += tv[c][(size_t)ts[slot] * 8 + re]; cnt[vs]++; }
                if (!rn.closed || rn.half) {
                    double t = tv[c][(size_t)ts[re] * 8 + slot];
                    // INV_SQRT3 is the unparenthesised macro "1.0 / SQRT3" (include/macro.h:20),
                    // so "e * INV_SQRT3" evaluates as e * 1.0 / SQRT3
                    v[vs] = cnt[vs] == 0 ? t
                                         : ((v[vs] * (hsq - rn.e * 1.0 / SQRT3) + t * (hsq - n.e * 1.0 / SQRT3)) /
                                            (sq - n.e * 1.0 / SQRT3 - rn.e * 1.0 / SQRT3));
                    cnt[vs]++;
                }
            }
            for (int i = 0; i < 3; ++i) v[i] = v[i] / (cnt[i] + EPS);
            int bits = dualBits(cnt[0] > 0, cnt[1] > 0, cnt[2] > 0, cnt[3] > 1 || nj[0] || nj[6], cnt[4] > 1 || nj[1] || nj[7],
                                cnt[5] > 1 || nj[2] || nj[4], cnt[6] > 1 || nj[3] || nj[5]);
            V3 f = applyM37(bits, v);
            DO[3 * s] = f.x; DO[3 * s + 1] = f.y; DO[3 * s + 2] = f.z;
        }
        for (int hs : halfTilts) {
            const TiltE& n = te[hs];
            const double* g = &tv[c][(size_t)hs * 8];
            double v[7] = {0, 0, 0, 0, 0, 0, 0};
            int axis = n.dir % 3;
            v[axis] = g[HALF_SLOT[n.dir][4]];
            for (int i = 0; i < 4; ++i) {
                int slot = HALF_SLOT[n.dir][i];
                int re = ((slot & 1) ? 8 : 6) - slot;
                int idx = slot < re ? slot : re;
                v[idx + 3] = g[slot];
            }
            V3 f = applyM37(dualBits(axis == 0, axis == 1, axis == 2, 1, 1, 1, 1), v);
            DT[3 * hs] = f.x; DT[3 * hs + 1] = f.y; DT[3 * hs + 2] = f.z;
        }
    }

    // src/octree_omnigrid_solver3.cpp:1125-1166
    void adjustE(double dt) {
        int c = cur, nx = 1 - cur;
        const double dTh = 0.02, vTh = EPS, maxTh = 1000;
#pragma omp parallel for schedule(dynamic, 256)
        for (int s = 0; s < S; ++s) {
            if (sflag[s] & F_GHOST) continue;
            if (tFixed[s]) continue;
            if (tOpen[s]) {
                double d = dT[c][s];
                if (d < dTh || d > maxTh) tOpen[s] = 0;
            } else {
                V3 pos = vertPos(s);
                V3 v = velSample(pos, c);
                if (std::sqrt(v.x * v.x + v.y * v.y + v.z * v.z) > vTh) {
                    V3 old = pos - v * dt;
                    double d = scalarSample(old, dO[c], dT[c], tiltE[c]);
                    if (d > dTh && d < maxTh) tOpen[s] = 1;
                }
            }
        }
        // TiltENodeS ghost copy
        for (int l = 0; l < L; ++l)
            for (int i = lN[l]; i < lN[l] + lG[l]; ++i) {
                int s = loff[l] + i;
                int x = sx[s], y = sy[s], z = sz[s];
                int src;
                if (sflag[s] & F_FROM_COARSE) {
                    if ((x & 1) || (y & 1) || (z & 1)) continue;
                    src = slotReq(l + 1, x >> 1, y >> 1, z >> 1);
                } else src = slotReq(l - 1, x << 1, y << 1, z << 1);
                tOpen[s] = tOpen[src];
                tFixed[s] = tFixed[src];
            }
        for (int s = 0; s < S; ++s) {
            if (sflag[s] & F_GHOST) continue;
            if (tFixed[s]) continue;
            TiltE& n = tiltE[nx][s];
            if (tOpen[s]) {
                double m = dh(slev[s]) * 0.5;
                n.setE(m, m);
            } else n.setE(0);
        }
        vertexCopyGhost(tiltE[nx]);
    }

    // src/octree_omnigrid_solver3.cpp:850-914 and include/advection.h:195-239
    void advect(double dt) {
        int c = cur, nx = 1 - cur;
        if (P.tiltAdaptivity) adjustE(dt);
        const std::vector<TiltE>& te = tiltE[c];
#pragma omp parallel for schedule(dynamic, 256)
        for (int s = 0; s < S; ++s) {
            if (sflag[s] & F_GHOST) continue;
            V3 o = backTrace(cellPos(s), dt, c);
            dO[nx][s] = scalarSample(o, dO[c], dT[c], te);
            hO[nx][s] = scalarSample(o, hO[c], hT[c], te);
        }
#pragma omp parallel for schedule(dynamic, 256)
        for (int s = 0; s < S; ++s) {
            if (sflag[s] & F_GHOST) continue;
            if (!tOpen[s]) continue;
            V3 o = backTrace(vertPos(s), dt, c);
            dT[nx][s] = scalarSample(o, dO[c], dT[c], te);
            hT[nx][s] = scalarSample(o, hO[c], hT[c], te);
        }
        for (int hs : halfTilts) {
            V3 o = backTrace(vertPos(hs), dt, c);
            dT[nx][hs] = scalarSample(o, dO[c], dT[c], te);
            hT[nx][hs] = scalarSample(o, hO[c], hT[c], te);
        }
        scalarGhost(dO[nx], dT[nx], tiltE[nx]);
        scalarGhost(hO[nx], hT[nx], tiltE[nx]);
        // velocity: src = buffer c, dst = buffer nx (whose tilt-E is the adjusted one)
        const std::vector<TiltE>& tn = tiltE[nx];
        for (int a = 0; a < 3; ++a)
#pragma omp parallel for schedule(dynamic, 256)
            for (int s = 0; s < S; ++s) {
                if (sflag[s] & F_GHOST) continue;
                V3 o = backTrace(macPos(a, s), dt, c);
                mac[nx][a][s] = velSample(o, c)[a];
            }
#pragma omp parallel for schedule(dynamic, 256)
        for (int s = 0; s < S; ++s) {
            if (sflag[s] & F_GHOST) continue;
            if (tn[s].closed) continue;
            double nv[8];
            for (int k = 0; k < 8; ++k) {
                V3 o = backTrace(tiltPos(vertPos(s), k, tn[s].e), dt, c);
                nv[k] = dot3(velSample(o, c), v3(tilt_up(k, 0), tilt_up(k, 1), tilt_up(k, 2)));
            }
            for (int k = 0; k < 8; ++k) tv[nx][(size_t)s * 8 + k] = nv[k];
        }
        for (int hs : halfTilts) {
            double nv[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            const TiltE& n = tn[hs];
            for (int i = 0; i < 5; ++i) {
                int k = HALF_SLOT[n.dir][i];
                V3 pos = (i == 4) ? vertPos(hs) : tiltPos(vertPos(hs), k, n.e);
                V3 o = backTrace(pos, dt, c);
                V3 d = (i == 4) ? v3(HALF_DIR_POS[k][0], HALF_DIR_POS[k][1], HALF_DIR_POS[k][2])
                                : v3(tilt_up(k, 0), tilt_up(k, 1), tilt_up(k, 2));
                nv[k] = dot3(velSample(o, c), d);
            }
            for (int k = 0; k < 8; ++k) tv[nx][(size_t)hs * 8 + k] = nv[k];
        }
        cur = nx;
        for (int s = 0; s < S; ++s) {
            dO[cur][s] *= P.decay; dT[cur][s] *= P.decay;
            hO[cur][s] *= P.decay; hT[cur][s] *= P.decay;
        }
    }

    // stage ids used by the C API: 0 source, 1 force, 2 pre-projection (walls + ghost),
    // 3 projection, 4 post-projection (walls + ghost + dual + dual ghost), 5 advection
    void stage(int id, double dt) {
        switch (id) {
            case 0: source(); break;
            case 1: wipeBoundary(); addForce(dt); break;
            case 2: colliderMac(); constrainWalls(); colliderTilt(); velocityGhost(cur); break;
            case 3: updateIndex(); assemble(dt); pcg(); pressureUpdate(dt); break;
            case 4:
                colliderMac(); constrainWalls(); colliderTilt(); velocityGhost(cur);
                updateDual(); colliderDual(); dualGhost(cur);
                break;
            case 5: advect(dt); break;
            default: throw std::runtime_error("oracle: bad stage");
        }
    }
    void step(double dt) {
        for (int i = 0; i < 6; ++i) stage(i, dt);
    }
    // OctreeOmniGridSolver3::cfl (src/octree_omnigrid_solver3.cpp:1066-1122): the largest MAC face
    // value over all faces of all levels (ghost slots included, starting from 0, so negative
    // values never count), times dt over the finest spacing, truncated to int
    int cfl(double dt) const {
        double maxV = 0;
        for (int a = 0; a < 3; ++a)
            for (double v : mac[cur][a]) maxV = std::max(maxV, v);
        return (int)(dt * maxV / dx);
    }
    // numberOfSubTimeSteps (:1060-1063)
    int numberOfSubTimeSteps(double dt, double maxCfl) const {
        int k = (int)std::ceil(cfl(dt) / maxCfl);
        return k > 1 ? k : 1;
    }
    // Solver::update's adaptive branch (src/solver.cpp:21-41, useFixedTimeStep = false): sub-steps
    // of remaining / k until less than EPSILON (general.h:48) remains, k recomputed from the
    // current velocity before each sub-step; returns the sub-step counts in order
    std::vector<int> update(double dt, double maxCfl) {
        std::vector<int> ks;
        double remaining = dt;
        while (remaining > std::numeric_limits<double>::epsilon()) {
            int k = numberOfSubTimeSteps(remaining, maxCfl);
            ks.push_back(k);
            double actual = remaining / (double)k;
            step(actual);
            remaining -= actual;
        }
        return ks;
    }
    void finishInit() {
        halfMark.assign(S, 0);
        for (int hs : halfTilts) halfMark[hs] = 1;
    }

    // ---------------------------------------------------------------- extrapolation
    // CellCenteredGrid<REAL,3>::sample (include/cell_centered_grid.h:40-54) on a res^3 signed
    // distance grid of spacing 1/res (index (z*res + y)*res + x)
    double sdfSample(const std::vector<double>& sdf, int sres, const V3& p) const {
        double sd = 1.0 / sres;
        double rp[3] = {p.x / sd - 0.5, p.y / sd - 0.5, p.z / sd - 0.5};
        int i[3], i1[3];
        double f[3];
        for (int k = 0; k < 3; ++k) {
            bary_vec(rp[k], sres - 1, &i[k], &f[k]);
            i1[k] = std::min(i[k] + 1, sres - 1);
        }
        auto g = [&](int x, int y, int z) { return sdf[((size_t)z * sres + y) * sres + x]; };
        return trilerp(g(i[0], i[1], i[2]), g(i1[0], i[1], i[2]), g(i[0], i1[1], i[2]), g(i1[0], i1[1], i[2]),
                       g(i[0], i[1], i1[2]), g(i1[0], i[1], i1[2]), g(i[0], i1[1], i1[2]), g(i1[0], i1[1], i1[2]),
                       f[0], f[1], f[2]);
    }
    // FmmLevelSetSolver3::extrapolate (include/jet/fmm_levelset_solver3.h:84-408) with no cached
    // marker: the scalar omni field (oct, til) of the current buffer is extrapolated in place
    // from the nodes where sdf < -offset * d (d: dx_l sqrt(3)/2 for octagons, e for tilts, dx_l
    // for half tilts) outward, in increasing order of the SDF sampled at each node, up to
    // maxFactor * dx_0.  Sequential: the reference gathers its first candidates per worker slice
    // in slice order, which is this node order.  Returns the number of nodes assigned.
    enum { K_UNKNOWN = 0, K_KNOWN = 1, K_TRIAL = 2, K_DONT_TOUCH = 3, K_GHOST = 4 };
    enum { M_TILT = 0, M_OCT = 1, M_HALF = 2 };
    long long extrapolate(std::vector<double>& oct, std::vector<double>& til, const std::vector<double>& sdf, int sres,
                          double offset, double maxFactor) {
        const std::vector<TiltE>& te = tiltE[cur];
        auto valid = [&](double d, double v) { return v < -offset * d; };
        std::vector<char> mO(S, K_UNKNOWN), mT(S, K_UNKNOWN);
        for (int s = 0; s < S; ++s) {
            if (sflag[s] & F_GHOST) continue;
            int l = slev[s];
            if (octValid(l, sx[s], sy[s], sz[s])) {
                if (valid(dh(l) * SQRT3 * 0.5, sdfSample(sdf, sres, cellPos(s)))) mO[s] = K_KNOWN;
            } else {
                mO[s] = K_DONT_TOUCH;
            }
        }
        for (int s = 0; s < S; ++s) {
            if (sflag[s] & F_GHOST) continue;
            if (te[s].closed) mT[s] = K_DONT_TOUCH;
            else if (valid(te[s].e, sdfSample(sdf, sres, vertPos(s)))) mT[s] = K_KNOWN;
        }
        for (int s = 0; s < S; ++s)
            if (sflag[s] & F_GHOST) { mO[s] = K_GHOST; mT[s] = K_GHOST; }
        for (int hs : halfTilts)
            if (valid(dh(slev[hs]), sdfSample(sdf, sres, vertPos(hs)))) mT[hs] = K_KNOWN;

        typedef std::tuple<char, int, double> Item;
        auto cmp = [](const Item& a, const Item& b) { return std::get<2>(a) * 1.0 > std::get<2>(b) * 1.0; };
        std::vector<Item> arr;
        auto sdfO = [&](int t) { return sdfSample(sdf, sres, cellPos(t)); };
        auto sdfT = [&](int t) { return sdfSample(sdf, sres, vertPos(t)); };
        // a tilt vertex that is a ghost stands for the non-ghost node getUntil finds, when that
        // node is finer or sits at the same corner (the reference's test, :176-178 and :322-325)
        auto ghostTilt = [&](int l, int x, int y, int z) {
            int c0 = getUntil(l, x, y, z, true);
            if (c0 < 0) c0 = getUntil(l, x, y, z, false);
            if (c0 < 0) return -1;
            if (slev[c0] < l || ((sx[c0] << 1) == x && (sy[c0] << 1) == y && (sz[c0] << 1) == z)) return c0;
            return -1;
        };
        auto halfNb = [&](int hs, int out[8]) {  // halfTiltNeighborOctagon3 + the big octagon
            const TiltE& n = te[hs];
            int l = slev[hs], x = sx[hs], y = sy[hs], z = sz[hs];
            for (int k = 0; k < 8; ++k) out[k] = -1;
            for (int i = 0; i < 4; ++i) {
                int k = HALF_SLOT[n.dir][i];
                out[k] = slotOf(l, x + TILT_NB_OCT[k][0], y + TILT_NB_OCT[k][1], z + TILT_NB_OCT[k][2]);
            }
            int id[3] = {x >> 1, y >> 1, z >> 1};
            id[n.dir % 3] -= n.dir < 3 ? 1 : 0;
            out[HALF_SLOT[n.dir][4]] = (l + 1 < L) ? slotOf(l + 1, id[0], id[1], id[2]) : -1;
        };
        auto tiltNbSlots = [&](int s, int out[8]) {  // tiltNeighborOctagon3 as slots (-1: none)
            NbOct nb[8];
            tiltNbOct(slev[s], sx[s], sy[s], sz[s], nb);
            for (int k = 0; k < 8; ++k) out[k] = nb[k].some ? slotOf(nb[k].l, nb[k].x, nb[k].y, nb[k].z) : -1;
        };
        // first ring (:154-205), node order
        for (int s = 0; s < S; ++s) {
            if (sflag[s] & F_GHOST) continue;
            int l = slev[s], x = sx[s], y = sy[s], z = sz[s];
            if (mO[s] == K_KNOWN) {
                for (int k = 0; k < 6; ++k) {
                    int tx = x + OCT_NB[k][0], ty = y + OCT_NB[k][1], tz = z + OCT_NB[k][2];
                    if (!octValid(l, tx, ty, tz)) continue;
                    int t = slotOf(l, tx, ty, tz);
                    if (t >= 0 && mO[t] == K_UNKNOWN) { mO[t] = K_TRIAL; arr.emplace_back(M_OCT, t, sdfO(t)); }
                }
                if (l >= 1) {
                    for (int k = 0; k < 6; ++k) {
                        int axis = k >> 1;
                        int id[3] = {2 * x + 1, 2 * y + 1, 2 * z + 1};
                        id[axis] += (k & 1) ? 1 : -1;
                        int t = slotOf(l - 1, id[0], id[1], id[2]);
                        if (t >= 0 && te[t].half && mT[t] == K_UNKNOWN) { mT[t] = K_TRIAL; arr.emplace_back(M_HALF, t, sdfT(t)); }
                    }
                }
                for (int k = 0; k < 8; ++k) {
                    int tx = x + OCT_NB_TILT[k][0], ty = y + OCT_NB_TILT[k][1], tz = z + OCT_NB_TILT[k][2];
                    int t = slotOf(l, tx, ty, tz);
                    if (t < 0) continue;
                    if (mT[t] == K_UNKNOWN) {
                        mT[t] = K_TRIAL;
                        arr.emplace_back(te[t].half ? M_HALF : M_TILT, t, sdfT(t));
                    } else if (mT[t] == K_GHOST) {
                        int c0 = ghostTilt(l, tx, ty, tz);
                        if (c0 >= 0 && mT[c0] == K_UNKNOWN) {
                            mT[c0] = K_TRIAL;
                            arr.emplace_back(te[c0].half ? M_HALF : M_TILT, c0, sdfT(c0));
                        }
                    }
                }
            }
            if (mT[s] == K_KNOWN && !te[s].half) {
                int nb[8];
                tiltNbSlots(s, nb);
                for (int k = 0; k < 8; ++k) {
                    int t = nb[k];
                    if (t >= 0 && mO[t] == K_UNKNOWN) { mO[t] = K_TRIAL; arr.emplace_back(M_OCT, t, sdfO(t)); }
                }
            }
        }
        for (int hs : halfTilts) {
            if (mT[hs] != K_KNOWN) continue;
            int nb[8];
            halfNb(hs, nb);
            for (int k = 0; k < 8; ++k) {
                int t = nb[k];
                if (t >= 0 && mO[t] == K_UNKNOWN) { mO[t] = K_TRIAL; arr.emplace_back(M_OCT, t, sdfO(t)); }
            }
        }
        std::priority_queue<Item, std::vector<Item>, decltype(cmp)> heap{cmp, std::move(arr)};
        // propagation (:257-405)
        long long assigned = 0;
        const double limit = dh(0) * maxFactor;
        while (!heap.empty()) {
            Item it = heap.top();
            heap.pop();
            int mark = std::get<0>(it), c = std::get<1>(it);
            if (std::fabs(std::get<2>(it)) > limit) break;
            if ((mark == M_OCT ? mO[c] : mT[c]) == K_KNOWN) continue;
            int l = slev[c], x = sx[c], y = sy[c], z = sz[c];
            double sum = 0.0, count = 0.0;
            if (mark == M_TILT) {
                int nb[8];
                tiltNbSlots(c, nb);
                for (int k = 0; k < 8; ++k) {
                    int t = nb[k];
                    if (t < 0) continue;
                    if (mO[t] == K_KNOWN) { sum += oct[t]; count += 1; }
                    else if (mO[t] == K_UNKNOWN) { mO[t] = K_TRIAL; heap.push(Item(M_OCT, t, sdfO(t))); }
                }
            } else if (mark == M_OCT) {
                for (int k = 0; k < 6; ++k) {
                    int tx = x + OCT_NB[k][0], ty = y + OCT_NB[k][1], tz = z + OCT_NB[k][2];
                    if (!octValid(l, tx, ty, tz)) continue;
                    int t = slotOf(l, tx, ty, tz);
                    if (t < 0) continue;
                    if (mO[t] == K_KNOWN) { sum += oct[t]; count += 1; }
                    else if (mO[t] == K_UNKNOWN) { mO[t] = K_TRIAL; heap.push(Item(M_OCT, t, sdfO(t))); }
                }
                if (l >= 1) {
                    for (int k = 0; k < 6; ++k) {
                        int axis = k / 2;
                        int id[3] = {2 * x + 1, 2 * y + 1, 2 * z + 1};
                        id[axis] += (k & 1) ? 1 : -1;
                        int t = slotOf(l - 1, id[0], id[1], id[2]);
                        if (t < 0 || !te[t].half) continue;
                        if (mT[t] == K_KNOWN) { sum += til[t]; count += 1; }
                        else if (mT[t] == K_UNKNOWN) { mT[t] = K_TRIAL; heap.push(Item(M_HALF, t, sdfT(t))); }
                    }
                }
                for (int k = 0; k < 8; ++k) {
                    int tx = x + OCT_NB_TILT[k][0], ty = y + OCT_NB_TILT[k][1], tz = z + OCT_NB_TILT[k][2];
                    int t = slotOf(l, tx, ty, tz);
                    if (t < 0) continue;
                    if (mT[t] == K_KNOWN) { sum += til[t]; count += 1; }
                    else if (mT[t] == K_UNKNOWN) {
                        mT[t] = K_TRIAL;
                        heap.push(Item(te[t].half ? M_HALF : M_TILT, t, sdfT(t)));
                    } else if (mT[t] == K_GHOST) {
                        int c0 = ghostTilt(l, tx, ty, tz);
                        if (c0 < 0) continue;
                        if (mT[c0] == K_KNOWN) { sum += til[t]; count += 1; }  // the ghost slot's own value
                        else if (mT[c0] == K_UNKNOWN) {
                            mT[c0] = K_TRIAL;
                            heap.push(Item(te[c0].half ? M_HALF : M_TILT, c0, sdfT(c0)));
                        }
                    }
                }
            } else {
                int nb[8];
                halfNb(c, nb);
                for (int k = 0; k < 8; ++k) {
                    int t = nb[k];
                    if (t < 0) continue;
                    if (mO[t] == K_KNOWN) { sum += oct[t]; count += 1; }
                    else { mO[t] = K_TRIAL; heap.push(Item(M_OCT, t, sdfO(t))); }
                }
            }
            if (mark == M_OCT) { oct[c] = sum / count; mO[c] = K_KNOWN; }
            else { til[c] = sum / count; mT[c] = K_KNOWN; }
            ++assigned;
        }
        return assigned;
    }
};

}  // namespace oracle

// ---------------------------------------------------------------------------- C API
extern "C" {

struct orc_params {
    double tol, buoy_d, buoy_t, decay, rho, noise;
    double src_cx, src_cy, src_cz, src_r;
    unsigned long long seed;
    int max_iter, tilt_adaptivity, closed_mask;
    int reduce_mode, ref_workers;
};

void* orc_create(int coarsest, int levels, const orc_params* p, char* err, int errlen) {
    try {
        auto* s = new oracle::Solver();
        oracle::Params P;
        if (p) {
            P.tol = p->tol; P.buoyD = p->buoy_d; P.buoyT = p->buoy_t; P.decay = p->decay; P.rho = p->rho;
            P.noise = p->noise; P.seed = p->seed; P.maxIter = p->max_iter; P.tiltAdaptivity = p->tilt_adaptivity != 0;
            P.src = astg_scene::Sphere{p->src_cx, p->src_cy, p->src_cz, p->src_r};
            P.closedMask = p->closed_mask;
            P.reduceMode = p->reduce_mode;
            P.refWorkers = p->ref_workers > 0 ? p->ref_workers : 8;
        }
        s->init(coarsest, levels, P);
        s->finishInit();
        s->initNoise();
        return s;
    } catch (std::exception& e) {
        if (err && errlen > 0) snprintf(err, errlen, "%s", e.what());
        return nullptr;
    }
}

void orc_destroy(void* h) { delete (oracle::Solver*)h; }

int orc_stage(void* h, int id, double dt, char* err, int errlen) {
    try {
        ((oracle::Solver*)h)->stage(id, dt);
        return 0;
    } catch (std::exception& e) {
        if (err && errlen > 0) snprintf(err, errlen, "%s", e.what());
        return 1;
    }
}

int orc_step(void* h, double dt, char* err, int errlen) {
    try {
        ((oracle::Solver*)h)->step(dt);
        return 0;
    } catch (std::exception& e) {
        if (err && errlen > 0) snprintf(err, errlen, "%s", e.what());
        return 1;
    }
}

// Solver::update with useFixedTimeStep = false: writes the sub-step counts (at most cap) to
// substeps and returns how many there were, or -1 on failure
int orc_update(void* h, double dt, double max_cfl, int* substeps, int cap, char* err, int errlen) {
    try {
        std::vector<int> ks = ((oracle::Solver*)h)->update(dt, max_cfl);
        for (int i = 0; i < (int)ks.size() && i < cap; ++i) substeps[i] = ks[i];
        return (int)ks.size();
    } catch (std::exception& e) {
        if (err && errlen > 0) snprintf(err, errlen, "%s", e.what());
        return -1;
    }
}

// Copies the named array (same names and layouts as the fixture archives) into buf, which
// holds cap elements of the array's type (f64 / i32 / u8); returns the element count, or -1
// for an unknown name.  buf may be null to query the size.
long long orc_get(void* h, const char* name, void* buf, long long cap) {
    auto* s = (oracle::Solver*)h;
    std::string n = name;
    int c = s->cur;
    auto outd = [&](const std::vector<double>& v) -> long long {
        if (buf) memcpy(buf, v.data(), sizeof(double) * std::min<long long>(cap, v.size()));
        return v.size();
    };
    auto outi = [&](const std::vector<int>& v) -> long long {
        if (buf) memcpy(buf, v.data(), sizeof(int) * std::min<long long>(cap, v.size()));
        return v.size();
    };
    if (n == "density_oct") return outd(s->dO[c]);
    if (n == "density_tilt") return outd(s->dT[c]);
    if (n == "heat_oct") return outd(s->hO[c]);
    if (n == "heat_tilt") return outd(s->hT[c]);
    if (n == "mac") {
        std::vector<double> v;
        for (int a = 0; a < 3; ++a) v.insert(v.end(), s->mac[c][a].begin(), s->mac[c][a].end());
        return outd(v);
    }
    if (n == "tilt_vel") return outd(s->tv[c]);
    if (n == "dual_oct") return outd(s->dual[c][0]);
    if (n == "dual_tilt") return outd(s->dual[c][1]);
    if (n == "tilt_e") {
        std::vector<double> v(s->S);
        for (int i = 0; i < s->S; ++i) v[i] = s->tiltE[c][i].e;
        return outd(v);
    }
    if (n == "tilt_flags") {
        std::vector<int> v(2 * s->S);
        for (int i = 0; i < s->S; ++i) {
            const auto& t = s->tiltE[c][i];
            v[2 * i] = (t.largest ? 1 : 0) | (t.closed ? 2 : 0) | (t.fixed ? 4 : 0) | (t.tjoint ? 8 : 0) |
                       (t.closedByT ? 16 : 0) | (t.half ? 32 : 0);
            v[2 * i + 1] = t.dir;
        }
        return outi(v);
    }
    if (n == "tilt_open") {
        if (buf)
            for (long long i = 0; i < std::min<long long>(cap, s->S); ++i)
                ((uint8_t*)buf)[i] = (s->tOpen[i] ? 1 : 0) | (s->tFixed[i] ? 2 : 0);
        return s->S;
    }
    if (n == "slot_coords") {
        std::vector<int> v(4 * s->S);
        for (int i = 0; i < s->S; ++i) {
            v[4 * i] = s->sx[i]; v[4 * i + 1] = s->sy[i]; v[4 * i + 2] = s->sz[i]; v[4 * i + 3] = s->sflag[i];
        }
        return outi(v);
    }
    if (n == "level_sizes") {
        std::vector<int> v;
        for (int l = 0; l < s->L; ++l) { v.push_back(s->lN[l]); v.push_back(s->lG[l]); v.push_back(s->lN[l] + s->lG[l]); }
        return outi(v);
    }
    if (n == "split_map") return outi(std::vector<int>(s->split.begin(), s->split.end()));
    if (n == "half_tilts" || n == "t_joints" || n == "closed_by_half_tilt") {
        const std::vector<int>& sl = n == "half_tilts" ? s->halfTilts : (n == "t_joints" ? s->tJoints : s->closedByHalf);
        // packed level coordinates as in include/macro.h:39-45
        std::vector<long long> v;
        for (int q : sl)
            v.push_back(((long long)s->slev[q] << 60) | ((long long)s->sx[q] << 40) | ((long long)s->sy[q] << 20) | (long long)s->sz[q]);
        if (n == "t_joints") std::sort(v.begin(), v.end());
        if (buf) memcpy(buf, v.data(), sizeof(long long) * std::min<long long>(cap, v.size()));
        return v.size();
    }
    if (n == "w_mac") {
        std::vector<double> v;
        for (int a = 0; a < 3; ++a) v.insert(v.end(), s->wMac[a].begin(), s->wMac[a].end());
        return outd(v);
    }
    if (n == "w_tilt") return outd(s->wTilt);
    if (n == "collider_sdf") return outd(s->colSdf);
    if (n == "pindex_oct") return outi(s->pO);
    if (n == "pindex_tilt") return outi(s->pT);
    if (n == "A_rowptr") return outi(s->csrPtr);
    if (n == "A_col") return outi(s->csrCol);
    if (n == "A_val") return outd(s->csrVal);
    if (n == "b") return outd(s->b);
    if (n == "p") return outd(s->p);
    if (n == "pcg_iters") return outi(std::vector<int>{s->pcgIters, s->pcgOk ? 1 : 0});
    if (n == "pcg_err") return outd(std::vector<double>{s->pcgErr});
    if (n == "ambT") return outd(std::vector<double>{s->ambT});
    if (n == "anomalies") return outi(std::vector<int>{s->anomalies});
    if (n == "dual_tables") {
        std::vector<double> v(&s->M37[0][0][0], &s->M37[0][0][0] + 128 * 21);
        return outd(v);
    }
    return -1;
}

// Overwrites a state array (same names as orc_get; a "t_" prefix addresses the swap-partner
// buffer); returns 0 on success.
int orc_set(void* h, const char* name, const void* buf, long long count) {
    auto* s = (oracle::Solver*)h;
    std::string n = name;
    if (n == "collider_sdf") {  // res^3 doubles (count 0: no collider); the cut-cell weights follow
        long long r = s->res;
        if (count != 0 && count != r * r * r) return 1;
        s->colSdf.assign((const double*)buf, (const double*)buf + count);
        s->cuttingCellWeights();
        return 0;
    }
    if (n == "collider_sphere") {  // cx cy cz r: the SDF grid of a sphere collider (r <= 0: none)
        if (count != 4) return 1;
        const double* q = (const double*)buf;
        s->sphereSdf(oracle::v3(q[0], q[1], q[2]), q[3]);
        s->cuttingCellWeights();
        return 0;
    }
    if (n == "collider_centre") {
        if (count != 3) return 1;
        const double* c3 = (const double*)buf;
        s->colCentre = oracle::v3(c3[0], c3[1], c3[2]);
        return 0;
    }
    int c = s->cur;
    static const char* fields[] = {"density_oct", "density_tilt", "heat_oct", "heat_tilt", "mac", "tilt_vel",
                                   "dual_oct", "dual_tilt", "tilt_e", "tilt_flags", "tilt_open"};
    if (n.compare(0, 2, "t_") == 0)
        for (const char* f : fields)
            if (n.compare(2, std::string::npos, f) == 0) {
                c = 1 - c;
                n = n.substr(2);
                break;
            }
    auto ind = [&](std::vector<double>& v) {
        if ((long long)v.size() != count) return 1;
        memcpy(v.data(), buf, sizeof(double) * count);
        return 0;
    };
    if (n == "density_oct") return ind(s->dO[c]);
    if (n == "density_tilt") return ind(s->dT[c]);
    if (n == "heat_oct") return ind(s->hO[c]);
    if (n == "heat_tilt") return ind(s->hT[c]);
    if (n == "tilt_vel") return ind(s->tv[c]);
    if (n == "dual_oct") return ind(s->dual[c][0]);
    if (n == "dual_tilt") return ind(s->dual[c][1]);
    if (n == "mac") {
        if (count != 3LL * s->S) return 1;
        for (int a = 0; a < 3; ++a) memcpy(s->mac[c][a].data(), (const double*)buf + (size_t)a * s->S, sizeof(double) * s->S);
        return 0;
    }
    if (n == "tilt_e") {
        if (count != s->S) return 1;
        for (int i = 0; i < s->S; ++i) s->tiltE[c][i].e = ((const double*)buf)[i];
        return 0;
    }
    if (n == "tilt_flags") {  // int32 pairs (flag bits, half direction)
        if (count != 2LL * s->S) return 1;
        const int* f = (const int*)buf;
        for (int i = 0; i < s->S; ++i) {
            auto& t = s->tiltE[c][i];
            t.largest = f[2 * i] & 1; t.closed = f[2 * i] & 2; t.fixed = f[2 * i] & 4;
            t.tjoint = f[2 * i] & 8; t.closedByT = f[2 * i] & 16; t.half = f[2 * i] & 32;
            t.dir = f[2 * i + 1];
        }
        return 0;
    }
    if (n == "tilt_open") {  // uint8 (bit0 open, bit1 fixed)
        if (count != s->S) return 1;
        const uint8_t* f = (const uint8_t*)buf;
        for (int i = 0; i < s->S; ++i) { s->tOpen[i] = f[i] & 1; s->tFixed[i] = (f[i] >> 1) & 1; }
        return 0;
    }
    return 2;
}

// PCGSolver::solve on a caller CSR system (rows sorted by column); x receives the solution.
// Returns the iteration count, or -1 on error.
int orc_solve(void* h, int n, const int* rowptr, const int* col, const double* val, const double* b, double* x,
              double tol, int max_iter) {
    auto* s = (oracle::Solver*)h;
    s->A.reset(n);
    for (int i = 0; i < n; ++i)
        for (int q = rowptr[i]; q < rowptr[i + 1]; ++q) {
            s->A.idx[i].push_back(col[q]);
            s->A.val[i].push_back(val[q]);
        }
    s->b.assign(b, b + n);
    double saveTol = s->P.tol;
    int saveIt = s->P.maxIter;
    s->P.tol = tol;
    s->P.maxIter = max_iter;
    s->pcg();
    s->P.tol = saveTol;
    s->P.maxIter = saveIt;
    memcpy(x, s->p.data(), sizeof(double) * n);
    return s->pcgIters;
}

// FmmLevelSetSolver3::extrapolate of "density" or "heat" (current buffer), in place; returns the
// number of nodes assigned, -1 on a bad argument
long long orc_extrapolate(void* h, const char* field, const double* sdf, int sres, double offset, double maxFactor) {
    auto* s = (oracle::Solver*)h;
    std::string f = field ? field : "";
    if ((f != "density" && f != "heat") || !sdf || sres <= 1) return -1;
    std::vector<double> g(sdf, sdf + (size_t)sres * sres * sres);
    int c = s->cur;
    if (f == "density") return s->extrapolate(s->dO[c], s->dT[c], g, sres, offset, maxFactor);
    return s->extrapolate(s->hO[c], s->hT[c], g, sres, offset, maxFactor);
}

int orc_size(void* h, int what) {
    auto* s = (oracle::Solver*)h;
    switch (what) {
        case 0: return s->S;
        case 1: return s->L;
        case 2: return s->res;
        case 3: return s->nDof;
        case 4: return (int)s->halfTilts.size();
        default: return -1;
    }
}
}
