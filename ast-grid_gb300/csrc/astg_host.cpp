// Host side of the GB300 octree smoke step: builds the octree topology once (it is static in
// the reference, src/octree_omnigrid_solver3.cpp:60-149), uploads it as flat device tables,
// sequences the kernels of each step on one CUDA stream and implements the C ABI of
// include/astg.h.  All per-step work runs on the GPU; the host only launches and, for the
// PCG's stopping test and the status word, reads a few bytes back.
#include <algorithm>
#include <chrono>
#include <exception>
#include <thread>
#include <utility>
#include <cmath>
#include <limits>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iterator>
#include <stdexcept>
#include <string>
#include <vector>

#define ASTG_HD
#include "astg.h"
#include "astg_launch.h"
#include "scene.h"

#include <sys/stat.h>

using namespace astg;

namespace {

const int OCT_NB_H[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
const int TILT_NB_OCT_H[8][3] = {{0, 0, 0},  {-1, 0, 0},  {-1, -1, 0},  {0, -1, 0},
                                 {0, 0, -1}, {-1, 0, -1}, {-1, -1, -1}, {0, -1, -1}};
const int HALF_SLOT_H[6][5] = {{0, 3, 4, 7, 1}, {0, 1, 4, 5, 2}, {0, 1, 2, 3, 5},
                               {1, 2, 5, 6, 0}, {2, 3, 6, 7, 4}, {4, 5, 6, 7, 3}};
const double HALF_DIR_POS_H[6][3] = {{1, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {0, 1, 0}, {0, 0, 1}};
const int TILT_UP_SIGN_H[8][3] = {{1, 1, 1},   {-1, 1, 1}, {-1, -1, 1}, {1, -1, 1},
                                  {-1, -1, 1}, {1, -1, 1}, {1, 1, 1},   {-1, 1, 1}};

struct CudaError : std::runtime_error {
    using std::runtime_error::runtime_error;
};
void ck(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw CudaError(std::string(what) + ": " + cudaGetErrorString(e));
}

// host copy of a tilt-E node (include/tilt_e_node.h:15-56)
struct HTilt {
    double e = 0;
    uint32_t f = TF_CLOSED;
    int dir = 0;
    bool has(uint32_t b) const { return (f & b) != 0; }
    void put(uint32_t b, bool v) { f = v ? (f | b) : (f & ~b); }
    void setE(double ne, double maxE = -1) {
        if (has(TF_FIXED)) return;
        if (ne <= 0) { put(TF_CLOSED, true); put(TF_LARGEST, false); ne = 0; }
        else if (maxE > 0 && ne >= maxE) { put(TF_CLOSED, false); put(TF_LARGEST, true); ne = maxE; }
        else { put(TF_CLOSED, false); put(TF_LARGEST, false); }
        e = ne;
    }
    uint32_t packed() const { return (f & 0xff) | ((uint32_t)(dir + 1) << 8); }
};

}  // namespace

struct astg_handle {
    astg_params P{};
    std::string err;
    cudaStream_t st = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, evA = nullptr, evB = nullptr;
    cudaEvent_t evF0 = nullptr, evF1 = nullptr, evAdv = nullptr;  // stage boundaries of astg_step

    // ---------------------------------------------------------------- topology (host)
    int L = 0, res = 0, S = 0, H = 0;
    double dx = 0;
    std::vector<int> lres, loff, lN, lG;
    std::vector<double> ldh;
    std::vector<std::vector<int>> brick;  // per level: global slot or -1
    std::vector<int> sx, sy, sz, slev, sflag;
    std::vector<int32_t> split;
    std::vector<int> half, tj, cbh;
    std::vector<HTilt> te[2];
    std::vector<uint8_t> tOpen, tFixed;
    std::vector<double> wMac, wTilt, M37;
    std::vector<double> wMac0, wTilt0;  // the collider-free weights

    // ---------------------------------------------------------------- device
    Dev d{};
    Fields F[2]{};
    int cur = 0;
    uint8_t* dOpen = nullptr;
    uint8_t* dFixed = nullptr;
    Proj J{};
    int refWorkers = 8;  // workers of the reference-order mean temperature
    double* dAmb = nullptr;
    double* dParts = nullptr;
    int* dPartOff = nullptr;
    std::vector<int> partOff;
    int* dHoPtr = nullptr;
    int* dHoIdx = nullptr;
    uint8_t* dLastWriter = nullptr;
    double* dSrcO = nullptr;  // per-slot source densities (octagon, tilt)
    double* dSrcT = nullptr;
    int* dStatus = nullptr;
    int epoch = 0;
    bool firstSource = true;
    astg_solve_stats last{};
    KProf prof;
    std::vector<void*> allocs;

    template <class T>
    T* dalloc(size_t n) {
        void* p = nullptr;
        ck(cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)), "cudaMalloc");
        ck(cudaMemsetAsync(p, 0, std::max<size_t>(n, 1) * sizeof(T), st), "cudaMemset");
        allocs.push_back(p);
        return (T*)p;
    }
    template <class T>
    T* upload(const std::vector<T>& v) {
        T* p = dalloc<T>(v.size());
        if (!v.empty()) ck(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st), "upload");
        return p;
    }

    ~astg_handle() {
        if (st) cudaStreamSynchronize(st);
        freeLanes();
        freeTape();
        for (void* p : allocs) cudaFree(p);
        if (J.hostDone) cudaFreeHost(J.hostDone);
        for (cudaEvent_t e : {ev0, ev1, evA, evB, evF0, evF1, evAdv})
            if (e) cudaEventDestroy(e);
        if (st) cudaStreamDestroy(st);
    }

    // ---------------------------------------------------------------- host lookups
    int get(int l, int x, int y, int z) const {
        if (l < 0 || l >= L) return -1;
        int r = lres[l];
        if (x < 0 || y < 0 || z < 0 || x >= r || y >= r || z >= r) return -1;
        return brick[l][((size_t)z * r + y) * r + x];
    }
    int req(int l, int x, int y, int z) const {
        int s = get(l, x, y, z);
        if (s < 0) {
            char m[128];
            snprintf(m, sizeof m, "layout: node (%d; %d, %d, %d) is missing", l, x, y, z);
            throw std::runtime_error(m);
        }
        return s;
    }
    bool octValid(int l, int x, int y, int z) const {
        int r = lres[l] - 1;
        return x >= 0 && y >= 0 && z >= 0 && x < r && y < r && z < r;
    }

    // ---------------------------------------------------------------- layout
    // OctreeLayer3 (src/octree_layer3.cpp:7-88) and constrainOctreeTiltE3 (src/octree_util.cpp:38-169)
    // are built on the device (astg_layout.cu); the host keeps copies for the set-up that follows
    LayoutBuild lay;
    void buildLayout() {
        ldh.assign(L, 0);
        for (int l = 0; l < L; ++l) ldh[l] = dx * (1 << l);
        build_layout_device(split.data(), res, L, ldh.data(), allocs, lay, st);
        S = lay.S;
        lres.assign(lay.lres, lay.lres + L);
        loff.assign(lay.loff, lay.loff + L);
        lN.assign(lay.lN, lay.lN + L);
        lG.assign(lay.lG, lay.lG + L);
        brick = std::move(lay.hbrick);
        sx.resize(S); sy.resize(S); sz.resize(S); slev.resize(S); sflag.resize(S);
        for (int s = 0; s < S; ++s) {
            const int4 q = lay.hslot[s];
            sx[s] = q.x; sy[s] = q.y; sz[s] = q.z; slev[s] = q.w & 0xff; sflag[s] = (q.w >> 8) & 0xff;
        }
        lay.hslot.clear();
        lay.hslot.shrink_to_fit();
        // both buffers of the tilt-E grid are constrained alike (src/octree_omnigrid_solver3.cpp:92-94)
        te[0].resize(S);
        for (int s = 0; s < S; ++s) {
            te[0][s].e = lay.te[s];
            te[0][s].f = lay.tf[s];
            te[0][s].dir = lay.tdir[s];
        }
        te[1] = te[0];
        half = lay.half;
        tj = lay.tj;
        cbh = lay.cbh;
        lay.te.clear(); lay.tf.clear(); lay.tdir.clear();
    }

    // Constants::init least-squares tables (src/constants.cpp:170-256), inverted through a
    // partial-pivoting LU in the order Eigen's MatrixXd::inverse() uses
    void buildTables() {
        M37.assign(128 * 21, 0.0);
        const double s = INV_SQRT3;
        const double rows[7][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {s, s, s}, {-s, s, s}, {-s, -s, s}, {s, -s, s}};
        for (int bits = 0; bits < 128; ++bits) {
            int use[7], cnt = 0;
            for (int k = 0; k < 7; ++k) { use[k] = (bits >> (6 - k)) & 1; cnt += use[k]; }
            if (cnt <= 1) continue;
            double G[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
            for (int r = 0; r < 7; ++r)
                if (use[r])
                    for (int i = 0; i < 3; ++i)
                        for (int j = 0; j < 3; ++j) G[i][j] += rows[r][i] * rows[r][j];
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
                for (int r = 0; r < 7; ++r)
                    if (use[r]) M37[(size_t)bits * 21 + k * 7 + r] = inv[k][0] * rows[r][0] + inv[k][1] * rows[r][1] + inv[k][2] * rows[r][2];
        }
    }

    V3 vertPos(int s) const { double h = ldh[slev[s]]; return v3(sx[s] * h, sy[s] * h, sz[s] * h); }
    V3 macPos(int a, int s) const {
        double h = ldh[slev[s]];
        double p[3] = {sx[s] * h + 0.5 * h, sy[s] * h + 0.5 * h, sz[s] * h + 0.5 * h};
        int c[3] = {sx[s], sy[s], sz[s]};
        p[a] = c[a] * h + 0.0 * h;
        return v3(p[0], p[1], p[2]);
    }
    static V3 tiltPos(V3 c, int dir, double e) {
        int m = dir & 3;
        double tz = (dir < 4 ? 1 : -1) * e / 3.0;
        double ty = (m < 2 ? 1 : -1) * e / 3.0;
        double tx = ((m == 0 || m == 3) ? 1 : -1) * e / 3.0;
        return v3(c.x + tx, c.y + ty, c.z + tz);
    }

    // ---------------------------------------------------------------- initialisation
    void init(const astg_params& p, const int32_t* splitMap) {
        P = p;
        if (P.levels < 2 || P.levels > MAXL || P.coarsest < 4) throw std::invalid_argument("levels must be 2..6, coarsest >= 4");
        L = P.levels;
        res = P.coarsest << (L - 1);
        dx = 1.0 / res;
        if (splitMap) split.assign(splitMap, splitMap + (size_t)res * res * res);
        else split = astg_scene::split_map(res, L, astg_scene::Sphere{P.src_x, P.src_y, P.src_z, P.src_r});
        for (int32_t v : split)
            if (v < 0 || v >= L) throw std::invalid_argument("split map holds a level outside [0, levels)");
        ck(cudaSetDevice(P.device), "cudaSetDevice");
        ck(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "stream");
        for (cudaEvent_t* e : {&ev0, &ev1, &evA, &evB, &evF0, &evF1, &evAdv}) ck(cudaEventCreate(e), "event");

        buildLayout();
        buildTables();
        tOpen.assign(S, 0);
        tFixed.assign(S, 0);
        H = (int)half.size();
        {
            std::vector<int> hs = half;
            std::sort(hs.begin(), hs.end());
            if (std::adjacent_find(hs.begin(), hs.end()) != hs.end())
                throw std::runtime_error("layout: a half tilt was recorded twice");
        }
        // fixed and outermost tilts (src/octree_omnigrid_solver3.cpp:128-145)
        for (int s = 0; s < S; ++s) {
            if (sflag[s] & SF_GHOST) continue;
            HTilt n = te[0][s];
            if (n.has(TF_TJOINT) || n.has(TF_FIXED)) {
                tOpen[s] = !n.has(TF_CLOSED);
                tFixed[s] = 1;
                continue;
            }
            int r = lres[slev[s]];
            if (sx[s] == 0 || sy[s] == 0 || sz[s] == 0 || sx[s] == r - 1 || sy[s] == r - 1 || sz[s] == r - 1) {
                n.setE(0);
                n.put(TF_FIXED, true);
                tOpen[s] = !n.has(TF_CLOSED);
                tFixed[s] = 1;
                te[0][s] = n;
                te[1][s] = n;
            }
        }
        // cut-cell weights of a collider-free domain (src/octree_omnigrid_solver3.cpp:1169-1238); a
        // collider set later recomputes them (setCollider), removing it restores these
        wMac.assign((size_t)3 * S, 1.0);
        wTilt.assign((size_t)8 * S, 1.0);
        for (int hs : half) {
            double w[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            int dir = te[0][hs].dir, l = slev[hs];
            int id[3] = {sx[hs] >> 1, sy[hs] >> 1, sz[hs] >> 1};
            id[dir % 3] -= dir < 3 ? 1 : 0;
            if (l + 1 < L && octValid(l + 1, id[0], id[1], id[2])) w[HALF_SLOT_H[dir][4]] = 1.0;
            for (int i = 0; i < 4; ++i) {
                int k = HALF_SLOT_H[dir][i];
                if (octValid(l, sx[hs] + TILT_NB_OCT_H[k][0], sy[hs] + TILT_NB_OCT_H[k][1], sz[hs] + TILT_NB_OCT_H[k][2])) w[k] = 1.0;
            }
            for (int k = 0; k < 8; ++k) wTilt[(size_t)hs * 8 + k] = w[k];
        }
        wMac0 = wMac;
        wTilt0 = wTilt;
        d.colCx = 0.5;  // the centre the reference's projection hard-codes
        d.colCy = 0.5;
        d.colCz = 0.45;
        uploadAll();
    }

    void uploadAll() {
        std::vector<uint8_t> halfMark(S, 0);
        for (int hs : half) halfMark[hs] = 1;
        // half tilts facing each coarse octagon, in list order (assembly, :572-581)
        std::vector<int> hoCnt(S + 1, 0), hoIdx;
        std::vector<std::vector<int>> ho(S);
        for (int i = 0; i < H; ++i) {
            int hs = half[i];
            int dir = te[0][hs].dir, l = slev[hs];
            int id[3] = {sx[hs] >> 1, sy[hs] >> 1, sz[hs] >> 1};
            id[dir % 3] -= dir < 3 ? 1 : 0;
            if (l + 1 < L && octValid(l + 1, id[0], id[1], id[2])) ho[req(l + 1, id[0], id[1], id[2])].push_back(i);
        }
        std::vector<int> hoPtr(S + 1, 0);
        for (int s = 0; s < S; ++s) {
            hoPtr[s + 1] = hoPtr[s] + (int)ho[s].size();
            hoIdx.insert(hoIdx.end(), ho[s].begin(), ho[s].end());
        }
        // only the last half tilt of the list that targets a MAC face writes it
        // (updateGhostFromHalfTilt, src/octree_omni_face_centered_grid3.cpp:162-173)
        std::vector<uint8_t> lastWriter(std::max(H, 1), 0);
        {
            std::vector<long long> seen;
            for (int i = H - 1; i >= 0; --i) {
                int hs = half[i];
                int a = te[0][hs].dir % 3;
                int t = req(slev[hs] + 1, sx[hs] >> 1, sy[hs] >> 1, sz[hs] >> 1);
                long long key = (long long)t * 3 + a;
                if (std::find(seen.begin(), seen.end(), key) == seen.end()) { lastWriter[i] = 1; seen.push_back(key); }
            }
        }
        d.L = L; d.res = res; d.S = S; d.H = H; d.nTJ = (int)tj.size(); d.nCBH = (int)cbh.size();
        d.dx = dx;
        for (int l = 0; l < L; ++l) {
            d.lres[l] = lres[l]; d.loff[l] = loff[l]; d.lN[l] = lN[l]; d.lG[l] = lG[l]; d.ldh[l] = ldh[l];
            d.brick[l] = lay.brick[l];  // built on the device
        }
        // power-of-two spacings: their reciprocals are exact, so x * (1 / h) == x / h (over_h)
        auto pow2 = [](double v) { int e; return std::frexp(v, &e) == 0.5; };
        d.pow2 = pow2(dx) ? 1 : 0;
        for (int l = 0; l < L; ++l) d.pow2 = d.pow2 && pow2(ldh[l]);
        d.dxInv = 1.0 / dx;
        for (int l = 0; l < L; ++l) d.ldhInv[l] = 1.0 / ldh[l];
        d.locate = lay.locate;
        d.slot = lay.slot;
        d.half = upload(half);
        d.halfMark = upload(halfMark);
        d.tj = upload(tj);
        d.cbh = upload(cbh);
        d.wMac = upload(wMac);
        d.wTilt = upload(wTilt);
        d.M37 = upload(M37);
        dStatus = dalloc<int>(1);
        d.status = dStatus;
        d.buoyD = P.buoy_density; d.buoyT = P.buoy_temp; d.rho = P.rho; d.decay = P.decay;
        d.closedMask = P.closed_mask;
        d.srcX = P.src_x; d.srcY = P.src_y; d.srcZ = P.src_z; d.srcR = P.src_r;
        dSrcO = upload(std::vector<double>(S, 1.0));
        dSrcT = upload(std::vector<double>(S, 1.0));
        d.srcO = dSrcO;
        d.srcT = dSrcT;
        dHoPtr = upload(hoPtr);
        dHoIdx = upload(hoIdx);
        dLastWriter = upload(lastWriter);
        // fields
        for (int b = 0; b < 2; ++b) {
            F[b].dO = dalloc<double>(S); F[b].dT = dalloc<double>(S);
            F[b].hO = dalloc<double>(S); F[b].hT = dalloc<double>(S);
            F[b].mac = dalloc<double>((size_t)3 * S);
            F[b].tv = dalloc<double>((size_t)8 * S);
            F[b].dualO = dalloc<double>((size_t)3 * S);
            F[b].dualT = dalloc<double>((size_t)3 * S);
            std::vector<double> e(S);
            std::vector<uint32_t> f(S);
            for (int s = 0; s < S; ++s) { e[s] = te[b][s].e; f[s] = te[b][s].packed(); }
            F[b].te = upload(e);
            F[b].tf = upload(f);
        }
        dOpen = upload(tOpen);
        dFixed = upload(tFixed);
        // initial velocity: seeded curl noise on valid MAC faces, open tilts and half tilts
        {
            astg_scene::CurlNoise cn(P.seed, P.noise);
            std::vector<double> mac((size_t)3 * S, 0.0), tv((size_t)8 * S, 0.0);
            auto vel = [&](V3 p) {
                double pp[3] = {p.x, p.y, p.z}, u[3];
                cn.velocity(pp, u);
                return v3(u[0], u[1], u[2]);
            };
            for (int s = 0; s < S; ++s) {
                if (sflag[s] & SF_GHOST) continue;
                int l = slev[s], r = lres[l];
                for (int a = 0; a < 3; ++a) {
                    int c[3] = {sx[s], sy[s], sz[s]};
                    bool ok = true;
                    for (int k = 0; k < 3; ++k) ok &= c[k] >= 0 && c[k] < (k == a ? r : r - 1);
                    if (!ok) continue;
                    mac[(size_t)a * S + s] = comp(vel(macPos(a, s)), a);
                }
                if (tOpen[s]) {
                    for (int k = 0; k < 8; ++k) {
                        V3 u = vel(tiltPos(vertPos(s), k, te[0][s].e));
                        V3 dn = v3(TILT_UP_SIGN_H[k][0] * INV_SQRT3, TILT_UP_SIGN_H[k][1] * INV_SQRT3, TILT_UP_SIGN_H[k][2] * INV_SQRT3);
                        tv[(size_t)s * 8 + k] = u.x * dn.x + u.y * dn.y + u.z * dn.z;
                    }
                }
            }
            for (int hs : half) {
                int dir = te[0][hs].dir;
                double nv[8] = {0, 0, 0, 0, 0, 0, 0, 0};
                for (int i = 0; i < 5; ++i) {
                    int k = HALF_SLOT_H[dir][i];
                    V3 p = (i == 4) ? vertPos(hs) : tiltPos(vertPos(hs), k, te[0][hs].e);
                    V3 u = vel(p);
                    V3 dn = (i == 4) ? v3(HALF_DIR_POS_H[k][0], HALF_DIR_POS_H[k][1], HALF_DIR_POS_H[k][2])
                                     : v3(TILT_UP_SIGN_H[k][0] * INV_SQRT3, TILT_UP_SIGN_H[k][1] * INV_SQRT3, TILT_UP_SIGN_H[k][2] * INV_SQRT3);
                    nv[k] = u.x * dn.x + u.y * dn.y + u.z * dn.z;
                }
                for (int k = 0; k < 8; ++k) tv[(size_t)hs * 8 + k] = nv[k];
            }
            ck(cudaMemcpyAsync(F[0].mac, mac.data(), mac.size() * 8, cudaMemcpyHostToDevice, st), "upload mac");
            ck(cudaMemcpyAsync(F[0].tv, tv.data(), tv.size() * 8, cudaMemcpyHostToDevice, st), "upload tilt");
        }
        // mean temperature partials
        partOff.assign(L + 1, 0);
        for (int l = 0; l < L; ++l) partOff[l + 1] = partOff[l] + (lN[l] + lG[l] + 2047) / 2048;
        dParts = dalloc<double>(partOff[L] + 1);
        dPartOff = upload(partOff);
        dAmb = dalloc<double>(1);
        allocProj();
        ck(cudaStreamSynchronize(st), "init");
    }

    // most rows a projection can have: an octagon and a tilt DOF on every non-ghost slot, plus the
    // half tilts
    long long rowCapacity() const {
        long long cells = 0;
        for (int l = 0; l < L; ++l) cells += lN[l];
        return 2 * cells + H;
    }

    void allocProj() {
        long long rows = rowCapacity();
        if (rows * ROW_W >= (1LL << 31)) throw std::invalid_argument("octree too large for 32-bit matrix indices");
        J.cnt = dalloc<int>(S);
        J.base = dalloc<int>(S);
        J.pO = dalloc<int>(S);
        J.pT = dalloc<int>(S);
        proj_alloc(J, rows, P.device, st, allocs);
    }

    // ---------------------------------------------------------------- step
    void checkStatus() {
        int s = 0;
        ck(cudaMemcpyAsync(&s, dStatus, sizeof(int), cudaMemcpyDeviceToHost, st), "status");
        ck(cudaStreamSynchronize(st), "sync");
        if (s != DS_OK) {
            int zero = 0;
            ck(cudaMemcpy(dStatus, &zero, sizeof(int), cudaMemcpyHostToDevice), "status reset");
            if (s == DS_WAIT_TIMEOUT) throw std::runtime_error("device wait timed out (status 3)");
            throw std::runtime_error("layout lookup failed on the device (status " + std::to_string(s) + ")");
        }
    }

    // factorises the system held in the projection workspace and runs the PCG; J.x holds the result
    // factorises the system held in the projection workspace and runs the PCG (mixed precision
    // when asked for and the FP32 preconditioner fits, else FP64); J.x holds the result
    void solveCurrent(double tol, int maxIter, int precision) {
        bool mixed = precision == ASTG_MIXED && J.pcActive32;
        launch_factor(d, J, P.omega, P.min_diag, epoch, st, &prof);
        bool owner = mixed || (J.pcActive && J.pcAsync);
        if (J.clusterSize > 0 || J.pcActive || mixed) launch_level_schedule(d, J, owner, st);
        ck(cudaEventRecord(evA, st), "event");
        lastOuter = 0;
        if (mixed) lastOuter = launch_pcg_mixed(d, J, tol, maxIter, 8, st, &prof);
        else launch_pcg_fp64(d, J, tol, maxIter, epoch, 8, st, &prof);
        ck(cudaEventRecord(evB, st), "event");
    }
    int lastOuter = 0;

    void project(double dt) {
        Fields& C = F[cur];
        launch_dof_numbering(d, dOpen, J, st);
        int n = 0;
        ck(cudaMemcpyAsync(&n, J.nDof, sizeof n, cudaMemcpyDeviceToHost, st), "dofs");
        ck(cudaStreamSynchronize(st), "dofs");
        if (n > J.rowsCap) throw std::runtime_error("projection has more rows than the workspace holds");
        select_preconditioner(J, n);
        launch_assemble(d, C, dOpen, J, dHoPtr, dHoIdx, dt, st);
        solveCurrent(P.tol, P.max_iter, P.precision);
        launch_pressure_update(d, C, dOpen, J.pO, J.pT, J.x, dt, st);
        readSolveStats();
    }

    // FmmLevelSetSolver3::extrapolate of "density" or "heat" (current buffer), in place
    double* exSdf = nullptr;
    size_t exSdfCap = 0;
    void* exScratch = nullptr;
    void extrapolate(const std::string& field, const double* sdf, int sres, double offset, double maxFactor,
                     astg_extrap_stats* stats) {
        if (field != "density" && field != "heat") throw std::invalid_argument("astg_extrapolate: field must be density or heat");
        if (sres < 2 || sres > 4096) throw std::invalid_argument("astg_extrapolate: sdf_res must be 2..4096");
        if (!(maxFactor >= 0) || !(offset == offset)) throw std::invalid_argument("astg_extrapolate: bad distance arguments");
        size_t n = (size_t)sres * sres * sres;
        if (n > exSdfCap) {
            exSdf = dalloc<double>(n);
            exSdfCap = n;
        }
        if (!exScratch) exScratch = dalloc<char>(extrapolate_scratch_bytes(S));
        ck(cudaMemcpyAsync(exSdf, sdf, n * sizeof(double), cudaMemcpyHostToDevice, st), "upload sdf");
        Fields& C = F[cur];
        double* oct = field == "density" ? C.dO : C.hO;
        double* til = field == "density" ? C.dT : C.hT;
        ck(cudaEventRecord(evA, st), "event");
        int passes = 0;
        long long got = launch_extrapolate(d, C, oct, til, exSdf, sres, offset, maxFactor, exScratch, &passes, st);
        ck(cudaEventRecord(evB, st), "event");
        ck(cudaStreamSynchronize(st), "extrapolate");
        if (got < 0) ck(cudaGetLastError(), "extrapolate");
        checkStatus();
        if (stats) {
            float ms = 0;
            cudaEventElapsedTime(&ms, evA, evB);
            stats->assigned = got;
            stats->passes = passes;
            stats->ms = ms;
        }
    }

    // ---------------------------------------------------------------- checkpoints
    // The binary dumps of src/viewer/grid_dump.cpp:280-615 (native little-endian, LP64): a level
    // count, then per level an entry count and the entries.  LayerNode3 (include/octree_layer3.h:
    // 11-20) and TiltENode (include/tilt_e_node.h:15-31) are written as their 24-byte structs; the
    // padding bytes carry no data (the reference leaves them uninitialised, they are written as 0).
    struct Reader {
        std::string file;
        std::vector<char> buf;
        size_t at = 0;
        explicit Reader(const std::string& f) : file(f) {
            std::ifstream in(f, std::ios::binary);
            if (!in) throw std::invalid_argument("checkpoint: cannot open " + f);
            buf.assign(std::istreambuf_iterator<char>(in), std::istreambuf_iterator<char>());
        }
        void raw(void* dst, size_t n) {
            if (at + n > buf.size()) throw std::invalid_argument("checkpoint " + file + ": truncated");
            memcpy(dst, buf.data() + at, n);
            at += n;
        }
        int i32() { int32_t v; raw(&v, 4); return v; }
        long long i64() { int64_t v; raw(&v, 8); return v; }
        double f64() { double v; raw(&v, 8); return v; }
        void end() {
            if (at != buf.size()) throw std::invalid_argument("checkpoint " + file + ": trailing bytes");
        }
    };
    struct Writer {
        std::string file;
        std::vector<char> buf;
        void raw(const void* src, size_t n) { buf.insert(buf.end(), (const char*)src, (const char*)src + n); }
        void i32(int v) { int32_t x = v; raw(&x, 4); }
        void i64(long long v) { int64_t x = v; raw(&x, 8); }
        void f64(double v) { raw(&v, 8); }
        void save() {
            // create the parent directories, as the reference's createDir does (src/util.cpp:50-58)
            for (size_t p = file.find('/', 1); p != std::string::npos; p = file.find('/', p + 1))
                mkdir(file.substr(0, p).c_str(), 0755);
            std::ofstream out(file, std::ios::binary);
            if (!out) throw std::invalid_argument("checkpoint: cannot write " + file);
            out.write(buf.data(), buf.size());
            if (!out) throw std::runtime_error("checkpoint: write failed: " + file);
        }
    };
    long long coor3(int s) const {  // PACK_COOR3 (include/macro.h:39): a layer's own keys, no level
        return ((long long)sx[s] << 40) | ((long long)sy[s] << 20) | (long long)sz[s];
    }
    long long lcoor(int s) const {  // PACK_LCOOR3, include/macro.h:39-45
        return ((long long)slev[s] << 60) | ((long long)sx[s] << 40) | ((long long)sy[s] << 20) | (long long)sz[s];
    }
    uint32_t nodeFlag(int s) const {  // VALID | IS_GHOST | GHOST_FROM_COARSE
        return 1u | ((sflag[s] & SF_GHOST) ? 2u : 0u) | ((sflag[s] & SF_FROM_COARSE) ? 4u : 0u);
    }
    void writeLayout(const std::string& f) {
        Writer w{f, {}};
        w.i32(L);
        for (int l = 0; l < L; ++l) {
            int n = lN[l], g = lG[l];
            w.i32(n + g);
            for (int i = 0; i < n + g; ++i) {
                int s = loff[l] + i;
                unsigned char node[24] = {0};
                uint64_t index = (uint64_t)i;
                uint16_t xyz[3] = {(uint16_t)sx[s], (uint16_t)sy[s], (uint16_t)sz[s]};
                uint32_t flag = nodeFlag(s);
                memcpy(node, &index, 8);
                memcpy(node + 8, xyz, 6);
                memcpy(node + 16, &flag, 4);
                w.i64(coor3(s));
                w.raw(node, 24);
            }
            w.i32(g);
            for (int i = n; i < n + g; ++i) w.i64(coor3(loff[l] + i));
            w.i32(n);
            for (int i = 0; i < n; ++i) w.i64(coor3(loff[l] + i));
        }
        w.i32((int)half.size());
        for (int hs : half) w.i64(lcoor(hs));
        w.save();
    }
    // readOctreeLayout3dBinary into an existing layout keeps the handle's octree: the file must
    // describe the same nodes (the library does not rebuild its octree on restart)
    void checkLayout(const std::string& f) {
        Reader r(f);
        auto fail = [&](const std::string& what) {
            throw std::runtime_error("checkpoint " + f + ": layout differs from the handle's (" + what + ")");
        };
        if (r.i32() != L) fail("level count");
        for (int l = 0; l < L; ++l) {
            int n = lN[l], g = lG[l];
            int m = r.i32();
            if (m != n + g) fail("nodes of level " + std::to_string(l));
            for (int k = 0; k < m; ++k) {
                long long c = r.i64();
                unsigned char node[24];
                r.raw(node, 24);
                uint64_t index;
                uint16_t xyz[3];
                uint32_t flag;
                memcpy(&index, node, 8);
                memcpy(xyz, node + 8, 6);
                memcpy(&flag, node + 16, 4);
                if (index >= (uint64_t)m) fail("node index");
                int s = loff[l] + (int)index;
                if (c != coor3(s) || xyz[0] != sx[s] || xyz[1] != sy[s] || xyz[2] != sz[s] || (flag & 7u) != nodeFlag(s))
                    fail("node of level " + std::to_string(l));
            }
            if (r.i32() != g) fail("ghosts of level " + std::to_string(l));
            for (int i = n; i < n + g; ++i)
                if (r.i64() != coor3(loff[l] + i)) fail("ghost order of level " + std::to_string(l));
            if (r.i32() != n) fail("cells of level " + std::to_string(l));
            for (int i = 0; i < n; ++i)
                if (r.i64() != coor3(loff[l] + i)) fail("cell order of level " + std::to_string(l));
        }
        if (r.i32() != (int)half.size()) fail("half tilts");
        for (int hs : half)
            if (r.i64() != lcoor(hs)) fail("half tilt order");
        r.end();
    }
    // per-level record arrays of `width` doubles per slot
    void writeLevels(Writer& w, const std::vector<double>& v, int width) {
        w.i32(L);
        for (int l = 0; l < L; ++l) {
            int m = lN[l] + lG[l];
            w.i32(m);
            w.raw(v.data() + (size_t)loff[l] * width, (size_t)m * width * 8);
        }
    }
    void readLevels(Reader& r, std::vector<double>& v, int width) {
        if (r.i32() != L) throw std::invalid_argument("checkpoint " + r.file + ": level count differs");
        v.assign((size_t)S * width, 0.0);
        for (int l = 0; l < L; ++l) {
            int m = lN[l] + lG[l];
            if (r.i32() != m) throw std::invalid_argument("checkpoint " + r.file + ": level size differs");
            r.raw(v.data() + (size_t)loff[l] * width, (size_t)m * width * 8);
        }
    }
    void saveCheckpoint(const char* layoutF, const char* tiltF, const char* densityF, const char* heatF,
                        const char* velocityF) {
        if (layoutF) writeLayout(layoutF);
        if (tiltF) {
            std::vector<double> e(S);
            std::vector<int32_t> fl(2 * (size_t)S);
            getArray("tilt_e", e.data(), 8 * (size_t)S);
            getArray("tilt_flags", fl.data(), 8 * (size_t)S);
            Writer w{tiltF, {}};
            w.i32(L);
            for (int l = 0; l < L; ++l) {
                int m = lN[l] + lG[l];
                w.i32(m);
                for (int i = 0; i < m; ++i) {
                    int s = loff[l] + i;
                    unsigned char node[24] = {0};
                    memcpy(node, &e[s], 8);
                    for (int b = 0; b < 6; ++b) node[8 + b] = (fl[2 * s] >> b) & 1;
                    int32_t dir = fl[2 * s + 1];
                    memcpy(node + 16, &dir, 4);
                    w.raw(node, 24);
                }
            }
            w.save();
        }
        auto scalar = [&](const char* f, const char* oct, const char* til) {
            std::vector<double> o(S), t(S);
            getArray(oct, o.data(), 8 * (size_t)S);
            getArray(til, t.data(), 8 * (size_t)S);
            Writer w{f, {}};
            writeLevels(w, o, 1);
            writeLevels(w, t, 1);
            w.save();
        };
        if (densityF) scalar(densityF, "density_oct", "density_tilt");
        if (heatF) scalar(heatF, "heat_oct", "heat_tilt");
        if (velocityF) {
            std::vector<double> mac(3 * (size_t)S), tv(8 * (size_t)S);
            getArray("mac", mac.data(), 24 * (size_t)S);
            getArray("tilt_vel", tv.data(), 64 * (size_t)S);
            Writer w{velocityF, {}};
            for (int a = 0; a < 3; ++a) {
                std::vector<double> u(mac.begin() + (size_t)a * S, mac.begin() + (size_t)(a + 1) * S);
                writeLevels(w, u, 1);
            }
            writeLevels(w, tv, 8);
            w.save();
        }
    }
    // OctreeOmniGridSolver3::restart (src/octree_omnigrid_solver3.cpp:1015-1057): tilt-E, density,
    // heat and velocity into both buffers, then the velocity ghosts, the dual grid and its ghosts
    // of both.  The boundary file is not read (the reference does not read it either); the
    // tilt open/closed layout flags stay as they are, as in the reference.
    void restart(const char* layoutF, const char* tiltF, const char* densityF, const char* heatF,
                 const char* velocityF) {
        if (!tiltF || !densityF || !heatF || !velocityF)
            throw std::invalid_argument("astg_restart: tilt, density, heat and velocity files are required");
        if (layoutF) checkLayout(layoutF);
        // read everything before touching the handle, so a bad file leaves the state as it was
        std::vector<double> e(S), dO, dT, hO, hT, ux, uy, uz, tv;
        std::vector<int32_t> fl(2 * (size_t)S);
        {
            Reader r(tiltF);
            if (r.i32() != L) throw std::invalid_argument("checkpoint " + r.file + ": level count differs");
            for (int l = 0; l < L; ++l) {
                int m = lN[l] + lG[l];
                if (r.i32() != m) throw std::invalid_argument("checkpoint " + r.file + ": level size differs");
                for (int i = 0; i < m; ++i) {
                    int s = loff[l] + i;
                    unsigned char node[24];
                    r.raw(node, 24);
                    memcpy(&e[s], node, 8);
                    int f = 0;
                    for (int b = 0; b < 6; ++b) f |= (node[8 + b] ? 1 : 0) << b;
                    int32_t dir;
                    memcpy(&dir, node + 16, 4);
                    fl[2 * s] = f;
                    fl[2 * s + 1] = dir;
                }
            }
            r.end();
        }
        {
            Reader r(densityF);
            readLevels(r, dO, 1);
            readLevels(r, dT, 1);
            r.end();
        }
        {
            Reader r(heatF);
            readLevels(r, hO, 1);
            readLevels(r, hT, 1);
            r.end();
        }
        {
            Reader r(velocityF);
            readLevels(r, ux, 1);
            readLevels(r, uy, 1);
            readLevels(r, uz, 1);
            readLevels(r, tv, 8);
            r.end();
        }
        std::vector<double> mac;
        mac.reserve(3 * (size_t)S);
        mac.insert(mac.end(), ux.begin(), ux.end());
        mac.insert(mac.end(), uy.begin(), uy.end());
        mac.insert(mac.end(), uz.begin(), uz.end());
        for (const char* p : {"", "t_"}) {
            std::string q = p;
            setArray(q + "tilt_e", e.data(), 8 * (size_t)S);
            setArray(q + "tilt_flags", fl.data(), 8 * (size_t)S);
            setArray(q + "density_oct", dO.data(), 8 * (size_t)S);
            setArray(q + "density_tilt", dT.data(), 8 * (size_t)S);
            setArray(q + "heat_oct", hO.data(), 8 * (size_t)S);
            setArray(q + "heat_tilt", hT.data(), 8 * (size_t)S);
            setArray(q + "mac", mac.data(), 24 * (size_t)S);
            setArray(q + "tilt_vel", tv.data(), 64 * (size_t)S);
        }
        for (int b : {cur, 1 - cur}) {
            launch_velocity_ghost(d, F[b], dLastWriter, st);
            launch_dual(d, F[b], st);
        }
        ck(cudaStreamSynchronize(st), "restart");
        checkStatus();
    }

    void readSolveStats() {
        int isc[ISC_COUNT], n = 0, nnz = 0;
        double sc[SC_COUNT];
        ck(cudaMemcpyAsync(isc, J.isc, sizeof isc, cudaMemcpyDeviceToHost, st), "stats");
        ck(cudaMemcpyAsync(sc, J.sc, sizeof sc, cudaMemcpyDeviceToHost, st), "stats");
        ck(cudaMemcpyAsync(&n, J.nDof, sizeof n, cudaMemcpyDeviceToHost, st), "stats");
        ck(cudaMemcpyAsync(&nnz, J.nnz, sizeof nnz, cudaMemcpyDeviceToHost, st), "stats");
        ck(cudaStreamSynchronize(st), "project");
        if (g_cluster_error != cudaSuccess) {
            cudaError_t e = g_cluster_error;
            g_cluster_error = cudaSuccess;
            ck(e, "cluster sweep launch");
        }
        float ms = 0;
        cudaEventElapsedTime(&ms, evA, evB);
        last.iterations = isc[ISC_ITERS];
        last.converged = isc[ISC_CONVERGED];
        last.outer = lastOuter;
        last.n = n;
        last.nnz = nnz;
        last.residual = sc[SC_RESID];
        last.tolerance = sc[SC_TOL];
        last.ms = ms;
    }

    // PCGSolver::solve on a caller-supplied CSR system (uses and overwrites the projection
    // workspace of the handle)
    void solveExternal(int n, const int32_t* rowptr, const int32_t* col, const double* val, const double* b,
                       double* x, double tol, int maxIter, int precision, astg_solve_stats* stats) {
        long long rows = J.rowsCap;
        if (n <= 0 || n > rows)
            throw std::invalid_argument("astg_solve: n exceeds the handle's capacity (2 x cells + half tilts)");
        long long nnz = rowptr[n];
        if (nnz <= 0 || nnz > rows * ROW_W) throw std::invalid_argument("astg_solve: too many non-zeros for the workspace");
        for (int i = 0; i < n; ++i)
            if (rowptr[i + 1] - rowptr[i] > ROW_W || rowptr[i + 1] < rowptr[i])
                throw std::invalid_argument("astg_solve: malformed row pointer or row longer than 32 entries");
        int nn = n, nz = (int)nnz;
        ck(cudaMemcpyAsync(J.nDof, &nn, sizeof(int), cudaMemcpyHostToDevice, st), "upload");
        ck(cudaMemcpyAsync(J.nnz, &nz, sizeof(int), cudaMemcpyHostToDevice, st), "upload");
        ck(cudaMemcpyAsync(J.rowPtr, rowptr, sizeof(int) * (n + 1), cudaMemcpyHostToDevice, st), "upload");
        ck(cudaMemcpyAsync(J.col, col, sizeof(int) * nnz, cudaMemcpyHostToDevice, st), "upload");
        ck(cudaMemcpyAsync(J.val, val, sizeof(double) * nnz, cudaMemcpyHostToDevice, st), "upload");
        ck(cudaMemcpyAsync(J.b, b, sizeof(double) * n, cudaMemcpyHostToDevice, st), "upload");
        select_preconditioner(J, n);
        launch_external_system(d, J, n, st);
        checkStatus();
        solveCurrent(tol, maxIter, precision);
        readSolveStats();
        checkStatus();
        ck(cudaMemcpyAsync(x, J.x, sizeof(double) * n, cudaMemcpyDeviceToHost, st), "download");
        ck(cudaStreamSynchronize(st), "solve");
        if (stats) *stats = last;
    }

    // ---- several right-hand sides of one matrix (astg_solve_batch).  The matrix, its MIC(0) factor
    // and the level schedule are computed once and shared; each lane owns the PCG's vectors and
    // scalars and a stream and runs the launches astg_solve runs, so every solution is the one
    // astg_solve returns, bit for bit.  A solve keeps one 16-CTA cluster busy in its
    // preconditioner, so lanes on other SMs use the GPU that a single solve leaves idle; lanes are
    // driven by one host thread each.
    struct Lane {
        double *b = nullptr, *x = nullptr, *r = nullptr, *s = nullptr, *z = nullptr, *part = nullptr, *sc = nullptr;
        double *rl = nullptr, *yl = nullptr;
        float *rl32 = nullptr, *yl32 = nullptr, *e32 = nullptr, *r32 = nullptr, *s32 = nullptr, *z32 = nullptr,
              *q32 = nullptr;
        int *isc = nullptr, *done = nullptr, *hostDone = nullptr;
        unsigned long long* amax = nullptr;
        cudaStream_t st = nullptr;
        cudaEvent_t e0 = nullptr, e1 = nullptr;
    };
    std::vector<Lane> lanes;
    void ensureLanes(int k) {
        const size_t rows = J.rowsCap;
        while ((int)lanes.size() < k) {
            Lane L;
            L.b = dalloc<double>(rows); L.x = dalloc<double>(rows); L.r = dalloc<double>(rows);
            L.s = dalloc<double>(rows); L.z = dalloc<double>(rows);
            L.part = dalloc<double>((rows + 2047) / 2048 + 1);
            L.sc = dalloc<double>(SC_COUNT);
            L.isc = dalloc<int>(ISC_COUNT);
            L.amax = dalloc<unsigned long long>(1);
            L.done = dalloc<int>(1);
            if (J.rl) L.rl = dalloc<double>(rows);
            if (J.yl) L.yl = dalloc<double>(rows);
            if (J.rl32) {
                L.rl32 = dalloc<float>(rows); L.yl32 = dalloc<float>(rows); L.e32 = dalloc<float>(rows);
                L.r32 = dalloc<float>(rows); L.s32 = dalloc<float>(rows); L.z32 = dalloc<float>(rows);
                L.q32 = dalloc<float>(rows);
            }
            lanes.push_back(L);  // owned from here on: the destructor releases what follows
            Lane& M = lanes.back();
            ck(cudaMallocHost(&M.hostDone, sizeof(int)), "cudaMallocHost");
            ck(cudaStreamCreateWithFlags(&M.st, cudaStreamNonBlocking), "stream");
            ck(cudaEventCreate(&M.e0), "event");
            ck(cudaEventCreate(&M.e1), "event");
        }
        // dalloc zeroes on the handle's stream: done before any lane stream touches the memory
        ck(cudaStreamSynchronize(st), "lanes");
    }
    void freeLanes() {
        for (Lane& L : lanes) {
            if (L.st) cudaStreamSynchronize(L.st);
            if (L.e0) cudaEventDestroy(L.e0);
            if (L.e1) cudaEventDestroy(L.e1);
            if (L.st) cudaStreamDestroy(L.st);
            if (L.hostDone) cudaFreeHost(L.hostDone);
        }
        lanes.clear();
    }
    // the handle's workspace with lane L's vectors and scalars
    Proj laneView(const Lane& L) const {
        Proj Q = J;
        Q.b = L.b; Q.x = L.x; Q.r = L.r; Q.s = L.s; Q.z = L.z; Q.part = L.part; Q.sc = L.sc; Q.isc = L.isc;
        Q.amax = L.amax; Q.done = L.done; Q.hostDone = L.hostDone;
        Q.rl = L.rl; Q.yl = L.yl;
        Q.rl32 = L.rl32; Q.yl32 = L.yl32; Q.e32 = L.e32; Q.r32 = L.r32; Q.s32 = L.s32; Q.z32 = L.z32; Q.q32 = L.q32;
        return Q;
    }
    void solveBatch(int n, const int32_t* rowptr, const int32_t* col, const double* val, int nrhs, const double* B,
                    double* X, double tol, int maxIter, int precision, astg_solve_stats* stats, double* wallMs) {
        long long rows = J.rowsCap;
        if (nrhs <= 0) throw std::invalid_argument("astg_solve_batch: nrhs must be positive");
        if (n <= 0 || n > rows)
            throw std::invalid_argument("astg_solve_batch: n exceeds the handle's capacity (2 x cells + half tilts)");
        long long nnz = rowptr[n];
        if (nnz <= 0 || nnz > rows * ROW_W) throw std::invalid_argument("astg_solve_batch: too many non-zeros for the workspace");
        for (int i = 0; i < n; ++i)
            if (rowptr[i + 1] - rowptr[i] > ROW_W || rowptr[i + 1] < rowptr[i])
                throw std::invalid_argument("astg_solve_batch: malformed row pointer or row longer than 32 entries");
        const auto t0 = std::chrono::steady_clock::now();
        int nn = n, nz = (int)nnz;
        ck(cudaMemcpyAsync(J.nDof, &nn, sizeof(int), cudaMemcpyHostToDevice, st), "upload");
        ck(cudaMemcpyAsync(J.nnz, &nz, sizeof(int), cudaMemcpyHostToDevice, st), "upload");
        ck(cudaMemcpyAsync(J.rowPtr, rowptr, sizeof(int) * (n + 1), cudaMemcpyHostToDevice, st), "upload");
        ck(cudaMemcpyAsync(J.col, col, sizeof(int) * nnz, cudaMemcpyHostToDevice, st), "upload");
        ck(cudaMemcpyAsync(J.val, val, sizeof(double) * nnz, cudaMemcpyHostToDevice, st), "upload");
        select_preconditioner(J, n);
        launch_external_system(d, J, n, st);
        checkStatus();
        const bool mixed = precision == ASTG_MIXED && J.pcActive32;
        launch_factor(d, J, P.omega, P.min_diag, epoch, st, nullptr);
        const bool owner = mixed || (J.pcActive && J.pcAsync);
        if (J.clusterSize > 0 || J.pcActive || mixed) launch_level_schedule(d, J, owner, st);
        ck(cudaStreamSynchronize(st), "factor");
        checkStatus();
        // lanes only with the barrier-free preconditioner: the other forms hand rows out from one
        // counter and epoch flags of the handle
        const bool concurrent = mixed || (J.pcActive && J.pcAsync);
        const int k = concurrent ? std::min(nrhs, precond_concurrency(J, mixed)) : 0;
        auto record = [&](int i, int outer, const int* isc, const double* sc, float ms) {
            astg_solve_stats o{};
            o.iterations = isc[ISC_ITERS];
            o.converged = isc[ISC_CONVERGED];
            o.outer = outer;
            o.n = n;
            o.nnz = (int)nnz;
            o.residual = sc[SC_RESID];
            o.tolerance = sc[SC_TOL];
            o.ms = ms;
            if (stats) stats[i] = o;
            last = o;
        };
        if (k == 0) {  // one after another on the handle's own workspace
            for (int i = 0; i < nrhs; ++i) {
                ck(cudaMemcpyAsync(J.b, B + (size_t)i * n, sizeof(double) * n, cudaMemcpyHostToDevice, st), "upload");
                ck(cudaEventRecord(evA, st), "event");
                int outer = 0;
                if (mixed) outer = launch_pcg_mixed(d, J, tol, maxIter, 8, st, nullptr);
                else launch_pcg_fp64(d, J, tol, maxIter, epoch, 8, st, nullptr);
                ck(cudaEventRecord(evB, st), "event");
                ck(cudaMemcpyAsync(X + (size_t)i * n, J.x, sizeof(double) * n, cudaMemcpyDeviceToHost, st), "download");
                int isc[ISC_COUNT];
                double sc[SC_COUNT];
                ck(cudaMemcpyAsync(isc, J.isc, sizeof isc, cudaMemcpyDeviceToHost, st), "stats");
                ck(cudaMemcpyAsync(sc, J.sc, sizeof sc, cudaMemcpyDeviceToHost, st), "stats");
                ck(cudaStreamSynchronize(st), "solve");
                float ms = 0;
                cudaEventElapsedTime(&ms, evA, evB);
                record(i, outer, isc, sc, ms);
            }
        } else {
            ensureLanes(k);
            std::vector<std::exception_ptr> errs(k);
            std::vector<std::vector<std::pair<int, std::vector<double>>>> out(k);
            std::vector<std::thread> th;
            for (int w = 0; w < k; ++w)
                th.emplace_back([&, w] {
                    try {
                        ck(cudaSetDevice(P.device), "cudaSetDevice");
                        Lane& L = lanes[w];
                        Proj Q = laneView(L);
                        int ep = 0;  // the barrier-free forms use no epoch flags
                        for (int i = w; i < nrhs; i += k) {
                            ck(cudaMemcpyAsync(Q.b, B + (size_t)i * n, sizeof(double) * n, cudaMemcpyHostToDevice, L.st), "upload");
                            ck(cudaEventRecord(L.e0, L.st), "event");
                            int outer = 0;
                            if (mixed) outer = launch_pcg_mixed(d, Q, tol, maxIter, 8, L.st, nullptr);
                            else launch_pcg_fp64(d, Q, tol, maxIter, ep, 8, L.st, nullptr);
                            ck(cudaEventRecord(L.e1, L.st), "event");
                            ck(cudaMemcpyAsync(X + (size_t)i * n, Q.x, sizeof(double) * n, cudaMemcpyDeviceToHost, L.st), "download");
                            int isc[ISC_COUNT];
                            double sc[SC_COUNT];
                            ck(cudaMemcpyAsync(isc, Q.isc, sizeof isc, cudaMemcpyDeviceToHost, L.st), "stats");
                            ck(cudaMemcpyAsync(sc, Q.sc, sizeof sc, cudaMemcpyDeviceToHost, L.st), "stats");
                            ck(cudaStreamSynchronize(L.st), "solve");
                            float ms = 0;
                            cudaEventElapsedTime(&ms, L.e0, L.e1);
                            out[w].push_back({i, {(double)isc[ISC_ITERS], (double)isc[ISC_CONVERGED], (double)outer,
                                                  sc[SC_RESID], sc[SC_TOL], (double)ms}});
                        }
                    } catch (...) {
                        errs[w] = std::current_exception();
                    }
                });
            for (auto& t : th) t.join();
            for (auto& e : errs)
                if (e) std::rethrow_exception(e);
            for (int w = 0; w < k; ++w)
                for (auto& rec : out[w]) {
                    const std::vector<double>& v = rec.second;
                    int isc[ISC_COUNT] = {(int)v[0], (int)v[1]};
                    double sc[SC_COUNT] = {};
                    sc[SC_RESID] = v[3];
                    sc[SC_TOL] = v[4];
                    record(rec.first, (int)v[2], isc, sc, (float)v[5]);
                }
        }
        if (g_cluster_error != cudaSuccess) {
            cudaError_t e = g_cluster_error;
            g_cluster_error = cudaSuccess;
            ck(e, "cluster sweep launch");
        }
        checkStatus();
        lastLanes = std::max(k, 1);
        if (wallMs)
            *wallMs = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
    int lastLanes = 1;

    void stage(int id, double dt) {
        Fields& C = F[cur];
        Fields& N = F[1 - cur];
        switch (id) {
            case 0:
                if (P.src_r > 0) launch_source(d, C, st);
                if (firstSource) {
                    launch_scalar_ghost(d, C.dO, C.dT, C.te, C.tf, st);
                    launch_scalar_ghost(d, C.hO, C.hT, C.te, C.tf, st);
                    firstSource = false;
                }
                break;
            case 1:
                if (d.sdf) launch_collider_wipe(d, C, st);  // wipeBoundary (:226)
                if (J.refOrder) launch_mean_temperature_ref(d, C.hO, refWorkers, dAmb, st);
                else launch_mean_temperature(d, C.hO, dParts, dPartOff, partOff.data(), dAmb, st);
                launch_force(d, C, dOpen, dAmb, dt, st);
                break;
            case 2: constrainVelocity(C); break;
            case 3: project(dt); break;
            case 4:
                constrainVelocity(C);
                launch_dual_update(d, C, st);
                if (d.sdf) launch_collider_dual(d, C, st);
                launch_dual_ghost(d, C, st);
                break;
            case 5: {
                // the velocity is final for this step: its tilt corrections once, read by every sample
                if (!dCorrT) dCorrT = dalloc<double>((size_t)3 * S);
                Fields Cc = C;
                Cc.corrT = dCorrT;
                launch_tilt_corr(d, Cc, dCorrT, st);
                if (P.tilt_adaptivity) launch_adjust(d, Cc, N, dOpen, dFixed, dt, st);
                launch_advect_scalars(d, Cc, N, dOpen, dt, st);
                launch_advect_velocity(d, Cc, N, dt, st);
                cur = 1 - cur;
                launch_decay(d, F[cur], st);
                break;
            }
            default: throw std::invalid_argument("stage must be 0..5");
        }
        ck(cudaGetLastError(), "launch");
    }

    void step(double dt, astg_step_stats* out) {
        ck(cudaEventRecord(ev0, st), "event");
        double* advDst = advTarget;
        if (T.on && T.recording) advDst = tapeBeforeStep(dt);
        for (int i = 0; i < 6; ++i) {
            if (i == 5 && advDst) saveAdvectionInput(advDst);
            if (i == 1) ck(cudaEventRecord(evF0, st), "event");
            if (i == 3) ck(cudaEventRecord(evF1, st), "event");
            if (i == 5) ck(cudaEventRecord(evAdv, st), "event");
            stage(i, dt);
        }
        if (T.on && T.recording) ++T.steps;
        ck(cudaEventRecord(ev1, st), "event");
        checkStatus();
        if (out) {
            float ms = 0;
            cudaEventElapsedTime(&ms, ev0, ev1);
            float msF = 0, msA = 0;
            cudaEventElapsedTime(&msF, evF0, evF1);
            cudaEventElapsedTime(&msA, evAdv, ev1);
            out->solve = last;
            out->ms_total = ms;
            out->ms_project = last.ms;
            out->ms_force = msF;
            out->ms_advect = msA;
        }
    }

    // ---------------------------------------------------------------- adaptive update
    // Solver::update's adaptive branch (src/solver.cpp:21-41, useFixedTimeStep = false) with
    // numberOfSubTimeSteps / cfl (src/octree_omnigrid_solver3.cpp:1060-1122)
    double maxCfl = 3.0;  // the reference's default (include/octree_omnigrid_solver3.h:84)
    bool updateConverged = true;  // every sub-step's solve of the last update converged
    unsigned long long* dMaxV = nullptr;
    double maxFace() {
        if (!dMaxV) dMaxV = dalloc<unsigned long long>(1);
        ck(cudaMemsetAsync(dMaxV, 0, sizeof(unsigned long long), st), "memset");
        launch_max_face(d, F[cur].mac, dMaxV, st);
        unsigned long long bits = 0;
        ck(cudaMemcpyAsync(&bits, dMaxV, sizeof bits, cudaMemcpyDeviceToHost, st), "max velocity");
        ck(cudaStreamSynchronize(st), "sync");
        double v;
        memcpy(&v, &bits, sizeof v);
        return v;
    }
    // cfl(dt): dt * maxV / delta_h (delta_h = the finest spacing), truncated to int as the reference
    // returns it
    int cfl(double dt) { return (int)(dt * maxFace() / dx); }
    int numberOfSubTimeSteps(double dt) {
        int k = (int)std::ceil(cfl(dt) / maxCfl);
        return k > 1 ? k : 1;
    }
    // sub-steps of remaining / k while more than EPSILON remains, k recomputed from the current
    // velocity before each; the statistics are the last sub-step's, with the times summed
    void update(double dt, int* substeps, astg_step_stats* out) {
        double remaining = dt;
        int n = 0;
        astg_step_stats one{}, sum{};
        updateConverged = true;
        while (remaining > std::numeric_limits<double>::epsilon()) {
            int k = numberOfSubTimeSteps(remaining);
            double actual = remaining / (double)k;
            step(actual, &one);
            if (last.converged == 0) updateConverged = false;
            sum.ms_total += one.ms_total;
            sum.ms_force += one.ms_force;
            sum.ms_project += one.ms_project;
            sum.ms_advect += one.ms_advect;
            remaining -= actual;
            ++n;
        }
        if (substeps) *substeps = n;
        if (out) {
            *out = one;
            out->ms_total = sum.ms_total;
            out->ms_force = sum.ms_force;
            out->ms_project = sum.ms_project;
            out->ms_advect = sum.ms_advect;
        }
    }

    // ---------------------------------------------------------------- adjoint
    // Reverse mode of astg_step with the topology frozen (tilt adaptivity off).  The cotangent of
    // the state lives in GA[ga] (Fields layout; te / tf point at the frozen forward arrays), the
    // source-density gradients in dGsO / dGsT.  Only the advection transpose reads field values of
    // the forward state; the other stages are linear in the state with frozen coefficients.
    Fields GA[2]{};
    int ga = 0;
    double* dGsO = nullptr;
    double* dGsT = nullptr;
    double* dGamb = nullptr;
    double* dAdjB = nullptr;  // rows: cotangent of the pressure
    int* dOwnJ = nullptr;
    int* dOwnH = nullptr;
    double ambInvCount = 0;
    bool adjReady = false;
    int adjN = -1;            // rows of the factorised system the adjoint solves use (-1: none)
    long long adjSolves = 0, adjIters = 0;

    void allocAdjoint() {
        if (adjReady) return;
        for (int b = 0; b < 2; ++b) {
            GA[b].dO = dalloc<double>(S); GA[b].dT = dalloc<double>(S);
            GA[b].hO = dalloc<double>(S); GA[b].hT = dalloc<double>(S);
            GA[b].mac = dalloc<double>((size_t)3 * S);
            GA[b].tv = dalloc<double>((size_t)8 * S);
            GA[b].dualO = dalloc<double>((size_t)3 * S);
            GA[b].dualT = dalloc<double>((size_t)3 * S);
        }
        dGsO = dalloc<double>(S);
        dGsT = dalloc<double>(S);
        dGamb = dalloc<double>(1);
        dAdjB = dalloc<double>(J.rowsCap);
        dOwnJ = dalloc<int>(S);
        dOwnH = dalloc<int>(S);
        long long count = 0;
        for (int l = 0; l < L; ++l) count += (long long)(lN[l] + lG[l]) * (l == 0 ? 1 : 8);
        ambInvCount = 1.0 / (double)count;
        adjReady = true;
        adjustFrozen();
    }
    // the frozen tilt-E arrays the transposes read, and the single writers of the ghost passes
    void adjustFrozen() {
        for (int b = 0; b < 2; ++b) { GA[b].te = F[cur].te; GA[b].tf = F[cur].tf; }
        launch_adj_owners(d, F[cur].te, dOwnJ, dOwnH, st);
    }
    void zeroCotangent(Fields& g) {
        ck(cudaMemsetAsync(g.dO, 0, 8 * (size_t)S, st), "memset");
        ck(cudaMemsetAsync(g.dT, 0, 8 * (size_t)S, st), "memset");
        ck(cudaMemsetAsync(g.hO, 0, 8 * (size_t)S, st), "memset");
        ck(cudaMemsetAsync(g.hT, 0, 8 * (size_t)S, st), "memset");
        ck(cudaMemsetAsync(g.mac, 0, 24 * (size_t)S, st), "memset");
        ck(cudaMemsetAsync(g.tv, 0, 64 * (size_t)S, st), "memset");
        ck(cudaMemsetAsync(g.dualO, 0, 24 * (size_t)S, st), "memset");
        ck(cudaMemsetAsync(g.dualT, 0, 24 * (size_t)S, st), "memset");
    }
    void resetAdjoint() {
        allocAdjoint();
        zeroCotangent(GA[ga]);
        ck(cudaMemsetAsync(dGsO, 0, 8 * (size_t)S, st), "memset");
        ck(cudaMemsetAsync(dGsT, 0, 8 * (size_t)S, st), "memset");
        ck(cudaStreamSynchronize(st), "sync");
    }
    // assembles and factorises the (state-independent) pressure matrix for the adjoint solves
    void prepareAdjointSystem() {
        launch_dof_numbering(d, dOpen, J, st);
        int n = 0;
        ck(cudaMemcpyAsync(&n, J.nDof, sizeof n, cudaMemcpyDeviceToHost, st), "dofs");
        ck(cudaStreamSynchronize(st), "dofs");
        if (n > J.rowsCap) throw std::runtime_error("projection has more rows than the workspace holds");
        select_preconditioner(J, n);
        launch_assemble(d, F[cur], dOpen, J, dHoPtr, dHoIdx, 1.0, st);
        launch_factor(d, J, P.omega, P.min_diag, epoch, st, nullptr);
        bool mixed = P.precision == ASTG_MIXED && J.pcActive32;
        bool owner = mixed || (J.pcActive && J.pcAsync);
        if (J.clusterSize > 0 || J.pcActive || mixed) launch_level_schedule(d, J, owner, st);
        adjN = n;
    }
    // transpose of project(): u_bar -> p_bar (pressure update), lambda = A^-1 p_bar (A is
    // symmetric), u_bar += B^T lambda (right-hand side of the assembly)
    void projectAdjoint(double dt, const Fields& C, Fields& g) {
        if (adjN < 0) prepareAdjointSystem();
        ck(cudaMemsetAsync(dAdjB, 0, 8 * (size_t)J.rowsCap, st), "memset");
        launch_adj_pressure_update(d, C, g, dOpen, J.pO, J.pT, dAdjB, dt, st);
        ck(cudaMemcpyAsync(J.b, dAdjB, 8 * (size_t)adjN, cudaMemcpyDeviceToDevice, st), "copy");
        bool mixed = P.precision == ASTG_MIXED && J.pcActive32;
        if (mixed) launch_pcg_mixed(d, J, P.tol, P.max_iter, 8, st, nullptr);
        else launch_pcg_fp64(d, J, P.tol, P.max_iter, epoch, 8, st, nullptr);
        int it[2] = {0, 0};
        ck(cudaMemcpyAsync(it, J.isc, sizeof it, cudaMemcpyDeviceToHost, st), "iters");
        ck(cudaStreamSynchronize(st), "sync");
        ++adjSolves;
        adjIters += it[ISC_ITERS];
        launch_adj_rhs(d, C, g, dOpen, J, dHoPtr, dHoIdx, J.x, P.rho / dt, st);
    }
    // cotangent of a stage's input from that of its output (GA[ga], in place); C is the stage's
    // input state (field values are read by stage 5 only)
    void adjStage(int id, double dt, const Fields& C, bool firstSrc) {
        Fields& g = GA[ga];
        switch (id) {
            case 0:
                if (firstSrc) {
                    launch_adj_scalar_ghost(d, g.hO, g.hT, g.te, g.tf, dOwnJ, dOwnH, st);
                    launch_adj_scalar_ghost(d, g.dO, g.dT, g.te, g.tf, dOwnJ, dOwnH, st);
                }
                if (P.src_r > 0) launch_adj_source(d, g, dGsO, dGsT, st);
                break;
            case 1: launch_adj_force(d, C, g, dOpen, dt, dGamb, ambInvCount, st); break;
            case 2: launch_adj_walls_and_ghost(d, C, g, dLastWriter, st); break;
            case 3: projectAdjoint(dt, C, g); break;
            case 4:
                launch_adj_dual(d, C, g, dOwnJ, dOwnH, st);
                launch_adj_walls_and_ghost(d, C, g, dLastWriter, st);
                break;
            case 5: {
                Fields& gc = GA[1 - ga];
                zeroCotangent(gc);
                launch_adj_advect(d, C, gc, g, dOpen, dt, dOwnJ, dOwnH, st);
                ga = 1 - ga;
                break;
            }
            default: throw std::invalid_argument("stage must be 0..5");
        }
        ck(cudaGetLastError(), "launch");
    }
    void requireFrozen(const char* what) {
        if (P.tilt_adaptivity) throw std::invalid_argument(std::string(what) + ": needs tilt adaptivity off (frozen topology)");
        if (d.sdf) throw std::invalid_argument(std::string(what) + ": reverse mode is not available with a collider");
    }

    // ---------------------------------------------------------------- collider
    // OmniBoundarySolver3::updateCollider (src/omni_boundary_solver3.cpp:17-32) takes a shape and
    // samples its SDF at the finest cell centres; here the caller passes that grid (res^3 doubles,
    // index (z * res + y) * res + x) or a sphere whose grid is computed on the device (the stock
    // obstacle), or nothing to remove the collider.  The cut-cell weights
    // (initCuttingCellWeights, which initialize() runs right after initObstacle) are recomputed on
    // the device and copied back so astg_get("w_mac" / "w_tilt") returns them.
    double* dSdf = nullptr;
    uint16_t* dColMask = nullptr;
    int* dHalfDir = nullptr;
    double* dMacBefore = nullptr;
    double* dCorrT = nullptr;  // tilt corrections of the current velocity (stage 5)
    void setCollider(const double* sdf, size_t bytes) {
        size_t n = (size_t)res * res * res;
        if (bytes == 0) {
            d.sdf = nullptr;
            d.colMask = nullptr;
            wMac = wMac0;
            wTilt = wTilt0;
            up(const_cast<double*>(d.wMac), wMac.data(), wMac.size());
            up(const_cast<double*>(d.wTilt), wTilt.data(), wTilt.size());
            return;
        }
        if (bytes != 8 * n) throw std::invalid_argument("astg_set collider_sdf: expected res^3 doubles (" + std::to_string(8 * n) + " bytes)");
        if (T.on) throw std::invalid_argument("astg_set collider_sdf: a tape is active");
        allocCollider();
        up(dSdf, sdf, n);
        colliderFromSdf();
    }
    // the stock obstacle: a sphere's SDF grid computed on the device (radius <= 0 removes the collider)
    void setColliderSphere(double cx, double cy, double cz, double r) {
        if (!(r > 0)) {
            setCollider(nullptr, 0);
            return;
        }
        if (T.on) throw std::invalid_argument("astg_set_collider_sphere: a tape is active");
        allocCollider();
        launch_collider_sphere_sdf(res, cx, cy, cz, r, dSdf, st);
        colliderFromSdf();
    }
    void allocCollider() {
        size_t n = (size_t)res * res * res;
        if (!dSdf) {
            dSdf = dalloc<double>(n);
            dColMask = dalloc<uint16_t>(S);
            dMacBefore = dalloc<double>((size_t)3 * S);
            std::vector<int> dirs(H > 0 ? H : 1, 0);
            for (int i = 0; i < H; ++i) dirs[i] = te[0][half[i]].dir;
            dHalfDir = upload(dirs);
        }
    }
    // the cut-cell weights and solid masks of the SDF grid in dSdf
    void colliderFromSdf() {
        d.sdf = dSdf;
        d.colMask = dColMask;
        launch_collider_setup(d, dHalfDir, dColMask, const_cast<double*>(d.wMac), const_cast<double*>(d.wTilt), st);
        down(d.wMac, wMac.data(), wMac.size());
        down(d.wTilt, wTilt.data(), wTilt.size());
    }
    // constrainVelocity(MAC) + walls, constrainVelocity(tilt), velocity ghosts (onUpdate :230-232, :236-238)
    void constrainVelocity(Fields& C) {
        if (d.sdf) launch_collider_mac(d, C, dMacBefore, st);
        launch_walls(d, C.mac, st);
        if (d.sdf) launch_collider_tilt(d, C, st);
        launch_velocity_ghost(d, C, dLastWriter, st);
    }
    // astg_stage_vjp: the current state is the stage's input
    void stageVjp(int id, double dt) {
        requireFrozen("astg_stage_vjp");
        allocAdjoint();
        adjustFrozen();
        if (id == 3) prepareAdjointSystem();
        adjStage(id, dt, F[cur], firstSource);
        checkStatus();
    }

    // ---- tape: state needed to run the step transposes in reverse
    // per step: the advection input (density, heat, MAC, dual), 13 S doubles; per checkpoint: both
    // buffers of the state (dO dT hO hT mac tv dualO dualT), 42 S doubles
    struct Tape {
        bool on = false;
        int recording = 1;
        int every = 0;  // 0: keep each step's advection input, else a checkpoint every `every` steps
        int steps = 0;
        std::vector<double> dt;
        std::vector<uint8_t> first;
        std::vector<double*> adv;   // store mode: per step; checkpoint mode: per step of a segment
        std::vector<double*> ckpt;
        std::vector<int> ckCur;
        std::vector<uint8_t> ckFirst;
        double* endState = nullptr;
        long long bytes = 0;
    } T;
    double* advTarget = nullptr;  // step() copies the advection input here when set
    static constexpr size_t ADV_DOUBLES = 13;
    static constexpr size_t FULL_DOUBLES = 42;
    double* rawAlloc(size_t doubles) {
        void* p = nullptr;
        ck(cudaMalloc(&p, doubles * 8 * (size_t)S), "cudaMalloc (tape)");
        return (double*)p;
    }
    double* tapeAlloc(size_t doubles) {
        double* p = rawAlloc(doubles);
        T.bytes += (long long)(doubles * 8 * (size_t)S);
        return p;
    }
    void freeTape() {
        if (st) cudaStreamSynchronize(st);
        for (double* p : T.adv) cudaFree(p);
        for (double* p : T.ckpt) cudaFree(p);
        if (T.endState) cudaFree(T.endState);
        T = Tape{};
    }
    void copyD(double* dst, const double* src, size_t n) {
        ck(cudaMemcpyAsync(dst, src, n * 8, cudaMemcpyDeviceToDevice, st), "copy");
    }
    void saveAdvectionInput(double* o) {
        const Fields& C = F[cur];
        size_t n = S;
        copyD(o, C.dO, n); copyD(o + n, C.dT, n); copyD(o + 2 * n, C.hO, n); copyD(o + 3 * n, C.hT, n);
        copyD(o + 4 * n, C.mac, 3 * n); copyD(o + 7 * n, C.dualO, 3 * n); copyD(o + 10 * n, C.dualT, 3 * n);
    }
    Fields advectionView(double* o) const {
        Fields C = F[cur];
        size_t n = S;
        C.dO = o; C.dT = o + n; C.hO = o + 2 * n; C.hT = o + 3 * n;
        C.mac = o + 4 * n; C.dualO = o + 7 * n; C.dualT = o + 10 * n;
        C.tv = nullptr;
        return C;
    }
    void saveFull(double* o) {
        size_t n = S;
        for (int b = 0; b < 2; ++b) {
            double* q = o + (size_t)b * 21 * n;
            const Fields& G = F[b];
            copyD(q, G.dO, n); copyD(q + n, G.dT, n); copyD(q + 2 * n, G.hO, n); copyD(q + 3 * n, G.hT, n);
            copyD(q + 4 * n, G.mac, 3 * n); copyD(q + 7 * n, G.tv, 8 * n);
            copyD(q + 15 * n, G.dualO, 3 * n); copyD(q + 18 * n, G.dualT, 3 * n);
        }
    }
    void restoreFull(const double* o) {
        size_t n = S;
        for (int b = 0; b < 2; ++b) {
            const double* q = o + (size_t)b * 21 * n;
            Fields& G = F[b];
            copyD(G.dO, q, n); copyD(G.dT, q + n, n); copyD(G.hO, q + 2 * n, n); copyD(G.hT, q + 3 * n, n);
            copyD(G.mac, q + 4 * n, 3 * n); copyD(G.tv, q + 7 * n, 8 * n);
            copyD(G.dualO, q + 15 * n, 3 * n); copyD(G.dualT, q + 18 * n, 3 * n);
        }
    }
    void tapeStart(int every) {
        requireFrozen("astg_tape_start");
        if (every < 0) throw std::invalid_argument("astg_tape_start: checkpoint_every must be >= 0");
        freeTape();
        T.on = true;
        T.every = every;
    }
    // records the step about to run; returns where its advection input goes (store mode)
    double* tapeBeforeStep(double dt) {
        int k = T.steps;
        if (T.every > 0 && k % T.every == 0) {
            size_t j = (size_t)(k / T.every);
            if (T.ckpt.size() <= j) T.ckpt.push_back(tapeAlloc(FULL_DOUBLES));
            saveFull(T.ckpt[j]);
            T.ckCur.push_back(cur);
            T.ckFirst.push_back(firstSource ? 1 : 0);
        }
        T.dt.push_back(dt);
        T.first.push_back(firstSource ? 1 : 0);
        if (T.every > 0) return nullptr;
        if (T.adv.size() <= (size_t)k) T.adv.push_back(tapeAlloc(ADV_DOUBLES));
        return T.adv[k];
    }
    // the step transposes for taped step k, whose advection input is at adv
    void adjStep(int k, double* adv) {
        double dt = T.dt[k];
        Fields C = advectionView(adv);
        adjStage(5, dt, C, false);
        const Fields& Fr = F[cur];
        for (int i = 4; i >= 0; --i) adjStage(i, dt, Fr, T.first[k] != 0);
    }
    // reverse pass over every taped step: GA[ga] holds the cotangent of the final state on entry
    // and that of the state at astg_tape_start on return; source gradients accumulate
    void backward(astg_adjoint_stats* out) {
        if (!T.on || T.steps == 0) throw std::invalid_argument("astg_backward: no taped steps");
        allocAdjoint();
        adjustFrozen();
        int n = T.steps;
        if (!T.endState) T.endState = tapeAlloc(FULL_DOUBLES);
        saveFull(T.endState);
        int endCur = cur;
        bool endFirst = firstSource;
        astg_solve_stats endLast = last;
        adjSolves = adjIters = 0;
        adjN = -1;
        int recomputed = 0;
        float msRe = 0;
        T.recording = 0;
        cudaEvent_t e0, e1, r0, r1;
        cudaEventCreate(&e0); cudaEventCreate(&e1); cudaEventCreate(&r0); cudaEventCreate(&r1);
        ck(cudaEventRecord(e0, st), "event");
        try {
            if (T.every <= 0) {
                for (int k = n - 1; k >= 0; --k) adjStep(k, T.adv[k]);
            } else {
                int K = T.every;
                while ((int)T.adv.size() < std::min(K, n)) T.adv.push_back(tapeAlloc(ADV_DOUBLES));
                int nseg = (n + K - 1) / K;
                for (int j = nseg - 1; j >= 0; --j) {
                    int a = j * K, b = std::min(n, a + K);
                    restoreFull(T.ckpt[j]);
                    cur = T.ckCur[j];
                    firstSource = T.ckFirst[j] != 0;
                    ck(cudaEventRecord(r0, st), "event");
                    for (int k = a; k < b; ++k) {
                        advTarget = T.adv[k - a];
                        step(T.dt[k], nullptr);
                        ++recomputed;
                    }
                    advTarget = nullptr;
                    ck(cudaEventRecord(r1, st), "event");
                    ck(cudaEventSynchronize(r1), "sync");
                    float ms = 0;
                    cudaEventElapsedTime(&ms, r0, r1);
                    msRe += ms;
                    adjN = -1;  // the recomputed steps re-assembled the same matrix; factor once more
                    for (int k = b - 1; k >= a; --k) adjStep(k, T.adv[k - a]);
                }
            }
        } catch (...) {
            advTarget = nullptr;
            T.recording = 1;
            restoreFull(T.endState);
            cur = endCur;
            firstSource = endFirst;
            last = endLast;
            cudaStreamSynchronize(st);
            for (cudaEvent_t e : {e0, e1, r0, r1}) cudaEventDestroy(e);
            throw;
        }
        ck(cudaEventRecord(e1, st), "event");
        restoreFull(T.endState);
        cur = endCur;
        firstSource = endFirst;
        last = endLast;
        T.recording = 1;
        checkStatus();
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        for (cudaEvent_t e : {e0, e1, r0, r1}) cudaEventDestroy(e);
        if (out) {
            out->steps = n;
            out->checkpoints = (int)T.ckCur.size();
            out->recomputed_steps = recomputed;
            out->solves = (int)adjSolves;
            out->pcg_iterations = adjIters;
            out->ms = ms;
            out->ms_recompute = msRe;
            out->tape_bytes = T.bytes;
        }
    }
    // VJP of one step at the current state, which is left as it is
    void stepVjp(double dt) {
        requireFrozen("astg_step_vjp");
        allocAdjoint();
        adjustFrozen();
        if (T.on && T.recording) throw std::invalid_argument("astg_step_vjp: not while a tape is recording");
        double* full = rawAlloc(FULL_DOUBLES);
        double* adv = nullptr;
        try {
            adv = rawAlloc(ADV_DOUBLES);
        } catch (...) {
            cudaFree(full);
            throw;
        }
        int c0 = cur;
        bool f0 = firstSource;
        astg_solve_stats l0 = last;
        try {
            saveFull(full);
            for (int i = 0; i < 5; ++i) stage(i, dt);
            saveAdvectionInput(adv);
            restoreFull(full);
            cur = c0;
            firstSource = f0;
            last = l0;
            adjN = -1;
            Fields C = advectionView(adv);
            adjStage(5, dt, C, false);
            for (int i = 4; i >= 0; --i) adjStage(i, dt, F[cur], f0);
            checkStatus();
        } catch (...) {
            cudaStreamSynchronize(st);
            cudaFree(full);
            cudaFree(adv);
            throw;
        }
        ck(cudaStreamSynchronize(st), "sync");
        cudaFree(full);
        cudaFree(adv);
    }

    // ---------------------------------------------------------------- array exchange
    // "t_<field>" addresses the swap partner of a double-buffered state array
    static bool isPartner(const std::string& n) {
        static const char* fields[] = {"density_oct", "density_tilt", "heat_oct", "heat_tilt", "mac", "tilt_vel",
                                       "dual_oct", "dual_tilt", "tilt_e", "tilt_flags", "tilt_open"};
        if (n.compare(0, 2, "t_") != 0) return false;
        for (const char* f : fields)
            if (n.compare(2, std::string::npos, f) == 0) return true;
        return false;
    }
    // the caller's buffer may be host or device memory (unified addressing)
    template <class T>
    void down(const T* src, void* dst, size_t n) {
        ck(cudaMemcpyAsync(dst, src, n * sizeof(T), cudaMemcpyDefault, st), "download");
        ck(cudaStreamSynchronize(st), "download");
    }
    template <class T>
    void up(T* dst, const void* src, size_t n) {
        ck(cudaMemcpyAsync(dst, src, n * sizeof(T), cudaMemcpyDefault, st), "upload");
        ck(cudaStreamSynchronize(st), "upload");
    }
    int lastN() {
        int n = 0;
        down(J.nDof, &n, 1);
        return n;
    }

    // "adj_<field>": the cotangent arrays of the adjoint (f64, same shapes as the state arrays)
    double* adjArray(const std::string& name, size_t* n) {
        if (name.compare(0, 4, "adj_") != 0) return nullptr;
        allocAdjoint();
        std::string f = name.substr(4);
        Fields& g = GA[ga];
        size_t S1 = (size_t)S;
        if (f == "density_oct") { *n = S1; return g.dO; }
        if (f == "density_tilt") { *n = S1; return g.dT; }
        if (f == "heat_oct") { *n = S1; return g.hO; }
        if (f == "heat_tilt") { *n = S1; return g.hT; }
        if (f == "mac") { *n = 3 * S1; return g.mac; }
        if (f == "tilt_vel") { *n = 8 * S1; return g.tv; }
        if (f == "dual_oct") { *n = 3 * S1; return g.dualO; }
        if (f == "dual_tilt") { *n = 3 * S1; return g.dualT; }
        if (f == "source_density_oct") { *n = S1; return dGsO; }
        if (f == "source_density_tilt") { *n = S1; return dGsT; }
        throw std::invalid_argument("unknown adjoint array " + name);
    }

    // returns the byte size of a named array; copies it out when dst != nullptr
    size_t getArray(const std::string& name0, void* dst, size_t bytes) {
        {
            size_t n = 0;
            if (double* a = adjArray(name0, &n)) {
                if (dst && bytes != 8 * n) throw std::invalid_argument("astg_get " + name0 + ": expected " + std::to_string(8 * n) + " bytes");
                if (dst) down(a, dst, n);
                return 8 * n;
            }
        }
        std::string name = name0;
        int b = cur;
        if (isPartner(name)) { b = 1 - cur; name = name.substr(2); }
        Fields& G = F[b];
        auto need = [&](size_t nb) {
            if (dst && bytes != nb) throw std::invalid_argument("astg_get " + name0 + ": expected " + std::to_string(nb) + " bytes");
            return nb;
        };
        if (name == "density_oct") { size_t nb = need(8 * (size_t)S); if (dst) down(G.dO, dst, S); return nb; }
        if (name == "density_tilt") { size_t nb = need(8 * (size_t)S); if (dst) down(G.dT, dst, S); return nb; }
        if (name == "heat_oct") { size_t nb = need(8 * (size_t)S); if (dst) down(G.hO, dst, S); return nb; }
        if (name == "heat_tilt") { size_t nb = need(8 * (size_t)S); if (dst) down(G.hT, dst, S); return nb; }
        if (name == "mac") { size_t nb = need(24 * (size_t)S); if (dst) down(G.mac, dst, 3 * (size_t)S); return nb; }
        if (name == "tilt_vel") { size_t nb = need(64 * (size_t)S); if (dst) down(G.tv, dst, 8 * (size_t)S); return nb; }
        if (name == "dual_oct") { size_t nb = need(24 * (size_t)S); if (dst) down(G.dualO, dst, 3 * (size_t)S); return nb; }
        if (name == "dual_tilt") { size_t nb = need(24 * (size_t)S); if (dst) down(G.dualT, dst, 3 * (size_t)S); return nb; }
        if (name == "tilt_e") { size_t nb = need(8 * (size_t)S); if (dst) down(G.te, dst, S); return nb; }
        if (name == "tilt_flags") {
            size_t nb = need(8 * (size_t)S);
            if (dst) {
                std::vector<uint32_t> f(S);
                down(G.tf, f.data(), S);
                int32_t* o = (int32_t*)dst;
                for (int s = 0; s < S; ++s) { o[2 * s] = (int32_t)(f[s] & 0xff); o[2 * s + 1] = tf_dir(f[s]); }
            }
            return nb;
        }
        if (name == "tilt_open") {
            size_t nb = need((size_t)S);
            if (dst) {
                std::vector<uint8_t> o(S), fx(S);
                down(dOpen, o.data(), S);
                down(dFixed, fx.data(), S);
                uint8_t* q = (uint8_t*)dst;
                for (int s = 0; s < S; ++s) q[s] = (o[s] ? 1 : 0) | (fx[s] ? 2 : 0);
            }
            return nb;
        }
        if (b != cur) throw std::invalid_argument("astg_get: no swap partner for " + name);
        if (name == "source_density_oct") { size_t nb = need(8 * (size_t)S); if (dst) down(dSrcO, dst, S); return nb; }
        if (name == "source_density_tilt") { size_t nb = need(8 * (size_t)S); if (dst) down(dSrcT, dst, S); return nb; }
        if (name == "slot_coords") {
            size_t nb = need(16 * (size_t)S);
            if (dst) {
                int32_t* o = (int32_t*)dst;
                for (int s = 0; s < S; ++s) {
                    o[4 * s] = sx[s]; o[4 * s + 1] = sy[s]; o[4 * s + 2] = sz[s];
                    // reference flags: VALID | IS_GHOST | GHOST_FROM_COARSE
                    o[4 * s + 3] = 1 | ((sflag[s] & SF_GHOST) ? 2 : 0) | ((sflag[s] & SF_FROM_COARSE) ? 4 : 0);
                }
            }
            return nb;
        }
        if (name == "level_sizes") {
            size_t nb = need(12 * (size_t)L);
            if (dst) {
                int32_t* o = (int32_t*)dst;
                for (int l = 0; l < L; ++l) { o[3 * l] = lN[l]; o[3 * l + 1] = lG[l]; o[3 * l + 2] = lN[l] + lG[l]; }
            }
            return nb;
        }
        if (name == "split_map") { size_t nb = need(4 * split.size()); if (dst) memcpy(dst, split.data(), nb); return nb; }
        if (name == "half_tilts" || name == "t_joints" || name == "closed_by_half_tilt") {
            const std::vector<int>& v = name == "half_tilts" ? half : (name == "t_joints" ? tj : cbh);
            std::vector<long long> o;
            for (int q : v) o.push_back(((long long)slev[q] << 60) | ((long long)sx[q] << 40) | ((long long)sy[q] << 20) | (long long)sz[q]);
            if (name == "t_joints") std::sort(o.begin(), o.end());
            size_t nb = need(8 * o.size());
            if (dst && nb) memcpy(dst, o.data(), nb);
            return nb;
        }
        if (name == "w_mac") { size_t nb = need(8 * wMac.size()); if (dst) memcpy(dst, wMac.data(), nb); return nb; }
        if (name == "w_tilt") { size_t nb = need(8 * wTilt.size()); if (dst) memcpy(dst, wTilt.data(), nb); return nb; }
        if (name == "dual_tables") { size_t nb = need(8 * M37.size()); if (dst) memcpy(dst, M37.data(), nb); return nb; }
        if (name == "collider_sdf") {
            size_t n = d.sdf ? (size_t)res * res * res : 0;
            size_t nb = need(8 * n);
            if (dst && n) down(dSdf, dst, n);
            return nb;
        }
        if (name == "pindex_oct") { size_t nb = need(4 * (size_t)S); if (dst) down(J.pO, dst, S); return nb; }
        if (name == "pindex_tilt") { size_t nb = need(4 * (size_t)S); if (dst) down(J.pT, dst, S); return nb; }
        if (name == "A_rowptr") { int n = lastN(); size_t nb = need(4 * (size_t)(n + 1)); if (dst) down(J.rowPtr, dst, n + 1); return nb; }
        if (name == "A_col" || name == "A_val") {
            int n = lastN(), nnz = 0;
            down(J.nnz, &nnz, 1);
            (void)n;
            size_t nb = need((name == "A_col" ? 4 : 8) * (size_t)nnz);
            if (dst) {
                if (name == "A_col") down(J.col, dst, nnz);
                else down(J.val, dst, nnz);
            }
            return nb;
        }
        if (name == "b") { int n = lastN(); size_t nb = need(8 * (size_t)n); if (dst) down(J.b, dst, n); return nb; }
        if (name == "p") { int n = lastN(); size_t nb = need(8 * (size_t)n); if (dst) down(J.x, dst, n); return nb; }
        if (name == "pcg_iters") {
            size_t nb = need(8);
            if (dst) {
                int32_t* o = (int32_t*)dst;
                o[0] = last.iterations;
                o[1] = last.converged;
            }
            return nb;
        }
        if (name == "ambT") { size_t nb = need(8); if (dst) down(dAmb, dst, 1); return nb; }
        if (name == "kernel_ms") {  // f64 x 8: (ms, launches) for fwd sweep, bwd sweep, SpMV+dot, factor
            size_t nb = need(64);
            if (dst) {
                double* o = (double*)dst;
                for (int k = 0; k < KPROF_KINDS; ++k) { o[2 * k] = prof.ms[k]; o[2 * k + 1] = (double)prof.count[k]; }
            }
            return nb;
        }
        throw std::invalid_argument("astg_get: unknown array " + name0);
    }

    void setArray(const std::string& name0, const void* src, size_t bytes) {
        {
            size_t n = 0;
            if (double* a = adjArray(name0, &n)) {
                if (bytes != 8 * n) throw std::invalid_argument("astg_set " + name0 + ": expected " + std::to_string(8 * n) + " bytes");
                up(a, src, n);
                return;
            }
        }
        std::string name = name0;
        int b = cur;
        if (isPartner(name)) { b = 1 - cur; name = name.substr(2); }
        Fields& G = F[b];
        auto need = [&](size_t nb) {
            if (bytes != nb) throw std::invalid_argument("astg_set " + name0 + ": expected " + std::to_string(nb) + " bytes");
        };
        if (b == cur && name == "collider_sdf") { setCollider((const double*)src, bytes); return; }
        if (b == cur && name == "collider_centre") {
            need(24);
            const double* c3 = (const double*)src;
            d.colCx = c3[0];
            d.colCy = c3[1];
            d.colCz = c3[2];
            return;
        }
        if (name == "density_oct") { need(8 * (size_t)S); up(G.dO, src, S); return; }
        if (name == "density_tilt") { need(8 * (size_t)S); up(G.dT, src, S); return; }
        if (name == "heat_oct") { need(8 * (size_t)S); up(G.hO, src, S); return; }
        if (name == "heat_tilt") { need(8 * (size_t)S); up(G.hT, src, S); return; }
        if (name == "mac") { need(24 * (size_t)S); up(G.mac, src, 3 * (size_t)S); return; }
        if (name == "tilt_vel") { need(64 * (size_t)S); up(G.tv, src, 8 * (size_t)S); return; }
        if (name == "dual_oct") { need(24 * (size_t)S); up(G.dualO, src, 3 * (size_t)S); return; }
        if (name == "dual_tilt") { need(24 * (size_t)S); up(G.dualT, src, 3 * (size_t)S); return; }
        if (name == "tilt_e") { need(8 * (size_t)S); up(G.te, src, S); return; }
        if (name == "tilt_flags") {
            need(8 * (size_t)S);
            const int32_t* f = (const int32_t*)src;
            std::vector<uint32_t> v(S);
            for (int s = 0; s < S; ++s) v[s] = ((uint32_t)f[2 * s] & 0xff) | ((uint32_t)(f[2 * s + 1] + 1) << 8);
            up(G.tf, v.data(), S);
            return;
        }
        if (b == cur && name == "source_density_oct") { need(8 * (size_t)S); up(dSrcO, src, S); return; }
        if (b == cur && name == "source_density_tilt") { need(8 * (size_t)S); up(dSrcT, src, S); return; }
        if (name == "tilt_open") {
            need((size_t)S);
            const uint8_t* q = (const uint8_t*)src;
            std::vector<uint8_t> o(S), fx(S);
            for (int s = 0; s < S; ++s) { o[s] = q[s] & 1; fx[s] = (q[s] >> 1) & 1; }
            up(dOpen, o.data(), S);
            up(dFixed, fx.data(), S);
            return;
        }
        throw std::invalid_argument("astg_set: unknown or read-only array " + name0);
    }
};

// ==================================================================== C ABI
namespace {
astg_status fail(astg_handle* h, const std::exception& e, astg_status code) {
    if (h) h->err = e.what();
    return code;
}
template <class F>
astg_status guard(astg_handle* h, F&& f) {
    if (!h) return ASTG_BAD_ARG;
    try {
        f();
        return ASTG_OK;
    } catch (CudaError& e) {
        return fail(h, e, ASTG_CUDA_ERROR);
    } catch (std::invalid_argument& e) {
        return fail(h, e, ASTG_BAD_ARG);
    } catch (std::runtime_error& e) {
        std::string m = e.what();
        if (m.find("timed out") != std::string::npos) return fail(h, e, ASTG_DEVICE_WAIT_TIMEOUT);
        if (m.find("layout") != std::string::npos) return fail(h, e, ASTG_LAYOUT_ERROR);
        return fail(h, e, ASTG_CUDA_ERROR);
    } catch (std::exception& e) {
        return fail(h, e, ASTG_CUDA_ERROR);
    }
}
// message of a handle-less call into the caller's buffer (which may be NULL)
astg_status noalloc_fail(char* err, size_t errlen, astg_status s, const char* fmt, ...) {
    if (err && errlen) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(err, errlen, fmt, ap);
        va_end(ap);
    }
    return s;
}
}  // namespace

extern "C" {

void astg_default_params(astg_params* p, int coarsest, int levels) {
    if (!p) return;
    memset(p, 0, sizeof *p);
    p->coarsest = coarsest;
    p->levels = levels;
    p->tol = 1e-6;
    p->max_iter = 3000;
    p->omega = 0.97;
    p->min_diag = 0.25;
    p->rho = 2.0;
    p->buoy_density = -0.1;
    p->buoy_temp = 1.0;
    p->decay = 1.0;
    p->closed_mask = 1 | 2 | 4 | 8 | 32;
    p->tilt_adaptivity = 1;
    astg_scene::Sphere s = astg_scene::default_source();
    p->src_x = s.cx; p->src_y = s.cy; p->src_z = s.cz; p->src_r = s.r;
    p->noise = 1e-3;
    p->seed = 0;
    p->precision = ASTG_FP64;
    p->device = 0;
}

astg_status astg_create(const astg_params* p, const int32_t* split_map, astg_handle** out) {
    if (!p || !out) return ASTG_BAD_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return ASTG_NO_DEVICE;
    auto* h = new astg_handle();
    astg_status s = guard(h, [&] { h->init(*p, split_map); });
    if (s != ASTG_OK) {
        // keep the handle so the caller can read the message; it must still be destroyed
        *out = h;
        return s;
    }
    *out = h;
    return ASTG_OK;
}

void astg_destroy(astg_handle* h) { delete h; }

const char* astg_last_error(const astg_handle* h) { return h ? h->err.c_str() : "null handle"; }

astg_status astg_step(astg_handle* h, double dt, astg_step_stats* stats) {
    if (!(dt > 0)) return ASTG_BAD_ARG;
    astg_status s = guard(h, [&] { h->step(dt, stats); });
    if (s == ASTG_OK && h->last.converged == 0) return ASTG_NOT_CONVERGED;
    return s;
}

astg_status astg_stage(astg_handle* h, int stage, double dt) {
    return guard(h, [&] {
        if (h->T.on && h->T.recording) throw std::invalid_argument("astg_stage: a tape is recording (use astg_step)");
        h->stage(stage, dt);
        h->checkStatus();
    });
}

astg_status astg_set_solver_parameters(astg_handle* h, double tol, int max_iter, double omega, double min_diag) {
    if (!h || max_iter <= 0) return ASTG_BAD_ARG;
    h->P.tol = tol < 1e-30 ? 1e-30 : tol;
    h->P.max_iter = max_iter;
    h->P.omega = omega;
    h->P.min_diag = min_diag;
    return ASTG_OK;
}

astg_status astg_set_profiling(astg_handle* h, int on) {
    if (!h) return ASTG_BAD_ARG;
    h->prof.on = on != 0;
    for (int k = 0; k < KPROF_KINDS; ++k) { h->prof.ms[k] = 0; h->prof.count[k] = 0; }
    return ASTG_OK;
}

astg_status astg_set_precision(astg_handle* h, astg_precision prec) {
    if (!h || (prec != ASTG_FP64 && prec != ASTG_MIXED)) return ASTG_BAD_ARG;
    h->P.precision = prec;
    return ASTG_OK;
}

namespace {
// CellCenteredGrid<REAL,3>::sample (include/cell_centered_grid.h:40-54) on the host: getBarycentric's
// truncating, clamped form (include/util.h:243-256) and the nested lerps of trilerp (:179-187)
double h_lerp(double a, double b, double f) { return a * (1 - f) + b * f; }
void h_bary_vec(double x, int high, int* i, double* f) {
    int c = (int)x;
    if (c < 0) c = 0;
    if (c > high - 1) c = high - 1;
    *i = c;
    double t = x - c;
    *f = t < 0 ? 0 : (t > 1 ? 1 : t);
}
double h_sdf_sample(const double* sdf, int sres, double px, double py, double pz) {
    double sd = 1.0 / sres;
    double rp[3] = {px / sd - 0.5, py / sd - 0.5, pz / sd - 0.5};
    int i[3], i1[3];
    double f[3];
    for (int k = 0; k < 3; ++k) {
        h_bary_vec(rp[k], sres - 1, &i[k], &f[k]);
        i1[k] = std::min(i[k] + 1, sres - 1);
    }
    auto g = [&](int x, int y, int z) { return sdf[((size_t)z * sres + y) * sres + x]; };
    double a = h_lerp(h_lerp(g(i[0], i[1], i[2]), g(i1[0], i[1], i[2]), f[0]),
                      h_lerp(g(i[0], i1[1], i[2]), g(i1[0], i1[1], i[2]), f[0]), f[1]);
    double b = h_lerp(h_lerp(g(i[0], i[1], i1[2]), g(i1[0], i[1], i1[2]), f[0]),
                      h_lerp(g(i[0], i1[1], i1[2]), g(i1[0], i1[1], i1[2]), f[0]), f[1]);
    return h_lerp(a, b, f[2]);
}
}  // namespace

astg_status astg_refine_split_map(int32_t* split_map, int res, int level, const double* sdf, double lo, double hi) {
    if (!split_map || !sdf || res <= 0 || level < 1 || level > 30) return ASTG_BAD_ARG;
    const int k = 1 << level;
    if (res % k != 0) return ASTG_BAD_ARG;  // "resolution is not dividable by level"
    const int cres = res >> level;
    const double dh = (1.0 / res) * k;
    auto at = [&](int x, int y, int z) -> int32_t& { return split_map[((size_t)z * res + y) * res + x]; };
    for (int tz = 0; tz < cres; ++tz)
        for (int ty = 0; ty < cres; ++ty)
            for (int tx = 0; tx < cres; ++tx) {
                if (at(tx << level, ty << level, tz << level) != level) continue;
                double v = h_sdf_sample(sdf, res, (tx + 0.5) * dh, (ty + 0.5) * dh, (tz + 0.5) * dh);
                if (v >= lo && v <= hi)
                    for (int z = tz << level; z < (tz << level) + k; ++z)
                        for (int y = ty << level; y < (ty << level) + k; ++y)
                            for (int x = tx << level; x < (tx << level) + k; ++x) at(x, y, z) = level - 1;
            }
    return ASTG_OK;
}

astg_status astg_refine_split_map_device(int32_t* d_split_map, int res, int level, const double* d_sdf, double lo,
                                         double hi, void* stream) {
    if (!d_split_map || !d_sdf || res <= 0 || level < 1 || level > 30) return ASTG_BAD_ARG;
    if (res % (1 << level) != 0) return ASTG_BAD_ARG;  // "resolution is not dividable by level"
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return ASTG_CUDA_ERROR;
    const void* ptrs[2] = {d_split_map, d_sdf};
    for (const void* q : ptrs) {
        cudaPointerAttributes a;
        if (cudaPointerGetAttributes(&a, q) != cudaSuccess) {
            cudaGetLastError();
            return ASTG_BAD_ARG;
        }
        bool onDevice = a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
        if (!onDevice || (a.type == cudaMemoryTypeDevice && a.device != dev)) return ASTG_BAD_ARG;
    }
    cudaError_t e = launch_refine_split_map(d_split_map, res, level, d_sdf, lo, hi, (cudaStream_t)stream);
    return e == cudaSuccess ? ASTG_OK : ASTG_CUDA_ERROR;
}

astg_status astg_update(astg_handle* h, double dt, int* substeps, astg_step_stats* stats) {
    if (!h || !(dt >= 0)) return ASTG_BAD_ARG;
    astg_status s = guard(h, [&] { h->update(dt, substeps, stats); });
    if (s == ASTG_OK && !h->updateConverged) return ASTG_NOT_CONVERGED;
    return s;
}

astg_status astg_set_collider_sphere(astg_handle* h, double cx, double cy, double cz, double radius) {
    if (!h || !std::isfinite(cx) || !std::isfinite(cy) || !std::isfinite(cz) || std::isnan(radius)) return ASTG_BAD_ARG;
    return guard(h, [&] { h->setColliderSphere(cx, cy, cz, radius); });
}

astg_status astg_set_max_cfl(astg_handle* h, double max_cfl) {
    if (!h || !(max_cfl > 0)) return ASTG_BAD_ARG;
    h->maxCfl = max_cfl;
    return ASTG_OK;
}

astg_status astg_cfl(astg_handle* h, double dt, int* cfl, int* substeps) {
    if (!h || !(dt >= 0)) return ASTG_BAD_ARG;
    return guard(h, [&] {
        int c = h->cfl(dt);
        if (cfl) *cfl = c;
        if (substeps) {
            int k = (int)std::ceil(c / h->maxCfl);
            *substeps = k > 1 ? k : 1;
        }
    });
}

astg_status astg_set_reduction_order(astg_handle* h, astg_order order, int workers) {
    if (!h || (order != ASTG_ORDER_LIBRARY && order != ASTG_ORDER_REFERENCE)) return ASTG_BAD_ARG;
    if (order == ASTG_ORDER_REFERENCE && (workers < 1 || workers > astg::REF_MAX_WORKERS)) return ASTG_BAD_ARG;
    h->J.refOrder = order == ASTG_ORDER_REFERENCE;
    h->J.unfused = h->J.refOrder;
    if (h->J.refOrder) h->refWorkers = workers;
    return ASTG_OK;
}

astg_status astg_last_solve(const astg_handle* h, astg_solve_stats* out) {
    if (!h || !out) return ASTG_BAD_ARG;
    *out = h->last;
    return ASTG_OK;
}

long long astg_size(const astg_handle* h, int what) {
    if (!h) return -1;
    switch (what) {
        case 0: return h->S;
        case 1: return h->L;
        case 2: return h->res;
        case 3: return h->last.n;
        case 4: return h->H;
        case 5: return h->last.nnz;
        case 6: return astg::g_launches;
        case 7: return h->J.pcActive ? (h->J.pcAsync ? 200 : 100) + h->J.pcCluster : h->J.clusterSize;
        default: return -1;
    }
}

astg_status astg_get(astg_handle* h, const char* name, void* dst, size_t bytes, size_t* bytes_needed) {
    if (!h || !name) return ASTG_BAD_ARG;
    size_t nb = 0;
    astg_status s = guard(h, [&] { nb = h->getArray(name, dst, bytes); });
    if (bytes_needed) *bytes_needed = nb;
    if (s == ASTG_OK && !dst) return ASTG_BAD_ARG;
    return s;
}

astg_status astg_set(astg_handle* h, const char* name, const void* src, size_t bytes) {
    if (!h || !name || !src) return ASTG_BAD_ARG;
    return guard(h, [&] { h->setArray(name, src, bytes); });
}

astg_status astg_solve(astg_handle* h, int n, const int32_t* rowptr, const int32_t* col, const double* val,
                       const double* b, double* x, double rel_tol, int max_iter, astg_precision prec,
                       astg_solve_stats* stats) {
    if (!h || !rowptr || !col || !val || !b || !x || max_iter <= 0) return ASTG_BAD_ARG;
    if (prec != ASTG_FP64 && prec != ASTG_MIXED) return ASTG_BAD_ARG;
    astg_status s = guard(h, [&] { h->solveExternal(n, rowptr, col, val, b, x, rel_tol, max_iter, prec, stats); });
    if (s == ASTG_OK && !h->last.converged) return ASTG_NOT_CONVERGED;
    return s;
}

astg_status astg_solve_batch(astg_handle* h, int n, const int32_t* rowptr, const int32_t* col, const double* val,
                             int nrhs, const double* b, double* x, double rel_tol, int max_iter, astg_precision prec,
                             astg_solve_stats* stats, double* wall_ms, int* lanes) {
    if (!h || !rowptr || !col || !val || !b || !x || max_iter <= 0 || nrhs <= 0) return ASTG_BAD_ARG;
    if (prec != ASTG_FP64 && prec != ASTG_MIXED) return ASTG_BAD_ARG;
    bool all = true;
    astg_status s = guard(h, [&] {
        std::vector<astg_solve_stats> st(nrhs);
        h->solveBatch(n, rowptr, col, val, nrhs, b, x, rel_tol, max_iter, prec, st.data(), wall_ms);
        for (int i = 0; i < nrhs; ++i) all = all && st[i].converged;
        if (stats) std::copy(st.begin(), st.end(), stats);
        if (lanes) *lanes = h->lastLanes;
    });
    if (s == ASTG_OK && !all) return ASTG_NOT_CONVERGED;
    return s;
}

astg_status astg_set_tilt_adaptivity(astg_handle* h, int on) {
    return guard(h, [&] {
        if (h->T.on && h->T.recording && on) throw std::invalid_argument("astg_set_tilt_adaptivity: a tape is recording");
        h->P.tilt_adaptivity = on != 0;
        if (!on) {
            // freeze: both buffers carry the current tilt-E state from now on
            const Fields& C = h->F[h->cur];
            Fields& N = h->F[1 - h->cur];
            h->copyD(N.te, C.te, (size_t)h->S);
            ck(cudaMemcpyAsync(N.tf, C.tf, sizeof(uint32_t) * (size_t)h->S, cudaMemcpyDeviceToDevice, h->st), "copy");
            ck(cudaStreamSynchronize(h->st), "sync");
        }
    });
}

astg_status astg_tape_start(astg_handle* h, int checkpoint_every) {
    return guard(h, [&] { h->tapeStart(checkpoint_every); });
}

astg_status astg_tape_stop(astg_handle* h) {
    return guard(h, [&] { h->freeTape(); });
}

astg_status astg_adjoint_reset(astg_handle* h) {
    return guard(h, [&] { h->resetAdjoint(); });
}

astg_status astg_backward(astg_handle* h, astg_adjoint_stats* stats) {
    return guard(h, [&] { h->backward(stats); });
}

astg_status astg_stage_vjp(astg_handle* h, int stage, double dt) {
    if (!(dt > 0)) return ASTG_BAD_ARG;
    return guard(h, [&] { h->stageVjp(stage, dt); });
}

astg_status astg_step_vjp(astg_handle* h, double dt) {
    if (!(dt > 0)) return ASTG_BAD_ARG;
    return guard(h, [&] { h->stepVjp(dt); });
}

astg_status astg_adjoint_probe(astg_handle* h, int what, int n, const double* pos, double* out) {
    if (!h || (what != 0 && what != 1) || n < 0 || (n > 0 && (!pos || !out))) return ASTG_BAD_ARG;
    return guard(h, [&] {
        if (n == 0) return;
        size_t per = what == 0 ? 5 : 15;
        double* dp = nullptr;
        double* dout = nullptr;
        ck(cudaMalloc(&dp, 24 * (size_t)n), "cudaMalloc");
        if (cudaMalloc(&dout, 8 * per * (size_t)n) != cudaSuccess) {
            cudaFree(dp);
            throw CudaError("cudaMalloc");
        }
        cudaError_t e = cudaMemcpyAsync(dp, pos, 24 * (size_t)n, cudaMemcpyDefault, h->st);
        if (e == cudaSuccess) e = astg::launch_adj_probe(h->d, h->F[h->cur], what, n, dp, dout, h->st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(out, dout, 8 * per * (size_t)n, cudaMemcpyDefault, h->st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
        cudaFree(dp);
        cudaFree(dout);
        ck(e, "adjoint probe");
        h->checkStatus();
    });
}

astg_status astg_max_velocity(astg_handle* h, double* out) {
    if (!h || !out) return ASTG_BAD_ARG;
    return guard(h, [&] {
        std::vector<double> mac((size_t)3 * h->S);
        h->down(h->F[h->cur].mac, mac.data(), mac.size());
        double m = 0;
        for (double v : mac) m = std::max(m, v);
        *out = m;
    });
}

astg_status astg_restart(astg_handle* h, int frame, const char* layout_file, const char* boundary_file,
                         const char* tilt_file, const char* density_file, const char* heat_file,
                         const char* velocity_file) {
    (void)frame;
    (void)boundary_file;
    if (!h) return ASTG_BAD_ARG;
    return guard(h, [&] { h->restart(layout_file, tilt_file, density_file, heat_file, velocity_file); });
}

astg_status astg_save_checkpoint(astg_handle* h, const char* layout_file, const char* tilt_file,
                                 const char* density_file, const char* heat_file, const char* velocity_file) {
    if (!h) return ASTG_BAD_ARG;
    return guard(h, [&] { h->saveCheckpoint(layout_file, tilt_file, density_file, heat_file, velocity_file); });
}

astg_status astg_extrapolate(astg_handle* h, const char* field, const double* sdf, int sdf_res, double valid_offset,
                             double max_distance_factor, astg_extrap_stats* stats) {
    if (!h || !field || !sdf) return ASTG_BAD_ARG;
    return guard(h, [&] { h->extrapolate(field, sdf, sdf_res, valid_offset, max_distance_factor, stats); });
}

// Takes no handle and allocates nothing, on the device or the host: the chunk partials go to a
// static device array (launch_mean_temperature_static), so callers that must not allocate can
// use it.  Which callers those are, and the rules on the shared array, are in include/astg.h.
astg_status astg_mean_temperature_noalloc(const double* d_heat_oct, const int64_t* level_slots, int levels,
                                          double* d_amb, void* stream, char* err, size_t errlen) {
    if (err && errlen) err[0] = 0;
    if (!d_heat_oct || !d_amb || !level_slots) return noalloc_fail(err, errlen, ASTG_BAD_ARG, "null pointer argument");
    if (levels < 1 || levels > MAXL)
        return noalloc_fail(err, errlen, ASTG_BAD_ARG, "levels = %d, must be 1..%d", levels, MAXL);
    LevelSpans sp;
    sp.L = levels;
    sp.off[0] = 0;
    sp.partOff[0] = 0;
    for (int l = 0; l < levels; ++l) {
        long long n = level_slots[l];
        if (n < 0) return noalloc_fail(err, errlen, ASTG_BAD_ARG, "level %d has a negative slot count %lld", l, n);
        long long m = (n + AMB_CHUNK - 1) / AMB_CHUNK;
        if (m > AMB_MAX_LEVEL_PARTIALS)
            return noalloc_fail(err, errlen, ASTG_BAD_ARG, "level %d has %lld slots, more than %d * %d", l, n,
                                AMB_CHUNK, AMB_MAX_LEVEL_PARTIALS);
        sp.off[l + 1] = sp.off[l] + n;
        if (sp.partOff[l] + m > NOALLOC_MAX_PARTIALS)
            return noalloc_fail(err, errlen, ASTG_BAD_ARG,
                                "%lld slots need more than the %d partials of the static scratch "
                                "(sum over levels of ceil(slots / %d) must be <= %d)",
                                sp.off[l + 1], NOALLOC_MAX_PARTIALS, AMB_CHUNK, NOALLOC_MAX_PARTIALS);
        sp.partOff[l + 1] = sp.partOff[l] + (int)m;
    }
    if (sp.off[levels] == 0) return noalloc_fail(err, errlen, ASTG_BAD_ARG, "no slots");
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return noalloc_fail(err, errlen, ASTG_NO_DEVICE, "no CUDA device");
    }
    const void* ptrs[2] = {d_heat_oct, d_amb};
    const char* names[2] = {"d_heat_oct", "d_amb"};
    for (int k = 0; k < 2; ++k) {
        cudaPointerAttributes a;
        if (cudaPointerGetAttributes(&a, ptrs[k]) != cudaSuccess) {
            cudaGetLastError();
            return noalloc_fail(err, errlen, ASTG_BAD_ARG, "%s is not a CUDA pointer", names[k]);
        }
        bool onDevice = a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
        if (!onDevice || (a.type == cudaMemoryTypeDevice && a.device != dev))
            return noalloc_fail(err, errlen, ASTG_BAD_ARG, "%s is not device memory of the current device %d",
                                names[k], dev);
    }
    cudaError_t e = launch_mean_temperature_static(d_heat_oct, sp, d_amb, (cudaStream_t)stream);
    if (e != cudaSuccess) return noalloc_fail(err, errlen, ASTG_CUDA_ERROR, "CUDA error: %s", cudaGetErrorString(e));
    return ASTG_OK;
}

}  // extern "C"
