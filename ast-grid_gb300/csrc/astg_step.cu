// Per-node kernels of the octree smoke step: source, buoyancy, wall constraints, ghost
// propagation, dual (collocated) velocity, pressure-gradient update, tilt adaptivity and
// semi-Lagrangian advection.  One thread per slot (or per list entry); each kernel restates one
// reference loop, cited on the kernel.
//
// Passes whose reference loop reads values written by the same loop on other ghosts are split
// into one launch per level, finest first, which reproduces the reference's sequential order
// (a ghost of level l only ever reads ghosts of levels l-1 and l+1).
#include "astg_launch.h"
#include "astg_sample.cuh"

namespace astg {

constexpr int TB = 256;
static inline int nblk(long long n) { return (int)((n + TB - 1) / TB); }

ASTG_HD inline bool in_src(const Dev& d, V3 p) {
    double dx = p.x - d.srcX, dy = p.y - d.srcY, dz = p.z - d.srcZ;
    return dx * dx + dy * dy + dz * dz < d.srcR * d.srcR;
}
ASTG_HD inline bool ghost(const Dev& d, int s) { return slot_f(d, s) & SF_GHOST; }

// ------------------------------------------------------------------ source
// example/octree_smoke_3d/main.cpp:23-86 with heat = 1, an upward velocity of 1 and the density
// of each slot's source (1 unless set as a differentiable parameter)
__global__ void k_source_slots(Dev d, Fields F) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.S || ghost(d, s)) return;
    if (in_src(d, cell_pos(d, s))) { F.dO[s] = d.srcO[s]; F.hO[s] = 1; }
    V3 vp = vert_pos(d, s);
    if (in_src(d, vp)) {
        F.dT[s] = d.srcT[s];
        F.hT[s] = 1;
        for (int k = 0; k < 8; ++k) F.tv[(size_t)s * 8 + k] = 1.0 * INV_SQRT3;
    }
    if (in_src(d, mac_pos(d, 2, s))) F.mac[2 * (size_t)d.S + s] = 1.0;
}
__global__ void k_source_half(Dev d, Fields F) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.H) return;
    int hs = d.half[i];
    V3 vp = vert_pos(d, hs);
    if (!in_src(d, vp)) return;
    F.dT[hs] = d.srcT[hs];
    F.hT[hs] = 1;
    int dir = tf_dir(F.tf[hs]);
    double nv[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int q = 0; q < 4; ++q) nv[HALF_SLOT[dir][q]] = 1.0 * INV_SQRT3;
    if (dir % 3 == 2) nv[HALF_SLOT[dir][4]] = 1.0;
    for (int k = 0; k < 8; ++k) F.tv[(size_t)hs * 8 + k] = nv[k];
}

// ------------------------------------------------------------------ omni ghost update
// OctreeCellCenteredGrid3<T>::updateGhost, include/octree_cell_centered_grid3.h:184-208:
// fine-to-coarse average (ghosts covered by finer cells)
template <class T, class A>
__global__ void k_cell_ghost_avg(Dev d, A acc, int l) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.lG[l]) return;
    int s = d.loff[l] + d.lN[l] + i;
    if (slot_f(d, s) & SF_FROM_COARSE) return;
    int x = slot_x(d, s) << 1, y = slot_y(d, s) << 1, z = slot_z(d, s) << 1;
    T v = acc.zero();
    for (int a = 0; a <= 1; ++a)
        for (int b = 0; b <= 1; ++b)
            for (int c = 0; c <= 1; ++c) v = v + acc.get(req(d, l - 1, x + a, y + b, z + c));
    acc.set(s, v * (1 / 8.0));
}
// ... and coarse-to-fine: trilinear sample at the ghost's centre
template <class T, class A>
__global__ void k_cell_ghost_sample(Dev d, A acc, int l) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.lG[l]) return;
    int s = d.loff[l] + d.lN[l] + i;
    if (!(slot_f(d, s) & SF_FROM_COARSE)) return;
    acc.set(s, cell_sample<T>(d, acc, cell_pos(d, s)));
}
// OctreeVertexCenteredGrid3<T>::updateGhost, include/octree_vertex_centered_grid3.h:129-153,
// leaving half-tilt slots alone (include/base_octree_omni_grid.h:20-28).  Reads non-ghost
// slots only, so one launch covers every level.
template <class T, class A>
__global__ void k_vertex_ghost(Dev d, A til) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.S || !ghost(d, s) || d.halfMark[s]) return;
    int l = slot_l(d, s), x = slot_x(d, s), y = slot_y(d, s), z = slot_z(d, s);
    if (slot_f(d, s) & SF_FROM_COARSE) {
        T v = til.zero();
        int count = 0;
        for (int a = 0; a <= (x & 1); ++a)
            for (int b = 0; b <= (y & 1); ++b)
                for (int c = 0; c <= (z & 1); ++c) {
                    int t = get_until(d, l + 1, (x >> 1) + a, (y >> 1) + b, (z >> 1) + c, true);
                    if (t >= 0) { v = v + til.get(t); count += 1; }
                }
        til.set(s, v * (1.0 / (count + EPS)));
    } else {
        int t = get_until(d, l - 1, x << 1, y << 1, z << 1, true);
        if (t < 0) { report(d, DS_MISSING_NODE); t = 0; }
        til.set(s, til.get(t));
    }
}
// OctreeOmniGrid3<T>::updateCellGhost, include/octree_omni_grid3.h:289-303
template <class T, class A>
__global__ void k_cell_ghost_joint(Dev d, A oct, A til, int l) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.lG[l]) return;
    int s = d.loff[l] + d.lN[l] + i;
    int x = slot_x(d, s), y = slot_y(d, s), z = slot_z(d, s);
    if (!oct_valid(d, l, x, y, z) || !(slot_f(d, s) & SF_FROM_COARSE)) return;
    int dp = req(d, l, x + (x & 1), y + (y & 1), z + (z & 1));
    oct.set(s, (til.get(dp) + oct.get(req(d, l + 1, x >> 1, y >> 1, z >> 1))) * 0.5);
}
// getTiltFromOctagonNeighbor3, include/octree_util.h:103-121
template <class T, class A>
ASTG_HD T tilt_from_oct(const Dev& d, int l, int x, int y, int z, const A& oct) {
    T v = oct.get(req(d, l, x, y, z));
    double count = 1;
    for (int m = -1; m <= 0; ++m)
        for (int n = -1; n <= 0; ++n)
            for (int k = -1; k <= 0; ++k) {
                if (m == 0 && n == 0 && k == 0) continue;
                if (oct_valid(d, l, x + m, y + n, z + k)) {
                    int t = get(d, l, x + m, y + n, z + k);
                    if (t >= 0) { v = v + oct.get(t); count += 1; }
                }
            }
    return v / count;
}
// OctreeOmniGrid3<T>::interpolateClosedJoint, include/octree_omni_grid3.h:306-337
template <class T, class A>
__global__ void k_closed_joint(Dev d, A oct, A til, const double* te) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.nTJ) return;
    int tj = d.tj[i];
    int l = slot_l(d, tj), x = slot_x(d, tj), y = slot_y(d, tj), z = slot_z(d, tj);
    if (te[tj] < d.ldh[l]) { l -= 1; x <<= 1; y <<= 1; z <<= 1; }
    for (int k = 0; k < 6; ++k) {
        int tx = x + OCT_NB[k][0], ty = y + OCT_NB[k][1], tz = z + OCT_NB[k][2];
        int t = get(d, l, tx, ty, tz);
        if (t >= 0) til.set(t, tilt_from_oct<T>(d, l, tx, ty, tz, oct));
    }
}
template <class T, class A>
__global__ void k_closed_by_half(Dev d, A oct, A til, const uint32_t* tf) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.nCBH) return;
    int s = d.cbh[i];
    if ((tf[s] & TF_CLOSED) && tf_dir(tf[s]) == -1)
        til.set(s, tilt_from_oct<T>(d, slot_l(d, s), slot_x(d, s), slot_y(d, s), slot_z(d, s), oct));
}

struct ScalarAcc {
    double* p;
    ASTG_HD double zero() const { return 0.0; }
    ASTG_HD double get(int s) const { return p[s]; }
    ASTG_HD void set(int s, double v) const { p[s] = v; }
    ASTG_HD double operator()(int s) const { return p[s]; }
};
struct Vec3Acc {
    double* p;
    ASTG_HD V3 zero() const { return v3(0, 0, 0); }
    ASTG_HD V3 get(int s) const { return v3(p[3 * s], p[3 * s + 1], p[3 * s + 2]); }
    ASTG_HD void set(int s, V3 v) const { p[3 * s] = v.x; p[3 * s + 1] = v.y; p[3 * s + 2] = v.z; }
    ASTG_HD V3 operator()(int s) const { return get(s); }
};

// OctreeOmniGrid3<T>::updateGhost, include/octree_omni_grid3.h:136-143
template <class T, class A>
static void omni_ghost(const Dev& d, A oct, A til, const double* te, const uint32_t* tf, cudaStream_t st) {
    for (int l = 0; l < d.L; ++l)
        if (d.lG[l]) ASTG_LAUNCH(k_cell_ghost_avg<T, A><<<nblk(d.lG[l]), TB, 0, st>>>(d, oct, l));
    for (int l = 0; l < d.L; ++l)
        if (d.lG[l]) ASTG_LAUNCH(k_cell_ghost_sample<T, A><<<nblk(d.lG[l]), TB, 0, st>>>(d, oct, l));
    ASTG_LAUNCH(k_vertex_ghost<T, A><<<nblk(d.S), TB, 0, st>>>(d, til));
    for (int l = 0; l < d.L; ++l)
        if (d.lG[l]) ASTG_LAUNCH(k_cell_ghost_joint<T, A><<<nblk(d.lG[l]), TB, 0, st>>>(d, oct, til, l));
    if (d.nTJ) ASTG_LAUNCH(k_closed_joint<T, A><<<nblk(d.nTJ), TB, 0, st>>>(d, oct, til, te));
    if (d.nCBH) ASTG_LAUNCH(k_closed_by_half<T, A><<<nblk(d.nCBH), TB, 0, st>>>(d, oct, til, tf));
}

void launch_scalar_ghost(const Dev& d, double* oct, double* til, const double* te, const uint32_t* tf, cudaStream_t st) {
    omni_ghost<double, ScalarAcc>(d, ScalarAcc{oct}, ScalarAcc{til}, te, tf, st);
}
void launch_dual_ghost(const Dev& d, const Fields& F, cudaStream_t st) {
    omni_ghost<V3, Vec3Acc>(d, Vec3Acc{F.dualO}, Vec3Acc{F.dualT}, F.te, F.tf, st);
}

void launch_source(const Dev& d, const Fields& F, cudaStream_t st) {
    ASTG_LAUNCH(k_source_slots<<<nblk(d.S), TB, 0, st>>>(d, F));
    if (d.H) ASTG_LAUNCH(k_source_half<<<nblk(d.H), TB, 0, st>>>(d, F));
}

// ------------------------------------------------------------------ buoyancy
// src/octree_omnigrid_solver3.cpp:917-972; amb points at the device mean temperature
ASTG_HD inline double force_at(const Dev& d, const Fields& F, V3 p, double amb) {
    double dv, hv;
    scalar_sample2(d, p, F.dO, F.dT, F.hO, F.hT, F.tf, &dv, &hv);
    return d.buoyD * dv + d.buoyT * (hv - amb);
}
__global__ void k_force_mac(Dev d, Fields F, const double* amb, double dt) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.S || ghost(d, s)) return;
    if (!mac_valid(d, 2, slot_l(d, s), slot_x(d, s), slot_y(d, s), slot_z(d, s))) return;
    double* w = F.mac + 2 * (size_t)d.S + s;
    *w = *w + dt * force_at(d, F, mac_pos(d, 2, s), *amb);
}
// one thread per (tilt, slot)
__global__ void k_force_tilt(Dev d, Fields F, const uint8_t* open, const double* amb, double dt) {
    long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= 8LL * d.S) return;
    int s = (int)(idx >> 3), k = (int)(idx & 7);
    if (ghost(d, s) || !open[s]) return;
    double nf = tilt_up(k, 2) * force_at(d, F, tilt_pos(vert_pos(d, s), k, F.te[s]), *amb);
    F.tv[(size_t)s * 8 + k] = F.tv[(size_t)s * 8 + k] + dt * nf;
}
// one thread per (half tilt, slot); slots the half tilt does not use get + dt * 0
__global__ void k_force_half(Dev d, Fields F, const double* amb, double dt) {
    long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= 8LL * d.H) return;
    int i = (int)(idx >> 3), k = (int)(idx & 7);
    int hs = d.half[i];
    int dir = tf_dir(F.tf[hs]);
    int q = -1;
    for (int j = 0; j < 5; ++j)
        if (HALF_SLOT[dir][j] == k) q = j;
    double nf = 0;
    if (q >= 0) {
        V3 c = vert_pos(d, hs);
        V3 p = (q == 4) ? c : tilt_pos(c, k, F.te[hs]);
        double tf = force_at(d, F, p, *amb);
        V3 dv = (q == 4) ? v3(HALF_DIR_POS[k][0], HALF_DIR_POS[k][1], HALF_DIR_POS[k][2]) : tilt_up3(k);
        nf = dot3(v3(0, 0, tf), dv);
    }
    F.tv[(size_t)hs * 8 + k] = F.tv[(size_t)hs * 8 + k] + dt * nf;
}
void launch_force(const Dev& d, const Fields& F, const uint8_t* open, const double* amb, double dt, cudaStream_t st) {
    ASTG_LAUNCH(k_force_mac<<<nblk(d.S), TB, 0, st>>>(d, F, amb, dt));
    ASTG_LAUNCH(k_force_tilt<<<nblk(8LL * d.S), TB, 0, st>>>(d, F, open, amb, dt));
    if (d.H) ASTG_LAUNCH(k_force_half<<<nblk(8LL * d.H), TB, 0, st>>>(d, F, amb, dt));
}

// ------------------------------------------------------------------ walls and velocity ghosts
// OmniBoundarySolver3::constrainVelocity(MAC), include/omni_boundary_solver3.h:97-161: the
// normal faces of closed walls are zeroed on every level, ghosts included
__global__ void k_walls(Dev d, double* mac) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.S) return;
    int r = d.lres[slot_l(d, s)];
    int x = slot_x(d, s), y = slot_y(d, s), z = slot_z(d, s);
    size_t S = d.S;
    if ((d.closedMask & 1) && x == r - 1) mac[s] = 0;
    if ((d.closedMask & 2) && x == 0) mac[s] = 0;
    if ((d.closedMask & 4) && y == r - 1) mac[S + s] = 0;
    if ((d.closedMask & 8) && y == 0) mac[S + s] = 0;
    if ((d.closedMask & 16) && z == r - 1) mac[2 * S + s] = 0;
    if ((d.closedMask & 32) && z == 0) mac[2 * S + s] = 0;
}
// OctreeOmniFaceCenteredGrid3::updateGhost, include/octree_omni_face_centered_grid3.h:97-120
__global__ void k_mac_ghost_zero(Dev d, double* mac) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.S || !ghost(d, s)) return;
    mac[s] = 0;
    mac[(size_t)d.S + s] = 0;
    mac[2 * (size_t)d.S + s] = 0;
}
__global__ void k_mac_ghost_sample(Dev d, double* mac, int l, int fromCoarse) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.lG[l]) return;
    int s = d.loff[l] + d.lN[l] + i;
    if (((slot_f(d, s) & SF_FROM_COARSE) != 0) != (fromCoarse != 0)) return;
    for (int a = 0; a < 3; ++a) mac[(size_t)a * d.S + s] = mac_sample_one(d, a, mac_pos(d, a, s), mac);
}
// updateGhostFromHalfTilt, src/octree_omni_face_centered_grid3.cpp:162-173 (only the last half
// tilt of the list that targets a face writes it, as in the reference's sequential loop)
__global__ void k_mac_from_half(Dev d, Fields F, const uint8_t* lastWriter) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.H || !lastWriter[i]) return;
    int hs = d.half[i];
    int dir = tf_dir(F.tf[hs]);
    int a = dir % 3;
    int t = req(d, slot_l(d, hs) + 1, slot_x(d, hs) >> 1, slot_y(d, hs) >> 1, slot_z(d, hs) >> 1);
    F.mac[(size_t)a * d.S + t] = F.tv[(size_t)hs * 8 + HALF_SLOT[dir][4]];
}
// OctreeOmniTiltGrid3::updateGhost, include/octree_omni_tilt_grid3.h:56-74
__global__ void k_tilt_ghost(Dev d, Fields F, int l) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.lG[l]) return;
    int s = d.loff[l] + d.lN[l] + i;
    if (F.tf[s] & TF_HALF) return;
    int x = slot_x(d, s), y = slot_y(d, s), z = slot_z(d, s);
    int src;
    if (slot_f(d, s) & SF_FROM_COARSE) {
        if ((x & 1) || (y & 1) || (z & 1)) {
            for (int k = 0; k < 8; ++k) F.tv[(size_t)s * 8 + k] = 0;
            return;
        }
        src = req(d, l + 1, x >> 1, y >> 1, z >> 1);
    } else {
        src = req(d, l - 1, x << 1, y << 1, z << 1);
    }
    for (int k = 0; k < 8; ++k) F.tv[(size_t)s * 8 + k] = F.tv[(size_t)src * 8 + k];
}
void launch_walls(const Dev& d, double* mac, cudaStream_t st) { ASTG_LAUNCH(k_walls<<<nblk(d.S), TB, 0, st>>>(d, mac)); }
void launch_walls_and_ghost(const Dev& d, const Fields& F, const uint8_t* lastWriter, cudaStream_t st) {
    ASTG_LAUNCH(k_walls<<<nblk(d.S), TB, 0, st>>>(d, F.mac));
    launch_velocity_ghost(d, F, lastWriter, st);
}
// OctreeOmniFaceCenteredGrid3::updateGhost (include/octree_omni_face_centered_grid3.h:97-120)
void launch_velocity_ghost(const Dev& d, const Fields& F, const uint8_t* lastWriter, cudaStream_t st) {
    ASTG_LAUNCH(k_mac_ghost_zero<<<nblk(d.S), TB, 0, st>>>(d, F.mac));
    for (int l = 0; l < d.L; ++l)
        if (d.lG[l]) ASTG_LAUNCH(k_mac_ghost_sample<<<nblk(d.lG[l]), TB, 0, st>>>(d, F.mac, l, 0));
    if (d.H) ASTG_LAUNCH(k_mac_from_half<<<nblk(d.H), TB, 0, st>>>(d, F, lastWriter));
    for (int l = 0; l < d.L; ++l)
        if (d.lG[l]) ASTG_LAUNCH(k_mac_ghost_sample<<<nblk(d.lG[l]), TB, 0, st>>>(d, F.mac, l, 1));
    for (int l = 0; l < d.L; ++l)
        if (d.lG[l]) ASTG_LAUNCH(k_tilt_ghost<<<nblk(d.lG[l]), TB, 0, st>>>(d, F, l));
}

// ------------------------------------------------------------------ pressure-gradient update
// src/octree_omnigrid_solver3.cpp:682-847
ASTG_HD inline int p_oct_at(const Dev& d, const int* pO, int l, int x, int y, int z) { return pO[req(d, l, x, y, z)]; }

__global__ void k_pu_mac(Dev d, Fields F, const int* pO, const double* p, double dt) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.S || ghost(d, s)) return;
    int l = slot_l(d, s), x = slot_x(d, s), y = slot_y(d, s), z = slot_z(d, s);
    double h = d.ldh[l];
    double k0 = dt / d.rho;
    double p0 = 0;
    if (oct_valid(d, l, x, y, z) && pO[s] >= 0) p0 = p[pO[s]];
    for (int a = 0; a < 3; ++a) {
        if (!mac_valid(d, a, l, x, y, z)) continue;
        double* u = F.mac + (size_t)a * d.S + s;
        if (d.wMac[(size_t)a * d.S + s] <= 0) { *u = 0; continue; }
        int id0 = x - (a == 0), id1 = y - (a == 1), id2 = z - (a == 2);
        double p1 = 0;
        if (oct_valid(d, l, id0, id1, id2)) {
            int ti = p_oct_at(d, pO, l, id0, id1, id2);
            if (ti >= 0) p1 = p[ti];
        }
        *u = *u - k0 * (p0 - p1) / h;
    }
}
__global__ void k_pu_tilt(Dev d, Fields F, const uint8_t* open, const int* pO, const int* pT, const double* p, double dt) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.S || ghost(d, s) || !open[s]) return;
    int ci = pT[s];
    double k0 = dt / d.rho;
    double p0 = ci >= 0 ? p[ci] : 0;
    double* nv = F.tv + (size_t)s * 8;
    const double* tw = d.wTilt + (size_t)s * 8;
    int l = slot_l(d, s), x = slot_x(d, s), y = slot_y(d, s), z = slot_z(d, s);
    double out[8];
    for (int k = 0; k < 8; ++k) {
        NbOct nb = tilt_nb_oct(d, l, x, y, z, k);
        if (tw[k] > 0 && nb.some) {
            double h2 = d.ldh[nb.l];
            double p1 = 0;
            if (oct_valid(d, nb.l, nb.x, nb.y, nb.z)) {
                int ti = p_oct_at(d, pO, nb.l, nb.x, nb.y, nb.z);
                if (ti >= 0) p1 = p[ti];
            }
            out[k] = nv[k] - k0 * (k < 4 ? 1 : -1) / (h2 * SQRT3 * 0.5) * (p1 - p0);
        } else out[k] = 0;
    }
    for (int k = 0; k < 8; ++k) nv[k] = out[k];
}
__global__ void k_pu_half(Dev d, Fields F, const int* pO, const int* pT, const double* p, double dt) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.H) return;
    int hs = d.half[i];
    int dir = tf_dir(F.tf[hs]);
    int ci = pT[hs];
    int l = slot_l(d, hs), x = slot_x(d, hs), y = slot_y(d, hs), z = slot_z(d, hs);
    double k0 = dt / d.rho;
    double p0 = ci >= 0 ? p[ci] : 0;
    double nv[8];
    for (int k = 0; k < 8; ++k) nv[k] = F.tv[(size_t)hs * 8 + k];
    const double* tw = d.wTilt + (size_t)hs * 8;
    int id[3] = {x >> 1, y >> 1, z >> 1};
    id[dir % 3] -= dir < 3 ? 1 : 0;
    int fsl = HALF_SLOT[dir][4];
    if (tw[fsl] > 0) {
        int ti = p_oct_at(d, pO, l + 1, id[0], id[1], id[2]);
        double p1 = ti >= 0 ? p[ti] : 0;
        nv[fsl] -= k0 * (dir < 3 ? 1 : -1) / d.ldh[l] * (p0 - p1);
    } else nv[fsl] = 0;
    for (int k = 0; k < 8; ++k) {
        if (tw[k] > 0 && half_listed(dir, k)) {
            int nx = x + TILT_NB_OCT[k][0], ny = y + TILT_NB_OCT[k][1], nz = z + TILT_NB_OCT[k][2];
            double p1 = 0;
            if (oct_valid(d, l, nx, ny, nz)) {
                int ti = p_oct_at(d, pO, l, nx, ny, nz);
                if (ti >= 0) p1 = p[ti];
            }
            nv[k] = nv[k] - k0 * (k < 4 ? 1 : -1) / (d.ldh[l] * SQRT3 * 0.5) * (p1 - p0);
        } else if (k != fsl) nv[k] = 0;
    }
    for (int k = 0; k < 8; ++k) F.tv[(size_t)hs * 8 + k] = nv[k];
}
void launch_pressure_update(const Dev& d, const Fields& F, const uint8_t* open, const int* pO, const int* pT,
                            const double* p, double dt, cudaStream_t st) {
    ASTG_LAUNCH(k_pu_mac<<<nblk(d.S), TB, 0, st>>>(d, F, pO, p, dt));
    ASTG_LAUNCH(k_pu_tilt<<<nblk(d.S), TB, 0, st>>>(d, F, open, pO, pT, p, dt));
    if (d.H) ASTG_LAUNCH(k_pu_half<<<nblk(d.H), TB, 0, st>>>(d, F, pO, pT, p, dt));
}

// ------------------------------------------------------------------ dual velocity
// OctreeOmniFaceCenteredGrid3::updateDualGrid, src/octree_omni_face_centered_grid3.cpp:32-159.
// Matrix-vector products follow Eigen 3.3.7's evaluation into a Vector3d: rows 0-1 accumulate
// in column order (one SSE2 packet), row 2 is an unrolled pairwise tree.
__global__ void k_dual_tilt(Dev d, Fields F) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.S || ghost(d, s)) return;
    double* o = F.dualT + 3 * (size_t)s;
    if (F.tf[s] & TF_CLOSED) { o[0] = o[1] = o[2] = 0; return; }
    const double* g = F.tv + (size_t)s * 8;
    double v4[4] = {(g[0] + g[6]) * 0.5, (g[1] + g[7]) * 0.5, (g[2] + g[4]) * 0.5, (g[3] + g[5]) * 0.5};
    const double s3 = INV_SQRT3 * (3.0 / 4.0);
    const double M[3][4] = {{s3, -s3, -s3, s3}, {s3, s3, -s3, -s3}, {s3, s3, s3, s3}};
    for (int k = 0; k < 2; ++k) o[k] = ((M[k][0] * v4[0] + M[k][1] * v4[1]) + M[k][2] * v4[2]) + M[k][3] * v4[3];
    o[2] = (M[2][0] * v4[0] + M[2][1] * v4[1]) + (M[2][2] * v4[2] + M[2][3] * v4[3]);
}
ASTG_HD inline V3 apply_m37(const Dev& d, int bits, const double v[7]) {
    const double* M = d.M37 + (size_t)bits * 21;
    double o[3];
    for (int k = 0; k < 2; ++k) {
        double acc = M[k * 7 + 0] * v[0];
        for (int r = 1; r < 7; ++r) acc = acc + M[k * 7 + r] * v[r];
        o[k] = acc;
    }
    double a[7];
    for (int r = 0; r < 7; ++r) a[r] = M[14 + r] * v[r];
    o[2] = (a[0] + (a[1] + a[2])) + ((a[3] + a[4]) + (a[5] + a[6]));
    return v3(o[0], o[1], o[2]);
}
__global__ void k_dual_oct(Dev d, Fields F) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.S || ghost(d, s)) return;
    int l = slot_l(d, s), x = slot_x(d, s), y = slot_y(d, s), z = slot_z(d, s);
    double* out = F.dualO + 3 * (size_t)s;
    if (!oct_valid(d, l, x, y, z)) { out[0] = out[1] = out[2] = 0; return; }
    double h = d.ldh[l];
    double sq = SQRT3 * h, hsq = sq * 0.5;
    int nj[8], ts[8];
    for (int i = 0; i < 8; ++i) {
        ts[i] = req(d, l, x + OCT_NB_TILT[i][0], y + OCT_NB_TILT[i][1], z + OCT_NB_TILT[i][2]);
        uint32_t f = F.tf[ts[i]];
        nj[i] = ((f & TF_TJOINT) && fabs(F.te[ts[i]] - h) < EPS) || (f & TF_HALF);
    }
    const double* U0 = F.mac;
    const double* U1 = F.mac + d.S;
    const double* U2 = F.mac + 2 * (size_t)d.S;
    double v[7] = {0, 0, 0, 0, 0, 0, 0};
    int cnt[7] = {0, 0, 0, 0, 0, 0, 0};
    if (!((nj[1] && nj[6]) || (nj[2] && nj[5]))) { v[0] += U0[s]; cnt[0]++; }
    if (!((nj[0] && nj[7]) || (nj[3] && nj[4]))) { v[0] += U0[req(d, l, x + 1, y, z)]; cnt[0]++; }
    if (!((nj[2] && nj[7]) || (nj[3] && nj[6]))) { v[1] += U1[s]; cnt[1]++; }
    if (!((nj[0] && nj[5]) || (nj[1] && nj[4]))) { v[1] += U1[req(d, l, x, y + 1, z)]; cnt[1]++; }
    if (!((nj[4] && nj[6]) || (nj[5] && nj[7]))) { v[2] += U2[s]; cnt[2]++; }
    if (!((nj[0] && nj[2]) || (nj[1] && nj[3]))) { v[2] += U2[req(d, l, x, y, z + 1)]; cnt[2]++; }
    for (int i = 0; i < 4; ++i) {
        int slot = i, re = ((i & 1) ? 8 : 6) - i, vs = i + 3;
        uint32_t fn = F.tf[ts[slot]], fr = F.tf[ts[re]];
        double en = F.te[ts[slot]], er = F.te[ts[re]];
        if (!(fn & TF_CLOSED) || (fn & TF_HALF)) { v[vs] += F.tv[(size_t)ts[slot] * 8 + re]; cnt[vs]++; }
        if (!(fr & TF_CLOSED) || (fr & TF_HALF)) {
            double t = F.tv[(size_t)ts[re] * 8 + slot];
            // "e * INV_SQRT3" with the reference's unparenthesised macro is e * 1.0 / SQRT3
            v[vs] = cnt[vs] == 0 ? t
                                 : ((v[vs] * (hsq - er * 1.0 / SQRT3) + t * (hsq - en * 1.0 / SQRT3)) /
                                    (sq - en * 1.0 / SQRT3 - er * 1.0 / SQRT3));
            cnt[vs]++;
        }
    }
    for (int i = 0; i < 3; ++i) v[i] = v[i] / (cnt[i] + EPS);
    int bits = ((cnt[0] > 0) << 6) | ((cnt[1] > 0) << 5) | ((cnt[2] > 0) << 4) | ((cnt[3] > 1 || nj[0] || nj[6]) << 3) |
               ((cnt[4] > 1 || nj[1] || nj[7]) << 2) | ((cnt[5] > 1 || nj[2] || nj[4]) << 1) | (cnt[6] > 1 || nj[3] || nj[5]);
    V3 f = apply_m37(d, bits, v);
    out[0] = f.x; out[1] = f.y; out[2] = f.z;
}
__global__ void k_dual_half(Dev d, Fields F) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.H) return;
    int hs = d.half[i];
    int dir = tf_dir(F.tf[hs]);
    const double* g = F.tv + (size_t)hs * 8;
    double v[7] = {0, 0, 0, 0, 0, 0, 0};
    int axis = dir % 3;
    v[axis] = g[HALF_SLOT[dir][4]];
    for (int q = 0; q < 4; ++q) {
        int slot = HALF_SLOT[dir][q];
        int re = ((slot & 1) ? 8 : 6) - slot;
        int idx = slot < re ? slot : re;
        v[idx + 3] = g[slot];
    }
    int bits = ((axis == 0) << 6) | ((axis == 1) << 5) | ((axis == 2) << 4) | 0xf;
    V3 f = apply_m37(d, bits, v);
    double* o = F.dualT + 3 * (size_t)hs;
    o[0] = f.x; o[1] = f.y; o[2] = f.z;
}
void launch_dual_update(const Dev& d, const Fields& F, cudaStream_t st) {
    ASTG_LAUNCH(k_dual_tilt<<<nblk(d.S), TB, 0, st>>>(d, F));
    ASTG_LAUNCH(k_dual_oct<<<nblk(d.S), TB, 0, st>>>(d, F));
    if (d.H) ASTG_LAUNCH(k_dual_half<<<nblk(d.H), TB, 0, st>>>(d, F));
}
void launch_dual(const Dev& d, const Fields& F, cudaStream_t st) {
    launch_dual_update(d, F, st);
    launch_dual_ghost(d, F, st);
}

// ------------------------------------------------------------------ tilt adaptivity
// src/octree_omnigrid_solver3.cpp:1125-1166 (dThreshold 0.02, vThreshold epsilon, max 1000)
__global__ void k_adjust_open(Dev d, Fields F, uint8_t* open, const uint8_t* fixedf, double dt) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.S || ghost(d, s) || fixedf[s]) return;
    const double dTh = 0.02, vTh = EPS, maxTh = 1000;
    if (open[s]) {
        double dd = F.dT[s];
        if (dd < dTh || dd > maxTh) open[s] = 0;
    } else {
        V3 pos = vert_pos(d, s);
        V3 v = vel_sample(d, pos, F);
        if (sqrt(v.x * v.x + v.y * v.y + v.z * v.z) > vTh) {
            V3 old = pos - v * dt;
            double dd = scalar_sample(d, old, F.dO, F.dT, F.tf);
            if (dd > dTh && dd < maxTh) open[s] = 1;
        }
    }
}
// OctreeVertexCenteredGrid3<TiltENodeS>::updateGhost, src/octree_vertex_centered_grid3.cpp:26-45
__global__ void k_layout_ghost(Dev d, uint8_t* open, uint8_t* fixedf, int l) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.lG[l]) return;
    int s = d.loff[l] + d.lN[l] + i;
    int x = slot_x(d, s), y = slot_y(d, s), z = slot_z(d, s);
    int src;
    if (slot_f(d, s) & SF_FROM_COARSE) {
        if ((x & 1) || (y & 1) || (z & 1)) return;
        src = req(d, l + 1, x >> 1, y >> 1, z >> 1);
    } else src = req(d, l - 1, x << 1, y << 1, z << 1);
    open[s] = open[src];
    fixedf[s] = fixedf[src];
}
// TiltENode::setE (include/tilt_e_node.h:41-56) on the adjusted buffer
__global__ void k_adjust_e(Dev d, double* te, uint32_t* tf, const uint8_t* open, const uint8_t* fixedf) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.S || ghost(d, s) || fixedf[s]) return;
    uint32_t f = tf[s];
    if (f & TF_FIXED) return;
    double ne;
    if (open[s]) {
        double m = d.ldh[slot_l(d, s)] * 0.5;
        ne = m;
        if (ne <= 0) { f |= TF_CLOSED; f &= ~TF_LARGEST; ne = 0; }
        else if (m > 0 && ne >= m) { f &= ~TF_CLOSED; f |= TF_LARGEST; ne = m; }
        else { f &= ~(TF_CLOSED | TF_LARGEST); }
    } else {
        f |= TF_CLOSED;
        f &= ~TF_LARGEST;
        ne = 0;
    }
    te[s] = ne;
    tf[s] = f;
}
// OctreeVertexCenteredGrid3<TiltENode>::updateGhost, src/octree_vertex_centered_grid3.cpp:6-24
__global__ void k_te_ghost(Dev d, double* te, uint32_t* tf, int l) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.lG[l]) return;
    int s = d.loff[l] + d.lN[l] + i;
    int x = slot_x(d, s), y = slot_y(d, s), z = slot_z(d, s);
    int src;
    if (slot_f(d, s) & SF_FROM_COARSE) {
        if ((x & 1) || (y & 1) || (z & 1)) return;
        src = req(d, l + 1, x >> 1, y >> 1, z >> 1);
    } else src = req(d, l - 1, x << 1, y << 1, z << 1);
    te[s] = te[src];
    tf[s] = tf[src];
}
void launch_tilt_e_ghost(const Dev& d, double* te, uint32_t* tf, cudaStream_t st) {
    for (int l = 0; l < d.L; ++l)
        if (d.lG[l]) ASTG_LAUNCH(k_te_ghost<<<nblk(d.lG[l]), TB, 0, st>>>(d, te, tf, l));
}
void launch_adjust(const Dev& d, const Fields& cur, const Fields& nxt, uint8_t* open, uint8_t* fixedf, double dt,
                   cudaStream_t st) {
    ASTG_LAUNCH(k_adjust_open<<<nblk(d.S), TB, 0, st>>>(d, cur, open, fixedf, dt));
    for (int l = 0; l < d.L; ++l)
        if (d.lG[l]) ASTG_LAUNCH(k_layout_ghost<<<nblk(d.lG[l]), TB, 0, st>>>(d, open, fixedf, l));
    ASTG_LAUNCH(k_adjust_e<<<nblk(d.S), TB, 0, st>>>(d, nxt.te, nxt.tf, open, fixedf));
    launch_tilt_e_ghost(d, nxt.te, nxt.tf, st);
}

// ------------------------------------------------------------------ advection
// src/octree_omnigrid_solver3.cpp:850-914 and SemiLagrangianOctreeOmniFace3,
// include/advection.h:195-239.  cur is the source, nxt the destination (its tilt-E is the
// adjusted one).
__global__ void k_adv_scalar_oct(Dev d, Fields cur, Fields nxt, double dt) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.S || ghost(d, s)) return;
    V3 o = back_trace(d, cell_pos(d, s), dt, cur);
    scalar_sample2(d, o, cur.dO, cur.dT, cur.hO, cur.hT, cur.tf, &nxt.dO[s], &nxt.hO[s]);
}
__global__ void k_adv_scalar_tilt(Dev d, Fields cur, Fields nxt, const uint8_t* open, double dt) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.S || ghost(d, s) || !open[s]) return;
    V3 o = back_trace(d, vert_pos(d, s), dt, cur);
    scalar_sample2(d, o, cur.dO, cur.dT, cur.hO, cur.hT, cur.tf, &nxt.dT[s], &nxt.hT[s]);
}
__global__ void k_adv_scalar_half(Dev d, Fields cur, Fields nxt, double dt) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.H) return;
    int hs = d.half[i];
    V3 o = back_trace(d, vert_pos(d, hs), dt, cur);
    scalar_sample2(d, o, cur.dO, cur.dT, cur.hO, cur.hT, cur.tf, &nxt.dT[hs], &nxt.hT[hs]);
}
// one thread per (axis, slot)
__global__ void k_adv_mac(Dev d, Fields cur, Fields nxt, double dt) {
    long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= 3LL * d.S) return;
    int a = (int)(idx / d.S), s = (int)(idx - (long long)a * d.S);
    if (ghost(d, s)) return;
    V3 o = back_trace(d, mac_pos(d, a, s), dt, cur);
    nxt.mac[(size_t)a * d.S + s] = vel_sample_axis(d, o, cur, a);
}
// one thread per (tilt, slot)
__global__ void k_adv_tilt(Dev d, Fields cur, Fields nxt, double dt) {
    long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= 8LL * d.S) return;
    int s = (int)(idx >> 3), k = (int)(idx & 7);
    if (ghost(d, s) || (nxt.tf[s] & TF_CLOSED)) return;
    V3 o = back_trace(d, tilt_pos(vert_pos(d, s), k, nxt.te[s]), dt, cur);
    nxt.tv[(size_t)s * 8 + k] = dot3(vel_sample(d, o, cur), tilt_up3(k));
}
// one thread per (half tilt, slot); unused slots are zero
__global__ void k_adv_half(Dev d, Fields cur, Fields nxt, double dt) {
    long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= 8LL * d.H) return;
    int i = (int)(idx >> 3), k = (int)(idx & 7);
    int hs = d.half[i];
    int dir = tf_dir(nxt.tf[hs]);
    int q = -1;
    for (int j = 0; j < 5; ++j)
        if (HALF_SLOT[dir][j] == k) q = j;
    double v = 0;
    if (q >= 0) {
        V3 c = vert_pos(d, hs);
        V3 pos = (q == 4) ? c : tilt_pos(c, k, nxt.te[hs]);
        V3 o = back_trace(d, pos, dt, cur);
        V3 dv = (q == 4) ? v3(HALF_DIR_POS[k][0], HALF_DIR_POS[k][1], HALF_DIR_POS[k][2]) : tilt_up3(k);
        v = dot3(vel_sample(d, o, cur), dv);
    }
    nxt.tv[(size_t)hs * 8 + k] = v;
}
__global__ void k_decay(Dev d, Fields F) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.S) return;
    F.dO[s] *= d.decay;
    F.dT[s] *= d.decay;
    F.hO[s] *= d.decay;
    F.hT[s] *= d.decay;
}
void launch_advect_scalars(const Dev& d, const Fields& cur, const Fields& nxt, const uint8_t* open, double dt,
                           cudaStream_t st) {
    ASTG_LAUNCH(k_adv_scalar_oct<<<nblk(d.S), TB, 0, st>>>(d, cur, nxt, dt));
    ASTG_LAUNCH(k_adv_scalar_tilt<<<nblk(d.S), TB, 0, st>>>(d, cur, nxt, open, dt));
    if (d.H) ASTG_LAUNCH(k_adv_scalar_half<<<nblk(d.H), TB, 0, st>>>(d, cur, nxt, dt));
    launch_scalar_ghost(d, nxt.dO, nxt.dT, nxt.te, nxt.tf, st);
    launch_scalar_ghost(d, nxt.hO, nxt.hT, nxt.te, nxt.tf, st);
}
// the dual-grid correction of every tilt for the current velocity (see Fields::corrT)
__global__ void k_tilt_corr(Dev d, Fields F, double* corr) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.S) return;
    V3 m = mac_sample(d, vert_pos(d, s), F.mac);
    corr[3 * s] = F.dualT[3 * s] - m.x;
    corr[3 * s + 1] = F.dualT[3 * s + 1] - m.y;
    corr[3 * s + 2] = F.dualT[3 * s + 2] - m.z;
}
void launch_tilt_corr(const Dev& d, const Fields& F, double* corr, cudaStream_t st) {
    ASTG_LAUNCH(k_tilt_corr<<<nblk(d.S), TB, 0, st>>>(d, F, corr));
}
void launch_advect_velocity(const Dev& d, const Fields& cur, const Fields& nxt, double dt, cudaStream_t st) {
    ASTG_LAUNCH(k_adv_mac<<<nblk(3LL * d.S), TB, 0, st>>>(d, cur, nxt, dt));
    ASTG_LAUNCH(k_adv_tilt<<<nblk(8LL * d.S), TB, 0, st>>>(d, cur, nxt, dt));
    if (d.H) ASTG_LAUNCH(k_adv_half<<<nblk(8LL * d.H), TB, 0, st>>>(d, cur, nxt, dt));
}
void launch_decay(const Dev& d, const Fields& F, cudaStream_t st) { ASTG_LAUNCH(k_decay<<<nblk(d.S), TB, 0, st>>>(d, F)); }

// Largest MAC face value over all faces (3 x slots, ghosts included), starting from 0, as
// OctreeOmniGridSolver3::cfl takes it (src/octree_omnigrid_solver3.cpp:1066-1122): only positive
// values can raise it, and for those the IEEE bit patterns order like the values, so the maximum
// is an atomicMax on the bits (order-independent, exact).  *out must start at 0.
__global__ void k_max_face(const double* mac, long long n, unsigned long long* out) {
    unsigned long long m = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        double v = mac[i];
        if (v > 0) m = max(m, (unsigned long long)__double_as_longlong(v));
    }
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m > 0) atomicMax(out, m);
}
void launch_max_face(const Dev& d, const double* mac, unsigned long long* out, cudaStream_t st) {
    long long n = 3LL * d.S;
    int blocks = (int)std::min<long long>(nblk(n), 4LL * 152);
    ASTG_LAUNCH(k_max_face<<<blocks, TB, 0, st>>>(mac, n, out));
}

}  // namespace astg
