// Interpolation on the AST octree: scalar, MAC and velocity samplers, the level-transition
// sub-sampler and the cell-centred trilinear sampler.  Each function restates one reference
// routine (cited per function) with the same operand order.
#pragma once
#include "astg_device.cuh"

#ifndef ASTG_CONST
#define ASTG_CONST static __constant__
#endif

namespace astg {

// include/constants.h:85-155
ASTG_CONST int OCT_NB[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
ASTG_CONST int OCT_NB_TILT[8][3] = {{1, 1, 1}, {0, 1, 1}, {0, 0, 1}, {1, 0, 1}, {1, 1, 0}, {0, 1, 0}, {0, 0, 0}, {1, 0, 0}};
ASTG_CONST int OCT_NB_FACE[6][3] = {{1, 0, 0}, {0, 0, 0}, {0, 1, 0}, {0, 0, 0}, {0, 0, 1}, {0, 0, 0}};
ASTG_CONST int TILT_NB_OCT[8][3] = {{0, 0, 0},  {-1, 0, 0},  {-1, -1, 0},  {0, -1, 0},
                                    {0, 0, -1}, {-1, 0, -1}, {-1, -1, -1}, {0, -1, -1}};
ASTG_CONST int HALF_SLOT[6][5] = {{0, 3, 4, 7, 1}, {0, 1, 4, 5, 2}, {0, 1, 2, 3, 5},
                                  {1, 2, 5, 6, 0}, {2, 3, 6, 7, 4}, {4, 5, 6, 7, 3}};
ASTG_CONST double HALF_DIR_POS[6][3] = {{1, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {0, 1, 0}, {0, 0, 1}};
ASTG_CONST int TILT_UP_SIGN[8][3] = {{1, 1, 1},   {-1, 1, 1}, {-1, -1, 1}, {1, -1, 1},
                                     {-1, -1, 1}, {1, -1, 1}, {1, 1, 1},   {-1, 1, 1}};
ASTG_CONST int SAMPLE_MARKER[8][8] = {
    {0x1000, 0x011, 0x001, 0x101, 0x110, 0x010, 0x1000, 0x100},
    {0x011, 0x1000, 0x201, 0x001, 0x010, 0x210, 0x200, 0x1000},
    {0x001, 0x201, 0x1000, 0x021, 0x1000, 0x200, 0x220, 0x020},
    {0x101, 0x001, 0x021, 0x1000, 0x100, 0x1000, 0x020, 0x120},
    {0x110, 0x010, 0x1000, 0x100, 0x1000, 0x012, 0x002, 0x102},
    {0x010, 0x210, 0x200, 0x1000, 0x012, 0x1000, 0x202, 0x002},
    {0x1000, 0x200, 0x220, 0x020, 0x002, 0x202, 0x1000, 0x022},
    {0x100, 0x1000, 0x020, 0x120, 0x102, 0x002, 0x022, 0x1000}};

ASTG_HD inline double tilt_up(int k, int c) { return TILT_UP_SIGN[k][c] * INV_SQRT3; }
ASTG_HD inline V3 tilt_up3(int k) { return v3(tilt_up(k, 0), tilt_up(k, 1), tilt_up(k, 2)); }
ASTG_HD inline bool half_listed(int dir, int k) {
    return HALF_SLOT[dir][0] == k || HALF_SLOT[dir][1] == k || HALF_SLOT[dir][2] == k || HALF_SLOT[dir][3] == k;
}

// field accessors
struct ScalarAt {
    const double* p;
    ASTG_HD double operator()(int s) const { return p[s]; }
};
struct Vec3At {
    const double* p;
    ASTG_HD V3 operator()(int s) const { return v3(p[3 * s], p[3 * s + 1], p[3 * s + 2]); }
};

// cell-centred trilinear sample, include/octree_cell_centered_grid3.h:97-123
template <class T, class G>
ASTG_HD T cell_sample(const Dev& d, const G& g, V3 p) {
    int l = level_of(d, p.x, p.y, p.z);
    double h = d.ldh[l];
    int r = d.lres[l];
    int xi, yi, zi;
    double fx, fy, fz;
    bary(over_h(d, p.x, l) - 0.5, 0, r - 2, &xi, &fx);
    bary(over_h(d, p.y, l) - 0.5, 0, r - 2, &yi, &fy);
    bary(over_h(d, p.z, l) - 0.5, 0, r - 2, &zi, &fz);
    int x1 = imin(xi + 1, r - 2), y1 = imin(yi + 1, r - 2), z1 = imin(zi + 1, r - 2);
    return trilerp<T>(g(req(d, l, xi, yi, zi)), g(req(d, l, x1, yi, zi)), g(req(d, l, xi, y1, zi)), g(req(d, l, x1, y1, zi)),
                      g(req(d, l, xi, yi, z1)), g(req(d, l, x1, yi, z1)), g(req(d, l, xi, y1, z1)), g(req(d, l, x1, y1, z1)),
                      fx, fy, fz);
}

// getNeighborCubeValue, include/octree_util.h:133-185
template <class T, class GO, class GT>
ASTG_HD void neighbor_cube(const Dev& d, int l, int xi, int yi, int zi, int dir, T* v, const GO& oct, const GT& til,
                           const uint32_t* tf, bool tj) {
    int reDir = ((dir & 1) ? 8 : 6) - dir;
    T c = oct(req(d, l, xi, yi, zi));
    v[reDir] = c;
    for (int i = 0; i < 8; ++i) {
        int mk = SAMPLE_MARKER[dir][i];
        if (mk == 0x1000) continue;
        T t = c;
        double count = 1;
        int m0 = (mk >> 8) & 0xf, m1 = (mk >> 4) & 0xf, m2 = mk & 0xf;
        int m[3] = {m0, m1, m2};
        if (tj && l > 0) {
            bool flag = false;
            for (int k = 0; k < 3; ++k) {
                if (m[k] != 0 && m[(k + 1) % 3] == 0 && m[(k + 2) % 3] == 0) {  // face node
                    int id[3] = {xi, yi, zi};
                    id[k] += (m[k] == 1);
                    id[0] *= 2; id[1] *= 2; id[2] *= 2;
                    id[(k + 1) % 3] += 1;
                    id[(k + 2) % 3] += 1;
                    int s = get(d, l - 1, id[0], id[1], id[2]);
                    if (s >= 0 && (tf[s] & TF_HALF)) { v[i] = til(s); flag = true; }
                }
                if (m[k] == 0 && m[(k + 1) % 3] != 0 && m[(k + 2) % 3] != 0) {  // edge node
                    int tx = (xi << 1) + (dir == 0 || dir == 3 || dir == 4 || dir == 7) + OCT_NB_TILT[i][0];
                    int ty = (yi << 1) + ((dir % 4) < 2) + OCT_NB_TILT[i][1];
                    int tz = (zi << 1) + (dir < 4) + OCT_NB_TILT[i][2];
                    int s = get(d, l - 1, tx, ty, tz);
                    if (s >= 0 && !(slot_f(d, s) & SF_GHOST) && (tf[s] & TF_CLOSED_BY_T)) { v[i] = til(s); flag = true; }
                }
            }
            if (flag) continue;
        }
        int r2 = d.lres[l] - 2;
        for (int x = -(m0 == 2); x <= (m0 == 1); ++x)
            for (int y = -(m1 == 2); y <= (m1 == 1); ++y)
                for (int z = -(m2 == 2); z <= (m2 == 1); ++z) {
                    if (x == 0 && y == 0 && z == 0) continue;
                    int cx = imin(imax(0, xi + x), r2), cy = imin(imax(0, yi + y), r2), cz = imin(imax(0, zi + z), r2);
                    t = t + oct(req(d, l, cx, cy, cz));
                    count += 1;
                }
        v[i] = t / count;
    }
}

// OctreeOmniGrid3<T>::sampleSub, include/octree_omni_grid3.h:243-286.  Out of line: it runs only
// near level transitions, and inlining it at every sample site multiplies the samplers' code size
// (instruction-cache misses were the largest stall of the advection kernels)
template <class T, class GO, class GT>
__device__ __noinline__ T omni_sample_sub(const Dev& d, V3 p, const GO& oct, const GT& til, const uint32_t* tf) {
    int l = level_of(d, p.x, p.y, p.z);
    double h = d.ldh[l];
    int r = d.lres[l];
    double rx = over_h(d, p.x, l), ry = over_h(d, p.y, l), rz = over_h(d, p.z, l);
    int xi, yi, zi;
    double fx, fy, fz;
    bary(rx, 0, r - 1, &xi, &fx);
    bary(ry, 0, r - 1, &yi, &fy);
    bary(rz, 0, r - 1, &zi, &fz);
    int dir = fz >= 0.5 ? 0 : 4;
    dir += (fx >= 0.5) ? (fy >= 0.5 ? 0 : 3) : (fy >= 0.5 ? 1 : 2);
    int ts = req(d, l, xi + OCT_NB_TILT[dir][0], yi + OCT_NB_TILT[dir][1], zi + OCT_NB_TILT[dir][2]);
    uint32_t tn = tf[ts];
    if (!(tn & TF_HALF) && !(tn & TF_CLOSED_BY_T) && (tn & TF_CLOSED)) {
        // sampleGivenRelativePosition, include/octree_cell_centered_grid3.h:158-179
        int a, b, c;
        double ga, gb, gc;
        bary(rx - 0.5, 0, r - 2, &a, &ga);
        bary(ry - 0.5, 0, r - 2, &b, &gb);
        bary(rz - 0.5, 0, r - 2, &c, &gc);
        int a1 = imin(a + 1, r - 2), b1 = imin(b + 1, r - 2), c1 = imin(c + 1, r - 2);
        return trilerp<T>(oct(req(d, l, a, b, c)), oct(req(d, l, a1, b, c)), oct(req(d, l, a, b1, c)), oct(req(d, l, a1, b1, c)),
                          oct(req(d, l, a, b, c1)), oct(req(d, l, a1, b, c1)), oct(req(d, l, a, b1, c1)),
                          oct(req(d, l, a1, b1, c1)), ga, gb, gc);
    }
    T v[8];
    v[dir] = til(ts);
    neighbor_cube<T>(d, l, xi, yi, zi, dir, v, oct, til, tf, (tn & TF_TJOINT) != 0);
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
    return trilerp<T>(v[6], v[7], v[5], v[4], v[2], v[3], v[1], v[0], fx, fy, fz);
}

// level-transition test, include/octree_omni_grid3.h:172-175 and
// include/octree_omni_face_centered_grid3.h:61-64
ASTG_HD inline bool near_transition(const Dev& d, int l, int xi, int yi, int zi) {
    if (is_ghost_node(d, l, xi, yi, zi)) return true;
    if (l == 0 && get(d, 1, xi >> 1, yi >> 1, zi >> 1) >= 0) return true;
    if (l == 1 && get(d, 0, (xi << 1) + 1, (yi << 1) + 1, (zi << 1) + 1) >= 0) return true;
    if (l == 1 && get(d, 0, xi << 1, yi << 1, zi << 1) >= 0) return true;
    return false;
}

// OctreeOmniGrid3<double>::sample, correction-based, include/octree_omni_grid3.h:147-187, for one or
// two fields at the same point (density and heat): the point is located once; each value takes the
// same operations on the same inputs as a sample of its field alone
template <int NF>
ASTG_HD inline void scalar_sample_n(const Dev& d, V3 p, const double* const* oct, const double* const* til,
                                    const uint32_t* tf, double* out) {
    int l = level_of(d, p.x, p.y, p.z);
    int r = d.lres[l];
    int xi, yi, zi;
    double fx, fy, fz;
    bary(over_h(d, p.x, l) - 0.5, 0, r - 2, &xi, &fx);
    bary(over_h(d, p.y, l) - 0.5, 0, r - 2, &yi, &fy);
    bary(over_h(d, p.z, l) - 0.5, 0, r - 2, &zi, &fz);
    int x1 = imin(xi + 1, r - 2), y1 = imin(yi + 1, r - 2), z1 = imin(zi + 1, r - 2);
    int ts = req(d, l, xi + 1, yi + 1, zi + 1);
    if (near_transition(d, l, xi, yi, zi)) {
#pragma unroll
        for (int f = 0; f < NF; ++f) out[f] = omni_sample_sub<double>(d, p, ScalarAt{oct[f]}, ScalarAt{til[f]}, tf);
        return;
    }
    const int s000 = req(d, l, xi, yi, zi), s100 = req(d, l, x1, yi, zi), s010 = req(d, l, xi, y1, zi),
              s110 = req(d, l, x1, y1, zi), s001 = req(d, l, xi, yi, z1), s101 = req(d, l, x1, yi, z1),
              s011 = req(d, l, xi, y1, z1), s111 = req(d, l, x1, y1, z1);
    const uint32_t tn = tf[ts];
    const bool plain = (tn & TF_CLOSED) && !(tn & TF_HALF);
    const double mn = dmin(dmin(dmin(fx, fy), fz), dmin(dmin(1 - fx, 1 - fy), 1 - fz));
#pragma unroll
    for (int f = 0; f < NF; ++f) {
        const double* o = oct[f];
        double o000 = o[s000], o100 = o[s100], o010 = o[s010], o110 = o[s110], o001 = o[s001], o101 = o[s101],
               o011 = o[s011], o111 = o[s111];
        double ret = trilerp<double>(o000, o100, o010, o110, o001, o101, o011, o111, fx, fy, fz);
        if (!plain) {
            double diff = til[f][ts] - (1 / 8.0) * (o000 + o100 + o010 + o110 + o001 + o101 + o011 + o111);
            ret = ret + diff * 2.0 * mn;
        }
        out[f] = ret;
    }
}
ASTG_HD inline double scalar_sample(const Dev& d, V3 p, const double* oct, const double* til, const uint32_t* tf) {
    double v;
    scalar_sample_n<1>(d, p, &oct, &til, tf, &v);
    return v;
}
// density and heat at one point
ASTG_HD inline void scalar_sample2(const Dev& d, V3 p, const double* o0, const double* t0, const double* o1,
                                   const double* t1, const uint32_t* tf, double* v0, double* v1) {
    const double* o[2] = {o0, o1};
    const double* t[2] = {t0, t1};
    double v[2];
    scalar_sample_n<2>(d, p, o, t, tf, v);
    *v0 = v[0];
    *v1 = v[1];
}

// OctreeFaceCenteredGrid3::sampleX/Y/Z, src/octree_face_centered_grid3.cpp:36-121
ASTG_HD inline double mac_axis(const Dev& d, int a, int l, double rx, double ry, double rz, const double* U) {
    int r = d.lres[l];
    double q[3] = {rx, ry, rz};
    int id[3], id1[3];
    double f[3];
    for (int k = 0; k < 3; ++k) {
        if (k == a) {
            bary(q[k], 0, r - 1, &id[k], &f[k]);
            id1[k] = imin(id[k] + 1, r - 1);
        } else {
            bary(q[k] - 0.5, 0, r - 2, &id[k], &f[k]);
            id1[k] = imin(id[k] + 1, r - 2);
        }
    }
    return trilerp<double>(U[req(d, l, id[0], id[1], id[2])], U[req(d, l, id1[0], id[1], id[2])],
                           U[req(d, l, id[0], id1[1], id[2])], U[req(d, l, id1[0], id1[1], id[2])],
                           U[req(d, l, id[0], id[1], id1[2])], U[req(d, l, id1[0], id[1], id1[2])],
                           U[req(d, l, id[0], id1[1], id1[2])], U[req(d, l, id1[0], id1[1], id1[2])], f[0], f[1], f[2]);
}
// the MAC grid's velocity at level l, (rx, ry, rz) = p / dx_l
ASTG_HD inline V3 mac_sample_at(const Dev& d, int l, double rx, double ry, double rz, const double* mac) {
    return v3(mac_axis(d, 0, l, rx, ry, rz, mac), mac_axis(d, 1, l, rx, ry, rz, mac + d.S),
              mac_axis(d, 2, l, rx, ry, rz, mac + 2 * (size_t)d.S));
}
ASTG_HD inline V3 mac_sample(const Dev& d, V3 p, const double* mac) {
    int l = level_of(d, p.x, p.y, p.z);
    return mac_sample_at(d, l, over_h(d, p.x, l), over_h(d, p.y, l), over_h(d, p.z, l), mac);
}
ASTG_HD inline double mac_sample_one(const Dev& d, int a, V3 p, const double* mac) {
    int l = level_of(d, p.x, p.y, p.z);
    double h = d.ldh[l];
    return mac_axis(d, a, l, over_h(d, p.x, l), over_h(d, p.y, l), over_h(d, p.z, l), mac + (size_t)a * d.S);
}

// one component of the dual vectors
struct CompAt {
    const double* p;
    int a;
    ASTG_HD double operator()(int s) const { return p[3 * s + a]; }
};
// the correction of the tilt at slot ts: its dual vector minus the MAC velocity at its vertex
ASTG_HD inline V3 tilt_corr(const Dev& d, int ts, const Fields& F) {
    if (F.corrT) return v3(F.corrT[3 * ts], F.corrT[3 * ts + 1], F.corrT[3 * ts + 2]);
    V3 dt = v3(F.dualT[3 * ts], F.dualT[3 * ts + 1], F.dualT[3 * ts + 2]);
    return dt - mac_sample(d, vert_pos(d, ts), F.mac);
}

// OctreeOmniFaceCenteredGrid3::sample, include/octree_omni_face_centered_grid3.h:37-80
ASTG_HD inline V3 vel_sample(const Dev& d, V3 p, const Fields& F) {
    int l = level_of(d, p.x, p.y, p.z);
    int r = d.lres[l];
    const double rx = over_h(d, p.x, l), ry = over_h(d, p.y, l), rz = over_h(d, p.z, l);
    int id0, id1, id2;
    double f0, f1, f2;
    bary_vec(rx - 0.5, r - 1, &id0, &f0);
    bary_vec(ry - 0.5, r - 1, &id1, &f1);
    bary_vec(rz - 0.5, r - 1, &id2, &f2);
    int ts = req(d, l, id0 + 1, id1 + 1, id2 + 1);
    if (near_transition(d, l, id0, id1, id2)) return omni_sample_sub<V3>(d, p, Vec3At{F.dualO}, Vec3At{F.dualT}, F.tf);
    V3 v = mac_sample_at(d, l, rx, ry, rz, F.mac);
    uint32_t tn = F.tf[ts];
    if (!(tn & TF_HALF) && (tn & TF_CLOSED)) return v;
    V3 diff = tilt_corr(d, ts, F);
    double mn = dmin(dmin(dmin(f0, f1), f2), dmin(dmin(1 - f0, 1 - f1), 1 - f2));
    return v + diff * 2 * mn;
}
// component a of vel_sample: every component is computed on its own (the same operations on the
// same values), so this is vel_sample(d, p, F)'s component a bit for bit at a third of the MAC work
ASTG_HD inline double vel_sample_axis(const Dev& d, V3 p, const Fields& F, int a) {
    int l = level_of(d, p.x, p.y, p.z);
    int r = d.lres[l];
    const double rx = over_h(d, p.x, l), ry = over_h(d, p.y, l), rz = over_h(d, p.z, l);
    int id0, id1, id2;
    double f0, f1, f2;
    bary_vec(rx - 0.5, r - 1, &id0, &f0);
    bary_vec(ry - 0.5, r - 1, &id1, &f1);
    bary_vec(rz - 0.5, r - 1, &id2, &f2);
    int ts = req(d, l, id0 + 1, id1 + 1, id2 + 1);
    if (near_transition(d, l, id0, id1, id2))
        return omni_sample_sub<double>(d, p, CompAt{F.dualO, a}, CompAt{F.dualT, a}, F.tf);
    double v = mac_axis(d, a, l, rx, ry, rz, F.mac + (size_t)a * d.S);
    uint32_t tn = F.tf[ts];
    if (!(tn & TF_HALF) && (tn & TF_CLOSED)) return v;
    double diff;
    if (F.corrT) {
        diff = F.corrT[3 * ts + a];
    } else {
        V3 q = vert_pos(d, ts);
        diff = F.dualT[3 * ts + a] - mac_sample_one(d, a, q, F.mac);
    }
    double mn = dmin(dmin(dmin(f0, f1), f2), dmin(dmin(1 - f0, 1 - f1), 1 - f2));
    return v + diff * 2 * mn;
}

// CellCenteredGrid<REAL,3>::sample (include/cell_centered_grid.h:40-54) on a res^3 grid of spacing
// 1 / res, index (z * res + y) * res + x
ASTG_HD inline double sdf_sample(const double* sdf, int sres, V3 p) {
    // p / (1 / sres) as the reference computes it; for a power-of-two sres, p * sres is the same number
    double sd = 1.0 / sres;
    const bool p2 = (sres & (sres - 1)) == 0;
    double rp[3] = {(p2 ? p.x * sres : p.x / sd) - 0.5, (p2 ? p.y * sres : p.y / sd) - 0.5,
                    (p2 ? p.z * sres : p.z / sd) - 0.5};
    int i[3], i1[3];
    double f[3];
    for (int k = 0; k < 3; ++k) {
        bary_vec(rp[k], sres - 1, &i[k], &f[k]);
        i1[k] = min(i[k] + 1, sres - 1);
    }
    auto g = [&](int x, int y, int z) { return sdf[((size_t)z * sres + y) * sres + x]; };
    return trilerp(g(i[0], i[1], i[2]), g(i1[0], i[1], i[2]), g(i[0], i1[1], i[2]), g(i1[0], i1[1], i[2]),
                   g(i[0], i[1], i1[2]), g(i1[0], i[1], i1[2]), g(i[0], i1[1], i1[2]), g(i1[0], i1[1], i1[2]), f[0],
                   f[1], f[2]);
}
// boundarySdf->sample(p): the collider grid, or the reference's constant 1 without a collider
ASTG_HD inline double bsdf(const Dev& d, V3 p) { return d.sdf ? sdf_sample(d.sdf, d.res, p) : 1.0; }

// BackTrace, include/advection.h:49-62: RK2 midpoint, then the boundary clamp: when the SDF changes
// sign between p and the traced point, the point moves back toward p by |phi1| / (|phi0| + |phi1|)
// (never without a collider: the SDF is 1 everywhere)
ASTG_HD inline V3 back_trace(const Dev& d, V3 p, double dt, const Fields& F) {
    // mid = p - v(p) dt / 2, ret = p - v(mid) dt; a loop, so the sampler's code is emitted once
    V3 q = p, ret = p;
#pragma unroll 1
    for (int i = 0; i < 2; ++i) {
        V3 v = vel_sample(d, q, F) * dt;
        if (i == 0) q = p - v * 0.5;
        else ret = p - v;
    }
    if (d.sdf) {
        double phi0 = bsdf(d, p), phi1 = bsdf(d, ret);
        if (phi0 * phi1 < 0.0) {
            double w = fabs(phi1) / (fabs(phi0) + fabs(phi1));
            return v3(w * p.x + (1.0 - w) * ret.x, w * p.y + (1.0 - w) * ret.y, w * p.z + (1.0 - w) * ret.z);
        }
    }
    return ret;
}

// tiltNeighborOctagon3, src/octree_util.cpp:172-194: the coordinates of the octagon behind
// tilted face i (possibly one level finer), or some = false
struct NbOct {
    bool some;
    int l, x, y, z;
};
ASTG_HD inline NbOct tilt_nb_oct(const Dev& d, int l, int x, int y, int z, int i) {
    NbOct o;
    o.some = false;
    o.l = o.x = o.y = o.z = 0;
    int nx = x + TILT_NB_OCT[i][0], ny = y + TILT_NB_OCT[i][1], nz = z + TILT_NB_OCT[i][2];
    if (!lay_valid(d, l, nx, ny, nz)) return o;
    int c = get_until(d, l, nx, ny, nz, true);
    if (c < 0) c = get_until(d, l, nx, ny, nz, false);
    if (c < 0) return o;
    int tl = slot_l(d, c), tx = slot_x(d, c), ty = slot_y(d, c), tz = slot_z(d, c);
    if (tl < l) {
        int m = i % 4;
        tz += i >= 4 ? 1 : 0;
        ty += m >= 2 ? 1 : 0;
        tx += (m == 1 || m == 2) ? 1 : 0;
    }
    o.some = true;
    o.l = tl; o.x = tx; o.y = ty; o.z = tz;
    return o;
}
}  // namespace astg
