// Reverse mode (adjoint) of the octree smoke step with the octree topology frozen (tilt
// adaptivity off, so the tilt-E state, the DOF map and the pressure matrix do not change).
//
// Every forward kernel of astg_step.cu / astg_pcg.cu has a transpose here that walks the same
// stencil and scatters the output cotangent into the input cotangents with atomics.  A kernel
// that overwrites a value consumes (zeroes) that value's cotangent; the launches of a stage run
// in the reverse order of the forward's.
//
// Interpolation is handled through "emission" forms of the samplers of astg_sample.cuh: for a
// sample position p they enumerate every field value the sample reads, with its weight w and the
// gradient of w with respect to p.  The forward value is sum(w * q), so one enumeration gives both
// the transposed interpolation (q_bar += w * y_bar) and the position cotangent
// (p_bar += y_bar * sum(grad_p w * q)), which carries the cotangent through the RK2 back-trace
// into the velocity that moved the sample point.  The weights follow the forward's branches
// (level location, clamping, the level-transition sub-sampler, the tilt correction), so the
// emitted sum equals the forward sample up to rounding.
#include "astg_launch.h"
#include "astg_sample.cuh"

namespace astg {

namespace {
constexpr int TB = 256;
inline int nblk(long long n) { return (int)((n + TB - 1) / TB); }
}  // namespace

// kinds of emitted field values
enum { K_OCT = 0, K_TIL = 1 };   // scalar samplers: octagon, tilt value
enum { K_DO = 3, K_DT = 4 };     // velocity sampler: 0..2 = MAC axis, dual at octagon / tilt

__device__ inline bool adj_ghost(const Dev& d, int s) { return slot_f(d, s) & SF_GHOST; }
__device__ inline bool adj_in_src(const Dev& d, V3 p) {
    double dx = p.x - d.srcX, dy = p.y - d.srcY, dz = p.z - d.srcZ;
    return dx * dx + dy * dy + dz * dz < d.srcR * d.srcR;
}

// ------------------------------------------------------------------ weights of the samplers
// 1-D linear weights (1 - f, f) and their derivatives with respect to the position
struct Ax {
    double w[2], g[2];
};
__device__ inline Ax ax(double f, double df) {
    Ax a;
    a.w[0] = 1 - f; a.w[1] = f;
    a.g[0] = -df; a.g[1] = df;
    return a;
}
// bary, returning d f / d x (1 where f = x - floor(x), 0 where the index is clamped)
__device__ inline double bary_d(double x, int lo, int hi, int* i, double* f) {
    bary(x, lo, hi, i, f);
    int c = (int)floor(x);
    int off = -lo;
    int L0 = lo + off, H0 = hi + off;
    return (L0 == H0 || c < L0 || c > H0 - 1) ? 0.0 : 1.0;
}
__device__ inline double bary_vec_d(double x, int high, int* i, double* f) {
    bary_vec(x, high, i, f);
    double t = x - *i;
    return (t < 0 || t > 1) ? 0.0 : 1.0;
}
// a value with its gradient
struct DG {
    double v;
    V3 g;
};
__device__ inline DG dg_min(DG a, DG b) { return (b.v < a.v) ? b : a; }  // dmin
// min(fx, fy, fz, 1 - fx, 1 - fy, 1 - fz) in the forward's evaluation order
__device__ inline DG corner_min(double fx, double dx, double fy, double dy, double fz, double dz) {
    DG X{fx, v3(dx, 0, 0)}, Y{fy, v3(0, dy, 0)}, Z{fz, v3(0, 0, dz)};
    DG X1{1 - fx, v3(-dx, 0, 0)}, Y1{1 - fy, v3(0, -dy, 0)}, Z1{1 - fz, v3(0, 0, -dz)};
    return dg_min(dg_min(dg_min(X, Y), Z), dg_min(dg_min(X1, Y1), Z1));
}
// the 8 corners of a trilerp (argument order f000 f100 f010 f110 f001 f101 f011 f111): weight
// c * w and gradient c * grad w + dc * w
template <class E>
__device__ inline void emit_tri(E& e, int kind, const int sl[8], const Ax& X, const Ax& Y, const Ax& Z, double c, V3 dc) {
    for (int q = 0; q < 8; ++q) {
        int i = q & 1, j = (q >> 1) & 1, k = (q >> 2) & 1;
        double w = X.w[i] * Y.w[j] * Z.w[k];
        V3 g = v3(X.g[i] * Y.w[j] * Z.w[k], X.w[i] * Y.g[j] * Z.w[k], X.w[i] * Y.w[j] * Z.g[k]);
        e(kind, sl[q], c * w, g * c + dc * w);
    }
}

// a corner value of the sub-sampler's cube: c * sum of n values of one kind
struct Src {
    int kind, n;
    int slot[8];
    double c;
};
__device__ inline Src src_one(int kind, int s) {
    Src r;
    r.kind = kind; r.n = 1; r.slot[0] = s; r.c = 1;
    return r;
}
// getNeighborCubeValue (include/octree_util.h:133-185) as value sources
__device__ void cube_src(const Dev& d, int l, int xi, int yi, int zi, int dir, Src* v, const uint32_t* tf, bool tj,
                         int kO, int kT) {
    int reDir = ((dir & 1) ? 8 : 6) - dir;
    int c = req(d, l, xi, yi, zi);
    v[reDir] = src_one(kO, c);
    for (int i = 0; i < 8; ++i) {
        int mk = SAMPLE_MARKER[dir][i];
        if (mk == 0x1000) continue;
        int m0 = (mk >> 8) & 0xf, m1 = (mk >> 4) & 0xf, m2 = mk & 0xf;
        int m[3] = {m0, m1, m2};
        if (tj && l > 0) {
            bool flag = false;
            for (int k = 0; k < 3; ++k) {
                if (m[k] != 0 && m[(k + 1) % 3] == 0 && m[(k + 2) % 3] == 0) {
                    int id[3] = {xi, yi, zi};
                    id[k] += (m[k] == 1);
                    id[0] *= 2; id[1] *= 2; id[2] *= 2;
                    id[(k + 1) % 3] += 1;
                    id[(k + 2) % 3] += 1;
                    int s = get(d, l - 1, id[0], id[1], id[2]);
                    if (s >= 0 && (tf[s] & TF_HALF)) { v[i] = src_one(kT, s); flag = true; }
                }
                if (m[k] == 0 && m[(k + 1) % 3] != 0 && m[(k + 2) % 3] != 0) {
                    int tx = (xi << 1) + (dir == 0 || dir == 3 || dir == 4 || dir == 7) + OCT_NB_TILT[i][0];
                    int ty = (yi << 1) + ((dir % 4) < 2) + OCT_NB_TILT[i][1];
                    int tz = (zi << 1) + (dir < 4) + OCT_NB_TILT[i][2];
                    int s = get(d, l - 1, tx, ty, tz);
                    if (s >= 0 && !(slot_f(d, s) & SF_GHOST) && (tf[s] & TF_CLOSED_BY_T)) { v[i] = src_one(kT, s); flag = true; }
                }
            }
            if (flag) continue;
        }
        Src t;
        t.kind = kO; t.n = 1; t.slot[0] = c;
        int r2 = d.lres[l] - 2;
        for (int x = -(m0 == 2); x <= (m0 == 1); ++x)
            for (int y = -(m1 == 2); y <= (m1 == 1); ++y)
                for (int z = -(m2 == 2); z <= (m2 == 1); ++z) {
                    if (x == 0 && y == 0 && z == 0) continue;
                    int cx = imin(imax(0, xi + x), r2), cy = imin(imax(0, yi + y), r2), cz = imin(imax(0, zi + z), r2);
                    if (t.n < 8) t.slot[t.n] = req(d, l, cx, cy, cz);
                    t.n += 1;
                }
        t.c = 1.0 / (double)t.n;
        if (t.n > 8) { report(d, DS_MISSING_NODE); t.n = 8; }
        v[i] = t;
    }
}
// OctreeOmniGrid3<T>::sampleSub (include/octree_omni_grid3.h:243-286)
template <class E>
__device__ void sub_w(const Dev& d, V3 p, const uint32_t* tf, E& e, int kO, int kT) {
    int l = level_of(d, p.x, p.y, p.z);
    double h = d.ldh[l];
    int r = d.lres[l];
    double rx = p.x / h, ry = p.y / h, rz = p.z / h;
    int xi, yi, zi;
    double fx, fy, fz;
    double dx = bary_d(rx, 0, r - 1, &xi, &fx) / h;
    double dy = bary_d(ry, 0, r - 1, &yi, &fy) / h;
    double dz = bary_d(rz, 0, r - 1, &zi, &fz) / h;
    int dir = fz >= 0.5 ? 0 : 4;
    dir += (fx >= 0.5) ? (fy >= 0.5 ? 0 : 3) : (fy >= 0.5 ? 1 : 2);
    int ts = req(d, l, xi + OCT_NB_TILT[dir][0], yi + OCT_NB_TILT[dir][1], zi + OCT_NB_TILT[dir][2]);
    uint32_t tn = tf[ts];
    if (!(tn & TF_HALF) && !(tn & TF_CLOSED_BY_T) && (tn & TF_CLOSED)) {
        int a, b, c;
        double ga, gb, gc;
        double da = bary_d(rx - 0.5, 0, r - 2, &a, &ga) / h;
        double db = bary_d(ry - 0.5, 0, r - 2, &b, &gb) / h;
        double dc = bary_d(rz - 0.5, 0, r - 2, &c, &gc) / h;
        int a1 = imin(a + 1, r - 2), b1 = imin(b + 1, r - 2), c1 = imin(c + 1, r - 2);
        int sl[8] = {req(d, l, a, b, c),  req(d, l, a1, b, c),  req(d, l, a, b1, c),  req(d, l, a1, b1, c),
                     req(d, l, a, b, c1), req(d, l, a1, b, c1), req(d, l, a, b1, c1), req(d, l, a1, b1, c1)};
        emit_tri(e, kO, sl, ax(ga, da), ax(gb, db), ax(gc, dc), 1.0, v3(0, 0, 0));
        return;
    }
    Src v[8];
    v[dir] = src_one(kT, ts);
    cube_src(d, l, xi, yi, zi, dir, v, tf, (tn & TF_TJOINT) != 0, kO, kT);
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
    Ax X = ax(fx, 2 * dx), Y = ax(fy, 2 * dy), Z = ax(fz, 2 * dz);
    const int corner[8] = {6, 7, 5, 4, 2, 3, 1, 0};  // trilerp(v6, v7, v5, v4, v2, v3, v1, v0)
    for (int q = 0; q < 8; ++q) {
        int i = q & 1, j = (q >> 1) & 1, k = (q >> 2) & 1;
        double w = X.w[i] * Y.w[j] * Z.w[k];
        V3 g = v3(X.g[i] * Y.w[j] * Z.w[k], X.w[i] * Y.g[j] * Z.w[k], X.w[i] * Y.w[j] * Z.g[k]);
        const Src& s = v[corner[q]];
        for (int m = 0; m < s.n; ++m) e(s.kind, s.slot[m], w * s.c, g * s.c);
    }
}
// OctreeOmniGrid3<double>::sample (include/octree_omni_grid3.h:147-187)
template <class E>
__device__ void scalar_w(const Dev& d, V3 p, const uint32_t* tf, E& e) {
    int l = level_of(d, p.x, p.y, p.z);
    double h = d.ldh[l];
    int r = d.lres[l];
    int xi, yi, zi;
    double fx, fy, fz;
    double dx = bary_d(p.x / h - 0.5, 0, r - 2, &xi, &fx) / h;
    double dy = bary_d(p.y / h - 0.5, 0, r - 2, &yi, &fy) / h;
    double dz = bary_d(p.z / h - 0.5, 0, r - 2, &zi, &fz) / h;
    int x1 = imin(xi + 1, r - 2), y1 = imin(yi + 1, r - 2), z1 = imin(zi + 1, r - 2);
    int ts = req(d, l, xi + 1, yi + 1, zi + 1);
    if (near_transition(d, l, xi, yi, zi)) {
        sub_w(d, p, tf, e, K_OCT, K_TIL);
        return;
    }
    int sl[8] = {req(d, l, xi, yi, zi), req(d, l, x1, yi, zi), req(d, l, xi, y1, zi), req(d, l, x1, y1, zi),
                 req(d, l, xi, yi, z1), req(d, l, x1, yi, z1), req(d, l, xi, y1, z1), req(d, l, x1, y1, z1)};
    emit_tri(e, K_OCT, sl, ax(fx, dx), ax(fy, dy), ax(fz, dz), 1.0, v3(0, 0, 0));
    uint32_t tn = tf[ts];
    if ((tn & TF_CLOSED) && !(tn & TF_HALF)) return;
    // + (til - mean of the 8 octagons) * 2 * mn
    DG mn = corner_min(fx, dx, fy, dy, fz, dz);
    e(K_TIL, ts, 2.0 * mn.v, mn.g * 2.0);
    for (int q = 0; q < 8; ++q) e(K_OCT, sl[q], -(1 / 8.0) * 2.0 * mn.v, mn.g * (-(1 / 8.0) * 2.0));
}
// OctreeFaceCenteredGrid3::sampleX/Y/Z (src/octree_face_centered_grid3.cpp:36-121) on level l;
// grad = false treats the position as fixed
template <class E>
__device__ void mac_axis_w(const Dev& d, int a, int l, V3 p, E& e, double c, V3 dc, bool grad) {
    int r = d.lres[l];
    double h = d.ldh[l];
    double q[3] = {p.x / h, p.y / h, p.z / h};
    int id[3], id1[3];
    double f[3], df[3];
    for (int k = 0; k < 3; ++k) {
        if (k == a) {
            df[k] = bary_d(q[k], 0, r - 1, &id[k], &f[k]) / h;
            id1[k] = imin(id[k] + 1, r - 1);
        } else {
            df[k] = bary_d(q[k] - 0.5, 0, r - 2, &id[k], &f[k]) / h;
            id1[k] = imin(id[k] + 1, r - 2);
        }
        if (!grad) df[k] = 0;
    }
    int sl[8] = {req(d, l, id[0], id[1], id[2]),  req(d, l, id1[0], id[1], id[2]),  req(d, l, id[0], id1[1], id[2]),
                 req(d, l, id1[0], id1[1], id[2]), req(d, l, id[0], id[1], id1[2]),  req(d, l, id1[0], id[1], id1[2]),
                 req(d, l, id[0], id1[1], id1[2]), req(d, l, id1[0], id1[1], id1[2])};
    emit_tri(e, a, sl, ax(f[0], df[0]), ax(f[1], df[1]), ax(f[2], df[2]), c, dc);
}
// OctreeOmniFaceCenteredGrid3::sample (include/octree_omni_face_centered_grid3.h:37-80)
template <class E>
__device__ void vel_w(const Dev& d, V3 p, const uint32_t* tf, E& e) {
    int l = level_of(d, p.x, p.y, p.z);
    double h = d.ldh[l];
    int r = d.lres[l];
    int id0, id1, id2;
    double f0, f1, f2;
    double d0 = bary_vec_d(p.x / h - 0.5, r - 1, &id0, &f0) / h;
    double d1 = bary_vec_d(p.y / h - 0.5, r - 1, &id1, &f1) / h;
    double d2 = bary_vec_d(p.z / h - 0.5, r - 1, &id2, &f2) / h;
    int ts = req(d, l, id0 + 1, id1 + 1, id2 + 1);
    if (near_transition(d, l, id0, id1, id2)) {
        sub_w(d, p, tf, e, K_DO, K_DT);
        return;
    }
    for (int a = 0; a < 3; ++a) mac_axis_w(d, a, l, p, e, 1.0, v3(0, 0, 0), true);
    uint32_t tn = tf[ts];
    if (!(tn & TF_HALF) && (tn & TF_CLOSED)) return;
    // + (dual at the tilt - MAC sampled at the tilt's vertex) * 2 * mn
    DG mn = corner_min(f0, d0, f1, d1, f2, d2);
    e(K_DT, ts, 2 * mn.v, mn.g * 2.0);
    V3 vp = vert_pos(d, ts);
    int lv = level_of(d, vp.x, vp.y, vp.z);
    for (int a = 0; a < 3; ++a) mac_axis_w(d, a, lv, vp, e, -2 * mn.v, mn.g * -2.0, false);
}
// cell-centred trilinear sample (include/octree_cell_centered_grid3.h:97-123), position fixed
template <class E>
__device__ void cell_w(const Dev& d, V3 p, E& e) {
    int l = level_of(d, p.x, p.y, p.z);
    double h = d.ldh[l];
    int r = d.lres[l];
    int xi, yi, zi;
    double fx, fy, fz;
    bary(p.x / h - 0.5, 0, r - 2, &xi, &fx);
    bary(p.y / h - 0.5, 0, r - 2, &yi, &fy);
    bary(p.z / h - 0.5, 0, r - 2, &zi, &fz);
    int x1 = imin(xi + 1, r - 2), y1 = imin(yi + 1, r - 2), z1 = imin(zi + 1, r - 2);
    int sl[8] = {req(d, l, xi, yi, zi), req(d, l, x1, yi, zi), req(d, l, xi, y1, zi), req(d, l, x1, y1, zi),
                 req(d, l, xi, yi, z1), req(d, l, x1, yi, z1), req(d, l, xi, y1, z1), req(d, l, x1, y1, z1)};
    emit_tri(e, 0, sl, ax(fx, 0), ax(fy, 0), ax(fz, 0), 1.0, v3(0, 0, 0));
}

// ------------------------------------------------------------------ emitters
// value and gradient of a scalar sample (probe)
struct ScalarValE {
    const double *o, *t;
    double v;
    V3 g;
    __device__ void operator()(int kind, int s, double w, V3 gw) {
        double q = kind == K_OCT ? o[s] : t[s];
        v += w * q;
        g = g + gw * q;
    }
};
// value and Jacobian of a velocity sample (probe and back-trace)
struct VelValE {
    Fields F;
    size_t S;
    double v[3];
    V3 J[3];  // J[c] = d v_c / d p
    __device__ void add(int c, double w, V3 gw, double q) {
        v[c] += w * q;
        J[c] = J[c] + gw * q;
    }
    __device__ void operator()(int kind, int s, double w, V3 gw) {
        if (kind < 3) add(kind, w, gw, F.mac[(size_t)kind * S + s]);
        else {
            const double* q = (kind == K_DO ? F.dualO : F.dualT) + 3 * (size_t)s;
            for (int c = 0; c < 3; ++c) add(c, w, gw, q[c]);
        }
    }
};
// transposed scalar sample: q_bar += w * y_bar for density and heat; position cotangent
struct ScalarAdjE {
    Fields C, G;
    double yd, yh;
    V3 pb;
    __device__ void operator()(int kind, int s, double w, V3 gw) {
        if (kind == K_OCT) {
            if (yd != 0) atomicAdd(G.dO + s, w * yd);
            if (yh != 0) atomicAdd(G.hO + s, w * yh);
            pb = pb + gw * (yd * C.dO[s] + yh * C.hO[s]);
        } else {
            if (yd != 0) atomicAdd(G.dT + s, w * yd);
            if (yh != 0) atomicAdd(G.hT + s, w * yh);
            pb = pb + gw * (yd * C.dT[s] + yh * C.hT[s]);
        }
    }
};
// transposed scalar sample at a fixed position, density and heat weighted separately (force)
struct ForceAdjE {
    Fields G;
    double cd, ch;
    __device__ void operator()(int kind, int s, double w, V3) {
        if (kind == K_OCT) {
            if (cd != 0) atomicAdd(G.dO + s, w * cd);
            if (ch != 0) atomicAdd(G.hO + s, w * ch);
        } else {
            if (cd != 0) atomicAdd(G.dT + s, w * cd);
            if (ch != 0) atomicAdd(G.hT + s, w * ch);
        }
    }
};
// transposed velocity sample: MAC / dual cotangents += w * v_bar; position cotangent
struct VelAdjE {
    Fields C, G;
    size_t S;
    V3 vb;
    V3 pb;
    __device__ void operator()(int kind, int s, double w, V3 gw) {
        if (kind < 3) {
            double y = comp(vb, kind);
            if (y == 0) return;
            size_t i = (size_t)kind * S + s;
            atomicAdd(G.mac + i, w * y);
            pb = pb + gw * (y * C.mac[i]);
        } else {
            const double* q = (kind == K_DO ? C.dualO : C.dualT) + 3 * (size_t)s;
            double* gq = (kind == K_DO ? G.dualO : G.dualT) + 3 * (size_t)s;
            if (vb.x != 0) atomicAdd(gq, w * vb.x);
            if (vb.y != 0) atomicAdd(gq + 1, w * vb.y);
            if (vb.z != 0) atomicAdd(gq + 2, w * vb.z);
            pb = pb + gw * (vb.x * q[0] + vb.y * q[1] + vb.z * q[2]);
        }
    }
};
// transposed field sample at a fixed position into one array of NC components (ghost passes)
template <int NC>
struct FieldAdjE {
    double* g;
    double y[NC];
    __device__ void operator()(int, int s, double w, V3) {
        for (int c = 0; c < NC; ++c)
            if (y[c] != 0) atomicAdd(g + (size_t)NC * s + c, w * y[c]);
    }
};
// transposed MAC sample of one axis at a fixed position (velocity ghosts)
struct MacAdjE {
    double* g;
    size_t S;
    double y;
    __device__ void operator()(int kind, int s, double w, V3) { atomicAdd(g + (size_t)kind * S + s, w * y); }
};

// ------------------------------------------------------------------ sampler probe
// what 0: per point {scalar_sample of density, emitted value, emitted gradient (3)}
// what 1: per point {vel_sample (3), emitted value (3), emitted Jacobian (9, row c = d v_c / d p)}
__global__ void k_adj_probe(Dev d, Fields F, int what, int n, const double* pos, double* out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    V3 p = v3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
    if (what == 0) {
        double y = scalar_sample(d, p, F.dO, F.dT, F.tf);
        ScalarValE e{F.dO, F.dT, 0.0, v3(0, 0, 0)};
        scalar_w(d, p, F.tf, e);
        double* o = out + 5 * (size_t)i;
        o[0] = y; o[1] = e.v; o[2] = e.g.x; o[3] = e.g.y; o[4] = e.g.z;
    } else {
        V3 y = vel_sample(d, p, F);
        VelValE e;
        e.F = F;
        e.S = d.S;
        for (int c = 0; c < 3; ++c) { e.v[c] = 0; e.J[c] = v3(0, 0, 0); }
        vel_w(d, p, F.tf, e);
        double* o = out + 15 * (size_t)i;
        o[0] = y.x; o[1] = y.y; o[2] = y.z;
        for (int c = 0; c < 3; ++c) {
            o[3 + c] = e.v[c];
            o[6 + 3 * c] = e.J[c].x; o[7 + 3 * c] = e.J[c].y; o[8 + 3 * c] = e.J[c].z;
        }
    }
}
cudaError_t launch_adj_probe(const Dev& d, const Fields& F, int what, int n, const double* pos, double* out, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    ASTG_LAUNCH(k_adj_probe<<<nblk(n), TB, 0, st>>>(d, F, what, n, pos, out));
    return cudaGetLastError();
}

// ------------------------------------------------------------------ stage 0: source
__global__ void k_adj_source_slots(Dev d, Fields G, double* gsO, double* gsT) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.S || adj_ghost(d, s)) return;
    if (adj_in_src(d, cell_pos(d, s))) {
        gsO[s] += G.dO[s];
        G.dO[s] = 0;
        G.hO[s] = 0;
    }
    if (adj_in_src(d, vert_pos(d, s))) {
        gsT[s] += G.dT[s];
        G.dT[s] = 0;
        G.hT[s] = 0;
        for (int k = 0; k < 8; ++k) G.tv[(size_t)s * 8 + k] = 0;
    }
    if (adj_in_src(d, mac_pos(d, 2, s))) G.mac[2 * (size_t)d.S + s] = 0;
}
__global__ void k_adj_source_half(Dev d, Fields G, double* gsT) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.H) return;
    int hs = d.half[i];
    if (!adj_in_src(d, vert_pos(d, hs))) return;
    gsT[hs] += G.dT[hs];
    G.dT[hs] = 0;
    G.hT[hs] = 0;
    for (int k = 0; k < 8; ++k) G.tv[(size_t)hs * 8 + k] = 0;
}

// ------------------------------------------------------------------ omni ghost update (NC components)
template <int NC>
__global__ void k_adj_cell_ghost_avg(Dev d, double* go, int l) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.lG[l]) return;
    int s = d.loff[l] + d.lN[l] + i;
    if (slot_f(d, s) & SF_FROM_COARSE) return;
    double y[NC];
    bool any = false;
    for (int c = 0; c < NC; ++c) { y[c] = go[(size_t)NC * s + c]; go[(size_t)NC * s + c] = 0; any |= y[c] != 0; }
    if (!any) return;
    int x = slot_x(d, s) << 1, yy = slot_y(d, s) << 1, z = slot_z(d, s) << 1;
    for (int a = 0; a <= 1; ++a)
        for (int b = 0; b <= 1; ++b)
            for (int cc = 0; cc <= 1; ++cc) {
                int t = req(d, l - 1, x + a, yy + b, z + cc);
                for (int c = 0; c < NC; ++c)
                    if (y[c] != 0) atomicAdd(go + (size_t)NC * t + c, y[c] * (1 / 8.0));
            }
}
template <int NC>
__global__ void k_adj_cell_ghost_sample(Dev d, double* go, int l) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.lG[l]) return;
    int s = d.loff[l] + d.lN[l] + i;
    if (!(slot_f(d, s) & SF_FROM_COARSE)) return;
    FieldAdjE<NC> e;
    e.g = go;
    bool any = false;
    for (int c = 0; c < NC; ++c) { e.y[c] = go[(size_t)NC * s + c]; go[(size_t)NC * s + c] = 0; any |= e.y[c] != 0; }
    if (any) cell_w(d, cell_pos(d, s), e);
}
template <int NC>
__global__ void k_adj_vertex_ghost(Dev d, double* gt) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.S || !adj_ghost(d, s) || d.halfMark[s]) return;
    double y[NC];
    bool any = false;
    for (int c = 0; c < NC; ++c) { y[c] = gt[(size_t)NC * s + c]; gt[(size_t)NC * s + c] = 0; any |= y[c] != 0; }
    if (!any) return;
    int l = slot_l(d, s), x = slot_x(d, s), yy = slot_y(d, s), z = slot_z(d, s);
    if (slot_f(d, s) & SF_FROM_COARSE) {
        int ts[8], count = 0;
        for (int a = 0; a <= (x & 1); ++a)
            for (int b = 0; b <= (yy & 1); ++b)
                for (int cc = 0; cc <= (z & 1); ++cc) {
                    int t = get_until(d, l + 1, (x >> 1) + a, (yy >> 1) + b, (z >> 1) + cc, true);
                    if (t >= 0) ts[count++] = t;
                }
        double w = 1.0 / (count + EPS);
        for (int q = 0; q < count; ++q)
            for (int c = 0; c < NC; ++c)
                if (y[c] != 0) atomicAdd(gt + (size_t)NC * ts[q] + c, y[c] * w);
    } else {
        int t = get_until(d, l - 1, x << 1, yy << 1, z << 1, true);
        if (t < 0) { report(d, DS_MISSING_NODE); t = 0; }
        for (int c = 0; c < NC; ++c)
            if (y[c] != 0) atomicAdd(gt + (size_t)NC * t + c, y[c]);
    }
}
template <int NC>
__global__ void k_adj_cell_ghost_joint(Dev d, double* go, double* gt, int l) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.lG[l]) return;
    int s = d.loff[l] + d.lN[l] + i;
    int x = slot_x(d, s), y = slot_y(d, s), z = slot_z(d, s);
    if (!oct_valid(d, l, x, y, z) || !(slot_f(d, s) & SF_FROM_COARSE)) return;
    int dp = req(d, l, x + (x & 1), y + (y & 1), z + (z & 1));
    int par = req(d, l + 1, x >> 1, y >> 1, z >> 1);
    for (int c = 0; c < NC; ++c) {
        double v = go[(size_t)NC * s + c];
        go[(size_t)NC * s + c] = 0;
        if (v == 0) continue;
        atomicAdd(gt + (size_t)NC * dp + c, v * 0.5);
        atomicAdd(go + (size_t)NC * par + c, v * 0.5);
    }
}
// getTiltFromOctagonNeighbor3 (include/octree_util.h:103-121) transposed
template <int NC>
__device__ void adj_tilt_from_oct(const Dev& d, int l, int x, int y, int z, double* go, const double* v) {
    int sl[8];
    int n = 0;
    sl[n++] = req(d, l, x, y, z);
    for (int m = -1; m <= 0; ++m)
        for (int q = -1; q <= 0; ++q)
            for (int k = -1; k <= 0; ++k) {
                if (m == 0 && q == 0 && k == 0) continue;
                if (oct_valid(d, l, x + m, y + q, z + k)) {
                    int t = get(d, l, x + m, y + q, z + k);
                    if (t >= 0) sl[n++] = t;
                }
            }
    double w = 1.0 / (double)n;
    for (int j = 0; j < n; ++j)
        for (int c = 0; c < NC; ++c)
            if (v[c] != 0) atomicAdd(go + (size_t)NC * sl[j] + c, v[c] * w);
}
// one writer per tilt the closed-joint pass writes (several T-joints may write the same tilt the
// same value; the lowest (joint, neighbour) index owns it) and per tilt of the closed-by-half list
__global__ void k_adj_owner_joint(Dev d, const double* te, int* own) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.nTJ) return;
    int tj = d.tj[i];
    int l = slot_l(d, tj), x = slot_x(d, tj), y = slot_y(d, tj), z = slot_z(d, tj);
    if (te[tj] < d.ldh[l]) { l -= 1; x <<= 1; y <<= 1; z <<= 1; }
    for (int k = 0; k < 6; ++k) {
        int t = get(d, l, x + OCT_NB[k][0], y + OCT_NB[k][1], z + OCT_NB[k][2]);
        if (t >= 0) atomicMin(own + t, i * 8 + k);
    }
}
__global__ void k_adj_owner_cbh(Dev d, int* own) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.nCBH) return;
    atomicMin(own + d.cbh[i], i);
}
template <int NC>
__global__ void k_adj_closed_joint(Dev d, double* go, double* gt, const double* te, const int* own) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.nTJ) return;
    int tj = d.tj[i];
    int l = slot_l(d, tj), x = slot_x(d, tj), y = slot_y(d, tj), z = slot_z(d, tj);
    if (te[tj] < d.ldh[l]) { l -= 1; x <<= 1; y <<= 1; z <<= 1; }
    for (int k = 0; k < 6; ++k) {
        int tx = x + OCT_NB[k][0], ty = y + OCT_NB[k][1], tz = z + OCT_NB[k][2];
        int t = get(d, l, tx, ty, tz);
        if (t < 0 || own[t] != i * 8 + k) continue;
        double v[NC];
        for (int c = 0; c < NC; ++c) { v[c] = gt[(size_t)NC * t + c]; gt[(size_t)NC * t + c] = 0; }
        adj_tilt_from_oct<NC>(d, l, tx, ty, tz, go, v);
    }
}
template <int NC>
__global__ void k_adj_closed_by_half(Dev d, double* go, double* gt, const uint32_t* tf, const int* own) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.nCBH) return;
    int s = d.cbh[i];
    if (own[s] != i) return;
    if (!((tf[s] & TF_CLOSED) && tf_dir(tf[s]) == -1)) return;
    double v[NC];
    for (int c = 0; c < NC; ++c) { v[c] = gt[(size_t)NC * s + c]; gt[(size_t)NC * s + c] = 0; }
    adj_tilt_from_oct<NC>(d, slot_l(d, s), slot_x(d, s), slot_y(d, s), slot_z(d, s), go, v);
}
// transpose of OctreeOmniGrid3<T>::updateGhost (include/octree_omni_grid3.h:136-143)
template <int NC>
static void adj_omni_ghost(const Dev& d, double* go, double* gt, const double* te, const uint32_t* tf, const int* ownJ,
                           const int* ownH, cudaStream_t st) {
    if (d.nCBH) ASTG_LAUNCH(k_adj_closed_by_half<NC><<<nblk(d.nCBH), TB, 0, st>>>(d, go, gt, tf, ownH));
    if (d.nTJ) ASTG_LAUNCH(k_adj_closed_joint<NC><<<nblk(d.nTJ), TB, 0, st>>>(d, go, gt, te, ownJ));
    for (int l = d.L - 1; l >= 0; --l)
        if (d.lG[l]) ASTG_LAUNCH(k_adj_cell_ghost_joint<NC><<<nblk(d.lG[l]), TB, 0, st>>>(d, go, gt, l));
    ASTG_LAUNCH(k_adj_vertex_ghost<NC><<<nblk(d.S), TB, 0, st>>>(d, gt));
    for (int l = d.L - 1; l >= 0; --l)
        if (d.lG[l]) ASTG_LAUNCH(k_adj_cell_ghost_sample<NC><<<nblk(d.lG[l]), TB, 0, st>>>(d, go, l));
    for (int l = d.L - 1; l >= 0; --l)
        if (d.lG[l]) ASTG_LAUNCH(k_adj_cell_ghost_avg<NC><<<nblk(d.lG[l]), TB, 0, st>>>(d, go, l));
}

// ------------------------------------------------------------------ stage 1: buoyancy
// warp sum, then one atomic per warp
__device__ inline void warp_atomic_add(double* p, double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0 && v != 0) atomicAdd(p, v);
}
__global__ void k_adj_force_mac(Dev d, Fields F, Fields G, double dt, double* gamb) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    double ga = 0;
    if (s < d.S && !adj_ghost(d, s) && mac_valid(d, 2, slot_l(d, s), slot_x(d, s), slot_y(d, s), slot_z(d, s))) {
        double k = dt * G.mac[2 * (size_t)d.S + s];
        if (k != 0) {
            ForceAdjE e{G, k * d.buoyD, k * d.buoyT};
            scalar_w(d, mac_pos(d, 2, s), F.tf, e);
            ga = -k * d.buoyT;
        }
    }
    warp_atomic_add(gamb, ga);
}
__global__ void k_adj_force_tilt(Dev d, Fields F, Fields G, const uint8_t* open, double dt, double* gamb) {
    long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double ga = 0;
    if (idx < 8LL * d.S) {
        int s = (int)(idx >> 3), k = (int)(idx & 7);
        if (!adj_ghost(d, s) && open[s]) {
            double c = dt * G.tv[(size_t)s * 8 + k] * tilt_up(k, 2);
            if (c != 0) {
                ForceAdjE e{G, c * d.buoyD, c * d.buoyT};
                scalar_w(d, tilt_pos(vert_pos(d, s), k, F.te[s]), F.tf, e);
                ga = -c * d.buoyT;
            }
        }
    }
    warp_atomic_add(gamb, ga);
}
__global__ void k_adj_force_half(Dev d, Fields F, Fields G, double dt, double* gamb) {
    long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double ga = 0;
    if (idx < 8LL * d.H) {
        int i = (int)(idx >> 3), k = (int)(idx & 7);
        int hs = d.half[i];
        int dir = tf_dir(F.tf[hs]);
        int q = -1;
        for (int j = 0; j < 5; ++j)
            if (HALF_SLOT[dir][j] == k) q = j;
        if (q >= 0) {
            V3 c0 = vert_pos(d, hs);
            V3 p = (q == 4) ? c0 : tilt_pos(c0, k, F.te[hs]);
            V3 dv = (q == 4) ? v3(HALF_DIR_POS[k][0], HALF_DIR_POS[k][1], HALF_DIR_POS[k][2]) : tilt_up3(k);
            double c = dt * G.tv[(size_t)hs * 8 + k] * dv.z;
            if (c != 0) {
                ForceAdjE e{G, c * d.buoyD, c * d.buoyT};
                scalar_w(d, p, F.tf, e);
                ga = -c * d.buoyT;
            }
        }
    }
    warp_atomic_add(gamb, ga);
}
// ambT = sum over levels of w_l * sum(heat) / sum(w_l * slots), w_0 = 1, w_l = 8
__global__ void k_adj_amb(Dev d, Fields G, const double* gamb, double invCount) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.S) return;
    double g = *gamb;
    if (g == 0) return;
    G.hO[s] += g * (slot_l(d, s) == 0 ? 1.0 : 8.0) * invCount;
}

// ------------------------------------------------------------------ walls and velocity ghosts
__global__ void k_adj_walls(Dev d, double* mac) {
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
__global__ void k_adj_mac_ghost_zero(Dev d, double* mac) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.S || !adj_ghost(d, s)) return;
    mac[s] = 0;
    mac[(size_t)d.S + s] = 0;
    mac[2 * (size_t)d.S + s] = 0;
}
__global__ void k_adj_mac_ghost_sample(Dev d, double* mac, int l, int fromCoarse) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.lG[l]) return;
    int s = d.loff[l] + d.lN[l] + i;
    if (((slot_f(d, s) & SF_FROM_COARSE) != 0) != (fromCoarse != 0)) return;
    for (int a = 0; a < 3; ++a) {
        double y = mac[(size_t)a * d.S + s];
        mac[(size_t)a * d.S + s] = 0;
        if (y == 0) continue;
        V3 p = mac_pos(d, a, s);
        int lp = level_of(d, p.x, p.y, p.z);
        MacAdjE e{mac, (size_t)d.S, y};
        mac_axis_w(d, a, lp, p, e, 1.0, v3(0, 0, 0), false);
    }
}
__global__ void k_adj_mac_from_half(Dev d, Fields F, Fields G, const uint8_t* lastWriter) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.H || !lastWriter[i]) return;
    int hs = d.half[i];
    int dir = tf_dir(F.tf[hs]);
    int a = dir % 3;
    int t = req(d, slot_l(d, hs) + 1, slot_x(d, hs) >> 1, slot_y(d, hs) >> 1, slot_z(d, hs) >> 1);
    double y = G.mac[(size_t)a * d.S + t];
    G.mac[(size_t)a * d.S + t] = 0;
    if (y != 0) atomicAdd(G.tv + (size_t)hs * 8 + HALF_SLOT[dir][4], y);
}
__global__ void k_adj_tilt_ghost(Dev d, Fields F, Fields G, int l) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.lG[l]) return;
    int s = d.loff[l] + d.lN[l] + i;
    if (F.tf[s] & TF_HALF) return;
    int x = slot_x(d, s), y = slot_y(d, s), z = slot_z(d, s);
    int src;
    if (slot_f(d, s) & SF_FROM_COARSE) {
        if ((x & 1) || (y & 1) || (z & 1)) {
            for (int k = 0; k < 8; ++k) G.tv[(size_t)s * 8 + k] = 0;
            return;
        }
        src = req(d, l + 1, x >> 1, y >> 1, z >> 1);
    } else {
        src = req(d, l - 1, x << 1, y << 1, z << 1);
    }
    for (int k = 0; k < 8; ++k) {
        double v = G.tv[(size_t)s * 8 + k];
        G.tv[(size_t)s * 8 + k] = 0;
        if (v != 0) atomicAdd(G.tv + (size_t)src * 8 + k, v);
    }
}
// transpose of launch_walls_and_ghost (walls, then OctreeOmniFaceCenteredGrid3::updateGhost)
void launch_adj_walls_and_ghost(const Dev& d, const Fields& F, const Fields& G, const uint8_t* lastWriter, cudaStream_t st) {
    for (int l = d.L - 1; l >= 0; --l)
        if (d.lG[l]) ASTG_LAUNCH(k_adj_tilt_ghost<<<nblk(d.lG[l]), TB, 0, st>>>(d, F, G, l));
    for (int l = d.L - 1; l >= 0; --l)
        if (d.lG[l]) ASTG_LAUNCH(k_adj_mac_ghost_sample<<<nblk(d.lG[l]), TB, 0, st>>>(d, G.mac, l, 1));
    if (d.H) ASTG_LAUNCH(k_adj_mac_from_half<<<nblk(d.H), TB, 0, st>>>(d, F, G, lastWriter));
    for (int l = d.L - 1; l >= 0; --l)
        if (d.lG[l]) ASTG_LAUNCH(k_adj_mac_ghost_sample<<<nblk(d.lG[l]), TB, 0, st>>>(d, G.mac, l, 0));
    ASTG_LAUNCH(k_adj_mac_ghost_zero<<<nblk(d.S), TB, 0, st>>>(d, G.mac));
    ASTG_LAUNCH(k_adj_walls<<<nblk(d.S), TB, 0, st>>>(d, G.mac));
}

// ------------------------------------------------------------------ stage 3: projection
__device__ inline int adj_p_oct(const Dev& d, const int* pO, int l, int x, int y, int z) { return pO[req(d, l, x, y, z)]; }

// transpose of the pressure-gradient update (src/octree_omnigrid_solver3.cpp:682-847): velocity
// cotangents of faces the update zeroes are consumed, the others pass through, and
// gp += (d u_new / d p) * u_bar
__global__ void k_adj_pu_mac(Dev d, Fields G, const int* pO, double* gp, double dt) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.S || adj_ghost(d, s)) return;
    int l = slot_l(d, s), x = slot_x(d, s), y = slot_y(d, s), z = slot_z(d, s);
    double h = d.ldh[l];
    double k0 = dt / d.rho;
    int i0 = (oct_valid(d, l, x, y, z) && pO[s] >= 0) ? pO[s] : -1;
    for (int a = 0; a < 3; ++a) {
        if (!mac_valid(d, a, l, x, y, z)) continue;
        double* u = G.mac + (size_t)a * d.S + s;
        if (d.wMac[(size_t)a * d.S + s] <= 0) { *u = 0; continue; }
        double yb = *u;
        if (yb == 0) continue;
        int id0 = x - (a == 0), id1 = y - (a == 1), id2 = z - (a == 2);
        int i1 = -1;
        if (oct_valid(d, l, id0, id1, id2)) {
            int ti = adj_p_oct(d, pO, l, id0, id1, id2);
            if (ti >= 0) i1 = ti;
        }
        double c = k0 / h;  // u -= k0 * (p0 - p1) / h
        if (i0 >= 0) atomicAdd(gp + i0, -c * yb);
        if (i1 >= 0) atomicAdd(gp + i1, c * yb);
    }
}
__global__ void k_adj_pu_tilt(Dev d, Fields F, Fields G, const uint8_t* open, const int* pO, const int* pT, double* gp, double dt) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.S || adj_ghost(d, s) || !open[s]) return;
    int ci = pT[s];
    double k0 = dt / d.rho;
    const double* tw = d.wTilt + (size_t)s * 8;
    int l = slot_l(d, s), x = slot_x(d, s), y = slot_y(d, s), z = slot_z(d, s);
    for (int k = 0; k < 8; ++k) {
        double* u = G.tv + (size_t)s * 8 + k;
        NbOct nb = tilt_nb_oct(d, l, x, y, z, k);
        if (tw[k] > 0 && nb.some) {
            double yb = *u;
            if (yb == 0) continue;
            double h2 = d.ldh[nb.l];
            int i1 = -1;
            if (oct_valid(d, nb.l, nb.x, nb.y, nb.z)) {
                int ti = adj_p_oct(d, pO, nb.l, nb.x, nb.y, nb.z);
                if (ti >= 0) i1 = ti;
            }
            double c = k0 * (k < 4 ? 1 : -1) / (h2 * SQRT3 * 0.5);  // u -= c * (p1 - p0)
            if (i1 >= 0) atomicAdd(gp + i1, -c * yb);
            if (ci >= 0) atomicAdd(gp + ci, c * yb);
        } else {
            *u = 0;
        }
    }
}
__global__ void k_adj_pu_half(Dev d, Fields F, Fields G, const int* pO, const int* pT, double* gp, double dt) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.H) return;
    int hs = d.half[i];
    int dir = tf_dir(F.tf[hs]);
    int ci = pT[hs];
    int l = slot_l(d, hs), x = slot_x(d, hs), y = slot_y(d, hs), z = slot_z(d, hs);
    double k0 = dt / d.rho;
    double* g = G.tv + (size_t)hs * 8;
    const double* tw = d.wTilt + (size_t)hs * 8;
    int id[3] = {x >> 1, y >> 1, z >> 1};
    id[dir % 3] -= dir < 3 ? 1 : 0;
    int fsl = HALF_SLOT[dir][4];
    if (tw[fsl] > 0) {
        int ti = adj_p_oct(d, pO, l + 1, id[0], id[1], id[2]);
        double yb = g[fsl];
        double c = k0 * (dir < 3 ? 1 : -1) / d.ldh[l];  // u -= c * (p0 - p1)
        if (yb != 0) {
            if (ci >= 0) atomicAdd(gp + ci, -c * yb);
            if (ti >= 0) atomicAdd(gp + ti, c * yb);
        }
    } else {
        g[fsl] = 0;
    }
    for (int k = 0; k < 8; ++k) {
        if (tw[k] > 0 && half_listed(dir, k)) {
            double yb = g[k];
            if (yb == 0) continue;
            int nx = x + TILT_NB_OCT[k][0], ny = y + TILT_NB_OCT[k][1], nz = z + TILT_NB_OCT[k][2];
            int i1 = -1;
            if (oct_valid(d, l, nx, ny, nz)) {
                int ti = adj_p_oct(d, pO, l, nx, ny, nz);
                if (ti >= 0) i1 = ti;
            }
            double c = k0 * (k < 4 ? 1 : -1) / (d.ldh[l] * SQRT3 * 0.5);  // u -= c * (p1 - p0)
            if (i1 >= 0) atomicAdd(gp + i1, -c * yb);
            if (ci >= 0) atomicAdd(gp + ci, c * yb);
        } else if (k != fsl) {
            g[k] = 0;
        }
    }
}
void launch_adj_pressure_update(const Dev& d, const Fields& F, const Fields& G, const uint8_t* open, const int* pO,
                                const int* pT, double* gp, double dt, cudaStream_t st) {
    if (d.H) ASTG_LAUNCH(k_adj_pu_half<<<nblk(d.H), TB, 0, st>>>(d, F, G, pO, pT, gp, dt));
    ASTG_LAUNCH(k_adj_pu_tilt<<<nblk(d.S), TB, 0, st>>>(d, F, G, open, pO, pT, gp, dt));
    ASTG_LAUNCH(k_adj_pu_mac<<<nblk(d.S), TB, 0, st>>>(d, G, pO, gp, dt));
}

// transpose of the right-hand side of the assembly (k_asm_oct / k_asm_tilt / k_asm_half, then
// b = bRaw * rho / dt): u_bar += scale * coefficient * lambda[row]
__global__ void k_adj_b_oct(Dev d, Fields F, Fields G, Proj P, const int* hoPtr, const int* hoIdx, const double* lam, double scale) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.S || (slot_f(d, s) & SF_GHOST)) return;
    int ci = P.pO[s];
    int l = slot_l(d, s), x = slot_x(d, s), y = slot_y(d, s), z = slot_z(d, s);
    if (ci < 0 || !oct_valid(d, l, x, y, z)) return;
    double yb = lam[ci] * scale;
    if (yb == 0) return;
    double h = d.ldh[l];
    // two passes over the faces: the forward drops them (tb = 0) when the diagonal vanishes
    double center = 0;
    for (int pass = 0; pass < 2; ++pass) {
        if (pass == 1 && fabs(center) < EPS) break;
        for (int i = 0; i < 6; ++i) {
            int axis = i / 2;
            int nx = x + OCT_NB[i][0], ny = y + OCT_NB[i][1], nz = z + OCT_NB[i][2];
            if (oct_valid(d, l, nx, ny, nz) && is_ghost_node(d, l, nx, ny, nz)) continue;
            double area = h * h;
            for (int m = 0; m <= 1; ++m)
                for (int n = 0; n <= 1; ++n) {
                    int t[3] = {x, y, z};
                    t[axis] += (i & 1) ? 0 : 1;
                    t[(axis + 1) % 3] += m;
                    t[(axis + 2) % 3] += n;
                    double e = F.te[req(d, l, t[0], t[1], t[2])];
                    area -= e * e * 0.5;
                }
            int fs = req(d, l, x + OCT_NB_FACE[i][0], y + OCT_NB_FACE[i][1], z + OCT_NB_FACE[i][2]);
            double tC, tK;
            if (oct_valid(d, l, nx, ny, nz)) {
                double term = d.wMac[(size_t)axis * d.S + fs];
                int ti = P.pO[req(d, l, nx, ny, nz)];
                if (ti >= 0) { tC = term * area / h; tK = area * term; }
                else { tC = 0; tK = 0; }
            } else if ((d.closedMask >> i) & 1) {
                tC = 0; tK = 0;
            } else {
                tK = area;
                tC = tK / h;
            }
            if (pass == 0) center += tC;
            else if (tK != 0) atomicAdd(G.mac + (size_t)axis * d.S + fs, ((i & 1) ? 1 : -1) * tK * yb);
        }
        for (int i = 0; i < 8; ++i) {
            int ns = req(d, l, x + OCT_NB_TILT[i][0], y + OCT_NB_TILT[i][1], z + OCT_NB_TILT[i][2]);
            uint32_t f = F.tf[ns];
            int re = ((i & 1) ? 8 : 6) - i;
            if (!(f & TF_CLOSED) || (f & TF_HALF)) {
                double e = F.te[ns];
                double area = e * e * SQRT3 * 0.5;
                double term = d.wTilt[(size_t)ns * 8 + re];
                int ti = P.pT[ns];
                double tC = 0, tK = 0;
                if (ti >= 0) { tC = term * area / (h * SQRT3 * 0.5); tK = area * term; }
                if (pass == 0) center += tC;
                else if (tK != 0) atomicAdd(G.tv + (size_t)ns * 8 + re, (i < 4 ? -1 : 1) * tK * yb);
            }
        }
    }
    // half tilts facing this octagon are added after the diagonal test
    for (int q = hoPtr[s]; q < hoPtr[s + 1]; ++q) {
        int hs = d.half[hoIdx[q]];
        if (P.pT[hs] < 0) continue;
        int dir = tf_dir(F.tf[hs]);
        int oi = HALF_SLOT[dir][4];
        double e = F.te[hs];
        double area = e * e * 2;
        double tw = d.wTilt[(size_t)hs * 8 + oi];
        atomicAdd(G.tv + (size_t)hs * 8 + oi, (dir < 3 ? -1 : 1) * tw * area * yb);
    }
}
__global__ void k_adj_b_tilt(Dev d, Fields F, Fields G, Proj P, const uint8_t* open, const double* lam, double scale) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.S || (slot_f(d, s) & SF_GHOST)) return;
    int ci = P.pT[s];
    if (!open[s] || ci < 0) return;
    double yb = lam[ci] * scale;
    if (yb == 0) return;
    int l = slot_l(d, s), x = slot_x(d, s), y = slot_y(d, s), z = slot_z(d, s);
    double e = F.te[s];
    const double* tw = d.wTilt + (size_t)s * 8;
    double area = e * e * SQRT3 * 0.5;
    for (int i = 0; i < 8; ++i) {
        NbOct nb = tilt_nb_oct(d, l, x, y, z, i);
        double tK = 0;
        if (!nb.some) {
            if (!oct_valid(d, l, x + TILT_NB_OCT[i][0], y + TILT_NB_OCT[i][1], z + TILT_NB_OCT[i][2])) tK = area;
        } else if (oct_valid(d, nb.l, nb.x, nb.y, nb.z)) {
            int ti = P.pO[req(d, nb.l, nb.x, nb.y, nb.z)];
            tK = ti >= 0 ? area * tw[i] : 0;
        } else {
            tK = area;
        }
        if (tK != 0) atomicAdd(G.tv + (size_t)s * 8 + i, (i < 4 ? -1 : 1) * tK * yb);
    }
}
__global__ void k_adj_b_half(Dev d, Fields F, Fields G, Proj P, const double* lam, double scale) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.H) return;
    int hs = d.half[i];
    int ci = P.pT[hs];
    if (ci < 0) return;
    double yb = lam[ci] * scale;
    if (yb == 0) return;
    int l = slot_l(d, hs), x = slot_x(d, hs), y = slot_y(d, hs), z = slot_z(d, hs);
    int dir = tf_dir(F.tf[hs]);
    double e = F.te[hs];
    double area = e * e * 2;
    double* g = G.tv + (size_t)hs * 8;
    const double* tw = d.wTilt + (size_t)hs * 8;
    int id[3] = {x >> 1, y >> 1, z >> 1};
    id[dir % 3] -= dir < 3 ? 1 : 0;
    int oi = HALF_SLOT[dir][4];
    if (l + 1 < d.L && oct_valid(d, l + 1, id[0], id[1], id[2])) {
        int ti = P.pO[req(d, l + 1, id[0], id[1], id[2])];
        if (ti >= 0) atomicAdd(g + oi, (dir < 3 ? 1 : -1) * tw[oi] * area * yb);
    } else {
        atomicAdd(g + oi, (dir < 3 ? 1 : -1) * area * yb);
    }
    area = e * e * SQRT3 * 0.5;
    for (int k = 0; k < 8; ++k) {
        if (!half_listed(dir, k)) continue;
        int nx = x + TILT_NB_OCT[k][0], ny = y + TILT_NB_OCT[k][1], nz = z + TILT_NB_OCT[k][2];
        double tK = 0;
        if (oct_valid(d, l, nx, ny, nz)) {
            int ti = P.pO[req(d, l, nx, ny, nz)];
            tK = ti >= 0 ? area * tw[k] : 0;
        }
        if (tK != 0) atomicAdd(g + k, (k < 4 ? -1 : 1) * tK * yb);
    }
}
void launch_adj_rhs(const Dev& d, const Fields& F, const Fields& G, const uint8_t* open, const Proj& P, const int* hoPtr,
                    const int* hoIdx, const double* lam, double scale, cudaStream_t st) {
    ASTG_LAUNCH(k_adj_b_oct<<<nblk(d.S), TB, 0, st>>>(d, F, G, P, hoPtr, hoIdx, lam, scale));
    ASTG_LAUNCH(k_adj_b_tilt<<<nblk(d.S), TB, 0, st>>>(d, F, G, P, open, lam, scale));
    if (d.H) ASTG_LAUNCH(k_adj_b_half<<<nblk(d.H), TB, 0, st>>>(d, F, G, P, lam, scale));
}

// ------------------------------------------------------------------ stage 4: dual velocity
__global__ void k_adj_dual_tilt(Dev d, Fields F, Fields G) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.S || adj_ghost(d, s)) return;
    double* go = G.dualT + 3 * (size_t)s;
    double ob[3] = {go[0], go[1], go[2]};
    go[0] = go[1] = go[2] = 0;
    if (F.tf[s] & TF_CLOSED) return;
    if (ob[0] == 0 && ob[1] == 0 && ob[2] == 0) return;
    const double s3 = INV_SQRT3 * (3.0 / 4.0);
    const double M[3][4] = {{s3, -s3, -s3, s3}, {s3, s3, -s3, -s3}, {s3, s3, s3, s3}};
    double vb[4];
    for (int j = 0; j < 4; ++j) vb[j] = M[0][j] * ob[0] + M[1][j] * ob[1] + M[2][j] * ob[2];
    double* g = G.tv + (size_t)s * 8;
    const int pair[4][2] = {{0, 6}, {1, 7}, {2, 4}, {3, 5}};  // v4[j] = (g[a] + g[b]) * 0.5
    for (int j = 0; j < 4; ++j) {
        atomicAdd(g + pair[j][0], vb[j] * 0.5);
        atomicAdd(g + pair[j][1], vb[j] * 0.5);
    }
}
__global__ void k_adj_dual_oct(Dev d, Fields F, Fields G) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.S || adj_ghost(d, s)) return;
    double* go = G.dualO + 3 * (size_t)s;
    double ob[3] = {go[0], go[1], go[2]};
    go[0] = go[1] = go[2] = 0;
    int l = slot_l(d, s), x = slot_x(d, s), y = slot_y(d, s), z = slot_z(d, s);
    if (!oct_valid(d, l, x, y, z)) return;
    if (ob[0] == 0 && ob[1] == 0 && ob[2] == 0) return;
    double h = d.ldh[l];
    double sq = SQRT3 * h, hsq = sq * 0.5;
    int nj[8], ts[8];
    for (int i = 0; i < 8; ++i) {
        ts[i] = req(d, l, x + OCT_NB_TILT[i][0], y + OCT_NB_TILT[i][1], z + OCT_NB_TILT[i][2]);
        uint32_t f = F.tf[ts[i]];
        nj[i] = ((f & TF_TJOINT) && fabs(F.te[ts[i]] - h) < EPS) || (f & TF_HALF);
    }
    // v[j] = sum of at most two cotangent targets with coefficients
    double* ref[7][2];
    double cf[7][2];
    int nr[7] = {0, 0, 0, 0, 0, 0, 0};
    int cnt[7] = {0, 0, 0, 0, 0, 0, 0};
    size_t S = d.S;
    auto put = [&](int j, double* p, double c) { ref[j][nr[j]] = p; cf[j][nr[j]] = c; ++nr[j]; };
    if (!((nj[1] && nj[6]) || (nj[2] && nj[5]))) { put(0, G.mac + s, 1); cnt[0]++; }
    if (!((nj[0] && nj[7]) || (nj[3] && nj[4]))) { put(0, G.mac + req(d, l, x + 1, y, z), 1); cnt[0]++; }
    if (!((nj[2] && nj[7]) || (nj[3] && nj[6]))) { put(1, G.mac + S + s, 1); cnt[1]++; }
    if (!((nj[0] && nj[5]) || (nj[1] && nj[4]))) { put(1, G.mac + S + req(d, l, x, y + 1, z), 1); cnt[1]++; }
    if (!((nj[4] && nj[6]) || (nj[5] && nj[7]))) { put(2, G.mac + 2 * S + s, 1); cnt[2]++; }
    if (!((nj[0] && nj[2]) || (nj[1] && nj[3]))) { put(2, G.mac + 2 * S + req(d, l, x, y, z + 1), 1); cnt[2]++; }
    for (int i = 0; i < 4; ++i) {
        int slot = i, re = ((i & 1) ? 8 : 6) - i, vs = i + 3;
        uint32_t fn = F.tf[ts[slot]], fr = F.tf[ts[re]];
        double en = F.te[ts[slot]], er = F.te[ts[re]];
        if (!(fn & TF_CLOSED) || (fn & TF_HALF)) { put(vs, G.tv + (size_t)ts[slot] * 8 + re, 1); cnt[vs]++; }
        if (!(fr & TF_CLOSED) || (fr & TF_HALF)) {
            double* tp = G.tv + (size_t)ts[re] * 8 + slot;
            if (cnt[vs] == 0) {
                put(vs, tp, 1);
            } else {
                double den = sq - en * 1.0 / SQRT3 - er * 1.0 / SQRT3;
                double a = (hsq - er * 1.0 / SQRT3) / den, b = (hsq - en * 1.0 / SQRT3) / den;
                for (int m = 0; m < nr[vs]; ++m) cf[vs][m] *= a;
                put(vs, tp, b);
            }
            cnt[vs]++;
        }
    }
    for (int i = 0; i < 3; ++i)
        for (int m = 0; m < nr[i]; ++m) cf[i][m] /= (cnt[i] + EPS);
    int bits = ((cnt[0] > 0) << 6) | ((cnt[1] > 0) << 5) | ((cnt[2] > 0) << 4) | ((cnt[3] > 1 || nj[0] || nj[6]) << 3) |
               ((cnt[4] > 1 || nj[1] || nj[7]) << 2) | ((cnt[5] > 1 || nj[2] || nj[4]) << 1) | (cnt[6] > 1 || nj[3] || nj[5]);
    const double* M = d.M37 + (size_t)bits * 21;
    for (int j = 0; j < 7; ++j) {
        double vb = M[j] * ob[0] + M[7 + j] * ob[1] + M[14 + j] * ob[2];
        if (vb == 0) continue;
        for (int m = 0; m < nr[j]; ++m) atomicAdd(ref[j][m], cf[j][m] * vb);
    }
}
__global__ void k_adj_dual_half(Dev d, Fields F, Fields G) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.H) return;
    int hs = d.half[i];
    double* go = G.dualT + 3 * (size_t)hs;
    double ob[3] = {go[0], go[1], go[2]};
    go[0] = go[1] = go[2] = 0;
    if (ob[0] == 0 && ob[1] == 0 && ob[2] == 0) return;
    int dir = tf_dir(F.tf[hs]);
    int axis = dir % 3;
    int srcSlot[7] = {-1, -1, -1, -1, -1, -1, -1};
    srcSlot[axis] = HALF_SLOT[dir][4];
    for (int q = 0; q < 4; ++q) {
        int slot = HALF_SLOT[dir][q];
        int re = ((slot & 1) ? 8 : 6) - slot;
        int idx = slot < re ? slot : re;
        srcSlot[idx + 3] = slot;
    }
    int bits = ((axis == 0) << 6) | ((axis == 1) << 5) | ((axis == 2) << 4) | 0xf;
    const double* M = d.M37 + (size_t)bits * 21;
    for (int j = 0; j < 7; ++j) {
        if (srcSlot[j] < 0) continue;
        double vb = M[j] * ob[0] + M[7 + j] * ob[1] + M[14 + j] * ob[2];
        if (vb != 0) atomicAdd(G.tv + (size_t)hs * 8 + srcSlot[j], vb);
    }
}
// transpose of launch_dual (dual grid, then its omni ghost update)
void launch_adj_dual(const Dev& d, const Fields& F, const Fields& G, const int* ownJ, const int* ownH, cudaStream_t st) {
    adj_omni_ghost<3>(d, G.dualO, G.dualT, F.te, F.tf, ownJ, ownH, st);
    if (d.H) ASTG_LAUNCH(k_adj_dual_half<<<nblk(d.H), TB, 0, st>>>(d, F, G));
    ASTG_LAUNCH(k_adj_dual_oct<<<nblk(d.S), TB, 0, st>>>(d, F, G));
    ASTG_LAUNCH(k_adj_dual_tilt<<<nblk(d.S), TB, 0, st>>>(d, F, G));
}

// ------------------------------------------------------------------ stage 5: advection
// transpose of one semi-Lagrangian sample through BackTrace (include/advection.h:49-62):
// P = x - dt v(m), m = x - dt/2 v(x).  pb is the cotangent of P; the velocity cotangents of the
// two back-trace samples are scattered into G (MAC and dual arrays).
__device__ void adj_back_trace(const Dev& d, const Fields& C, const Fields& G, V3 x, V3 m, double dt, V3 pb) {
    V3 vbm = pb * (-dt);
    VelAdjE em{C, G, (size_t)d.S, vbm, v3(0, 0, 0)};
    vel_w(d, m, C.tf, em);
    V3 vbx = em.pb * (-0.5 * dt);
    VelAdjE ex{C, G, (size_t)d.S, vbx, v3(0, 0, 0)};
    vel_w(d, x, C.tf, ex);
}
__device__ void adj_advect_scalar(const Dev& d, const Fields& C, const Fields& G, V3 x, double dt, double yd, double yh) {
    V3 m = x - vel_sample(d, x, C) * dt * 0.5;
    V3 P = x - vel_sample(d, m, C) * dt;
    ScalarAdjE e{C, G, yd, yh, v3(0, 0, 0)};
    scalar_w(d, P, C.tf, e);
    adj_back_trace(d, C, G, x, m, dt, e.pb);
}
__device__ void adj_advect_velocity(const Dev& d, const Fields& C, const Fields& G, V3 x, double dt, V3 vb) {
    V3 m = x - vel_sample(d, x, C) * dt * 0.5;
    V3 P = x - vel_sample(d, m, C) * dt;
    VelAdjE e{C, G, (size_t)d.S, vb, v3(0, 0, 0)};
    vel_w(d, P, C.tf, e);
    adj_back_trace(d, C, G, x, m, dt, e.pb);
}
__global__ void k_adj_decay(Dev d, Fields G) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.S) return;
    G.dO[s] *= d.decay;
    G.dT[s] *= d.decay;
    G.hO[s] *= d.decay;
    G.hT[s] *= d.decay;
}
__global__ void k_adj_adv_scalar_oct(Dev d, Fields C, Fields GC, Fields GN, double dt) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.S || adj_ghost(d, s)) return;
    double yd = GN.dO[s], yh = GN.hO[s];
    GN.dO[s] = 0;
    GN.hO[s] = 0;
    if (yd == 0 && yh == 0) return;
    adj_advect_scalar(d, C, GC, cell_pos(d, s), dt, yd, yh);
}
__global__ void k_adj_adv_scalar_tilt(Dev d, Fields C, Fields GC, Fields GN, const uint8_t* open, double dt) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.S || adj_ghost(d, s) || !open[s]) return;
    double yd = GN.dT[s], yh = GN.hT[s];
    GN.dT[s] = 0;
    GN.hT[s] = 0;
    if (yd == 0 && yh == 0) return;
    adj_advect_scalar(d, C, GC, vert_pos(d, s), dt, yd, yh);
}
__global__ void k_adj_adv_scalar_half(Dev d, Fields C, Fields GC, Fields GN, double dt) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.H) return;
    int hs = d.half[i];
    double yd = GN.dT[hs], yh = GN.hT[hs];
    GN.dT[hs] = 0;
    GN.hT[hs] = 0;
    if (yd == 0 && yh == 0) return;
    adj_advect_scalar(d, C, GC, vert_pos(d, hs), dt, yd, yh);
}
__global__ void k_adj_adv_mac(Dev d, Fields C, Fields GC, Fields GN, double dt) {
    long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= 3LL * d.S) return;
    int a = (int)(idx / d.S), s = (int)(idx - (long long)a * d.S);
    if (adj_ghost(d, s)) return;
    double y = GN.mac[(size_t)a * d.S + s];
    GN.mac[(size_t)a * d.S + s] = 0;
    if (y == 0) return;
    V3 vb = v3(a == 0 ? y : 0, a == 1 ? y : 0, a == 2 ? y : 0);
    adj_advect_velocity(d, C, GC, mac_pos(d, a, s), dt, vb);
}
__global__ void k_adj_adv_tilt(Dev d, Fields C, Fields GC, Fields GN, double dt) {
    long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= 8LL * d.S) return;
    int s = (int)(idx >> 3), k = (int)(idx & 7);
    if (adj_ghost(d, s) || (C.tf[s] & TF_CLOSED)) return;
    double y = GN.tv[(size_t)s * 8 + k];
    GN.tv[(size_t)s * 8 + k] = 0;
    if (y == 0) return;
    adj_advect_velocity(d, C, GC, tilt_pos(vert_pos(d, s), k, C.te[s]), dt, tilt_up3(k) * y);
}
__global__ void k_adj_adv_half(Dev d, Fields C, Fields GC, Fields GN, double dt) {
    long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= 8LL * d.H) return;
    int i = (int)(idx >> 3), k = (int)(idx & 7);
    int hs = d.half[i];
    int dir = tf_dir(C.tf[hs]);
    int q = -1;
    for (int j = 0; j < 5; ++j)
        if (HALF_SLOT[dir][j] == k) q = j;
    double y = GN.tv[(size_t)hs * 8 + k];
    GN.tv[(size_t)hs * 8 + k] = 0;
    if (q < 0 || y == 0) return;
    V3 c0 = vert_pos(d, hs);
    V3 pos = (q == 4) ? c0 : tilt_pos(c0, k, C.te[hs]);
    V3 dv = (q == 4) ? v3(HALF_DIR_POS[k][0], HALF_DIR_POS[k][1], HALF_DIR_POS[k][2]) : tilt_up3(k);
    adj_advect_velocity(d, C, GC, pos, dt, dv * y);
}
// transpose of stage 5 (scalar and velocity advection into the next buffer, the next buffer's
// scalar ghosts, decay): GN holds the cotangent of the state after the step and is consumed; the
// cotangents of the advected-from state C accumulate into GC
void launch_adj_advect(const Dev& d, const Fields& C, const Fields& GC, const Fields& GN, const uint8_t* open, double dt,
                       const int* ownJ, const int* ownH, cudaStream_t st) {
    ASTG_LAUNCH(k_adj_decay<<<nblk(d.S), TB, 0, st>>>(d, GN));
    if (d.H) ASTG_LAUNCH(k_adj_adv_half<<<nblk(8LL * d.H), TB, 0, st>>>(d, C, GC, GN, dt));
    ASTG_LAUNCH(k_adj_adv_tilt<<<nblk(8LL * d.S), TB, 0, st>>>(d, C, GC, GN, dt));
    ASTG_LAUNCH(k_adj_adv_mac<<<nblk(3LL * d.S), TB, 0, st>>>(d, C, GC, GN, dt));
    adj_omni_ghost<1>(d, GN.hO, GN.hT, C.te, C.tf, ownJ, ownH, st);
    adj_omni_ghost<1>(d, GN.dO, GN.dT, C.te, C.tf, ownJ, ownH, st);
    if (d.H) ASTG_LAUNCH(k_adj_adv_scalar_half<<<nblk(d.H), TB, 0, st>>>(d, C, GC, GN, dt));
    ASTG_LAUNCH(k_adj_adv_scalar_tilt<<<nblk(d.S), TB, 0, st>>>(d, C, GC, GN, open, dt));
    ASTG_LAUNCH(k_adj_adv_scalar_oct<<<nblk(d.S), TB, 0, st>>>(d, C, GC, GN, dt));
}

// ------------------------------------------------------------------ remaining launchers
void launch_adj_owners(const Dev& d, const double* te, int* ownJ, int* ownH, cudaStream_t st) {
    cudaMemsetAsync(ownJ, 0x7f, sizeof(int) * (size_t)d.S, st);
    cudaMemsetAsync(ownH, 0x7f, sizeof(int) * (size_t)d.S, st);
    if (d.nTJ) ASTG_LAUNCH(k_adj_owner_joint<<<nblk(d.nTJ), TB, 0, st>>>(d, te, ownJ));
    if (d.nCBH) ASTG_LAUNCH(k_adj_owner_cbh<<<nblk(d.nCBH), TB, 0, st>>>(d, ownH));
}
void launch_adj_source(const Dev& d, const Fields& G, double* gsO, double* gsT, cudaStream_t st) {
    if (d.H) ASTG_LAUNCH(k_adj_source_half<<<nblk(d.H), TB, 0, st>>>(d, G, gsT));
    ASTG_LAUNCH(k_adj_source_slots<<<nblk(d.S), TB, 0, st>>>(d, G, gsO, gsT));
}
void launch_adj_scalar_ghost(const Dev& d, double* go, double* gt, const double* te, const uint32_t* tf, const int* ownJ,
                             const int* ownH, cudaStream_t st) {
    adj_omni_ghost<1>(d, go, gt, te, tf, ownJ, ownH, st);
}
void launch_adj_force(const Dev& d, const Fields& F, const Fields& G, const uint8_t* open, double dt, double* gamb,
                      double invCount, cudaStream_t st) {
    cudaMemsetAsync(gamb, 0, sizeof(double), st);
    ASTG_LAUNCH(k_adj_force_mac<<<nblk(d.S), TB, 0, st>>>(d, F, G, dt, gamb));
    ASTG_LAUNCH(k_adj_force_tilt<<<nblk(8LL * d.S), TB, 0, st>>>(d, F, G, open, dt, gamb));
    if (d.H) ASTG_LAUNCH(k_adj_force_half<<<nblk(8LL * d.H), TB, 0, st>>>(d, F, G, dt, gamb));
    ASTG_LAUNCH(k_adj_amb<<<nblk(d.S), TB, 0, st>>>(d, G, gamb, invCount));
}

}  // namespace astg
