// Device data model and per-point operators of the octree smoke step (GB300 / sm_103a).
//
// Storage: "slots".  Level l (0 = finest) holds its non-ghost cells in raster (z, y, x) order
// followed by its ghost cells in discovery order -- the reference's layout index order
// (src/octree_layer3.cpp:14-85) -- and the levels are concatenated finest first, so a slot is
// the reference's (level, layout index) flattened.  Keeping that order makes the DOF numbering,
// the matrix rows and every field array identical to the reference's without a permutation.
// Point location uses dense per-level index bricks instead of the reference's hash map
// (include/octree_layer3.h:24-80) plus one byte per finest cell holding the finest non-ghost
// level that contains it (OctreeGridLayout3::levelCoordinate, src/octree_grid_layout3.cpp:16-41).
//
// Every floating-point expression below keeps the operand order of the reference (and of the
// oracle that restates it); the library is compiled with FMA contraction off so that the FP64
// step reproduces the oracle bit for bit.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#ifndef ASTG_HD
#define ASTG_HD __device__
#endif

namespace astg {

constexpr int MAXL = 6;
constexpr double SQRT3 = 1.7320508075688772;   // include/macro.h:17
constexpr double INV_SQRT3 = 1.0 / SQRT3;       // include/macro.h:20 (standalone use)
constexpr double EPS = 2.220446049250313e-16;   // numeric_limits<double>::epsilon()

enum : uint8_t { SF_GHOST = 1, SF_FROM_COARSE = 2 };
// tilt-E state bits (include/tilt_e_node.h:15-24); bits 8..15 hold half_direction + 1
enum : uint32_t { TF_LARGEST = 1, TF_CLOSED = 2, TF_FIXED = 4, TF_TJOINT = 8, TF_CLOSED_BY_T = 16, TF_HALF = 32 };
ASTG_HD inline int tf_dir(uint32_t f) { return (int)((f >> 8) & 0xff) - 1; }

// device status codes (first error wins)
enum : int { DS_OK = 0, DS_MISSING_NODE = 1, DS_NO_CELL = 2, DS_WAIT_TIMEOUT = 3, DS_NAN = 4 };

struct V3 {
    double x, y, z;
};
ASTG_HD inline V3 v3(double a, double b, double c) { V3 r; r.x = a; r.y = b; r.z = c; return r; }
ASTG_HD inline V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
ASTG_HD inline V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
ASTG_HD inline V3 operator*(V3 a, double s) { return v3(a.x * s, a.y * s, a.z * s); }
ASTG_HD inline V3 operator/(V3 a, double s) { return v3(a.x / s, a.y / s, a.z / s); }
ASTG_HD inline double comp(V3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
ASTG_HD inline double dot3(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
ASTG_HD inline double dmin(double a, double b) { return (b < a) ? b : a; }  // std::min
ASTG_HD inline int imin(int a, int b) { return (b < a) ? b : a; }
ASTG_HD inline int imax(int a, int b) { return (a < b) ? b : a; }

// include/util.h:164-187
ASTG_HD inline double lerp(double a, double b, double f) { return a * (1 - f) + b * f; }
ASTG_HD inline V3 lerp(V3 a, V3 b, double f) { return a * (1 - f) + b * f; }
template <class T>
ASTG_HD inline T trilerp(T f000, T f100, T f010, T f110, T f001, T f101, T f011, T f111, double tx, double ty, double tz) {
    T a = lerp(lerp(f000, f100, tx), lerp(f010, f110, tx), ty);
    T b = lerp(lerp(f001, f101, tx), lerp(f011, f111, tx), ty);
    return lerp(a, b, tz);
}
// include/util.h:258-282
ASTG_HD inline void bary(double x, int iLow, int iHigh, int* i, double* f) {
    double s = floor(x);
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
// include/util.h:243-256: truncating cast, clamped
ASTG_HD inline void bary_vec(double x, int high, int* i, double* f) {
    int c = (int)x;
    if (c < 0) c = 0;
    if (c > high - 1) c = high - 1;
    *i = c;
    double t = x - c;
    *f = t < 0 ? 0 : (t > 1 ? 1 : t);
}

// stencil tables, include/constants.h:85-155
struct Tables {
    int oct_nb[6][3];
    int oct_nb_tilt[8][3];
    int oct_nb_face[6][3];
    int tilt_nb_oct[8][3];
    int half_slot[6][5];
    double half_dir_pos[6][3];
    int tilt_up_sign[8][3];
    int sample_marker[8][8];
};

// Everything a kernel needs, passed by value.
struct Dev {
    int L, res, S, H, nTJ, nCBH;
    double dx;
    int lres[MAXL], loff[MAXL], lN[MAXL], lG[MAXL];
    double ldh[MAXL];
    // 1 when the finest resolution is a power of two: then every spacing is a power of two and
    // dxInv, ldhInv hold their exact reciprocals (see over_h)
    int pow2;
    double dxInv;
    double ldhInv[MAXL];
    const int* brick[MAXL];       // per level: global slot or -1
    const uint8_t* locate;        // per finest cell: finest non-ghost level containing it (0xff none)
    const int4* slot;             // x, y, z, level | flags << 8
    const int* half;              // half-tilt slots in the reference's list order
    const uint8_t* halfMark;      // 1 on half-tilt slots
    const int* tj;                // T-joint slots
    const int* cbh;               // tilts closed by a half tilt
    const double* wMac;           // 3 * S
    const double* wTilt;          // S * 8
    const double* M37;            // 128 * 3 * 7 least-squares tables
    int* status;                  // device error word
    // physics
    double buoyD, buoyT, rho, decay;
    int closedMask;
    double srcX, srcY, srcZ, srcR;
    const double* srcO;           // per slot: density the source sets on the octagon (default 1)
    const double* srcT;           // per slot: density the source sets on the tilt / half tilt
    // collider (OmniBoundarySolver3): SDF grid res^3 at the finest cell centres, index
    // (z * res + y) * res + x; null when there is none (the reference's grid of 1s, on which every
    // collider test is false); per-slot COL_* bits; the centre the inside-solid projection takes
    // its normals from
    const double* sdf;
    const uint16_t* colMask;
    double colCx, colCy, colCz;
};
// per-slot collider bits (set once per collider)
enum {
    COL_OCT_FLUID = 1,    // octagon may carry a DOF: SDF at the cell centre > -3 dx_l
    COL_TILT_FLUID = 2,   // tilt (or half tilt) may carry a DOF: SDF at the vertex > -3 dx_l
    COL_WIPE_OCT = 4,     // wipeBoundary zeroes density and heat of the octagon (SDF < 0)
    COL_WIPE_TILT = 8,    // ... of the tilt or half tilt
    COL_MAC_IN = 16,      // << a: MAC face a inside the solid (SDF <= 0), three bits
    COL_DUAL_IN = 128,    // tilt position inside the solid: the dual vector is projected
    COL_TILT_NEAR = 256   // SDF(vertex) - dx_l <= 0: the tilt slots are tested
};

struct Fields {
    double* dO;  // density on octagons (cells)
    double* dT;  // density on tilts (vertices)
    double* hO;
    double* hT;
    double* mac;    // 3 * S, axis-major
    double* tv;     // S * 8 tilted-face velocities
    double* dualO;  // S * 3
    double* dualT;  // S * 3
    double* te;     // tilt size e
    uint32_t* tf;   // tilt-E flag bits
    // S * 3 or null: per tilt, the dual vector minus the MAC velocity sampled at its vertex, the
    // correction the velocity sampler adds near open tilts; filled once per step before the
    // advection (k_tilt_corr) so the samplers read it instead of sampling the MAC grid again
    const double* corrT;
};

ASTG_HD inline void report(const Dev& d, int code) {
#ifdef __CUDA_ARCH__
    atomicCAS(d.status, 0, code);
#else
    if (*d.status == 0) *d.status = code;
#endif
}

ASTG_HD inline int slot_x(const Dev& d, int s) { return d.slot[s].x; }
ASTG_HD inline int slot_y(const Dev& d, int s) { return d.slot[s].y; }
ASTG_HD inline int slot_z(const Dev& d, int s) { return d.slot[s].z; }
ASTG_HD inline int slot_l(const Dev& d, int s) { return d.slot[s].w & 0xff; }
ASTG_HD inline int slot_f(const Dev& d, int s) { return (d.slot[s].w >> 8) & 0xff; }

// layout->get: slot or -1 (ghosts included)
ASTG_HD inline int get(const Dev& d, int l, int x, int y, int z) {
    if (l < 0 || l >= d.L) return -1;
    int r = d.lres[l];
    if (x < 0 || y < 0 || z < 0 || x >= r || y >= r || z >= r) return -1;
    return d.brick[l][((size_t)z * r + y) * r + x];
}
// a lookup the reference performs without a check: a missing node is reported and slot 0 used
ASTG_HD inline int req(const Dev& d, int l, int x, int y, int z) {
    int s = get(d, l, x, y, z);
    if (s < 0) {
        report(d, DS_MISSING_NODE);
        return 0;
    }
    return s;
}
ASTG_HD inline bool oct_valid(const Dev& d, int l, int x, int y, int z) {
    int r = d.lres[l] - 1;
    return x >= 0 && y >= 0 && z >= 0 && x < r && y < r && z < r;
}
ASTG_HD inline bool lay_valid(const Dev& d, int l, int x, int y, int z) {
    int r = d.lres[l];
    return x >= 0 && y >= 0 && z >= 0 && x < r && y < r && z < r;
}
ASTG_HD inline bool mac_valid(const Dev& d, int a, int l, int x, int y, int z) {
    int r = d.lres[l];
    int c0 = x, c1 = y, c2 = z;
    int h0 = a == 0 ? r : r - 1, h1 = a == 1 ? r : r - 1, h2 = a == 2 ? r : r - 1;
    return c0 >= 0 && c1 >= 0 && c2 >= 0 && c0 < h0 && c1 < h1 && c2 < h2;
}
// src/octree_grid_layout3.cpp:51-69 (returns a non-ghost slot or -1)
ASTG_HD inline int get_until(const Dev& d, int l, int x, int y, int z, bool toFinest) {
    int r = d.lres[l];
    if (x < 0 || y < 0 || z < 0 || x >= r || y >= r || z >= r) return -1;
    for (;;) {
        int s = get(d, l, x, y, z);
        if (s >= 0 && !(slot_f(d, s) & SF_GHOST)) return s;
        if (toFinest) { x <<= 1; y <<= 1; z <<= 1; l -= 1; }
        else { x >>= 1; y >>= 1; z >>= 1; l += 1; }
        if (l < 0 || l >= d.L) return -1;
    }
}
// x / h for the spacing of level l (l < 0: the finest spacing d.dx), as the reference divides.  With
// a power-of-two resolution every spacing is a power of two, and x * (1 / h) is then the same
// number bit for bit (the factor only moves the exponent; positions are far from overflow): one
// FP64 multiply instead of an IEEE division, which costs about ten FP64 instructions on a part
// where FP64 issue bounds the samplers.
ASTG_HD inline double over_h(const Dev& d, double x, int l) {
    if (d.pow2) return x * (l < 0 ? d.dxInv : d.ldhInv[l]);
    return x / (l < 0 ? d.dx : d.ldh[l]);
}
// src/octree_grid_layout3.cpp:16-41
ASTG_HD inline int level_of(const Dev& d, double px, double py, double pz) {
    int xi, yi, zi;
    double f;
    bary(over_h(d, px, -1), 0, d.res, &xi, &f);
    bary(over_h(d, py, -1), 0, d.res, &yi, &f);
    bary(over_h(d, pz, -1), 0, d.res, &zi, &f);
    int l = d.locate[((size_t)zi * d.res + yi) * d.res + xi];
    if (l == 0xff) {
        report(d, DS_NO_CELL);
        return d.L - 1;
    }
    return l;
}
ASTG_HD inline bool is_ghost_node(const Dev& d, int l, int x, int y, int z) {
    int s = get(d, l, x, y, z);
    return s >= 0 && (slot_f(d, s) & SF_GHOST);
}

// positions (include/octree_cell_centered_grid3.h:44, include/octree_face_centered_grid3.h:17-22,
// include/octree_omni_tilt_grid3.h:35-42)
ASTG_HD inline V3 cell_pos(const Dev& d, int s) {
    double h = d.ldh[slot_l(d, s)];
    return v3(slot_x(d, s) * h + 0.5 * h, slot_y(d, s) * h + 0.5 * h, slot_z(d, s) * h + 0.5 * h);
}
ASTG_HD inline V3 vert_pos(const Dev& d, int s) {
    double h = d.ldh[slot_l(d, s)];
    return v3(slot_x(d, s) * h, slot_y(d, s) * h, slot_z(d, s) * h);
}
ASTG_HD inline V3 mac_pos(const Dev& d, int a, int s) {
    double h = d.ldh[slot_l(d, s)];
    double x = slot_x(d, s) * h + 0.5 * h, y = slot_y(d, s) * h + 0.5 * h, z = slot_z(d, s) * h + 0.5 * h;
    if (a == 0) x = slot_x(d, s) * h + 0.0 * h;
    if (a == 1) y = slot_y(d, s) * h + 0.0 * h;
    if (a == 2) z = slot_z(d, s) * h + 0.0 * h;
    return v3(x, y, z);
}
ASTG_HD inline V3 tilt_pos(V3 c, int dir, double e) {
    int m = dir & 3;
    double tz = (dir < 4 ? 1 : -1) * e / 3.0;
    double ty = (m < 2 ? 1 : -1) * e / 3.0;
    double tx = ((m == 0 || m == 3) ? 1 : -1) * e / 3.0;
    return v3(c.x + tx, c.y + ty, c.z + tz);
}

}  // namespace astg
