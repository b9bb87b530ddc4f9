// Collider branch of the octree step (OmniBoundarySolver3 with an SDF grid): cut-cell weights,
// wipeBoundary, the three inside-solid constrainVelocity overloads.  The DOF threshold lives in the
// numbering kernels (astg_pcg.cu) and the back-trace clamp in back_trace (astg_sample.cuh).
//
// Everything that depends only on the (static) SDF is evaluated once per collider into per-slot
// COL_* bits and the weights; the per-step kernels read the bits.
#include "astg_launch.h"
#include "astg_sample.cuh"

namespace astg {

constexpr int CTB = 256;
static inline int cblk(long long n) { return (int)((n + CTB - 1) / CTB); }

// fractionInside, include/util.h:340-349
__device__ __forceinline__ double fraction_inside(double l, double r) {
    if (l < 0 && r < 0) return 1;
    if (l < 0 && r >= 0) return l / (l - r);
    if (l >= 0 && r < 0) return r / (r - l);
    return 0;
}
// isInsideSdf, include/util.h:324
__device__ __forceinline__ bool inside_sdf(double phi) { return phi <= 0; }
__device__ __forceinline__ V3 oct_pos_l(const Dev& d, int l, int x, int y, int z) {
    double h = d.ldh[l];
    return v3(x * h + 0.5 * h, y * h + 0.5 * h, z * h + 0.5 * h);
}
// Eigen 3.3.7 on 3-vectors (no packet access: the unrolled redux splits the range in halves,
// Eigen/src/Core/Redux.h:91-105, so three terms sum as t0 + (t1 + t2)): the squared norm, and the
// tangential part v - (v . n) n with n normalised by normalize() (division by sqrt of the squared
// norm when it is positive, Eigen/src/Core/Dot.h:145-151)
__device__ __forceinline__ double sq3(V3 n) { return n.x * n.x + (n.y * n.y + n.z * n.z); }
__device__ __forceinline__ V3 tangential(V3 v, V3 n) {
    double z = sq3(n);
    if (z > 0) {
        double q = sqrt(z);
        n = v3(n.x / q, n.y / q, n.z / q);
    }
    double dd = v.x * n.x + (v.y * n.y + v.z * n.z);
    return v3(v.x - dd * n.x, v.y - dd * n.y, v.z - dd * n.z);
}
__device__ __forceinline__ V3 col_centre(const Dev& d) { return v3(d.colCx, d.colCy, d.colCz); }

// ------------------------------------------------------------------ set-up (once per collider)
// COL_* bits of every slot (ghosts get only the DOF bits, which ghosts never use)
__global__ void k_col_mask(Dev d, uint16_t* mask) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.S) return;
    const int l = slot_l(d, s), x = slot_x(d, s), y = slot_y(d, s), z = slot_z(d, s);
    const double h = d.ldh[l];
    const double so = bsdf(d, cell_pos(d, s)), sv = bsdf(d, vert_pos(d, s));
    uint16_t m = 0;
    if (so > -h * 3.0) m |= COL_OCT_FLUID;
    if (sv > -h * 3.0) m |= COL_TILT_FLUID;
    if (!(slot_f(d, s) & SF_GHOST)) {
        if (so < 0) m |= COL_WIPE_OCT;
        if (sv < 0) m |= COL_WIPE_TILT;
        for (int a = 0; a < 3; ++a)
            if (mac_valid(d, a, l, x, y, z) && inside_sdf(bsdf(d, mac_pos(d, a, s)))) m |= (uint16_t)(COL_MAC_IN << a);
        if (inside_sdf(sv)) m |= COL_DUAL_IN;
        if (inside_sdf(sv - h)) m |= COL_TILT_NEAR;
    }
    mask[s] = m;
}
// half tilts (ghost slots): their wipe bit (src/octree_omnigrid_solver3.cpp:1286-1292)
__global__ void k_col_mask_half(Dev d, uint16_t* mask) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.H) return;
    int s = d.half[i];
    if (bsdf(d, vert_pos(d, s)) < 0) mask[s] |= COL_WIPE_TILT;
}
// initCuttingCellWeights, src/octree_omnigrid_solver3.cpp:1169-1223: MAC faces and tilt slots of
// non-ghost nodes; the weights start at 1 (weightsCC->setAll(1), :83) and a face or slot whose
// neighbouring octagon is valid gets 1 - fractionInside of the SDF at the two centres
__global__ void k_col_weights(Dev d, double* wMac, double* wTilt) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.S) return;
    for (int a = 0; a < 3; ++a) wMac[(size_t)a * d.S + s] = 1.0;
    for (int k = 0; k < 8; ++k) wTilt[(size_t)s * 8 + k] = 1.0;
    if (slot_f(d, s) & SF_GHOST) return;
    const int l = slot_l(d, s), x = slot_x(d, s), y = slot_y(d, s), z = slot_z(d, s);
    const double current = bsdf(d, oct_pos_l(d, l, x, y, z));
    for (int a = 0; a < 3; ++a) {
        int id[3] = {x, y, z};
        id[a] -= 1;
        if (mac_valid(d, a, l, x, y, z) && oct_valid(d, l, id[0], id[1], id[2]))
            wMac[(size_t)a * d.S + s] = 1 - fraction_inside(bsdf(d, oct_pos_l(d, l, id[0], id[1], id[2])), current);
    }
    const double cv = bsdf(d, vert_pos(d, s));
    for (int i = 0; i < 8; ++i) {
        int nx = x + TILT_NB_OCT[i][0], ny = y + TILT_NB_OCT[i][1], nz = z + TILT_NB_OCT[i][2];
        if (oct_valid(d, l, nx, ny, nz))
            wTilt[(size_t)s * 8 + i] = 1 - fraction_inside(cv, bsdf(d, oct_pos_l(d, l, nx, ny, nz)));
    }
}
// half tilts (:1204-1223): from zero, the big octagon's slot and the four same-level slots.  Kept as
// the reference has them: the big octagon's position is taken at the half tilt's own level with the
// coarse index, and the same-level slots sample the SDF at the last position computed (the big
// octagon's when it was valid, else the half tilt's centre), not at their own octagon.
__global__ void k_col_weights_half(Dev d, const int* halfDir, double* wTilt) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.H) return;
    const int s = d.half[i];
    const int l = slot_l(d, s), x = slot_x(d, s), y = slot_y(d, s), z = slot_z(d, s);
    const int dir = halfDir[i];
    double w[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    V3 pos = vert_pos(d, s);
    const double current = bsdf(d, pos);
    int id[3] = {x >> 1, y >> 1, z >> 1};
    id[dir % 3] -= dir < 3 ? 1 : 0;
    if (l + 1 < d.L && oct_valid(d, l + 1, id[0], id[1], id[2])) {
        pos = oct_pos_l(d, l, id[0], id[1], id[2]);
        w[HALF_SLOT[dir][4]] = 1 - fraction_inside(current, bsdf(d, pos));
    }
    for (int j = 0; j < 4; ++j) {
        int k = HALF_SLOT[dir][j];
        if (oct_valid(d, l, x + TILT_NB_OCT[k][0], y + TILT_NB_OCT[k][1], z + TILT_NB_OCT[k][2]))
            w[k] = 1 - fraction_inside(current, bsdf(d, pos));
    }
    for (int k = 0; k < 8; ++k) wTilt[(size_t)s * 8 + k] = w[k];
}

// ------------------------------------------------------------------ per step
// wipeBoundary, src/octree_omnigrid_solver3.cpp:1240-1293 (EXTRAPOLATE_DENSITY undefined: the
// values become 0 / EPSILON = 0)
__global__ void k_col_wipe(Dev d, Fields F) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.S) return;
    uint16_t m = d.colMask[s];
    if (m & COL_WIPE_OCT) { F.dO[s] = 0.0; F.hO[s] = 0.0; }
    if (m & COL_WIPE_TILT) { F.dT[s] = 0.0; F.hT[s] = 0.0; }
}
// OmniBoundarySolver3::constrainVelocity(MAC grid), include/omni_boundary_solver3.h:74-92: a face
// inside the solid becomes the matching component of the tangential part of the MAC velocity
// sampled there (0 at the centre itself).  Every sample reads the velocity as it was before this
// kernel (`before`): the reference's own loop writes the grid it samples from several workers at
// once, an order that depends on thread timing; this one is defined and agrees with it wherever no
// sample reads another solid face.
__global__ void k_col_mac(Dev d, Fields F, const double* before) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.S) return;
    uint16_t m = d.colMask[s];
    if (!(m & (7 * COL_MAC_IN))) return;
    for (int a = 0; a < 3; ++a) {
        if (!(m & (COL_MAC_IN << a))) continue;
        V3 pos = mac_pos(d, a, s);
        V3 n = pos - col_centre(d);
        double out = 0;
        if (sqrt(sq3(n)) >= EPS) {
            V3 t = tangential(mac_sample(d, pos, before), n);
            out = a == 0 ? t.x : (a == 1 ? t.y : t.z);
        }
        F.mac[(size_t)a * d.S + s] = out;
    }
}
// constrainVelocity(tilt grid, MAC grid), include/omni_boundary_solver3.h:26-52: for open tilts with
// SDF(centre) - dx <= 0, slot k (at centre + e/3, e = dx/2) inside the solid.  The reference writes
// its projected value into a shadowing local Vector3f, not into the tilt, so only a slot sitting on
// the centre itself changes (to 0).
__global__ void k_col_tilt(Dev d, Fields F) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.S) return;
    if (!(d.colMask[s] & COL_TILT_NEAR) || (F.tf[s] & TF_CLOSED)) return;
    V3 c = vert_pos(d, s);
    double e = d.ldh[slot_l(d, s)] * 0.5;
    for (int k = 0; k < 8; ++k) {
        V3 p1 = tilt_pos(c, k, e);
        if (inside_sdf(bsdf(d, p1)) && sqrt(sq3(p1 - col_centre(d))) < EPS) F.tv[(size_t)s * 8 + k] = 0;
    }
}
// constrainVelocity(OctreeOmniVector3Grid3), include/omni_boundary_solver3.h:55-71: dual vectors at
// tilt positions inside the solid lose their normal part (0 at the centre itself)
__global__ void k_col_dual(Dev d, Fields F) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.S) return;
    if (!(d.colMask[s] & COL_DUAL_IN)) return;
    V3 n = vert_pos(d, s) - col_centre(d);
    V3 v = v3(F.dualT[3 * s], F.dualT[3 * s + 1], F.dualT[3 * s + 2]);
    V3 t = sqrt(sq3(n)) < EPS ? v3(0, 0, 0) : tangential(v, n);
    F.dualT[3 * s] = t.x;
    F.dualT[3 * s + 1] = t.y;
    F.dualT[3 * s + 2] = t.z;
}

// OmniBoundarySolver3::updateCollider (src/omni_boundary_solver3.cpp:17-32) for a Sphere3 collider
// wrapped in ShapeToImplicit3 (the stock obstacle, src/octree_omnigrid_solver3.cpp:157-158): the
// signed distance of ShapeToImplicit3::signedDistanceLocal (include/geometry/shape_to_implicit3.h:41-46)
// at each finest cell centre (i + 0.5) * dx.  Both transforms have identity orientations, so toLocal
// and toWorld are exact translations; the closest point is the centre plus the radius times the
// normalised offset, (1, 0, 0) when the offset's norm is below epsilon (include/geometry/sphere3.h:20-26).
// Norms and the dot product of these plain 3-vectors are Eigen's packet reductions: the first two
// terms as one SSE2 packet, then the third, (t0 + t1) + t2 (Eigen/src/Core/Redux.h:306-329).
__device__ __forceinline__ double sq3p(V3 n) { return (n.x * n.x + n.y * n.y) + n.z * n.z; }
__global__ void k_col_sphere_sdf(int res, double dx, double cx, double cy, double cz, double r, double* sdf) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long n = (long long)res * res * res;
    if (i >= n) return;
    const int x = (int)(i % res), y = (int)((i / res) % res), z = (int)(i / ((long long)res * res));
    const V3 p = v3((x + 0.5) * dx, (y + 0.5) * dx, (z + 0.5) * dx);
    const V3 c = v3(cx, cy, cz);
    const V3 q = p - c;
    V3 nl = v3(1, 0, 0);
    if (!(sqrt(sq3p(q)) < EPS)) {
        double zz = sq3p(q);
        nl = q;
        if (zz > 0) {
            double k = sqrt(zz);
            nl = v3(q.x / k, q.y / k, q.z / k);
        }
    }
    const V3 xc = v3(nl.x * r, nl.y * r, nl.z * r) + c;
    const V3 off = p - xc;
    const double dot = (nl.x * off.x + nl.y * off.y) + nl.z * off.z;
    const double len = sqrt(sq3p(xc - p));
    sdf[i] = dot < 0.0 ? -len : len;
}
void launch_collider_sphere_sdf(int res, double cx, double cy, double cz, double r, double* sdf, cudaStream_t st) {
    const long long n = (long long)res * res * res;
    ASTG_LAUNCH(k_col_sphere_sdf<<<(unsigned)((n + CTB - 1) / CTB), CTB, 0, st>>>(res, 1.0 / res, cx, cy, cz, r, sdf));
}

// refineSplitMapByObstacleSdf (include/octree_util.h:17-47) on device arrays: one thread per block
// of 2^level finest cells; a block whose corner cell carries split value `level` and whose SDF,
// sampled at the block centre, lies in [lo, hi] is set to level - 1.  Blocks read and write only
// their own cells, as in the reference's parallel loop.
__global__ void k_refine_split(int32_t* split, int res, int level, const double* sdf, double lo, double hi) {
    const long long c = res >> level;
    long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= c * c * c) return;
    const int tx = (int)(t % c), ty = (int)((t / c) % c), tz = (int)(t / (c * c));
    auto at = [&](int x, int y, int z) -> int32_t& { return split[((size_t)z * res + y) * res + x]; };
    if (at(tx << level, ty << level, tz << level) != level) return;
    const double dh = (1.0 / res) * (1 << level);
    const double v = sdf_sample(sdf, res, v3((tx + 0.5) * dh, (ty + 0.5) * dh, (tz + 0.5) * dh));
    if (!(v >= lo && v <= hi)) return;
    const int k = 1 << level;
    for (int z = tz << level; z < (tz << level) + k; ++z)
        for (int y = ty << level; y < (ty << level) + k; ++y)
            for (int x = tx << level; x < (tx << level) + k; ++x) at(x, y, z) = level - 1;
}
cudaError_t launch_refine_split_map(int32_t* split, int res, int level, const double* sdf, double lo, double hi,
                                    cudaStream_t st) {
    const long long c = res >> level, n = c * c * c;
    void* args[] = {&split, &res, &level, &sdf, &lo, &hi};
    count_launch();
    return cudaLaunchKernel((const void*)k_refine_split, dim3((unsigned)((n + CTB - 1) / CTB)), dim3(CTB), args, 0, st);
}

// halfDir: each half tilt's direction (0-5, the list order of d.half)
void launch_collider_setup(const Dev& d, const int* halfDir, uint16_t* mask, double* wMac, double* wTilt,
                           cudaStream_t st) {
    ASTG_LAUNCH(k_col_mask<<<cblk(d.S), CTB, 0, st>>>(d, mask));
    if (d.H) ASTG_LAUNCH(k_col_mask_half<<<cblk(d.H), CTB, 0, st>>>(d, mask));
    ASTG_LAUNCH(k_col_weights<<<cblk(d.S), CTB, 0, st>>>(d, wMac, wTilt));
    if (d.H) ASTG_LAUNCH(k_col_weights_half<<<cblk(d.H), CTB, 0, st>>>(d, halfDir, wTilt));
}
void launch_collider_wipe(const Dev& d, const Fields& F, cudaStream_t st) {
    ASTG_LAUNCH(k_col_wipe<<<cblk(d.S), CTB, 0, st>>>(d, F));
}
void launch_collider_mac(const Dev& d, const Fields& F, double* before, cudaStream_t st) {
    cudaMemcpyAsync(before, F.mac, sizeof(double) * 3 * (size_t)d.S, cudaMemcpyDeviceToDevice, st);
    ASTG_LAUNCH(k_col_mac<<<cblk(d.S), CTB, 0, st>>>(d, F, before));
}
void launch_collider_tilt(const Dev& d, const Fields& F, cudaStream_t st) {
    ASTG_LAUNCH(k_col_tilt<<<cblk(d.S), CTB, 0, st>>>(d, F));
}
void launch_collider_dual(const Dev& d, const Fields& F, cudaStream_t st) {
    ASTG_LAUNCH(k_col_dual<<<cblk(d.S), CTB, 0, st>>>(d, F));
}

}  // namespace astg
