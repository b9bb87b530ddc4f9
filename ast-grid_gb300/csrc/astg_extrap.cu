// Velocity/scalar extrapolation: FmmLevelSetSolver3::extrapolate (include/jet/fmm_levelset_solver3.h
// :84-408) on the AST octree, as level-synchronous GPU passes instead of a sequential heap.
//
// The reference marks the nodes whose signed distance sample passes its validity test as known,
// then pops unknown nodes from a heap ordered by their SDF sample ("key") and gives each the mean
// of its neighbours known at that moment, pushing the unknown ones.  Three facts let the GPU
// reproduce the pop order without the heap:
//   * tau(v), the heap's key threshold when v is popped, is max(key(v), min over the nodes u that
//     push v of tau(u)), with tau = -inf for the nodes known from the start (a minimax path value,
//     found by Bellman-Ford relaxation);
//   * the march stops at the first popped key above max_distance_factor * dx_0, so exactly the
//     nodes with tau <= that limit are assigned;
//   * a node pushed after its key has been passed ("late": key < tau) is popped right after the
//     node that pushed it; nodes are therefore ordered by (tau, late, key, slot).
// A node's value depends only on neighbours earlier in that order, so the nodes are grouped into
// rounds (1 + the latest round among such neighbours) and each round is one parallel pass.  The
// neighbour stencils and the summation order are the reference's; the order of nodes pushed late
// in a chain is approximated by their keys (the reference pops those by heap dynamics).
#include <cstdio>

#include "astg_launch.h"
#include "astg_sample.cuh"

namespace astg {

namespace {

enum : uint8_t { X_UNKNOWN = 0, X_KNOWN = 1, X_DONT_TOUCH = 3, X_GHOST = 4 };
constexpr double X_SQRT3 = 1.7320508075688772;  // include/macro.h:17
constexpr int XTB = 256;
inline int xblk(long long n) { return (int)((n + XTB - 1) / XTB); }

// doubles as order-preserving unsigned keys (for atomicMin)
__device__ __forceinline__ unsigned long long ord_bits(double v) {
    unsigned long long b = (unsigned long long)__double_as_longlong(v);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double from_ord(unsigned long long b) {
    return __longlong_as_double((long long)((b >> 63) ? (b & 0x7fffffffffffffffull) : ~b));
}


struct XState {
    uint8_t* mark;            // 2S: node 2s octagon, 2s + 1 tilt
    double* key;              // 2S: SDF sample at the node
    unsigned long long* tau;  // 2S: order-preserving bits of tau
    int* round;               // 2S: 0 = not assigned, else the pass that assigns it
    int* changed;
    int* maxRound;
    unsigned long long* assigned;
    double limit;             // max_distance_factor * dx_0
    double offset;
};

__device__ __forceinline__ int half_dir(const Fields& F, int s) { return (int)((F.tf[s] >> 8) & 0xff) - 1; }
__device__ __forceinline__ bool is_half(const Fields& F, int s) { return F.tf[s] & TF_HALF; }

// a tilt vertex that is a ghost stands for the non-ghost node getUntil finds when that node is
// finer or sits at the same corner (:176-178, :322-325)
__device__ int ghost_tilt(const Dev& d, int l, int x, int y, int z) {
    int c0 = get_until(d, l, x, y, z, true);
    if (c0 < 0) c0 = get_until(d, l, x, y, z, false);
    if (c0 < 0) return -1;
    if (slot_l(d, c0) < l || ((slot_x(d, c0) << 1) == x && (slot_y(d, c0) << 1) == y && (slot_z(d, c0) << 1) == z))
        return c0;
    return -1;
}
// tiltNeighborOctagon3 as a slot (-1: none or not in the layout)
__device__ int tilt_nb_slot(const Dev& d, int s, int k) {
    NbOct nb = tilt_nb_oct(d, slot_l(d, s), slot_x(d, s), slot_y(d, s), slot_z(d, s), k);
    return nb.some ? get(d, nb.l, nb.x, nb.y, nb.z) : -1;
}
// halfTiltNeighborOctagon3 + the big octagon on the coarse side, as slots (-1: none)
__device__ int half_nb_slot(const Dev& d, const Fields& F, int hs, int k) {
    int dir = half_dir(F, hs);
    int l = slot_l(d, hs), x = slot_x(d, hs), y = slot_y(d, hs), z = slot_z(d, hs);
    if (k == HALF_SLOT[dir][4]) {
        int id[3] = {x >> 1, y >> 1, z >> 1};
        id[dir % 3] -= dir < 3 ? 1 : 0;
        return l + 1 < d.L ? get(d, l + 1, id[0], id[1], id[2]) : -1;
    }
    for (int i = 0; i < 4; ++i)
        if (HALF_SLOT[dir][i] == k) return get(d, l, x + TILT_NB_OCT[k][0], y + TILT_NB_OCT[k][1], z + TILT_NB_OCT[k][2]);
    return -1;
}
// the half tilt on face k of octagon (l, x, y, z), or -1
__device__ int oct_half_slot(const Dev& d, const Fields& F, int l, int x, int y, int z, int k) {
    if (l < 1) return -1;
    int id[3] = {2 * x + 1, 2 * y + 1, 2 * z + 1};
    id[k >> 1] += (k & 1) ? 1 : -1;
    int t = get(d, l - 1, id[0], id[1], id[2]);
    return (t >= 0 && is_half(F, t)) ? t : -1;
}

// ---------------------------------------------------------------- markers and keys (:92-140)
__global__ void k_x_init(Dev d, Fields F, const double* sdf, int sres, XState X) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.S) return;
    uint8_t mo = X_UNKNOWN, mt = X_UNKNOWN;
    double ko = 0, kt = 0;
    if (slot_f(d, s) & SF_GHOST) {
        mo = mt = X_GHOST;
        kt = sdf_sample(sdf, sres, vert_pos(d, s));
    } else {
        int l = slot_l(d, s);
        ko = sdf_sample(sdf, sres, cell_pos(d, s));
        kt = sdf_sample(sdf, sres, vert_pos(d, s));
        if (oct_valid(d, l, slot_x(d, s), slot_y(d, s), slot_z(d, s))) {
            if (ko < -X.offset * (d.ldh[l] * X_SQRT3 * 0.5)) mo = X_KNOWN;
        } else {
            mo = X_DONT_TOUCH;
        }
        if (F.tf[s] & TF_CLOSED) mt = X_DONT_TOUCH;
        else if (kt < -X.offset * F.te[s]) mt = X_KNOWN;
    }
    X.mark[2 * s] = mo;
    X.mark[2 * s + 1] = mt;
    X.key[2 * s] = ko;
    X.key[2 * s + 1] = kt;
    X.round[2 * s] = 0;
    X.round[2 * s + 1] = 0;
    X.tau[2 * s] = ord_bits(mo == X_KNOWN ? -INFINITY : INFINITY);
    X.tau[2 * s + 1] = ord_bits(mt == X_KNOWN ? -INFINITY : INFINITY);
}
__global__ void k_x_half(Dev d, Fields F, XState X) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.H) return;
    int hs = d.half[i];
    if (X.key[2 * hs + 1] < -X.offset * d.ldh[slot_l(d, hs)]) {
        X.mark[2 * hs + 1] = X_KNOWN;
        X.tau[2 * hs + 1] = ord_bits(-INFINITY);
    }
}

// ---------------------------------------------------------------- tau relaxation
__device__ __forceinline__ void x_offer(XState& X, int v, double tu) {
    if (X.mark[v] != X_UNKNOWN) return;
    double nt = fmax(X.key[v], tu);
    unsigned long long b = ord_bits(nt);
    if (b < X.tau[v]) {
        unsigned long long old = atomicMin(X.tau + v, b);
        if (b < old) *X.changed = 1;
    }
}
// every node that is known or will be assigned offers its tau to the nodes it pushes
__global__ void k_x_tau(Dev d, Fields F, XState X) {
    int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= 2 * d.S) return;
    double tu = from_ord(X.tau[u]);
    bool active = X.mark[u] == X_KNOWN || (X.mark[u] == X_UNKNOWN && tu <= X.limit);
    if (!active) return;
    int s = u >> 1;
    if ((u & 1) == 0) {  // octagon: face octagons, tilt vertices (ghosts resolved)
        int l = slot_l(d, s), x = slot_x(d, s), y = slot_y(d, s), z = slot_z(d, s);
        for (int k = 0; k < 6; ++k) {
            int tx = x + OCT_NB[k][0], ty = y + OCT_NB[k][1], tz = z + OCT_NB[k][2];
            if (!oct_valid(d, l, tx, ty, tz)) continue;
            int t = get(d, l, tx, ty, tz);
            if (t >= 0) x_offer(X, 2 * t, tu);
        }
        for (int k = 0; k < 8; ++k) {
            int tx = x + OCT_NB_TILT[k][0], ty = y + OCT_NB_TILT[k][1], tz = z + OCT_NB_TILT[k][2];
            int t = get(d, l, tx, ty, tz);
            if (t < 0) continue;
            if (X.mark[2 * t + 1] == X_GHOST) {
                int c0 = ghost_tilt(d, l, tx, ty, tz);
                if (c0 >= 0) x_offer(X, 2 * c0 + 1, tu);
            } else {
                x_offer(X, 2 * t + 1, tu);
            }
        }
    } else if (is_half(F, s)) {  // known half tilt: the octagons around it
        for (int k = 0; k < 8; ++k) {
            int t = half_nb_slot(d, F, s, k);
            if (t >= 0) x_offer(X, 2 * t, tu);
        }
    } else {  // tilt: the octagons behind its eight faces
        for (int k = 0; k < 8; ++k) {
            int t = tilt_nb_slot(d, s, k);
            if (t >= 0) x_offer(X, 2 * t, tu);
        }
    }
}

// ---------------------------------------------------------------- order and rounds
struct XOrd {
    double tau, key;
    int late, id;
};
__device__ __forceinline__ bool x_assigned(const XState& X, int v) {
    return X.mark[v] == X_UNKNOWN && from_ord(X.tau[v]) <= X.limit;
}
__device__ __forceinline__ XOrd x_ord(const XState& X, int v) {
    XOrd o;
    o.tau = from_ord(X.tau[v]);
    o.key = X.key[v];
    o.late = o.key < o.tau ? 1 : 0;
    o.id = v;
    return o;
}
__device__ __forceinline__ bool x_before(const XOrd& a, const XOrd& b) {
    if (a.tau != b.tau) return a.tau < b.tau;
    if (a.late != b.late) return a.late < b.late;
    if (a.key != b.key) return a.key < b.key;
    return a.id < b.id;
}
// Visits, in the reference's summation order, the neighbours a node reads, calling
// f(node id that decides known-ness, value pointer) for each.
template <typename Fn>
__device__ void x_neighbours(const Dev& d, const Fields& F, const uint8_t* mark, const double* oct, const double* til,
                             int v, Fn f) {
    int s = v >> 1;
    if ((v & 1) == 0) {
        int l = slot_l(d, s), x = slot_x(d, s), y = slot_y(d, s), z = slot_z(d, s);
        for (int k = 0; k < 6; ++k) {
            int tx = x + OCT_NB[k][0], ty = y + OCT_NB[k][1], tz = z + OCT_NB[k][2];
            if (!oct_valid(d, l, tx, ty, tz)) continue;
            int t = get(d, l, tx, ty, tz);
            if (t >= 0) f(2 * t, oct + t);
        }
        for (int k = 0; k < 6; ++k) {
            int t = oct_half_slot(d, F, l, x, y, z, k);
            if (t >= 0) f(2 * t + 1, til + t);
        }
        for (int k = 0; k < 8; ++k) {
            int tx = x + OCT_NB_TILT[k][0], ty = y + OCT_NB_TILT[k][1], tz = z + OCT_NB_TILT[k][2];
            int t = get(d, l, tx, ty, tz);
            if (t < 0) continue;
            if (mark[2 * t + 1] == X_GHOST) {
                // the ghost slot's own value, counted when the node it stands for is known
                int c0 = ghost_tilt(d, l, tx, ty, tz);
                if (c0 >= 0) f(2 * c0 + 1, til + t);
            } else {
                f(2 * t + 1, til + t);
            }
        }
    } else {
        for (int k = 0; k < 8; ++k) {
            int t = tilt_nb_slot(d, s, k);
            if (t >= 0) f(2 * t, oct + t);
        }
    }
}
__global__ void k_x_round(Dev d, Fields F, XState X, const double* oct, const double* til) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= 2 * d.S || !x_assigned(X, v)) return;
    XOrd me = x_ord(X, v);
    int r = 1;
    x_neighbours(d, F, X.mark, oct, til, v, [&](int n, const double*) {
        if (x_assigned(X, n) && x_before(x_ord(X, n), me)) r = max(r, X.round[n] + 1);
    });
    if (r > X.round[v]) {
        X.round[v] = r;
        *X.changed = 1;
        atomicMax(X.maxRound, r);
    }
}
__global__ void k_x_value(Dev d, Fields F, XState X, double* oct, double* til, int pass) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= 2 * d.S || X.round[v] != pass || !x_assigned(X, v)) return;
    XOrd me = x_ord(X, v);
    double sum = 0.0, count = 0.0;
    x_neighbours(d, F, X.mark, oct, til, v, [&](int n, const double* val) {
        bool known = X.mark[n] == X_KNOWN || (x_assigned(X, n) && x_before(x_ord(X, n), me));
        if (known) {
            sum += *val;
            count += 1;
        }
    });
    int s = v >> 1;
    if ((v & 1) == 0) oct[s] = sum / count;
    else til[s] = sum / count;
    atomicAdd(X.assigned, 1ull);
}

}  // namespace

// Extrapolates (oct, til) in place; returns the nodes assigned, and the passes in *passes.
long long launch_extrapolate(const Dev& d, const Fields& F, double* oct, double* til, const double* sdf, int sres,
                             double offset, double maxFactor, void* scratch, int* passes, cudaStream_t st) {
    // scratch layout: mark 2S | key 2S | tau 2S | round 2S | changed, maxRound | assigned
    size_t n = 2 * (size_t)d.S;
    char* p = (char*)scratch;
    XState X;
    X.key = (double*)p;
    X.tau = (unsigned long long*)(p + 8 * n);
    X.round = (int*)(p + 16 * n);
    X.changed = (int*)(p + 20 * n);
    X.maxRound = X.changed + 1;
    X.assigned = (unsigned long long*)(p + 20 * n + 8);
    X.mark = (uint8_t*)(p + 20 * n + 16);
    X.limit = d.ldh[0] * maxFactor;
    X.offset = offset;
    ASTG_LAUNCH(k_x_init<<<xblk(d.S), XTB, 0, st>>>(d, F, sdf, sres, X));
    if (d.H) ASTG_LAUNCH(k_x_half<<<xblk(d.H), XTB, 0, st>>>(d, F, X));
    int flags[2];
    // tau: every relaxation pass lowers some tau or ends the loop; bounded by the node count
    for (long long it = 0; it < (long long)n + 8; it += 4) {
        cudaMemsetAsync(X.changed, 0, sizeof(int), st);
        for (int k = 0; k < 4; ++k) ASTG_LAUNCH(k_x_tau<<<xblk((long long)n), XTB, 0, st>>>(d, F, X));
        cudaMemcpyAsync(flags, X.changed, sizeof(int), cudaMemcpyDeviceToHost, st);
        if (cudaStreamSynchronize(st) != cudaSuccess) return -1;
        if (!flags[0]) break;
    }
    // rounds: the longest chain of order-earlier neighbours
    cudaMemsetAsync(X.maxRound, 0, sizeof(int), st);
    cudaMemsetAsync(X.assigned, 0, sizeof(unsigned long long), st);
    for (long long it = 0; it < (long long)n + 8; it += 4) {
        cudaMemsetAsync(X.changed, 0, sizeof(int), st);
        for (int k = 0; k < 4; ++k) ASTG_LAUNCH(k_x_round<<<xblk((long long)n), XTB, 0, st>>>(d, F, X, oct, til));
        cudaMemcpyAsync(flags, X.changed, sizeof(int) * 2, cudaMemcpyDeviceToHost, st);
        if (cudaStreamSynchronize(st) != cudaSuccess) return -1;
        if (!flags[0]) break;
    }
    int rounds = flags[1];
    for (int r = 1; r <= rounds; ++r)
        ASTG_LAUNCH(k_x_value<<<xblk((long long)n), XTB, 0, st>>>(d, F, X, oct, til, r));
    unsigned long long assigned = 0;
    cudaMemcpyAsync(&assigned, X.assigned, sizeof assigned, cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return -1;
    if (passes) *passes = rounds;
    return (long long)assigned;
}
size_t extrapolate_scratch_bytes(int S) { return 2 * (size_t)S * 21 + 64; }

}  // namespace astg
