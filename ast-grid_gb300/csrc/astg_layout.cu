// The octree layout and its tilt constraint, built on the device once per handle.
//
// OctreeLayer3 (src/octree_layer3.cpp:7-88): the non-ghost cells of level l are the cells whose
// corner finest cell carries split value l, numbered in raster order; the ghosts of level l are
// the 26-neighbours of those cells whose split value is l - 1 or l + 1, numbered in the order the
// reference discovers them (its non-ghost cells in index order, each visiting its neighbours in
// (a, b, c) loop order, a neighbour taking the next index the first time it is seen).  Both
// numberings are data-parallel here: a flag per cell and a scan for the raster order, and for the
// ghosts the discovery key min over non-ghost neighbours n = g - o_k of index(n) * 26 + k, which is
// unique per (n, k), so marking the keys and scanning the marks yields the discovery order.
//
// constrainOctreeTiltE3 (src/octree_util.cpp:38-169) in its four parts, each in the reference's
// semantics: T-joints (independent per vertex), tilts closed by T-joints (idempotent per target,
// resolved from the first part's state), the ghost copy (OctreeVertexCenteredGrid3::updateGhost,
// src/octree_vertex_centered_grid3.cpp:6-24: levels in ascending order; a ghost fed from the
// coarser level reads that level's value before its own ghosts were copied, a ghost fed from the
// finer level the value after), and half tilts (detected per (vertex, axis) in parallel, applied in
// the reference's (vertex, axis) order by one thread, which also yields the half-tilt list and the
// deduplicated list of tilts they close).  Detection reads a T-joint's size e, which an earlier
// half tilt could only have changed if a half tilt landed on a T-joint; when that happens the whole
// half-tilt part runs in order on one thread instead.
#include <climits>
#include <stdexcept>
#include <string>

#include "astg_launch.h"
#include "astg_sample.cuh"

namespace astg {

namespace {
constexpr int LTB = 256;
inline unsigned lblk(long long n) { return (unsigned)((n + LTB - 1) / LTB); }

void lck(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string("layout: ") + what + ": " + cudaGetErrorString(e));
}
template <class T>
T* lalloc(size_t n, std::vector<void*>& list) {
    void* p = nullptr;
    lck(cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)), "cudaMalloc");
    list.push_back(p);
    return (T*)p;
}

__device__ __forceinline__ void cell_xyz(long long c, int r, int* x, int* y, int* z) {
    *x = (int)(c % r);
    *y = (int)((c / r) % r);
    *z = (int)(c / ((long long)r * r));
}
__device__ __forceinline__ int split_at(const int* split, int res, int l, int x, int y, int z) {
    return split[((size_t)(z << l) * res + (y << l)) * res + (x << l)];
}
}  // namespace

// ------------------------------------------------------------------ OctreeLayer3
__global__ void k_lay_flag(const int* split, int res, int l, int r, int* flag) {
    long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (c >= (long long)r * r * r) return;
    int x, y, z;
    cell_xyz(c, r, &x, &y, &z);
    flag[c] = split_at(split, res, l, x, y, z) == l;
}
__global__ void k_lay_cells(int l, int r, int off, const int* flag, const int* idx, int* brick, int4* lslot) {
    long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (c >= (long long)r * r * r) return;
    if (!flag[c]) {
        brick[c] = -1;
        return;
    }
    int x, y, z;
    cell_xyz(c, r, &x, &y, &z);
    brick[c] = off + idx[c];
    lslot[idx[c]] = make_int4(x, y, z, l);
}
__global__ void k_lay_ghost_key(const int* split, int res, int l, int r, int off, const int* brick, int* mark,
                                int* cellOf) {
    long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (c >= (long long)r * r * r) return;
    int x, y, z;
    cell_xyz(c, r, &x, &y, &z);
    int tv = split_at(split, res, l, x, y, z);
    if (tv != l - 1 && tv != l + 1) return;
    int best = INT_MAX, k = 0;
    for (int a = -1; a <= 1; ++a)
        for (int b = -1; b <= 1; ++b)
            for (int e = -1; e <= 1; ++e) {
                if (a == 0 && b == 0 && e == 0) continue;
                int nx = x - a, ny = y - b, nz = z - e;
                if (nx >= 0 && ny >= 0 && nz >= 0 && nx < r && ny < r && nz < r) {
                    int s = brick[((size_t)nz * r + ny) * r + nx];
                    if (s >= 0) best = min(best, (s - off) * 26 + k);
                }
                ++k;
            }
    if (best == INT_MAX) return;
    mark[best] = 1;
    cellOf[best] = (int)c;
}
__global__ void k_lay_ghosts(const int* split, int res, int l, int r, int off, int n0, long long keys, const int* mark,
                             const int* rank, const int* cellOf, int* brick, int4* lslot) {
    long long key = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (key >= keys || !mark[key]) return;
    int c = cellOf[key];
    int x, y, z;
    cell_xyz(c, r, &x, &y, &z);
    int i = n0 + rank[key];
    brick[c] = off + i;
    int fl = SF_GHOST | (split_at(split, res, l, x, y, z) == l + 1 ? SF_FROM_COARSE : 0);
    lslot[i] = make_int4(x, y, z, l | (fl << 8));
}
// OctreeGridLayout3::levelCoordinate: the finest non-ghost level holding each finest cell
__global__ void k_lay_locate(Dev d, uint8_t* loc) {
    long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (c >= (long long)d.res * d.res * d.res) return;
    int x, y, z;
    cell_xyz(c, d.res, &x, &y, &z);
    uint8_t v = 0xff;
    for (int l = 0; l < d.L; ++l) {
        int s = get(d, l, x >> l, y >> l, z >> l);
        if (s >= 0 && !(slot_f(d, s) & SF_GHOST)) {
            v = (uint8_t)l;
            break;
        }
    }
    loc[c] = v;
}

// ------------------------------------------------------------------ constrainOctreeTiltE3
struct TiltState {
    double* e;
    uint32_t* f;
    int* dir;
};
__device__ __forceinline__ void set_e_zero(TiltState t, int s) {  // TiltENode::setE(0)
    uint32_t v = t.f[s];
    if (v & TF_FIXED) return;
    t.f[s] = (v | TF_CLOSED) & ~TF_LARGEST;
    t.e[s] = 0;
}
// T-joints at level transitions (src/octree_util.cpp:41-73)
__global__ void k_tc_tjoint(Dev d, TiltState t, int* isTj) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.S) return;
    isTj[s] = 0;
    if (slot_f(d, s) & SF_GHOST) return;
    int l = slot_l(d, s), x = slot_x(d, s), y = slot_y(d, s), z = slot_z(d, s);
    int minL = l, maxL = l;
    for (int i = -1; i <= 0; ++i)
        for (int j = -1; j <= 0; ++j)
            for (int k = -1; k <= 0; ++k) {
                int c = get_until(d, l, x + i, y + j, z + k, true);
                if (c < 0) c = get_until(d, l, x + i, y + j, z + k, false);
                // the packed-coordinate test "c > 0" of the reference skips level 0, (0, 0, 0)
                if (c >= 0 && !(slot_l(d, c) == 0 && slot_x(d, c) == 0 && slot_y(d, c) == 0 && slot_z(d, c) == 0)) {
                    minL = min(minL, slot_l(d, c));
                    maxL = max(maxL, slot_l(d, c));
                }
            }
    if (minL < l || (maxL > l && !(x & 1) && !(y & 1) && !(z & 1))) {
        t.f[s] = (t.f[s] | TF_TJOINT | TF_FIXED) & ~TF_CLOSED;
        t.e[s] = d.ldh[minL];
        isTj[s] = 1;
    }
}
// tilts closed by T-joints (:75-96): every target gets the same update whichever T-joint reaches
// it first, and the T-joints themselves are fixed, so the targets are marked, then updated
__global__ void k_tc_closed_by_t_mark(Dev d, TiltState t, int* hit) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.S || (slot_f(d, s) & SF_GHOST) || !(t.f[s] & TF_TJOINT)) return;
    int l = slot_l(d, s), x = slot_x(d, s), y = slot_y(d, s), z = slot_z(d, s);
    if (t.e[s] < d.ldh[l]) {
        l -= 1;
        x *= 2;
        y *= 2;
        z *= 2;
    }
    for (int i = 0; i < 6; ++i) {
        int q = get(d, l, x + OCT_NB[i][0], y + OCT_NB[i][1], z + OCT_NB[i][2]);
        if (q >= 0) hit[q] = 1;
    }
}
__global__ void k_tc_closed_by_t_apply(Dev d, TiltState t, const int* hit) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= d.S || !hit[q]) return;
    set_e_zero(t, q);
    t.f[q] |= TF_FIXED | TF_CLOSED_BY_T;
}
// updateGhost of the tilt-E grid, one level: ghosts fed from the coarser level read `snap` (the
// state before any ghost of this pass was copied), ghosts fed from the finer level the current one
__global__ void k_tc_ghost_copy(Dev d, int l, TiltState t, TiltState snap) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.lG[l]) return;
    int s = d.loff[l] + d.lN[l] + i;
    int x = slot_x(d, s), y = slot_y(d, s), z = slot_z(d, s);
    int src;
    TiltState from = t;
    if (slot_f(d, s) & SF_FROM_COARSE) {
        if ((x & 1) || (y & 1) || (z & 1)) return;
        src = req(d, l + 1, x >> 1, y >> 1, z >> 1);
        from = snap;
    } else {
        src = req(d, l - 1, x << 1, y << 1, z << 1);
    }
    t.e[s] = from.e[src];
    t.f[s] = from.f[src];
    t.dir[s] = from.dir[src];
}
// half tilts on coarse faces surrounded by T-joints (:98-169): the half tilt (hs), its direction
// and the tilt it closes (ts) for T-joint s and axis; false when there is none
__device__ bool tc_half_event(const Dev& d, TiltState t, int s, int axis, int* hs, int* ts, int* dir) {
    int l = slot_l(d, s);
    int coarse = t.e[s] < d.ldh[l] ? 1 : 0;
    int sx = slot_x(d, s), sy = slot_y(d, s), sz = slot_z(d, s);
    int ci[3] = {coarse ? sx : sx >> 1, coarse ? sy : sy >> 1, coarse ? sz : sz >> 1};
    int lc = l + (1 - coarse);
    if (ci[axis] == 0 || ci[axis] == d.lres[l - coarse] - 1) return false;
    bool flag = true;
    for (int i = 0; i <= 1 && flag; ++i)
        for (int j = 0; j <= 1 && flag; ++j) {
            if (i == 0 && j == 0) continue;
            int id[3] = {ci[0], ci[1], ci[2]};
            id[(axis + 1) % 3] += i;
            id[(axis + 2) % 3] += j;
            int c = lc < d.L ? get_until(d, lc, id[0], id[1], id[2], true) : -1;
            if (c < 0 && lc < d.L) c = get_until(d, lc, id[0], id[1], id[2], false);
            if (c < 0 || !(t.f[c] & TF_TJOINT)) flag = false;
        }
    if (flag) {
        int nb[3] = {ci[0], ci[1], ci[2]};
        nb[axis] -= 1;
        int c = lc < d.L ? get_until(d, lc, ci[0], ci[1], ci[2], true) : -1;
        int c1 = lc < d.L ? get_until(d, lc, nb[0], nb[1], nb[2], true) : -1;
        int lvc = c >= 0 ? slot_l(d, c) : 15;  // UNPACK_LEVEL3(-1)
        if (c1 < 0 || lvc == slot_l(d, c1)) flag = false;
    }
    if (!flag) return false;
    int id[3] = {ci[0] * 2, ci[1] * 2, ci[2] * 2};
    id[(axis + 1) % 3] += 1;
    id[(axis + 2) % 3] += 1;
    int hl = l - coarse;
    *hs = get(d, hl, id[0], id[1], id[2]);
    if (*hs < 0) return false;
    *dir = axis + (coarse ? 3 : 0);
    int tp[3] = {id[0], id[1], id[2]};
    tp[axis] += *dir < 3 ? 1 : -1;
    *ts = req(d, hl, tp[0], tp[1], tp[2]);
    return true;
}
__device__ void tc_half_apply(const Dev& d, TiltState t, int hs, int ts, int dir, int* half, int* nHalf, int* cbh,
                              int* nCbh, int* seen) {
    t.f[hs] |= TF_CLOSED | TF_HALF | TF_FIXED;
    t.dir[hs] = dir;
    t.e[hs] = d.ldh[slot_l(d, hs)];
    half[(*nHalf)++] = hs;
    if (!seen[ts]) {
        seen[ts] = 1;
        cbh[(*nCbh)++] = ts;
    }
    set_e_zero(t, ts);
    t.f[ts] |= TF_CLOSED_BY_T | TF_FIXED;
    t.dir[ts] = -1;
}
__global__ void k_tc_half_detect(Dev d, TiltState t, int* mark, int* evHs, int* evTs, int* evDir) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.S) return;
    for (int a = 0; a < 3; ++a) mark[3 * s + a] = 0;
    if ((slot_f(d, s) & SF_GHOST) || !(t.f[s] & TF_TJOINT)) return;
    for (int a = 0; a < 3; ++a) {
        int hs, ts, dir;
        if (!tc_half_event(d, t, s, a, &hs, &ts, &dir)) continue;
        mark[3 * s + a] = 1;
        evHs[3 * s + a] = hs;
        evTs[3 * s + a] = ts;
        evDir[3 * s + a] = dir;
    }
}
// one thread, the detected events (keys 3 * vertex + axis, ascending); counts[0] = half tilts,
// [1] = closed tilts, [2] = 1 when a half tilt landed on a T-joint (the parallel detection may then
// differ from the reference's order)
__global__ void k_tc_half_apply(Dev d, TiltState t, const int* nEv, const int* ev, const int* evHs, const int* evTs,
                                const int* evDir, int* half, int* cbh, int* seen, int* counts) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    int nh = 0, nc = 0, clash = 0;
    for (int i = 0; i < *nEv; ++i) {
        int k = ev[i];
        if (t.f[evHs[k]] & TF_TJOINT) clash = 1;
        tc_half_apply(d, t, evHs[k], evTs[k], evDir[k], half, &nh, cbh, &nc, seen);
    }
    counts[0] = nh;
    counts[1] = nc;
    counts[2] = clash;
}
// the same part strictly in order, for layouts where a half tilt lands on a T-joint
__global__ void k_tc_half_serial(Dev d, TiltState t, int* half, int* cbh, int* seen, int* counts) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    int nh = 0, nc = 0;
    for (int s = 0; s < d.S; ++s) {
        if ((slot_f(d, s) & SF_GHOST) || !(t.f[s] & TF_TJOINT)) continue;
        for (int a = 0; a < 3; ++a) {
            int hs, ts, dir;
            if (tc_half_event(d, t, s, a, &hs, &ts, &dir)) tc_half_apply(d, t, hs, ts, dir, half, &nh, cbh, &nc, seen);
        }
    }
    counts[0] = nh;
    counts[1] = nc;
    counts[2] = 0;
}
__global__ void k_tc_init(int S, TiltState t) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    t.e[s] = 0;
    t.f[s] = TF_CLOSED;
    t.dir[s] = 0;
}
__global__ void k_compact(long long n, const int* mark, const int* pos, int* out) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n && mark[i]) out[pos[i]] = (int)i;
}

void build_layout_device(const int32_t* hsplit, int res, int L, const double* ldh, std::vector<void*>& keep,
                         LayoutBuild& out, cudaStream_t st) {
    struct Free {
        std::vector<void*>& v;
        ~Free() {
            for (void* p : v) cudaFree(p);
        }
    };
    std::vector<void*> tmp;
    Free freeTmp{tmp};
    const long long cells = (long long)res * res * res;
    int* split = lalloc<int>(cells, tmp);
    lck(cudaMemcpyAsync(split, hsplit, sizeof(int) * cells, cudaMemcpyHostToDevice, st), "split map");
    int* flag = lalloc<int>(cells, tmp);
    int* idx = lalloc<int>(cells, tmp);
    int4* lslot = lalloc<int4>(cells, tmp);
    int* bsum = lalloc<int>((cells * 26 + 1023) / 1024 + 1, tmp);
    int* total = lalloc<int>(2, tmp);
    Dev d{};
    d.L = L;
    d.res = res;
    d.dx = ldh[0];
    out.L = L;
    out.res = res;
    out.hslot.clear();
    out.hbrick.assign(L, {});
    int off = 0;
    for (int l = 0; l < L; ++l) {
        const int r = res >> l;
        const long long rc = (long long)r * r * r;
        int* brick = lalloc<int>(rc, keep);
        d.lres[l] = r;
        d.ldh[l] = ldh[l];
        ASTG_LAUNCH(k_lay_flag<<<lblk(rc), LTB, 0, st>>>(split, res, l, r, flag));
        exclusive_scan(flag, idx, bsum, total, rc, st);
        int n = 0;
        lck(cudaMemcpyAsync(&n, total, sizeof(int), cudaMemcpyDeviceToHost, st), "count");
        lck(cudaStreamSynchronize(st), "count");
        // the fixed reduction tree folds at most 2048 chunk partials in one block (this also keeps
        // the discovery keys, index * 26 + k, inside int)
        if (2LL * (off + n) > 2048LL * 2048LL) throw std::runtime_error("layout: too many cells for the reduction tree");
        ASTG_LAUNCH(k_lay_cells<<<lblk(rc), LTB, 0, st>>>(l, r, off, flag, idx, brick, lslot));
        long long keys = (long long)n * 26;
        int g = 0;
        std::vector<void*> lvl;
        Free freeLvl{lvl};
        if (keys > 0) {
            int* mark = lalloc<int>(keys, lvl);
            int* rank = lalloc<int>(keys, lvl);
            int* cellOf = lalloc<int>(keys, lvl);
            lck(cudaMemsetAsync(mark, 0, sizeof(int) * keys, st), "memset");
            ASTG_LAUNCH(k_lay_ghost_key<<<lblk(rc), LTB, 0, st>>>(split, res, l, r, off, brick, mark, cellOf));
            exclusive_scan(mark, rank, bsum, total, keys, st);
            lck(cudaMemcpyAsync(&g, total, sizeof(int), cudaMemcpyDeviceToHost, st), "count");
            ASTG_LAUNCH(k_lay_ghosts<<<lblk(keys), LTB, 0, st>>>(split, res, l, r, off, n, keys, mark, rank, cellOf, brick,
                                                                 lslot));
        }
        lck(cudaStreamSynchronize(st), "ghosts");
        out.lres[l] = r;
        out.loff[l] = off;
        out.lN[l] = n;
        out.lG[l] = g;
        size_t base = out.hslot.size();
        out.hslot.resize(base + n + g);
        lck(cudaMemcpyAsync(out.hslot.data() + base, lslot, sizeof(int4) * (n + g), cudaMemcpyDeviceToHost, st), "slots");
        out.hbrick[l].resize(rc);
        lck(cudaMemcpyAsync(out.hbrick[l].data(), brick, sizeof(int) * rc, cudaMemcpyDeviceToHost, st), "brick");
        out.brick[l] = brick;
        d.brick[l] = brick;
        d.loff[l] = off;
        d.lN[l] = n;
        d.lG[l] = g;
        off += n + g;
        // the fixed reduction tree folds at most 2048 chunk partials in one block
        if (2LL * off > 2048LL * 2048LL) throw std::runtime_error("layout: too many cells for the reduction tree");
    }
    const int S = off;
    out.S = S;
    d.S = S;
    int4* slot = lalloc<int4>(S, keep);
    lck(cudaMemcpyAsync(slot, out.hslot.data(), sizeof(int4) * S, cudaMemcpyHostToDevice, st), "slots");
    d.slot = slot;
    out.slot = slot;
    int* status = lalloc<int>(1, tmp);
    lck(cudaMemsetAsync(status, 0, sizeof(int), st), "memset");
    d.status = status;
    uint8_t* loc = lalloc<uint8_t>(cells, keep);
    ASTG_LAUNCH(k_lay_locate<<<lblk(cells), LTB, 0, st>>>(d, loc));
    out.locate = loc;

    // constrainOctreeTiltE3
    TiltState t{lalloc<double>(S, tmp), lalloc<uint32_t>(S, tmp), lalloc<int>(S, tmp)};
    TiltState snap{lalloc<double>(S, tmp), lalloc<uint32_t>(S, tmp), lalloc<int>(S, tmp)};
    auto snapshot = [&] {
        lck(cudaMemcpyAsync(snap.e, t.e, sizeof(double) * S, cudaMemcpyDeviceToDevice, st), "snapshot");
        lck(cudaMemcpyAsync(snap.f, t.f, sizeof(uint32_t) * S, cudaMemcpyDeviceToDevice, st), "snapshot");
        lck(cudaMemcpyAsync(snap.dir, t.dir, sizeof(int) * S, cudaMemcpyDeviceToDevice, st), "snapshot");
    };
    auto ghost_copy = [&] {
        snapshot();
        for (int l = 0; l < L; ++l)
            if (out.lG[l]) ASTG_LAUNCH(k_tc_ghost_copy<<<lblk(out.lG[l]), LTB, 0, st>>>(d, l, t, snap));
    };
    ASTG_LAUNCH(k_tc_init<<<lblk(S), LTB, 0, st>>>(S, t));
    int* isTj = lalloc<int>(S, tmp);
    int* tjPos = lalloc<int>(S, tmp);
    int* tjList = lalloc<int>(S, tmp);
    ASTG_LAUNCH(k_tc_tjoint<<<lblk(S), LTB, 0, st>>>(d, t, isTj));
    exclusive_scan(isTj, tjPos, bsum, total, S, st);
    ASTG_LAUNCH(k_compact<<<lblk(S), LTB, 0, st>>>(S, isTj, tjPos, tjList));
    int nTj = 0;
    lck(cudaMemcpyAsync(&nTj, total, sizeof(int), cudaMemcpyDeviceToHost, st), "count");
    int* hit = lalloc<int>(S, tmp);
    lck(cudaMemsetAsync(hit, 0, sizeof(int) * S, st), "memset");
    ASTG_LAUNCH(k_tc_closed_by_t_mark<<<lblk(S), LTB, 0, st>>>(d, t, hit));
    ASTG_LAUNCH(k_tc_closed_by_t_apply<<<lblk(S), LTB, 0, st>>>(d, t, hit));
    ghost_copy();
    // half tilts: detect in parallel on a copy, apply in order
    const long long keys = 3LL * S;
    int* mark = lalloc<int>(keys, tmp);
    int* evHs = lalloc<int>(keys, tmp);
    int* evTs = lalloc<int>(keys, tmp);
    int* evDir = lalloc<int>(keys, tmp);
    int* half = lalloc<int>(keys, tmp);
    int* cbh = lalloc<int>(keys, tmp);
    int* seen = lalloc<int>(S, tmp);
    int* counts = lalloc<int>(3, tmp);
    lck(cudaMemsetAsync(seen, 0, sizeof(int) * S, st), "memset");
    TiltState before{lalloc<double>(S, tmp), lalloc<uint32_t>(S, tmp), lalloc<int>(S, tmp)};
    lck(cudaMemcpyAsync(before.e, t.e, sizeof(double) * S, cudaMemcpyDeviceToDevice, st), "copy");
    lck(cudaMemcpyAsync(before.f, t.f, sizeof(uint32_t) * S, cudaMemcpyDeviceToDevice, st), "copy");
    lck(cudaMemcpyAsync(before.dir, t.dir, sizeof(int) * S, cudaMemcpyDeviceToDevice, st), "copy");
    int* evPos = lalloc<int>(keys, tmp);
    int* ev = lalloc<int>(keys, tmp);
    ASTG_LAUNCH(k_tc_half_detect<<<lblk(S), LTB, 0, st>>>(d, t, mark, evHs, evTs, evDir));
    exclusive_scan(mark, evPos, bsum, total, keys, st);
    ASTG_LAUNCH(k_compact<<<lblk(keys), LTB, 0, st>>>(keys, mark, evPos, ev));
    ASTG_LAUNCH(k_tc_half_apply<<<1, 1, 0, st>>>(d, t, total, ev, evHs, evTs, evDir, half, cbh, seen, counts));
    int cnt[3] = {0, 0, 0};
    lck(cudaMemcpyAsync(cnt, counts, sizeof(cnt), cudaMemcpyDeviceToHost, st), "counts");
    lck(cudaStreamSynchronize(st), "half tilts");
    if (cnt[2]) {  // a half tilt on a T-joint: redo the part strictly in order from the state before it
        lck(cudaMemcpyAsync(t.e, before.e, sizeof(double) * S, cudaMemcpyDeviceToDevice, st), "copy");
        lck(cudaMemcpyAsync(t.f, before.f, sizeof(uint32_t) * S, cudaMemcpyDeviceToDevice, st), "copy");
        lck(cudaMemcpyAsync(t.dir, before.dir, sizeof(int) * S, cudaMemcpyDeviceToDevice, st), "copy");
        lck(cudaMemsetAsync(seen, 0, sizeof(int) * S, st), "memset");
        ASTG_LAUNCH(k_tc_half_serial<<<1, 1, 0, st>>>(d, t, half, cbh, seen, counts));
        lck(cudaMemcpyAsync(cnt, counts, sizeof(cnt), cudaMemcpyDeviceToHost, st), "counts");
        lck(cudaStreamSynchronize(st), "half tilts");
    }
    ghost_copy();
    out.te.resize(S);
    out.tf.resize(S);
    out.tdir.resize(S);
    out.tj.resize(nTj);
    out.half.resize(cnt[0]);
    out.cbh.resize(cnt[1]);
    lck(cudaMemcpyAsync(out.te.data(), t.e, sizeof(double) * S, cudaMemcpyDeviceToHost, st), "tilts");
    lck(cudaMemcpyAsync(out.tf.data(), t.f, sizeof(uint32_t) * S, cudaMemcpyDeviceToHost, st), "tilts");
    lck(cudaMemcpyAsync(out.tdir.data(), t.dir, sizeof(int) * S, cudaMemcpyDeviceToHost, st), "tilts");
    if (nTj) lck(cudaMemcpyAsync(out.tj.data(), tjList, sizeof(int) * nTj, cudaMemcpyDeviceToHost, st), "lists");
    if (cnt[0]) lck(cudaMemcpyAsync(out.half.data(), half, sizeof(int) * cnt[0], cudaMemcpyDeviceToHost, st), "lists");
    if (cnt[1]) lck(cudaMemcpyAsync(out.cbh.data(), cbh, sizeof(int) * cnt[1], cudaMemcpyDeviceToHost, st), "lists");
    int stat = 0;
    lck(cudaMemcpyAsync(&stat, status, sizeof(int), cudaMemcpyDeviceToHost, st), "status");
    lck(cudaStreamSynchronize(st), "layout");
    lck(cudaGetLastError(), "launch");
    if (stat == DS_MISSING_NODE) throw std::runtime_error("layout: the tilt constraint reads a node the layout does not hold");
    if (stat != 0) throw std::runtime_error("layout: device status " + std::to_string(stat));
}

}  // namespace astg
