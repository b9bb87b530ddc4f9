// Host-side declarations of the kernel launchers (implemented in astg_step.cu and astg_pcg.cu).
#pragma once
#include <cuda_runtime.h>
#include <atomic>
#include <vector>
#include "astg_device.cuh"

namespace astg {

// number of kernels this library has launched (all handles of the process; calls on several host
// threads may count at once)
extern std::atomic<long long> g_launches;
// the calling thread's launches (a graph capture counts the kernels of its own thread only)
extern thread_local long long t_launches;
inline void count_launch() {
    g_launches.fetch_add(1, std::memory_order_relaxed);
    ++t_launches;
}
#define ASTG_LAUNCH(...)                                                       \
    do {                                                                       \
        ::astg::count_launch();                                                \
        __VA_ARGS__;                                                           \
    } while (0)

// optional CUDA-event timing of the PCG's kernels: 0 forward sweep, 1 backward sweep,
// 2 SpMV + dot, 3 MIC(0) factorisation
constexpr int KPROF_KINDS = 4;
struct KProf {
    bool on = false;
    double ms[KPROF_KINDS] = {0, 0, 0, 0};
    long long count[KPROF_KINDS] = {0, 0, 0, 0};
    cudaEvent_t ev[2 * 128];  // pairs recorded by direct launches since the last drain
    int kind[128];
    int used = 0;
    cudaEvent_t gev[2 * 64];  // pairs recorded by the nodes of the current PCG batch graph
    int gkind[64];
    int gused = 0;
    bool created = false;
    KProf() = default;
    KProf(const KProf&) = delete;
    KProf& operator=(const KProf&) = delete;
    ~KProf() {
        if (!created) return;
        for (auto& e : ev) cudaEventDestroy(e);
        for (auto& e : gev) cudaEventDestroy(e);
    }
};

constexpr int ROW_W = 32;   // padded row width during assembly (rows have at most ~21 entries)
constexpr int PC_MAXE = 8;  // factor entries per row held in the padded records
constexpr int REF_MAX_WORKERS = 256;  // worker count of the reference-order mean temperature

// scalars of the PCG kept on the device
enum { SC_RESID0 = 0, SC_TOL, SC_RHO, SC_RESID, SC_ALPHA, SC_BETA, SC_COUNT };
enum { ISC_ITERS = 0, ISC_CONVERGED, ISC_COUNT };

// Projection workspace (device pointers unless noted); sized for S + H rows.
struct Proj {
    int* cnt;      // S
    int* base;     // S
    int* bsum;     // scan block sums
    int* n0;       // device scalars
    int* nDof;
    int* nnz;
    int* pO;       // S
    int* pT;       // S
    int* rowCnt;   // rows
    int* rowPtr;   // rows + 1
    int* padCol;   // rows * ROW_W
    double* padVal;
    double* bRaw;  // rows
    int* col;      // rows * ROW_W (CSR, compacted)
    double* val;
    int* diagPos;  // rows
    int* tpos;     // CSR position of the mirrored entry
    double* b;     // rows
    // MIC(0)
    double* Lv;      // CSR-aligned factor values (upper entries = columns of L)
    double* invdiag;
    double* adiag;
    int* ready;      // rows, epoch flags
    // pattern-only plan of the factorisation: for lower entry q of row j (column k), one code per
    // upper entry of row k (k's column of L), in order: 0 nothing, 1 missing, 2 diagonal,
    // (bb - first upper entry of row j) << 2 | 3 matched entry bb
    int* planPtr;    // nnz capacity + 1
    int* plan;
    long long planCap;
    int* planTotal;  // device scalar
    int* counter;
    int sweepBlocks;
    // level schedule of the lower factor (rows grouped by dependency depth), rebuilt per solve
    int* level;      // rows: 1 + max level of the rows it depends on
    int* levelCnt;   // rows + 1
    int* levelPtr;   // rows + 1
    int* nLevels;    // device scalar
    int* fill;       // rows + 1
    int* perm;       // rows in level order
    int* cntF;       // rows: lower entries per level-ordered row
    int* cntB;       // rows: upper entries
    int* fptr;       // rows + 1
    int* bptr;
    int* fcol;       // nnz: level-ordered lower entries (column, factor value)
    double* fval;
    int* bcol;       // nnz: level-ordered upper entries
    double* bval;
    int clusterSize; // CTAs per cluster of the level-synchronous sweeps (0: sync-free sweeps)
    int pcCluster;   // CTAs per cluster of the fused DSMEM preconditioner (0: not available)
    int pcActive;    // the current solve uses it (its vector fits in the cluster's shared memory)
    size_t pcSmemMax;  // largest dynamic shared memory per CTA it may use
    // padded level-ordered records for the fused preconditioner (entry e of row p at e * rowsCap + p)
    int rowsCap;
    int* pos;        // rows: level position of each row (inverse of perm)
    int* lcntF;      // rows: lower entries of the row at level position p
    int* lcntB;
    double* linvd;   // rows: pivot reciprocal in level order
    double* rl;      // rows: right-hand side of the preconditioner in level order
    // barrier-free form: row j is computed by, and stored in, CTA (j >> lgB) mod CS; each CTA walks
    // its own rows sorted by level (positions [ownStart[c], ownStart[c + 1]))
    int pcAsync;     // 1: barrier-free fused preconditioner, 0: one cluster barrier per level
    int pcLgBlock;   // log2 of the rows per ownership block: row j belongs to CTA (j >> lgB) mod CS
    int* chunk;      // device scalar: shared-memory slots per CTA
    int* ownStart;   // CS + 1: first position of each CTA's rows
    int* lself;      // rows: local (shared-memory) index of the row at each position
    double* yl;      // rows: forward-sweep result at each position
    int* ownCnt;     // pcCluster * (rows + 1): rows per (owner CTA, level)
    int* ownPtr;
    int* ownFill;
    int* fcolP;      // PC_MAXE * rowsCap
    double* fvalP;
    int* bcolP;
    double* bvalP;
    // mixed precision: FP32 copies of the matrix and of the factor records, FP32 inner vectors
    int pcActive32;   // the current solve can run the FP32 barrier-free preconditioner
    size_t pcSmem32;  // its dynamic shared memory per CTA
    float* val32;     // rowsCap * ROW_W
    float* fvalP32;   // PC_MAXE * rowsCap
    float* bvalP32;
    float* linvd32;
    float* rl32;
    float* yl32;
    float* fval32;    // compact entries
    float* bval32;
    float* e32;       // inner correction
    float* r32;       // inner residual
    float* s32;
    float* z32;
    float* q32;
    size_t pcSmem;   // its dynamic shared memory per CTA in the current solve
    // reduction order: 0 the library's (fixed tree, fused sweep updates), 1 the reference's (Eigen
    // dot order, separate multiply and subtract in the sweeps)
    int refOrder;
    int unfused;     // sweep updates as a product and a subtraction
    // PCG
    double* x;
    double* r;
    double* s;
    double* z;
    double* part;    // chunk partials
    double* sc;      // SC_COUNT
    int* isc;        // ISC_COUNT
    unsigned long long* amax;
    int* done;
    int* hostDone;   // pinned host
    int tolAbsolute; // 1: the PCG stops at |r|_inf <= tol (the std::vector PCGSolver::solve overload,
                     // include/pcgsolver/pcg_solver.h:302-363); 0: at tol * |b|_inf
    // wavefront form of the MIC(0) sweeps on a uniform 2-D grid (cells x + y * wnx first, then one
    // row per open tilt), astg2d.cu.  Per cell, diagonal-major (cell (x, y) at j = x + (x + y) * wnx,
    // wnx * (wnx + wny - 1) slots), two double2 each:
    // wRecF = (L to the cell below, L to the cell on the left), (pivot reciprocal, flags);
    // wRecB = (L from the cell on the right, L from the cell above), (pivot reciprocal, flags); the
    // flags (an integer in the bits of a double) are 1 below, 2 left, 4 right, 8 above and 16 << k
    // for corner tilt k of (x, y), (x + 1, y), (x, y + 1), (x + 1, y + 1).  wTt / wTl: those tilts'
    // rows and entries (4 per cell); wTc / wTv: each tilt row's cells and entries, ascending.
    // wR: the residual of the cells in the same order (written by the PCG's update), wZ: the
    // sweeps' result of the cells in that order.
    int wave;        // 1: precond runs the wavefront kernel
    int wnx, wny;
    double2* wRecF;
    double2* wRecB;
    double* wR;
    double* wZ;
    int* wTt;
    double* wTl;
    int* wTc;
    double* wTv;
    int* wStatus;    // device status word for wait time-outs
};

void launch_source(const Dev& d, const Fields& F, cudaStream_t st);
void launch_scalar_ghost(const Dev& d, double* oct, double* til, const double* te, const uint32_t* tf, cudaStream_t st);
void launch_dual_ghost(const Dev& d, const Fields& F, cudaStream_t st);
void launch_mean_temperature(const Dev& d, const double* hO, double* parts, const int* partOffDev,
                             const int* partOffHost, double* amb, cudaStream_t st);
// mean temperature over a caller's device array with its scratch in a static device array
constexpr int AMB_CHUNK = 2048;                 // elements per partial of the fixed reduction tree
constexpr int AMB_MAX_LEVEL_PARTIALS = 2048;    // partials of one level folded by one block
constexpr int NOALLOC_MAX_PARTIALS = 8192;      // 64 KiB of static scratch per device
constexpr int NOALLOC_MAX_DEVICES = 64;
struct LevelSpans {
    int L;
    long long off[MAXL + 1];  // first slot of each level; off[L] = all slots
    int partOff[MAXL + 1];    // first partial of each level
};
cudaError_t launch_mean_temperature_static(const double* heat, const LevelSpans& sp, double* amb, cudaStream_t st);
// the same in the reference's order (BLAS::sum's per-worker slices, `workers` workers)
void launch_mean_temperature_ref(const Dev& d, const double* hO, int workers, double* amb, cudaStream_t st);
// largest positive MAC face value (0 when none) into *out (which must start at 0)
void launch_max_face(const Dev& d, const double* mac, unsigned long long* out, cudaStream_t st);
// collider (astg_collider.cu): per-slot bits and cut-cell weights once per collider; the per-step
// wipe and inside-solid constraints (before: 3 * S doubles of scratch for the MAC projection)
// OctreeLayer3 and constrainOctreeTiltE3 built on the device (astg_layout.cu).  Device arrays named
// here are allocated into the caller's list (freed with it); the host copies feed the host-side
// set-up that follows (tables, weights, initial velocity).
struct LayoutBuild {
    int L = 0, res = 0, S = 0;
    int lres[MAXL] = {}, loff[MAXL] = {}, lN[MAXL] = {}, lG[MAXL] = {};
    int* brick[MAXL] = {};   // device, per level res_l^3 slots or -1
    int4* slot = nullptr;    // device, S
    uint8_t* locate = nullptr;  // device, res^3: finest non-ghost level of each finest cell
    std::vector<int4> hslot;
    std::vector<std::vector<int>> hbrick;
    std::vector<double> te;  // tilt-E size, flags and half direction after the constraint
    std::vector<uint32_t> tf;
    std::vector<int> tdir;
    std::vector<int> half, tj, cbh;
};
void build_layout_device(const int32_t* split, int res, int L, const double* ldh, std::vector<void*>& keep,
                         LayoutBuild& out, cudaStream_t st);
// out = exclusive scan of in[0..n), *total = the sum; bsum holds ceil(n / 1024) ints
void exclusive_scan(const int* in, int* out, int* bsum, int* total, long long n, cudaStream_t st);

// refineSplitMapByObstacleSdf on device arrays; the launch's own error, the thread's error state untouched
cudaError_t launch_refine_split_map(int32_t* split, int res, int level, const double* sdf, double lo, double hi,
                                    cudaStream_t st);
// the SDF grid of a sphere collider at the finest cell centres (res^3 doubles)
void launch_collider_sphere_sdf(int res, double cx, double cy, double cz, double r, double* sdf, cudaStream_t st);
void launch_collider_setup(const Dev& d, const int* halfDir, uint16_t* mask, double* wMac, double* wTilt,
                           cudaStream_t st);
void launch_collider_wipe(const Dev& d, const Fields& F, cudaStream_t st);
void launch_collider_mac(const Dev& d, const Fields& F, double* before, cudaStream_t st);
void launch_collider_tilt(const Dev& d, const Fields& F, cudaStream_t st);
void launch_collider_dual(const Dev& d, const Fields& F, cudaStream_t st);
void launch_walls(const Dev& d, double* mac, cudaStream_t st);
// Fields::corrT for the velocity F (3 * S doubles)
void launch_tilt_corr(const Dev& d, const Fields& F, double* corr, cudaStream_t st);
void launch_dual_update(const Dev& d, const Fields& F, cudaStream_t st);
void launch_force(const Dev& d, const Fields& F, const uint8_t* open, const double* amb, double dt, cudaStream_t st);
void launch_walls_and_ghost(const Dev& d, const Fields& F, const uint8_t* lastWriter, cudaStream_t st);
void launch_velocity_ghost(const Dev& d, const Fields& F, const uint8_t* lastWriter, cudaStream_t st);
void launch_dof_numbering(const Dev& d, const uint8_t* open, Proj& P, cudaStream_t st);
void launch_assemble(const Dev& d, const Fields& F, const uint8_t* open, Proj& P, const int* hoPtr, const int* hoIdx,
                     double dt, cudaStream_t st);
// owner: the owner-major walk of the barrier-free preconditioner, else the level order
void launch_level_schedule(const Dev& d, Proj& P, bool owner, cudaStream_t st);
void launch_external_system(const Dev& d, Proj& P, int rows, cudaStream_t st);
// padded rows (rowCnt, padCol, padVal, bRaw over maxRows rows, *nDof set) -> CSR with b = bRaw *
// scale, diagonal positions and mirrored-entry positions
void launch_rows_to_csr(const Dev& d, Proj& P, int maxRows, double scale, cudaStream_t st);
// out = exclusive scan of in[0..n), *total = its sum; bsum holds ceil(n / 1024) + 1 ints
void launch_exclusive_scan(const int* in, int* out, int* bsum, int* total, long long n, cudaStream_t st);
// the row-sized projection workspace (everything but the per-slot numbering arrays cnt, base, pO,
// pT) for `rows` rows on `device`, zeroed on `st`; each allocation is appended to `allocs`, which the
// caller frees with cudaFree (and J.hostDone with cudaFreeHost).  Throws std::runtime_error.
void proj_alloc(Proj& J, long long rows, int device, cudaStream_t st, std::vector<void*>& allocs);
int choose_cluster_size(int device);
// cluster size (16 or 8) for the fused preconditioner (barrier-free form when async), or 0
int choose_dsmem_cluster(bool async, size_t* smemMax);
// per solve: whether the fused preconditioner holds a vector of n rows (sets pcActive, pcSmem)
void select_preconditioner(Proj& P, int n);
extern cudaError_t g_cluster_error;  // last failed cluster launch (cudaSuccess if none)
void launch_factor(const Dev& d, Proj& P, double omega, double minDiag, int& epoch, cudaStream_t st, KProf* prof);
// the wavefront preconditioner z = (L L^T)^-1 r of a uniform 2-D system (Proj::wave), astg2d.cu
void launch_precond_wave(const Proj& P, const double* r, double* z, cudaStream_t st);
int launch_pcg_fp64(const Dev& d, Proj& P, double tolFactor, int maxIter, int& epoch, int batch, cudaStream_t st,
                    KProf* prof);
// mixed-precision PCG (FP32 inner PCG inside FP64 defect correction); returns the outer cycles, or
// -1 when the FP32 preconditioner is not available for this solve (nothing was run)
int launch_pcg_mixed(const Dev& d, Proj& P, double tolFactor, int maxIter, int batch, cudaStream_t st, KProf* prof);
// clusters of the barrier-free preconditioner that fit on the device at once (1..8)
int precond_concurrency(const Proj& P, bool fp32);
void launch_pressure_update(const Dev& d, const Fields& F, const uint8_t* open, const int* pO, const int* pT,
                            const double* p, double dt, cudaStream_t st);
void launch_dual(const Dev& d, const Fields& F, cudaStream_t st);
void launch_adjust(const Dev& d, const Fields& cur, const Fields& nxt, uint8_t* open, uint8_t* fixedf, double dt,
                   cudaStream_t st);
void launch_tilt_e_ghost(const Dev& d, double* te, uint32_t* tf, cudaStream_t st);
void launch_advect_scalars(const Dev& d, const Fields& cur, const Fields& nxt, const uint8_t* open, double dt,
                           cudaStream_t st);
void launch_advect_velocity(const Dev& d, const Fields& cur, const Fields& nxt, double dt, cudaStream_t st);
void launch_decay(const Dev& d, const Fields& F, cudaStream_t st);
// FmmLevelSetSolver3::extrapolate of (oct, til) in place from a res^3 signed distance grid on the
// device; scratch holds extrapolate_scratch_bytes(S); returns the nodes assigned (-1: CUDA error)
size_t extrapolate_scratch_bytes(int S);
long long launch_extrapolate(const Dev& d, const Fields& F, double* oct, double* til, const double* sdf, int sres,
                             double offset, double maxFactor, void* scratch, int* passes, cudaStream_t st);

// ---------------------------------------------------------------- adjoint (astg_adjoint.cu)
// Transposes of the step's stages with the topology frozen.  F supplies the frozen tilt-E state
// (te, tf) and, for the advection, the field values of the stage's input state; G holds
// cotangents in the Fields layout and is updated in place from the cotangent of the stage's output
// to that of its input.
cudaError_t launch_adj_probe(const Dev& d, const Fields& F, int what, int n, const double* pos, double* out, cudaStream_t st);
void launch_adj_owners(const Dev& d, const double* te, int* ownJ, int* ownH, cudaStream_t st);
void launch_adj_source(const Dev& d, const Fields& G, double* gsO, double* gsT, cudaStream_t st);
void launch_adj_scalar_ghost(const Dev& d, double* go, double* gt, const double* te, const uint32_t* tf, const int* ownJ,
                             const int* ownH, cudaStream_t st);
void launch_adj_force(const Dev& d, const Fields& F, const Fields& G, const uint8_t* open, double dt, double* gamb,
                      double invCount, cudaStream_t st);
void launch_adj_walls_and_ghost(const Dev& d, const Fields& F, const Fields& G, const uint8_t* lastWriter, cudaStream_t st);
void launch_adj_pressure_update(const Dev& d, const Fields& F, const Fields& G, const uint8_t* open, const int* pO,
                                const int* pT, double* gp, double dt, cudaStream_t st);
void launch_adj_rhs(const Dev& d, const Fields& F, const Fields& G, const uint8_t* open, const Proj& P, const int* hoPtr,
                    const int* hoIdx, const double* lam, double scale, cudaStream_t st);
void launch_adj_dual(const Dev& d, const Fields& F, const Fields& G, const int* ownJ, const int* ownH, cudaStream_t st);
// GN: cotangent of the state after the step (consumed); GC: cotangent of the advected-from state C
void launch_adj_advect(const Dev& d, const Fields& C, const Fields& GC, const Fields& GN, const uint8_t* open, double dt,
                       const int* ownJ, const int* ownH, cudaStream_t st);

}  // namespace astg
