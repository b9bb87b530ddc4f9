// Pressure projection on the GPU: DOF numbering, Laplacian assembly, MIC(0) factorisation and
// preconditioned CG (FP64 and mixed precision), plus the mean-temperature reduction.
//
// Determinism.  Every floating-point reduction uses one fixed tree: chunks of 2048 elements, 256
// lanes per chunk, lane t adds elements t, t+256, ..., t+1792 of its chunk in order starting from
// 0.0, the lanes are folded by halving strides (t += t + s for s = 128 ... 1) and the chunk partials
// are reduced by the same rule.  The CPU oracle implements the same tree, so the FP64 solve is
// reproducible bit for bit.  Matrix rows are summed sequentially in column order, and the
// triangular sweeps and the factorisation apply their updates in the reference's order.  Every
// product the PCG accumulates is one fused multiply-add (one rounding instead of two; the
// oracle's library-order mode does the same): each sweep update z_i -= L_ij z_j as
// fma(-L_ij, z_j, z_i), each CSR row term, each dot-product lane term and the vector updates.
// FP64 issue is the scarce resource on this part, and the fused form halves it (sweeps: measured
// 0.58 -> 0.46 ms per application at the 256^3-equivalent size).
//
// Reference order (astg_set_reduction_order, P.refOrder): the same solve in the reference's own
// arithmetic, for bit-for-bit parity with it: the dot products in Eigen 3.3.7's order (two SSE2
// packets of two doubles, so four running lanes over groups of four, Eigen/src/Core/Redux.h, as
// the reference's BLAS::dot calls a.dot(b), include/pcgsolver/blas_wrapper.h:112-115), the sweep
// updates as a product and a subtraction, and the mean temperature as BLAS::sum's per-worker
// slice sums added in worker order (blas_wrapper.h:101-110 over ThreadPool::parallelForPlainTF,
// include/thread_pool.h:319-348).  These are serial chains (n / 4 and n / workers additions):
// a parity mode, not the fast path.
//
// Dependencies between rows (factorisation, both sweeps) are resolved without global barriers:
// rows are handed out in dependency order from an atomic counter and each row waits on per-row
// ready flags of the rows it reads.  Every wait is bounded; on timeout the kernel records
// DS_WAIT_TIMEOUT in the device status word and carries on, so a wait can never hang the GPU.
#include <cooperative_groups.h>
#include <cuda.h>
#include <cstdio>
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "astg_launch.h"
#include "astg_sample.cuh"

namespace cg = cooperative_groups;

namespace astg {

std::atomic<long long> g_launches{0};
thread_local long long t_launches = 0;

// event pairs around profiled launches; drained after each host synchronisation.  On a capturing
// stream the records become event-record nodes of the graph (external records) in a separate set
// of pairs, which every replay records again.
static bool capturing(cudaStream_t st) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    return cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs == cudaStreamCaptureStatusActive;
}
static void prof_begin(KProf* p, int kind, cudaStream_t st) {
    if (!p || !p->on) return;
    if (!p->created) {
        for (auto& e : p->ev) cudaEventCreate(&e);
        for (auto& e : p->gev) cudaEventCreate(&e);
        p->created = true;
    }
    if (capturing(st)) {
        if (p->gused >= 64) return;
        p->gkind[p->gused] = kind;
        cudaEventRecordWithFlags(p->gev[2 * p->gused], st, cudaEventRecordExternal);
    } else {
        if (p->used >= 128) return;
        p->kind[p->used] = kind;
        cudaEventRecord(p->ev[2 * p->used], st);
    }
}
static void prof_end(KProf* p, cudaStream_t st) {
    if (!p || !p->on) return;
    if (capturing(st)) {
        if (p->gused >= 64) return;
        cudaEventRecordWithFlags(p->gev[2 * p->gused + 1], st, cudaEventRecordExternal);
        ++p->gused;
    } else {
        if (p->used >= 128) return;
        cudaEventRecord(p->ev[2 * p->used + 1], st);
        ++p->used;
    }
}
static void prof_add(KProf* p, cudaEvent_t a, cudaEvent_t b, int kind) {
    float ms = 0;
    if (cudaEventElapsedTime(&ms, a, b) == cudaSuccess) {
        p->ms[kind] += ms;
        p->count[kind] += 1;
    } else {
        cudaGetLastError();  // a pair that was not recorded is not a launch error of the step
    }
}
// direct pairs, and the graph's pairs when a replay ran since the last drain
static void prof_drain(KProf* p, bool replayed = false) {
    if (!p || !p->on) return;
    for (int i = 0; i < p->used; ++i) prof_add(p, p->ev[2 * i], p->ev[2 * i + 1], p->kind[i]);
    p->used = 0;
    if (replayed)
        for (int i = 0; i < p->gused; ++i) prof_add(p, p->gev[2 * i], p->gev[2 * i + 1], p->gkind[i]);
}

// One batch of PCG iterations, either launched directly or replayed from a CUDA graph captured
// on the first full batch (the kernels skip themselves once the device's done flag is set, so a
// batch is the same work every time).  Replaying saves the launch gaps of the ~9 small kernels of
// an iteration.  Not used with the sync-free sweeps, whose epoch counter changes every launch.
// While kernel profiling is on, one replay in KPROF_GRAPH_EVERY runs a second graph whose kernels
// are bracketed by event-record nodes (those nodes cost about 3 us each), the others the plain one.
bool g_pcg_graphs = getenv("ASTG_PCG_GRAPH") ? atoi(getenv("ASTG_PCG_GRAPH")) != 0 : true;
constexpr int KPROF_GRAPH_EVERY = 4;
struct BatchGraph {
    cudaGraphExec_t exec[2] = {nullptr, nullptr};  // plain, with profiling event nodes
    long long launches[2] = {0, 0};                 // kernels per replay
    bool failed = false;
    long long replays = 0;
    bool profiled = false;  // the last replay recorded the event pairs
    ~BatchGraph() {
        for (auto e : exec)
            if (e) cudaGraphExecDestroy(e);
    }
    // runs body(nb, prof) for a full batch through a graph; returns false to run it directly
    template <typename Body>
    bool run(Body body, int nb, cudaStream_t st, KProf* prof) {
        if (failed) return false;
        const int k = (prof && prof->on && replays % KPROF_GRAPH_EVERY == 0) ? 1 : 0;
        if (!exec[k]) {
            if (k) prof->gused = 0;
            long long l0 = t_launches;
            if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
                cudaGetLastError();
                failed = true;
                return false;
            }
            body(nb, k ? prof : nullptr);
            cudaGraph_t g = nullptr;
            cudaError_t e = cudaStreamEndCapture(st, &g);
            if (e == cudaSuccess) e = cudaGraphInstantiate(&exec[k], g, 0);
            if (g) cudaGraphDestroy(g);
            launches[k] = t_launches - l0;
            g_launches -= launches[k];  // captured, not launched: counted at each replay
            t_launches -= launches[k];
            if (e != cudaSuccess) {
                cudaGetLastError();
                exec[k] = nullptr;
                failed = true;
                return false;
            }
        }
        if (cudaGraphLaunch(exec[k], st) != cudaSuccess) {
            cudaGetLastError();
            failed = true;
            return false;
        }
        g_launches += launches[k];
        t_launches += launches[k];
        ++replays;
        profiled = k == 1;
        return true;
    }
};

constexpr int TB = 256;
static inline int nblk(long long n) { return (int)((n + TB - 1) / TB); }
static int log2_exact(int v) {
    int lg = 0;
    while ((1 << lg) < v) ++lg;
    return lg;
}
constexpr int RED_LANES = 256, RED_PER_LANE = 8, RED_CHUNK = RED_LANES * RED_PER_LANE;
constexpr long long SPIN_LIMIT = 1LL << 24;
// One update z_i -= L_ij z_j of a MIC(0) sweep: the library's order is one fused multiply-subtract;
// the reference's order (P.unfused) is a product, then a subtraction, as its column loops
// (include/pcgsolver/pcg_solver.h:211-253) compute it.
template <typename T>
__device__ __forceinline__ T sweep_update(bool unfused, T acc, T v, T zk) {
    if (unfused) {
        T prod = v * zk;
        return acc - prod;
    }
    return fma(-v, zk, acc);
}  // ~seconds at nanosleep(64): far above any real wait

// ------------------------------------------------------------------ programmatic dependent launch
// The PCG's per-iteration kernels are launched so that each may be scheduled while its predecessor
// on the stream finishes (its implicit trigger is the predecessor's completion); the kernel's first
// statement waits for that predecessor's results to be visible.  Launched without the attribute
// (or outside a dependent pair) the wait returns at once.
__device__ __forceinline__ void grid_dep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
template <typename... KArgs, typename... Args>
static void launch_pdl(void (*k)(KArgs...), int grid, int block, cudaStream_t st, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    count_launch();
    cudaLaunchKernelEx(&cfg, k, static_cast<KArgs>(args)...);
}

// ------------------------------------------------------------------ fixed-tree reduction
__device__ inline double block_tree(double v, double* sh) {
    int t = threadIdx.x;
    sh[t] = v;
    __syncthreads();
    for (int st = RED_LANES / 2; st >= 1; st >>= 1) {
        if (t < st) sh[t] = sh[t] + sh[t + st];
        __syncthreads();
    }
    double r = sh[0];
    __syncthreads();
    return r;
}
// sum of a[i] over [0, n) (chunk partials)
__global__ void k_tree_sum(const double* a, const long long* nptr, long long nconst, double* part) {
    __shared__ double sh[RED_LANES];
    long long n = nptr ? *nptr : nconst;
    long long base = (long long)blockIdx.x * RED_CHUNK;
    if (base >= n && blockIdx.x > 0) return;
    double acc = 0.0;
    for (int k = 0; k < RED_PER_LANE; ++k) {
        long long i = base + threadIdx.x + (long long)RED_LANES * k;
        if (i < n) acc = acc + a[i];
    }
    double r = block_tree(acc, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = r;
}
// sum of a[i] * b[i]; each lane accumulates with fused multiply-adds (the library's order)
__global__ void k_tree_dot(const double* a, const double* b, const int* nptr, double* part) {
    grid_dep_wait();
    __shared__ double sh[RED_LANES];
    long long n = *nptr;
    long long base = (long long)blockIdx.x * RED_CHUNK;
    if (base >= n && blockIdx.x > 0) return;
    double acc = 0.0;
    for (int k = 0; k < RED_PER_LANE; ++k) {
        long long i = base + threadIdx.x + (long long)RED_LANES * k;
        if (i < n) acc = fma(a[i], b[i], acc);
    }
    double r = block_tree(acc, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = r;
}
// one block: folds m <= 2048 chunk partials with the same rule
__device__ inline double fold_partials(const double* part, long long m, double* sh) {
    double acc = 0.0;
    for (int k = 0; k < RED_PER_LANE; ++k) {
        long long i = threadIdx.x + (long long)RED_LANES * k;
        if (i < m) acc = acc + part[i];
    }
    return block_tree(acc, sh);
}

// ------------------------------------------------------------------ reference-order reductions
// Eigen's dot of a and b (no fused multiply-add): lanes l_k, k = 0..3, start at a[k] b[k] and add
// a[i] b[i] for i = k + 4, k + 8, ... below the largest multiple of four; then l0 + l2 and l1 + l3,
// one more pair when n mod 4 >= 2, their sum, and the scalar tail.  The result goes to part[0] and
// part[1 .. chunks) are zeroed, so the fixed-tree fold of the partials that follows returns it
// unchanged (adding zeros is exact).  One block of 32 threads.
__global__ void k_dot_ref(const double* a, const double* b, const int* nptr, double* part) {
    __shared__ double lane[4];
    const long long n = *nptr;
    const long long asz2 = (n / 4) * 4, asz = (n / 2) * 2;
    const int t = threadIdx.x;
    if (asz > 2 && t < 4) {
        double l = a[t] * b[t];
#pragma unroll 8
        for (long long i = 4 + t; i < asz2; i += 4) {
            double prod = a[i] * b[i];
            l = l + prod;
        }
        lane[t] = l;
    }
    __syncthreads();
    if (t == 0) {
        double r;
        if (asz == 0) {
            r = 0.0;
            for (long long i = 0; i < n; ++i) {
                double prod = a[i] * b[i];
                r = r + prod;
            }
        } else {
            double l0, l1;
            if (asz > 2) {
                l0 = lane[0] + lane[2];
                l1 = lane[1] + lane[3];
                if (asz > asz2) {
                    double p0 = a[asz2] * b[asz2], p1 = a[asz2 + 1] * b[asz2 + 1];
                    l0 = l0 + p0;
                    l1 = l1 + p1;
                }
            } else {
                l0 = a[0] * b[0];
                l1 = a[1] * b[1];
            }
            r = l0 + l1;
            for (long long i = asz; i < n; ++i) {
                double prod = a[i] * b[i];
                r = r + prod;
            }
        }
        part[0] = r;
    }
    const long long chunks = (n + RED_CHUNK - 1) / RED_CHUNK;
    for (long long c = 1 + t; c < chunks; c += blockDim.x) part[c] = 0.0;
}
void launch_dot_ref(const double* a, const double* b, const int* nptr, double* part, cudaStream_t st) {
    ASTG_LAUNCH(k_dot_ref<<<1, 32, 0, st>>>(a, b, nptr, part));
}
// BLAS::sum over [0, size) with `workers` workers: slice = round((size + 1) / workers) (at least 1,
// the reference counts end - start + 1), worker i < workers - 1 sums [i slice, (i + 1) slice) while
// slices remain, the last running worker takes the rest; each slice from 0.0 in index order, the
// slice sums added from 0.0 in worker order
__device__ double ref_sum(const double* v, long long size, int workers, double* sums, long long* lo, long long* hi) {
    const int t = threadIdx.x;
    if (t == 0) {
        long long slice = llround((double)(size + 1) / (double)workers);
        if (slice < 1) slice = 1;
        long long i1 = 0, i2 = min(slice, size);
        int i = 0;
        for (int w = 0; w < workers; ++w) lo[w] = hi[w] = 0;
        for (; i + 1 < workers && i1 < size; ++i) {
            lo[i] = i1;
            hi[i] = i2;
            i1 = i2;
            i2 = min(i2 + slice, size);
        }
        if (i1 < size) {
            lo[i] = i1;
            hi[i] = size;
        }
    }
    __syncthreads();
    for (int w = t; w < workers; w += blockDim.x) {
        double x = 0.0;
        for (long long k = lo[w]; k < hi[w]; ++k) x = x + v[k];
        sums[w] = x;
    }
    __syncthreads();
    double acc = 0.0;
    if (t == 0)
        for (int w = 0; w < workers; ++w) acc = acc + sums[w];
    __syncthreads();
    return acc;
}
// addForce's ambT in the reference's order (src/octree_omnigrid_solver3.cpp:922-929 with
// BLAS::sum per level); one block
__global__ void k_amb_ref(Dev d, const double* hO, int workers, double* amb) {
    __shared__ double sums[REF_MAX_WORKERS];
    __shared__ long long lo[REF_MAX_WORKERS], hi[REF_MAX_WORKERS];
    double total = 0.0;
    long long count = 0;
    for (int l = 0; l < d.L; ++l) {
        long long nl = d.lN[l] + d.lG[l];
        double s = ref_sum(hO + d.loff[l], nl, workers, sums, lo, hi);
        total += s * (l == 0 ? 1 : 8);
        count += nl * (l == 0 ? 1 : 8);
    }
    if (threadIdx.x == 0) *amb = total / (double)count;
}
void launch_mean_temperature_ref(const Dev& d, const double* hO, int workers, double* amb, cudaStream_t st) {
    ASTG_LAUNCH(k_amb_ref<<<1, REF_MAX_WORKERS, 0, st>>>(d, hO, workers, amb));
}

// ------------------------------------------------------------------ mean temperature
// addForce, src/octree_omnigrid_solver3.cpp:922-929: per-level sums of the octagon heat (ghosts
// included) weighted 1 on level 0 and 8 elsewhere, divided by the weighted count
__global__ void k_amb(Dev d, const double* parts, const int* partOff, double* amb) {
    __shared__ double sh[RED_LANES];
    double total = 0.0;
    long long count = 0;
    for (int l = 0; l < d.L; ++l) {
        long long m = partOff[l + 1] - partOff[l];
        double s = m > 0 ? fold_partials(parts + partOff[l], m, sh) : 0.0;
        total += s * (l == 0 ? 1 : 8);
        count += (long long)(d.lN[l] + d.lG[l]) * (l == 0 ? 1 : 8);
    }
    if (threadIdx.x == 0) *amb = total / (double)count;
}
void launch_mean_temperature(const Dev& d, const double* hO, double* parts, const int* partOffDev,
                             const int* partOffHost, double* amb, cudaStream_t st) {
    for (int l = 0; l < d.L; ++l) {
        long long n = d.lN[l] + d.lG[l];
        int m = partOffHost[l + 1] - partOffHost[l];
        if (m > 0) ASTG_LAUNCH(k_tree_sum<<<m, RED_LANES, 0, st>>>(hO + d.loff[l], nullptr, n, parts + partOffHost[l]));
    }
    ASTG_LAUNCH(k_amb<<<1, RED_LANES, 0, st>>>(d, parts, partOffDev, amb));
}

// ------------------------------------------------------------------ mean temperature, static scratch
// The same reduction for callers that hold the heat array in their own device memory and must not
// allocate: a framework whose caching allocator has already reserved most of HBM (a cudaMalloc
// there can fail or force the framework to release its cache), or a per-step loop on a shared
// device that cannot take the device-wide synchronisation cudaMalloc and cudaFree imply.  The chunk
// partials live in one file-scope device array instead of handle memory.  Each call writes every
// partial it later reads, on the same stream, so nothing in the array has to start at zero.  All
// calls on one device share the array: two calls whose kernels overlap in time (different streams,
// or different host threads without ordering between them) race on it.
static_assert(RED_CHUNK == AMB_CHUNK, "one chunk size for both forms of the reduction");
static __device__ __align__(256) double g_amb_scratch[NOALLOC_MAX_PARTIALS];

// one block per chunk of any level: the arithmetic of k_tree_sum on that level's slice
__global__ void k_tree_sum_levels(const double* a, LevelSpans sp, double* part) {
    __shared__ double sh[RED_LANES];
    int b = blockIdx.x, l = 0;
    while (l + 1 < sp.L && b >= sp.partOff[l + 1]) ++l;
    long long n = sp.off[l + 1] - sp.off[l];
    long long base = (long long)(b - sp.partOff[l]) * RED_CHUNK;
    const double* al = a + sp.off[l];
    double acc = 0.0;
    for (int k = 0; k < RED_PER_LANE; ++k) {
        long long i = base + threadIdx.x + (long long)RED_LANES * k;
        if (i < n) acc = acc + al[i];
    }
    double r = block_tree(acc, sh);
    if (threadIdx.x == 0) part[b] = r;
}
// the arithmetic of k_amb with the level bounds passed by value
__global__ void k_amb_levels(LevelSpans sp, const double* parts, double* amb) {
    __shared__ double sh[RED_LANES];
    double total = 0.0;
    long long count = 0;
    for (int l = 0; l < sp.L; ++l) {
        long long m = sp.partOff[l + 1] - sp.partOff[l];
        double s = m > 0 ? fold_partials(parts + sp.partOff[l], m, sh) : 0.0;
        total += s * (l == 0 ? 1 : 8);
        count += (sp.off[l + 1] - sp.off[l]) * (l == 0 ? 1 : 8);
    }
    if (threadIdx.x == 0) *amb = total / (double)count;
}

// Address of g_amb_scratch in the current context, looked up on the first call made with each
// device current and kept with the context it belongs to; the lookup may load this library's device
// code on that device.  A context that is destroyed and created again (cudaDeviceReset, or a
// primary context released by every user and retained anew) reloads the module, possibly at another
// address, so the cached address is only used while the current context is the one it was taken
// in; otherwise it is looked up again.  The context handle comes from the driver's cuCtxGetCurrent,
// reached through the runtime's entry-point query, so this library links no driver library.
using CtxGetCurrentFn = CUresult (*)(CUcontext*);
static std::mutex g_amb_scratch_mu;
static CtxGetCurrentFn g_ctx_get_current = nullptr;
static bool g_ctx_query_done = false;
static CUcontext g_amb_scratch_ctx[NOALLOC_MAX_DEVICES];
static double* g_amb_scratch_ptr[NOALLOC_MAX_DEVICES];
cudaError_t mean_temperature_scratch(double** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_amb_scratch_mu);
    if (!g_ctx_query_done) {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(fn);
        g_ctx_query_done = true;
    }
    // make the device's primary context current (a no-op when it already is), then name it
    e = cudaFree(nullptr);
    if (e != cudaSuccess) return e;
    CUcontext ctx = nullptr;
    if (g_ctx_get_current && g_ctx_get_current(&ctx) != CUDA_SUCCESS) ctx = nullptr;
    if (!g_amb_scratch_ptr[dev] || !ctx || ctx != g_amb_scratch_ctx[dev]) {
        double* p = nullptr;
        e = cudaGetSymbolAddress((void**)&p, g_amb_scratch);
        if (e != cudaSuccess) return e;
        g_amb_scratch_ptr[dev] = p;
        g_amb_scratch_ctx[dev] = ctx;
    }
    *out = g_amb_scratch_ptr[dev];
    return cudaSuccess;
}
// Each launch's own status is returned (cudaLaunchKernel), so an error that another call on this
// host thread left pending is neither reported as this call's nor cleared.
cudaError_t launch_mean_temperature_static(const double* heat, const LevelSpans& sp, double* amb, cudaStream_t st) {
    double* parts = nullptr;
    cudaError_t e = mean_temperature_scratch(&parts);
    if (e != cudaSuccess) return e;
    int m = sp.partOff[sp.L];
    LevelSpans spv = sp;
    if (m > 0) {
        void* args[] = {(void*)&heat, (void*)&spv, (void*)&parts};
        count_launch();
        e = cudaLaunchKernel((const void*)k_tree_sum_levels, dim3(m), dim3(RED_LANES), args, 0, st);
        if (e != cudaSuccess) return e;
    }
    const double* pc = parts;
    void* args2[] = {(void*)&spv, (void*)&pc, (void*)&amb};
    count_launch();
    return cudaLaunchKernel((const void*)k_amb_levels, dim3(1), dim3(RED_LANES), args2, 0, st);
}

// ------------------------------------------------------------------ exclusive scan (int)
constexpr int SCAN_B = 1024;
__global__ void k_scan_block(const int* in, int* out, int* bsum, long long n) {
    __shared__ int sh[SCAN_B];
    long long i = (long long)blockIdx.x * SCAN_B + threadIdx.x;
    int v = i < n ? in[i] : 0;
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int off = 1; off < SCAN_B; off <<= 1) {
        int t = threadIdx.x >= off ? sh[threadIdx.x - off] : 0;
        __syncthreads();
        sh[threadIdx.x] += t;
        __syncthreads();
    }
    if (i < n) out[i] = sh[threadIdx.x] - v;
    if (threadIdx.x == SCAN_B - 1) bsum[blockIdx.x] = sh[threadIdx.x];
}
// exclusive scan of the block sums by one block: each thread scans a contiguous run
__global__ void k_scan_sums(int* bsum, int nb, int* total) {
    __shared__ int sh[SCAN_B];
    int per = (nb + SCAN_B - 1) / SCAN_B;
    int t = threadIdx.x, a = t * per, b = min(a + per, nb);
    int s = 0;
    for (int i = a; i < b; ++i) s += bsum[i];
    sh[t] = s;
    __syncthreads();
    for (int off = 1; off < SCAN_B; off <<= 1) {
        int v = t >= off ? sh[t - off] : 0;
        __syncthreads();
        sh[t] += v;
        __syncthreads();
    }
    int run = sh[t] - s;
    for (int i = a; i < b; ++i) {
        int v = bsum[i];
        bsum[i] = run;
        run += v;
    }
    if (t == SCAN_B - 1) *total = sh[t];
}
__global__ void k_scan_add(int* out, const int* bsum, long long n) {
    long long i = (long long)blockIdx.x * SCAN_B + threadIdx.x;
    if (i < n) out[i] += bsum[blockIdx.x];
}
// out = exclusive scan of in[0..n); *total = sum.  bsum needs ceil(n/1024) ints.
void exclusive_scan(const int* in, int* out, int* bsum, int* total, long long n, cudaStream_t st) {
    int nb = (int)((n + SCAN_B - 1) / SCAN_B);
    ASTG_LAUNCH(k_scan_block<<<nb, SCAN_B, 0, st>>>(in, out, bsum, n));
    ASTG_LAUNCH(k_scan_sums<<<1, SCAN_B, 0, st>>>(bsum, nb, total));
    ASTG_LAUNCH(k_scan_add<<<nb, SCAN_B, 0, st>>>(out, bsum, n));
}

// ------------------------------------------------------------------ DOF numbering
// updateIndexParallel, src/octree_omnigrid_solver3.cpp:292-347: in slot order, a valid octagon
// then an open tilt take the next index; ghosts get -1; half tilts are appended in list order;
// the tilt indices are then propagated to ghosts (OctreeVertexCenteredGrid3<int>::updateGhost,
// src/octree_vertex_centered_grid3.cpp:47-64)
// an octagon / tilt carries a DOF when it is valid / open and, with a collider, the SDF at its position
// exceeds -3 dx_l (:297-309)
__device__ __forceinline__ bool dof_oct(const Dev& d, int s) {
    return oct_valid(d, slot_l(d, s), slot_x(d, s), slot_y(d, s), slot_z(d, s)) &&
           (!d.colMask || (d.colMask[s] & COL_OCT_FLUID));
}
__device__ __forceinline__ bool dof_tilt(const Dev& d, const uint8_t* open, int s) {
    return open[s] && (!d.colMask || (d.colMask[s] & COL_TILT_FLUID));
}
__global__ void k_dof_count(Dev d, const uint8_t* open, int* cnt) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.S) return;
    int c = 0;
    if (!(slot_f(d, s) & SF_GHOST)) c = (dof_oct(d, s) ? 1 : 0) + (dof_tilt(d, open, s) ? 1 : 0);
    cnt[s] = c;
}
__global__ void k_dof_assign(Dev d, const uint8_t* open, const int* base, int* pO, int* pT) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.S) return;
    if (slot_f(d, s) & SF_GHOST) { pO[s] = -1; pT[s] = -1; return; }
    bool ov = dof_oct(d, s);
    pO[s] = ov ? base[s] : -1;
    pT[s] = dof_tilt(d, open, s) ? base[s] + (ov ? 1 : 0) : -1;
}
__global__ void k_dof_half(Dev d, int* pT, const int* n0, int* nDof) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < d.H) pT[d.half[i]] = *n0 + i;
    if (i == 0) *nDof = *n0 + d.H;
}
// with a collider: half tilts in list order, those in the fluid numbered consecutively
__global__ void k_dof_half_flag(Dev d, int* flag) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < d.H) flag[i] = (d.colMask[d.half[i]] & COL_TILT_FLUID) ? 1 : 0;
}
__global__ void k_dof_half_masked(Dev d, int* pT, const int* flag, const int* base, const int* n0) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < d.H) pT[d.half[i]] = flag[i] ? *n0 + base[i] : -1;
}
__global__ void k_dof_total(int* nDof, const int* n0, const int* nHalf) { *nDof = *n0 + *nHalf; }
__global__ void k_dof_ghost(Dev d, int* pT, int l) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.lG[l]) return;
    int s = d.loff[l] + d.lN[l] + i;
    int x = slot_x(d, s), y = slot_y(d, s), z = slot_z(d, s);
    if (slot_f(d, s) & SF_FROM_COARSE) {
        if ((x & 1) || (y & 1) || (z & 1)) return;
        pT[s] = pT[req(d, l + 1, x >> 1, y >> 1, z >> 1)];
    } else {
        pT[s] = pT[req(d, l - 1, x << 1, y << 1, z << 1)];
    }
}
void launch_dof_numbering(const Dev& d, const uint8_t* open, Proj& P, cudaStream_t st) {
    ASTG_LAUNCH(k_dof_count<<<nblk(d.S), TB, 0, st>>>(d, open, P.cnt));
    exclusive_scan(P.cnt, P.base, P.bsum, P.n0, d.S, st);
    ASTG_LAUNCH(k_dof_assign<<<nblk(d.S), TB, 0, st>>>(d, open, P.base, P.pO, P.pT));
    if (d.colMask && d.H > 0) {  // P.cnt / P.base are free again once the slots are numbered
        ASTG_LAUNCH(k_dof_half_flag<<<nblk(d.H), TB, 0, st>>>(d, P.cnt));
        exclusive_scan(P.cnt, P.base, P.bsum, P.nnz + 1, d.H, st);
        ASTG_LAUNCH(k_dof_half_masked<<<nblk(d.H), TB, 0, st>>>(d, P.pT, P.cnt, P.base, P.n0));
        ASTG_LAUNCH(k_dof_total<<<1, 1, 0, st>>>(P.nDof, P.n0, P.nnz + 1));
    } else {
        ASTG_LAUNCH(k_dof_half<<<nblk(d.H > 0 ? d.H : 1), TB, 0, st>>>(d, P.pT, P.n0, P.nDof));
    }
    for (int l = 0; l < d.L; ++l)
        if (d.lG[l]) ASTG_LAUNCH(k_dof_ghost<<<nblk(d.lG[l]), TB, 0, st>>>(d, P.pT, l));
}

// ------------------------------------------------------------------ assembly
// project(), src/octree_omnigrid_solver3.cpp:350-653.  Each row is built in registers with the
// reference's set/add semantics (PCG::SparseMatrix::set_element / add_to_element), sorted by
// column and written to a padded row buffer of width ROW_W; contributions of half tilts to the
// coarse octagon rows they face are gathered per octagon in half-tilt list order.
struct RowBuf {
    int n;
    int col[ROW_W];
    double val[ROW_W];
    ASTG_HD void set(int c, double v) {
        for (int k = 0; k < n; ++k)
            if (col[k] == c) { val[k] = v; return; }
        if (n < ROW_W) { col[n] = c; val[n] = v; }
        ++n;
    }
    ASTG_HD void add(int c, double v) {
        for (int k = 0; k < n; ++k)
            if (col[k] == c) { val[k] += v; return; }
        if (n < ROW_W) { col[n] = c; val[n] = v; }
        ++n;
    }
};
__device__ inline void store_row(const Dev& d, const Proj& P, int r, RowBuf& rb, double b) {
    if (rb.n > ROW_W) { report(d, DS_MISSING_NODE); rb.n = ROW_W; }
    for (int i = 1; i < rb.n; ++i) {  // insertion sort by column
        int c = rb.col[i];
        double v = rb.val[i];
        int j = i - 1;
        while (j >= 0 && rb.col[j] > c) { rb.col[j + 1] = rb.col[j]; rb.val[j + 1] = rb.val[j]; --j; }
        rb.col[j + 1] = c;
        rb.val[j + 1] = v;
    }
    P.rowCnt[r] = rb.n;
    for (int i = 0; i < rb.n; ++i) {
        P.padCol[(size_t)r * ROW_W + i] = rb.col[i];
        P.padVal[(size_t)r * ROW_W + i] = rb.val[i];
    }
    P.bRaw[r] = b;
}
__global__ void k_asm_oct(Dev d, Fields F, Proj P, const int* hoPtr, const int* hoIdx) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.S || (slot_f(d, s) & SF_GHOST)) return;
    int ci = P.pO[s];
    int l = slot_l(d, s), x = slot_x(d, s), y = slot_y(d, s), z = slot_z(d, s);
    if (ci < 0 || !oct_valid(d, l, x, y, z)) return;
    double h = d.ldh[l];
    double center = 0, tb = 0, tC = 0, tK = 0;
    RowBuf rb;
    rb.n = 0;
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
        if (oct_valid(d, l, nx, ny, nz)) {
            double term = d.wMac[(size_t)axis * d.S + fs];
            int ti = P.pO[req(d, l, nx, ny, nz)];
            if (ti >= 0) {
                tC = term * area / h;
                tK = area * term;
                rb.set(ti, -tC);
            } else { tC = 0; tK = 0; }
        } else if ((d.closedMask >> i) & 1) {
            tC = 0; tK = 0;
        } else {
            tK = area;
            tC = tK / h;
        }
        center += tC;
        tb += ((i & 1) ? 1 : -1) * tK * F.mac[(size_t)axis * d.S + fs];
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
            if (ti >= 0) {
                tC = term * area / (h * SQRT3 * 0.5);
                tK = area * term;
                rb.add(ti, -tC);
            } else { tC = 0; tK = 0; }
            center += tC;
            tb += (i < 4 ? -1 : 1) * tK * F.tv[(size_t)ns * 8 + re];
        }
    }
    if (fabs(center) < EPS) { center = 1; tb = 0; }
    rb.set(ci, center);
    // half tilts facing this octagon (src/octree_omnigrid_solver3.cpp:572-581)
    for (int q = hoPtr[s]; q < hoPtr[s + 1]; ++q) {
        int hs = d.half[hoIdx[q]];
        int hci = P.pT[hs];
        if (hci < 0) continue;
        int dir = tf_dir(F.tf[hs]);
        int oi = HALF_SLOT[dir][4];
        double e = F.te[hs];
        double area = e * e * 2;
        double hh = d.ldh[slot_l(d, hs)];
        double tw = d.wTilt[(size_t)hs * 8 + oi];
        double u = F.tv[(size_t)hs * 8 + oi];
        rb.add(ci, tw * area / hh);
        rb.add(hci, -tw * area / hh);
        tb += (dir < 3 ? -1 : 1) * u * tw * area;
    }
    store_row(d, P, ci, rb, tb);
}
__global__ void k_asm_tilt(Dev d, Fields F, Proj P, const uint8_t* open) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.S || (slot_f(d, s) & SF_GHOST)) return;
    int ci = P.pT[s];
    if (!open[s] || ci < 0) return;
    int l = slot_l(d, s), x = slot_x(d, s), y = slot_y(d, s), z = slot_z(d, s);
    double e = F.te[s];
    double center = 0, tb = 0, tC = 0, tK = 0;
    const double* u = F.tv + (size_t)s * 8;
    const double* tw = d.wTilt + (size_t)s * 8;
    double area = e * e * SQRT3 * 0.5;
    RowBuf rb;
    rb.n = 0;
    for (int i = 0; i < 8; ++i) {
        NbOct nb = tilt_nb_oct(d, l, x, y, z, i);
        if (!nb.some) {
            if (!oct_valid(d, l, x + TILT_NB_OCT[i][0], y + TILT_NB_OCT[i][1], z + TILT_NB_OCT[i][2])) {
                tC = area / (d.ldh[l] * SQRT3 / 3.0);
                tK = area;
                center += tC;
                tb += (i < 4 ? -1 : 1) * tK * u[i];
            }
            continue;
        }
        if (oct_valid(d, nb.l, nb.x, nb.y, nb.z)) {
            double h2 = d.ldh[nb.l];
            int ti = P.pO[req(d, nb.l, nb.x, nb.y, nb.z)];
            if (ti >= 0) {
                tC = tw[i] * area / (h2 * SQRT3 * 0.5);
                tK = area * tw[i];
                rb.set(ti, -tC);
            } else { tC = 0; tK = 0; }
        } else {
            tC = area / (d.ldh[l] * SQRT3 / 3.0);
            tK = area;
        }
        center += tC;
        tb += (i < 4 ? -1 : 1) * tK * u[i];
    }
    if (fabs(center) < EPS) center = 1;
    rb.set(ci, center);
    store_row(d, P, ci, rb, tb);
}
__global__ void k_asm_half(Dev d, Fields F, Proj P) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.H) return;
    int hs = d.half[i];
    int ci = P.pT[hs];
    if (ci < 0) return;
    int l = slot_l(d, hs), x = slot_x(d, hs), y = slot_y(d, hs), z = slot_z(d, hs);
    int dir = tf_dir(F.tf[hs]);
    double e = F.te[hs];
    double area = e * e * 2;
    double h = d.ldh[l];
    double center = 0, tb = 0, tC = 0, tK = 0;
    const double* u = F.tv + (size_t)hs * 8;
    const double* tw = d.wTilt + (size_t)hs * 8;
    int id[3] = {x >> 1, y >> 1, z >> 1};
    id[dir % 3] -= dir < 3 ? 1 : 0;
    int oi = HALF_SLOT[dir][4];
    RowBuf rb;
    rb.n = 0;
    if (l + 1 < d.L && oct_valid(d, l + 1, id[0], id[1], id[2])) {
        int ti = P.pO[req(d, l + 1, id[0], id[1], id[2])];
        if (ti >= 0) {
            center += tw[oi] * area / h;
            rb.add(ti, -tw[oi] * area / h);
            tb += (dir < 3 ? 1 : -1) * u[oi] * tw[oi] * area;
        }
    } else {
        int axis = (dir % 3) * 2 + (dir >= 3);
        if ((d.closedMask >> axis) & 1) { tC = 0; tK = area; }
        else { tC = 1000; tK = area; }
        center += tC;
        tb += (dir < 3 ? 1 : -1) * u[oi] * area;
    }
    area = e * e * SQRT3 * 0.5;
    for (int k = 0; k < 8; ++k) {
        if (!half_listed(dir, k)) continue;
        int nx = x + TILT_NB_OCT[k][0], ny = y + TILT_NB_OCT[k][1], nz = z + TILT_NB_OCT[k][2];
        if (oct_valid(d, l, nx, ny, nz)) {
            int ti = P.pO[req(d, l, nx, ny, nz)];
            if (ti >= 0) {
                tC = area * tw[k] / (h * SQRT3 * 0.5);
                tK = area * tw[k];
                rb.set(ti, -tC);
            } else { tC = 0; tK = 0; }
        } else {
            report(d, DS_MISSING_NODE);  // the reference throws here (:641)
            tC = 0; tK = 0;
        }
        center += tC;
        tb += (k < 4 ? -1 : 1) * tK * u[k];
    }
    rb.add(ci, center);
    store_row(d, P, ci, rb, tb);
}
// rows -> CSR, b scaled by rho/dt (BLAS::scale, :651), diagonal positions
__global__ void k_csr_fill(Proj P, double scale) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= *P.nDof) return;
    int o = P.rowPtr[r], n = P.rowCnt[r];
    int dg = -1;
    for (int i = 0; i < n; ++i) {
        int c = P.padCol[(size_t)r * ROW_W + i];
        P.col[o + i] = c;
        P.val[o + i] = P.padVal[(size_t)r * ROW_W + i];
        if (c == r) dg = o + i;
    }
    P.diagPos[r] = dg;
    P.b[r] = P.bRaw[r] * scale;
}
__global__ void k_rowptr_last(Proj P) {
    int n = *P.nDof;
    P.rowPtr[n] = *P.nnz;
}
// position of the mirrored entry (c, r) for every off-diagonal entry (r, c); the pattern is
// symmetric (the reference asserts it, :654), a missing mirror is reported
__global__ void k_transpose_map(const Dev d, Proj P) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= *P.nDof) return;
    for (int q = P.rowPtr[r]; q < P.rowPtr[r + 1]; ++q) {
        int c = P.col[q];
        int t = -1;
        if (c != r) {
            int lo = P.rowPtr[c], hi = P.rowPtr[c + 1] - 1;
            while (lo <= hi) {
                int mid = (lo + hi) >> 1;
                int v = P.col[mid];
                if (v == r) { t = mid; break; }
                if (v < r) lo = mid + 1; else hi = mid - 1;
            }
            if (t < 0) report(d, DS_MISSING_NODE);
        }
        P.tpos[q] = t;
    }
}
// diagonal positions of a caller-supplied CSR matrix (astg_solve); a row without one is reported
__global__ void k_find_diag(const Dev d, Proj P) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= *P.nDof) return;
    int dg = -1;
    for (int q = P.rowPtr[r]; q < P.rowPtr[r + 1]; ++q)
        if (P.col[q] == r) dg = q;
    if (dg < 0) report(d, DS_MISSING_NODE);
    P.diagPos[r] = dg;
}
void launch_external_system(const Dev& d, Proj& P, int rows, cudaStream_t st) {
    ASTG_LAUNCH(k_find_diag<<<nblk(rows), TB, 0, st>>>(d, P));
    ASTG_LAUNCH(k_transpose_map<<<nblk(rows), TB, 0, st>>>(d, P));
}
__global__ void k_zero_rows(Proj P, int maxRows) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < maxRows) { P.rowCnt[r] = 0; P.bRaw[r] = 0; }
}
void launch_assemble(const Dev& d, const Fields& F, const uint8_t* open, Proj& P, const int* hoPtr, const int* hoIdx,
                     double dt, cudaStream_t st) {
    int maxRows = P.rowsCap;
    ASTG_LAUNCH(k_zero_rows<<<nblk(maxRows), TB, 0, st>>>(P, maxRows));
    ASTG_LAUNCH(k_asm_oct<<<nblk(d.S), TB, 0, st>>>(d, F, P, hoPtr, hoIdx));
    ASTG_LAUNCH(k_asm_tilt<<<nblk(d.S), TB, 0, st>>>(d, F, P, open));
    if (d.H) ASTG_LAUNCH(k_asm_half<<<nblk(d.H), TB, 0, st>>>(d, F, P));
    launch_rows_to_csr(d, P, maxRows, d.rho / dt, st);
}
void launch_rows_to_csr(const Dev& d, Proj& P, int maxRows, double scale, cudaStream_t st) {
    exclusive_scan(P.rowCnt, P.rowPtr, P.bsum, P.nnz, maxRows, st);
    ASTG_LAUNCH(k_rowptr_last<<<1, 1, 0, st>>>(P));
    ASTG_LAUNCH(k_csr_fill<<<nblk(maxRows), TB, 0, st>>>(P, scale));
    ASTG_LAUNCH(k_transpose_map<<<nblk(maxRows), TB, 0, st>>>(d, P));
}
void launch_exclusive_scan(const int* in, int* out, int* bsum, int* total, long long n, cudaStream_t st) {
    exclusive_scan(in, out, bsum, total, n, st);
}

// ------------------------------------------------------------------ sync-free helpers
__device__ inline int ld_flag(const int* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ inline void st_flag(int* p, int v) { asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory"); }
__device__ inline bool wait_flag(const Dev& d, const int* flag, int epoch) {
    long long n = 0;
    while (ld_flag(flag) != epoch) {
        if (++n > SPIN_LIMIT) {
            report(d, DS_WAIT_TIMEOUT);
            return false;
        }
        __nanosleep(32);
    }
    return true;
}
// next row handed out in dependency order (ascending, or descending when rev)
__device__ inline int grab_row(int* counter) { return atomicAdd(counter, 1); }

// ------------------------------------------------------------------ MIC(0) factorisation
// factor_modified_incomplete_cholesky0, include/pcgsolver/pcg_solver.h:89-190, in left-looking
// form: column j applies, for every k < j with L(j,k) != 0 in increasing k, exactly the update
// the reference's step k applies to column j, then finalises itself.  Column k of L is the upper
// part of row k of A (same positions in the CSR arrays); Lv holds its values.
__global__ void k_mic_init(Proj P) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= *P.nDof) return;
    int dg = P.diagPos[r];
    double a = dg >= 0 ? P.val[dg] : 0.0;
    P.invdiag[r] = a;
    P.adiag[r] = a;
    for (int q = P.rowPtr[r]; q < P.rowPtr[r + 1]; ++q) P.Lv[q] = P.val[q];
}
__global__ void k_mic_factor(Dev d, Proj P, double omega, double minDiag, int epoch) {
    int n = *P.nDof;
    for (;;) {
        int j = grab_row(P.counter);
        if (j >= n) return;
        int rj0 = P.rowPtr[j], rj1 = P.rowPtr[j + 1];
        int dgj = P.diagPos[j];
        int upj = dgj >= 0 ? dgj + 1 : rj1;  // first entry of column j of L
        double invd = P.invdiag[j];
        int lev = 0;
        for (int qq = rj0; qq < rj1; ++qq) {
            int k = P.col[qq];
            if (k >= j) break;
            wait_flag(d, P.ready + k, epoch);
            lev = max(lev, P.level[k] + 1);
            if (P.adiag[k] == 0) continue;
            int tq = P.tpos[qq];  // entry (k, j): L(j, k)
            double mult = P.Lv[tq];
            double missing = 0;
            int a = P.diagPos[k] + 1, ak = P.rowPtr[k + 1];
            int b = rj0;
            while (a < ak && P.col[a] < j) {
                while (b < rj1) {
                    if (P.col[b] < P.col[a]) ++b;
                    else if (P.col[b] == P.col[a]) break;
                    else { missing += P.Lv[a]; break; }
                }
                ++a;
            }
            if (a < ak && P.col[a] == j) invd -= mult * P.Lv[a];
            ++a;
            int bb = upj;
            while (a < ak && bb < rj1) {
                if (P.col[bb] < P.col[a]) ++bb;
                else if (P.col[bb] == P.col[a]) { P.Lv[bb] -= mult * P.Lv[a]; ++a; ++bb; }
                else { missing += P.Lv[a]; ++a; }
            }
            while (a < ak) { missing += P.Lv[a]; ++a; }
            invd -= omega * mult * missing;
        }
        double ad = P.adiag[j];
        if (ad != 0) {
            if (invd < minDiag * ad) invd = 1 / sqrt(ad);
            else invd = 1 / sqrt(invd);
            for (int q = upj; q < rj1; ++q) P.Lv[q] *= invd;
        }
        P.invdiag[j] = invd;
        P.level[j] = lev;
        __threadfence();
        st_flag(P.ready + j, epoch);
    }
}

// ------------------------------------------------------------------ level schedule
// Rows grouped by dependency depth: a row of level g reads only rows of levels < g in the
// forward sweep and only rows of levels > g in the backward sweep, so rows of one level are
// independent in both.  The order inside a level does not change any result.
__global__ void k_level_hist(Proj P) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= *P.nDof) return;
    int g = P.level[j];
    atomicAdd(P.levelCnt + g, 1);
    atomicMax(P.nLevels, g + 1);
}
__global__ void k_level_scatter(Proj P) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= *P.nDof) return;
    int g = P.level[j];
    P.perm[P.levelPtr[g] + atomicAdd(P.fill + g, 1)] = j;
}
__global__ void k_level_counts(Proj P) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= *P.nDof) return;
    int i = P.perm[p];
    int dg = P.diagPos[i];
    P.cntF[p] = dg - P.rowPtr[i];
    P.cntB[p] = P.rowPtr[i + 1] - dg - 1;
}
__global__ void k_level_fill(Proj P) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= *P.nDof) return;
    int i = P.perm[p];
    int dg = P.diagPos[i];
    if (P.fcolP) {
        int cap = P.rowsCap;
        P.pos[i] = p;
        P.linvd[p] = P.invdiag[i];
        int nf = dg - P.rowPtr[i], nb = P.rowPtr[i + 1] - dg - 1;
        P.lcntF[p] = nf;
        P.lcntB[p] = nb;
        for (int e = 0; e < PC_MAXE; ++e) {
            int qf = P.rowPtr[i] + e, qb = dg + 1 + e;
            P.fcolP[(size_t)e * cap + p] = e < nf ? P.col[qf] : 0;
            P.fvalP[(size_t)e * cap + p] = e < nf ? P.Lv[P.tpos[qf]] : 0.0;
            P.bcolP[(size_t)e * cap + p] = e < nb ? P.col[qb] : 0;
            P.bvalP[(size_t)e * cap + p] = e < nb ? P.Lv[qb] : 0.0;
        }
    }
    int o = P.fptr[p];
    for (int q = P.rowPtr[i]; q < dg; ++q, ++o) {
        P.fcol[o] = P.col[q];
        P.fval[o] = P.Lv[P.tpos[q]];  // L(i, k), held in column k's storage
    }
    o = P.bptr[p];
    for (int q = dg + 1; q < P.rowPtr[i + 1]; ++q, ++o) {
        P.bcol[o] = P.col[q];
        P.bval[o] = P.Lv[q];
    }
}
__global__ void k_level_fptr_last(Proj P) {
    int n = *P.nDof;
    P.fptr[n] = P.nnz[2];
    P.bptr[n] = P.nnz[3];
}
__global__ void k_level_reset(Proj P, int rows) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j <= rows) { P.levelCnt[j] = 0; P.fill[j] = 0; }
    if (j == 0) *P.nLevels = 0;
}

// ------------------------------------------------------------------ cluster sweeps
constexpr int CLUSTER_THREADS = 512;
constexpr int PC_THREADS = 256;
cudaError_t g_cluster_error = cudaSuccess;
// One thread-block cluster walks the levels; a hardware cluster barrier (release/acquire at
// cluster scope) separates consecutive levels, so no row ever polls a flag.  Per row the
// operations are the reference's, in the same order.
__global__ void k_sweep_fwd_cluster(Proj P, const double* r, double* z) {
    if (*P.done) return;
    cg::cluster_group cl = cg::this_cluster();
    int nth = cl.num_blocks() * blockDim.x;
    int t = cl.block_rank() * blockDim.x + threadIdx.x;
    int nl = *P.nLevels;
    for (int g = 0; g < nl; ++g) {
        int p1 = P.levelPtr[g + 1];
        for (int p = P.levelPtr[g] + t; p < p1; p += nth) {
            int i = P.perm[p];
            double acc = r[i];
            for (int q = P.fptr[p]; q < P.fptr[p + 1]; ++q) acc = sweep_update(P.unfused != 0, acc, P.fval[q], __ldcg(z + P.fcol[q]));
            z[i] = acc * P.invdiag[i];
        }
        cl.sync();
    }
}
__global__ void k_sweep_bwd_cluster(Proj P, const double* unused, double* z) {
    (void)unused;
    if (*P.done) return;
    cg::cluster_group cl = cg::this_cluster();
    int nth = cl.num_blocks() * blockDim.x;
    int t = cl.block_rank() * blockDim.x + threadIdx.x;
    int nl = *P.nLevels;
    for (int g = nl - 1; g >= 0; --g) {
        int p1 = P.levelPtr[g + 1];
        for (int p = P.levelPtr[g] + t; p < p1; p += nth) {
            int i = P.perm[p];
            double acc = __ldcg(z + i);
            for (int q = P.bptr[p]; q < P.bptr[p + 1]; ++q) acc = sweep_update(P.unfused != 0, acc, P.bval[q], __ldcg(z + P.bcol[q]));
            z[i] = acc * P.invdiag[i];
        }
        cl.sync();
    }
}
// Both sweeps in one cluster launch with the vector held in distributed shared memory: entry i
// lives in CTA (i & (CS-1)) at index (i >> log2 CS).  Each thread owns at most one row of a level
// (rows beyond blockDim * CS take a slower loop).  While the cluster barrier between two levels is
// in flight, every thread already loads the next level's row (index, right-hand side, pivot and
// up to PC_MAXE factor entries) into registers, so after the barrier only the DSMEM reads of
// finished entries remain on the critical path.  Per row the updates are the reference's, in the
// reference's order, each one fused multiply-subtract.
__device__ __forceinline__ void cl_arrive() { asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory"); }
__device__ __forceinline__ void cl_wait() { asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory"); }
__device__ __forceinline__ double ld_ds(uint32_t a) {
    double v;
    asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(a) : "memory");
    return v;
}
__device__ __forceinline__ void st_ds(uint32_t a, double v) {
    asm volatile("st.shared::cluster.f64 [%0], %1;" ::"r"(a), "d"(v) : "memory");
}
struct PcRow {
    int i, p, cnt;
    double rhs, invd;
    int col[PC_MAXE];
    double val[PC_MAXE];
};
// record of level position p (p < p1): independent loads only
__device__ __forceinline__ void pc_load(const Proj& P, int p, int p1, bool fwd, PcRow& w) {
    w.cnt = -1;
    if (p >= p1) return;
    const int cap = P.rowsCap;
    const int* cc = fwd ? P.fcolP : P.bcolP;
    const double* vv = fwd ? P.fvalP : P.bvalP;
    w.p = p;
    w.i = P.perm[p];
    w.cnt = fwd ? P.lcntF[p] : P.lcntB[p];
    w.invd = P.linvd[p];
    w.rhs = fwd ? P.rl[p] : 0.0;
#pragma unroll
    for (int e = 0; e < PC_MAXE; ++e) {
        w.col[e] = cc[(size_t)e * cap + p];
        w.val[e] = vv[(size_t)e * cap + p];
    }
}
// row i lives in CTA (i & msk) of the cluster at local index (i >> lg)
__device__ __forceinline__ void pc_row(const Proj& P, const PcRow& w, bool fwd, const uint32_t* rb, int lg, int msk) {
    uint32_t ai = rb[w.i & msk] + (uint32_t)(w.i >> lg) * 8u;
    double zk[PC_MAXE];
#pragma unroll
    for (int e = 0; e < PC_MAXE; ++e)
        if (e < w.cnt) zk[e] = ld_ds(rb[w.col[e] & msk] + (uint32_t)(w.col[e] >> lg) * 8u);
    double acc = fwd ? w.rhs : ld_ds(ai);
#pragma unroll
    for (int e = 0; e < PC_MAXE; ++e)
        if (e < w.cnt) acc = sweep_update(P.unfused != 0, acc, w.val[e], zk[e]);
    if (w.cnt > PC_MAXE) {  // rows longer than the padded record: the rest from the compact arrays
        const int* cc = fwd ? P.fcol : P.bcol;
        const double* vv = fwd ? P.fval : P.bval;
        int q0 = (fwd ? P.fptr : P.bptr)[w.p];
        for (int e = PC_MAXE; e < w.cnt; ++e) {
            int k = cc[q0 + e];
            acc = sweep_update(P.unfused != 0, acc, vv[q0 + e], ld_ds(rb[k & msk] + (uint32_t)(k >> lg) * 8u));
        }
    }
    st_ds(ai, acc * w.invd);
}
constexpr int PC_MAX_LEVELS = 4096;  // level bounds staged in shared memory
__device__ __forceinline__ void pc_level(const Proj& P, const PcRow& w, bool fwd, const uint32_t* rb, int lg, int msk,
                                         int p0, int p1, int t, int nth) {
    if (w.cnt >= 0) pc_row(P, w, fwd, rb, lg, msk);
    for (int p = p0 + t + nth; p < p1; p += nth) {  // levels wider than the cluster
        PcRow x;
        pc_load(P, p, p1, fwd, x);
        pc_row(P, x, fwd, rb, lg, msk);
    }
    __syncwarp();  // the .aligned cluster barrier needs converged warps
    cl_arrive();
}
// Both MIC(0) triangular sweeps of one preconditioner application in one cluster launch.  z lives
// in the CTAs' shared memory (row i in CTA i mod CS), every level is one split cluster barrier,
// and the next levels' records are loaded into registers while the barrier completes.
__global__ void __launch_bounds__(256, 1) k_precond_dsmem(Proj P, double* z, int lgCS) {
    if (*P.done) return;
    extern __shared__ double zsh[];
    __shared__ uint32_t rb[16];
    __shared__ int lp[PC_MAX_LEVELS + 1];
    cg::cluster_group cl = cg::this_cluster();
    const int msk = (1 << lgCS) - 1;
    const int rank = cl.block_rank();
    const int nth = blockDim.x << lgCS;
    const int t = rank * blockDim.x + threadIdx.x;
    const int nl = *P.nLevels;
    if (threadIdx.x < (1 << lgCS)) {
        uint32_t a = (uint32_t)__cvta_generic_to_shared(zsh), m;
        asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(m) : "r"(a), "r"((uint32_t)threadIdx.x));
        rb[threadIdx.x] = m;
    }
    for (int g = threadIdx.x; g <= nl && g <= PC_MAX_LEVELS; g += blockDim.x) lp[g] = P.levelPtr[g];
    cl.sync();  // every CTA of the cluster is running; rb and lp are set
    // level bounds (staged in shared memory up to PC_MAX_LEVELS levels)
    auto LP = [&](int g) { return g <= PC_MAX_LEVELS ? lp[g] : P.levelPtr[g]; };
    for (int dir = 0; dir < 2; ++dir) {
        const bool fwd = dir == 0;
        // level of step k: k (forward) or nl-1-k (backward); rows of step k+2 are fetched while
        // step k+1 waits at the barrier, so the loads have two steps to arrive
        auto lvl = [&](int k) { return fwd ? k : nl - 1 - k; };
        PcRow A, B;
        pc_load(P, LP(lvl(0)) + t, LP(lvl(0) + 1), fwd, A);
        if (nl > 1) pc_load(P, LP(lvl(1)) + t, LP(lvl(1) + 1), fwd, B);
        for (int k = 0; k < nl; k += 2) {
            int g = lvl(k);
            pc_level(P, A, fwd, rb, lgCS, msk, LP(g), LP(g + 1), t, nth);
            if (k + 2 < nl) pc_load(P, LP(lvl(k + 2)) + t, LP(lvl(k + 2) + 1), fwd, A);
            __syncwarp();
            cl_wait();
            if (k + 1 < nl) {
                g = lvl(k + 1);
                pc_level(P, B, fwd, rb, lgCS, msk, LP(g), LP(g + 1), t, nth);
                if (k + 3 < nl) pc_load(P, LP(lvl(k + 3)) + t, LP(lvl(k + 3) + 1), fwd, B);
                __syncwarp();
                cl_wait();
            }
        }
    }
    int n = *P.nDof;
    for (int j = threadIdx.x; (j << lgCS) + rank < n; j += blockDim.x) z[(j << lgCS) + rank] = zsh[j];
    cl.sync();
}
// ---- barrier-free fused preconditioner.  Same vector placement idea (z in the distributed
// shared memory of one cluster), but no barrier per level: CTA c computes the rows it stores
// (rows [c * chunk, (c + 1) * chunk)), each thread takes every blockDim-th of its CTA's rows in
// level order, and a row waits only for the entries it reads.  An entry's readiness is its own
// value: every slot starts as PCA_EMPTY, a signalling-NaN bit pattern that no floating-point
// operation produces (arithmetic on NaN returns a quiet NaN), and a single aligned 8-byte store
// makes the value visible, so no separate flag is needed.  Deadlock cannot occur: every thread
// walks its rows in non-decreasing level order, rows read only rows of strictly lower levels
// (forward) or higher levels (backward, walked in reverse), and all CTAs of a cluster are
// resident together.  Every wait is bounded; on timeout the kernel records DS_WAIT_TIMEOUT, stops
// waiting everywhere and finishes with invalid values.  Per row the updates are the reference's,
// in the reference's order, each one fused multiply-subtract.
constexpr int PCA_THREADS = 256;
constexpr long long PCA_SPIN_LIMIT = 1LL << 22;
// Value-type traits of the barrier-free preconditioner (FP64 drop-in form, FP32 inner solve of the
// mixed-precision form).  EMPTY is a signalling-NaN bit pattern: no floating-point operation
// produces it (arithmetic on a NaN returns a quiet NaN).
template <typename T> struct Pca;
template <> struct Pca<double> {
    typedef unsigned long long Bits;
    static constexpr Bits EMPTY = 0x7FF4DEADBEEF0001ull;
    // Polls are plain (weak) loads of shared-memory slots kept in place by asm volatile: shared
    // memory is not cached, so each one reads the slot's current contents, and an aligned store is seen
    // whole or not at all.  The value itself is the signal, so nothing else needs ordering; the
    // cluster barrier at the end of each sweep orders everything for what follows.  (Loads with
    // .relaxed.cluster semantics measured about 20x slower per polling pass with every warp of
    // the cluster polling.)
    static __device__ __forceinline__ Bits ld(const void* a) {
        Bits v;
        asm volatile("ld.b64 %0, [%1];" : "=l"(v) : "l"(a) : "memory");
        return v;
    }
    static __device__ __forceinline__ void st(uint32_t a, double v) {
        asm volatile("st.shared.b64 [%0], %1;" ::"r"(a), "l"((Bits)__double_as_longlong(v)) : "memory");
    }
    static __device__ __forceinline__ double val(Bits b) { return __longlong_as_double((long long)b); }
};
template <> struct Pca<float> {
    typedef unsigned int Bits;
    static constexpr Bits EMPTY = 0x7FA5DEADu;
    static __device__ __forceinline__ Bits ld(const void* a) {
        Bits v;
        asm volatile("ld.b32 %0, [%1];" : "=r"(v) : "l"(a) : "memory");
        return v;
    }
    static __device__ __forceinline__ void st(uint32_t a, float v) {
        asm volatile("st.shared.b32 [%0], %1;" ::"r"(a), "r"(__float_as_uint(v)) : "memory");
    }
    static __device__ __forceinline__ float val(Bits b) { return __uint_as_float(b); }
};
// per-precision arrays of the preconditioner (the schedule and columns are shared)
template <typename T> struct PcaData {
    const T* fvalP;  // PC_MAXE x rowsCap, level-ordered factor values (forward / backward)
    const T* bvalP;
    const T* linvd;  // pivot reciprocals at each position
    const T* rl;     // right-hand side at each position
    T* yl;           // forward result at each position
    const T* fval;   // compact entries (read beyond PC_MAXE)
    const T* bval;
};
template <typename T> struct PcaRow {
    int p, self, cnt;
    T rhs, invd;
    int col[PC_MAXE];
    T val[PC_MAXE];
};
// record of position p (valid when q < cnt): independent loads only
template <typename T>
__device__ __forceinline__ void pca_load(const Proj& P, const PcaData<T>& D, int base, int q, int rows, bool fwd,
                                         PcaRow<T>& w) {
    w.cnt = -1;
    if (q < 0 || q >= rows) return;
    const int p = base + q;
    const int cap = P.rowsCap;
    const int* cc = fwd ? P.fcolP : P.bcolP;
    const T* vv = fwd ? D.fvalP : D.bvalP;
    w.p = p;
    w.self = P.lself[p];
    w.cnt = fwd ? P.lcntF[p] : P.lcntB[p];
    w.invd = D.linvd[p];
    w.rhs = fwd ? D.rl[p] : D.yl[p];
#pragma unroll
    for (int e = 0; e < PC_MAXE; ++e) {
        w.col[e] = cc[(size_t)e * cap + p];
        w.val[e] = vv[(size_t)e * cap + p];
    }
}
// One row per lane; the warp polls until every lane's row is done.  A lane stores its row the
// moment its last entry arrives, so no lane ever waits for a lane of its own warp while holding its
// own result back.  The loop and its exit are warp-uniform.  Entry addresses are resolved once per
// row into generic addresses: a slot of the CTA's own shared memory is read there directly, a slot
// of another CTA through the cluster's distributed shared memory, with one load form for both
// (measured 2-3 % faster than routing every entry through the cluster window); every pass
// re-loads all entries still missing, so they resolve in parallel.  Bounded: after PCA_SPIN_LIMIT
// polls (or once any wait of the launch has given up) the warp stops waiting and reports.
constexpr int PCA_MAXE = 2 * PC_MAXE;  // entries a row resolves in registers (8 from the record)
// The polling pass is integer-only: it re-loads the entries not yet known to hold values and
// extends the prefix of present ones.  The arithmetic runs once per row, after every entry is
// present, in the reference's order (FP64 issue is scarce on this part, and predicated-off FP64
// instructions in a polling pass would still occupy the FP64 pipe on every pass).
// generic address of packed entry (owner << 24 | local): the CTA's own slots resolve to its shared
// memory, other CTAs' slots to the cluster's distributed shared memory
template <typename T>
__device__ __forceinline__ const T* pca_gptr(T* const* win, int packed) {
    return win[packed >> 24] + (packed & 0xffffff);
}
template <typename T, bool UNFUSED>
__device__ __forceinline__ void pca_solve_row(const Proj& P, const PcaData<T>& D, const PcaRow<T>& w, bool fwd,
                                              uint32_t own, T* const* win, int* status) {
    typedef Pca<T> K;
    typedef typename K::Bits Bits;
    const uint32_t es = sizeof(T);
    bool done = w.cnt < 0;
    const T* a[PCA_MAXE];
    T val[PCA_MAXE];
#pragma unroll
    for (int e = 0; e < PC_MAXE; ++e) {
        a[e] = pca_gptr(win, w.col[e]);
        val[e] = w.val[e];
    }
    // entries 8..15 of a longer row: loaded once, together, before any polling
    const int* oc = fwd ? P.fcol : P.bcol;
    const T* ov = fwd ? D.fval : D.bval;
    const int q0 = (!done && w.cnt > PC_MAXE) ? (fwd ? P.fptr : P.bptr)[w.p] : 0;
#pragma unroll
    for (int e = PC_MAXE; e < PCA_MAXE; ++e) {
        bool has = e < w.cnt;
        a[e] = pca_gptr(win, has ? oc[q0 + e] : 0);
        val[e] = has ? ov[q0 + e] : T(0);
    }
    const int lim = min(w.cnt, PCA_MAXE);
    Bits v[PCA_MAXE];
    int got = 0;        // leading entries known to hold values
    bool part = false;  // the first lim entries are accumulated (rows longer than PCA_MAXE)
    T acc = w.rhs;
    for (long long it = 0;; ++it) {
        if (!done) {
            if (!part) {
                const int g0 = got;
#pragma unroll
                for (int e = 0; e < PCA_MAXE; ++e)
                    if (e >= g0 && e < lim) v[e] = K::ld(a[e]);
#pragma unroll
                for (int e = 0; e < PCA_MAXE; ++e)
                    if (e == got && e < lim && v[e] != K::EMPTY) got = e + 1;
                if (got == lim) {
#pragma unroll
                    for (int e = 0; e < PCA_MAXE; ++e) {
                        if (e >= lim) break;
                        acc = sweep_update(UNFUSED, acc, val[e], K::val(v[e]));
                    }
                    part = true;
                }
            }
            // rows longer than PCA_MAXE entries: the rest one at a time from the compact arrays
            while (part && got < w.cnt) {
                Bits x = K::ld(pca_gptr(win, oc[q0 + got]));
                if (x == K::EMPTY) break;
                acc = sweep_update(UNFUSED, acc, ov[q0 + got], K::val(x));
                ++got;
            }
            if (part && got >= w.cnt) {
                T y = acc * w.invd;
                if (fwd) D.yl[w.p] = y;
                K::st(own + (uint32_t)w.self * es, y);
                done = true;
            }
        }
        if (__all_sync(0xffffffffu, done)) break;
        if ((it & 255) == 255) {
            bool over = it > PCA_SPIN_LIMIT;
            if (over) atomicCAS(status, 0, DS_WAIT_TIMEOUT);
            if (__any_sync(0xffffffffu, over || *(volatile int*)status != 0)) break;
        }
    }
}
template <typename T, bool UNFUSED>
__global__ void __launch_bounds__(PCA_THREADS, 1) k_precond_async(Proj P, PcaData<T> D, T* z, int* status, int lgCS) {
    grid_dep_wait();
    typedef Pca<T> K;
    if (*P.done) return;
    extern __shared__ __align__(16) unsigned char pca_smem[];
    typename K::Bits* zraw = reinterpret_cast<typename K::Bits*>(pca_smem);
    T* zsh = reinterpret_cast<T*>(pca_smem);
    cg::cluster_group cl = cg::this_cluster();
    const int rank = cl.block_rank();
    const int n = *P.nDof, chunk = *P.chunk;
    const int base = P.ownStart[rank];
    const int rows = P.ownStart[rank + 1] - base;
    const int lgB = P.pcLgBlock;
    const uint32_t own = (uint32_t)__cvta_generic_to_shared(pca_smem);
    __shared__ T* win[16];
    if (threadIdx.x < cl.num_blocks()) win[threadIdx.x] = cl.map_shared_rank(zsh, (int)threadIdx.x);
    if (threadIdx.x == rank) win[threadIdx.x] = zsh;
    for (int l = threadIdx.x; l < chunk; l += blockDim.x) zraw[l] = K::EMPTY;
    cl.sync();  // every CTA is running and every slot of the cluster is empty
    for (int dir = 0; dir < 2; ++dir) {
        const bool fwd = dir == 0;
        // list index k of this CTA's walk -> position offset (forward: ascending levels, backward:
        // descending)
        auto qof = [&](int k) { return fwd ? k : rows - 1 - k; };
        // thread t takes entries t, t + blockDim, ...: the same number of rounds for every thread,
        // so warps stay whole; the next record is loaded while the current row waits
        const int T_ = (int)blockDim.x;
        const int rounds = (rows + T_ - 1) / T_;
        auto pick = [&](int k) {
            int q = threadIdx.x + k * T_;
            return q < rows ? qof(q) : -1;
        };
        PcaRow<T> W, X;
        pca_load(P, D, base, pick(0), rows, fwd, W);
        for (int k = 0; k < rounds; ++k) {
            pca_load(P, D, base, pick(k + 1), rows, fwd, X);
            pca_solve_row<T, UNFUSED>(P, D, W, fwd, own, win, status);
            W = X;
        }
        cl.sync();  // sweep finished everywhere (global and shared writes ordered at cluster scope)
        if (fwd) {
            for (int l = threadIdx.x; l < chunk; l += blockDim.x) zraw[l] = K::EMPTY;
            cl.sync();
        }
    }
    // local slot l holds row ((l >> lgB) << lgCS | rank) << lgB | (l mod B)
    for (int l = threadIdx.x; l < chunk; l += blockDim.x) {
        int j = ((((l >> lgB) << lgCS) | rank) << lgB) | (l & ((1 << lgB) - 1));
        if (j < n) z[j] = zsh[l];
    }
}
// how many clusters of the barrier-free preconditioner (FP64 or FP32 form) can be resident at
// once, at most 8: the number of solves that can run side by side on disjoint SMs
int precond_concurrency(const Proj& P, bool fp32) {
    if (P.pcCluster <= 0) return 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(P.pcCluster);
    cfg.blockDim = dim3(PCA_THREADS);
    cfg.dynamicSmemBytes = fp32 ? P.pcSmem32 : P.pcSmem;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = P.pcCluster;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    const void* k = fp32 ? (const void*)k_precond_async<float, false> : (const void*)k_precond_async<double, false>;
    int nc = 0;
    if (cudaOccupancyMaxActiveClusters(&nc, k, &cfg) != cudaSuccess) {
        cudaGetLastError();
        nc = 1;
    }
    return std::max(1, std::min(nc, 8));
}
static cudaError_t launch_precond_dsmem(const Proj& P, const double* r, double* z, cudaStream_t st) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(P.pcCluster);
    cfg.blockDim = dim3(PC_THREADS);
    cfg.dynamicSmemBytes = P.pcSmem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = P.pcCluster;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    count_launch();
    (void)r;
    return cudaLaunchKernelEx(&cfg, k_precond_dsmem, P, z, log2_exact(P.pcCluster));
}
template <typename T>
static cudaError_t launch_precond_async(const Dev& d, const Proj& P, const PcaData<T>& D, T* z, size_t smem,
                                       cudaStream_t st) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(P.pcCluster);
    cfg.blockDim = dim3(PCA_THREADS);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[2];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = P.pcCluster;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    at[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;  // see launch_pdl
    at[1].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 2;
    count_launch();
    if (P.unfused) return cudaLaunchKernelEx(&cfg, k_precond_async<T, true>, P, D, z, d.status, log2_exact(P.pcCluster));
    return cudaLaunchKernelEx(&cfg, k_precond_async<T, false>, P, D, z, d.status, log2_exact(P.pcCluster));
}
static PcaData<double> pca_data64(const Proj& P) {
    return PcaData<double>{P.fvalP, P.bvalP, P.linvd, P.rl, P.yl, P.fval, P.bval};
}
// Cluster size (16, else 8) at which the fused preconditioner (barrier-free form when async) can
// run with the largest dynamic shared memory a CTA may have, or 0; *smemMax = that largest size.
// Each solve then uses ceil(n / CS) doubles per CTA and falls back to the global-memory sweeps
// when they do not fit.
int choose_dsmem_cluster(bool async, size_t* smemMax) {
    const void* kern = async ? (const void*)k_precond_async<double, false> : (const void*)k_precond_dsmem;
    const int threads = async ? PCA_THREADS : PC_THREADS;
    *smemMax = 0;
    cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    // the attribute is process-wide: allow the device maximum (minus the kernel's static shared
    // memory) once, size each launch per solve
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, kern) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    optin -= (int)fa.sharedSizeBytes;
    if (optin <= 0 || cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, optin) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    if (async) {  // the FP32 instance of the mixed-precision solve: same launch shape
        // the other instances (FP32 of the mixed-precision solve; the reference order's separate
        // multiply and subtract): same launch shape
        const void* others[3] = {(const void*)k_precond_async<float, false>, (const void*)k_precond_async<float, true>,
                                 (const void*)k_precond_async<double, true>};
        for (const void* k2 : others) {
            cudaFuncSetAttribute(k2, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
            if (cudaFuncSetAttribute(k2, cudaFuncAttributeMaxDynamicSharedMemorySize, optin) != cudaSuccess) {
                cudaGetLastError();
                return 0;
            }
        }
    }
    for (int cs : {16, 8}) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(cs);
        cfg.blockDim = dim3(threads);
        cfg.dynamicSmemBytes = (size_t)optin;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = cs;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        int nc = 0;
        cudaError_t e = cudaOccupancyMaxActiveClusters(&nc, kern, &cfg);
        if (getenv("ASTG_VERBOSE"))
            fprintf(stderr, "astg: %s preconditioner cluster %d, up to %d B smem/CTA: %d clusters (%s)\n",
                    async ? "barrier-free" : "level-barrier", cs, optin, nc, cudaGetErrorString(e));
        if (e == cudaSuccess && nc > 0) {
            *smemMax = (size_t)optin;
            return cs;
        }
        cudaGetLastError();
    }
    return 0;
}
static cudaError_t launch_cluster(void (*kern)(Proj, const double*, double*), int csize, cudaStream_t st, Proj P,
                                  const double* r, double* z) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(csize);
    cfg.blockDim = dim3(CLUSTER_THREADS);
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = csize;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    count_launch();
    return cudaLaunchKernelEx(&cfg, kern, P, r, z);
}
// largest cluster size (16, 8, 4, 2) that can be resident for the sweep kernels
int choose_cluster_size(int device) {
    (void)device;
    cudaFuncSetAttribute((const void*)k_sweep_fwd_cluster, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    cudaFuncSetAttribute((const void*)k_sweep_bwd_cluster, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    for (int cs : {16, 8, 4, 2}) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(cs);
        cfg.blockDim = dim3(CLUSTER_THREADS);
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = cs;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        int nc = 0;
        if (cudaOccupancyMaxActiveClusters(&nc, (const void*)k_sweep_fwd_cluster, &cfg) == cudaSuccess && nc > 0) {
            int nc2 = 0;
            if (cudaOccupancyMaxActiveClusters(&nc2, (const void*)k_sweep_bwd_cluster, &cfg) == cudaSuccess && nc2 > 0)
                return cs;
        }
        cudaGetLastError();
    }
    return 0;
}
// ---- owner-major schedule of the barrier-free preconditioner.  Rows are dealt to the CTAs in
// blocks of B = 2^lgB consecutive rows, round robin: row j is computed by, and keeps its value in,
// CTA (j >> lgB) mod CS at local slot ((j >> (lgB + lgCS)) << lgB) | (j mod B).  Consecutive rows
// (x neighbours, mostly y neighbours) share a CTA while every dependency level is spread over
// all CTAs.  Each CTA's rows are sorted by level, so a row's dependencies always come earlier in
// some CTA's walk.  Keys (owner, level) are counted, scanned and scattered.
__device__ __forceinline__ int own_of(int j, int lgB, int lgCS) { return (j >> lgB) & ((1 << lgCS) - 1); }
__device__ __forceinline__ int local_of(int j, int lgB, int lgCS) {
    return ((j >> (lgB + lgCS)) << lgB) | (j & ((1 << lgB) - 1));
}
// column k as (owner CTA << 24 | local slot)
__device__ __forceinline__ int pack_owner(int k, int lgB, int lgCS) {
    return (own_of(k, lgB, lgCS) << 24) | local_of(k, lgB, lgCS);
}
__global__ void k_own_setup(Proj P, int cs, long long keys) {
    long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j < keys) { P.ownCnt[j] = 0; P.ownFill[j] = 0; }
    if (j == 0) {
        int B = 1 << P.pcLgBlock;
        int blocks = (*P.nDof + B - 1) / B;
        *P.chunk = ((blocks + cs - 1) / cs) * B;
    }
}
__global__ void k_own_hist(Proj P, int rows1, int lgCS) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= *P.nDof) return;
    atomicAdd(P.ownCnt + (long long)own_of(j, P.pcLgBlock, lgCS) * rows1 + P.level[j], 1);
}
__global__ void k_own_scatter(Proj P, int rows1, int lgCS) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= *P.nDof) return;
    long long key = (long long)own_of(j, P.pcLgBlock, lgCS) * rows1 + P.level[j];
    int p = P.ownPtr[key] + atomicAdd(P.ownFill + key, 1);
    P.perm[p] = j;
    P.pos[j] = p;
}
__global__ void k_own_bounds(Proj P, int rows1, int cs) {
    int c = threadIdx.x;
    if (c < cs) P.ownStart[c] = P.ownPtr[(long long)c * rows1];
    if (c == cs) P.ownStart[cs] = *P.nDof;
}
__global__ void k_own_fill(Proj P, int lgCS) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= *P.nDof) return;
    int i = P.perm[p];
    int dg = P.diagPos[i];
    int lgB = P.pcLgBlock;
    int cap = P.rowsCap;
    P.lself[p] = local_of(i, lgB, lgCS);
    P.linvd[p] = P.invdiag[i];
    int nf = dg - P.rowPtr[i], nb = P.rowPtr[i + 1] - dg - 1;
    P.lcntF[p] = nf;
    P.lcntB[p] = nb;
    P.cntF[p] = nf;
    P.cntB[p] = nb;
    for (int e = 0; e < PC_MAXE; ++e) {
        int qf = P.rowPtr[i] + e, qb = dg + 1 + e;
        P.fcolP[(size_t)e * cap + p] = e < nf ? pack_owner(P.col[qf], lgB, lgCS) : 0;
        P.fvalP[(size_t)e * cap + p] = e < nf ? P.Lv[P.tpos[qf]] : 0.0;
        P.bcolP[(size_t)e * cap + p] = e < nb ? pack_owner(P.col[qb], lgB, lgCS) : 0;
        P.bvalP[(size_t)e * cap + p] = e < nb ? P.Lv[qb] : 0.0;
        if (P.fvalP32) {  // the factor is computed in FP64 and rounded once
            P.fvalP32[(size_t)e * cap + p] = (float)P.fvalP[(size_t)e * cap + p];
            P.bvalP32[(size_t)e * cap + p] = (float)P.bvalP[(size_t)e * cap + p];
        }
    }
    if (P.linvd32) P.linvd32[p] = (float)P.invdiag[i];
}
// all entries of the row at position p, packed, in the compact arrays (read beyond PC_MAXE)
__global__ void k_own_overflow(Proj P, int lgCS) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= *P.nDof) return;
    int i = P.perm[p];
    int dg = P.diagPos[i];
    int lgB = P.pcLgBlock;
    int o = P.fptr[p];
    for (int q = P.rowPtr[i]; q < dg; ++q, ++o) {
        P.fcol[o] = pack_owner(P.col[q], lgB, lgCS);
        P.fval[o] = P.Lv[P.tpos[q]];
        if (P.fval32) P.fval32[o] = (float)P.fval[o];
    }
    o = P.bptr[p];
    for (int q = dg + 1; q < P.rowPtr[i + 1]; ++q, ++o) {
        P.bcol[o] = pack_owner(P.col[q], lgB, lgCS);
        P.bval[o] = P.Lv[q];
        if (P.bval32) P.bval32[o] = (float)P.bval[o];
    }
}
static void launch_owner_schedule(const Dev& d, Proj& P, cudaStream_t st) {
    (void)d;
    int maxRows = P.rowsCap;
    int cs = P.pcCluster, lgCS = log2_exact(cs);
    long long keys = (long long)cs * (maxRows + 1);
    ASTG_LAUNCH(k_own_setup<<<nblk(keys), TB, 0, st>>>(P, cs, keys));
    ASTG_LAUNCH(k_own_hist<<<nblk(maxRows), TB, 0, st>>>(P, maxRows + 1, lgCS));
    exclusive_scan(P.ownCnt, P.ownPtr, P.bsum, P.nnz + 1, keys, st);
    ASTG_LAUNCH(k_own_bounds<<<1, 32, 0, st>>>(P, maxRows + 1, cs));
    ASTG_LAUNCH(k_own_scatter<<<nblk(maxRows), TB, 0, st>>>(P, maxRows + 1, lgCS));
    ASTG_LAUNCH(k_own_fill<<<nblk(maxRows), TB, 0, st>>>(P, lgCS));
    exclusive_scan(P.cntF, P.fptr, P.bsum, P.nnz + 2, maxRows, st);
    exclusive_scan(P.cntB, P.bptr, P.bsum, P.nnz + 3, maxRows, st);
    ASTG_LAUNCH(k_level_fptr_last<<<1, 1, 0, st>>>(P));
    ASTG_LAUNCH(k_own_overflow<<<nblk(maxRows), TB, 0, st>>>(P, lgCS));
}

void launch_level_schedule(const Dev& d, Proj& P, bool owner, cudaStream_t st) {
    if (owner) {
        launch_owner_schedule(d, P, st);
        return;
    }
    int maxRows = P.rowsCap;
    ASTG_LAUNCH(k_level_reset<<<nblk(maxRows + 1), TB, 0, st>>>(P, maxRows));
    ASTG_LAUNCH(k_level_hist<<<nblk(maxRows), TB, 0, st>>>(P));

    exclusive_scan(P.levelCnt, P.levelPtr, P.bsum, P.nnz + 1, maxRows + 1, st);
    ASTG_LAUNCH(k_level_scatter<<<nblk(maxRows), TB, 0, st>>>(P));
    ASTG_LAUNCH(k_level_counts<<<nblk(maxRows), TB, 0, st>>>(P));
    exclusive_scan(P.cntF, P.fptr, P.bsum, P.nnz + 2, maxRows, st);
    exclusive_scan(P.cntB, P.bptr, P.bsum, P.nnz + 3, maxRows, st);
    ASTG_LAUNCH(k_level_fptr_last<<<1, 1, 0, st>>>(P));
    ASTG_LAUNCH(k_level_fill<<<nblk(maxRows), TB, 0, st>>>(P));
}

// ------------------------------------------------------------------ triangular sweeps (FP64)
// solve_lower (:196-208) row-oriented and solve_lower_transpose_in_place (:226-238); same
// per-row operation order as the reference's column-oriented loops
__global__ void k_sweep_fwd(Dev d, Proj P, const double* r, double* z, int epoch) {
    if (*P.done) return;
    int n = *P.nDof;
    for (;;) {
        int i = grab_row(P.counter);
        if (i >= n) return;
        double acc = r[i];
        int q0 = P.rowPtr[i], dg = P.diagPos[i];
        int qend = dg >= 0 ? dg : P.rowPtr[i + 1];
        for (int q = q0; q < qend; ++q) {
            int k = P.col[q];
            if (k >= i) break;
            wait_flag(d, P.ready + k, epoch);
            acc = sweep_update(P.unfused != 0, acc, P.Lv[P.tpos[q]], z[k]);
        }
        z[i] = acc * P.invdiag[i];
        __threadfence();
        st_flag(P.ready + i, epoch);
    }
}
__global__ void k_sweep_bwd(Dev d, Proj P, double* z, int epoch) {
    if (*P.done) return;
    int n = *P.nDof;
    for (;;) {
        int g = grab_row(P.counter);
        if (g >= n) return;
        int i = n - 1 - g;
        double acc = z[i];
        int dg = P.diagPos[i];
        int q0 = dg >= 0 ? dg + 1 : P.rowPtr[i];
        for (int q = q0; q < P.rowPtr[i + 1]; ++q) {
            int c = P.col[q];
            if (c <= i) continue;
            wait_flag(d, P.ready + c, epoch);
            acc = sweep_update(P.unfused != 0, acc, P.Lv[q], z[c]);
        }
        z[i] = acc * P.invdiag[i];
        __threadfence();
        st_flag(P.ready + i, epoch);
    }
}

// ------------------------------------------------------------------ PCG (FP64)
// PCGSolver::solve(VectorXd), include/pcgsolver/pcg_solver.h:366-426
__global__ void k_copy(const double* a, double* b, const int* nptr) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < *nptr) b[i] = a[i];
}
// right-hand side of the preconditioner in level order
__global__ void k_to_level_order(Proj P, const double* r) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < *P.nDof) P.rl[P.pos[i]] = r[i];
}
// the residual of a cell row in the wavefront preconditioner's diagonal-major order (Proj::wave)
__device__ __forceinline__ void wave_put_r(const Proj& P, int i, double ri) {
    const int nx = P.wnx;
    if (i < nx * P.wny) {
        const int x = i % nx;
        P.wR[x + (x + i / nx) * nx] = ri;
    }
}
__global__ void k_to_wave_order(Proj P, const double* r) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < *P.nDof) wave_put_r(P, i, r[i]);
}
__global__ void k_zero_vec(double* a, const int* nptr) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < *nptr) a[i] = 0;
}
// max |a| over [0, n): non-negative doubles order like their bit patterns
// the largest of the block's v (all threads of the block call it) into *out: a warp maximum by
// shuffles, the block's over its warps in shared memory, one atomic per block (non-negative doubles
// order as their bit patterns).  One atomic per warp on the same word serialised at the L2.
__device__ __forceinline__ void block_absmax_to(double v, unsigned long long* out) {
    __shared__ double wm[32];
    for (int o = 16; o > 0; o >>= 1) {
        double w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w > v ? w : v;
    }
    if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double m = wm[0];
        for (int k = 1; k < (int)((blockDim.x + 31) >> 5); ++k) m = wm[k] > m ? wm[k] : m;
        if (m > 0) atomicMax(out, (unsigned long long)__double_as_longlong(m));
    }
}
__global__ void k_absmax(const double* a, const int* nptr, unsigned long long* out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v = 0;
    if (i < *nptr) v = fabs(a[i]);
    block_absmax_to(v, out);
}
__global__ void k_pcg_start(Proj P, const double* partRho, double tolFactor) {
    __shared__ double sh[RED_LANES];
    int n = *P.nDof;
    long long m = (n + RED_CHUNK - 1) / RED_CHUNK;
    double rho = fold_partials(partRho, m, sh);
    if (threadIdx.x == 0) {
        double r0 = __longlong_as_double((long long)*P.amax);
        P.sc[SC_RESID0] = r0;
        P.sc[SC_TOL] = P.tolAbsolute ? tolFactor : tolFactor * r0;
        P.sc[SC_RHO] = rho;
        P.sc[SC_RESID] = r0;
        if (r0 == 0) { *P.done = 1; P.isc[ISC_ITERS] = 0; P.isc[ISC_CONVERGED] = 1; }
        else if (rho == 0 || rho != rho) { *P.done = 1; P.isc[ISC_ITERS] = 0; P.isc[ISC_CONVERGED] = 0; }
        else { *P.done = 0; P.isc[ISC_ITERS] = 0; P.isc[ISC_CONVERGED] = 0; }
        *P.amax = 0;
    }
}
// z = A s, partial dots of s . z (lane layout of the fixed tree: thread t owns rows t + 256 k)
// y = A s over one chunk of RED_CHUNK rows, SPMV_THREADS threads per chunk (each row summed in
// column order by one thread, staged in shared memory), then the chunk's partial of s . y in the
// fixed tree's order: lane t adds rows t, t + 256, ... of the chunk, the lanes fold by halving.
// Four times the threads of one lane per 8 rows, same values bit for bit.
constexpr int SPMV_THREADS = 1024;
__device__ __forceinline__ double chunk_fold(double acc, double* sh) {
    const int t = threadIdx.x;
    if (t < RED_LANES) sh[t] = acc;
    __syncthreads();
    for (int st = RED_LANES / 2; st >= 1; st >>= 1) {
        if (t < st) sh[t] = sh[t] + sh[t + st];
        __syncthreads();
    }
    return sh[0];
}
// FUSED (the library's order): each product-accumulate is one fused multiply-add; otherwise (the
// reference's order) a product, then an addition, as its CSR multiply computes them
template <bool FUSED>
__device__ __forceinline__ double mac_add(double acc, double a, double b) {
    if (FUSED) return fma(a, b, acc);
    double prod = a * b;
    return acc + prod;
}
template <bool FUSED>
__global__ void __launch_bounds__(SPMV_THREADS) k_spmv_dot(Proj P, const double* s, double* z, double* part) {
    grid_dep_wait();
    __shared__ double ys[RED_CHUNK];
    __shared__ double sh[RED_LANES];
    if (*P.done) return;
    int n = *P.nDof;
    long long base = (long long)blockIdx.x * RED_CHUNK;
    if (base >= n) return;
    for (int k = threadIdx.x; k < RED_CHUNK; k += SPMV_THREADS) {
        long long i = base + k;
        double t = 0;
        if (i < n) {
            for (int q = P.rowPtr[i]; q < P.rowPtr[i + 1]; ++q) t = mac_add<FUSED>(t, P.val[q], s[P.col[q]]);
            z[i] = t;
        }
        ys[k] = t;
    }
    __syncthreads();
    const int tl = threadIdx.x;
    double acc = 0.0;
    if (tl < RED_LANES)
        for (int k = 0; k < RED_PER_LANE; ++k) {
            long long i = base + tl + (long long)RED_LANES * k;
            if (i < n) acc = mac_add<FUSED>(acc, s[i], ys[tl + RED_LANES * k]);
        }
    double r = chunk_fold(acc, sh);
    if (tl == 0) part[blockIdx.x] = r;
}
__global__ void k_alpha(Proj P, const double* part) {
    grid_dep_wait();
    __shared__ double sh[RED_LANES];
    if (*P.done) return;
    int n = *P.nDof;
    long long m = (n + RED_CHUNK - 1) / RED_CHUNK;
    double dsz = fold_partials(part, m, sh);
    if (threadIdx.x == 0) P.sc[SC_ALPHA] = P.sc[SC_RHO] / dsz;
}
template <bool FUSED>
__global__ void k_update_xr(Proj P, double* x, double* r, const double* s, const double* z) {
    grid_dep_wait();
    if (*P.done) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int n = *P.nDof;
    double alpha = P.sc[SC_ALPHA];
    double v = 0;
    if (i < n) {
        x[i] = mac_add<FUSED>(x[i], alpha, s[i]);
        double ri = mac_add<FUSED>(r[i], -alpha, z[i]);
        r[i] = ri;
        if (P.pcActive) P.rl[P.pos[i]] = ri;
        if (P.wave) wave_put_r(P, i, ri);
        v = fabs(ri);
    }
    block_absmax_to(v, P.amax);
}
__global__ void k_check(Proj P, int maxIter) {
    grid_dep_wait();
    if (*P.done) return;
    double res = __longlong_as_double((long long)*P.amax);
    *P.amax = 0;
    int it = P.isc[ISC_ITERS];
    P.sc[SC_RESID] = res;
    if (res <= P.sc[SC_TOL]) {
        P.isc[ISC_ITERS] = it + 1;
        P.isc[ISC_CONVERGED] = 1;
        *P.done = 1;
    } else if (it + 1 >= maxIter) {
        P.isc[ISC_ITERS] = it + 1;
        P.isc[ISC_CONVERGED] = 0;
        *P.done = 1;
    } else {
        P.isc[ISC_ITERS] = it + 1;
    }
}
__global__ void k_beta(Proj P, const double* part) {
    grid_dep_wait();
    __shared__ double sh[RED_LANES];
    if (*P.done) return;
    int n = *P.nDof;
    long long m = (n + RED_CHUNK - 1) / RED_CHUNK;
    double rn = fold_partials(part, m, sh);
    if (threadIdx.x == 0) {
        P.sc[SC_BETA] = rn / P.sc[SC_RHO];
        P.sc[SC_RHO] = rn;
    }
}
template <bool FUSED>
__global__ void k_update_s(Proj P, double* s, const double* z) {
    grid_dep_wait();
    if (*P.done) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= *P.nDof) return;
    s[i] = mac_add<FUSED>(z[i], P.sc[SC_BETA], s[i]);
}
__global__ void k_reset_counter(int* c) { *c = 0; }

// one preconditioner application z = (L L^T)^-1 r
void select_preconditioner(Proj& P, int n) {
    P.pcActive = 0;
    P.pcSmem = 0;
    P.pcActive32 = 0;
    P.pcSmem32 = 0;
    if (P.pcCluster <= 0 || n <= 0) return;
    size_t slots = (size_t)((n + P.pcCluster - 1) / P.pcCluster);
    if (P.pcAsync) {  // whole ownership blocks per CTA
        size_t B = (size_t)1 << P.pcLgBlock, blocks = (n + B - 1) / B;
        slots = (blocks + P.pcCluster - 1) / P.pcCluster * B;
    }
    size_t bytes = slots * sizeof(double);
    if (n > P.rowsCap) return;
    if (P.pcAsync && P.val32 && slots * sizeof(float) <= P.pcSmemMax) {
        P.pcActive32 = 1;
        P.pcSmem32 = slots * sizeof(float);
    }
    if (bytes > P.pcSmemMax) return;
    P.pcActive = 1;
    P.pcSmem = bytes;
}
static void precond(const Dev& d, Proj& P, const double* r, double* z, int& epoch, cudaStream_t st, KProf* prof) {
    if (P.wave) {
        prof_begin(prof, 0, st);
        launch_precond_wave(P, r, z, st);
        prof_end(prof, st);
        return;
    }
    if (P.pcActive) {
        prof_begin(prof, 0, st);
        cudaError_t e = P.pcAsync ? launch_precond_async(d, P, pca_data64(P), z, P.pcSmem, st)
                                  : launch_precond_dsmem(P, r, z, st);
        prof_end(prof, st);
        if (e != cudaSuccess) g_cluster_error = e;
        return;
    }
    if (P.clusterSize > 0) {
        prof_begin(prof, 0, st);
        cudaError_t e = launch_cluster(k_sweep_fwd_cluster, P.clusterSize, st, P, r, z);
        prof_end(prof, st);
        prof_begin(prof, 1, st);
        cudaError_t e2 = launch_cluster(k_sweep_bwd_cluster, P.clusterSize, st, P, nullptr, z);
        prof_end(prof, st);
        if (e != cudaSuccess) g_cluster_error = e;
        if (e2 != cudaSuccess) g_cluster_error = e2;
        return;
    }
    int warps = P.sweepBlocks;
    ASTG_LAUNCH(k_reset_counter<<<1, 1, 0, st>>>(P.counter));
    prof_begin(prof, 0, st);
    ASTG_LAUNCH(k_sweep_fwd<<<warps, 128, 0, st>>>(d, P, r, z, ++epoch));
    prof_end(prof, st);
    ASTG_LAUNCH(k_reset_counter<<<1, 1, 0, st>>>(P.counter));
    prof_begin(prof, 1, st);
    ASTG_LAUNCH(k_sweep_bwd<<<warps, 128, 0, st>>>(d, P, z, ++epoch));
    prof_end(prof, st);
}

// ---- the factorisation with its merge plan computed first.  What k_mic_factor works out per
// (column j, earlier column k) while it waits on the chain -- which of k's entries are missing
// from j's pattern, which one is the diagonal, which entry of j each matched one updates -- depends
// on the pattern only, so one parallel pass records it and the chained pass only applies it: the
// same updates in the same order (bit-identical), with the loads of k's values independent of
// one another once k is ready.
enum { PLAN_NONE = 0, PLAN_MISSING = 1, PLAN_DIAG = 2, PLAN_MATCH = 3 };
__global__ void k_plan_count(Proj P, int* cnt) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= *P.nDof) return;
    for (int q = P.rowPtr[j]; q < P.rowPtr[j + 1]; ++q) {
        int k = P.col[q];
        cnt[q] = (k < j && P.adiag[k] != 0) ? P.rowPtr[k + 1] - (P.diagPos[k] + 1) : 0;
    }
}
__global__ void k_plan_fill(Proj P) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= *P.nDof) return;
    int rj0 = P.rowPtr[j], rj1 = P.rowPtr[j + 1];
    int dgj = P.diagPos[j];
    int upj = dgj >= 0 ? dgj + 1 : rj1;
    for (int qq = rj0; qq < rj1; ++qq) {
        int k = P.col[qq];
        if (k >= j) break;
        if (P.adiag[k] == 0) continue;
        int* out = P.plan + P.planPtr[qq];
        int a0 = P.diagPos[k] + 1, a = a0, ak = P.rowPtr[k + 1];
        if (P.planPtr[qq] + (ak - a0) > P.planCap) return;  // checked on the host through planTotal
        int b = rj0;
        while (a < ak && P.col[a] < j) {
            int code = PLAN_NONE;
            while (b < rj1) {
                if (P.col[b] < P.col[a]) ++b;
                else if (P.col[b] == P.col[a]) break;
                else { code = PLAN_MISSING; break; }
            }
            out[a - a0] = code;
            ++a;
        }
        if (a < ak) out[a - a0] = P.col[a] == j ? PLAN_DIAG : PLAN_NONE;
        ++a;
        int bb = upj;
        while (a < ak && bb < rj1) {
            if (P.col[bb] < P.col[a]) ++bb;
            else if (P.col[bb] == P.col[a]) { out[a - a0] = ((bb - upj) << 2) | PLAN_MATCH; ++a; ++bb; }
            else { out[a - a0] = PLAN_MISSING; ++a; }
        }
        while (a < ak) { out[a - a0] = PLAN_MISSING; ++a; }
    }
}
constexpr int PLAN_MAXU = 16;  // upper entries of a column applied from registers (more: in place)
constexpr int FACTOR_ROW = 24;  // a row's upper entries updated in a thread-local copy (longer rows: in place)
__global__ void k_mic_factor_plan(Dev d, Proj P, double omega, double minDiag, int epoch) {
    int n = *P.nDof;
    for (;;) {
        int j = grab_row(P.counter);
        if (j >= n) return;
        int rj0 = P.rowPtr[j], rj1 = P.rowPtr[j + 1];
        int dgj = P.diagPos[j];
        int upj = dgj >= 0 ? dgj + 1 : rj1;
        double invd = P.invdiag[j];
        int lev = 0;
        // row j's upper entries are written by this thread alone until its flag is set: they are
        // updated in a thread-local copy (L1) instead of read-modify-writes through L2, the same
        // operations in the same order
        const int nup = rj1 - upj;
        const bool own = nup <= FACTOR_ROW;
        double up[FACTOR_ROW];
        if (own)
            for (int q = 0; q < nup; ++q) up[q] = P.Lv[upj + q];
        for (int qq = rj0; qq < rj1; ++qq) {
            int k = P.col[qq];
            if (k >= j) break;
            const int pp = P.planPtr[qq], pe = P.planPtr[qq + 1];
            const int a0 = P.diagPos[k] + 1;
            const int tq = P.tpos[qq];
            int code[PLAN_MAXU];
            const int m = pe - pp;
#pragma unroll
            for (int u = 0; u < PLAN_MAXU; ++u) code[u] = u < m ? P.plan[pp + u] : PLAN_NONE;
            wait_flag(d, P.ready + k, epoch);
            lev = max(lev, P.level[k] + 1);
            if (m == 0 && P.adiag[k] == 0) continue;
            double mult = P.Lv[tq];
            double lv[PLAN_MAXU];
#pragma unroll
            for (int u = 0; u < PLAN_MAXU; ++u) lv[u] = (u < m && code[u] != PLAN_NONE) ? P.Lv[a0 + u] : 0.0;
            double missing = 0;
#pragma unroll
            for (int u = 0; u < PLAN_MAXU; ++u) {
                if (u >= m) break;
                int c = code[u] & 3;
                if (c == PLAN_MISSING) missing += lv[u];
                else if (c == PLAN_DIAG) invd -= mult * lv[u];
                else if (c == PLAN_MATCH) {
                    if (own) up[code[u] >> 2] -= mult * lv[u];
                    else P.Lv[upj + (code[u] >> 2)] -= mult * lv[u];
                }
            }
            for (int u = PLAN_MAXU; u < m; ++u) {
                int cu = P.plan[pp + u], c = cu & 3;
                double v = P.Lv[a0 + u];
                if (c == PLAN_MISSING) missing += v;
                else if (c == PLAN_DIAG) invd -= mult * v;
                else if (c == PLAN_MATCH) {
                    if (own) up[cu >> 2] -= mult * v;
                    else P.Lv[upj + (cu >> 2)] -= mult * v;
                }
            }
            invd -= omega * mult * missing;
        }
        double ad = P.adiag[j];
        if (ad != 0) {
            if (invd < minDiag * ad) invd = 1 / sqrt(ad);
            else invd = 1 / sqrt(invd);
            if (own)
                for (int q = 0; q < nup; ++q) up[q] *= invd;
            else
                for (int q = upj; q < rj1; ++q) P.Lv[q] *= invd;
        }
        if (own)
            for (int q = 0; q < nup; ++q) P.Lv[upj + q] = up[q];
        P.invdiag[j] = invd;
        P.level[j] = lev;
        __threadfence();
        st_flag(P.ready + j, epoch);
    }
}
void launch_factor(const Dev& d, Proj& P, double omega, double minDiag, int& epoch, cudaStream_t st, KProf* prof) {
    int maxRows = P.rowsCap;
    ASTG_LAUNCH(k_mic_init<<<nblk(maxRows), TB, 0, st>>>(P));
    ASTG_LAUNCH(k_reset_counter<<<1, 1, 0, st>>>(P.counter));
    bool plan = P.plan != nullptr;
    if (plan) {
        // counts in place (entries past nnz stay 0), exclusive scan in place: planPtr[q] = start of
        // entry q's codes, planPtr[nnz] = total
        long long nz = (long long)maxRows * ROW_W;
        cudaMemsetAsync(P.planPtr, 0, sizeof(int) * (nz + 1), st);
        ASTG_LAUNCH(k_plan_count<<<nblk(maxRows), TB, 0, st>>>(P, P.planPtr));
        exclusive_scan(P.planPtr, P.planPtr, P.bsum, P.planTotal, nz, st);
        int total = 0;
        cudaMemcpyAsync(&total, P.planTotal, sizeof total, cudaMemcpyDeviceToHost, st);
        cudaStreamSynchronize(st);
        plan = total >= 0 && total <= P.planCap;  // a larger plan: this solve uses the direct form
        if (plan) ASTG_LAUNCH(k_plan_fill<<<nblk(maxRows), TB, 0, st>>>(P));
    }
    prof_begin(prof, 3, st);
    if (plan) ASTG_LAUNCH(k_mic_factor_plan<<<P.sweepBlocks, 128, 0, st>>>(d, P, omega, minDiag, ++epoch));
    else ASTG_LAUNCH(k_mic_factor<<<P.sweepBlocks, 128, 0, st>>>(d, P, omega, minDiag, ++epoch));
    prof_end(prof, st);
}

// Runs the FP64 PCG to completion.  Iterations are launched in batches; every kernel returns at
// once when the device "done" flag is set, so a batch that overshoots does no work.
int launch_pcg_fp64(const Dev& d, Proj& P, double tolFactor, int maxIter, int& epoch, int batch, cudaStream_t st,
                    KProf* prof) {
    int maxRows = P.rowsCap;
    int chunks = (maxRows + RED_CHUNK - 1) / RED_CHUNK;
    double* x = P.x;
    double* r = P.r;
    double* s = P.s;
    double* z = P.z;
    ASTG_LAUNCH(k_zero_vec<<<nblk(maxRows), TB, 0, st>>>(x, P.nDof));
    ASTG_LAUNCH(k_copy<<<nblk(maxRows), TB, 0, st>>>(P.b, r, P.nDof));
    cudaMemsetAsync(P.amax, 0, sizeof(unsigned long long), st);
    cudaMemsetAsync(P.done, 0, sizeof(int), st);
    ASTG_LAUNCH(k_absmax<<<nblk(maxRows), TB, 0, st>>>(r, P.nDof, P.amax));
    if (P.pcActive) ASTG_LAUNCH(k_to_level_order<<<nblk(maxRows), TB, 0, st>>>(P, r));
    if (P.wave) ASTG_LAUNCH(k_to_wave_order<<<nblk(maxRows), TB, 0, st>>>(P, r));
    precond(d, P, r, z, epoch, st, prof);
    if (P.refOrder) launch_dot_ref(z, r, P.nDof, P.part, st);
    else ASTG_LAUNCH(k_tree_dot<<<chunks, RED_LANES, 0, st>>>(z, r, P.nDof, P.part));
    ASTG_LAUNCH(k_pcg_start<<<1, RED_LANES, 0, st>>>(P, P.part, tolFactor));
    ASTG_LAUNCH(k_copy<<<nblk(maxRows), TB, 0, st>>>(z, s, P.nDof));
    int launched = 0;
    int hostDone = 0;
    auto body = [&](int nb, KProf* pf) {
        for (int it = 0; it < nb; ++it) {
            prof_begin(pf, 2, st);
            if (P.refOrder) launch_pdl(k_spmv_dot<false>, chunks, SPMV_THREADS, st, P, s, z, P.part);
            else launch_pdl(k_spmv_dot<true>, chunks, SPMV_THREADS, st, P, s, z, P.part);
            prof_end(pf, st);
            if (P.refOrder) launch_dot_ref(s, z, P.nDof, P.part, st);
            launch_pdl(k_alpha, 1, RED_LANES, st, P, P.part);
            if (P.refOrder) launch_pdl(k_update_xr<false>, nblk(maxRows), TB, st, P, x, r, s, z);
            else launch_pdl(k_update_xr<true>, nblk(maxRows), TB, st, P, x, r, s, z);
            launch_pdl(k_check, 1, 1, st, P, maxIter);
            precond(d, P, r, z, epoch, st, pf);
            if (P.refOrder) launch_dot_ref(z, r, P.nDof, P.part, st);
            else launch_pdl(k_tree_dot, chunks, RED_LANES, st, z, r, P.nDof, P.part);
            launch_pdl(k_beta, 1, RED_LANES, st, P, P.part);
            if (P.refOrder) launch_pdl(k_update_s<false>, nblk(maxRows), TB, st, P, s, z);
            else launch_pdl(k_update_s<true>, nblk(maxRows), TB, st, P, s, z);
        }
    };
    BatchGraph graph;
    const bool graphs = g_pcg_graphs && (P.pcActive || P.clusterSize > 0);
    while (launched < maxIter) {
        int nb = batch;
        if (launched + nb > maxIter) nb = maxIter - launched;
        bool replayed = graphs && nb == batch && graph.run(body, nb, st, prof);
        if (!replayed) body(nb, prof);
        launched += nb;
        cudaMemcpyAsync(P.hostDone, P.done, sizeof(int), cudaMemcpyDeviceToHost, st);
        cudaStreamSynchronize(st);
        prof_drain(prof, replayed && graph.profiled);
        hostDone = *P.hostDone;
        if (hostDone) break;
    }
    return launched;
}

}  // namespace astg

namespace astg {
// ------------------------------------------------------------------ mixed-precision PCG
// Defect correction: x = 0, r = b; while |r|_inf > tol |b|_inf: solve A e = r with an FP32 PCG
// (FP32 matrix, FP32 MIC(0) factor rounded from the FP64 one, FP32 vectors; dot products reduced
// in FP64 by the fixed tree; alpha and beta in FP64) until its residual drops below
// max(1e-5 |r|_inf, 0.5 tol |b|_inf), then x += e and r = b - A x in FP64.  The stopping test is
// the reference's, on the FP64 residual.  The inner solve owes no bit pattern to anything, so its
// FP32 row sums and vector updates and the FP64 lanes of its dots are fused multiply-adds
// (fmaf / fma written out: the library is compiled without contraction for the FP64 paths).
constexpr double MIXED_INNER_REDUCTION = 1e-5;
constexpr int MIXED_MAX_OUTER = 20;
__global__ void k_to_f32(const double* a, float* b, const int* nptr) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < *nptr) b[i] = (float)a[i];
}
// r = b - A x (FP64, row sums in column order), |r|_inf into amax
__global__ void k_resid64(Proj P, const double* x, double* r) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v = 0;
    if (i < *P.nDof) {
        double t = 0;
        for (int q = P.rowPtr[i]; q < P.rowPtr[i + 1]; ++q) t += P.val[q] * x[P.col[q]];
        double ri = P.b[i] - t;
        r[i] = ri;
        v = fabs(ri);
    }
    block_absmax_to(v, P.amax);
}
// start of an inner solve: r32 = r (also in walk order), e32 = 0
__global__ void k_inner_init(Proj P, const double* r) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= *P.nDof) return;
    float ri = (float)r[i];
    P.r32[i] = ri;
    P.rl32[P.pos[i]] = ri;
    P.e32[i] = 0.0f;
}
// partial dots of FP32 vectors, products and sums in FP64 (fixed tree)
__global__ void k_tree_dot32(const float* a, const float* b, const int* nptr, double* part) {
    __shared__ double sh[RED_LANES];
    long long n = *nptr;
    long long base = (long long)blockIdx.x * RED_CHUNK;
    if (base >= n && blockIdx.x > 0) return;
    double acc = 0.0;
    for (int k = 0; k < RED_PER_LANE; ++k) {
        long long i = base + threadIdx.x + (long long)RED_LANES * k;
        if (i < n) acc = fma((double)a[i], (double)b[i], acc);
    }
    double r = block_tree(acc, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = r;
}
// inner start: rho = z.r, tolerance of this inner solve; the iteration count carries on
__global__ void k_inner_start(Proj P, const double* partRho, double innerTol) {
    __shared__ double sh[RED_LANES];
    int n = *P.nDof;
    long long m = (n + RED_CHUNK - 1) / RED_CHUNK;
    double rho = fold_partials(partRho, m, sh);
    if (threadIdx.x == 0) {
        P.sc[SC_TOL] = innerTol;
        P.sc[SC_RHO] = rho;
        *P.done = (rho == 0 || rho != rho) ? 1 : 0;
        *P.amax = 0;
    }
}
__global__ void k_copy32(const float* a, float* b, const int* nptr) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < *nptr) b[i] = a[i];
}
// q = A32 s (FP32 row sums), partial dots s.q in FP64
__global__ void __launch_bounds__(SPMV_THREADS) k_spmv32_dot(Proj P, const float* s, float* q, double* part) {
    __shared__ float ys[RED_CHUNK];
    __shared__ double sh[RED_LANES];
    if (*P.done) return;
    int n = *P.nDof;
    long long base = (long long)blockIdx.x * RED_CHUNK;
    if (base >= n) return;
    for (int k = threadIdx.x; k < RED_CHUNK; k += SPMV_THREADS) {
        long long i = base + k;
        float t = 0;
        if (i < n) {
            for (int c = P.rowPtr[i]; c < P.rowPtr[i + 1]; ++c) t = fmaf(P.val32[c], s[P.col[c]], t);
            q[i] = t;
        }
        ys[k] = t;
    }
    __syncthreads();
    const int tl = threadIdx.x;
    double acc = 0.0;
    if (tl < RED_LANES)
        for (int k = 0; k < RED_PER_LANE; ++k) {
            long long i = base + tl + (long long)RED_LANES * k;
            if (i < n) acc = fma((double)s[i], (double)ys[tl + RED_LANES * k], acc);
        }
    double r = chunk_fold(acc, sh);
    if (tl == 0) part[blockIdx.x] = r;
}
__global__ void k_update_er32(Proj P) {
    if (*P.done) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    float alpha = (float)P.sc[SC_ALPHA];
    double v = 0;
    if (i < *P.nDof) {
        P.e32[i] = fmaf(alpha, P.s32[i], P.e32[i]);
        float ri = fmaf(-alpha, P.q32[i], P.r32[i]);
        P.r32[i] = ri;
        P.rl32[P.pos[i]] = ri;
        v = fabs((double)ri);
    }
    block_absmax_to(v, P.amax);
}
__global__ void k_update_s32(Proj P) {
    if (*P.done) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < *P.nDof) P.s32[i] = fmaf((float)P.sc[SC_BETA], P.s32[i], P.z32[i]);
}
__global__ void k_add_correction(Proj P, double* x) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < *P.nDof) x[i] += (double)P.e32[i];
}
__global__ void k_mixed_finish(Proj P, double res, double tolAbs, double res0, int converged) {
    P.sc[SC_RESID0] = res0;
    P.sc[SC_RESID] = res;
    P.sc[SC_TOL] = tolAbs;
    P.isc[ISC_CONVERGED] = converged;
}
static PcaData<float> pca_data32(const Proj& P) {
    return PcaData<float>{P.fvalP32, P.bvalP32, P.linvd32, P.rl32, P.yl32, P.fval32, P.bval32};
}
static double read_amax(Proj& P, cudaStream_t st) {
    unsigned long long bits = 0;
    cudaMemcpyAsync(&bits, P.amax, sizeof bits, cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);
    double v;
    memcpy(&v, &bits, sizeof v);
    return v;
}
int launch_pcg_mixed(const Dev& d, Proj& P, double tolFactor, int maxIter, int batch, cudaStream_t st, KProf* prof) {
    if (!P.pcActive32) return -1;
    int maxRows = P.rowsCap;
    int chunks = (maxRows + RED_CHUNK - 1) / RED_CHUNK;
    double* x = P.x;
    double* r = P.r;
    ASTG_LAUNCH(k_to_f32<<<nblk((long long)maxRows * ROW_W), TB, 0, st>>>(P.val, P.val32, P.nnz));
    ASTG_LAUNCH(k_zero_vec<<<nblk(maxRows), TB, 0, st>>>(x, P.nDof));
    ASTG_LAUNCH(k_copy<<<nblk(maxRows), TB, 0, st>>>(P.b, r, P.nDof));
    cudaMemsetAsync(P.amax, 0, sizeof(unsigned long long), st);
    cudaMemsetAsync(P.isc, 0, sizeof(int) * ISC_COUNT, st);
    ASTG_LAUNCH(k_absmax<<<nblk(maxRows), TB, 0, st>>>(r, P.nDof, P.amax));
    const double res0 = read_amax(P, st);
    const double tolAbs = P.tolAbsolute ? tolFactor : tolFactor * res0;
    double res = res0;
    int outer = 0, converged = 0;
    PcaData<float> D = pca_data32(P);
    BatchGraph graph;  // one inner batch; the same work in every outer cycle
    for (;;) {
        if (res <= tolAbs) {
            converged = 1;
            break;
        }
        int iters = 0;
        cudaMemcpyAsync(&iters, P.isc + ISC_ITERS, sizeof iters, cudaMemcpyDeviceToHost, st);
        cudaStreamSynchronize(st);
        if (outer >= MIXED_MAX_OUTER || iters >= maxIter || res != res) break;
        double innerTol = std::max(MIXED_INNER_REDUCTION * res, 0.5 * tolAbs);
        ASTG_LAUNCH(k_inner_init<<<nblk(maxRows), TB, 0, st>>>(P, r));
        cudaMemsetAsync(P.done, 0, sizeof(int), st);
        prof_begin(prof, 0, st);
        cudaError_t e = launch_precond_async(d, P, D, P.z32, P.pcSmem32, st);
        prof_end(prof, st);
        if (e != cudaSuccess) g_cluster_error = e;
        ASTG_LAUNCH(k_tree_dot32<<<chunks, RED_LANES, 0, st>>>(P.z32, P.r32, P.nDof, P.part));
        ASTG_LAUNCH(k_inner_start<<<1, RED_LANES, 0, st>>>(P, P.part, innerTol));
        ASTG_LAUNCH(k_copy32<<<nblk(maxRows), TB, 0, st>>>(P.z32, P.s32, P.nDof));
        auto body = [&](int nb, KProf* pf) {
            for (int it = 0; it < nb; ++it) {
                prof_begin(pf, 2, st);
                ASTG_LAUNCH(k_spmv32_dot<<<chunks, SPMV_THREADS, 0, st>>>(P, P.s32, P.q32, P.part));
                prof_end(pf, st);
                ASTG_LAUNCH(k_alpha<<<1, RED_LANES, 0, st>>>(P, P.part));
                ASTG_LAUNCH(k_update_er32<<<nblk(maxRows), TB, 0, st>>>(P));
                ASTG_LAUNCH(k_check<<<1, 1, 0, st>>>(P, maxIter));
                prof_begin(pf, 0, st);
                cudaError_t pe = launch_precond_async(d, P, D, P.z32, P.pcSmem32, st);
                prof_end(pf, st);
                if (pe != cudaSuccess) g_cluster_error = pe;
                ASTG_LAUNCH(k_tree_dot32<<<chunks, RED_LANES, 0, st>>>(P.z32, P.r32, P.nDof, P.part));
                ASTG_LAUNCH(k_beta<<<1, RED_LANES, 0, st>>>(P, P.part));
                ASTG_LAUNCH(k_update_s32<<<nblk(maxRows), TB, 0, st>>>(P));
            }
        };
        for (int launched = 0; launched < maxIter;) {
            bool replayed = g_pcg_graphs && graph.run(body, batch, st, prof);
            if (!replayed) body(batch, prof);
            launched += batch;
            cudaMemcpyAsync(P.hostDone, P.done, sizeof(int), cudaMemcpyDeviceToHost, st);
            cudaStreamSynchronize(st);
            prof_drain(prof, replayed && graph.profiled);
            if (*P.hostDone) break;
        }
        ASTG_LAUNCH(k_add_correction<<<nblk(maxRows), TB, 0, st>>>(P, x));
        cudaMemsetAsync(P.amax, 0, sizeof(unsigned long long), st);
        prof_begin(prof, 2, st);
        ASTG_LAUNCH(k_resid64<<<nblk(maxRows), TB, 0, st>>>(P, x, r));
        prof_end(prof, st);
        res = read_amax(P, st);
        ++outer;
    }
    ASTG_LAUNCH(k_mixed_finish<<<1, 1, 0, st>>>(P, res, tolAbs, res0, converged));
    return outer;
}
// ------------------------------------------------------------------ workspace
namespace {
struct ProjArena {
    cudaStream_t st;
    std::vector<void*>& allocs;
    void ck(cudaError_t e, const char* what) {
        if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
    }
    template <class T>
    T* get(long long n) {
        void* p = nullptr;
        size_t bytes = (size_t)std::max<long long>(n, 1) * sizeof(T);
        ck(cudaMalloc(&p, bytes), "cudaMalloc");
        allocs.push_back(p);
        ck(cudaMemsetAsync(p, 0, bytes, st), "cudaMemset");
        return (T*)p;
    }
};
}  // namespace

void proj_alloc(Proj& J, long long rows, int device, cudaStream_t st, std::vector<void*>& allocs) {
    if (rows <= 0 || rows * ROW_W >= (1LL << 31)) throw std::runtime_error("projection too large for 32-bit matrix indices");
    ProjArena A{st, allocs};
    J.rowsCap = (int)rows;
    J.n0 = A.get<int>(1);
    J.nDof = A.get<int>(1);
    J.nnz = A.get<int>(4);  // nnz, then scan totals of the level schedule
    J.rowCnt = A.get<int>(rows);
    J.rowPtr = A.get<int>(rows + 1);
    J.padCol = A.get<int>(rows * ROW_W);
    J.padVal = A.get<double>(rows * ROW_W);
    J.bRaw = A.get<double>(rows);
    J.col = A.get<int>(rows * ROW_W);
    J.val = A.get<double>(rows * ROW_W);
    J.diagPos = A.get<int>(rows);
    J.tpos = A.get<int>(rows * ROW_W);
    J.b = A.get<double>(rows);
    J.Lv = A.get<double>(rows * ROW_W);
    J.invdiag = A.get<double>(rows);
    J.adiag = A.get<double>(rows);
    J.ready = A.get<int>(rows);
    J.planPtr = A.get<int>(rows * ROW_W + 1);
    J.planCap = rows * ROW_W * 2;
    J.plan = A.get<int>(J.planCap);
    J.planTotal = A.get<int>(1);
    J.counter = A.get<int>(1);
    J.level = A.get<int>(rows);
    J.levelCnt = A.get<int>(rows + 1);
    J.levelPtr = A.get<int>(rows + 2);
    J.nLevels = A.get<int>(1);
    J.fill = A.get<int>(rows + 1);
    J.perm = A.get<int>(rows);
    J.cntF = A.get<int>(rows);
    J.cntB = A.get<int>(rows);
    J.fptr = A.get<int>(rows + 1);
    J.bptr = A.get<int>(rows + 1);
    J.fcol = A.get<int>(rows * ROW_W / 2 + 1);
    J.fval = A.get<double>(rows * ROW_W / 2 + 1);
    J.bcol = A.get<int>(rows * ROW_W / 2 + 1);
    J.bval = A.get<double>(rows * ROW_W / 2 + 1);
    // MIC(0) sweep form: ASTG_SWEEP = async (default: fused, barrier-free), dsmem (fused, one
    // cluster barrier per level), cluster (global-memory level sweeps) or syncfree (per-row
    // flags); a form the device cannot run falls back to the next one
    const char* env = getenv("ASTG_SWEEP");
    std::string mode = env ? env : "async";
    if (mode != "async" && mode != "dsmem" && mode != "cluster" && mode != "syncfree")
        throw std::invalid_argument("ASTG_SWEEP must be async, dsmem, cluster or syncfree");
    J.clusterSize = mode == "syncfree" ? 0 : choose_cluster_size(device);
    J.pcAsync = mode == "async";
    J.pcCluster = (mode == "async" || mode == "dsmem") ? choose_dsmem_cluster(J.pcAsync, &J.pcSmemMax) : 0;
    J.pcActive = 0;
    J.pcSmem = 0;
    J.pcLgBlock = 8;  // 256-row ownership blocks (measured: 64 to 4096 within 3 %)
    long long scanMax = std::max(rows * ROW_W + 1, (long long)std::max(J.pcCluster, 1) * (rows + 1));
    J.bsum = A.get<int>((scanMax + 1023) / 1024 + 1);
    if (J.pcCluster && J.pcAsync) {
        J.chunk = A.get<int>(1);
        J.ownStart = A.get<int>(J.pcCluster + 1);
        // FP32 copies for the mixed-precision solve
        J.val32 = A.get<float>(rows * ROW_W);
        J.fvalP32 = A.get<float>(rows * PC_MAXE);
        J.bvalP32 = A.get<float>(rows * PC_MAXE);
        J.linvd32 = A.get<float>(rows);
        J.rl32 = A.get<float>(rows);
        J.yl32 = A.get<float>(rows);
        J.fval32 = A.get<float>(rows * ROW_W / 2 + 1);
        J.bval32 = A.get<float>(rows * ROW_W / 2 + 1);
        J.e32 = A.get<float>(rows);
        J.r32 = A.get<float>(rows);
        J.s32 = A.get<float>(rows);
        J.z32 = A.get<float>(rows);
        J.q32 = A.get<float>(rows);
        J.lself = A.get<int>(rows);
        J.yl = A.get<double>(rows);
        J.ownCnt = A.get<int>((rows + 1) * J.pcCluster);
        J.ownPtr = A.get<int>((rows + 1) * J.pcCluster + 1);
        J.ownFill = A.get<int>((rows + 1) * J.pcCluster);
    }
    if (J.pcCluster) {
        J.pos = A.get<int>(rows);
        J.lcntF = A.get<int>(rows);
        J.lcntB = A.get<int>(rows);
        J.linvd = A.get<double>(rows);
        J.rl = A.get<double>(rows);
        J.fcolP = A.get<int>(rows * PC_MAXE);
        J.fvalP = A.get<double>(rows * PC_MAXE);
        J.bcolP = A.get<int>(rows * PC_MAXE);
        J.bvalP = A.get<double>(rows * PC_MAXE);
    }
    int sms = 0;
    A.ck(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device), "attr");
    J.sweepBlocks = std::max(1, sms) * 8;
    J.x = A.get<double>(rows);
    J.r = A.get<double>(rows);
    J.s = A.get<double>(rows);
    J.z = A.get<double>(rows);
    J.part = A.get<double>((rows + 2047) / 2048 + 1);
    J.sc = A.get<double>(SC_COUNT);
    J.isc = A.get<int>(ISC_COUNT);
    J.amax = A.get<unsigned long long>(1);
    J.done = A.get<int>(1);
    A.ck(cudaMallocHost(&J.hostDone, sizeof(int)), "cudaMallocHost");
    *J.hostDone = 0;
}

}  // namespace astg
