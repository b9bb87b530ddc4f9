// Host side of the uniform 2-D AST smoke solver (kernels in astg2d.cu) and the C ABI of
// include/astg2d.h.  The handle mirrors ASTSolver<2> (include/ast_solver.h): initialize() numbers
// the cells, update(dt) runs Solver::update's CFL sub-stepping (src/solver.cpp:8-46) and each
// sub-step is onUpdate's source -> force -> project -> advect (:100-108).  The projection reuses
// the octree path's CSR, MIC(0) factorisation and PCG with the absolute stopping test of the
// std::vector PCGSolver::solve overload (include/pcgsolver/pcg_solver.h:302-363).  The host reads
// back only the CFL maximum and the unknown count of each sub-step and the PCG's stopping flag.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "astg2d.h"
#include "astg2d_launch.h"
#include "astg_launch.h"

using namespace astg;

namespace {

struct CudaError2 : std::runtime_error {
    using std::runtime_error::runtime_error;
};
void ck2(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw CudaError2(std::string(what) + ": " + cudaGetErrorString(e));
}
constexpr double SQRT2_H = 1.4142135623730951;  // include/macro.h:16
constexpr double EPS_H = 2.220446049250313e-16;  // include/general.h:48
constexpr long long MAX_ROWS_2D = 2048LL * 2048LL;
constexpr int MAX_SUBSTEPS_2D = 100000;  // per astg2_update

}  // namespace

struct astg2_handle {
    std::string err;
    int nx = 0, ny = 0, device = 0;
    double dx = 0;
    bool adaptive = true;
    double tol = 1e-5, omega = 0.97, minDiag = 0.95;  // ASTSolver::initialize (:40), SOLVER_ACCURACY
    int maxIter = 5000, precision = ASTG_FP64;
    cudaStream_t st = nullptr;
    cudaEvent_t evA = nullptr, evB = nullptr;
    std::vector<void*> allocs;

    Grid2 g{};
    Dev d{};
    Fields2 F[2]{};
    int cur = 0;
    double* dual = nullptr;
    uint8_t* fixedT = nullptr;
    int* vIdx = nullptr;
    int* cnt = nullptr;
    int* scanTotal = nullptr;
    unsigned long long* cflMax = nullptr;
    int* status = nullptr;
    Proj J{};
    int epoch = 0;
    KProf prof;
    std::vector<double> subDt;
    std::vector<uint8_t> hostFixed;
    int lastN = 0, lastNnz = 0;
    bool useWave = false;  // the wavefront MIC(0) sweeps (ASTG_WAVE=0 selects the generic forms)
    astg2_stats last{};

    long long nc() const { return (long long)nx * ny; }
    long long nv() const { return (long long)(nx + 1) * (ny + 1); }
    long long nmx() const { return (long long)(nx + 1) * ny; }
    long long nmy() const { return (long long)nx * (ny + 1); }

    template <class T>
    T* dalloc(long long n) {
        void* p = nullptr;
        size_t bytes = (size_t)std::max<long long>(n, 1) * sizeof(T);
        ck2(cudaMalloc(&p, bytes), "cudaMalloc");
        allocs.push_back(p);
        ck2(cudaMemsetAsync(p, 0, bytes, st), "cudaMemset");
        return (T*)p;
    }

    ~astg2_handle() {
        if (st) cudaStreamSynchronize(st);
        for (void* p : allocs) cudaFree(p);
        if (J.hostDone) cudaFreeHost(J.hostDone);
        for (cudaEvent_t e : {evA, evB})
            if (e) cudaEventDestroy(e);
        if (st) cudaStreamDestroy(st);
    }

    // ASTSolver<2>(res, dx, adaptive) and initialize() (include/ast_solver.h:28-50, 75-93): fields
    // zero, every boundary tilt fixed closed, the cells numbered 0 .. nc-1
    void init(int nx_, int ny_, double dx_, bool adaptive_, int device_) {
        if (nx_ < 2 || ny_ < 2) throw std::invalid_argument("astg2_create: resolution must be at least 2 x 2");
        if (!(dx_ > 0) || !std::isfinite(dx_)) throw std::invalid_argument("astg2_create: dx must be positive");
        if ((long long)nx_ * ny_ + (long long)(nx_ + 1) * (ny_ + 1) > MAX_ROWS_2D)
            throw std::invalid_argument("astg2_create: nx * ny + (nx + 1) * (ny + 1) must not exceed 4194304");
        nx = nx_;
        ny = ny_;
        dx = dx_;
        adaptive = adaptive_;
        device = device_;
        ck2(cudaSetDevice(device), "cudaSetDevice");
        ck2(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "cudaStreamCreate");
        ck2(cudaEventCreate(&evA), "cudaEventCreate");
        ck2(cudaEventCreate(&evB), "cudaEventCreate");
        for (int b = 0; b < 2; ++b) {
            F[b].dC = dalloc<double>(nc());
            F[b].hC = dalloc<double>(nc());
            F[b].dV = dalloc<double>(nv());
            F[b].hV = dalloc<double>(nv());
            F[b].mx = dalloc<double>(nmx());
            F[b].my = dalloc<double>(nmy());
            F[b].tv = dalloc<double>(4 * nv());
            F[b].open = dalloc<uint8_t>(nv());
        }
        dual = dalloc<double>(2 * nv());
        vIdx = dalloc<int>(nv());
        cnt = dalloc<int>(nv());
        scanTotal = dalloc<int>(1);
        cflMax = dalloc<unsigned long long>(1);
        status = dalloc<int>(1);
        hostFixed.assign(nv(), 0);
        for (int y = 0; y <= ny; ++y)
            for (int x = 0; x <= nx; ++x)
                if (x == 0 || y == 0 || x == nx || y == ny) hostFixed[x + y * (nx + 1)] = 1;
        fixedT = dalloc<uint8_t>(nv());
        ck2(cudaMemcpyAsync(fixedT, hostFixed.data(), nv(), cudaMemcpyHostToDevice, st), "upload");
        const double hdx = dx / 2.0;
        g = Grid2{nx, ny, dx, hdx, hdx * SQRT2_H, 2.0, status};
        d.status = status;
        d.rho = 2.0;
        proj_alloc(J, nc() + nv(), device, st, allocs);
        J.tolAbsolute = 1;
        const char* wenv = getenv("ASTG_WAVE");
        useWave = wave_supported(nx, ny) && !(wenv && std::string(wenv) == "0");
        if (useWave) {
            J.wnx = nx;
            J.wny = ny;
            const long long skew = (long long)nx * (nx + ny - 1);  // diagonal-major slots
            J.wRecF = dalloc<double2>(2 * skew);
            J.wRecB = dalloc<double2>(2 * skew);
            J.wR = dalloc<double>(skew);
            J.wZ = dalloc<double>(skew);
            J.wStatus = status;
            J.wTt = dalloc<int>(4 * skew);
            J.wTl = dalloc<double>(4 * skew);
            J.wTc = dalloc<int>(4 * nv());
            J.wTv = dalloc<double>(4 * nv());
        }
        launch2_numbering(g, F[cur], cnt, vIdx, J.bsum, scanTotal, J.nDof, st);
        ck2(cudaStreamSynchronize(st), "init");
    }

    void checkStatus() {
        int s = 0;
        ck2(cudaMemcpyAsync(&s, status, sizeof(int), cudaMemcpyDeviceToHost, st), "status");
        ck2(cudaStreamSynchronize(st), "sync");
        if (s != DS_OK) {
            int zero = 0;
            ck2(cudaMemcpy(status, &zero, sizeof(int), cudaMemcpyHostToDevice), "status reset");
            if (s == DS_WAIT_TIMEOUT) throw std::runtime_error("device wait timed out (status 3)");
            throw std::runtime_error("layout check failed on the device (status " + std::to_string(s) + ")");
        }
    }

    // ---------------------------------------------------------------- stages
    // project (include/ast_solver.h:326-469): updateIndex, assembly, b *= rho / dt, MIC(0)-PCG,
    // correctVelocityByPressure, constrainVelocity
    void project(double dt) {
        Fields2& C = F[cur];
        launch2_numbering(g, C, cnt, vIdx, J.bsum, scanTotal, J.nDof, st);
        int n = 0;
        ck2(cudaMemcpyAsync(&n, J.nDof, sizeof n, cudaMemcpyDeviceToHost, st), "unknowns");
        ck2(cudaStreamSynchronize(st), "unknowns");
        if (n <= 0 || n > J.rowsCap) throw std::runtime_error("projection has more rows than the workspace holds");
        select_preconditioner(J, n);
        launch2_assemble(g, d, C, vIdx, J, dt, st);
        bool mixed = precision == ASTG_MIXED && J.pcActive32;
        // FP64 solves take the wavefront sweeps (one CTA along the anti-diagonals); the mixed form
        // keeps the FP32 fused preconditioner
        J.wave = (useWave && !mixed) ? 1 : 0;
        if (J.wave) J.pcActive = 0;
        launch_factor(d, J, omega, minDiag, epoch, st, &prof);
        if (J.wave) {
            launch2_wave_gather(J, vIdx, n, st);
        } else {
            bool owner = mixed || (J.pcActive && J.pcAsync);
            if (J.clusterSize > 0 || J.pcActive || mixed) launch_level_schedule(d, J, owner, st);
        }
        if (mixed) launch_pcg_mixed(d, J, tol, maxIter, 8, st, &prof);
        else launch_pcg_fp64(d, J, tol, maxIter, epoch, 8, st, &prof);
        launch2_correct(g, C, vIdx, J.x, dt, st);
        int isc[ISC_COUNT];
        double sc[SC_COUNT];
        int nnz = 0;
        ck2(cudaMemcpyAsync(isc, J.isc, sizeof isc, cudaMemcpyDeviceToHost, st), "stats");
        ck2(cudaMemcpyAsync(sc, J.sc, sizeof sc, cudaMemcpyDeviceToHost, st), "stats");
        ck2(cudaMemcpyAsync(&nnz, J.nnz, sizeof nnz, cudaMemcpyDeviceToHost, st), "stats");
        ck2(cudaStreamSynchronize(st), "project");
        if (g_cluster_error != cudaSuccess) {
            cudaError_t e = g_cluster_error;
            g_cluster_error = cudaSuccess;
            ck2(e, "cluster sweep launch");
        }
        lastN = n;
        lastNnz = nnz;
        last.unknowns = n;
        last.nnz = nnz;
        last.pcg_iterations = isc[ISC_ITERS];
        last.pcg_converged = isc[ISC_CONVERGED];
        last.pcg_residual = sc[SC_RESID];
    }
    // advect (include/ast_solver.h:533-553): dual velocities, then the fused advection into the
    // other buffer, which becomes the state
    void advect(double dt) {
        launch2_dual(g, F[cur], dual, st);
        launch2_advect(g, F[cur], F[1 - cur], dual, fixedT, adaptive, dt, st);
        cur = 1 - cur;
    }
    void stage(int id, double dt) {
        if (!(dt > 0) || !std::isfinite(dt)) throw std::invalid_argument("astg2_stage: dt must be positive");
        switch (id) {
            case 0: launch2_source(g, F[cur], st); break;
            case 1: launch2_force(g, F[cur], dt, st); break;
            case 2: project(dt); break;
            case 3: advect(dt); break;
            case 4: substep(dt); break;
            default: throw std::invalid_argument("astg2_stage: stage must be 0..4");
        }
    }
    // onUpdate (include/ast_solver.h:100-108)
    void substep(double dt) {
        subDt.push_back(dt);
        launch2_source(g, F[cur], st);
        launch2_force(g, F[cur], dt, st);
        project(dt);
        advect(dt);
    }
    // ASTSolver::numberOfSubTimeSteps / cfl (include/ast_solver.h:51-70): int(dt |v|max / dx),
    // then ceil of an integer division by max_cfl = 2
    int numberOfSubTimeSteps(double dt) {
        launch2_cfl(g, F[cur], cflMax, st);
        unsigned long long bits = 0;
        ck2(cudaMemcpyAsync(&bits, cflMax, sizeof bits, cudaMemcpyDeviceToHost, st), "cfl");
        ck2(cudaStreamSynchronize(st), "cfl");
        double m;
        std::memcpy(&m, &bits, sizeof m);
        double c = dt * std::sqrt(m) / dx;
        if (!(c < 2147483647.0)) throw std::runtime_error("CFL number out of range: the velocity diverged");
        int cfl = (int)c;
        int step = cfl / 2;
        return step > 1 ? step : 1;
    }
    // Solver::update without a fixed time step (src/solver.cpp:8-46)
    void update(double dt) {
        if (!(dt > 0) || !std::isfinite(dt)) throw std::invalid_argument("astg2_update: dt must be positive");
        ck2(cudaEventRecord(evA, st), "event");
        double remaining = dt;
        int subs = 0;
        while (remaining > EPS_H) {
            int n = numberOfSubTimeSteps(remaining);
            // the reference would run them all; a frame this split has a diverged velocity field
            if (n > MAX_SUBSTEPS_2D)
                throw std::runtime_error("CFL asks for " + std::to_string(n) +
                                         " sub-steps in one frame: the velocity diverged");
            double actual = remaining / (double)n;
            substep(actual);
            ++subs;
            remaining -= actual;
        }
        ck2(cudaEventRecord(evB, st), "event");
        ck2(cudaEventSynchronize(evB), "update");
        float ms = 0;
        cudaEventElapsedTime(&ms, evA, evB);
        last.ms = ms;
        last.substeps = subs;
        last.substeps_total = (long long)subDt.size();
        checkStatus();
    }

    // ---------------------------------------------------------------- arrays
    struct Arr {
        int kind;  // 0 double, 1 uint8, 2 int32
        void* dev;
        long long n;
        bool settable;
    };
    bool array(const std::string& n, Arr* a) {
        Fields2& C = F[cur];
        auto f64 = [&](double* p, long long c, bool s) { *a = Arr{0, p, c, s}; return true; };
        if (n == "density_cell") return f64(C.dC, nc(), true);
        if (n == "heat_cell") return f64(C.hC, nc(), true);
        if (n == "density_vert") return f64(C.dV, nv(), true);
        if (n == "heat_vert") return f64(C.hV, nv(), true);
        if (n == "mac_x") return f64(C.mx, nmx(), true);
        if (n == "mac_y") return f64(C.my, nmy(), true);
        if (n == "tilt_vel") return f64(C.tv, 4 * nv(), true);
        if (n == "dual_vert") return f64(dual, 2 * nv(), false);
        if (n == "b") return f64(J.b, lastN, false);
        if (n == "p") return f64(J.x, lastN, false);
        if (n == "A_val") return f64(J.val, lastNnz, false);
        if (n == "sub_dt") { *a = Arr{0, nullptr, (long long)subDt.size(), false}; return true; }
        if (n == "tilt_open") { *a = Arr{1, C.open, nv(), true}; return true; }
        if (n == "pindex_cell") { *a = Arr{2, nullptr, nc(), false}; return true; }
        if (n == "pindex_vert") { *a = Arr{2, vIdx, nv(), false}; return true; }
        if (n == "A_rowptr") { *a = Arr{2, J.rowPtr, lastN ? lastN + 1 : 0, false}; return true; }
        if (n == "A_col") { *a = Arr{2, J.col, lastNnz, false}; return true; }
        return false;
    }
    static size_t esize(int kind) { return kind == 0 ? 8 : (kind == 1 ? 1 : 4); }
    void get(const std::string& n, void* dst, long long count) {
        Arr a;
        if (!array(n, &a)) throw std::invalid_argument("astg2_get: unknown array " + n);
        if (count != a.n) throw std::invalid_argument("astg2_get: " + n + " holds " + std::to_string(a.n) + " elements");
        if (a.n == 0) return;
        if (!dst) throw std::invalid_argument("astg2_get: null destination");
        if (n == "sub_dt") { std::memcpy(dst, subDt.data(), sizeof(double) * subDt.size()); return; }
        if (n == "pindex_cell") {
            int32_t* o = (int32_t*)dst;
            for (long long i = 0; i < a.n; ++i) o[i] = (int32_t)i;
            return;
        }
        ck2(cudaMemcpyAsync(dst, a.dev, esize(a.kind) * a.n, cudaMemcpyDeviceToHost, st), "download");
        ck2(cudaStreamSynchronize(st), "download");
    }
    void set(const std::string& n, const void* src, long long count) {
        Arr a;
        if (!array(n, &a) || !a.settable) throw std::invalid_argument("astg2_set: " + n + " is not a settable state array");
        if (count != a.n) throw std::invalid_argument("astg2_set: " + n + " holds " + std::to_string(a.n) + " elements");
        if (!src) throw std::invalid_argument("astg2_set: null source");
        if (n == "tilt_open") {
            const uint8_t* o = (const uint8_t*)src;
            for (long long i = 0; i < a.n; ++i) {
                if (o[i] > 1) throw std::invalid_argument("astg2_set: tilt_open entries must be 0 or 1");
                if (o[i] && hostFixed[i]) throw std::invalid_argument("astg2_set: boundary tilts are fixed closed");
            }
        }
        ck2(cudaMemcpyAsync(a.dev, src, esize(a.kind) * a.n, cudaMemcpyHostToDevice, st), "upload");
        ck2(cudaStreamSynchronize(st), "upload");
    }
};

// ---------------------------------------------------------------- C ABI
namespace {
astg_status fail2(astg2_handle* h, const std::exception& e, astg_status code) {
    if (h) h->err = e.what();
    return code;
}
template <class Fn>
astg_status guard2(astg2_handle* h, Fn&& f) {
    if (!h) return ASTG_BAD_ARG;
    try {
        f();
        return ASTG_OK;
    } catch (CudaError2& e) {
        return fail2(h, e, ASTG_CUDA_ERROR);
    } catch (std::invalid_argument& e) {
        return fail2(h, e, ASTG_BAD_ARG);
    } catch (std::runtime_error& e) {
        std::string m = e.what();
        if (m.find("timed out") != std::string::npos) return fail2(h, e, ASTG_DEVICE_WAIT_TIMEOUT);
        if (m.find("layout") != std::string::npos) return fail2(h, e, ASTG_LAYOUT_ERROR);
        if (m.find("diverged") != std::string::npos) return fail2(h, e, ASTG_NAN_DETECTED);
        return fail2(h, e, ASTG_CUDA_ERROR);
    } catch (std::exception& e) {
        return fail2(h, e, ASTG_CUDA_ERROR);
    }
}
}  // namespace

extern "C" {

astg_status astg2_create(int nx, int ny, double dx, int adaptive_dofs, int device, astg2_handle** out) {
    if (!out) return ASTG_BAD_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return ASTG_NO_DEVICE;
    if (device < 0 || device >= ndev) return ASTG_BAD_ARG;
    auto* h = new astg2_handle();
    astg_status s = guard2(h, [&] { h->init(nx, ny, dx, adaptive_dofs != 0, device); });
    *out = h;
    return s;
}

void astg2_destroy(astg2_handle* h) { delete h; }

const char* astg2_last_error(const astg2_handle* h) { return h ? h->err.c_str() : "null handle"; }

astg_status astg2_update(astg2_handle* h, double dt) {
    return guard2(h, [&] {
        ck2(cudaSetDevice(h->device), "cudaSetDevice");
        h->update(dt);
    });
}

astg_status astg2_stage(astg2_handle* h, int stage, double dt) {
    return guard2(h, [&] {
        ck2(cudaSetDevice(h->device), "cudaSetDevice");
        ck2(cudaEventRecord(h->evA, h->st), "event");
        h->stage(stage, dt);
        ck2(cudaEventRecord(h->evB, h->st), "event");
        ck2(cudaEventSynchronize(h->evB), "stage");
        float ms = 0;
        cudaEventElapsedTime(&ms, h->evA, h->evB);
        h->last.ms = ms;
        h->last.substeps_total = (long long)h->subDt.size();
        h->checkStatus();
    });
}

astg_status astg2_get_density(astg2_handle* h, double* out, long long count) {
    return guard2(h, [&] { h->get("density_cell", out, count); });
}

long long astg2_count(const astg2_handle* h, const char* name, int* kind) {
    if (!h || !name) return -1;
    astg2_handle::Arr a;
    if (!const_cast<astg2_handle*>(h)->array(name, &a)) return -1;
    if (kind) *kind = a.kind;
    return a.n;
}

astg_status astg2_get(astg2_handle* h, const char* name, void* dst, long long count) {
    return guard2(h, [&] {
        if (!name) throw std::invalid_argument("astg2_get: null name");
        h->get(name, dst, count);
    });
}

astg_status astg2_set(astg2_handle* h, const char* name, const void* src, long long count) {
    return guard2(h, [&] {
        if (!name) throw std::invalid_argument("astg2_set: null name");
        h->set(name, src, count);
    });
}

astg_status astg2_set_solver(astg2_handle* h, double tol, int max_iter, double omega, double min_diag, int precision) {
    return guard2(h, [&] {
        if (!(tol > 0) || max_iter < 1 || !(omega >= 0 && omega <= 1) || !(min_diag >= 0 && min_diag <= 1) ||
            (precision != ASTG_FP64 && precision != ASTG_MIXED))
            throw std::invalid_argument("astg2_set_solver: tol > 0, max_iter >= 1, omega and min_diag in [0, 1], "
                                        "precision ASTG_FP64 or ASTG_MIXED");
        h->tol = tol;
        h->maxIter = max_iter;
        h->omega = omega;
        h->minDiag = min_diag;
        h->precision = precision;
    });
}

astg_status astg2_last_stats(const astg2_handle* h, astg2_stats* out) {
    if (!h || !out) return ASTG_BAD_ARG;
    *out = h->last;
    return ASTG_OK;
}

}  // extern "C"
