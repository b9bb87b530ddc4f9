// A C++ host program driving the octree smoke step through the C ABI only (include/astg.h), in the
// shape of the reference's example/octree_smoke_3d/main.cpp: the scene's source sphere, optionally
// the stock sphere obstacle (OctreeOmniGridSolver3::initObstacle), frames advanced with the
// reference's CFL sub-stepping (Solver::update with setMaxCfl(2)) or with fixed steps, and the
// density read back after every frame as a sceneSetup / dump step would.
//
//   octree_smoke [frames=3] [coarsest=32] [levels=3] [--collider] [--fixed] [--dt=0.01]
//
// One line per frame: frame, sub-steps, PCG iterations of the last sub-step, device ms, and the
// sum of the octagon densities printed with 17 significant digits (the same handle driven from
// Python gives the same digits).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "astg.h"

int main(int argc, char** argv) {
    int frames = 3, coarsest = 32, levels = 3, pos = 0;
    bool collider = false, fixed = false;
    double dt = 0.01;
    for (int i = 1; i < argc; ++i) {
        std::string a = argv[i];
        if (a == "--collider") collider = true;
        else if (a == "--fixed") fixed = true;
        else if (a.rfind("--dt=", 0) == 0) dt = std::atof(a.c_str() + 5);
        else if (pos == 0) { frames = std::atoi(a.c_str()); ++pos; }
        else if (pos == 1) { coarsest = std::atoi(a.c_str()); ++pos; }
        else if (pos == 2) { levels = std::atoi(a.c_str()); ++pos; }
    }
    astg_params p;
    astg_default_params(&p, coarsest, levels);
    astg_handle* h = nullptr;
    if (astg_create(&p, nullptr, &h) != ASTG_OK) {
        std::fprintf(stderr, "astg_create: %s\n", h ? astg_last_error(h) : "failed");
        astg_destroy(h);
        return 1;
    }
    auto check = [&](astg_status s, const char* what) {
        if (s == ASTG_OK || s == ASTG_NOT_CONVERGED) return true;
        std::fprintf(stderr, "%s: status %d: %s\n", what, (int)s, astg_last_error(h));
        return false;
    };
    bool ok = true;
    if (collider) ok = check(astg_set_collider_sphere(h, 0.5, 0.5, 0.45, 0.1), "astg_set_collider_sphere");
    if (ok) ok = check(astg_set_max_cfl(h, 2.0), "astg_set_max_cfl");
    std::vector<double> density;
    for (int f = 0; ok && f < frames; ++f) {
        astg_step_stats st;
        std::memset(&st, 0, sizeof st);
        int sub = 1;
        ok = check(fixed ? astg_step(h, dt, &st) : astg_update(h, dt, &sub, &st), fixed ? "astg_step" : "astg_update");
        if (!ok) break;
        size_t bytes = 0;
        astg_get(h, "density_oct", nullptr, 0, &bytes);
        density.resize(bytes / sizeof(double));
        ok = check(astg_get(h, "density_oct", density.data(), bytes, nullptr), "astg_get");
        if (!ok) break;
        double sum = 0;
        for (double v : density) sum += v;
        std::printf("frame %d substeps %d pcg_iterations %d ms %.3f density_sum %.17g\n", f, sub, st.solve.iterations,
                    st.ms_total, sum);
    }
    astg_destroy(h);
    return ok ? 0 : 1;
}
