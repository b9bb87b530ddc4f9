// Fixture harness for the reference's uniform 2-D AST smoke solver, ASTSolver<2>
// (include/ast_solver.h), the solver behind the reference's pybind ASTSolver2 (test
// infrastructure only).
//
// Links the reference's own sources (built by oracle/ref/Makefile) and runs the solver the way
// Solver::update (src/solver.cpp:8-46) does, dumping its state in the reference's storage order
// (x fastest).  onUpdate is restated stage by stage only to take per-stage snapshots: the stages
// are the reference's own member functions called in its order; the vortex image the reference
// writes at the start of a frame and saveResult's images are left out (they change no state).
// The grids' private members are read through an access-specifier redefinition applied after
// every standard and third-party header is in.
//
// Built twice.  ref_harness2d is the stock solver.  ref_harness2d_eval (-DASTG_EVALUATED_CORRECTION)
// differs in one expression only: ASTFaceGrid<double, 2>::sample's CORRECTION_MAC term
// (include/ast_face_grid.h:59-63) keeps `dual - mac_data->sample(vertex)` in an `auto` Eigen
// expression that refers to the temporary returned by sample(), which is destroyed before the
// expression is read; the stock build therefore reads a dead stack slot wherever an open tilt
// corrects the velocity (the adaptive runs from their second frame on).  The _eval build
// specialises that member with the difference evaluated into a vector, the arithmetic the
// expression spells out; every other function is the reference's own.
//
// usage: ref_harness2d RESX RESY FRAMES DT ADAPTIVE OUT [STAGE_FRAMES]
//   dumps the initial state, the state after every frame, and per-stage snapshots of every
//   sub-step of the first STAGE_FRAMES frames (default 1) into the archive OUT.
#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <functional>
#include <iostream>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <numeric>
#include <sstream>
#include <string>
#include <thread>
#include <tuple>
#include <type_traits>
#include <unordered_map>
#include <utility>
#include <vector>

#include "general.h"
#include "util.h"
#include "thread_pool.h"
#include "solver.h"
#include "static_for.h"
#include "box_iterator.h"
#include "cell_centered_grid.h"
#include "vertex_centered_grid.h"
#include "edge_centered_grid.h"
#include "pcgsolver/pcg_solver.h"
#include "viewer/image_dump.h"
#include "global_benchmark.h"
#include "archive.h"

#define private public
#define protected public
#include "ast_face_grid.h"
#ifdef ASTG_EVALUATED_CORRECTION
namespace ast {
template <>
Eigen::Matrix<double, 2, 1> ASTFaceGrid<double, 2>::sample(const Eigen::Matrix<double, 2, 1>& pos) const {
    using V2 = Eigen::Matrix<double, 2, 1>;
    using I2 = Eigen::Matrix<int, 2, 1>;
    V2 rp = pos / dx - V2::Ones() * 0.5, f;
    I2 idx;
    getBaryCentric(rp, resolution - I2::Ones(), idx, f);
    const V2 base = mac_data->sample(pos);
    const I2 corner = idx + I2::Ones();
    if (!layout->getTiltNode(corner).open) return base;
    const V2 atCorner = mac_data->sample(positionCenter<node_type::vertex_node>(corner));
    const V2 delta = dual_grid->template get<node_type::vertex_node>(corner) - atCorner;
    return base + 2 * delta * std::min(f.minCoeff(), (V2::Ones() - f).minCoeff());
}
}  // namespace ast
#endif
#include "ast_solver.h"
#undef private
#undef protected

using namespace ast;
using fixture::Archive;
using Idx2 = Eigen::Matrix<int, 2, 1>;

struct Harness : ASTSolver<2> {
    Harness(const Idx2& res, double dx, bool adaptive) : ASTSolver<2>(res, dx, adaptive, "harness2d") {}
    Archive* ar = nullptr;
    int frame = 0, stageFrames = 1, sub = 0;
    std::vector<double> subDt;

    void saveResult(int) override {}
    void onUpdate(REAL dt) override {
        subDt.push_back(dt);
        bool snap = frame < stageFrames;
        std::string p = "f" + std::to_string(frame + 1) + "/s" + std::to_string(sub) + "/";
        sphereSource2DSetup();
        if (snap) dumpState(p + "source/");
        addForce(dt);
        if (snap) dumpState(p + "force/");
        project(dt);
        if (snap) { dumpState(p + "project/"); dumpSystem(p + "project/"); }
        advect(dt);
        if (snap) dumpState(p + "advect/");
        start_of_frame = false;
        ++sub;
    }

    void dumpState(const std::string& p) {
        const int nx = resolution.x(), ny = resolution.y();
        std::vector<double> dc, dv, hc, hv, mx, my, tv, du;
        std::vector<uint8_t> open;
        std::vector<int32_t> pc, pv;
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) {
                Idx2 c(x, y);
                dc.push_back(density->get<node_type::cell_node>(c));
                hc.push_back(heat->get<node_type::cell_node>(c));
                pc.push_back(pIndex->get<node_type::cell_node>(c));
            }
        for (int y = 0; y <= ny; ++y)
            for (int x = 0; x <= nx; ++x) {
                Idx2 c(x, y);
                dv.push_back(density->get<node_type::vertex_node>(c));
                hv.push_back(heat->get<node_type::vertex_node>(c));
                const auto& u = velocity->get<node_type::vertex_node>(c);
                for (int k = 0; k < 4; ++k) tv.push_back(u[k]);
                const auto& w = velocity->dual_grid->get<node_type::vertex_node>(c);
                du.push_back(w[0]);
                du.push_back(w[1]);
                open.push_back(layout->getTiltNode(c).open ? 1 : 0);
                pv.push_back(pIndex->get<node_type::vertex_node>(c));
            }
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x <= nx; ++x) mx.push_back(velocity->get<node_type::cell_node, 0>(Idx2(x, y)));
        for (int y = 0; y <= ny; ++y)
            for (int x = 0; x < nx; ++x) my.push_back(velocity->get<node_type::cell_node, 1>(Idx2(x, y)));
        uint64_t cy = ny, cx = nx, vy = ny + 1, vx = nx + 1;
        ar->f64(p + "density_cell", dc, {cy, cx});
        ar->f64(p + "density_vert", dv, {vy, vx});
        ar->f64(p + "heat_cell", hc, {cy, cx});
        ar->f64(p + "heat_vert", hv, {vy, vx});
        ar->f64(p + "mac_x", mx, {cy, cx + 1});
        ar->f64(p + "mac_y", my, {cy + 1, cx});
        ar->f64(p + "tilt_vel", tv, {vy, vx, 4});
        ar->f64(p + "dual_vert", du, {vy, vx, 2});
        ar->u8(p + "tilt_open", open, {vy, vx});
        ar->i32(p + "pindex_cell", pc, {cy, cx});
        ar->i32(p + "pindex_vert", pv, {vy, vx});
    }
    void dumpSystem(const std::string& p) {
        std::vector<int32_t> rp(1, 0), col;
        std::vector<double> val;
        for (unsigned i = 0; i < A.n; ++i) {
            for (size_t j = 0; j < A.index[i].size(); ++j) {
                col.push_back((int32_t)A.index[i][j]);
                val.push_back(A.value[i][j]);
            }
            rp.push_back((int32_t)col.size());
        }
        ar->i32(p + "A_rowptr", rp);
        ar->i32(p + "A_col", col);
        ar->f64(p + "A_val", val);
        ar->f64(p + "b", b);
        ar->f64(p + "p", vRes);
    }
};

int main(int argc, char** argv) {
    if (argc < 7) {
        fprintf(stderr, "usage: ref_harness2d RESX RESY FRAMES DT ADAPTIVE OUT [STAGE_FRAMES]\n");
        return 2;
    }
    spdlog::set_level(spdlog::level::warn);
    int nx = atoi(argv[1]), ny = atoi(argv[2]), frames = atoi(argv[3]);
    double dt = atof(argv[4]);
    bool adaptive = atoi(argv[5]) != 0;
    Archive ar;
    Harness h(Idx2(nx, ny), 1.0 / nx, adaptive);
    h.ar = &ar;
    if (argc > 7) h.stageFrames = atoi(argv[7]);
    h.initialize();
    h.dumpState("init/");
    std::vector<int32_t> subs;
    for (int f = 0; f < frames; ++f) {
        h.frame = f;
        h.sub = 0;
        h.update(dt);
        subs.push_back(h.sub);
        h.dumpState("f" + std::to_string(f + 1) + "/");
    }
    ar.i32("substeps", subs);
    ar.f64("sub_dt", h.subDt);
    ar.write(argv[6]);
    return 0;
}
