// Fixture harness for the reference octree smoke solver (test infrastructure only).
//
// Links the reference's own sources (built by oracle/ref/Makefile) and runs the octree smoke
// step on the benchmark scene, dumping the solver state in the reference's own storage order:
// per level, slot = layout index (non-ghost nodes first in raster order, then ghosts in discovery
// order, src/octree_layer3.cpp:14-85), levels concatenated finest first.  The dumps are turned
// into the committed fixtures under tests/golden/ by tests/golden/make_golden.py, and they pin
// the oracle port in oracle/.
//
// Scene mapping (z-up reference frame):
//   * walls closed at x-, x+, y-, y+, z-; z+ open (Dirichlet p = 0); no collider, so the
//     collider SDF keeps the constant +1 that OmniBoundarySolver3's constructor gives it
//     (src/omni_boundary_solver3.cpp:13-17);
//   * sphere source re-injected every step as in example/octree_smoke_3d/main.cpp:23-86;
//   * split map and initial curl noise from ast-grid_gb300/csrc/scene.h;
//   * buoyancy, decay and PCG tolerance from the command line.
//
// usage: ref_harness --coarsest N --levels L --steps S --out DIR [--dt 0.01] [--tol 1e-6]
//        [--noise 1e-3] [--seed 0] [--buoy-d -0.1] [--buoy-t 1.0] [--decay 1.0] [--stages]
//        [--source cx,cy,cz,r] [--adaptive] [--max-cfl C] [--collider cx,cy,cz,r]
//        [--refine-obstacle level,lo,hi]...
#include "octree_omnigrid_solver3.h"
#include "octree_util.h"
#include "advection.h"
#include "jet/fmm_levelset_solver3.h"
#include "viewer/grid_dump.h"
#include "scene.h"
#include "archive.h"
#include "geometry/sphere3.h"
#include "geometry/rigid_body_collider3.h"

#include <array>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>
#include <sys/stat.h>

using namespace Omni;

namespace {

using fixture::Archive;

struct Options {
    int coarsest = 8, levels = 3, steps = 3;
    double dt = 0.01, tol = 1e-6, noise = 1e-3, buoyD = -0.1, buoyT = 1.0, decay = 1.0;
    uint64_t seed = 0;
    bool stages = false;
    // Solver::update's adaptive branch (useFixedTimeStep = false) with setMaxCfl(maxCfl)
    bool adaptive = false;
    double maxCfl = 3.0;
    // a sphere collider through OmniBoundarySolver3::updateCollider (the stock scene's obstacle
    // code path, src/omni_boundary_solver3.cpp:17-32, src/octree_omnigrid_solver3.cpp:153-158)
    bool collider = false;
    double col[4] = {0.5, 0.5, 0.45, 0.1};
    // refineSplitMapByObstacleSdf(splitMap, level, colliderSdf, [lo, hi]) after the scene's split map,
    // in the order given (include/octree_util.h:17-47)
    std::vector<std::array<double, 3>> refine;
    // FmmLevelSetSolver3::extrapolate of the density after the steps: sphere SDF (centre, radius),
    // maximum distance factor, validity offset (known where sdf < -offset * d)
    // checkpoint: after step ckptAt, write the reference's own binary dumps into ckptDir; restart:
    // start from such dumps through OctreeOmniGridSolver3::restart instead of the initial noise
    int ckptAt = -1;
    std::string ckptDir, restartDir;
    bool extrap = false;
    double exC[3] = {0, 0, 0}, exR = 0, exMax = 0, exOff = 0;
    std::string out = "ref_out";
    astg_scene::Sphere src = astg_scene::default_source();
};

}  // namespace

class Harness : public OctreeOmniGridSolver3 {
public:
    Options opt;
    std::vector<int32_t> split;
    int stepIdx = 0;
    // PCG record of the last projection
    int pcgIters = 0;
    double pcgErr = 0, ambT = 0;
    bool pcgConverged = false;

    Harness(const Options& o, int res)
        : OctreeOmniGridSolver3(Size3(res, res, res), 1.0 / res, "harness"), opt(o) {
        _buoyancySmokeDensityFactor = o.buoyD;
        _buoyancyTemperatureFactor = o.buoyT;
        _smokeDecayFactor = o.decay;
        _temperatureDecayFactor = o.decay;
        isRestart = true;  // only suppresses the layout.bin dump in initData (:147-148)
        useFixedTimeStep = !o.adaptive;
        if (o.adaptive) setMaxCfl(o.maxCfl);
        numOctreeLayer = o.levels;
        split = astg_scene::split_map(res, o.levels, o.src);
        splitMapSetup = [this, res](OctreeOmniGridSolver3* s) {
            auto& sm = s->getSplitMap();
            for (int z = 0; z < res; ++z)
                for (int y = 0; y < res; ++y)
                    for (int x = 0; x < res; ++x) sm->set(x, y, z, split[((size_t)z * res + y) * res + x]);
            if (!opt.refine.empty()) {
                // the collider's SDF grid, built the way initObstacle will build it
                OmniBoundarySolver3 bs(Size3(res, res, res), 1.0 / res);
                Sphere3Ptr sphere = std::make_shared<Sphere3>(opt.col[3], Transform3(Vector3f(opt.col[0], opt.col[1], opt.col[2]), Quaternion()));
                bs.updateCollider(std::make_shared<RigidBodyCollider3>(sphere));
                auto sdf = bs.colliderSdf();
                for (auto& r : opt.refine) refineSplitMapByObstacleSdf(sm, (int)r[0], sdf, Vector2f(r[1], r[2]));
                for (int z = 0; z < res; ++z)
                    for (int y = 0; y < res; ++y)
                        for (int x = 0; x < res; ++x) split[((size_t)z * res + y) * res + x] = sm->get(x, y, z);
            }
        };
        sceneSetup = [this](OctreeOmniGridSolver3* s) { source(s); };
    }

    // ------------------------------------------------------------ scene
    void initObstacle() override {
        boundarySolver->setClosedDomainBoundaryFlag(kDirectionXNegative | kDirectionXPositive | kDirectionYNegative |
                                                    kDirectionYPositive | kDirectionZNegative);
        if (opt.collider) {
            Sphere3Ptr sphere = std::make_shared<Sphere3>(opt.col[3], Transform3(Vector3f(opt.col[0], opt.col[1], opt.col[2]), Quaternion()));
            boundarySolver->updateCollider(std::make_shared<RigidBodyCollider3>(sphere));
        }
        boundarySdf = boundarySolver->colliderSdf();
    }
    void saveResult(int) override {}
    // sub-step counts the adaptive update computed during the current frame
    mutable std::vector<int> subLog;
    int numberOfSubTimeSteps(REAL dt) const override {
        int k = OctreeOmniGridSolver3::numberOfSubTimeSteps(dt);
        subLog.push_back(k);
        return k;
    }

    bool inSrc(const Vector3f& p) const { return astg_scene::inside(opt.src, p.x(), p.y(), p.z()); }

    // example/octree_smoke_3d/main.cpp:23-86 with the mapped sphere and initV = 1
    void source(OctreeOmniGridSolver3* s) {
        const double initV = 1.0;
        auto& d = s->getDensity();
        auto& h = s->getHeat();
        auto& dO = d->getOctagonGrid();
        auto& dT = d->getTiltGrid();
        auto& hO = h->getOctagonGrid();
        auto& hT = h->getTiltGrid();
        iterate_grid(iter, dO) {
            if (inSrc(dO->position(iter.levelCoor()))) {
                dO->set(iter.levelCoor(), 1);
                hO->set(iter.levelCoor(), 1);
            }
        }
        iterate_grid(iter, dT) {
            if (inSrc(dT->position(iter.levelCoor()))) {
                dT->set(iter.levelCoor(), 1);
                hT->set(iter.levelCoor(), 1);
            }
        }
        for (auto lCoor : s->getLayout()->getHalfGhostIdx()) {
            if (inSrc(dT->position(lCoor))) {
                dT->set(lCoor, 1);
                hT->set(lCoor, 1);
            }
        }
        auto& vel = s->getVelocity();
        auto& mac = vel->getMACGrid();
        auto& tg = vel->getTiltGrid();
        iterate_grid(iter, mac) {
            if (inSrc(mac->positionZ(iter.levelCoor()))) mac->setZ(iter.levelCoor(), initV);
            if (inSrc(tg->positionCenter(iter.levelCoor()))) tg->set(iter.levelCoor(), Vector8f::Ones() * initV * INV_SQRT3);
        }
        for (auto lCoor : s->getLayout()->getHalfGhostIdx()) {
            auto pos = tg->positionCenter(lCoor);
            if (inSrc(pos)) {
                Vector8f nv = Vector8f::Zero();
                auto tNode = s->getTiltEGrid()->get(lCoor);
                for (int i = 0; i < 4; ++i) nv(HALF_TILT_SLOT_INDEX[tNode.half_direction][i]) = initV * INV_SQRT3;
                if (tNode.half_direction % 3 == 2) nv(HALF_TILT_SLOT_INDEX[tNode.half_direction][4]) = initV;
                tg->set(lCoor, nv);
            }
        }
        static bool first = true;
        if (first) {
            d->updateGhost();
            h->updateGhost();
            first = false;
        }
    }

    // initial curl noise on non-ghost MAC faces, open tilts and half tilts
    void initNoise() {
        astg_scene::CurlNoise cn(opt.seed, opt.noise);
        auto& mac = velocity->getMACGrid();
        auto& tg = velocity->getTiltGrid();
        iterate_grid(iter, mac) {
            int l = iter.level, x = iter.xIdx(), y = iter.yIdx(), z = iter.zIdx();
            for (int axis = 0; axis < 3; ++axis) {
                if (!mac->isValid(axis, l, x, y, z)) continue;
                Vector3f p = mac->position(axis, l, x, y, z);
                double pp[3] = {p.x(), p.y(), p.z()}, u[3];
                cn.velocity(pp, u);
                mac->set(axis, iter.levelCoor(), u[axis]);
            }
            if (tilt_layout->isTiltOpen(iter.levelCoor())) {
                Vector8f v;
                for (int k = 0; k < 8; ++k) {
                    Vector3f p = tg->positionTilt(iter.levelCoor(), k);
                    double pp[3] = {p.x(), p.y(), p.z()}, u[3];
                    cn.velocity(pp, u);
                    v(k) = Vector3f(u[0], u[1], u[2]).dot(TILT3_UNIT_DIR_UP[k]);
                }
                tg->set(iter.levelCoor(), v);
            }
        }
        for (auto lCoor : layout->getHalfGhostIdx()) {
            Vector8f v = Vector8f::Zero();
            const auto& tNode = tiltE->get(lCoor);
            for (int i = 0; i < 5; ++i) {
                int k = HALF_TILT_SLOT_INDEX[tNode.half_direction][i];
                Vector3f p = (i == 4) ? tg->positionCenter(lCoor) : tg->positionTilt(lCoor, k);
                double pp[3] = {p.x(), p.y(), p.z()}, u[3];
                cn.velocity(pp, u);
                v(k) = Vector3f(u[0], u[1], u[2]).dot((i == 4) ? HALF_TILT_XYZ_DIR_POSITIVE[k] : TILT3_UNIT_DIR_UP[k]);
            }
            tg->set(lCoor, v);
        }
    }

    void setTolerance() { pcgSolver.set_solver_parameters(opt.tol, 3000); }
    // the reference's own dump functions (src/viewer/grid_dump.cpp:280-615) on the current state,
    // the files saveResult writes with saveStatus (src/octree_omnigrid_solver3.cpp:148, 996-1007)
    void writeCheckpoint(const std::string& d) {
        dumpOctreeLayout3dBinary(d + "/layout.bin", *layout);
        dumpOctreeOmniTiltE3dBinary(d + "/tilt.bin", *tiltE);
        dumpOctreeOmniScalar3dBinary(d + "/density.bin", *density);
        dumpOctreeOmniScalar3dBinary(d + "/heat.bin", *heat);
        dumpOctreeOmniFaceCentered3dBinary(d + "/velocity.bin", *velocity);
    }
    int pcgItersN() const { return (int)b.size(); }

    // ------------------------------------------------------------ dumps
    int levels() { return layout->level(); }
    size_t slots() {
        size_t s = 0;
        for (int l = 0; l < levels(); ++l) s += layout->levelSize(l);
        return s;
    }
    LCOOR_T slotLCoor(int l, int i) {
        auto layer = layout->getLayerPtr(l);
        int n = layer->nodeSize();
        LCOOR_T c = i < n ? layer->getNodeIdx()[i] : layer->getGhostNodeIdx()[i - n];
        return PACK_LCOOR3(l, UNPACK_X3(c), UNPACK_Y3(c), UNPACK_Z3(c));
    }

    void dumpLayout(Archive& ar) {
        std::vector<int32_t> meta = {resolution.x(), levels()};
        std::vector<int32_t> sizes, coords;
        for (int l = 0; l < levels(); ++l) {
            auto layer = layout->getLayerPtr(l);
            sizes.push_back(layer->nodeSize());
            sizes.push_back(layer->ghostNodeSize());
            sizes.push_back(layer->size());
            for (int i = 0; i < layer->size(); ++i) {
                LCOOR_T c = slotLCoor(l, i);
                auto& node = layer->node(UNPACK_COOR3(c));
                if ((int)node.index != i) throw std::runtime_error("layout index mismatch");
                coords.push_back(UNPACK_X3(c));
                coords.push_back(UNPACK_Y3(c));
                coords.push_back(UNPACK_Z3(c));
                coords.push_back((int32_t)node.flag);
            }
        }
        ar.i32("meta", meta);
        ar.i32("level_sizes", sizes, {(uint64_t)levels(), 3});
        ar.i32("slot_coords", coords, {(uint64_t)(coords.size() / 4), 4});
        ar.i32("split_map", split);
        if (opt.collider) {  // the collider SDF grid the solver samples, index (z * res + y) * res + x
            int r = resolution.x();
            std::vector<double> sd((size_t)r * r * r);
            for (int z = 0; z < r; ++z)
                for (int y = 0; y < r; ++y)
                    for (int x = 0; x < r; ++x) sd[((size_t)z * r + y) * r + x] = boundarySdf->get(x, y, z);
            ar.f64("collider_sdf", sd);
        }
        auto toVec = [](const std::vector<LCOOR_T>& v) { return std::vector<int64_t>(v.begin(), v.end()); };
        ar.i64("half_tilts", toVec(layout->getHalfGhostIdx()));
        std::vector<int64_t> tj = toVec(layout->getTJointArr());
        std::sort(tj.begin(), tj.end());  // recorded under a mutex in parallel: order is not defined
        ar.i64("t_joints", tj);
        ar.i64("closed_by_half_tilt", toVec(layout->getclosedByHalfTiltArr()));
        // weights (init-only)
        std::vector<double> wm, wt;
        for (int a = 0; a < 3; ++a)
            for (int l = 0; l < levels(); ++l)
                for (double v : weightsCC->getMACGrid()->getU(a)[l]) wm.push_back(v);
        for (int l = 0; l < levels(); ++l)
            for (auto& v : weightsCC->getTiltGrid()->getGridPtr()->getData()[l])
                for (int k = 0; k < 8; ++k) wt.push_back(v(k));
        ar.f64("w_mac", wm, {3, (uint64_t)slots()});
        // least-squares recovery tables, src/constants.cpp:170-256; index bits x y z n0 n1 n2 n3
        std::vector<double> tab;
        for (int bits = 0; bits < 128; ++bits) {
            int q[7];
            for (int k = 0; k < 7; ++k) q[k] = (bits >> (6 - k)) & 1;
            const Matrix37f& m = Constants::OCTREE_OMNI_DUAL_GRAPH_EIGEN_MATRIX3[q[0]][q[1]][q[2]][q[3]][q[4]][q[5]][q[6]];
            for (int r = 0; r < 3; ++r)
                for (int c = 0; c < 7; ++c) tab.push_back(m(r, c));
        }
        ar.f64("dual_tables", tab, {128, 3, 7});
        ar.f64("w_tilt", wt, {(uint64_t)slots(), 8});
    }

    void dumpGrids(Archive& ar, const std::string& p, OctreeOmniScalarGrid3Ptr& den, OctreeOmniScalarGrid3Ptr& hea,
                   OctreeOmniFaceCenteredGrid3Ptr& vel, bool withLayoutFlags) {
        size_t S = slots();
        auto scal = [&](OctreeOmniScalarGrid3Ptr& g, std::vector<double>& oct, std::vector<double>& til) {
            for (int l = 0; l < levels(); ++l) {
                for (double v : g->getOctagonGrid()->getData()[l]) oct.push_back(v);
                for (double v : g->getTiltGrid()->getData()[l]) til.push_back(v);
            }
        };
        std::vector<double> dO, dT, hO, hT;
        scal(den, dO, dT);
        scal(hea, hO, hT);
        ar.f64(p + "density_oct", dO);
        ar.f64(p + "density_tilt", dT);
        ar.f64(p + "heat_oct", hO);
        ar.f64(p + "heat_tilt", hT);
        std::vector<double> mac;
        for (int a = 0; a < 3; ++a)
            for (int l = 0; l < levels(); ++l)
                for (double v : vel->getMACGrid()->getU(a)[l]) mac.push_back(v);
        ar.f64(p + "mac", mac, {3, (uint64_t)S});
        std::vector<double> tv;
        for (int l = 0; l < levels(); ++l)
            for (auto& v : vel->getTiltGrid()->getGridPtr()->getData()[l])
                for (int k = 0; k < 8; ++k) tv.push_back(v(k));
        ar.f64(p + "tilt_vel", tv, {(uint64_t)S, 8});
        std::vector<double> dualO, dualT;
        auto& dual = vel->getDualGrid();
        for (int l = 0; l < levels(); ++l) {
            for (auto& v : dual->getOctagonGrid()->getData()[l])
                for (int k = 0; k < 3; ++k) dualO.push_back(v(k));
            for (auto& v : dual->getTiltGrid()->getData()[l])
                for (int k = 0; k < 3; ++k) dualT.push_back(v(k));
        }
        ar.f64(p + "dual_oct", dualO, {(uint64_t)S, 3});
        ar.f64(p + "dual_tilt", dualT, {(uint64_t)S, 3});
        // tilt-E state of the grid the velocity uses, and the open/fixed layout flags
        std::vector<double> e;
        std::vector<int32_t> fl;
        std::vector<uint8_t> open;
        auto& te = vel->getTiltEGridPtr();
        for (int l = 0; l < levels(); ++l) {
            for (int i = 0; i < layout->levelSize(l); ++i) {
                LCOOR_T c = slotLCoor(l, i);
                const TiltENode& n = te->get(c);
                e.push_back(n.e);
                fl.push_back((n.is_largest ? 1 : 0) | (n.is_closed ? 2 : 0) | (n.is_fixed ? 4 : 0) |
                             (n.is_T_joint ? 8 : 0) | (n.is_closed_by_T_joint ? 16 : 0) | (n.is_half_tilt ? 32 : 0));
                fl.push_back(n.half_direction);
                auto& s = tilt_layout->getTiltNode(c);
                open.push_back((s.is_open ? 1 : 0) | (s.is_fixed ? 2 : 0));
            }
        }
        ar.f64(p + "tilt_e", e);
        ar.i32(p + "tilt_flags", fl, {(uint64_t)S, 2});
        if (withLayoutFlags) ar.u8(p + "tilt_open", open);
    }

    // current grids, plus the swap partners under "t_" (the reference double-buffers them)
    void dumpState(Archive& ar, const std::string& p) {
        dumpGrids(ar, p, density, heat, velocity, true);
        dumpGrids(ar, p + "t_", tDensity, tHeat, tVelocity, false);
    }

    void dumpProjection(Archive& ar, const std::string& p) {
        std::vector<int32_t> pio, pit;
        for (int l = 0; l < levels(); ++l) {
            for (int v : pIndex->getOctagonGrid()->getData()[l]) pio.push_back(v);
            for (int v : pIndex->getTiltGrid()->getData()[l]) pit.push_back(v);
        }
        ar.i32(p + "pindex_oct", pio);
        ar.i32(p + "pindex_tilt", pit);
        FixedSparseMatrix<double> F;
        F.construct_from_matrix(A);
        ar.i32(p + "A_rowptr", std::vector<int32_t>(F.rowstart.begin(), F.rowstart.end()));
        ar.i32(p + "A_col", std::vector<int32_t>(F.colindex.begin(), F.colindex.end()));
        ar.f64(p + "A_val", F.value);
        ar.f64(p + "b", std::vector<double>(b.data(), b.data() + b.size()));
        ar.f64(p + "p", std::vector<double>(vRes.data(), vRes.data() + vRes.size()));
        ar.i32(p + "pcg_iters", std::vector<int32_t>{pcgIters, pcgConverged ? 1 : 0});
        ar.f64(p + "pcg_err", std::vector<double>{pcgErr});
        ar.f64(p + "ambT", std::vector<double>{ambT});
    }

    Archive stageAr;
    void stage(const std::string& name) {
        if (opt.stages) dumpState(stageAr, "s" + std::to_string(stepIdx) + "_" + name + "/");
    }

    // Same call sequence as OctreeOmniGridSolver3::onUpdate (src/octree_omnigrid_solver3.cpp:222-249),
    // with state snapshots between the stages and the PCG iteration count recorded.
    void onUpdate(REAL dt) override {
        if (sceneSetup) sceneSetup(this);
        stage("scene");
        wipeBoundary();
        {
            Real amb = 0.0;
            int count = 0;
            for (size_t i = 0; i < heat->getOctagonGrid()->getData().size(); ++i) {
                Real tSum = BLAS::sum(heat->getOctagonGrid()->getData()[i]);
                amb += tSum * (i == 0 ? 1 : 8);
                count += heat->getOctagonGrid()->getData()[i].size() * (i == 0 ? 1 : 8);
            }
            ambT = amb / Real(count);
        }
        addForce(dt);
        stage("force");
        boundarySolver->constrainVelocity(velocity->getMACGrid());
        boundarySolver->constrainVelocity(velocity->getTiltGrid(), velocity->getMACGrid());
        velocity->updateGhost();
        stage("preproject");
        project(dt);
        {
            // re-run the same deterministic solve on the assembled system to read its
            // iteration count, which project() only logs
            PCGSolver<REAL> s2;
            s2.set_solver_parameters(opt.tol, 3000);
            VectorXd x2(b.size());
            double err;
            int it;
            pcgConverged = s2.solve(A, b, x2, err, it);
            pcgIters = it;
            pcgErr = err;
            double maxd = 0;
            for (int i = 0; i < b.size(); ++i) maxd = std::max(maxd, std::fabs(x2[i] - vRes[i]));
            if (maxd != 0) fprintf(stderr, "warning: PCG re-solve differs by %g\n", maxd);
        }
        if (opt.stages) dumpProjection(stageAr, "s" + std::to_string(stepIdx) + "_proj/");
        stage("project");
        boundarySolver->constrainVelocity(velocity->getMACGrid());
        boundarySolver->constrainVelocity(velocity->getTiltGrid(), velocity->getMACGrid());
        velocity->updateGhost();
        velocity->updateDualGrid();
        boundarySolver->constrainVelocity(velocity->getDualGrid());
        velocity->getDualGrid()->updateGhost();
        stage("dual");
        advect(dt);
        stage("advect");
    }
};

static void parseSource(const char* s, astg_scene::Sphere& sp) {
    if (sscanf(s, "%lf,%lf,%lf,%lf", &sp.cx, &sp.cy, &sp.cz, &sp.r) != 4) throw std::runtime_error("bad --source");
}

int main(int argc, char** argv) {
    Options o;
    for (int i = 1; i < argc; ++i) {
        std::string a = argv[i];
        auto next = [&]() -> const char* {
            if (i + 1 >= argc) throw std::runtime_error("missing value for " + a);
            return argv[++i];
        };
        if (a == "--coarsest") o.coarsest = atoi(next());
        else if (a == "--levels") o.levels = atoi(next());
        else if (a == "--steps") o.steps = atoi(next());
        else if (a == "--dt") o.dt = atof(next());
        else if (a == "--tol") o.tol = atof(next());
        else if (a == "--noise") o.noise = atof(next());
        else if (a == "--seed") o.seed = strtoull(next(), nullptr, 10);
        else if (a == "--buoy-d") o.buoyD = atof(next());
        else if (a == "--buoy-t") o.buoyT = atof(next());
        else if (a == "--decay") o.decay = atof(next());
        else if (a == "--stages") o.stages = true;
        else if (a == "--adaptive") o.adaptive = true;
        else if (a == "--max-cfl") o.maxCfl = atof(next());
        else if (a == "--refine-obstacle") {
            std::array<double, 3> r;
            if (sscanf(next(), "%lf,%lf,%lf", &r[0], &r[1], &r[2]) != 3) throw std::runtime_error("--refine-obstacle level,lo,hi");
            o.refine.push_back(r);
        } else if (a == "--collider") {
            o.collider = true;
            if (sscanf(next(), "%lf,%lf,%lf,%lf", &o.col[0], &o.col[1], &o.col[2], &o.col[3]) != 4)
                throw std::runtime_error("--collider cx,cy,cz,r");
        }
        else if (a == "--out") o.out = next();
        else if (a == "--source") parseSource(next(), o.src);
        else if (a == "--checkpoint-at") o.ckptAt = atoi(next());
        else if (a == "--checkpoint-dir") o.ckptDir = next();
        else if (a == "--restart") o.restartDir = next();
        else if (a == "--extrapolate") {
            o.extrap = true;
            if (sscanf(next(), "%lf,%lf,%lf,%lf,%lf,%lf", &o.exC[0], &o.exC[1], &o.exC[2], &o.exR, &o.exMax, &o.exOff) != 6)
                throw std::runtime_error("--extrapolate cx,cy,cz,r,max_distance_factor,offset");
        }
        else throw std::runtime_error("unknown option " + a);
    }
    spdlog::set_level(spdlog::level::err);
    mkdir(o.out.c_str(), 0755);
    int res = o.coarsest << (o.levels - 1);
    Harness h(o, res);
    h.initialize();
    h.setTolerance();
    if (o.restartDir.empty()) {
        h.initNoise();
    } else {
        const std::string& d = o.restartDir;
        if (!h.restart(0, d + "/layout.bin", d + "/boundary.bin", d + "/tilt.bin", d + "/density.bin", d + "/heat.bin",
                       d + "/velocity.bin"))
            throw std::runtime_error("restart failed");
        Archive ra;
        h.dumpState(ra, "restart/");
        ra.write(o.out + "/restart.astg");
    }

    Archive lay;
    h.dumpLayout(lay);
    h.dumpState(lay, "init/");
    lay.write(o.out + "/layout.astg");
    std::vector<int> sizes0;
    for (int l = 0; l < h.levels(); ++l) sizes0.push_back(h.getLayout()->levelSize(l));

    for (int s = 0; s < o.steps; ++s) {
        h.stepIdx = s;
        h.stageAr.entries.clear();
        h.subLog.clear();
        Timer t;
        h.update(o.dt);
        double secs = t.durationInSeconds();
        Archive st;
        h.dumpState(st, "");
        h.dumpProjection(st, "");
        st.f64("wall_s", std::vector<double>{secs});
        if (o.adaptive) st.i32("substeps", h.subLog);
        char name[64];
        snprintf(name, sizeof name, "/step_%04d.astg", s + 1);
        st.write(o.out + name);
        if (o.stages) {
            snprintf(name, sizeof name, "/stages_%04d.astg", s + 1);
            h.stageAr.write(o.out + name);
        }
        fprintf(stderr, "step %d: n=%d iters=%d err=%.3e %.3fs\n", s + 1, (int)h.pcgItersN(), h.pcgIters, h.pcgErr, secs);
        if (s + 1 == o.ckptAt) h.writeCheckpoint(o.ckptDir);
    }
    for (int l = 0; l < h.levels(); ++l)
        if (h.getLayout()->levelSize(l) != sizes0[l]) fprintf(stderr, "warning: level %d grew during the run\n", l);
    if (o.extrap) {
        // sphere signed distance at the finest cell centres, sampled by the reference's trilinear
        // CellCenteredGrid::sample; the density is extrapolated in place (input and output are one grid)
        auto sdf = std::make_shared<CellCenteredScalarGrid3>(Size3(res, res, res), 1.0 / res, 0.0);
        std::vector<double> sv((size_t)res * res * res);
        for (int z = 0; z < res; ++z)
            for (int y = 0; y < res; ++y)
                for (int x = 0; x < res; ++x) {
                    double p[3] = {(x + 0.5) / res, (y + 0.5) / res, (z + 0.5) / res};
                    double dx = p[0] - o.exC[0], dy = p[1] - o.exC[1], dz = p[2] - o.exC[2];
                    double v = std::sqrt(dx * dx + dy * dy + dz * dz) - o.exR;
                    sdf->set(x, y, z, v);
                    sv[((size_t)z * res + y) * res + x] = v;
                }
        double off = o.exOff;
        auto& den = h.getDensity();
        jet::FmmLevelSetSolver3 fmm;
        fmm.extrapolate<REAL, CellCenteredScalarGrid3Ptr>(den, sdf, o.exMax, den, nullptr,
                                                          [off](REAL d, REAL v) { return v < -off * d; });
        Archive ex;
        ex.f64("sdf", sv);
        std::vector<double> dO, dT;
        for (int l = 0; l < h.levels(); ++l) {
            for (double v : den->getOctagonGrid()->getData()[l]) dO.push_back(v);
            for (double v : den->getTiltGrid()->getData()[l]) dT.push_back(v);
        }
        ex.f64("density_oct", dO);
        ex.f64("density_tilt", dT);
        ex.write(o.out + "/extrap.astg");
    }
    return 0;
}
