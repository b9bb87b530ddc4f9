"""Pins the CPU oracle against the reference solver's own output (golden fixtures made by
tests/golden/make_golden.py from the reference's sources).  With the reference's reduction
order (reduce_mode=0) the oracle reproduces the reference bit for bit: topology, DOF numbering,
matrix, PCG iterates and every field after every step."""
import numpy as np
import pytest

from fixtures import FIELDS, LAYOUT, PROJ, STAGES, assert_same, case, golden, state
from oracle.oracle import Oracle

DT = 0.01


@pytest.mark.parametrize("name", ["ref_c8_l3", "ref_c16_l2"])
def test_layout_and_initial_state(name):
    g = golden(name)
    c, lv, _ = case(name)
    o = Oracle(c, lv)
    for k in LAYOUT:
        assert_same(k, g[k], o.get(k))
    # least-squares tables (src/constants.cpp:170-256), NaN pattern included
    assert_same("dual_tables", g["dual_tables"], o.get("dual_tables"))
    init = state(g, "init/")
    for k in FIELDS:
        assert_same("init/" + k, init[k], o.get(k))
    assert_same("init/tilt_open", init["tilt_open"], o.get("tilt_open"))


@pytest.mark.parametrize("name", ["ref_c8_l3", "ref_c16_l2"])
def test_free_running_steps_bit_exact(name):
    g = golden(name)
    c, lv, steps = case(name)
    o = Oracle(c, lv)
    for k in range(1, steps + 1):
        o.step(DT)
        st = state(g, f"step{k}/")
        for f in FIELDS + ["tilt_open"]:
            assert_same(f"step{k}/{f}", st[f], o.get(f))
        for f in PROJ:
            assert_same(f"step{k}/{f}", st[f], o.get(f))
    assert o.get("anomalies")[0] == 0


def test_stages_bit_exact_from_reference_inputs():
    """Each stage of step 1, started from the reference's own input state for that stage."""
    g = golden("ref_c8_l3")
    c, lv, _ = case("ref_c8_l3")
    o = Oracle(c, lv)
    prev = state(g, "init/")
    for i, s in enumerate(STAGES):
        for f in FIELDS:
            o.set(f, prev[f])
            o.set("t_" + f, prev["t_" + f])
        o.set("tilt_open", prev["tilt_open"])
        o.stage(i, DT)
        cur = state(g, f"stage1_{s}/")
        for f in FIELDS + ["tilt_open"]:
            assert_same(f"{s}/{f}", cur[f], o.get(f))
        prev = cur


def test_tree_reduction_mode_matches_reference_order_closely():
    """The CUDA library's reduction tree changes only rounding of the dot products and of the
    mean temperature: one step agrees with the reference to the PCG tolerance."""
    g = golden("ref_c8_l3")
    c, lv, _ = case("ref_c8_l3")
    o = Oracle(c, lv, reduce_mode=1)
    o.step(DT)
    st = state(g, "step1/")
    assert abs(int(o.get("pcg_iters")[0]) - int(st["pcg_iters"][0])) <= 1
    p_ref = st["p"]
    assert np.abs(o.get("p") - p_ref).max() <= 1e-6 * np.abs(p_ref).max()
    for f in ["density_oct", "heat_oct", "mac", "tilt_vel"]:
        ref = st[f]
        assert np.abs(o.get(f) - ref).max() <= 1e-6 * max(np.abs(ref).max(), 1e-30), f


@pytest.mark.parametrize("name", ["ref_c8_l3", "ref_c16_l2"])
def test_standalone_pcg_reproduces_reference_solution(name):
    """PCGSolver::solve on the reference's own assembled system: same iterates, bit for bit."""
    g = golden(name)
    c, lv, steps = case(name)
    o = Oracle(c, lv)
    for k in range(1, steps + 1):
        st = state(g, f"step{k}/")
        x, it = o.solve(st["A_rowptr"], st["A_col"], st["A_val"], st["b"])
        assert it == int(st["pcg_iters"][0])
        assert_same(f"step{k}/p", st["p"], x)


@pytest.mark.parametrize("name", ["ref_extrap_c8_l3", "ref_extrap_c16_l2"])
def test_extrapolation_bit_exact(name):
    """FmmLevelSetSolver3::extrapolate (include/jet/fmm_levelset_solver3.h:84-408) on the
    reference's own state: the oracle's heap march assigns the same values bit for bit."""
    g = golden(name)
    c, lv, _ = g["meta/case"].tolist()
    cx, cy, cz, r, maxf, off = g["meta/extrap"].tolist()
    o = Oracle(c, lv)
    before = state(g, "before/")
    for k in FIELDS:
        o.set(k, before[k])
    n = o.extrapolate("density", g["sdf"], off, maxf)
    assert n > 100
    assert_same("after/density_oct", g["after/density_oct"], o.get("density_oct"))
    assert_same("after/density_tilt", g["after/density_tilt"], o.get("density_tilt"))
    changed = np.sum(g["after/density_oct"] != before["density_oct"]) + np.sum(g["after/density_tilt"] != before["density_tilt"])
    assert changed > 50


@pytest.mark.parametrize("name", ["ref_c32_l3_hashes", "ref_c64_l3_hashes"])
def test_full_size_hashes_match_reference(name):
    """Config 0 at its full length (32^3 coarsest x 3 levels, 50 steps) and the benchmark size (64^3
    x 3 levels, 20 steps): after every step the oracle (reference reduction order) hashes to the
    reference's own arrays -- every state field, the tilt layout, the DOF maps, the pressure and
    the PCG iteration count."""
    import json
    import os
    import sys

    from fixtures import GOLDEN

    sys.path.insert(0, GOLDEN)
    import make_golden

    rec = json.load(open(os.path.join(GOLDEN, name + ".json")))
    c, lv, steps = rec["case"]
    o = Oracle(c, lv, openmp=True)
    for k in range(steps):
        o.step(rec["dt"])
        got = make_golden.step_hashes(o.get)
        bad = [f for f in got if got[f] != rec["steps"][k][f]]
        assert not bad, f"step {k + 1}: {bad}"


def test_adaptive_substeps_bit_exact():
    """Solver::update's adaptive branch (useFixedTimeStep = false, setMaxCfl(2); src/solver.cpp:21-41,
    numberOfSubTimeSteps / cfl at src/octree_omnigrid_solver3.cpp:1060-1122) for six frames of dt 0.25:
    the oracle takes the reference's sub-step counts and reproduces every field after each frame."""
    g = golden("ref_cfl_c8_l3")
    c, lv, frames = case("ref_cfl_c8_l3")
    dt, max_cfl = g["meta/adaptive"].tolist()
    o = Oracle(c, lv)
    counts = []
    for k in range(1, frames + 1):
        ks = o.update(dt, max_cfl)
        st = state(g, f"frame{k}/")
        assert ks == st["substeps"].tolist(), f"frame {k}"
        counts += ks
        for f in FIELDS + ["tilt_open", "pindex_oct", "pindex_tilt", "p", "pcg_iters"]:
            assert_same(f"frame{k}/{f}", st[f], o.get(f))
    assert max(counts) >= 3  # the case does sub-step


def collider_oracle(name, **kw):
    g = golden(name)
    c, lv, _ = case(name)
    o = Oracle(c, lv, **kw)
    o.set("collider_sdf", g["collider_sdf"])
    return o, g


def test_collider_weights_and_steps_bit_exact():
    """The stock obstacle (a sphere r = 0.1 at (0.5, 0.5, 0.45), OmniBoundarySolver3::updateCollider) in
    the benchmark scene: with the reference's collider SDF grid the oracle reproduces its cut-cell
    weights (initCuttingCellWeights, src/octree_omnigrid_solver3.cpp:1169-1238) and every step --
    wipeBoundary, the inside-solid constrainVelocity, the DOF threshold and the back-trace clamp."""
    name = "ref_col_c8_l3"
    o, g = collider_oracle(name)
    c, lv, steps = case(name)
    for k in ["w_mac", "w_tilt"]:
        assert_same(k, g[k], o.get(k))
    assert (g["w_mac"] < 1).sum() > 10 and (g["w_tilt"] < 1).sum() > 100
    for k in range(1, steps + 1):
        o.step(DT)
        st = state(g, f"step{k}/")
        for f in FIELDS + ["tilt_open"] + ["pindex_oct", "pindex_tilt", "A_rowptr", "A_col", "A_val", "b", "p",
                                           "pcg_iters"]:
            assert_same(f"step{k}/{f}", st[f], o.get(f))


def test_collider_stages_bit_exact_from_reference_inputs():
    o, g = collider_oracle("ref_col_c8_l3")
    prev = state(g, "init/")
    for i, s in enumerate(STAGES):
        for f in FIELDS:
            o.set(f, prev[f])
            o.set("t_" + f, prev["t_" + f])
        o.set("tilt_open", prev["tilt_open"])
        o.stage(i, DT)
        cur = state(g, f"stage1_{s}/")
        for f in FIELDS + ["tilt_open"]:
            assert_same(f"{s}/{f}", cur[f], o.get(f))
        prev = cur


def test_collider_racy_case_close_to_reference():
    """16^3 x 2 levels: the sphere's solid faces span two of the reference's worker runs, whose
    concurrent writes make the inside-solid projection depend on thread timing there.  The oracle's
    order (every sample reads the velocity before the projection) gives the same cut-cell weights, DOF
    maps and iteration counts, and fields within the race's footprint: faces 1e-3, pressure 3e-3,
    density 1e-5 of their largest magnitudes over three steps."""
    from fixtures import max_rel

    o, g = collider_oracle("ref_col_c16_l2")
    _, _, steps = case("ref_col_c16_l2")
    for k in ["w_mac", "w_tilt"]:
        assert_same(k, g[k], o.get(k))
    for k in range(1, steps + 1):
        o.step(DT)
        st = state(g, f"step{k}/")
        for f in ["tilt_open", "pindex_oct", "pindex_tilt", "A_rowptr", "A_col", "pcg_iters"]:
            assert_same(f"step{k}/{f}", st[f], o.get(f))
        assert max_rel(st["mac"], o.get("mac")) <= 1e-3
        assert max_rel(st["p"], o.get("p")) <= 3e-3
        for f in ["density_oct", "density_tilt", "heat_oct", "heat_tilt"]:
            assert max_rel(st[f], o.get(f)) <= 1e-5, f


@pytest.mark.parametrize("name", ["ref_col_c8_l3", "ref_refine_c16_l3"])
def test_sphere_collider_sdf_bit_exact(name):
    """OmniBoundarySolver3::updateCollider's SDF grid of the stock sphere (r = 0.1 at (0.5, 0.5, 0.45),
    through ShapeToImplicit3::signedDistanceLocal) computed by the oracle equals the grid the
    reference filled, at res 32 and 64; the cut-cell weights follow from it unchanged."""
    g = golden(name)
    c, lv = g["meta/case"].tolist()[:2]
    o = Oracle(c, lv)
    o.set("collider_sphere", [0.5, 0.5, 0.45, 0.1])
    assert_same("collider_sdf", g["collider_sdf"].ravel(), o.get("collider_sdf"))
    if "w_mac" in g:
        for k in ["w_mac", "w_tilt"]:
            assert_same(k, g[k], o.get(k))
    o.set("collider_sphere", [0.5, 0.5, 0.45, 0.0])
    assert o.get("collider_sdf").size == 0
