"""Solver::update's adaptive branch on the GPU (astg_update: useFixedTimeStep = false, CFL sub-steps
with numberOfSubTimeSteps = max(1, ceil(cfl / maxCfl)) recomputed before every sub-step,
src/solver.cpp:21-41, src/octree_omnigrid_solver3.cpp:1060-1122) against the reference's own frames
(fixture ref_cfl_c8_l3: six frames of dt 0.25 with setMaxCfl(2)) and against the oracle."""
import numpy as np
import pytest

from fixtures import FIELDS, assert_same, case, golden, state

pytestmark = pytest.mark.gpu
CHECK = FIELDS + ["tilt_open", "pindex_oct", "pindex_tilt", "p"]


def adaptive_solver(c, lv, max_cfl, order):
    import ast_solver

    s = ast_solver.OctreeSmoke3(c, lv)
    s.useFixedTimeStep = False
    s.setMaxCfl(max_cfl)
    s.set_reduction_order(order, 8)
    return s


def test_frames_bit_identical_to_reference():
    """In the reference's reduction order: the same number of sub-steps in every frame and every
    field, the DOF maps and the last sub-step's pressure identical after each frame."""
    g = golden("ref_cfl_c8_l3")
    c, lv, frames = case("ref_cfl_c8_l3")
    dt, max_cfl = g["meta/adaptive"].tolist()
    s = adaptive_solver(c, lv, max_cfl, "reference")
    for k in range(1, frames + 1):
        st = state(g, f"frame{k}/")
        # the first sub-step count the reference computed from this frame's starting velocity
        assert s.numberOfSubTimeSteps(dt) == int(st["substeps"][0]), f"frame {k}"
        s.update(dt)
        assert s.last_substeps == len(st["substeps"]), f"frame {k}"
        assert s.last_solve().iterations == int(st["pcg_iters"][0])
        for f in CHECK:
            assert_same(f"frame{k}/{f}", st[f], s.get(f))
    s.close()


def test_library_order_matches_oracle_substeps():
    """In the library's order against the oracle's library-order restatement of the same loop."""
    from oracle.oracle import Oracle

    s = adaptive_solver(8, 3, 2.0, "library")
    o = Oracle(8, 3, reduce_mode=1)
    total = 0
    for k in range(5):
        ks = o.update(0.25, 2.0)
        s.update(0.25)
        assert s.last_substeps == len(ks), k
        total += len(ks)
        for f in ["density_oct", "heat_oct", "mac", "tilt_vel", "p"]:
            assert_same(f"frame{k + 1}/{f}", o.get(f), s.get(f))
    assert total > 5
    s.close()


def test_fixed_step_is_one_substep_and_cfl_truncates():
    import ast_solver

    s = ast_solver.OctreeSmoke3(8, 3)
    s.update(0.01)
    assert s.last_substeps == 1
    mac = s.get("mac")
    vmax = max(0.0, float(mac.max()))
    res = s.size(2)
    assert s.cfl(0.25) == int(0.25 * vmax / (1.0 / res))
    assert s.numberOfSubTimeSteps(0.0) == 1
    s.close()
