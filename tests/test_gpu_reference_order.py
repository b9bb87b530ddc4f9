"""The CUDA library in the reference's reduction order (astg_set_reduction_order ASTG_ORDER_REFERENCE)
against the reference solver's own output: Eigen's dot-product order, the sweep updates as a
multiply and a subtraction, and BLAS::sum's per-worker slices for the mean temperature make the
GPU step reproduce the reference bit for bit -- every field, the DOF maps, the matrix, the
pressure and the PCG iteration count, after every step.  The fixtures were made on an 8-core
host, so the reference's thread pool had 8 workers."""
import json
import os
import sys

import numpy as np
import pytest

from fixtures import FIELDS, GOLDEN, PROJ, STAGES, assert_same, case, golden, state

pytestmark = pytest.mark.gpu
DT = 0.01
WORKERS = 8


def solver(c, lv, **kw):
    import ast_solver

    s = ast_solver.OctreeSmoke3(c, lv, **kw)
    s.set_reduction_order("reference", WORKERS)
    return s


def getter(s):
    def get(f):
        if f == "pcg_iters":  # the fixtures' (iterations, converged) pair
            st = s.last_solve()
            return np.array([st.iterations, st.converged], dtype=np.int32)
        return s.get(f)

    return get


@pytest.mark.parametrize("name", ["ref_c8_l3", "ref_c16_l2"])
def test_free_running_steps_bit_identical_to_reference(name):
    g = golden(name)
    c, lv, steps = case(name)
    s = solver(c, lv)
    get = getter(s)
    for k in range(1, steps + 1):
        s.update(DT)
        st = state(g, f"step{k}/")
        for f in FIELDS + ["tilt_open"] + PROJ:
            assert_same(f"step{k}/{f}", st[f], get(f))
    s.close()


def test_every_stage_bit_identical_from_reference_inputs():
    """Each stage of step 1 from the reference's own input state, force and projection included."""
    g = golden("ref_c8_l3")
    c, lv, _ = case("ref_c8_l3")
    s = solver(c, lv)
    get = getter(s)
    prev = state(g, "init/")
    for i, st in enumerate(STAGES):
        for f in FIELDS:
            s.set(f, prev[f])
            s.set("t_" + f, prev["t_" + f])
        s.set("tilt_open", prev["tilt_open"])
        s.stage(i, DT)
        cur = state(g, f"stage1_{st}/")
        for f in FIELDS + ["tilt_open"]:
            assert_same(f"{st}/{f}", cur[f], s.get(f))
        if st == "project":
            proj = state(g, "step1/")
            for f in PROJ:
                assert_same(f"project/{f}", proj[f], get(f))
        prev = cur
    s.close()


@pytest.mark.parametrize("name", ["ref_c8_l3", "ref_c16_l2"])
def test_standalone_solve_reproduces_reference_iterates(name):
    """astg_solve (PCGSolver::solve) on the reference's assembled systems: the reference's solution
    and iteration count exactly."""
    g = golden(name)
    c, lv, steps = case(name)
    s = solver(c, lv)
    for k in range(1, steps + 1):
        st = state(g, f"step{k}/")
        x, stats = s.solve(st["A_rowptr"], st["A_col"], st["A_val"], st["b"])
        assert stats.converged == 1 and stats.iterations == int(st["pcg_iters"][0])
        assert_same(f"step{k}/p", st["p"], x)
    s.close()


@pytest.mark.parametrize("name", ["ref_c32_l3_hashes", "ref_c64_l3_hashes"])
def test_full_size_hash_identical_to_reference(name):
    """The reference's CPU-runnable configuration (32^3 coarsest x 3 levels, 128^3-equivalent) for its
    full 50 steps, and the benchmark size (64^3 x 3 levels, 256^3-equivalent) for 20 steps: after
    every step the sha256 of every state array, the tilt layout, the DOF maps, the pressure and the
    iteration count equal the reference's own."""
    sys.path.insert(0, GOLDEN)
    import make_golden

    rec = json.load(open(os.path.join(GOLDEN, name + ".json")))
    c, lv, steps = rec["case"]
    s = solver(c, lv)
    get = getter(s)
    for k in range(steps):
        s.update(rec["dt"])
        got = make_golden.step_hashes(get)
        bad = [f for f in got if got[f] != rec["steps"][k][f]]
        assert not bad, f"step {k + 1}: {bad}"
    s.close()


def test_library_order_is_the_default_and_can_be_restored():
    """The setting is per handle; the library order gives the oracle's library-order results."""
    from oracle.oracle import Oracle

    s = solver(8, 3)
    s.set_reduction_order("library")
    o = Oracle(8, 3, reduce_mode=1)
    for k in range(2):
        s.update(DT)
        o.step(DT)
        for f in ["density_oct", "heat_oct", "mac", "tilt_vel", "p"]:
            assert_same(f"step{k + 1}/{f}", o.get(f), s.get(f))
    s.close()


def test_bad_worker_counts_refused():
    import ast_solver

    s = ast_solver.OctreeSmoke3(8, 3)
    for w in (0, -1, 257):
        with pytest.raises(ast_solver.AstgError):
            s.set_reduction_order("reference", w)
    s.close()
