"""Parity of the CUDA library (through the C ABI) with the reference and with the oracle.

* Topology, DOF numbering and the assembled matrix are compared bit for bit with the
  reference's own output (golden fixtures).
* Each stage, started from the reference's input state, reproduces the reference bit for bit,
  except where a floating-point reduction is involved (the mean temperature and the PCG dot
  products): the library reduces with a fixed tree, the reference with Eigen's SSE lanes, and
  the stage is then compared with a tolerance (1e-13 for the buoyancy, the PCG tolerance for
  the pressure).
* Free-running steps are bit-identical to the oracle run with the library's reduction tree.
"""
import numpy as np
import pytest

from fixtures import FIELDS, LAYOUT, STAGES, assert_same, case, golden, max_rel, state

pytestmark = pytest.mark.gpu
DT = 0.01


def solver(c, lv, **kw):
    import ast_solver

    return ast_solver.OctreeSmoke3(c, lv, **kw)


def oracle(c, lv, **kw):
    from oracle.oracle import Oracle

    return Oracle(c, lv, reduce_mode=1, **kw)


@pytest.mark.parametrize("name", ["ref_c8_l3", "ref_c16_l2"])
def test_topology_and_initial_state_match_reference(name):
    g = golden(name)
    c, lv, _ = case(name)
    s = solver(c, lv)
    for k in LAYOUT:
        assert_same(k, g[k], s.get(k))
    assert_same("dual_tables", g["dual_tables"], s.get("dual_tables"))
    init = state(g, "init/")
    for k in FIELDS + ["tilt_open"]:
        assert_same("init/" + k, init[k], s.get(k))
    s.close()


def test_stages_from_reference_inputs():
    g = golden("ref_c8_l3")
    c, lv, _ = case("ref_c8_l3")
    s = solver(c, lv)
    prev = state(g, "init/")
    for i, st in enumerate(STAGES):
        for f in FIELDS:
            s.set(f, prev[f])
            s.set("t_" + f, prev["t_" + f])
        s.set("tilt_open", prev["tilt_open"])
        s.stage(i, DT)
        cur = state(g, f"stage1_{st}/")
        if st == "project":
            proj = state(g, "step1/")
            for k in ["pindex_oct", "pindex_tilt", "A_rowptr", "A_col", "A_val", "b"]:
                assert_same("project/" + k, proj[k], s.get(k))
            it = s.last_solve().iterations
            assert abs(it - int(proj["pcg_iters"][0])) <= 1
            assert max_rel(proj["p"], s.get("p")) <= 1e-6
            for f in ["mac", "tilt_vel"]:
                assert max_rel(cur[f], s.get(f)) <= 1e-6, f
        elif st == "force":
            for f in FIELDS + ["tilt_open"]:
                assert_same(f"{st}/{f}", cur[f], s.get(f), rel=1e-13)
        else:
            for f in FIELDS + ["tilt_open"]:
                assert_same(f"{st}/{f}", cur[f], s.get(f))
        prev = cur
    s.close()


@pytest.mark.parametrize("c,lv,steps", [(8, 3, 4), (16, 2, 3)])
def test_free_running_bit_identical_to_oracle(c, lv, steps):
    s = solver(c, lv)
    o = oracle(c, lv)
    for k in range(steps):
        s.update(DT)
        o.step(DT)
        assert s.last_solve().iterations == int(o.get("pcg_iters")[0])
        for f in FIELDS + ["tilt_open"]:
            assert_same(f"step{k + 1}/{f}", o.get(f), s.get(f))
        for f in ["pindex_oct", "pindex_tilt", "A_rowptr", "A_col", "A_val", "b", "p"]:
            assert_same(f"step{k + 1}/{f}", o.get(f), s.get(f))
    s.close()


def test_benchmark_size_bit_identical_to_oracle():
    """128^3-equivalent octree (32^3 coarsest, 3 levels): two steps."""
    s = solver(32, 3)
    o = oracle(32, 3)
    for k in range(2):
        s.update(DT)
        o.step(DT)
        assert s.last_solve().iterations == int(o.get("pcg_iters")[0])
        for f in ["density_oct", "density_tilt", "heat_oct", "mac", "tilt_vel", "dual_oct", "tilt_open", "p"]:
            assert_same(f"step{k + 1}/{f}", o.get(f), s.get(f))
    s.close()


@pytest.mark.parametrize("name", ["ref_c8_l3", "ref_c16_l2"])
def test_standalone_solve_on_reference_systems(name):
    """astg_solve (PCGSolver::solve) on the reference's assembled systems: bit-identical to the
    oracle with the library's reduction tree, and within the solver tolerance of the reference."""
    g = golden(name)
    c, lv, steps = case(name)
    s = solver(c, lv)
    o = oracle(c, lv)
    for k in range(1, steps + 1):
        st = state(g, f"step{k}/")
        x, stats = s.solve(st["A_rowptr"], st["A_col"], st["A_val"], st["b"])
        xo, ito = o.solve(st["A_rowptr"], st["A_col"], st["A_val"], st["b"])
        assert stats.converged == 1 and stats.iterations == ito
        assert_same(f"step{k}/p vs oracle", xo, x)
        assert abs(stats.iterations - int(st["pcg_iters"][0])) <= 1
        assert max_rel(st["p"], x) <= 1e-6
        # the residual test of the reference: |b - A x|_inf <= tol |b|_inf
        rp, col, val = st["A_rowptr"], st["A_col"], st["A_val"]
        ax = np.zeros_like(x)
        for i in range(len(x)):
            ax[i] = np.dot(val[rp[i]:rp[i + 1]], x[col[rp[i]:rp[i + 1]]])
        assert np.abs(st["b"] - ax).max() <= 1e-6 * np.abs(st["b"]).max() * 1.0000001
    s.close()


@pytest.mark.parametrize("mode", ["async", "dsmem", "cluster", "syncfree"])
def test_every_sweep_form_bit_identical_to_oracle(mode, monkeypatch):
    """Each form of the MIC(0) triangular sweeps (ASTG_SWEEP) gives the oracle's results bit for
    bit, and the form asked for is the one that ran (astg_size 7)."""
    monkeypatch.setenv("ASTG_SWEEP", mode)
    s = solver(16, 3)
    o = oracle(16, 3)
    for k in range(2):
        s.update(DT)
        o.step(DT)
        assert s.last_solve().iterations == int(o.get("pcg_iters")[0])
        for f in FIELDS + ["tilt_open", "p"]:
            assert_same(f"{mode}/step{k + 1}/{f}", o.get(f), s.get(f))
    form = s.size(7)
    if mode == "async":
        assert 200 < form < 300
    elif mode == "dsmem":
        assert 100 < form < 200
    elif mode == "cluster":
        assert 1 < form <= 16
    else:
        assert form == 0
    s.close()


def test_full_benchmark_size_steps_bit_identical_to_oracle():
    """256^3-equivalent octree (64^3 coarsest, 3 levels), the size the benchmark runs: ten steps,
    every field, the pressure and the iteration count after each (200 steps were checked the same
    way once; ten keep the suite short)."""
    from oracle.oracle import Oracle

    s = solver(64, 3)
    o = Oracle(64, 3, reduce_mode=1, openmp=True)
    for k in range(1, 11):
        s.update(DT)
        o.step(DT)
        assert s.size(7) > 200  # the barrier-free fused preconditioner ran
        assert s.last_solve().iterations == int(o.get("pcg_iters")[0]), f"step {k}"
        for f in ["density_oct", "density_tilt", "heat_oct", "mac", "tilt_vel", "dual_oct", "tilt_open", "p"]:
            assert_same(f"step{k}/{f}", o.get(f), s.get(f))
    s.close()


def test_config0_fifty_steps_bit_identical_to_oracle():
    """The reference's CPU-runnable configuration (32^3 coarsest, 3 levels = 128^3-equivalent) for
    its full 50 steps: state, DOF map, pressure and PCG iterations identical after every step."""
    from oracle.oracle import Oracle

    s = solver(32, 3)
    o = Oracle(32, 3, reduce_mode=1, openmp=True)
    for k in range(50):
        s.update(DT)
        o.step(DT)
        assert s.last_solve().iterations == int(o.get("pcg_iters")[0]), k
        for f in ["density_oct", "density_tilt", "heat_oct", "heat_tilt", "mac", "tilt_vel", "tilt_open", "p"]:
            assert_same(f"step{k + 1}/{f}", o.get(f), s.get(f))
    s.close()


def test_mixed_form_tracks_fp64_oracle():
    """The mixed-precision form against the FP64 oracle over 20 steps (16^3 coarsest, 3 levels):
    per step the density and the pressure within 1e-5 relative (L2), and the solve's true FP64
    residual at most 1e-6 |b|_inf."""
    import numpy as np

    s = solver(16, 3, precision="mixed")
    o = oracle(16, 3)
    worst_d = worst_p = 0.0
    for k in range(20):
        s.update(DT)
        o.step(DT)
        st = s.last_step.solve
        assert st.converged == 1 and st.outer >= 1
        assert st.residual <= st.tolerance
        a, b = o.get("density_oct"), s.get("density_oct")
        worst_d = max(worst_d, np.linalg.norm(b - a) / np.linalg.norm(a))
        pa, pb = o.get("p"), s.get("p")
        assert len(pa) == len(pb), k  # same DOF map: no tilt decision differs
        worst_p = max(worst_p, np.linalg.norm(pb - pa) / np.linalg.norm(pa))
    print(f"mixed vs FP64 over 20 steps: density {worst_d:.2e}, pressure {worst_p:.2e}")
    assert worst_d <= 1e-5 and worst_p <= 1e-5
    s.close()
