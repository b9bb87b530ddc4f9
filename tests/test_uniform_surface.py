"""CPU checks of the reference module's uniform-grid surface (python_bindings/ast_solver.cc:14-80)
as this package provides it: grid, node and layout classes, the benchmark timer functions, and the
refusals (ASTSolver3; ASTSolver2 without a device)."""
import io

import numpy as np
import pytest

import ast_solver


def test_grid_and_node_classes():
    assert ast_solver.ASTGrid2().dimension() == 2
    assert ast_solver.ASTGrid3().dimension() == 3
    assert ast_solver.TiltNode2().open() is False and ast_solver.TiltNode3(True).open() is True
    ast_solver.CellNode2()
    ast_solver.CellNode3()


def test_layout_properties():
    lay = ast_solver.ASTGridLayout2([192, 384], 1.0 / 192)
    assert lay.resolution.tolist() == [192, 384] and lay.dx == 1.0 / 192
    lay3 = ast_solver.ASTGridLayout3((8, 8, 16), 0.125)
    assert lay3.resolution.tolist() == [8, 8, 16] and lay3.dx == 0.125
    with pytest.raises(ValueError):
        ast_solver.ASTGridLayout2([4, 4, 4], 0.1)


def test_solver3_refuses_with_a_reason():
    s = ast_solver.ASTSolver3(resolution=[8, 8, 8], dx=0.125, adaptive_dofs=True, name="x")
    with pytest.raises(NotImplementedError, match="OctreeSmoke3"):
        s.update(0.01)


def test_solver2_keeps_the_bound_arguments():
    s = ast_solver.ASTSolver2(resolution=[48, 96], dx=1.0 / 48, adaptive_dofs=False, name="toy")
    assert s.resolution == (48, 96) and s.dx == 1.0 / 48 and s.adaptive_dofs is False and s.name == "toy"


def test_benchmark_timer_sections_and_report(monkeypatch):
    t = ast_solver._BenchmarkTimer()
    clock = iter(np.arange(0.0, 100.0, 1.0))
    monkeypatch.setattr(ast_solver.time, "perf_counter", lambda: float(next(clock)))
    t.start_section("project")
    t.start_section("pcg solve")
    t.stop_section("pcg solve")
    t.start_timer("assemble")
    t.stop_timer("assemble")
    t.stop_section("project")
    t.start_section("project")
    t.stop_section("project")
    out = io.StringIO()
    t.report(out)
    lines = out.getvalue().splitlines()
    assert lines[0].split("\t")[0] == "project" and lines[0].split("\t")[2] == "2"
    names = [ln.split("\t")[0] for ln in lines]
    assert "    assemble" in names and "    pcg solve" in names and names[-1] == "Full time"


def test_benchmark_module_functions():
    ast_solver.benchmark_reset()
    ast_solver.benchmark_start_timer_section("a")
    ast_solver.benchmark_start_timer("t")
    ast_solver.benchmark_stop_timer("t")
    ast_solver.benchmark_stop_timer_section("a")
    ast_solver.benchmark_report(include_messages=True)
    ast_solver.benchmark_reset()


def test_solver2_without_a_device_fails_loudly():
    """No CUDA device (this CPU host): ASTSolver2 raises instead of falling back to anything."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    try:
        ast_solver.lib()
    except OSError:
        pytest.skip("the CUDA library is not built here")
    s = ast_solver.ASTSolver2(resolution=[16, 32], dx=1.0 / 16, adaptive_dofs=True, name="cpu")
    with pytest.raises(ast_solver.AstgError) as e:
        s.initialize()
    assert e.value.status == ast_solver.ASTG_NO_DEVICE
