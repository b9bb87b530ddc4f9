"""The C++ example (examples/octree_smoke.cpp) drives the step through the C ABI alone: it runs the
scene with the stock sphere obstacle and the reference's CFL sub-stepping, and its per-frame
results equal those of the same handle driven from Python, digit for digit."""
import subprocess

import pytest

pytestmark = pytest.mark.gpu


def test_cpp_example_matches_the_python_front_end():
    import build_lib

    import ast_solver

    exe = build_lib.build_example()
    out = subprocess.run([exe, "3", "16", "3", "--collider"], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    lines = [l.split() for l in out.stdout.strip().splitlines()]
    assert len(lines) == 3
    s = ast_solver.OctreeSmoke3(16, 3)
    s.set_collider_sphere((0.5, 0.5, 0.45), 0.1)
    s.setMaxCfl(2.0)
    s.useFixedTimeStep = False
    for f, l in enumerate(lines):
        s.update(0.01)
        assert int(l[3]) == s.last_substeps
        assert int(l[5]) == s.last_step.solve.iterations
        total = 0.0
        for v in s.get("density_oct").tolist():  # left to right, as the C++ loop adds
            total += v
        assert l[9] == "%.17g" % total
    s.close()
