"""astg_solve_batch: several right-hand sides of one matrix solved side by side, each lane on its
own preconditioner cluster and stream.  Every solution must be the one astg_solve returns for the
same right-hand side, bit for bit, with the same iteration count (FP64 and mixed forms), and the
concurrent lanes must not disturb each other."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
DT = 0.01


def system(c=32, lv=3, steps=3, nrhs=6):
    import ast_solver

    s = ast_solver.OctreeSmoke3(c, lv)
    for _ in range(steps):
        s.update(DT)
    rp, col, val, b = s.get("A_rowptr"), s.get("A_col"), s.get("A_val"), s.get("b")
    rng = np.random.default_rng(7)
    B = np.stack([b] + [b + 1e-2 * np.abs(b).max() * rng.standard_normal(len(b)) for _ in range(nrhs - 1)])
    return s, (rp, col, val), B


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_equals_one_by_one(precision):
    s, (rp, col, val), B = system()
    X, stats, wall_ms, lanes = s.solve_batch(rp, col, val, B, precision=precision)
    assert lanes >= 2, "the preconditioner cluster should leave room for more than one solve"
    assert wall_ms > 0
    for i, b in enumerate(B):
        x, st = s.solve(rp, col, val, b, precision=precision)
        assert stats[i].iterations == st.iterations and stats[i].converged == 1
        assert np.array_equal(X[i], x), f"rhs {i}: max diff {np.abs(X[i] - x).max()}"
    s.close()


def test_batch_at_the_benchmark_size_converges_and_matches_the_first_solve():
    s, (rp, col, val), B = system(64, 3, 2, 9)
    X, stats, _, lanes = s.solve_batch(rp, col, val, B)
    assert all(st.converged == 1 for st in stats)
    x0, st0 = s.solve(rp, col, val, B[0])
    assert np.array_equal(X[0], x0) and stats[0].iterations == st0.iterations
    n = len(rp) - 1
    for i in range(len(B)):  # the FP64 stopping test of each solve holds
        r = B[i].copy()
        rows = np.repeat(np.arange(n), np.diff(rp))
        np.subtract.at(r, rows, val * X[i][col])
        assert np.abs(r).max() <= 1e-6 * np.abs(B[i]).max() * 1.0001
    s.close()
