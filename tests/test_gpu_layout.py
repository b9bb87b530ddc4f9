"""The octree layout (OctreeLayer3) and the tilt constraint (constrainOctreeTiltE3) built on the
device (astg_layout.cu) against the oracle's restatement, which is pinned to the reference's own
layouts: slot lists with the ghosts in discovery order, level sizes, T-joints, half tilts and the
tilts they close, the tilt-E state and the cut-cell weights -- for the benchmark scene at
64^3 x 3 and for source spheres that refine other parts of the domain."""
import numpy as np
import pytest

from fixtures import LAYOUT, assert_same

pytestmark = pytest.mark.gpu

CASES = [
    (64, 3, (0.5, 0.5, 0.12, 0.06)),
    (16, 3, (0.3, 0.6, 0.5, 0.1)),
    (8, 4, (0.1, 0.1, 0.1, 0.08)),
    (16, 3, (0.7, 0.25, 0.8, 0.15)),
    (12, 3, (0.5, 0.5, 0.5, 0.2)),
]


@pytest.mark.parametrize("c,lv,src", CASES)
def test_device_layout_matches_oracle(c, lv, src):
    import ast_solver
    from oracle.oracle import Oracle

    s = ast_solver.OctreeSmoke3(c, lv, source=src)
    o = Oracle(c, lv, source=src)
    for f in LAYOUT + ["tilt_flags", "tilt_e", "tilt_open"]:
        assert_same(f"{c}x{lv} {src} {f}", o.get(f), s.get(f))
    sizes = np.asarray(s.get("level_sizes")).reshape(-1, 3)
    assert sizes[:, 1].sum() > 0  # ghosts exist: the discovery order is exercised
    assert np.asarray(s.get("half_tilts")).size > 0 or c == 8
    s.close()
