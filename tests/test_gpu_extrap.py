"""FMM extrapolation on the GPU (astg_extrapolate) against the reference's own
FmmLevelSetSolver3::extrapolate (golden fixtures made by tests/golden/make_golden.py) and against
the oracle, which reproduces the reference's heap march bit for bit.

The GPU orders the march by parallel passes (see ast-grid_gb300/csrc/astg_extrap.cu); it assigns
exactly the reference's set of nodes.  On the reference's fixtures every value is bit-identical.
At the benchmark size the check against the oracle allows 1 % of the assigned values to differ by
at most 1e-3 of the field's maximum: nodes pushed late in a chain are ordered by their keys, which
the reference's heap does not guarantee (observed: no difference)."""
import numpy as np
import pytest

from fixtures import FIELDS, golden, state

pytestmark = pytest.mark.gpu


def compare(ref_oct, ref_til, got_oct, got_til, before_oct, before_til):
    ref = np.concatenate([ref_oct, ref_til])
    got = np.concatenate([got_oct, got_til])
    before = np.concatenate([before_oct, before_til])
    touched = (ref != before) | (got != before)
    same = (ref == got) | (np.isnan(ref) & np.isnan(got))
    bad = touched & ~same
    scale = max(np.abs(before[~np.isnan(before)]).max(), 1e-300)
    dev = np.abs(ref[bad] - got[bad]).max() / scale if bad.any() else 0.0
    return int(touched.sum()), int(bad.sum()), float(dev)


@pytest.mark.parametrize("name", ["ref_extrap_c8_l3", "ref_extrap_c16_l2"])
def test_extrapolation_matches_reference(name):
    import ast_solver

    g = golden(name)
    c, lv, _ = g["meta/case"].tolist()
    cx, cy, cz, r, maxf, off = g["meta/extrap"].tolist()
    s = ast_solver.OctreeSmoke3(c, lv)
    before = state(g, "before/")
    for k in FIELDS:
        s.set(k, before[k])
    st = s.extrapolate("density", g["sdf"], off, maxf)
    touched, bad, dev = compare(g["after/density_oct"], g["after/density_tilt"], s.get("density_oct"),
                                s.get("density_tilt"), before["density_oct"], before["density_tilt"])
    print(f"{name}: assigned {st.assigned} in {st.passes} passes, changed {touched}, differing {bad}, max dev {dev:.3e}")
    assert st.assigned > 100 and st.passes > 1
    assert bad == 0
    s.close()


def test_extrapolation_matches_oracle_at_benchmark_size():
    """64^3 coarsest x 3 levels after two steps, a sphere around the source: same inputs for the
    GPU and the oracle (the oracle's state is set from the GPU's); every assigned value identical."""
    import ast_solver
    from oracle.oracle import Oracle

    c, lv = 64, 3
    s = ast_solver.OctreeSmoke3(c, lv)
    for _ in range(2):
        s.update(0.01)
    res = c << (lv - 1)
    x = (np.arange(res) + 0.5) / res
    zz, yy, xx = np.meshgrid(x, x, x, indexing="ij")
    sdf = np.sqrt((xx - 0.503) ** 2 + (yy - 0.487) ** 2 + (zz - 0.141) ** 2) - 0.083
    o = Oracle(c, lv, openmp=True)
    for k in FIELDS:
        o.set(k, s.get(k))
    before_o, before_t = s.get("density_oct"), s.get("density_tilt")
    n = o.extrapolate("density", sdf, 0.0, 6.0)
    st = s.extrapolate("density", sdf, 0.0, 6.0)
    touched, bad, dev = compare(o.get("density_oct"), o.get("density_tilt"), s.get("density_oct"),
                                s.get("density_tilt"), before_o, before_t)
    print(f"benchmark size: oracle assigned {n}, GPU {st.assigned} in {st.passes} passes ({st.ms:.2f} ms), "
          f"changed {touched}, differing {bad}, max dev {dev:.3e}")
    assert st.assigned == n
    assert bad == 0 and dev == 0.0
    s.close()
    o.close()
