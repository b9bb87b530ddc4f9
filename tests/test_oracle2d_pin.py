"""The 2-D oracle (oracle/ast2d_oracle.cpp, the uniform ASTSolver<2> restatement) against the
reference's own runs (tests/golden/ref2d_*.npz, written by oracle/ref/ref_harness2d.cpp): every
frame, every stage snapshot and every projection system bit for bit, in the reference's own
arithmetic order (reduce mode 0).  Closed tilts hold stale pool memory in the reference, so their
vertex values are compared only where the tilt is open."""
import os

import numpy as np
import pytest

from oracle import oracle as orc

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
CASES = ["ref2d_stock_n32", "ref2d_stock_a48", "ref2d_eval_a48", "ref2d_eval_a32_substeps"]
STATE = ["density_cell", "heat_cell", "mac_x", "mac_y", "tilt_open", "pindex_cell", "pindex_vert"]
OPEN_ONLY = ["density_vert", "heat_vert", "tilt_vel"]
STAGES = ["source", "force", "project", "advect"]


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    return {k: z[k] for k in z.files}


def assert_state(o, R, prefix, what):
    is_open = R[prefix + "tilt_open"].astype(bool)
    for f in STATE:
        np.testing.assert_array_equal(o.get(f), R[prefix + f], err_msg=f"{what}: {f}")
    for f in OPEN_ONLY:
        np.testing.assert_array_equal(o.get(f)[is_open], R[prefix + f][is_open], err_msg=f"{what}: {f}")


@pytest.mark.parametrize("name", CASES)
def test_oracle2d_matches_reference_frames(name):
    R = load(name)
    nx, ny, frames, adaptive, stage_frames = (int(v) for v in R["meta/case"])
    dt = float(R["meta/dt"][0])
    o = orc.Oracle2D(nx, ny, adaptive=bool(adaptive))
    assert_state(o, R, "init/", "init")
    subs, start = [], 0
    for f in range(1, frames + 1):
        if f <= stage_frames:
            n = int(R["substeps"][f - 1])
            for j in range(n):
                sdt = float(R["sub_dt"][start + j])
                for st in STAGES:
                    o.stage(st, sdt)
                    p = f"f{f}/s{j}/{st}/"
                    assert_state(o, R, p, f"frame {f} sub-step {j} {st}")
                    if st == "project":
                        for k in ("A_rowptr", "A_col", "A_val", "b", "p"):
                            np.testing.assert_array_equal(o.get(k), R[p + k], err_msg=f"frame {f} {k}")
            subs.append(n)
        else:
            o.update(dt)
            subs.append(o.info()["substeps"])
        start += subs[-1]
        assert_state(o, R, f"f{f}/", f"frame {f}")
    assert subs == [int(v) for v in R["substeps"]]
    # the staged frames run their stages one by one, which records no sub-step length
    staged = int(R["substeps"][:stage_frames].sum())
    np.testing.assert_array_equal(o.get("sub_dt"), R["sub_dt"][staged:])


def test_substep_fixture_exercises_cfl_splitting():
    R = load("ref2d_eval_a32_substeps")
    assert int(R["substeps"].max()) >= 3 and len(set(R["sub_dt"].tolist())) >= 3


def test_stock_reference_correction_term_is_not_reproducible():
    """Frame 1 of the adaptive scene never opens a tilt before its advection, so the stock and the
    evaluated reference agree there; from frame 2 the stock build reads the destroyed temporary."""
    stock, ev = load("ref2d_stock_a48"), load("ref2d_eval_a48")
    for f in ("density_cell", "mac_x", "mac_y", "tilt_open"):
        np.testing.assert_array_equal(stock["f1/" + f], ev["f1/" + f])
    assert ev["f1/tilt_open"].sum() > 0


def test_oracle2d_reduce_modes_agree_closely():
    a, b = orc.Oracle2D(32, 64, adaptive=True, reduce_mode=0), orc.Oracle2D(32, 64, adaptive=True, reduce_mode=1)
    for _ in range(3):
        a.update(0.025)
        b.update(0.025)
    np.testing.assert_array_equal(a.get("tilt_open"), b.get("tilt_open"))
    np.testing.assert_allclose(a.get("density_cell"), b.get("density_cell"), rtol=0, atol=1e-6)


def test_oracle2d_rejects_bad_arguments():
    with pytest.raises(ValueError):
        orc.Oracle2D(1, 4)
    o = orc.Oracle2D(8, 8)
    with pytest.raises(KeyError):
        o.get("no_such_field")
    with pytest.raises(RuntimeError):
        o.set("p", np.zeros(3))


def test_substep_is_the_four_stages_in_order():
    """onUpdate = sphereSource2DSetup, addForce, project, advect: one sub-step equals the four
    stages run one by one, bit for bit."""
    a, b = orc.Oracle2D(24, 48, adaptive=True), orc.Oracle2D(24, 48, adaptive=True)
    for _ in range(3):
        a.stage("substep", 0.02)
        for st in STAGES:
            b.stage(st, 0.02)
    for f in STATE + OPEN_ONLY:
        np.testing.assert_array_equal(a.get(f), b.get(f), err_msg=f)


def test_non_adaptive_layout_never_opens():
    o = orc.Oracle2D(24, 48, adaptive=False)
    for _ in range(4):
        o.update(0.025)
    assert o.get("tilt_open").sum() == 0
    assert (o.get("pindex_vert") == -1).all()
    assert o.info()["unknowns"] == 24 * 48


def test_boundary_tilts_stay_closed_and_cells_keep_their_numbers():
    o = orc.Oracle2D(32, 64, adaptive=True)
    for _ in range(4):
        o.update(0.025)
    op = o.get("tilt_open")
    assert op.sum() > 0
    assert op[0, :].sum() == op[-1, :].sum() == op[:, 0].sum() == op[:, -1].sum() == 0
    np.testing.assert_array_equal(o.get("pindex_cell").ravel(), np.arange(32 * 64))
    # the tilts of the last projection's layout (the one before the last advection, as in the
    # reference, whose updateIndex runs in project) are numbered after the cells in vertex order
    pv = o.get("pindex_vert").ravel()
    numbered = pv[pv >= 0]
    assert len(numbered) > 0
    np.testing.assert_array_equal(numbered, np.arange(32 * 64, 32 * 64 + len(numbered)))


def test_worker_count_only_changes_the_dot_summation():
    """The reference's dot products depend on its worker count (one slice per taskflow worker):
    with another count the frames differ by round-off only, and the fixtures need the 8 workers of
    the host that made them."""
    R = load("ref2d_stock_n32")
    a = orc.Oracle2D(32, 64, adaptive=False, ref_workers=8)
    b = orc.Oracle2D(32, 64, adaptive=False, ref_workers=3)
    for _ in range(3):
        a.update(0.02500000037252903)
        b.update(0.02500000037252903)
    np.testing.assert_array_equal(a.get("mac_y"), R["f3/mac_y"])
    assert not np.array_equal(b.get("mac_y"), R["f3/mac_y"])
    np.testing.assert_allclose(b.get("mac_y"), R["f3/mac_y"], rtol=0, atol=1e-9)


@pytest.mark.parametrize("name", ["ref2d_eval_a192_hashes", "ref2d_stock_n192_hashes"])
def test_oracle2d_matches_reference_at_the_example_size(name):
    """The reference example's full size (192 x 384, dt 0.025f): six frames of the oracle hash to
    the reference's own arrays, every field of every frame, with the same CFL sub-steps -- adaptive
    with the correction term evaluated, and the stock reference without adaptivity."""
    import json
    import os as _os
    import sys as _sys

    _sys.path.insert(0, GOLDEN)
    import make_golden

    rec = json.load(open(_os.path.join(GOLDEN, name + ".json")))
    nx, ny, frames, adaptive = rec["case"]
    o = orc.Oracle2D(nx, ny, adaptive=bool(adaptive))
    subs = []
    for f in range(frames):
        o.update(rec["dt"])
        subs.append(o.info()["substeps"])
        is_open = o.get("tilt_open").astype(bool)
        got = make_golden.frame_hashes(o.get, is_open)
        assert got == rec["frames"][f], f"frame {f + 1}: " + ", ".join(
            k for k in got if got[k] != rec["frames"][f][k])
    assert subs == rec["substeps"]
    assert [float(v).hex() for v in o.get("sub_dt")] == rec["sub_dt"]
