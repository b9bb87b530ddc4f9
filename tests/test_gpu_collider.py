"""The collider branch on the GPU (astg_set "collider_sdf"): the stock scene's obstacle, a sphere
r = 0.1 at (0.5, 0.5, 0.45) through OmniBoundarySolver3::updateCollider, in the benchmark scene
(fixtures ref_col_c8_l3 / ref_col_c16_l2 made by the reference itself with its collider SDF grid).
Cut-cell weights, wipeBoundary, the inside-solid constrainVelocity, the DOF threshold and the
back-trace clamp against the reference and the oracle."""
import numpy as np
import pytest

from fixtures import FIELDS, PROJ, STAGES, assert_same, case, golden, max_rel, state

pytestmark = pytest.mark.gpu
DT = 0.01


def solver(name, order="reference"):
    import ast_solver

    g = golden(name)
    c, lv, _ = case(name)
    s = ast_solver.OctreeSmoke3(c, lv)
    s.set("collider_sdf", g["collider_sdf"])
    s.set_reduction_order(order, 8)
    return s, g


def get_all(s, f):
    if f == "pcg_iters":
        st = s.last_solve()
        return np.array([st.iterations, st.converged], dtype=np.int32)
    return s.get(f)


def test_weights_and_steps_bit_identical_to_reference():
    s, g = solver("ref_col_c8_l3")
    _, _, steps = case("ref_col_c8_l3")
    for k in ["w_mac", "w_tilt"]:
        assert_same(k, g[k], s.get(k))
    for k in range(1, steps + 1):
        s.update(DT)
        st = state(g, f"step{k}/")
        for f in FIELDS + ["tilt_open"] + PROJ:
            assert_same(f"step{k}/{f}", st[f], get_all(s, f))
    s.close()


def test_every_stage_bit_identical_from_reference_inputs():
    s, g = solver("ref_col_c8_l3")
    prev = state(g, "init/")
    for i, stg in enumerate(STAGES):
        for f in FIELDS:
            s.set(f, prev[f])
            s.set("t_" + f, prev["t_" + f])
        s.set("tilt_open", prev["tilt_open"])
        s.stage(i, DT)
        cur = state(g, f"stage1_{stg}/")
        for f in FIELDS + ["tilt_open"]:
            assert_same(f"{stg}/{f}", cur[f], s.get(f))
        prev = cur
    s.close()


def test_library_order_bit_identical_to_oracle():
    """Both cases, the one whose solid faces the reference's workers race on included: the GPU and
    the oracle share the defined order of the inside-solid projection."""
    from oracle.oracle import Oracle

    for name in ["ref_col_c8_l3", "ref_col_c16_l2"]:
        s, g = solver(name, "library")
        c, lv, steps = case(name)
        o = Oracle(c, lv, reduce_mode=1)
        o.set("collider_sdf", g["collider_sdf"])
        for k in range(steps):
            s.update(DT)
            o.step(DT)
            assert s.last_solve().iterations == int(o.get("pcg_iters")[0])
            for f in FIELDS + ["tilt_open", "pindex_oct", "pindex_tilt", "p"]:
                assert_same(f"{name}/step{k + 1}/{f}", o.get(f), s.get(f))
        s.close()


def test_racy_case_close_to_reference():
    s, g = solver("ref_col_c16_l2")
    _, _, steps = case("ref_col_c16_l2")
    for k in ["w_mac", "w_tilt"]:
        assert_same(k, g[k], s.get(k))
    for k in range(1, steps + 1):
        s.update(DT)
        st = state(g, f"step{k}/")
        for f in ["tilt_open", "pindex_oct", "pindex_tilt", "A_rowptr", "A_col"]:
            assert_same(f"step{k}/{f}", st[f], s.get(f))
        assert max_rel(st["mac"], s.get("mac")) <= 1e-3
        assert max_rel(st["p"], s.get("p")) <= 3e-3
        assert max_rel(st["density_oct"], s.get("density_oct")) <= 1e-5
    s.close()


def test_removing_the_collider_restores_the_free_domain():
    import ast_solver

    s, g = solver("ref_col_c8_l3", "library")
    s.set("collider_sdf", np.zeros(0))
    free = ast_solver.OctreeSmoke3(8, 3)
    assert_same("w_mac", free.get("w_mac"), s.get("w_mac"))
    assert_same("w_tilt", free.get("w_tilt"), s.get("w_tilt"))
    s.update(DT)
    free.update(DT)
    for f in ["density_oct", "mac", "p"]:
        assert_same(f, free.get(f), s.get(f))
    with pytest.raises(ast_solver.AstgError):
        s.set("collider_sdf", np.zeros(7))
    s.close()
    free.close()


def test_sphere_collider_on_device_bit_identical_to_reference():
    """astg_set_collider_sphere: the stock obstacle's SDF grid computed on the device equals the
    reference's grid; the weights and four steps then match the reference bit for bit as with the
    grid passed in.  radius 0 removes the collider."""
    import ast_solver

    name = "ref_col_c8_l3"
    g = golden(name)
    c, lv, steps = case(name)
    s = ast_solver.OctreeSmoke3(c, lv)
    s.set_reduction_order("reference", 8)
    s.set_collider_sphere((0.5, 0.5, 0.45), 0.1)
    assert_same("collider_sdf", g["collider_sdf"].ravel(), s.get("collider_sdf"))
    for k in ["w_mac", "w_tilt"]:
        assert_same(k, g[k], s.get(k))
    for k in range(1, steps + 1):
        s.update(DT)
        st = state(g, f"step{k}/")
        for f in FIELDS + ["tilt_open", "p"]:
            assert_same(f"step{k}/{f}", st[f], s.get(f))
    s.set_collider_sphere((0.5, 0.5, 0.45), 0.0)
    assert s.get("collider_sdf").size == 0
    free = ast_solver.OctreeSmoke3(c, lv)
    assert_same("w_mac", free.get("w_mac"), s.get("w_mac"))
    s.close()
    free.close()


def test_sphere_collider_sdf_at_full_resolution():
    """At 64^3 coarsest x 3 levels (res 256) the device grid equals the oracle's restatement, which
    is pinned to the reference's grid at res 32 and 64."""
    import ast_solver
    from oracle.oracle import Oracle

    s = ast_solver.OctreeSmoke3(64, 3)
    s.set_collider_sphere((0.5, 0.5, 0.45), 0.1)
    o = Oracle(64, 3)
    o.set("collider_sphere", [0.5, 0.5, 0.45, 0.1])
    assert_same("collider_sdf", o.get("collider_sdf"), s.get("collider_sdf"))
    s.close()


def test_refine_split_map_on_the_device_equals_the_reference():
    """astg_refine_split_map_device on CUDA tensors gives the reference's refined map (fixture made by
    refineSplitMapByObstacleSdf itself), pass by pass, and refuses host memory."""
    import torch

    import ast_solver
    from oracle.oracle import Oracle

    g = golden("ref_refine_c16_l3")
    c, lv, _ = g["meta/case"].tolist()
    split = torch.tensor(np.ascontiguousarray(Oracle(c, lv).get("split_map"), dtype=np.int32).ravel(), device="cuda")
    sdf = torch.tensor(np.ascontiguousarray(g["collider_sdf"], dtype=np.float64).ravel(), device="cuda")
    for level, lo, hi in g["meta/refine"].tolist():
        ast_solver.refine_split_map_tensor(split, int(level), sdf, (lo, hi))
    torch.cuda.synchronize()
    assert np.array_equal(split.cpu().numpy(), g["split_map"].ravel())
    with pytest.raises(ValueError):
        ast_solver.refine_split_map_tensor(split.cpu(), 1, sdf, (0.0, 1.0))
