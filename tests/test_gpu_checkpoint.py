"""Checkpoints in the reference's binary formats (src/viewer/grid_dump.cpp:280-615) through the C ABI:
astg_restart from the reference's own dumps restores exactly the state the reference's restart
restores, the step after it matches the reference's (and the oracle's, bit for bit), and
astg_save_checkpoint writes files the reference reads: the scalar and velocity dumps byte for byte,
the tilt-E and layout dumps field for field (the reference leaves struct padding uninitialised and
writes its layout map in hash-table order)."""
import os
import struct

import numpy as np
import pytest

from fixtures import FIELDS, assert_same, golden, max_rel, state

pytestmark = pytest.mark.gpu
FILES = ["layout.bin", "tilt.bin", "density.bin", "heat.bin", "velocity.bin"]
DT = 0.01


def write_files(g, d):
    os.makedirs(d, exist_ok=True)
    for f in FILES:
        g["file/" + f].tofile(os.path.join(d, f))


def parse_layout(raw):
    b = bytes(raw)
    at = 0

    def take(fmt):
        nonlocal at
        v = struct.unpack_from(fmt, b, at)
        at += struct.calcsize(fmt)
        return v

    (levels,) = take("<i")
    out = []
    for _ in range(levels):
        (m,) = take("<i")
        entries = {}
        for _ in range(m):
            (c,) = take("<q")
            index, x, y, z, _pad, flag = take("<QHHHHI")
            take("<4x")
            entries[c] = (index, x, y, z, flag & 7)
        (g,) = take("<i")
        ghosts = take(f"<{g}q")
        (n,) = take("<i")
        nodes = take(f"<{n}q")
        out.append((entries, ghosts, nodes))
    (h,) = take("<i")
    half = take(f"<{h}q")
    assert at == len(b)
    return out, half


def parse_tilt(raw):
    b = bytes(raw)
    (levels,) = struct.unpack_from("<i", b, 0)
    at, out = 4, []
    for _ in range(levels):
        (m,) = struct.unpack_from("<i", b, at)
        at += 4
        for _ in range(m):
            e, = struct.unpack_from("<d", b, at)
            flags = tuple(bool(x) for x in b[at + 8:at + 14])
            d, = struct.unpack_from("<i", b, at + 16)
            out.append((e, flags, d))
            at += 24
    assert at == len(b)
    return out


def parse_levels(b, at, width):
    """One per-level array of the dumps (level count, then per level a count and the values)."""
    (levels,) = struct.unpack_from("<i", b, at)
    at += 4
    parts = []
    for _ in range(levels):
        (m,) = struct.unpack_from("<i", b, at)
        at += 4
        parts.append(np.frombuffer(b, dtype="<f8", count=m * width, offset=at))
        at += 8 * m * width
    return np.concatenate(parts), at


def parse_velocity(raw):
    b = bytes(raw)
    at, axes = 0, []
    for _ in range(3):
        u, at = parse_levels(b, at, 1)
        axes.append(u)
    tv, at = parse_levels(b, at, 8)
    assert at == len(b)
    return np.stack(axes), tv.reshape(-1, 8)


def restarted(tmp_path, name="ref_ckpt_c8_l3"):
    import ast_solver

    g = golden(name)
    c, lv, _ = g["meta/case"].tolist()
    write_files(g, str(tmp_path))
    s = ast_solver.OctreeSmoke3(c, lv)
    s.restart(str(tmp_path))
    return g, s


def test_restart_restores_the_reference_state(tmp_path):
    g, s = restarted(tmp_path)
    ref = state(g, "restart/")
    for k in FIELDS + ["t_" + k for k in FIELDS] + ["tilt_open"]:
        assert_same("restart/" + k, ref[k], s.get(k))
    s.close()


def test_step_after_restart(tmp_path):
    from oracle.oracle import Oracle

    g, s = restarted(tmp_path)
    c, lv, _ = g["meta/case"].tolist()
    o = Oracle(c, lv, reduce_mode=1)
    for k in FIELDS + ["t_" + k for k in FIELDS] + ["tilt_open"]:
        o.set(k, s.get(k))
    s.update(DT)
    o.step(DT)
    for k in FIELDS + ["tilt_open", "p"]:
        assert_same("oracle/" + k, o.get(k), s.get(k))
    ref = state(g, "step1/")
    for k in ["pindex_oct", "pindex_tilt", "A_rowptr", "A_col", "A_val"]:
        assert_same("reference/" + k, ref[k], s.get(k))
    # b carries the buoyancy, whose mean temperature the library sums with its fixed tree (within
    # 1e-13 of the reference's summation order)
    assert max_rel(ref["b"], s.get("b")) <= 1e-12
    assert abs(s.last_solve().iterations - int(ref["pcg_iters"][0])) <= 1
    for k in ["p", "mac", "tilt_vel", "density_oct", "heat_oct"]:
        assert max_rel(ref[k], s.get(k)) <= 1e-6, k
    s.close()
    o.close()


def test_checkpoint_written_back_is_the_reference_dump(tmp_path):
    g, s = restarted(tmp_path / "in")
    out = tmp_path / "out" / "nested"
    s.save_checkpoint(str(out))
    for f in ["density.bin", "heat.bin"]:
        got = np.fromfile(str(out / f), dtype=np.uint8)
        assert np.array_equal(got, g["file/" + f]), f
    # restart recomputes the velocity ghosts (as the reference's does), so the velocity written back
    # is the reference's restored velocity
    mac, tv = parse_velocity(np.fromfile(str(out / "velocity.bin"), dtype=np.uint8))
    ref = state(g, "restart/")
    assert_same("velocity mac", ref["mac"], mac)
    assert_same("velocity tilt", ref["tilt_vel"], tv)
    assert parse_tilt(np.fromfile(str(out / "tilt.bin"), dtype=np.uint8)) == parse_tilt(g["file/tilt.bin"])
    assert parse_layout(np.fromfile(str(out / "layout.bin"), dtype=np.uint8)) == parse_layout(g["file/layout.bin"])
    s.close()


def test_bad_checkpoints_are_refused_and_leave_the_state(tmp_path):
    import ast_solver

    g = golden("ref_ckpt_c8_l3")
    write_files(g, str(tmp_path))
    s = ast_solver.OctreeSmoke3(8, 3)
    before = s.get("density_oct")
    raw = g["file/heat.bin"]
    raw[: len(raw) // 2].tofile(str(tmp_path / "heat.bin"))  # truncated
    with pytest.raises(ast_solver.AstgError) as e:
        s.restart(str(tmp_path))
    assert e.value.status == ast_solver.ASTG_BAD_ARG and "truncated" in str(e.value)
    assert np.array_equal(s.get("density_oct"), before)
    s.close()
    other = ast_solver.OctreeSmoke3(8, 2)  # another octree
    with pytest.raises(ast_solver.AstgError) as e:
        other.restart(str(tmp_path))
    assert e.value.status == ast_solver.ASTG_LAYOUT_ERROR
    other.close()


def test_round_trip_at_benchmark_size(tmp_path):
    """64^3 x 3 levels after 3 steps: save, restart a second handle; everything the checkpoint holds
    comes back (velocity ghosts are recomputed by the restart, so faces are compared off ghosts)."""
    import ast_solver

    a = ast_solver.OctreeSmoke3(64, 3)
    for _ in range(3):
        a.update(DT)
    a.save_checkpoint(str(tmp_path))
    b = ast_solver.OctreeSmoke3(64, 3)
    b.restart(str(tmp_path))
    for k in ["density_oct", "density_tilt", "heat_oct", "heat_tilt", "tilt_e", "tilt_flags"]:
        assert_same(k, a.get(k), b.get(k))
    cells = (a.get("slot_coords")[:, 3] & 2) == 0
    assert_same("mac", a.get("mac")[:, cells], b.get("mac")[:, cells])
    assert_same("tilt_vel", a.get("tilt_vel")[cells], b.get("tilt_vel")[cells])
    a.close()
    b.close()
