"""Regenerate the golden fixtures from the reference solver itself.

Builds the reference's own sources with oracle/ref/Makefile (reference checkout at $ASTG_REF,
default: a directory named "reference" beside this repository), runs the fixture harness oracle/ref/ref_harness.cpp on small cases
of the benchmark scene, and stores the dumps as compressed .npz files next to this script.

    python tests/golden/make_golden.py

Fixture keys (all arrays in the reference's slot order, see oracle/smoke_oracle.cpp):
  layout: level_sizes, slot_coords, split_map, half_tilts, t_joints, closed_by_half_tilt,
          w_mac, w_tilt, dual_tables, init/<field>, init/t_<field>
  per step k (1-based) final state: step<k>/<field>, step<k>/t_<field>, and the projection of
          that step: step<k>/A_rowptr, A_col, A_val, b, p, pcg_iters, pindex_oct, pindex_tilt, ambT
  stage snapshots of step 1 (when recorded): stage1_<name>/<field>, t_<field>

Extrapolation fixtures (ref_extrap_*.npz): the state after the steps (before/<field>), the sphere
signed distance grid the harness built (sdf, res^3), the density after the reference's
FmmLevelSetSolver3::extrapolate (after/density_oct, after/density_tilt), meta/case and
meta/extrap = [cx, cy, cz, r, max_distance_factor, offset].

    python tests/golden/make_golden.py --extrap-only

Checkpoint fixtures (ref_ckpt_*.npz): the reference's own dump files after `steps` steps
(file/layout.bin, file/tilt.bin, file/density.bin, file/heat.bin, file/velocity.bin, as raw bytes),
the state it restores from them with OctreeOmniGridSolver3::restart in a fresh solver
(restart/<field>, restart/t_<field>) and its first step after that restart (step1/<field> and the
projection, as in the step fixtures).

    python tests/golden/make_golden.py --ckpt-only

2-D fixtures (ref2d_*.npz): the uniform 2-D solver ASTSolver<2> run by oracle/ref/ref_harness2d.cpp
with Solver::update's CFL sub-stepping, in the reference's storage order (x fastest): init/<field>,
the state after every frame f<k>/<field>, per-stage snapshots f<k>/s<j>/<stage>/<field> of the
first frames (stages source, force, project, advect; project also holds A_rowptr, A_col, A_val,
b, p), substeps (per frame) and sub_dt.  The "stock" cases run the reference as it is; the "eval"
cases run ref_harness2d_eval, which evaluates the correction term of ASTFaceGrid<double, 2>::sample
that the stock code reads from a destroyed temporary (see ref_harness2d.cpp).  Values of closed
tilts are stale pool memory in the reference and are not meaningful.  The reference sums its PCG
dot products in slices of its taskflow workers, one per hardware thread of the host: the
committed fixtures came from an 8-thread host, which the 2-D oracle's ref_workers default
(8) matches; regenerating them elsewhere needs the same worker count on both sides.

    python tests/golden/make_golden.py --2d-only

Config 0 at its full length (32^3 coarsest x 3 levels, 50 steps) and the benchmark size (64^3 x 3,
20 steps) pinned by the sha256 of every state array, the DOF maps, the pressure and the iteration
count after every step (ref_c32_l3_hashes.json, ref_c64_l3_hashes.json):

    python tests/golden/make_golden.py --hashes-3d

The 2-D command also writes ref2d_eval_a192_hashes.json: the reference example's full size (192 x 384,
evaluated correction term, 6 frames) pinned by the sha256 of every array of every frame.
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
import astg_archive  # noqa: E402

CASES = [
    # name, coarsest, levels, steps, record stage snapshots of step 1
    ("ref_c8_l3", 8, 3, 4, True),
    ("ref_c16_l2", 16, 2, 3, False),
]
STAGES = ["scene", "force", "preproject", "project", "dual", "advect"]
CKPT_CASES = [
    # name, coarsest, levels, steps before the checkpoint
    ("ref_ckpt_c8_l3", 8, 3, 2),
]
COLLIDER_CASES = [
    # the stock scene's obstacle (src/octree_omnigrid_solver3.cpp:157-158): a sphere r = 0.1 at
    # (0.5, 0.5, 0.45) through OmniBoundarySolver3::updateCollider, in the benchmark scene
    ("ref_col_c8_l3", 8, 3, 4, True),
    ("ref_col_c16_l2", 16, 2, 3, False),
]
COLLIDER = ["--collider", "0.5,0.5,0.45,0.1"]
REFINE_CASES = [
    # refineSplitMapByObstacleSdf (include/octree_util.h:17-47) applied by the reference to the scene's
    # split map with the stock sphere obstacle's SDF: (level, lo, hi) in order, coarse to fine
    ("ref_refine_c16_l3", 16, 3, [(2, -1000.0, 0.3), (1, -1000.0, 0.05)]),
]
CFL_CASES = [
    # name, coarsest, levels, frames, frame time step, maxCfl: Solver::update's adaptive branch
    # (useFixedTimeStep = false, setMaxCfl), the sub-step counts the reference computed per frame
    ("ref_cfl_c8_l3", 8, 3, 6, 0.25, 2.0),
]
CFL_KEYS = ["density_oct", "density_tilt", "heat_oct", "heat_tilt", "mac", "tilt_vel", "dual_oct", "dual_tilt",
            "tilt_e", "tilt_flags", "tilt_open", "pindex_oct", "pindex_tilt", "p", "pcg_iters", "substeps"]
EXTRAP_CASES = [
    # name, coarsest, levels, steps, (centre x, y, z, radius, max distance factor, validity offset)
    ("ref_extrap_c8_l3", 8, 3, 2, (0.47, 0.53, 0.29, 0.15, 4.0, 0.0)),
    ("ref_extrap_c16_l2", 16, 2, 2, (0.52, 0.44, 0.21, 0.11, 6.0, 0.5)),
]

CASES2D = [
    # name, harness, nx, ny, frames, dt, adaptive, frames with stage snapshots
    ("ref2d_stock_n32", "ref_harness2d", 32, 64, 3, 0.02500000037252903, 0, 1),
    ("ref2d_stock_a48", "ref_harness2d", 48, 96, 1, 0.02500000037252903, 1, 1),
    ("ref2d_eval_a48", "ref_harness2d_eval", 48, 96, 4, 0.02500000037252903, 1, 2),
    ("ref2d_eval_a32_substeps", "ref_harness2d_eval", 32, 64, 3, 0.3, 1, 0),
]
DROP2D = ("dual_vert",)
# full-size pins as hashes (the arrays themselves are too large to commit): the reference example's
# 192 x 384 with the evaluated correction term, every frame of a short run
HASH2D = [
    # name, harness, nx, ny, frames, dt, adaptive
    ("ref2d_eval_a192_hashes", "ref_harness2d_eval", 192, 384, 6, 0.02500000037252903, 1),
    # the stock reference without adaptivity (never reaches the sampler's destroyed temporary)
    ("ref2d_stock_n192_hashes", "ref_harness2d", 192, 384, 6, 0.02500000037252903, 0),
]
HASH_FIELDS = ["density_cell", "heat_cell", "mac_x", "mac_y", "tilt_open", "pindex_cell", "pindex_vert"]
HASH_OPEN_ONLY = ["density_vert", "heat_vert", "tilt_vel"]


def frame_hashes(get, is_open):
    """sha256 of each array's bytes (little-endian, the reference's order); the tilt-vertex fields
    only where the tilt is open (closed tilts hold stale pool memory in the reference)."""
    import hashlib

    out = {}
    for f in HASH_FIELDS:
        out[f] = hashlib.sha256(np.ascontiguousarray(get(f)).tobytes()).hexdigest()
    for f in HASH_OPEN_ONLY:
        out[f] = hashlib.sha256(np.ascontiguousarray(get(f)[is_open]).tobytes()).hexdigest()
    return out


# config 0's full length pinned by hashes: 32^3 coarsest x 3 levels, 50 steps
HASH3D = [("ref_c32_l3_hashes", 32, 3, 50),
          # the benchmark size (config 1's 256^3-equivalent), its first 20 steps
          ("ref_c64_l3_hashes", 64, 3, 20)]
HASH3D_FIELDS = ["density_oct", "density_tilt", "heat_oct", "heat_tilt", "mac", "tilt_vel", "dual_oct", "dual_tilt",
                 "tilt_e", "tilt_flags", "tilt_open", "pindex_oct", "pindex_tilt", "p", "pcg_iters"]


def step_hashes(get):
    """sha256 of each array's bytes (the reference's slot order)."""
    import hashlib

    return {f: hashlib.sha256(np.ascontiguousarray(get(f)).tobytes()).hexdigest() for f in HASH3D_FIELDS}


def hashes_3d(harness):
    import json

    for name, c, lv, steps in HASH3D:
        with tempfile.TemporaryDirectory() as d:
            subprocess.check_call([harness, "--coarsest", str(c), "--levels", str(lv), "--steps", str(steps), "--out", d],
                                  stdout=subprocess.DEVNULL)
            rec = {"case": [c, lv, steps], "dt": 0.01, "steps": []}
            for k in range(1, steps + 1):
                st = astg_archive.read(os.path.join(d, f"step_{k:04d}.astg"))
                rec["steps"].append(step_hashes(lambda f: st[f]))
            dst = os.path.join(HERE, name + ".json")
            with open(dst, "w") as fh:
                json.dump(rec, fh, indent=1)
            print(f"{dst}: {os.path.getsize(dst) / 1e3:.1f} kB")


def hashes_2d():
    import json

    for name, exe, nx, ny, frames, dt, adaptive in HASH2D:
        with tempfile.TemporaryDirectory() as d:
            path = os.path.join(d, "out.astg")
            subprocess.check_call([os.path.join(ROOT, "oracle", "_ref", exe), str(nx), str(ny), str(frames), repr(dt),
                                   str(adaptive), path, "0"], stdout=subprocess.DEVNULL)
            R = astg_archive.read(path)
            rec = {"case": [nx, ny, frames, adaptive], "dt": dt, "substeps": R["substeps"].tolist(),
                   "sub_dt": [float(v).hex() for v in R["sub_dt"]], "frames": []}
            for f in range(1, frames + 1):
                p = f"f{f}/"
                is_open = R[p + "tilt_open"].astype(bool)
                rec["frames"].append(frame_hashes(lambda k: R[p + k], is_open))
            dst = os.path.join(HERE, name + ".json")
            with open(dst, "w") as fh:
                json.dump(rec, fh, indent=1)
            print(f"{dst}: {os.path.getsize(dst) / 1e3:.1f} kB")


def fixtures_2d():
    for name, exe, nx, ny, frames, dt, adaptive, stage_frames in CASES2D:
        with tempfile.TemporaryDirectory() as d:
            path = os.path.join(d, "out.astg")
            subprocess.check_call([os.path.join(ROOT, "oracle", "_ref", exe), str(nx), str(ny), str(frames), repr(dt),
                                   str(adaptive), path, str(stage_frames)], stdout=subprocess.DEVNULL)
            out = {k: v for k, v in astg_archive.read(path).items() if not k.endswith(DROP2D)}
            out["meta/case"] = np.array([nx, ny, frames, adaptive, stage_frames], dtype=np.int32)
            out["meta/dt"] = np.array([dt], dtype=np.float64)
            dst = os.path.join(HERE, name + ".npz")
            np.savez_compressed(dst, **out)
            print(f"{dst}: {os.path.getsize(dst) / 1e6:.2f} MB, {len(out)} arrays")


def extrap_fixtures(harness):
    for name, c, lv, steps, ex in EXTRAP_CASES:
        with tempfile.TemporaryDirectory() as d:
            cmd = [harness, "--coarsest", str(c), "--levels", str(lv), "--steps", str(steps), "--out", d,
                   "--extrapolate", ",".join(repr(v) for v in ex)]
            subprocess.check_call(cmd)
            out = {}
            st = astg_archive.read(os.path.join(d, f"step_{steps:04d}.astg"))
            for key, v in st.items():
                if key != "wall_s":
                    out[f"before/{key}"] = v
            exr = astg_archive.read(os.path.join(d, "extrap.astg"))
            out["sdf"] = exr["sdf"]
            out["after/density_oct"] = exr["density_oct"]
            out["after/density_tilt"] = exr["density_tilt"]
            out["meta/case"] = np.array([c, lv, steps], dtype=np.int32)
            out["meta/extrap"] = np.array(ex, dtype=np.float64)
            path = os.path.join(HERE, name + ".npz")
            np.savez_compressed(path, **out)
            print(f"{path}: {os.path.getsize(path) / 1e6:.2f} MB, {len(out)} arrays")


def ckpt_fixtures(harness):
    for name, c, lv, steps in CKPT_CASES:
        with tempfile.TemporaryDirectory() as d:
            files, a, b = (os.path.join(d, x) for x in ("files", "a", "b"))
            os.makedirs(a)
            os.makedirs(b)
            base = [harness, "--coarsest", str(c), "--levels", str(lv)]
            subprocess.check_call(base + ["--steps", str(steps), "--out", a, "--checkpoint-at", str(steps),
                                          "--checkpoint-dir", files], cwd=d)
            subprocess.check_call(base + ["--steps", "1", "--out", b, "--restart", files], cwd=d)
            out = {}
            for f in ("layout.bin", "tilt.bin", "density.bin", "heat.bin", "velocity.bin"):
                out["file/" + f] = np.fromfile(os.path.join(files, f), dtype=np.uint8)
            out.update(astg_archive.read(os.path.join(b, "restart.astg")))
            st = astg_archive.read(os.path.join(b, "step_0001.astg"))
            for key, v in st.items():
                if key != "wall_s":
                    out[f"step1/{key}"] = v
            out["meta/case"] = np.array([c, lv, steps], dtype=np.int32)
            path = os.path.join(HERE, name + ".npz")
            np.savez_compressed(path, **out)
            print(f"{path}: {os.path.getsize(path) / 1e6:.2f} MB, {len(out)} arrays")


def refine_fixtures(harness):
    for name, c, lv, ranges in REFINE_CASES:
        with tempfile.TemporaryDirectory() as d:
            cmd = [harness, "--coarsest", str(c), "--levels", str(lv), "--steps", "0", "--out", d] + COLLIDER
            for r in ranges:
                cmd += ["--refine-obstacle", ",".join(repr(x) for x in r)]
            subprocess.check_call(cmd, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
            lay = astg_archive.read(os.path.join(d, "layout.astg"))
            out = {"split_map": lay["split_map"], "collider_sdf": lay["collider_sdf"],
                   "meta/case": np.array([c, lv, 0], dtype=np.int32), "meta/refine": np.array(ranges)}
            path = os.path.join(HERE, name + ".npz")
            np.savez_compressed(path, **out)
            print(f"{path}: {os.path.getsize(path) / 1e6:.2f} MB")


def cfl_fixtures(harness):
    for name, c, lv, frames, dt, max_cfl in CFL_CASES:
        with tempfile.TemporaryDirectory() as d:
            subprocess.check_call([harness, "--coarsest", str(c), "--levels", str(lv), "--steps", str(frames),
                                   "--dt", repr(dt), "--adaptive", "--max-cfl", repr(max_cfl), "--out", d],
                                  stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
            out = {}
            for k in range(1, frames + 1):
                st = astg_archive.read(os.path.join(d, f"step_{k:04d}.astg"))
                for key in CFL_KEYS:
                    out[f"frame{k}/{key}"] = st[key]
            out["meta/case"] = np.array([c, lv, frames], dtype=np.int32)
            out["meta/adaptive"] = np.array([dt, max_cfl])
            path = os.path.join(HERE, name + ".npz")
            np.savez_compressed(path, **out)
            print(f"{path}: {os.path.getsize(path) / 1e6:.2f} MB, {len(out)} arrays")


def main():
    ref = os.environ.get("ASTG_REF", os.path.join(os.path.dirname(ROOT), "reference"))
    subprocess.check_call(["make", "-s", "-f", os.path.join(ROOT, "oracle", "ref", "Makefile"), f"REF={ref}",
                           "-j8"])
    harness = os.path.join(ROOT, "oracle", "_ref", "ref_harness")
    if "--hashes-3d" in sys.argv:
        hashes_3d(harness)
        return
    if "--collider-only" in sys.argv:
        run_cases(harness, COLLIDER_CASES, COLLIDER)
        refine_fixtures(harness)
        return
    if "--cfl-only" in sys.argv:
        cfl_fixtures(harness)
        return
    if "--2d-only" in sys.argv:
        fixtures_2d()
        hashes_2d()
        return
    if "--ckpt-only" not in sys.argv:
        extrap_fixtures(harness)
    if "--extrap-only" in sys.argv:
        return
    ckpt_fixtures(harness)
    if "--ckpt-only" in sys.argv:
        return
    run_cases(harness, CASES, [])


def run_cases(harness, cases, extra):
    for name, c, lv, steps, stages in cases:
        with tempfile.TemporaryDirectory() as d:
            cmd = [harness, "--coarsest", str(c), "--levels", str(lv), "--steps", str(steps), "--out", d] + extra
            if stages:
                cmd.append("--stages")
            subprocess.check_call(cmd)
            out = {}
            lay = astg_archive.read(os.path.join(d, "layout.astg"))
            out.update(lay)
            for k in range(1, steps + 1):
                st = astg_archive.read(os.path.join(d, f"step_{k:04d}.astg"))
                for key, v in st.items():
                    if key != "wall_s":
                        out[f"step{k}/{key}"] = v
            if stages:
                st = astg_archive.read(os.path.join(d, "stages_0001.astg"))
                for key, v in st.items():
                    out[key.replace("s0_", "stage1_", 1)] = v
            out["meta/case"] = np.array([c, lv, steps], dtype=np.int32)
            path = os.path.join(HERE, name + ".npz")
            np.savez_compressed(path, **out)
            print(f"{path}: {os.path.getsize(path) / 1e6:.2f} MB, {len(out)} arrays")


if __name__ == "__main__":
    main()
