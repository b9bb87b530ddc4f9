"""CPU checks of the drop-in boundary: the CUDA library builds, loads and exports every entry
point include/astg.h and include/astg2d.h declare; the Python front end refuses to run without it."""
import os
import re
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "ast-grid_gb300")
if PKG not in sys.path:
    sys.path.insert(0, PKG)


def declared_symbols():
    out = set()
    for h in ("astg.h", "astg2d.h"):
        txt = open(os.path.join(ROOT, "include", h)).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        out |= set(re.findall(r"\b(astg2?_[a-z_0-9]+)\s*\(", txt))
    return sorted(out)


def test_library_exports_every_declared_symbol():
    import ctypes

    import build_lib

    path = build_lib.build()
    so = ctypes.CDLL(path)
    syms = declared_symbols()
    assert len(syms) >= 10
    missing = [s for s in syms if not hasattr(so, s)]
    assert not missing, f"not exported: {missing}"


def test_python_front_end_lists_the_abi():
    import ast_solver

    assert sorted(ast_solver.SYMBOLS) == declared_symbols()


def test_missing_library_fails_loudly(tmp_path):
    import ast_solver

    saved = ast_solver._lib
    ast_solver._lib = None
    try:
        with pytest.raises(OSError):
            ast_solver.lib(str(tmp_path / "nope.so"))
    finally:
        ast_solver._lib = saved


def test_default_params_match_the_benchmark_scene():
    import ctypes

    import ast_solver

    p = ast_solver.Params()
    ast_solver.lib().astg_default_params(ctypes.byref(p), 32, 3)
    assert (p.coarsest, p.levels, p.max_iter) == (32, 3, 3000)
    assert (p.tol, p.omega, p.min_diag, p.rho) == (1e-6, 0.97, 0.25, 2.0)
    assert (p.buoy_density, p.buoy_temp, p.decay) == (-0.1, 1.0, 1.0)
    assert (p.src_x, p.src_y, p.src_z, p.src_r) == (0.5, 0.5, 0.12, 0.06)
    assert p.closed_mask == 0b101111  # z+ open


@pytest.mark.parametrize("header", ["astg.h", "astg2d.h"])
def test_headers_compile_as_c99(tmp_path, header):
    """The boundary is plain C: each header compiles on its own as C99 with -pedantic."""
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    src = tmp_path / "h.c"
    src.write_text(f'#include "{header}"\nint main(void) {{ return 0; }}\n')
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", os.path.join(ROOT, "include"),
                        "-c", str(src), "-o", str(tmp_path / "h.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_refine_split_map_matches_reference():
    """astg_refine_split_map (host-side, no device) against the reference's own
    refineSplitMapByObstacleSdf (include/octree_util.h:17-47) on the scene's split map with the stock
    sphere obstacle's SDF grid, two passes coarse to fine."""
    import ctypes

    import numpy as np

    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from fixtures import golden
    from oracle.oracle import Oracle

    g = golden("ref_refine_c16_l3")
    c, lv, _ = g["meta/case"].tolist()
    res = c << (lv - 1)
    split = np.ascontiguousarray(Oracle(c, lv).get("split_map"), dtype=np.int32)
    sdf = np.ascontiguousarray(g["collider_sdf"], dtype=np.float64)
    import build_lib

    L = ctypes.CDLL(build_lib.build())
    L.astg_refine_split_map.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_double,
                                        ctypes.c_double]
    before = split.copy()
    for level, lo, hi in g["meta/refine"].tolist():
        assert L.astg_refine_split_map(split.ctypes.data, res, int(level), sdf.ctypes.data, lo, hi) == 0
    assert (split != before).sum() > 100
    assert np.array_equal(split, g["split_map"].ravel())
    assert L.astg_refine_split_map(split.ctypes.data, res - 1, 1, sdf.ctypes.data, 0.0, 1.0) == 1


def test_cpp_example_builds_against_the_header_alone():
    """examples/octree_smoke.cpp (a host program using only include/astg.h) compiles and links
    against the library; it runs in tests/test_gpu_example.py."""
    import build_lib

    exe = build_lib.build_example()
    assert os.path.isfile(exe) and os.access(exe, os.X_OK)


def test_new_entry_points_refuse_bad_arguments_without_a_device():
    """Argument checks of the collider, batch-solve and device-refinement entry points run before any
    device work: a null handle or null arrays give ASTG_BAD_ARG (no GPU needed)."""
    import ctypes

    import ast_solver

    L = ast_solver.lib()
    assert L.astg_set_collider_sphere(None, 0.5, 0.5, 0.45, 0.1) == ast_solver.ASTG_BAD_ARG
    one = (ctypes.c_int * 2)(0, 1)
    val = (ctypes.c_double * 1)(1.0)
    st = (ast_solver.SolveStats * 1)()
    assert L.astg_solve_batch(None, 1, one, one, val, 1, val, val, 1e-6, 10, ast_solver.FP64, st, None,
                              None) == ast_solver.ASTG_BAD_ARG
    assert L.astg_refine_split_map_device(None, 8, 1, None, 0.0, 1.0, None) == ast_solver.ASTG_BAD_ARG
