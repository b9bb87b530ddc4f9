"""ctypes front end of the CPU oracle (test infrastructure only).

The oracle is a plain C++ restatement of the reference's octree smoke step
(oracle/smoke_oracle.cpp).  Only the tests, the smoke check and the CPU-baseline leg of
bench.py use it, as the checker; the CUDA library never loads it.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
LIB_OMP = os.path.join(BUILD, "liboracle_omp.so")  # same code, independent per-node loops on OpenMP threads
SRC = os.path.join(HERE, "smoke_oracle.cpp")
SCENE = os.path.join(ROOT, "ast-grid_gb300", "csrc")
LIB2D = os.path.join(BUILD, "libast2d_oracle.so")
SRC2D = os.path.join(HERE, "ast2d_oracle.cpp")

# array names and element types exposed by orc_get
F64 = {"density_oct", "density_tilt", "heat_oct", "heat_tilt", "mac", "tilt_vel", "dual_oct", "dual_tilt",
       "tilt_e", "w_mac", "w_tilt", "A_val", "b", "p", "pcg_err", "ambT", "dual_tables", "collider_sdf"}
I32 = {"tilt_flags", "slot_coords", "level_sizes", "split_map", "pindex_oct", "pindex_tilt", "A_rowptr",
       "A_col", "pcg_iters", "anomalies"}
I64 = {"half_tilts", "t_joints", "closed_by_half_tilt"}
U8 = {"tilt_open"}
SHAPES = {"mac": (3, -1), "tilt_vel": (-1, 8), "dual_oct": (-1, 3), "dual_tilt": (-1, 3), "tilt_flags": (-1, 2),
          "slot_coords": (-1, 4), "level_sizes": (-1, 3), "w_mac": (3, -1), "w_tilt": (-1, 8),
          "dual_tables": (128, 3, 7)}


def build(force=False, openmp=False):
    """Compile the oracle with g++ (IEEE order: no fast-math, no FP contraction).  The OpenMP
    variant runs the reference's parallel per-node loops on threads; its results are identical.
    The 2-D oracle (oracle/ast2d_oracle.cpp) is built alongside."""
    os.makedirs(BUILD, exist_ok=True)
    build2d(force)
    out = LIB_OMP if openmp else LIB
    deps = [SRC, os.path.join(SCENE, "scene.h")]
    if not force and os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(d) for d in deps):
        return out
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-I", SCENE, SRC, "-o", out + ".tmp"]
    if openmp:
        cmd.insert(1, "-fopenmp")
    subprocess.check_call(cmd)
    os.replace(out + ".tmp", out)
    return out


class _Params(ctypes.Structure):
    _fields_ = [("tol", ctypes.c_double), ("buoy_d", ctypes.c_double), ("buoy_t", ctypes.c_double),
                ("decay", ctypes.c_double), ("rho", ctypes.c_double), ("noise", ctypes.c_double),
                ("src_cx", ctypes.c_double), ("src_cy", ctypes.c_double), ("src_cz", ctypes.c_double),
                ("src_r", ctypes.c_double), ("seed", ctypes.c_ulonglong), ("max_iter", ctypes.c_int),
                ("tilt_adaptivity", ctypes.c_int), ("closed_mask", ctypes.c_int), ("reduce_mode", ctypes.c_int),
                ("ref_workers", ctypes.c_int)]


_libs = {}


def lib(openmp=False):
    if openmp not in _libs:
        _lib = ctypes.CDLL(build(openmp=openmp))
        _lib.orc_create.restype = ctypes.c_void_p
        _lib.orc_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(_Params), ctypes.c_char_p, ctypes.c_int]
        _lib.orc_destroy.argtypes = [ctypes.c_void_p]
        _lib.orc_stage.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_char_p, ctypes.c_int]
        _lib.orc_step.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_char_p, ctypes.c_int]
        _lib.orc_update.restype = ctypes.c_int
        _lib.orc_update.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_void_p, ctypes.c_int,
                                    ctypes.c_char_p, ctypes.c_int]
        _lib.orc_get.restype = ctypes.c_longlong
        _lib.orc_get.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_void_p, ctypes.c_longlong]
        _lib.orc_set.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_void_p, ctypes.c_longlong]
        _lib.orc_size.argtypes = [ctypes.c_void_p, ctypes.c_int]
        _lib.orc_extrapolate.restype = ctypes.c_longlong
        _lib.orc_extrapolate.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int,
                                         ctypes.c_double, ctypes.c_double]
        _lib.orc_solve.argtypes = [ctypes.c_void_p, ctypes.c_int] + [ctypes.c_void_p] * 5 + [ctypes.c_double,
                                                                                               ctypes.c_int]
        _libs[openmp] = _lib
    return _libs[openmp]


class Oracle:
    """One oracle solver on the benchmark scene (z-up, sphere source, closed walls but the top)."""

    def __init__(self, coarsest, levels, tol=1e-6, buoy_d=-0.1, buoy_t=1.0, decay=1.0, rho=2.0, noise=1e-3,
                 source=(0.5, 0.5, 0.12, 0.06), seed=0, max_iter=3000, tilt_adaptivity=True, closed_mask=47,
                 reduce_mode=0, ref_workers=8, openmp=False):
        """reduce_mode 0 follows the reference's own arithmetic order (Eigen's dot, per-worker
        partial sums over ref_workers workers); 1 follows the CUDA library's (its fixed reduction
        tree, and one fused multiply-add for every product the PCG accumulates: MIC(0) sweep
        updates, CSR rows, dot-product lanes, vector updates)."""
        p = _Params(tol, buoy_d, buoy_t, decay, rho, noise, source[0], source[1], source[2], source[3], seed,
                    max_iter, 1 if tilt_adaptivity else 0, closed_mask, reduce_mode, ref_workers)
        self._lib = lib(openmp)
        err = ctypes.create_string_buffer(512)
        self._h = self._lib.orc_create(coarsest, levels, ctypes.byref(p), err, 512)
        if not self._h:
            raise RuntimeError("oracle: " + err.value.decode())

    def close(self):
        if self._h:
            self._lib.orc_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def _check(self, rc, err):
        if rc != 0:
            raise RuntimeError("oracle: " + err.value.decode())

    def stage(self, i, dt):
        err = ctypes.create_string_buffer(512)
        self._check(self._lib.orc_stage(self._h, i, dt, err, 512), err)

    def step(self, dt):
        err = ctypes.create_string_buffer(512)
        self._check(self._lib.orc_step(self._h, dt, err, 512), err)

    def update(self, dt, max_cfl=3.0):
        """Solver::update with useFixedTimeStep = false (CFL sub-steps); returns the sub-step counts."""
        err = ctypes.create_string_buffer(512)
        buf = (ctypes.c_int * 4096)()
        n = self._lib.orc_update(self._h, dt, max_cfl, buf, 4096, err, 512)
        if n < 0:
            raise RuntimeError("oracle: " + err.value.decode())
        return list(buf[:n])

    def get(self, name):
        n = self._lib.orc_get(self._h, name.encode(), None, 0)
        if n < 0:
            raise KeyError(name)
        dt = np.float64 if name in F64 else np.int32 if name in I32 else np.int64 if name in I64 else np.uint8
        out = np.empty(n, dtype=dt)
        self._lib.orc_get(self._h, name.encode(), out.ctypes.data, n)
        if name in SHAPES:
            out = out.reshape(SHAPES[name])
        return out

    def set(self, name, arr):
        fields = {"density_oct", "density_tilt", "heat_oct", "heat_tilt", "mac", "tilt_vel", "dual_oct",
                  "dual_tilt", "tilt_e", "tilt_flags", "tilt_open"}
        base = name[2:] if name.startswith("t_") and name[2:] in fields else name
        dt = np.int32 if base == "tilt_flags" else np.uint8 if base == "tilt_open" else np.float64
        a = np.ascontiguousarray(arr, dtype=dt).ravel()
        rc = self._lib.orc_set(self._h, name.encode(), a.ctypes.data, a.size)
        if rc != 0:
            raise ValueError(f"oracle: cannot set {name} ({rc})")

    def solve(self, rowptr, col, val, b, tol=1e-6, max_iter=3000):
        """PCGSolver::solve on a CSR system; returns (x, iterations)."""
        rp = np.ascontiguousarray(rowptr, dtype=np.int32)
        c = np.ascontiguousarray(col, dtype=np.int32)
        v = np.ascontiguousarray(val, dtype=np.float64)
        bb = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros(len(bb))
        it = self._lib.orc_solve(self._h, len(bb), rp.ctypes.data, c.ctypes.data, v.ctypes.data, bb.ctypes.data,
                                 x.ctypes.data, tol, max_iter)
        return x, it

    def extrapolate(self, field, sdf, offset=0.0, max_distance_factor=4.0):
        """FmmLevelSetSolver3::extrapolate of "density" or "heat" in place from the nodes where
        sdf < -offset * d; sdf is res^3 (index (z*res + y)*res + x).  Returns the nodes assigned."""
        g = np.ascontiguousarray(sdf, dtype=np.float64).ravel()
        res = round(len(g) ** (1.0 / 3.0))
        if res ** 3 != len(g):
            raise ValueError("sdf must hold res^3 values")
        n = self._lib.orc_extrapolate(self._h, field.encode(), g.ctypes.data, res, offset, max_distance_factor)
        if n < 0:
            raise ValueError("oracle: bad extrapolation argument")
        return n

    @property
    def slots(self):
        return self._lib.orc_size(self._h, 0)

    @property
    def ndof(self):
        return self._lib.orc_size(self._h, 3)


def build2d(force=False):
    """Compile the 2-D oracle (uniform ASTSolver<2> restatement) with the same IEEE flags."""
    os.makedirs(BUILD, exist_ok=True)
    if not force and os.path.exists(LIB2D) and os.path.getmtime(LIB2D) >= os.path.getmtime(SRC2D):
        return LIB2D
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", SRC2D,
                           "-o", LIB2D + ".tmp"])
    os.replace(LIB2D + ".tmp", LIB2D)
    return LIB2D


_lib2d = None


def lib2d():
    global _lib2d
    if _lib2d is None:
        L = ctypes.CDLL(build2d())
        L.ast2o_error.restype = ctypes.c_char_p
        L.ast2o_create.restype = ctypes.c_void_p
        L.ast2o_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.ast2o_destroy.argtypes = [ctypes.c_void_p]
        L.ast2o_update.argtypes = [ctypes.c_void_p, ctypes.c_double]
        L.ast2o_stage.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double]
        L.ast2o_count.restype = ctypes.c_long
        L.ast2o_count.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.POINTER(ctypes.c_int)]
        L.ast2o_get.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_void_p, ctypes.c_long]
        L.ast2o_set.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_void_p, ctypes.c_long]
        L.ast2o_info.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_long)]
        _lib2d = L
    return _lib2d


SHAPES2D = {"density_cell": "c", "heat_cell": "c", "pindex_cell": "c", "density_vert": "v", "heat_vert": "v",
            "tilt_open": "v", "pindex_vert": "v", "mac_x": "x", "mac_y": "y", "tilt_vel": "t", "dual_vert": "d"}
STAGES2D = {"source": 0, "force": 1, "project": 2, "advect": 3, "substep": 4}


class Oracle2D:
    """The uniform 2-D AST smoke solver (ASTSolver<2>, sphere source at the bottom, closed x walls,
    open top and bottom) on an nx x ny grid of spacing dx.  reduce_mode 0 follows the reference's
    arithmetic order (its dot products summed in per-worker slices over ref_workers taskflow
    workers -- the reference's default is the host's hardware thread count; the committed
    fixtures came from an 8-thread host), 1 the CUDA library's (fixed reduction tree, fused
    multiply-subtract in the MIC(0) sweeps)."""

    def __init__(self, nx, ny, dx=None, adaptive=True, reduce_mode=0, ref_workers=8):
        self._lib = lib2d()
        self.nx, self.ny = nx, ny
        self.dx = 1.0 / nx if dx is None else dx
        self._h = self._lib.ast2o_create(nx, ny, self.dx, 1 if adaptive else 0, reduce_mode, ref_workers)
        if not self._h:
            raise ValueError(self._lib.ast2o_error().decode())

    def close(self):
        if self._h:
            self._lib.ast2o_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError(self._lib.ast2o_error().decode())

    def update(self, dt):
        """One frame: the CFL sub-stepping of Solver::update over dt."""
        self._check(self._lib.ast2o_update(self._h, dt))

    def stage(self, name, dt):
        self._check(self._lib.ast2o_stage(self._h, STAGES2D[name], dt))

    def _shape(self, name, n):
        nx, ny = self.nx, self.ny
        kind = SHAPES2D.get(name)
        return {"c": (ny, nx), "v": (ny + 1, nx + 1), "x": (ny, nx + 1), "y": (ny + 1, nx),
                "t": (ny + 1, nx + 1, 4), "d": (ny + 1, nx + 1, 2)}.get(kind, (n,))

    def get(self, name):
        kind = ctypes.c_int(0)
        n = self._lib.ast2o_count(self._h, name.encode(), ctypes.byref(kind))
        if n < 0:
            raise KeyError(name)
        out = np.empty(n, dtype=[np.float64, np.uint8, np.int32][kind.value])
        self._check(self._lib.ast2o_get(self._h, name.encode(), out.ctypes.data, n))
        return out.reshape(self._shape(name, n))

    def set(self, name, arr):
        a = np.ascontiguousarray(arr, dtype=np.uint8 if name == "tilt_open" else np.float64).ravel()
        self._check(self._lib.ast2o_set(self._h, name.encode(), a.ctypes.data, a.size))

    def info(self):
        """dict: substeps (last frame), unknowns, pcg_iters, pcg_ok, nnz, substeps_total."""
        out = (ctypes.c_long * 6)()
        self._lib.ast2o_info(self._h, out)
        keys = ["substeps", "unknowns", "pcg_iters", "pcg_ok", "nnz", "substeps_total"]
        return dict(zip(keys, list(out)))
