"""Python front end of the GB300 octree smoke step (module name and entry points follow the
reference's pybind module ``ast_solver``, python_bindings/ast_solver.cc:14-80).

``OctreeSmoke3`` wraps OctreeOmniGridSolver3 (include/octree_omnigrid_solver3.h:23-57) through
the C ABI of include/astg.h; ``ASTSolver2`` runs the reference module's uniform 2-D solver
(ASTSolver<2>, include/ast_solver.h) through include/astg2d.h, and the module's other bound names
(``ASTGridLayout2/3``, ``TiltNode2/3``, ``CellNode2/3``, ``ASTGrid2/3``, ``ASTSolver3``,
``benchmark_*``) keep their signatures.  The library must be built (``build_lib.build()``); using
a solver on a machine without it raises instead of falling back to anything.
"""
import ctypes
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libastgrid_gpu.so")

ASTG_OK, ASTG_BAD_ARG, ASTG_CUDA_ERROR, ASTG_NOT_CONVERGED = 0, 1, 2, 3
ASTG_DEVICE_WAIT_TIMEOUT, ASTG_NAN_DETECTED, ASTG_LAYOUT_ERROR, ASTG_NO_DEVICE = 4, 5, 6, 7
STATUS = {0: "ok", 1: "bad argument", 2: "CUDA error", 3: "not converged", 4: "device wait timeout",
          5: "NaN detected", 6: "layout error", 7: "no CUDA device"}
FP64, MIXED = 0, 1

# exported symbols of include/astg.h
SYMBOLS = ["astg_default_params", "astg_create", "astg_destroy", "astg_last_error", "astg_step", "astg_update",
           "astg_set_max_cfl", "astg_cfl", "astg_stage", "astg_refine_split_map", "astg_set_collider_sphere", "astg_solve_batch", "astg_refine_split_map_device",
           "astg_set_solver_parameters", "astg_set_precision", "astg_set_reduction_order", "astg_set_profiling", "astg_last_solve", "astg_size", "astg_get", "astg_set",
           "astg_solve", "astg_max_velocity", "astg_mean_temperature_noalloc", "astg_extrapolate",
           "astg_restart", "astg_save_checkpoint", "astg_tape_start", "astg_tape_stop", "astg_adjoint_reset",
           "astg_backward", "astg_step_vjp", "astg_stage_vjp", "astg_adjoint_probe", "astg_set_tilt_adaptivity",
           # include/astg2d.h (uniform 2-D AST solver)
           "astg2_create", "astg2_destroy", "astg2_last_error", "astg2_update", "astg2_stage", "astg2_get_density",
           "astg2_count", "astg2_get", "astg2_set", "astg2_set_solver", "astg2_last_stats"]


class AstgError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


class ExtrapStats(ctypes.Structure):
    _fields_ = [("assigned", ctypes.c_longlong), ("passes", ctypes.c_int), ("ms", ctypes.c_double)]


class AdjointStats(ctypes.Structure):
    _fields_ = [("steps", ctypes.c_int), ("checkpoints", ctypes.c_int), ("recomputed_steps", ctypes.c_int),
                ("solves", ctypes.c_int), ("pcg_iterations", ctypes.c_longlong), ("ms", ctypes.c_double),
                ("ms_recompute", ctypes.c_double), ("tape_bytes", ctypes.c_longlong)]


class Params(ctypes.Structure):
    _fields_ = [("coarsest", ctypes.c_int), ("levels", ctypes.c_int), ("tol", ctypes.c_double),
                ("max_iter", ctypes.c_int), ("omega", ctypes.c_double), ("min_diag", ctypes.c_double),
                ("rho", ctypes.c_double), ("buoy_density", ctypes.c_double), ("buoy_temp", ctypes.c_double),
                ("decay", ctypes.c_double), ("closed_mask", ctypes.c_int), ("tilt_adaptivity", ctypes.c_int),
                ("src_x", ctypes.c_double), ("src_y", ctypes.c_double), ("src_z", ctypes.c_double),
                ("src_r", ctypes.c_double), ("noise", ctypes.c_double), ("seed", ctypes.c_uint64),
                ("precision", ctypes.c_int), ("device", ctypes.c_int)]


class SolveStats(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int), ("outer", ctypes.c_int), ("converged", ctypes.c_int),
                ("n", ctypes.c_int), ("nnz", ctypes.c_longlong), ("residual", ctypes.c_double),
                ("tolerance", ctypes.c_double), ("ms", ctypes.c_double)]


class Stats2D(ctypes.Structure):
    _fields_ = [("substeps", ctypes.c_int), ("unknowns", ctypes.c_int), ("pcg_iterations", ctypes.c_int),
                ("pcg_converged", ctypes.c_int), ("nnz", ctypes.c_longlong), ("pcg_residual", ctypes.c_double),
                ("ms", ctypes.c_double), ("substeps_total", ctypes.c_longlong)]


class StepStats(ctypes.Structure):
    _fields_ = [("solve", SolveStats), ("ms_total", ctypes.c_double), ("ms_force", ctypes.c_double),
                ("ms_project", ctypes.c_double), ("ms_advect", ctypes.c_double)]


_lib = None


def lib(path=None):
    """Loads libastgrid_gpu.so (raises OSError when it has not been built)."""
    global _lib
    if _lib is None:
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise OSError(f"{p} is missing: build it with ast-grid_gb300/build_lib.py (nvcc, sm_103a)")
        L = ctypes.CDLL(p)
        c_p = ctypes.c_void_p
        L.astg_default_params.argtypes = [ctypes.POINTER(Params), ctypes.c_int, ctypes.c_int]
        L.astg_create.argtypes = [ctypes.POINTER(Params), ctypes.c_void_p, ctypes.POINTER(c_p)]
        L.astg_destroy.argtypes = [c_p]
        L.astg_last_error.argtypes = [c_p]
        L.astg_last_error.restype = ctypes.c_char_p
        L.astg_step.argtypes = [c_p, ctypes.c_double, ctypes.POINTER(StepStats)]
        L.astg_stage.argtypes = [c_p, ctypes.c_int, ctypes.c_double]
        L.astg_set_solver_parameters.argtypes = [c_p, ctypes.c_double, ctypes.c_int, ctypes.c_double, ctypes.c_double]
        L.astg_set_precision.argtypes = [c_p, ctypes.c_int]
        L.astg_update.argtypes = [c_p, ctypes.c_double, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(StepStats)]
        L.astg_set_max_cfl.argtypes = [c_p, ctypes.c_double]
        L.astg_refine_split_map_device.argtypes = [c_p, ctypes.c_int, ctypes.c_int, c_p, ctypes.c_double,
                                                   ctypes.c_double, c_p]
        L.astg_set_collider_sphere.argtypes = [c_p, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double]
        L.astg_refine_split_map.argtypes = [c_p, ctypes.c_int, ctypes.c_int, c_p, ctypes.c_double, ctypes.c_double]
        L.astg_cfl.argtypes = [c_p, ctypes.c_double, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
        L.astg_set_reduction_order.argtypes = [c_p, ctypes.c_int, ctypes.c_int]
        L.astg_set_profiling.argtypes = [c_p, ctypes.c_int]
        L.astg_last_solve.argtypes = [c_p, ctypes.POINTER(SolveStats)]
        L.astg_size.argtypes = [c_p, ctypes.c_int]
        L.astg_size.restype = ctypes.c_longlong
        L.astg_get.argtypes = [c_p, ctypes.c_char_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]
        L.astg_set.argtypes = [c_p, ctypes.c_char_p, ctypes.c_void_p, ctypes.c_size_t]
        L.astg_solve.argtypes = [c_p, ctypes.c_int, c_p, c_p, c_p, c_p, c_p, ctypes.c_double, ctypes.c_int,
                                 ctypes.c_int, ctypes.POINTER(SolveStats)]
        L.astg_solve_batch.argtypes = [c_p, ctypes.c_int, c_p, c_p, c_p, ctypes.c_int, c_p, c_p, ctypes.c_double,
                                       ctypes.c_int, ctypes.c_int, ctypes.POINTER(SolveStats), c_p, c_p]
        L.astg_max_velocity.argtypes = [c_p, ctypes.POINTER(ctypes.c_double)]
        L.astg_restart.argtypes = [c_p, ctypes.c_int] + [ctypes.c_char_p] * 6
        L.astg_save_checkpoint.argtypes = [c_p] + [ctypes.c_char_p] * 5
        L.astg_extrapolate.argtypes = [c_p, ctypes.c_char_p, c_p, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                       ctypes.POINTER(ExtrapStats)]
        L.astg_mean_temperature_noalloc.argtypes = [c_p, ctypes.POINTER(ctypes.c_int64), ctypes.c_int, c_p, c_p,
                                                    ctypes.c_char_p, ctypes.c_size_t]
        L.astg_tape_start.argtypes = [c_p, ctypes.c_int]
        L.astg_set_tilt_adaptivity.argtypes = [c_p, ctypes.c_int]
        L.astg_tape_stop.argtypes = [c_p]
        L.astg_adjoint_reset.argtypes = [c_p]
        L.astg_backward.argtypes = [c_p, ctypes.POINTER(AdjointStats)]
        L.astg_step_vjp.argtypes = [c_p, ctypes.c_double]
        L.astg_stage_vjp.argtypes = [c_p, ctypes.c_int, ctypes.c_double]
        L.astg_adjoint_probe.argtypes = [c_p, ctypes.c_int, ctypes.c_int, c_p, c_p]
        L.astg2_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                   ctypes.POINTER(c_p)]
        L.astg2_destroy.argtypes = [c_p]
        L.astg2_last_error.argtypes = [c_p]
        L.astg2_last_error.restype = ctypes.c_char_p
        L.astg2_update.argtypes = [c_p, ctypes.c_double]
        L.astg2_stage.argtypes = [c_p, ctypes.c_int, ctypes.c_double]
        L.astg2_get_density.argtypes = [c_p, c_p, ctypes.c_longlong]
        L.astg2_count.argtypes = [c_p, ctypes.c_char_p, ctypes.POINTER(ctypes.c_int)]
        L.astg2_count.restype = ctypes.c_longlong
        L.astg2_get.argtypes = [c_p, ctypes.c_char_p, c_p, ctypes.c_longlong]
        L.astg2_set.argtypes = [c_p, ctypes.c_char_p, c_p, ctypes.c_longlong]
        L.astg2_set_solver.argtypes = [c_p, ctypes.c_double, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                       ctypes.c_int]
        L.astg2_last_stats.argtypes = [c_p, ctypes.POINTER(Stats2D)]
        _lib = L
    return _lib


_F64 = {"kernel_ms", "density_oct", "density_tilt", "heat_oct", "heat_tilt", "mac", "tilt_vel", "dual_oct", "dual_tilt",
        "tilt_e", "w_mac", "w_tilt", "dual_tables", "A_val", "b", "p", "ambT", "source_density_oct",
        "source_density_tilt", "collider_sdf", "collider_centre"}
_I64 = {"half_tilts", "t_joints", "closed_by_half_tilt"}
_U8 = {"tilt_open"}
_SHAPES = {"mac": (3, -1), "tilt_vel": (-1, 8), "dual_oct": (-1, 3), "dual_tilt": (-1, 3), "tilt_flags": (-1, 2),
           "slot_coords": (-1, 4), "level_sizes": (-1, 3), "w_mac": (3, -1), "w_tilt": (-1, 8),
           "dual_tables": (128, 3, 7)}


_FIELDS = {"density_oct", "density_tilt", "heat_oct", "heat_tilt", "mac", "tilt_vel", "dual_oct", "dual_tilt",
           "tilt_e", "tilt_flags", "tilt_open"}


def _base(name):
    """Field name without the "t_" prefix that addresses the swap-partner buffer, or the "adj_"
    prefix of a cotangent array (same type and shape as the array it belongs to)."""
    if name.startswith("adj_"):
        return name[4:]
    return name[2:] if name.startswith("t_") and name[2:] in _FIELDS else name


def _dtype(name):
    base = _base(name)
    if base in _F64:
        return np.float64
    if base in _I64:
        return np.int64
    if base in _U8:
        return np.uint8
    return np.int32


def refine_split_map(split_map, level, sdf, split_range):
    """refineSplitMapByObstacleSdf (include/octree_util.h:17-47) on a res^3 split map (in place, int32,
    index (z * res + y) * res + x) with an SDF grid of the same shape at the finest cell centres:
    blocks of split value `level` whose centre SDF lies in split_range = (lo, hi) become level - 1."""
    sm = np.ascontiguousarray(split_map, dtype=np.int32)
    sd = np.ascontiguousarray(sdf, dtype=np.float64)
    res = round(sm.size ** (1 / 3))
    if res ** 3 != sm.size or sd.size != sm.size:
        raise ValueError("refine_split_map: split_map and sdf must be res^3 arrays")
    st = lib().astg_refine_split_map(sm.ctypes.data, res, int(level), sd.ctypes.data, float(split_range[0]),
                                     float(split_range[1]))
    if st != ASTG_OK:
        raise AstgError(st, "resolution not divisible by 2^level, or a bad argument")
    return sm.reshape(np.shape(split_map))


def refine_split_map_tensor(split_map, level, sdf, split_range):
    """refine_split_map on CUDA tensors (int32 and float64, res^3 elements each, contiguous), in place
    on the tensors' device and current stream (astg_refine_split_map_device)."""
    import torch

    if not (split_map.is_cuda and sdf.is_cuda) or split_map.dtype != torch.int32 or sdf.dtype != torch.float64:
        raise ValueError("refine_split_map_tensor: int32 and float64 CUDA tensors")
    if not (split_map.is_contiguous() and sdf.is_contiguous()) or split_map.numel() != sdf.numel():
        raise ValueError("refine_split_map_tensor: contiguous tensors of res^3 elements")
    res = round(split_map.numel() ** (1 / 3))
    if res ** 3 != split_map.numel():
        raise ValueError("refine_split_map_tensor: res^3 elements")
    stream = torch.cuda.current_stream(split_map.device).cuda_stream
    with torch.cuda.device(split_map.device):
        st = lib().astg_refine_split_map_device(split_map.data_ptr(), res, int(level), sdf.data_ptr(),
                                                float(split_range[0]), float(split_range[1]), stream)
    if st != ASTG_OK:
        raise AstgError(st, "resolution not divisible by 2^level, host memory, or a failed launch")
    return split_map


class OctreeSmoke3:
    """GPU OctreeOmniGridSolver3 on the benchmark scene (or on a caller-supplied split map).

    OctreeSmoke3(coarsest, levels, **params) builds the octree and initialises the fields
    (ctor + initialize(), src/octree_omnigrid_solver3.cpp:45-149); update(dt) is one fixed-time
    step (Solver::update with useFixedTimeStep, src/solver.cpp:8-46)."""

    def __init__(self, coarsest, levels, split_map=None, **kw):
        L = lib()
        p = Params()
        L.astg_default_params(ctypes.byref(p), coarsest, levels)
        for k, v in kw.items():
            if k == "source":
                p.src_x, p.src_y, p.src_z, p.src_r = v
            elif k == "precision":
                p.precision = {"fp64": FP64, "mixed": MIXED}.get(v, v)
            else:
                setattr(p, k, v)
        self.params = p
        h = ctypes.c_void_p()
        sm = None
        if split_map is not None:
            sm = np.ascontiguousarray(split_map, dtype=np.int32)
        st = L.astg_create(ctypes.byref(p), sm.ctypes.data if sm is not None else None, ctypes.byref(h))
        self._h = h
        if st != ASTG_OK:
            msg = L.astg_last_error(h).decode() if h.value else ""
            if h.value:
                L.astg_destroy(h)
            self._h = None
            raise AstgError(st, msg)
        self.last_step = StepStats()

    def close(self):
        if getattr(self, "_h", None):
            lib().astg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st, allow=()):
        if st != ASTG_OK and st not in allow:
            raise AstgError(st, lib().astg_last_error(self._h).decode())
        return st

    # Solver::useFixedTimeStep (include/solver.h:21).  The reference defaults to false (CFL sub-steps);
    # these handles default to the benchmark scene's fixed step.
    useFixedTimeStep = True

    def update(self, dt):
        """Solver::update(dt): one fixed step, or (useFixedTimeStep False) CFL sub-steps whose count
        is left in self.last_substeps."""
        if self.useFixedTimeStep:
            self.last_substeps = 1
            return self._check(lib().astg_step(self._h, dt, ctypes.byref(self.last_step)), allow=(ASTG_NOT_CONVERGED,))
        n = ctypes.c_int(0)
        st = self._check(lib().astg_update(self._h, dt, ctypes.byref(n), ctypes.byref(self.last_step)),
                         allow=(ASTG_NOT_CONVERGED,))
        self.last_substeps = n.value
        return st

    def setMaxCfl(self, cfl):
        self._check(lib().astg_set_max_cfl(self._h, cfl))

    def cfl(self, dt):
        c = ctypes.c_int(0)
        self._check(lib().astg_cfl(self._h, dt, ctypes.byref(c), None))
        return c.value

    def numberOfSubTimeSteps(self, dt):
        k = ctypes.c_int(0)
        self._check(lib().astg_cfl(self._h, dt, None, ctypes.byref(k)))
        return k.value

    def stage(self, i, dt):
        self._check(lib().astg_stage(self._h, i, dt))

    def set_solver_parameters(self, tol, max_iter, omega=0.97, min_diag=0.25):
        self._check(lib().astg_set_solver_parameters(self._h, tol, max_iter, omega, min_diag))

    def set_precision(self, prec):
        self._check(lib().astg_set_precision(self._h, {"fp64": FP64, "mixed": MIXED}.get(prec, prec)))

    def set_reduction_order(self, order, workers=8):
        """"library" (the default: fixed reduction tree, fused sweep updates) or "reference" (the
        reference's own arithmetic, bit for bit; `workers` is the reference's thread-pool size, on
        which its BLAS::sum slices depend)."""
        self._check(lib().astg_set_reduction_order(self._h, {"library": 0, "reference": 1}.get(order, order), workers))

    def set_profiling(self, on):
        self._check(lib().astg_set_profiling(self._h, 1 if on else 0))

    def kernel_ms(self):
        """{kernel: (total ms, launches)} of the profiled PCG kernels."""
        v = self.get("kernel_ms")
        names = ["sweep_fwd", "sweep_bwd", "spmv_dot", "mic_factor"]
        return {n: (float(v[2 * i]), int(v[2 * i + 1])) for i, n in enumerate(names)}

    @property
    def launches(self):
        return self.size(6)

    def last_solve(self):
        s = SolveStats()
        self._check(lib().astg_last_solve(self._h, ctypes.byref(s)))
        return s

    def size(self, what):
        return lib().astg_size(self._h, what)

    @property
    def slots(self):
        return self.size(0)

    def _nbytes(self, name):
        need = ctypes.c_size_t(0)
        st = lib().astg_get(self._h, name.encode(), None, 0, ctypes.byref(need))
        if st != ASTG_BAD_ARG:  # a size query answers BAD_ARG with the size filled in
            self._check(st)
        if st == ASTG_BAD_ARG and need.value == 0 and lib().astg_last_error(self._h):
            err = lib().astg_last_error(self._h).decode()
            if "unknown" in err:
                raise AstgError(st, err)
        return need.value

    def get(self, name):
        nb = self._nbytes(name)
        dt = _dtype(name)
        out = np.empty(nb // np.dtype(dt).itemsize, dtype=dt)
        if out.size:
            self._check(lib().astg_get(self._h, name.encode(), out.ctypes.data, nb, None))
        base = _base(name)
        return out.reshape(_SHAPES[base]) if base in _SHAPES else out

    def set(self, name, arr):
        a = np.ascontiguousarray(arr, dtype=_dtype(name)).ravel()
        self._check(lib().astg_set(self._h, name.encode(), a.ctypes.data, a.nbytes))

    def set_collider_sphere(self, center=(0.5, 0.5, 0.45), radius=0.1):
        """OmniBoundarySolver3::updateCollider with a Sphere3 (the stock obstacle by default); the SDF
        grid is computed on the device.  radius <= 0 removes the collider."""
        cx, cy, cz = (float(v) for v in center)
        self._check(lib().astg_set_collider_sphere(self._h, cx, cy, cz, float(radius)))

    # torch tensors: the library copies straight from / into device (or host) memory
    def get_tensor(self, name, device="cuda"):
        import torch

        if _dtype(name) is not np.float64:
            raise ValueError("get_tensor: only f64 arrays")
        nb = self._nbytes(name)
        out = torch.empty(nb // 8, dtype=torch.float64, device=device)
        if out.is_cuda:
            torch.cuda.current_stream(out.device).synchronize()
        if out.numel():
            self._check(lib().astg_get(self._h, name.encode(), out.data_ptr(), nb, None))
        base = _base(name)
        return out.reshape(_SHAPES[base]) if base in _SHAPES else out

    def set_tensor(self, name, t):
        import torch

        t = t.detach().to(torch.float64).contiguous()
        if t.is_cuda:
            torch.cuda.current_stream(t.device).synchronize()
        self._check(lib().astg_set(self._h, name.encode(), t.data_ptr(), t.numel() * 8))

    # ---- reverse mode (topology frozen: tilt adaptivity off)
    def set_tilt_adaptivity(self, on):
        """enableTiltAdaptivity; turning it off freezes the current tilt layout in both buffers."""
        self._check(lib().astg_set_tilt_adaptivity(self._h, 1 if on else 0))

    def tape_start(self, checkpoint_every=0):
        """Records the following update() calls for backward(); checkpoint_every = k > 0 keeps the
        state every k steps and recomputes the rest, 0 keeps every step's advection input."""
        self._check(lib().astg_tape_start(self._h, checkpoint_every))

    def tape_stop(self):
        self._check(lib().astg_tape_stop(self._h))

    def adjoint_reset(self):
        self._check(lib().astg_adjoint_reset(self._h))

    def backward(self):
        """Reverse pass over the taped steps: the adj_* arrays go from the cotangent of the final
        state to that of the state at tape_start (see astg_backward).  Returns AdjointStats."""
        st = AdjointStats()
        self._check(lib().astg_backward(self._h, ctypes.byref(st)))
        return st

    def step_vjp(self, dt):
        self._check(lib().astg_step_vjp(self._h, dt))

    def stage_vjp(self, stage, dt):
        self._check(lib().astg_stage_vjp(self._h, stage, dt))

    def adjoint_probe(self, what, pos):
        """Sampler weights at positions (n x 3): what 0 -> (n, 5), what 1 -> (n, 15); see astg.h."""
        p = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        per = 5 if what == 0 else 15
        out = np.zeros((len(p), per))
        self._check(lib().astg_adjoint_probe(self._h, what, len(p), p.ctypes.data, out.ctypes.data))
        return out

    # reference-style getters (copies, reference storage order)
    def getDensity(self):
        return self.get("density_oct")

    def getHeat(self):
        return self.get("heat_oct")

    def solve(self, rowptr, col, val, b, rel_tol=1e-6, max_iter=3000, precision="fp64"):
        """PCGSolver::solve(A, b, x) on a CSR system in host memory; returns (x, SolveStats)."""
        rp = np.ascontiguousarray(rowptr, dtype=np.int32)
        c = np.ascontiguousarray(col, dtype=np.int32)
        v = np.ascontiguousarray(val, dtype=np.float64)
        bb = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros(len(bb))
        st = SolveStats()
        prec = {"fp64": FP64, "mixed": MIXED}.get(precision, precision)
        self._check(lib().astg_solve(self._h, len(bb), rp.ctypes.data, c.ctypes.data, v.ctypes.data, bb.ctypes.data,
                                     x.ctypes.data, rel_tol, max_iter, prec, ctypes.byref(st)),
                    allow=(ASTG_NOT_CONVERGED,))
        return x, st

    def solve_batch(self, rowptr, col, val, B, rel_tol=1e-6, max_iter=3000, precision="fp64"):
        """astg_solve for every row of B (nrhs x n) on one matrix, the solves side by side on the
        device; returns (X, [SolveStats], wall_ms, lanes).  Each row of X is what solve() returns."""
        rp = np.ascontiguousarray(rowptr, dtype=np.int32)
        c = np.ascontiguousarray(col, dtype=np.int32)
        v = np.ascontiguousarray(val, dtype=np.float64)
        bb = np.ascontiguousarray(B, dtype=np.float64)
        if bb.ndim != 2:
            raise ValueError("B must be nrhs x n")
        nrhs, n = bb.shape
        x = np.zeros((nrhs, n))
        st = (SolveStats * nrhs)()
        wall = ctypes.c_double(0)
        lanes = ctypes.c_int(0)
        prec = {"fp64": FP64, "mixed": MIXED}.get(precision, precision)
        self._check(lib().astg_solve_batch(self._h, n, rp.ctypes.data, c.ctypes.data, v.ctypes.data, nrhs,
                                           bb.ctypes.data, x.ctypes.data, rel_tol, max_iter, prec, st,
                                           ctypes.byref(wall), ctypes.byref(lanes)),
                    allow=(ASTG_NOT_CONVERGED,))
        return x, list(st), wall.value, lanes.value

    def extrapolate(self, field, sdf, valid_offset=0.0, max_distance_factor=4.0):
        """FmmLevelSetSolver3::extrapolate (include/jet/fmm_levelset_solver3.h:84-408) of "density"
        or "heat" in place; sdf is res^3 (index (z*res + y)*res + x).  Returns ExtrapStats."""
        g = np.ascontiguousarray(sdf, dtype=np.float64).ravel()
        res = round(len(g) ** (1.0 / 3.0))
        if res ** 3 != len(g):
            raise ValueError("sdf must hold res^3 values")
        st = ExtrapStats()
        self._check(lib().astg_extrapolate(self._h, field.encode(), g.ctypes.data, res, valid_offset,
                                           max_distance_factor, ctypes.byref(st)))
        return st

    def restart(self, directory, frame=0, layout=True):
        """OctreeOmniGridSolver3::restart from <directory>/layout.bin, tilt.bin, density.bin, heat.bin
        and velocity.bin (the reference's binary dumps)."""
        f = lambda n: os.path.join(directory, n).encode()
        self._check(lib().astg_restart(self._h, frame, f("layout.bin") if layout else None, f("boundary.bin"),
                                       f("tilt.bin"), f("density.bin"), f("heat.bin"), f("velocity.bin")))

    def save_checkpoint(self, directory):
        """The reference's binary dumps of the current state into <directory>."""
        f = lambda n: os.path.join(directory, n).encode()
        self._check(lib().astg_save_checkpoint(self._h, f("layout.bin"), f("tilt.bin"), f("density.bin"),
                                               f("heat.bin"), f("velocity.bin")))

    def max_velocity(self):
        v = ctypes.c_double()
        self._check(lib().astg_max_velocity(self._h, ctypes.byref(v)))
        return v.value


def mean_temperature_noalloc(d_heat_oct, level_slots, d_amb, stream=0):
    """astg_mean_temperature_noalloc: ambT of the heat at device address ``d_heat_oct`` into the
    double at device address ``d_amb``, queued on ``stream`` (a cudaStream_t as an int), with no
    allocation; ``level_slots`` gives the slots (cells + ghosts) of each level."""
    slots = np.ascontiguousarray(level_slots, dtype=np.int64)
    err = ctypes.create_string_buffer(256)
    st = lib().astg_mean_temperature_noalloc(d_heat_oct, slots.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                             len(slots), d_amb, stream or None, err, len(err))
    if st != ASTG_OK:
        raise AstgError(st, err.value.decode())


def _autograd_function():
    import torch

    class OctreeSmokeFunction(torch.autograd.Function):
        """A differentiable window of octree smoke steps on one OctreeSmoke3 (created with
        tilt_adaptivity=0, so the topology stays frozen over the window).

        OctreeSmokeFunction.apply(solver, steps, dt, checkpoint_every, mac, tilt_vel,
        source_density_oct, source_density_tilt) loads the velocity (MAC faces (3, S), tilted faces
        (S, 8)) and the per-slot source densities into the solver, runs `steps` steps with the tape
        on and returns the final octagon density (S,).  backward() runs the adjoint kernels
        (astg_backward) and returns the gradients of those four inputs; the density and heat of
        the starting state are the solver's own and receive none."""

        @staticmethod
        def forward(ctx, solver, steps, dt, checkpoint_every, mac, tilt_vel, src_oct, src_tilt):
            solver.set_tensor("mac", mac)
            solver.set_tensor("tilt_vel", tilt_vel)
            solver.set_tensor("source_density_oct", src_oct)
            solver.set_tensor("source_density_tilt", src_tilt)
            solver.tape_start(checkpoint_every)
            for _ in range(steps):
                solver.update(dt)
            ctx.solver = solver
            ctx.device = mac.device
            return solver.get_tensor("density_oct", mac.device)

        @staticmethod
        def backward(ctx, grad):
            s = ctx.solver
            s.adjoint_reset()
            s.set_tensor("adj_density_oct", grad)
            ctx.stats = s.backward()
            dev = ctx.device
            return (None, None, None, None, s.get_tensor("adj_mac", dev), s.get_tensor("adj_tilt_vel", dev),
                    s.get_tensor("adj_source_density_oct", dev), s.get_tensor("adj_source_density_tilt", dev))

    return OctreeSmokeFunction


def __getattr__(name):
    # torch is imported only when the autograd function is asked for
    if name == "OctreeSmokeFunction":
        fn = _autograd_function()
        globals()[name] = fn
        return fn
    raise AttributeError(name)


# ----------------------------------------------------------------------------------------------
# The reference module's uniform-grid surface (python_bindings/ast_solver.cc:14-80)

def _index(res, d, what):
    t = tuple(int(v) for v in np.asarray(res).ravel())
    if len(t) != d or min(t) < 1:
        raise ValueError(f"{what}: resolution must hold {d} positive integers")
    return t


class ASTGrid2:
    """ASTGrid<REAL, 2> (include/ast_grid.h:30); the module binds only dimension()."""

    def dimension(self):
        return 2


class ASTGrid3:
    """ASTGrid<REAL, 3>; the module binds only dimension()."""

    def dimension(self):
        return 3


class TiltNode2:
    """TiltNode<2> (include/ast_grid_layout.h:14-58): one tilted cell of a layout."""

    def __init__(self, is_open=False):
        self._open = bool(is_open)

    def open(self):
        return self._open


class TiltNode3(TiltNode2):
    """TiltNode<3>."""


class CellNode2:
    """CellNode<2> (include/ast_grid_layout.h:60-92); the module binds no members."""


class CellNode3:
    """CellNode<3>; the module binds no members."""


class ASTGridLayout2:
    """ASTGridLayout<2>(res, dx) (include/ast_grid_layout.h:134-140) with the bound read-only
    properties ``resolution`` and ``dx``.  Every tilt of a new layout is closed."""

    _d = 2

    def __init__(self, res, dx):
        self._res = _index(res, self._d, type(self).__name__)
        self._dx = float(dx)

    @property
    def resolution(self):
        return np.array(self._res, dtype=np.int32)

    @property
    def dx(self):
        return self._dx


class ASTGridLayout3(ASTGridLayout2):
    """ASTGridLayout<3>(res, dx)."""

    _d = 3


class ASTSolver2:
    """ASTSolver<2>(resolution, dx, adaptive_dofs, name) on the GPU (include/astg2d.h): the
    reference's uniform 2-D AST smoke solver.  ``initialize()``, ``update(dt)`` (Solver::update's CFL
    sub-stepping) and ``getDensity()`` (the cell densities, a copy) are the bound methods; the rest
    (``get``, ``set``, ``stage``, ``last_stats``) read and drive the state for checks."""

    FIELDS = {"density_cell", "heat_cell", "density_vert", "heat_vert", "mac_x", "mac_y", "tilt_vel", "dual_vert",
              "tilt_open", "pindex_cell", "pindex_vert", "A_rowptr", "A_col", "A_val", "b", "p", "sub_dt"}
    STAGES = {"source": 0, "force": 1, "project": 2, "advect": 3, "substep": 4}

    def __init__(self, resolution, dx, adaptive_dofs=True, name="ASTSolver", device=0):
        self.resolution = _index(resolution, 2, "ASTSolver2")
        self.dx = float(dx)
        self.adaptive_dofs = bool(adaptive_dofs)
        self.name = name
        self.device = device
        self._h = None
        self._lib = lib()

    def initialize(self):
        """ASTSolver::initialize (include/ast_solver.h:35-50): zero fields, boundary tilts fixed
        closed, cells numbered."""
        self.close()
        h = ctypes.c_void_p()
        nx, ny = self.resolution
        st = self._lib.astg2_create(nx, ny, self.dx, 1 if self.adaptive_dofs else 0, self.device, ctypes.byref(h))
        self._h = h
        if st != ASTG_OK:
            msg = self._lib.astg2_last_error(h).decode() if h.value else STATUS.get(st, "")
            self.close()
            raise AstgError(st, msg)

    def close(self):
        if self._h is not None and self._h.value:
            self._lib.astg2_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _handle(self):
        if self._h is None:  # Solver::update initialises on first use (src/solver.cpp:9-11)
            self.initialize()
        return self._h

    def _check(self, st):
        if st != ASTG_OK:
            raise AstgError(st, self._lib.astg2_last_error(self._h).decode())

    def update(self, dt):
        h = self._handle()
        _benchmark_timer.start_section("update")
        try:
            self._check(self._lib.astg2_update(h, float(dt)))
        finally:
            _benchmark_timer.stop_section("update")

    def stage(self, name, dt):
        self._check(self._lib.astg2_stage(self._handle(), self.STAGES[name], float(dt)))

    def getDensity(self):
        h = self._handle()
        n = self.resolution[0] * self.resolution[1]
        out = np.empty(n, dtype=np.float64)
        self._check(self._lib.astg2_get_density(h, out.ctypes.data, n))
        return out

    def _shape(self, name, n):
        nx, ny = self.resolution
        shapes = {"density_cell": (ny, nx), "heat_cell": (ny, nx), "pindex_cell": (ny, nx),
                  "density_vert": (ny + 1, nx + 1), "heat_vert": (ny + 1, nx + 1), "tilt_open": (ny + 1, nx + 1),
                  "pindex_vert": (ny + 1, nx + 1), "mac_x": (ny, nx + 1), "mac_y": (ny + 1, nx),
                  "tilt_vel": (ny + 1, nx + 1, 4), "dual_vert": (ny + 1, nx + 1, 2)}
        return shapes.get(name, (n,))

    def get(self, name):
        h = self._handle()
        kind = ctypes.c_int(0)
        n = self._lib.astg2_count(h, name.encode(), ctypes.byref(kind))
        if n < 0:
            raise KeyError(name)
        out = np.empty(n, dtype=[np.float64, np.uint8, np.int32][kind.value])
        self._check(self._lib.astg2_get(h, name.encode(), out.ctypes.data, n))
        return out.reshape(self._shape(name, n))

    def set(self, name, arr):
        h = self._handle()
        a = np.ascontiguousarray(arr, dtype=np.uint8 if name == "tilt_open" else np.float64).ravel()
        self._check(self._lib.astg2_set(h, name.encode(), a.ctypes.data, a.size))

    def set_solver_parameters(self, tol=1e-5, max_iter=5000, omega=0.97, min_diag=0.95, precision=FP64):
        self._check(self._lib.astg2_set_solver(self._handle(), tol, max_iter, omega, min_diag, precision))

    def last_stats(self):
        s = Stats2D()
        self._lib.astg2_last_stats(self._handle(), ctypes.byref(s))
        return {k: getattr(s, k) for k, _ in Stats2D._fields_}


class ASTSolver3:
    """ASTSolver<3>(resolution, dx, adaptive_dofs, name).  The reference's uniform 3-D AST path is
    unfinished (its 3-D scene and edge nodes are TODO, include/ast_solver.h:97-100, 207) and its
    update aborts on an Eigen bounds assertion in the second step once tilts open, so it is not
    built here: construction keeps the arguments, initialize() and update() raise.  The octree
    smoke solver (``OctreeSmoke3``) is the 3-D path."""

    def __init__(self, resolution, dx, adaptive_dofs=True, name="ASTSolver"):
        self.resolution = _index(resolution, 3, "ASTSolver3")
        self.dx = float(dx)
        self.adaptive_dofs = bool(adaptive_dofs)
        self.name = name

    def _refuse(self, *a):
        raise NotImplementedError("ASTSolver3: the reference's uniform 3-D AST solver is incomplete (its update "
                                  "aborts once tilts open); use OctreeSmoke3")

    initialize = update = getDensity = _refuse


class _BenchmarkTimer:
    """BenchmarkTimer (include/timer.h:67-235): named sections (nested as outer:inner) and timers
    within the innermost open section, each with its elapsed seconds and invocation count."""

    class _T:
        def __init__(self):
            self.running, self.time, self.invocations, self.t0 = False, 0.0, 0, 0.0
            self.start()

        def elapsed(self):
            return self.time + (time.perf_counter() - self.t0 if self.running else 0.0)

        def start(self):
            if self.running:
                print("ERROR: timer already running. Reported timings will be inaccurate.", file=sys.stderr)
                self.stop()
            self.running, self.t0 = True, time.perf_counter()
            self.invocations += 1

        def stop(self):
            if self.running:
                self.time += time.perf_counter() - self.t0
                self.running = False

    def __init__(self):
        self.reset()

    def reset(self):
        self.sections = {"": (self._T(), {})}
        self.stack = []

    @staticmethod
    def _display(name):
        levels = name.count(":")
        return name if levels == 0 else " " * (4 * levels) + name[name.rfind(":") + 1:]

    def start_section(self, name):
        if self.stack:
            name = self.stack[-1] + ":" + name
        self.stack.append(name)
        if name in self.sections:
            self.sections[name][0].start()
        else:
            self.sections[name] = (self._T(), {})

    def stop_section(self, name):
        if not self.stack:
            raise RuntimeError("benchmark_stop_timer_section: no open section")
        current = self.stack.pop()
        if self.stack:
            name = self.stack[-1] + ":" + name
        if name != current:
            print(f"ERROR: sections must be stopped in the reverse of the order they were started.\n"
                  f"(Expected {current}, but got {name})", file=sys.stderr)
        t, timers = self.sections[name]
        t.stop()
        for k, v in timers.items():
            if v.running:
                print(f"WARNING: stopping timer {k} implicitly in enclosing section's stop()", file=sys.stderr)
                v.stop()

    def _timer_name(self, name):
        section = self.stack[-1] if self.stack else ""
        return section, (section + ":" + name if section else name)

    def start_timer(self, name):
        section, full = self._timer_name(name)
        timers = self.sections[section][1]
        if full in timers:
            timers[full].start()
        else:
            timers[full] = self._T()

    def stop_timer(self, name):
        section, full = self._timer_name(name)
        self.sections[section][1][full].stop()

    def report(self, out=None):
        out = out or sys.stdout
        for name in sorted(self.sections):
            if name == "":
                continue
            t, timers = self.sections[name]
            print(f"{self._display(name)}\t{t.elapsed()}\t{t.invocations}", file=out)
            for k in sorted(timers):
                print(f"{self._display(k)}\t{timers[k].elapsed()}\t{timers[k].invocations}", file=out)
        t, timers = self.sections[""]
        for k in sorted(timers):
            print(f"{self._display(k)}\t{timers[k].elapsed()}\t{timers[k].invocations}", file=out)
        print(f"Full time\t{t.elapsed()}", file=out)


_benchmark_timer = _BenchmarkTimer()
_benchmark_messages = []


def benchmark_reset():
    _benchmark_timer.reset()


def benchmark_start_timer_section(name):
    _benchmark_timer.start_section(name)


def benchmark_stop_timer_section(name):
    _benchmark_timer.stop_section(name)


def benchmark_start_timer(name):
    _benchmark_timer.start_timer(name)


def benchmark_stop_timer(name):
    _benchmark_timer.stop_timer(name)


def benchmark_report(include_messages=False):
    if include_messages:
        for m in _benchmark_messages:
            print(m)
    _benchmark_timer.report()
