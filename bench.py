#!/usr/bin/env python3
"""Benchmark of the GB300 octree smoke step.

One "step" is one OctreeOmniGridSolver3 time step (source, buoyancy, projection with MIC(0)-PCG
to relative residual 1e-6, dual velocity, tilt adaptivity, RK2 semi-Lagrangian advection) of the
benchmark scene on the 256^3-equivalent octree (64^3 coarsest cells, 2 refinement levels), with
synthetic inputs (seeded curl-noise velocity, sphere source).  The state (~0.3 GB) is larger than
the 129 MB L2, so no flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line.  Under torchrun each rank runs an independent replica on its own GPU (the
step does not shard: MIC(0) sweeps are globally ordered); value = all ranks' steps / max time.
The reference arm times the CPU restatement of the reference algorithm (oracle/, OpenMP over the
host cores, bit-identical results) on the same workload.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "ast-grid_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

COARSEST, LEVELS, DT = 64, 3, 0.01
WORKLOAD = "octree smoke step, 64^3 coarsest x 3 levels (256^3-eq.), FP64 MIC(0)-PCG to rel. res. 1e-6"
METRIC = "smoke steps/s"


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    """Host-side barrier and max over ranks (gloo); no collective touches the step's data."""

    def __init__(self, ws):
        self.ws = ws
        if ws > 1:
            import torch.distributed as dist

            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.ws > 1:
            self.dist.barrier()

    def max(self, v):
        if self.ws == 1:
            return v
        import torch

        t = torch.tensor([float(v)], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def sum(self, v):
        if self.ws == 1:
            return v
        import torch

        t = torch.tensor([float(v)], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.ws > 1:
            self.dist.destroy_process_group()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while running."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            for ln in open(self.path):
                f = [x.strip() for x in ln.split(",")]
                if len(f) >= 9 and f[1].replace(".", "").isdigit():
                    rows.append(f)
        finally:
            if self.path and os.path.exists(self.path):
                os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": float(rows[0][2]), "reasons": reasons,
                "samples": len(rows), "power_w_max": max(float(r[3]) for r in rows if r[3].replace(".", "").isdigit())}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def committed_traffic():
    """Per-row DRAM bytes of the dominant kernel from the committed ncu summary (or None)."""
    path = os.path.join(ROOT, "profiles", "roofline_traffic.txt")
    out = {}
    try:
        for ln in open(path):
            if ":" in ln and not ln.lstrip().startswith("#"):
                k, v = ln.split(":", 1)
                try:
                    out[k.strip()] = float(v.split()[0])
                except (ValueError, IndexError):
                    pass
    except OSError:
        pass
    return out


def cpu_baseline_sample(steps):
    """The CPU restatement of the reference's step (oracle, OpenMP) on the same workload."""
    from oracle.oracle import Oracle

    o = Oracle(COARSEST, LEVELS, openmp=True)
    t0 = time.perf_counter()
    for _ in range(steps):
        o.step(DT)
    el = time.perf_counter() - t0
    o.close()
    threads = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return {"value": steps / el, "unit": "steps/s", "cores": threads, "kind": "port",
            "sample": f"{steps} steps of the same scene from t=0 (oracle/smoke_oracle.cpp, OpenMP, "
                      f"bit-identical to the reference's CPU algorithm), {el:.1f} s",
            "sample_short": f"{steps} steps from t=0, OpenMP oracle port, {el:.1f} s"}


def isolated_solves(args, device):
    """Isolated pressure solves: the octree and tilt state frozen after `solve_steps` steps of the
    scene; each right-hand side is the AST divergence (the projection's own assembly) of face and
    tilted-face velocities drawn i.i.d. N(0,1) with a fixed seed, smoothed by 3 weighted Jacobi
    passes (omega 2/3 on A, include/pcgsolver/pcg_solver.h:276-300), then solved to |r| <= 1e-6 |b|
    in FP64 and in mixed precision.  ms excludes the MIC(0) factorisation."""
    import numpy as np

    import ast_solver

    s = ast_solver.OctreeSmoke3(COARSEST, LEVELS, device=device)
    for _ in range(args.solve_steps):
        s.update(DT)
    fields = ["density_oct", "density_tilt", "heat_oct", "heat_tilt", "mac", "tilt_vel", "dual_oct", "dual_tilt",
              "tilt_e", "tilt_flags"]
    snap = {k: s.get(k) for k in fields + ["t_" + k for k in fields] + ["tilt_open"]}
    S = s.slots
    out = {"fp64": [], "mixed": []}
    rhs, sols = [], {"fp64": [], "mixed": []}
    A = None
    for k in range(args.solve_rhs):
        rng = np.random.default_rng(1 + k)
        s.set("mac", rng.standard_normal(3 * S))
        s.set("tilt_vel", rng.standard_normal(8 * S))
        s.stage(3, DT)  # assembles A and b = div(u) for the frozen state
        b = s.get("b")
        if A is None:
            A = (s.get("A_rowptr"), s.get("A_col"), s.get("A_val"))
        for kk, v in snap.items():
            s.set(kk, v)
        rp, col, val = A
        n = len(rp) - 1
        diag = np.zeros(n)
        rows = np.repeat(np.arange(n), np.diff(rp))
        on = col == rows
        diag[rows[on]] = val[on]
        for _ in range(3):
            ax = np.add.reduceat(val * b[col], rp[:-1])
            b = (1 - 2 / 3.0) * b + (2 / 3.0) * (0.0 - (ax - diag * b)) / diag
        rhs.append(b)
        for prec in ("fp64", "mixed"):
            x, st = s.solve(rp, col, val, b, rel_tol=1e-6, precision=prec)
            out[prec].append((st.ms, st.iterations, st.outer, st.converged))
            sols[prec].append(x)
    rp, col, val = A
    n, nnz = len(rp) - 1, len(col)
    nnzL = (nnz - n) / 2
    res = {"config": f"{args.solve_rhs} right-hand sides on the octree frozen after {args.solve_steps} steps, "
                     "div of N(0,1) faces smoothed by 3 weighted Jacobi passes, rel. residual 1e-6",
           "n": n, "nnz": nnz}
    for prec, rows_ in out.items():
        ms = float(np.mean([r[0] for r in rows_]))
        it = float(np.mean([r[1] for r in rows_]))
        outer = float(np.mean([r[2] for r in rows_]))
        if prec == "fp64":
            bytes_ = it * (12 * nnz + 24 * nnzL + 180 * n)
        else:
            bytes_ = it * (8 * nnz + 16 * nnzL + 96 * n) + outer * (12 * nnz + 28 * n)
        res[prec] = {"ms_per_solve": ms, "iterations_mean": it, "outer_cycles_mean": outer,
                     "all_converged": all(r[3] == 1 for r in rows_), "algorithmic_GBps": bytes_ / (ms / 1e3) / 1e9}
    res["mixed_speedup"] = res["fp64"]["ms_per_solve"] / res["mixed"]["ms_per_solve"]
    # the same right-hand sides through astg_solve_batch: the solves side by side, one preconditioner
    # cluster each (host wall time of the whole call per right-hand side, factorisation and copies
    # included); the solutions must equal the one-by-one ones bit for bit
    if rhs:
        B = np.stack(rhs)
        for prec in ("fp64", "mixed"):
            s.solve_batch(rp, col, val, B[:2], rel_tol=1e-6, precision=prec)  # lanes allocated, warm
            X, stb, wall, lanes = s.solve_batch(rp, col, val, B, rel_tol=1e-6, precision=prec)
            same = all(np.array_equal(X[i], sols[prec][i]) for i in range(len(rhs)))
            res[prec]["batch"] = {"ms_per_solve": wall / len(rhs), "lanes": lanes, "identical": bool(same),
                                  "all_converged": all(st.converged == 1 for st in stb)}
    s.close()
    return res


def precision_comparison(args, device):
    """The mixed form against the FP64 form on the benchmark scene (200 steps by default, the length
    of the three-way comparison; the FP64 form is bit-identical to the FP64 oracle, so its numbers
    are also the mixed form's errors against the oracle): two handles from the same initial state
    step side by side; per step the relative L2 difference of the octagon density and of the
    pressure, and each form's final relative residual |b - A p|_inf / |b|_inf of its solve (both
    stop at 1e-6): b - A p is the projected velocity's discrete divergence (times rho / dt), so this
    is the divergence left after the projection relative to the divergence before it."""
    import numpy as np

    import ast_solver

    a = ast_solver.OctreeSmoke3(COARSEST, LEVELS, device=device)
    b = ast_solver.OctreeSmoke3(COARSEST, LEVELS, device=device, precision="mixed")
    dens, pres, ra, rb = [], [], [], []
    for _ in range(args.compare_steps):
        a.update(DT)
        b.update(DT)
        da, db = a.get("density_oct"), b.get("density_oct")
        pa, pb = a.get("p"), b.get("p")
        dens.append(float(np.linalg.norm(db - da) / max(np.linalg.norm(da), 1e-300)))
        pres.append(float(np.linalg.norm(pb - pa) / max(np.linalg.norm(pa), 1e-300)) if len(pa) == len(pb) else None)
        for h, out in ((a, ra), (b, rb)):
            st = h.last_step.solve
            out.append(st.residual / (st.tolerance / 1e-6) if st.tolerance > 0 else 0.0)
    a.close()
    b.close()
    pick = lambda v: {"step1": v[0], "max": max(x for x in v if x is not None), "last": v[-1]}
    return {"config": f"{args.compare_steps} steps of the benchmark scene from the same initial state, FP64 form vs "
                      "mixed form (separate handles)",
            "density_rel_l2_mixed_vs_fp64": pick(dens), "pressure_rel_l2_mixed_vs_fp64": pick(pres),
            "rel_residual_fp64": pick(ra), "rel_residual_mixed": pick(rb),
            "per_step_density": dens, "per_step_pressure": pres, "per_step_divergence_fp64": ra,
            "per_step_divergence_mixed": rb}


def ensemble(args, device):
    """Independent simulations side by side on one GPU: one handle per host thread, each with its
    own stream (the library's calls release the GIL), all stepping the benchmark scene.  One
    simulation keeps a single 16-SM cluster busy in its preconditioner for most of a step, so
    several take little longer than one.  Reports the aggregate steps/s of K simulations and checks
    one member bit for bit against a simulation stepped alone."""
    import threading

    import numpy as np
    import torch

    import ast_solver

    K, M = args.ensemble, args.ensemble_steps
    hs = [ast_solver.OctreeSmoke3(COARSEST, LEVELS, device=device) for _ in range(K)]
    for h in hs:
        for _ in range(3):
            h.update(DT)
    errs = []

    def run(h):
        try:
            for _ in range(M):
                h.update(DT)
        except Exception as e:  # surfaced after the join
            errs.append(e)

    th = [threading.Thread(target=run, args=(h,)) for h in hs]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for t in th:
        t.start()
    for t in th:
        t.join()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    if errs:
        raise errs[0]
    alone = ast_solver.OctreeSmoke3(COARSEST, LEVELS, device=device)
    for _ in range(3 + M):
        alone.update(DT)
    same = all(np.array_equal(alone.get(f), hs[0].get(f)) for f in ("density_oct", "mac", "p"))
    alone.close()
    for h in hs:
        h.close()
    return {"simulations": K, "steps_each": M, "wall_s": wall, "aggregate_steps_per_s": K * M / wall,
            "steps_per_s_each": M / wall, "member_identical_to_alone": bool(same),
            "note": "one handle per host thread, FP64, the benchmark scene; wall time of the K x M steps"}


def adjoint_window(args, device):
    """Reverse mode at scale: 64^3 coarsest cells, 2 levels (128^3-equivalent), tilts opened by 4
    adaptive steps and then frozen, `adjoint_steps` steps taped with a checkpoint every
    `adjoint_every` steps (the others recomputed during the reverse pass).  Loss = ||density - g||_2
    over the octagon cells (volume-weighted; g a Gaussian blob at (0.5, 0.5, 0.6) z-up, sigma 0.1,
    peak 1); gradients with respect to the initial face velocities and the per-slot source densities.
    Run in the mixed form (FP32 inner PCG in both the forward and the adjoint solves) and in FP64 on
    the same window; the FP64 gradient is the reference for the mixed one.  Times are device times:
    forward = the taped steps (checkpoint copies included), backward = astg_backward."""
    import numpy as np
    import torch

    import ast_solver

    free0 = torch.cuda.mem_get_info(device)[0]
    s = ast_solver.OctreeSmoke3(64, 2, device=device)
    for _ in range(4):
        s.update(DT)
    s.set_tilt_adaptivity(False)
    names = ["density_oct", "density_tilt", "heat_oct", "heat_tilt", "mac", "tilt_vel", "dual_oct", "dual_tilt"]
    X = {k: s.get(k) for k in names}
    Pt = {k: s.get("t_" + k) for k in names}
    coords, sizes = s.get("slot_coords"), s.get("level_sizes")
    lev = np.repeat(np.arange(len(sizes)), sizes[:, 2])
    res0 = s.size(2)
    h = (1.0 / res0) * (2.0 ** lev)
    cells = ((coords[:, 3] & 2) == 0) & np.all(coords[:, :3] < ((res0 >> lev) - 1)[:, None], axis=1)
    centre = (coords[:, :3] + 0.5) * h[:, None]
    g = np.exp(-((centre - np.array([0.5, 0.5, 0.6])) ** 2).sum(1) / (2 * 0.1 ** 2))
    w = np.where(cells, h ** 3, 0.0)
    peak_used = 0

    def run(prec):
        nonlocal peak_used
        for k, v in X.items():
            s.set(k, v)
        for k, v in Pt.items():
            s.set("t_" + k, v)
        s.set_precision(prec)
        s.tape_start(args.adjoint_every)
        fwd = 0.0
        for _ in range(args.adjoint_steps):
            s.update(DT)
            fwd += s.last_step.ms_total
        r = s.get("density_oct") - g
        loss = float(np.sqrt((w * r * r).sum()))
        s.adjoint_reset()
        s.set("adj_density_oct", w * r / loss)
        st = s.backward()
        peak_used = max(peak_used, free0 - torch.cuda.mem_get_info(device)[0])
        grads = [s.get("adj_mac"), s.get("adj_tilt_vel"), s.get("adj_source_density_oct"),
                 s.get("adj_source_density_tilt")]
        s.tape_stop()
        return {"loss": loss, "forward_ms": fwd, "backward_ms": st.ms, "recompute_ms": st.ms_recompute,
                "ratio": st.ms / fwd, "adjoint_pcg_iters_mean": st.pcg_iterations / max(st.solves, 1),
                "checkpoints": st.checkpoints, "recomputed_steps": st.recomputed_steps,
                "tape_bytes": st.tape_bytes}, grads

    mixed, gm = run("mixed")
    fp64, g64 = run("fp64")
    num = np.sqrt(sum(((a - b) ** 2).sum() for a, b in zip(gm, g64)))
    den = np.sqrt(sum((b * b).sum() for b in g64))
    out = {"config": f"64^3 coarsest x 2 levels (128^3-equivalent), {args.adjoint_steps} steps, checkpoint "
                     f"every {args.adjoint_every} with recompute, topology frozen after 4 adaptive steps; "
                     "loss ||density - g||_2; gradients w.r.t. initial faces and source densities",
           "slots": s.slots, "mixed": mixed, "fp64": fp64,
           "adjoint_fwd_cost_ratio": mixed["ratio"],
           "grad_rel_error_mixed_vs_fp64": float(num / den),
           "peak_device_bytes": int(peak_used),
           "fields": "FP64 fields; the mixed form runs the forward and adjoint PCG with FP32 inner iterations"}
    s.close()
    return out


def uniform2d(args, device):
    """The uniform 2-D AST solver (ASTSolver2) on the reference example's configuration
    (example/ast_smoke_2d/main.cpp: 192 x 384, dt = 0.025f, adaptive tilts): frames per second after
    a warm-up, device time (CUDA events around each update) and end to end (update plus the
    getDensity copy to the host), beside the 2-D oracle port on one host core over a short sample
    of the same frames."""
    import numpy as np

    import ast_solver
    from oracle.oracle import Oracle2D

    nx, ny, dt = 192, 384, 0.02500000037252903
    s = ast_solver.ASTSolver2(resolution=[nx, ny], dx=1.0 / nx, adaptive_dofs=True, name="bench2d", device=device)
    s.initialize()
    for _ in range(args.warmup2d):
        s.update(dt)
    dev_ms, wall_ms, subs, iters, unknowns = [], [], [], [], []
    for _ in range(args.frames2d):
        w0 = time.perf_counter()
        s.update(dt)
        d = s.getDensity()
        wall_ms.append(1e3 * (time.perf_counter() - w0))
        st = s.last_stats()
        dev_ms.append(st["ms"])
        subs.append(st["substeps"])
        iters.append(st["pcg_iterations"])
        unknowns.append(st["unknowns"])
    s.close()
    out = {"workload": f"ASTSolver2 {nx}x{ny}, dt 0.025f, adaptive tilts, frames {args.warmup2d + 1}.."
                       f"{args.warmup2d + args.frames2d}",
           "value": 1e3 / float(np.mean(dev_ms)), "unit": "frames/s", "ms_per_frame": float(np.mean(dev_ms)),
           "e2e": {"value": 1e3 / float(np.mean(wall_ms)), "unit": "frames/s", "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 8 * nx * ny},
           "substeps_mean": float(np.mean(subs)), "unknowns_mean": float(np.mean(unknowns)),
           "pcg_iters_last_substep_mean": float(np.mean(iters)), "density_sum": float(d.sum())}
    if args.cpu_frames2d > 0:
        o = Oracle2D(nx, ny, adaptive=True, reduce_mode=0)
        for _ in range(args.warmup2d):
            o.update(dt)
        c0 = time.perf_counter()
        for _ in range(args.cpu_frames2d):
            o.update(dt)
        cpu_s = (time.perf_counter() - c0) / args.cpu_frames2d
        o.close()
        out["cpu_baseline"] = {"value": 1.0 / cpu_s, "unit": "frames/s", "cores": 1, "kind": "port",
                               "sample": f"{args.cpu_frames2d} frames after the same {args.warmup2d}-frame warm-up, "
                                         "2-D oracle in the reference's arithmetic order"}
    return out


def run_reference(args):
    ws, rank, _ = dist_info()
    if ws > 1 and rank != 0:
        return 0
    from oracle.oracle import Oracle

    o = Oracle(COARSEST, LEVELS, openmp=True)
    for _ in range(args.warmup):
        o.step(DT)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        o.step(DT)
    el = time.perf_counter() - t0
    v = args.steps / el
    threads = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "steps/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "coarsest": COARSEST, "levels": LEVELS, "dt": DT,
                       "l2": "state larger than L2"},
            "cpu_baseline": {"value": v, "unit": "steps/s", "cores": threads, "kind": "port",
                             "sample": f"steps {args.warmup + 1}..{args.warmup + args.steps} of the scene on the host "
                                       f"cores (oracle/smoke_oracle.cpp, OpenMP)"},
            "e2e": {"value": v, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args):
    import numpy as np
    import torch

    import ast_solver

    ws, rank, local = dist_info()
    torch.cuda.set_device(local)
    D = Dist(ws)
    s = ast_solver.OctreeSmoke3(COARSEST, LEVELS, device=local)
    S = s.slots
    for _ in range(args.warmup):
        s.update(DT)
    torch.cuda.synchronize()
    D.barrier()

    # ---------------- device-resident timed region
    s.set_profiling(True)
    l0 = s.launches
    dev_ms = []
    iters = []
    pcg_ms = []
    dofs = []
    nnzs = []
    adv_ms = []
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        D.barrier()
        w0 = time.perf_counter()
        for _ in range(args.steps):
            s.update(DT)
            st = s.last_step
            dev_ms.append(st.ms_total)
            adv_ms.append(st.ms_advect)
            iters.append(st.solve.iterations)
            pcg_ms.append(st.solve.ms)
            dofs.append(st.solve.n)
            nnzs.append(st.solve.nnz)
        torch.cuda.synchronize()
        wall = time.perf_counter() - w0
    clocks = clk.summary()
    launches = s.launches - l0
    kms = s.kernel_ms()
    s.set_profiling(False)
    t_dev = sum(dev_ms) / 1e3
    t_max = D.max(max(t_dev, 1e-9))
    total_steps = D.sum(args.steps)
    value = total_steps / t_max

    # ---------------- the mixed-precision form on the same handle (FP32 inner PCG in FP64 defect
    # correction, same stopping test), after its own warm-up
    s.set_precision("mixed")
    for _ in range(max(args.warmup, 1)):
        s.update(DT)
    torch.cuda.synchronize()
    mixed_ms, mixed_pcg, mixed_it, mixed_outer, mixed_conv = [], [], [], [], []
    for _ in range(args.steps):
        s.update(DT)
        st = s.last_step
        mixed_ms.append(st.ms_total)
        mixed_pcg.append(st.solve.ms)
        mixed_it.append(st.solve.iterations)
        mixed_outer.append(st.solve.outer)
        mixed_conv.append(st.solve.converged)
    torch.cuda.synchronize()
    t_mixed = D.max(sum(mixed_ms) / 1e3)
    mixed = {"value": D.sum(args.steps) / t_mixed, "unit": "steps/s", "ms_per_step": 1e3 * t_mixed / args.steps,
             "pcg_ms_per_solve": float(np.mean(mixed_pcg)), "pcg_inner_iters_mean": float(np.mean(mixed_it)),
             "outer_cycles_mean": float(np.mean(mixed_outer)), "all_converged": bool(min(mixed_conv) == 1),
             "dtype": "f32 inner / f64 outer", "stopping_test": "|b - A x|_inf <= 1e-6 |b|_inf in FP64"}
    s.set_precision("fp64")

    # ---------------- end to end through the C ABI with pinned host buffers, on a second handle
    # with the same warm-up, so that it covers the same steps of the simulation as `value`
    s.close()
    s = ast_solver.OctreeSmoke3(COARSEST, LEVELS, device=local)
    for _ in range(args.warmup):
        s.update(DT)
    names_sync = ["density_oct", "density_tilt", "heat_oct", "heat_tilt"]
    host = {n: torch.empty(S, dtype=torch.float64, pin_memory=True) for n in names_sync}
    out = torch.empty(S, dtype=torch.float64, pin_memory=True)
    lib = ast_solver.lib()
    h2d = 8 * S * len(names_sync)
    d2h = 8 * S * len(names_sync) + 8 * S

    def e2e_step():
        # state to the host before the scene callback and back after it (the drop-in contract of
        # sceneSetup), one step, then the frame's density to the host
        for n in names_sync:
            s._check(lib.astg_get(s._h, n.encode(), host[n].data_ptr(), 8 * S, None))
        for n in names_sync:
            s._check(lib.astg_set(s._h, n.encode(), host[n].data_ptr(), 8 * S))
        s.update(DT)
        s._check(lib.astg_get(s._h, b"density_oct", out.data_ptr(), 8 * S, None))

    e2e_steps = max(1, min(args.steps, args.e2e_steps))
    torch.cuda.synchronize()
    D.barrier()
    e0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    torch.cuda.synchronize()
    e_el = D.max(time.perf_counter() - e0)
    e2e = {"value": D.sum(e2e_steps) / e_el, "unit": "steps/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
           "steps": e2e_steps}

    # ---------------- roofline of the dominant kernel
    peak, peak_kind = measured_peaks()
    # preconditioner form: > 100 = both sweeps fused in one cluster launch (timed as "sweep_fwd"),
    # > 200 its barrier-free variant
    form = s.size(7)
    fused = form > 100
    fused_name = "k_precond_async" if form > 200 else "k_precond_dsmem"
    names = {"sweep_fwd": fused_name if fused else "k_sweep_fwd", "sweep_bwd": "k_sweep_bwd",
             "spmv_dot": "k_spmv_dot", "mic_factor": "k_mic_factor"}
    # kernel times come from CUDA event pairs: every direct launch, and one PCG batch in four of
    # the graph replays; rank kernels by their average launch time x launches per step
    iters_per_step = float(np.mean(iters))
    per_step = {"sweep_fwd": iters_per_step + 1, "sweep_bwd": iters_per_step + 1, "spmv_dot": iters_per_step,
                "mic_factor": 1.0}
    avg = {k: v[0] / v[1] for k, v in kms.items() if v[1] > 0}
    top = max(avg, key=lambda k: avg[k] * per_step[k])
    n_mean = float(np.mean(dofs))
    nnz_mean = float(np.mean(nnzs))
    nnzL = (nnz_mean - n_mean) / 2  # strictly lower entries of the symmetric matrix
    sweep = 12 * nnzL + 28 * n_mean  # one triangular sweep: L values + columns, r, z, pivot, row bounds
    alg = {"sweep_fwd": 2 * sweep if fused else sweep, "sweep_bwd": sweep,
           "spmv_dot": 12 * nnz_mean + 4 * (n_mean + 1) + 16 * n_mean + 16 * n_mean,
           "mic_factor": 12 * nnz_mean + 12 * nnzL}[top]
    avg_ms = kms[top][0] / max(kms[top][1], 1)
    achieved = alg / (avg_ms / 1e3) / 1e9
    tr = committed_traffic()
    traffic = None
    if f"{names[top]}_bytes_per_row" in tr:
        traffic = tr[f"{names[top]}_bytes_per_row"] * n_mean
    roofline = {"bound": "hbm", "kernel": names[top], "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": peak_kind, "traffic": traffic,
                "algorithmic_bytes_per_launch": alg, "avg_launch_ms": avg_ms, "timed_launches": kms[top][1],
                "note": "MIC(0) sweeps are bounded by the dependency chain (wavefront latency), not HBM",
                "preconditioner_form": form}
    kernel_breakdown = {names[k]: {"avg_launch_ms": avg[k], "timed_launches": kms[k][1],
                                   "est_ms_per_step": avg[k] * per_step[k]} for k in avg}
    # advection stage (tilt adaptivity, scalars, faces, tilts, half tilts, decay) against its
    # compulsory traffic: 176 B read + 120 B written per slot (no SDF grid: the scene has no collider)
    adv_bytes = 296.0 * S
    adv_mean = float(np.mean(adv_ms))
    advection = {"algorithmic_bytes_per_step": adv_bytes, "ms_per_step": adv_mean,
                 "achieved_GBps": adv_bytes / (adv_mean / 1e3) / 1e9 if adv_mean > 0 else None,
                 "frac": (adv_bytes / (adv_mean / 1e3) / 1e9) / peak if adv_mean > 0 else None,
                 "note": "gather- and FP64-latency-bound sampling (2 RK2 velocity samples per advected point)"}

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline_sample(args.cpu_steps)
    solves = None
    if rank == 0 and args.solve_rhs > 0:
        solves = isolated_solves(args, local)
    adjoint = None
    if rank == 0 and args.adjoint_steps > 0:
        adjoint = adjoint_window(args, local)
    comparison = None
    if rank == 0 and args.compare_steps > 0:
        comparison = precision_comparison(args, local)
    flat2d = None
    if rank == 0 and args.frames2d > 0:
        flat2d = uniform2d(args, local)
    ens = None
    if rank == 0 and args.ensemble > 0:
        ens = ensemble(args, local)

    full = {"metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "coarsest": COARSEST, "levels": LEVELS, "dt": DT,
                       "dofs_mean": n_mean, "nnz_mean": nnz_mean, "slots": S, "precision": "fp64",
                       "l2": "state larger than L2 (no flush)", "parallelism": f"replicas x{ws}"},
            "pcg_ms_per_solve": float(np.mean(pcg_ms)), "pcg_iters_mean": float(np.mean(iters)), "mixed": mixed,
            "wall_ms_per_step": 1e3 * wall / args.steps,
            "roofline": roofline, "kernels": kernel_breakdown, "advection": advection, "cpu_baseline": cpu, "e2e": e2e,
            "clocks": clocks, "gpu_launches": launches, "isolated_solves": solves, "adjoint": adjoint,
            "precision_comparison": comparison, "uniform2d": flat2d, "ensemble": ens}
    s.close()
    D.barrier()
    if rank == 0:
        emit(full, args.detail_out)
    D.close()
    return 0


LINE_LIMIT = 1400  # characters of the printed line: harnesses that keep only the tail of stdout must see all of it


def _r(x, sig=5):
    """A float rounded to `sig` significant digits (the printed line stays short); other values as given."""
    if isinstance(x, float):
        return float(f"{x:.{sig}g}")
    return x


def _pick(d, keys, sig=5):
    return None if d is None else {k: _r(d.get(k), sig) for k in keys if k in d}


def compact_line(full, detail_path):
    """The one printed JSON line: the contract's keys first (value, unit, config, roofline, cpu_baseline,
    e2e, clocks, gpu_launches), then one-number summaries of the other sections.  Everything else of
    `full` (per-kernel times, per-step series of the FP64/mixed comparison, the adjoint and 2-D
    sections in full) goes to the side file `detail_path`."""
    cfg = full["config"]
    line = {k: _r(full[k]) for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                                     "higher_is_better", "scaling", "vs_baseline", "dtype", "data")}
    line["config"] = {"workload": cfg["workload"], "coarsest": cfg["coarsest"], "levels": cfg["levels"],
                      "dt": cfg["dt"], "dofs": _r(cfg["dofs_mean"], 6), "l2": "state>L2", "parallelism": cfg["parallelism"]}
    line["roofline"] = _pick(full["roofline"], ("bound", "kernel", "achieved", "peak", "unit", "frac", "traffic"), 4)
    line["roofline"]["alg_bytes"] = _r(full["roofline"]["algorithmic_bytes_per_launch"], 4)
    cb = full.get("cpu_baseline")
    line["cpu_baseline"] = None if cb is None else {"value": _r(cb["value"]), "unit": cb["unit"], "cores": cb["cores"],
                                                    "kind": cb["kind"], "sample": cb.get("sample_short", cb["sample"])}
    line["e2e"] = _pick(full["e2e"], ("value", "unit", "h2d_bytes_per_step", "d2h_bytes_per_step"))
    line["clocks"] = _pick(full["clocks"], ("sm_mhz", "sm_max_mhz", "reasons"))
    line["gpu_launches"] = full["gpu_launches"]
    line["pcg_ms_per_solve"] = _r(full["pcg_ms_per_solve"], 4)
    line["pcg_iters"] = _r(full["pcg_iters_mean"], 4)
    m = full.get("mixed")
    if m:
        line["mixed"] = {"value": _r(m["value"]), "ms_per_step": _r(m["ms_per_step"], 4),
                         "pcg_ms_per_solve": _r(m["pcg_ms_per_solve"], 4), "converged": m["all_converged"]}
    adv = full.get("advection")
    if adv:
        line["advection_ms"] = _r(adv["ms_per_step"], 4)
    iso = full.get("isolated_solves")
    if iso:
        # iteration counts and the mixed / FP64 ratio are in the detail file
        line["solves"] = {"fp64_ms": _r(iso["fp64"]["ms_per_solve"], 4), "mixed_ms": _r(iso["mixed"]["ms_per_solve"], 4)}
        if "batch" in iso["fp64"]:  # side by side (astg_solve_batch), per right-hand side
            line["solves"]["batch_fp64_ms"] = _r(iso["fp64"]["batch"]["ms_per_solve"], 4)
            line["solves"]["batch_mixed_ms"] = _r(iso["mixed"]["batch"]["ms_per_solve"], 4)
            line["solves"]["lanes"] = iso["fp64"]["batch"]["lanes"]
    ens = full.get("ensemble")
    if ens:
        line["ensemble"] = {"sims": ens["simulations"], "steps_s": _r(ens["aggregate_steps_per_s"], 4),
                            "same": ens["member_identical_to_alone"]}
    adj = full.get("adjoint")
    if adj:
        line["adjoint"] = {"ratio": _r(adj["adjoint_fwd_cost_ratio"], 3),
                           "grad_err_mixed": _r(adj["grad_rel_error_mixed_vs_fp64"], 3),
                           "peak_gb": _r(adj["peak_device_bytes"] / 1e9, 3)}
    pc = full.get("precision_comparison")
    if pc:
        line["compare"] = {"dens_max": _r(pc["density_rel_l2_mixed_vs_fp64"]["max"], 3),
                           "res_mixed": _r(pc["rel_residual_mixed"]["max"], 3),
                           "res_fp64": _r(pc["rel_residual_fp64"]["max"], 3)}
    u2 = full.get("uniform2d")
    if u2:
        line["uniform2d_fps"] = _r(u2["value"], 4)
    if detail_path:
        rel = os.path.relpath(os.path.abspath(detail_path), ROOT)
        line["detail"] = os.path.basename(detail_path) if rel.startswith("..") else rel  # outside the repo: the name
    return line


def emit(full, detail_path):
    """Writes `full` to the side file and prints the compact contract line as the last line of stdout."""
    if detail_path:
        try:
            os.makedirs(os.path.dirname(os.path.abspath(detail_path)), exist_ok=True)
            with open(detail_path, "w") as f:
                json.dump(full, f, indent=1)
        except OSError as e:
            print(f"warning: detail file not written ({e})", file=sys.stderr)
            detail_path = None
    s = json.dumps(compact_line(full, detail_path), separators=(",", ":"))
    if len(s) > LINE_LIMIT:
        print(f"warning: contract line is {len(s)} characters", file=sys.stderr)
    print(s, flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-steps", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=20, help="steps of the end-to-end loop (at most --steps)")
    ap.add_argument("--solve-steps", type=int, default=100, help="steps before the isolated solves")
    ap.add_argument("--solve-rhs", type=int, default=20, help="right-hand sides of the isolated solves (0: skip)")
    ap.add_argument("--adjoint-steps", type=int, default=128, help="steps of the differentiated window (0: skip)")
    ap.add_argument("--adjoint-every", type=int, default=16, help="checkpoint interval of the adjoint tape")
    ap.add_argument("--compare-steps", type=int, default=200, help="steps of the FP64 / mixed comparison (0: skip)")
    ap.add_argument("--frames2d", type=int, default=20, help="timed frames of the uniform 2-D solver (0: skip)")
    ap.add_argument("--warmup2d", type=int, default=10, help="warm-up frames of the uniform 2-D solver")
    ap.add_argument("--cpu-frames2d", type=int, default=2, help="frames of the 2-D oracle CPU sample (0: skip)")
    ap.add_argument("--only-2d", action="store_true", help="run only the uniform 2-D solver section and print it")
    ap.add_argument("--ensemble", type=int, default=7, help="simulations stepped side by side (0: skip)")
    ap.add_argument("--ensemble-steps", type=int, default=10, help="timed steps of each ensemble member")
    ap.add_argument("--detail-out", default=os.path.join(ROOT, "_build", "bench_detail.json"),
                    help="side file for the sections left out of the printed line ('' to skip)")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        print("warning: fewer than 3 warm-up steps", file=sys.stderr)
    if args.impl == "reference":
        return run_reference(args)
    if args.only_2d:
        print(json.dumps({"uniform2d": uniform2d(args, 0)}), flush=True)
        return 0
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
