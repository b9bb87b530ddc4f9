"""bench.py's JSON-line contract on the CPU: the reference arm (the oracle port of the reference's
step on the host cores) prints one line with the keys the harness reads, for one step."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 1 and line["steps"] == 1
    for k in ("metric", "value", "unit", "ms_per_step", "higher_is_better", "scaling", "dtype", "data", "config"):
        assert k in line, k
    assert line["value"] > 0 and line["unit"] == "steps/s" and line["higher_is_better"] is True
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": "steps/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert line["config"]["coarsest"] == 64 and line["config"]["levels"] == 3


def _fake_full():
    """A result dict of the GPU arm's shape at the default section sizes (200-step comparison series,
    20 right-hand sides, the adjoint and 2-D sections), with full-precision floats."""
    import math

    f = lambda i: math.pi * 1e-7 * (1 + i / 7.0)  # noqa: E731
    series = [f(i) for i in range(200)]
    pick = {"step1": f(1), "max": f(3), "last": f(5)}
    return {"metric": "smoke steps/s", "value": 11.123456789012345, "unit": "steps/s", "n_gpus": 1, "steps": 20,
            "warmup": 5, "ms_per_step": 89.90123456789012, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "octree smoke step, 64^3 coarsest x 3 levels (256^3-equivalent), FP64 MIC(0)-PCG "
                                   "to rel. residual 1e-6", "coarsest": 64, "levels": 3, "dt": 0.01,
                       "dofs_mean": 307823.45, "nnz_mean": 2351213.5, "slots": 374123, "precision": "fp64",
                       "l2": "state larger than L2 (no flush)", "parallelism": "replicas x1"},
            "pcg_ms_per_solve": 70.1234567, "pcg_iters_mean": 148.6, "wall_ms_per_step": 90.1234,
            "mixed": {"value": 12.0123456789, "unit": "steps/s", "ms_per_step": 83.2345678, "pcg_ms_per_solve": 63.2,
                      "pcg_inner_iters_mean": 160.2, "outer_cycles_mean": 2.0, "all_converged": True,
                      "dtype": "f32 inner / f64 outer", "stopping_test": "x"},
            "roofline": {"bound": "hbm", "kernel": "k_precond_async", "achieved": 90.812345, "peak": 6789.3,
                         "unit": "GB/s", "frac": 0.0133765432, "peak_source": "measured", "traffic": 65123456.7,
                         "algorithmic_bytes_per_launch": 41761234.5, "avg_launch_ms": 0.4601234,
                         "timed_launches": 1234, "note": "x" * 80, "preconditioner_form": 201},
            "kernels": {f"k_{i}": {"avg_launch_ms": f(i), "timed_launches": i, "est_ms_per_step": f(i)} for i in range(4)},
            "advection": {"algorithmic_bytes_per_step": 1.1e8, "ms_per_step": 8.1234567, "achieved_GBps": 13.5,
                          "frac": 0.002, "note": "x" * 80},
            "cpu_baseline": {"value": 1.3866847165536678, "unit": "steps/s", "cores": 16, "kind": "port",
                             "sample": "x" * 150, "sample_short": "3 steps from t=0, OpenMP oracle port, 12.2 s"},
            "e2e": {"value": 11.17234567, "unit": "steps/s", "h2d_bytes_per_step": 11971936,
                    "d2h_bytes_per_step": 14964920, "steps": 20},
            "clocks": {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": [], "samples": 600, "power_w_max": 226.7},
            "gpu_launches": 61234,
            "isolated_solves": {"config": "x" * 150, "n": 372862, "nnz": 2634386,
                                "fp64": {"ms_per_solve": 90.51234, "iterations_mean": 164.35, "outer_cycles_mean": 1.0,
                                         "all_converged": True, "algorithmic_GBps": 120.123,
                                         "batch": {"ms_per_solve": 17.4234567, "lanes": 7, "identical": True,
                                                   "all_converged": True}},
                                "mixed": {"ms_per_solve": 75.51234, "iterations_mean": 175.1, "outer_cycles_mean": 2.0,
                                          "all_converged": True, "algorithmic_GBps": 130.123,
                                          "batch": {"ms_per_solve": 14.8234567, "lanes": 8, "identical": True,
                                                    "all_converged": True}},
                                "mixed_speedup": 1.1987654},
            "adjoint": {"config": "x" * 200, "slots": 40000, "mixed": {"ratio": 2.0612345}, "fp64": {"ratio": 2.1},
                        "adjoint_fwd_cost_ratio": 2.0612345, "grad_rel_error_mixed_vs_fp64": 3.0123456e-05,
                        "peak_device_bytes": 2123456789, "fields": "x" * 100},
            "precision_comparison": {"config": "x" * 100, "density_rel_l2_mixed_vs_fp64": pick,
                                     "pressure_rel_l2_mixed_vs_fp64": pick, "rel_residual_fp64": pick,
                                     "rel_residual_mixed": pick, "per_step_density": series,
                                     "per_step_pressure": series, "per_step_divergence_fp64": series,
                                     "per_step_divergence_mixed": series},
            "ensemble": {"simulations": 7, "steps_each": 10, "wall_s": 1.2345678, "aggregate_steps_per_s": 56.789012345,
                         "steps_per_s_each": 8.1234567, "member_identical_to_alone": True, "note": "x" * 80},
            "uniform2d": {"workload": "x" * 80, "value": 3.310806460212116, "unit": "frames/s",
                          "ms_per_frame": 302.04121322631835, "e2e": {"value": 3.3}, "cpu_baseline": {"value": 1.4}}}


def test_gpu_arm_line_is_short_and_last(tmp_path, capsys):
    """The GPU arm's printed line at the default section sizes stays under the limit, is the last line of
    stdout, parses, and carries the contract's keys; the bulk goes to the side file."""
    sys.path.insert(0, ROOT)
    import bench

    full = _fake_full()
    detail = str(tmp_path / "detail.json")
    bench.emit(full, detail)
    out = capsys.readouterr().out
    last = out.strip().splitlines()[-1]
    assert len(last) <= bench.LINE_LIMIT, len(last)
    line = json.loads(last)
    assert line["value"] > 0 and line["unit"] == "steps/s" and line["metric"] == "smoke steps/s"
    for k in ("roofline", "cpu_baseline", "e2e", "clocks", "gpu_launches", "config", "mixed"):
        assert line.get(k) is not None, k
    for k in ("bound", "achieved", "peak", "unit", "frac", "traffic"):
        assert k in line["roofline"], k
    assert {"h2d_bytes_per_step", "d2h_bytes_per_step"} <= set(line["e2e"])
    # the last 1500 characters of stdout alone hold the whole line
    assert json.loads(out[-1500:].strip().splitlines()[-1]) == line
    with open(detail) as f:
        assert len(json.load(f)["precision_comparison"]["per_step_density"]) == 200
