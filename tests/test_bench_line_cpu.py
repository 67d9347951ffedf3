"""bench.py's printed line (no GPU): every key of the bench contract, the roofline
objects, vs_fp64, e2e, cpu_baseline and a serving summary survive, floats are rounded,
and the line stays under 3 KB so that a reader of the output's tail gets all of it."""
import importlib.util
import json
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _full_line():
    stage = {"ms": 10480.123, "jacobi_tflops": 8.6771, "peak": 65.76, "frac": 0.1320, "peak_source": "cuBLAS SGEMM"}
    roof = {"kernel": "svd", "per_launch_ms": 92.0123, "launches": 420, "traffic": 5.34e8,
            "traffic_of": "the mid-bond decomposition (ncu, profiles/)", "bound": "latency (block-Jacobi barriers)",
            "achieved": 0.37921, "peak": 65.7612, "unit": "TFLOP/s", "frac": 0.0057671,
            "peak_source": "cuBLAS SGEMM measured in this run",
            "stages": {"fp32_stage": stage, "fp64_stage": dict(stage, frac=0.95, peak_source="cuBLAS DGEMM")}}
    return {
        "metric": "s/DMRG sweep at D=2048, mixed vs FP64 plain at |dE|<1e-8/site; solves/s, p99",
        "value": 14.780904947916667, "unit": "s/sweep", "n_gpus": 1, "steps": 3, "warmup": 3,
        "ms_per_step": 14780.904947916668, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "tf32x3+f64svd+f64", "data": "synthetic",
        "config": {"workload": "Heisenberg 6x12 open cylinder (snake order, 72 sites), two-site DMRG sweep at "
                               "D=2048 after the ramp 256->512->1024->2048, U(1) Sz=0", "L": 72, "D": 2048,
                   "model": "a long model description " * 4, "cutoff": 1e-10, "update": "one-step Lanczos",
                   "start": "a long start description " * 4, "l2": "working set", "parallelism": "single GPU",
                   "mode": "tf32x3"},
        "gpu_launches": 37881, "clocks": {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": [], "samples": 210},
        "planner": {"host_calls": 4484, "device_calls": 0},
        "roofline": roof,
        "roofline_gemm": dict(roof, kernel="gemm", bound="tensor", stages=None),
        "roofline_f64": {"gemm": dict(roof, kernel="gemm", stages=None), "svd": roof},
        "kernel_time_ms": {"gemm": 3713.4, "permute": 11.2, "svd": 38645.9, "elementwise": 86.1, "pack": 1377.7,
                           "svd_fp64": 28164.2},
        "kernel_time_ms_f64": {"gemm": 64817.1, "permute": 593.3, "svd": 104358.2, "elementwise": 59.0,
                               "pack": 5.1, "svd_fp64": 0.0},
        "sweeps": {"times_s": [15.011, 14.673, 14.662], "middle_bond": [2050] * 3,
                   "truncated_weight": [1.5e-8] * 3, "ritz_E": [-47.3] * 3},
        "vs_fp64": {"fp64_s_per_sweep": 81.48, "mixed_s_per_sweep": 14.66, "speedup_vs_fp64": 5.556,
                    "dE_per_site": 2.039e-09, "E_fp64": -47.30466635751, "E_mixed": -47.30466621071, "sweeps": 2,
                    "truncated_weight_fp64": [1.54e-8, 1.53e-8], "truncated_weight_mixed": [1.537e-8, 1.53e-8],
                    "ritz_E_fp64": [-47.3] * 2, "ritz_E_mixed": [-47.3] * 2, "note": "a note " * 10},
        "state": {"ramp": [{"D": 256, "sweeps": 2, "lanczos_steps": 4, "s": 1.51, "E": -47.29}] * 4,
                  "warmup": {"sweeps": 3}, "prep_wall_s": 55.4},
        "e2e": {"value": 15.11, "unit": "s/sweep", "steps": 2, "sweep_times_s": [15.1, 15.1],
                "h2d_bytes_per_step": 610084664, "d2h_bytes_per_step": 610099728, "E": -47.3, "note": "n " * 40},
        "cpu_baseline": {"value": 170.4, "unit": "s/sweep", "cores": 16, "kind": "port",
                         "sample": "3 oracle bond updates on the timed state at bonds [11, 35, 59] " * 3},
        "serving": {"requests": 200, "rate_per_s": 0.25, "offered_load": 0.7, "solves_per_s": 0.13,
                    "p50_s": 405.1, "p99_s": 581.9, "capacity": {"solves_per_s": 0.137}, "errors": 0,
                    "truncated_weight": {"max": 7.4e-7, "median": 1e-13},
                    "serial_fp64": {"solves_per_s": 0.0265, "sample": 9, "dE_per_site": {"max": 5.5e-10},
                                    "truncated_weight": {"max": 7.4e-7}},
                    "capacity_vs_serial_fp64": 4.9},
        "autotune_classes": 57,
    }


def test_slim_line_keeps_the_contract_under_3_kb():
    b = _bench()
    out = b.slim_cylinder_line(_full_line())
    text = json.dumps(out)
    assert len(text) < 3000, len(text)
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "gpu_launches", "clocks", "roofline", "e2e", "cpu_baseline",
              "vs_fp64", "serving"):
        assert k in out, k
    assert out["value"] == 14.780904947916667          # the value itself is never rounded
    r = out["roofline"]
    for k in ("bound", "achieved", "peak", "unit", "frac", "traffic"):
        assert k in r, k
    assert set(r["stages"]) == {"fp32", "fp64"}
    assert out["vs_fp64"]["speedup_vs_fp64"] == 5.556 and out["vs_fp64"]["E_fp64"] == -47.3046663575
    for k in ("value", "unit", "h2d_bytes_per_step", "d2h_bytes_per_step"):
        assert k in out["e2e"], k
    for k in ("value", "unit", "cores", "kind", "sample"):
        assert k in out["cpu_baseline"], k
    assert len(out["cpu_baseline"]["sample"]) <= 150
    assert out["serving"]["p99_s"] == 581.9 and out["serving"]["capacity_solves_per_s"] == 0.137
    assert set(out["clocks"]) == {"sm_mhz", "sm_max_mhz", "reasons"}


def test_sig_rounds_floats_only():
    b = _bench()
    assert b.sig(3.14159265, 4) == 3.142
    assert b.sig({"a": [1.23456e-9, 7, "x"]}) == {"a": [1.235e-09, 7, "x"]}


def test_both_arms_print_the_same_config():
    """The reference arm and the GPU arm describe the cylinder workload identically."""
    import types
    b = _bench()
    args = types.SimpleNamespace(D=2048, seed=0, ramp_sweeps=2, converge_sweeps=2, ramp_lanczos=4, warmup=3)
    ours = dict(b.cylinder_config(args), parallelism="single GPU", mode="tf32x3")
    ref = dict(b.cylinder_config(args), parallelism="single GPU")
    assert b.slim_config(ours) == b.slim_config(ref)
    assert b.slim_config(ours)["D"] == 2048
