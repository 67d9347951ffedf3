"""Benchmark: seconds per two-site DMRG sweep at bond dimension D = 2048, mixed
precision against the plain FP64 path, on the spin-1/2 Heisenberg model of a 6 x 12
open cylinder (72 sites, snake order, U(1) total Sz = 0).

Workload (default, --model cylinder): H = J sum_<ij> S_i.S_j on the cylinder of
circumference 6 and length 12, as an MPO compressed to its Schmidt rank (bond
dimension 20).  A seeded random_bMPS at D = 256 is brought to canonical form and
swept with QuantiT's two-site update (one-step Lanczos, SVD cutoff 1e-10) along the
ramp D = 256 -> 512 -> 1024 (--ramp-sweeps each), then --warmup sweeps at D.  From
that state S0:
  value      : --steps mixed sweeps in ONE dmrg call (split-TF32 tensor-core block
               GEMMs, sector SVDs finished in FP64), CUDA events on the library stream.
  vs_fp64    : --compare-sweeps plain-FP64 sweeps from S0, set against the same number
               of the timed mixed sweeps: seconds per sweep of each (sweeps after the
               first of a call, which also builds the environments), and |dE| per site
               between the two states' FP64 energies, with their truncated weights.
  e2e        : one sweep per step through the public API from host buffers (upload the
               MPS, one dmrg call, read the optimised MPS and energy back).
  cpu_baseline / --impl reference: QuantiT's bond update restated in numpy (the
               oracle) on the host cores, on the same state S0: real bond updates at
               bonds spread evenly over the chain (stratified sample), times 2(L-2)
               bond updates per sweep.
Synthetic data: no dataset is involved.  Other workloads: --model heisenberg|hubbard
(chains), --workload contraction|svd|serving.

Prints one JSON line (rank 0).  Multi-GPU (torchrun) runs independent replicas,
one solve per GPU ("replicas only": a DMRG sweep is sequential).
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "s/DMRG sweep at D=2048, mixed vs FP64 plain at |dE|<1e-8/site; solves/s, p99"
UNIT = "s/sweep"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--model", default="cylinder", choices=["heisenberg", "hubbard", "cylinder"],
                   help="heisenberg: spin-1/2 chain, U(1) (defaults L=32, D=2048); hubbard: Fermi-Hubbard "
                        "U=8 at half filling, U(1)xU(1) (defaults L=64, D=1024); cylinder (default): spin-1/2 "
                        "Heisenberg on a 6 x 12 open cylinder, snake order (72 sites, MPO compressed to bond "
                        "dimension 20; D=2048 reached by the ramp 256 -> 512 -> 1024)")
    p.add_argument("--L", type=int, default=None)
    p.add_argument("--D", type=int, default=None)
    p.add_argument("--mode", default="tf32x3", choices=["f64", "tf32x3", "bf16x3"])
    p.add_argument("--compare-f64", type=int, default=1, help="also time FP64 sweeps from the same state")
    p.add_argument("--compare-sweeps", type=int, default=2,
                   help="cylinder: FP64 sweeps from the timed state for vs_fp64")
    p.add_argument("--ramp-sweeps", type=int, default=2, help="cylinder: sweeps at each ramp bond dimension")
    p.add_argument("--ramp-lanczos", type=int, default=4,
                   help="cylinder: Lanczos steps per bond in the ramp sweeps (state preparation only; the "
                        "warm-up and timed sweeps use QuantiT's one-step update)")
    p.add_argument("--converge-sweeps", type=int, default=2,
                   help="cylinder: ramp-style sweeps at D before the warm-up (state preparation)")
    p.add_argument("--e2e-steps", type=int, default=2, help="cylinder: sweeps timed through the public API")
    p.add_argument("--cpu-bonds", type=int, default=None,
                   help="cylinder: bonds (strata) of the CPU sample, spread evenly over the chain (default: one "
                        "per timed update, so that the timed updates visit every stratum once)")
    p.add_argument("--cpu-steps", type=int, default=3, help="cylinder: CPU bond updates in our arm's cpu_baseline")
    p.add_argument("--prepare-cpu-sample", default=None,
                   help="internal: build the timed state on the GPU and write it with the environments of "
                        "the sampled bonds to this directory, then exit")
    p.add_argument("--cpu-sample", default=None,
                   help="internal: time oracle bond updates on the state written to this directory")
    p.add_argument("--cpu-threads", type=int, default=0, help="internal: BLAS threads of --cpu-sample (0: all)")
    p.add_argument("--cpu-offset", type=int, default=0, help="internal: first stratum of --cpu-sample")
    p.add_argument("--seed", type=int, default=0)
    p.add_argument("--svd-deflation", type=int, default=None,
                   help="1/0: numerically null columns leave the sector-SVD sweeps of a truncating svd")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--workload", default="dmrg", choices=["dmrg", "serving", "contraction", "svd", "planner"],
                   help="dmrg: the D=2048 sweep line (with a short serving section); serving: the full "
                        "Poisson request stream of XXZ solves (L in 16..128, D in 32..512); contraction: the "
                        "synthetic theta-pair contraction + sector-SVD truncation microbench at D; svd: the "
                        "truncated sector SVD of a mid-chain DMRG theta at D (after --svd-sweeps sweeps)")
    p.add_argument("--svd-sweeps", type=int, default=3, help="svd workload: mixed sweeps before the theta is taken")
    p.add_argument("--save-state", default=None, help="svd workload: write the theta (block-list file)")
    p.add_argument("--state-file", default=None, help="svd workload: read the theta instead of sweeping")
    p.add_argument("--serving-requests", type=int, default=None,
                   help="requests of the serving stream (default: 200 for --workload serving, 0 otherwise)")
    p.add_argument("--serving-rate", type=float, default=0.0,
                   help="Poisson arrival rate (requests/s); <= 0 (the default): --serving-load x the capacity "
                        "measured on a burst first, so that the stream runs below saturation")
    p.add_argument("--serving-load", type=float, default=0.7, help="offered load of the automatic rate")
    p.add_argument("--serving-calibrate", type=int, default=48, help="requests of the capacity burst")
    p.add_argument("--serving-slots", type=int, default=8)
    p.add_argument("--serving-lanczos", type=int, default=4,
                   help="Lanczos steps per bond in the serving solves (1: QuantiT's one-step update)")
    p.add_argument("--serving-fp64-every", type=int, default=10,
                   help="serial FP64 baseline on every k-th request of the stream")
    p.add_argument("--serving-fp64-budget", type=float, default=300.0,
                   help="stop the serial FP64 sample once this many seconds are spent")
    p.add_argument("--planner", default="host", choices=["host", "device", "auto"],
                   help="block-sparsity planner of the contractions (auto: device for >= 3000 blocks in the two operands)")
    p.add_argument("--jacobi", default="block", choices=["block", "scalar"],
                   help="sector-SVD Jacobi kernel (block-cyclic where it fits, or scalar)")
    return p.parse_args()


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), \
        int(os.environ.get("LOCAL_RANK", "0"))


class ClockSampler:
    """nvidia-smi samples (SM clock, throttle reasons) during the timed region."""

    def __init__(self, index):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def start(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()

    def _run(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                f = [x.strip() for x in out.stdout.strip().split(",")]
                if len(f) >= 7:
                    self.samples.append(f)
            except Exception:
                pass
            self._stop.wait(0.2)

    def stop(self):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[3 + i].strip() == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


def build_state(q, L, D, seed=0, model="heisenberg"):
    if model == "cylinder":
        mpo = q.networks.cylinder_heisenberg(12, 6, 1.0, "snake")
        mps = q.networks.random_bmps(len(mpo), D, seed=seed)
    elif model == "hubbard":
        mpo = q.networks.hubbard(L, 8.0)
        mps = q.networks.random_bmps(L, D, q.networks.HUBBARD_PHYS, (L, 0), seed=seed, mods=(0, 0))
    else:
        mpo = q.networks.heisenberg(L)
        mps = q.networks.random_bmps(L, D, seed=seed)
    mps.move_oc(0)
    mps.normalize_center()
    return mpo, mps


def run_sweeps(q, mpo, mps, n, mode, D):
    """n single sweeps timed with CUDA events on the library's stream; the Ritz
    energy of each sweep and the final state."""
    import torch
    stream = torch.cuda.ExternalStream(q.lib().qtt_get_stream())
    opts = q.algorithms.dmrg_options(cutoff=1e-10, convergence_criterion=0.0, max_bond=D, min_bond=4,
                                     maximum_iterations=1, gemm=mode, final_energy_fp64=False)
    cur = q.networks.bMPS(list(mps), mps.orthogonality_center)
    Es, ts = [], []
    for _ in range(n):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        E = q.algorithms.dmrg(mpo, cur, opts)
        e1.record(stream)
        e1.synchronize()
        Es.append(E)
        ts.append(e0.elapsed_time(e1) / 1000.0)
    return Es, ts, cur


def bond_max(mps):
    """Largest bond dimension of a bMPS (the right leg of each site)."""
    return int(max(_leg_dim(t, 2) for t in mps))


def bond_sum(mps):
    return int(sum(_leg_dim(t, 2) for t in mps))


def _leg_dim(t, leg):
    sbd = t.sections_by_dim
    start = sum(sbd[:leg])
    return int(sum(t.section_sizes[start:start + sbd[leg]]))


def fp64_energy(q, mpo, mps):
    t0 = time.perf_counter()
    e, n2 = q.algorithms.mps_energy(mpo, mps)
    return e / n2, time.perf_counter() - t0


def matmul_peak_tflops(dtype, tf32=False):
    """cuBLAS GEMM throughput measured in this run (FP64 / FP32 SIMT denominators)."""
    import torch
    torch.backends.cuda.matmul.allow_tf32 = tf32
    n = 4096
    a = torch.randn(n, n, dtype=dtype, device="cuda")
    b = torch.randn(n, n, dtype=dtype, device="cuda")
    for _ in range(2):
        a @ b
    torch.cuda.synchronize()
    best = 1e9
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        a @ b
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1) / 1000)
    return 2 * n ** 3 / best / 1e12


class CpuSampler:
    """The oracle (numpy; BLAS on all host cores) at the workload's mid-chain bond:
    environments are built once, each sample is one two-site bond update at D."""

    def __init__(self, L, D):
        from oracle import qtt_oracle as o
        self.o, self.L, self.D = o, L, D
        rng = np.random.default_rng(0)
        self.mpo = o.heisenberg_mpo(L)
        self.mps = o.random_mps(L, D, [1, -1], 0, rng)
        self.mid = L // 2 - 1
        env = [None] * (L + 2)
        env[0] = o.trivial_edge((self.mps[0], 0), (self.mpo[0], 0))
        env[L + 1] = o.trivial_edge((self.mps[-1], 2), (self.mpo[-1], 2))
        for i in range(self.mid):
            env[i + 1] = o.compute_left_env(self.mpo[i], self.mps[i], env[i])
        for i in range(L - 1, self.mid + 1, -1):
            env[i + 1] = o.compute_right_env(self.mpo[i], self.mps[i], env[i + 2])
        self.env = env
        self.h2 = o.compute_2sites_hamil(self.mpo)
        self.opts = o.DmrgOptions(cutoff=1e-10, maximum_bond=D, minimum_bond=4)
        # bonds of a sweep weighted by their cost relative to the mid bond (sum over sectors of D_b^3)
        from quantit_gb300.networks import bond_sectors  # pure-python structure helper
        bonds = bond_sectors(L, D, [1, -1], 0)
        w = [sum(m ** 3 for m in b.values()) for b in bonds]
        sweep_bonds = list(range(0, L - 2)) + list(range(L - 2, 0, -1))
        self.factor = sum(w[b] / w[self.mid] for b in sweep_bonds)

    def bond(self):
        mps = [m for m in self.mps]
        env = list(self.env)
        t0 = time.perf_counter()
        self.o.dmrg_bond_update(self.mpo, self.h2, mps, env, self.mid, True, self.opts)
        return time.perf_counter() - t0


def reference_arm(args, cfg):
    """Each step = one mid-chain bond update of the oracle, extrapolated to a sweep."""
    s = CpuSampler(args.L, args.D)
    for _ in range(min(args.warmup, 1)):
        s.bond()
    per = [s.bond() for _ in range(args.steps)]
    t_sweep = float(np.mean(per)) * s.factor
    ncores = os.cpu_count()
    sample = (f"{args.steps} mid-chain bond update(s) at D={args.D} ({np.mean(per):.2f} s each) "
              f"x {s.factor:.1f} size-weighted bonds per sweep")
    return {"metric": METRIC, "value": t_sweep, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_sweep * 1e3, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": cfg, "impl": "reference",
            "cpu_baseline": {"value": t_sweep, "unit": UNIT, "cores": ncores, "kind": "port", "sample": sample},
            "e2e": {"value": t_sweep, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def roofline(kind, st, P, mode, peaks_cache):
    """Achieved algorithmic throughput of one kernel class against its roofline."""
    if st["ms"] <= 0:
        return None
    sec = st["ms"] / 1e3
    base = {"kernel": kind, "per_launch_ms": st["ms"] / max(st["launches"], 1), "launches": st["launches"],
            "traffic": None}
    if kind == "gemm" and mode == "bf16x3":
        bf16 = P.get("bf16_tflops", 1939.7)
        ach = st["work"] / sec / 1e12
        return dict(base, bound="tensor", achieved=ach, peak=bf16, unit="TFLOP/s", frac=ach / bf16,
                    tensor_ops_frac=6.0 * ach / bf16,
                    peak_source="dense BF16 = MEASURED_PEAKS.json bf16_tflops (of measured); "
                                "achieved counts useful FLOP, the split issues 6 tensor products each")
    if kind == "gemm" and mode != "f64":
        tf32 = P.get("bf16_tflops", 1939.7) / 2.0
        ach = st["work"] / sec / 1e12
        return dict(base, bound="tensor", achieved=ach, peak=tf32, unit="TFLOP/s", frac=ach / tf32,
                    tensor_ops_frac=3.0 * ach / tf32,
                    peak_source="dense TF32 = 1/2 of MEASURED_PEAKS.json bf16_tflops (of measured); "
                                "achieved counts useful FLOP, the split issues 3 tensor products each")
    if kind in ("gemm", "svd"):
        fp32 = kind == "svd" and mode != "f64"
        key = "fp32" if fp32 else "fp64"
        if key not in peaks_cache:
            import torch
            peaks_cache[key] = matmul_peak_tflops(torch.float32 if fp32 else torch.float64)
        ach = st["work"] / sec / 1e12
        return dict(base, bound="latency (block-Jacobi barriers)" if kind == "svd" else "fp64",
                    achieved=ach, peak=peaks_cache[key], unit="TFLOP/s", frac=ach / peaks_cache[key],
                    peak_source=f"cuBLAS {'SGEMM' if fp32 else 'DGEMM'} measured in this run")
    ach = st["work"] / sec / 1e9
    peak = P.get("hbm_gbs", 6800.0)
    return dict(base, bound="hbm", achieved=ach, peak=peak, unit="GB/s", frac=ach / peak,
                peak_source="MEASURED_PEAKS.json hbm_gbs (of measured)")


WORK_ONLY = ("jacobi_fp32", "jacobi_fp64")   # statistics kinds that carry FLOPs but no time
# DRAM bytes (read + write) of one mixed-path decomposition of the mid-cylinder theta at
# D = 2048, summed over its kernels from one ncu capture (cold cache, serialised launches;
# profiles/svd_mixed_cylinder_theta_D2048.md).  The decomposition is the svd class's
# largest launch in the cylinder sweep.
SVD_TRAFFIC_MID_THETA = 5.34e8


def timed_kinds(kinds):
    return {k: v for k, v in kinds.items() if k not in WORK_ONLY}


def svd_stages(kinds, mode, peaks_cache):
    """The sector SVDs by precision stage: each stage's time and the FLOPs its Jacobi
    sweeps performed (sweeps x (6 p q^2 + 3 q^3) per sector; the FP64 stage of the mixed
    path adds its Newton-Schulz and W V products), against the SGEMM / DGEMM measured in
    this run.  The algorithmic count of the roofline object does not depend on the method;
    these figures show how busy each stage keeps its pipe."""
    import torch
    out = {}
    t_all, t64 = kinds["svd"]["ms"], kinds["svd_fp64"]["ms"]
    stages = [("fp32_stage", t_all - t64, kinds["jacobi_fp32"]["work"], "fp32"),
              ("fp64_stage", t64, kinds["jacobi_fp64"]["work"], "fp64")] if mode != "f64" else \
        [("fp64_stage", t_all, kinds["jacobi_fp64"]["work"], "fp64")]
    for name, ms, work, key in stages:
        if ms <= 0:
            continue
        if key not in peaks_cache:
            peaks_cache[key] = matmul_peak_tflops(torch.float32 if key == "fp32" else torch.float64)
        tf = work / (ms / 1e3) / 1e12
        out[name] = {"ms": ms, "jacobi_tflops": tf, "peak": peaks_cache[key],
                     "frac": tf / peaks_cache[key], "peak_source": f"cuBLAS {'SGEMM' if key == 'fp32' else 'DGEMM'}"}
    return out


def e2e_sweep(q, mpo, mps, args):
    """The same sweeps as the device-timed ones (args.steps single sweeps from the same
    state), each through the public API: the MPS is uploaded from host buffers, one
    sweep runs, and the optimised MPS and the energy are read back to the host, all
    inside the timed region; the next sweep starts from those host buffers."""
    host = [(t.copy_structure(), t.blocks()) for t in mps]
    oc = mps.orthogonality_center
    opts = q.algorithms.dmrg_options(cutoff=1e-10, convergence_criterion=0.0, max_bond=args.D, min_bond=4,
                                     maximum_iterations=1, gemm=args.mode, final_energy_fp64=False)
    ts, h2d, d2h, E = [], [], [], None
    for _ in range(args.steps):
        h2d.append(sum(sum(v.nbytes for _, v in blks) for _, blks in host))
        t0 = time.perf_counter()
        dev = q.networks.bMPS([s.set_blocks(b) for s, b in host], oc)
        E = q.algorithms.dmrg(mpo, dev, opts)
        out = [t.blocks() for t in dev]
        ts.append(time.perf_counter() - t0)
        d2h.append(sum(sum(v.nbytes for _, v in blks) for blks in out) + 8)
        host = [(t.copy_structure(), blks) for t, blks in zip(dev, out)]
        oc = dev.orthogonality_center
    return {"value": float(np.mean(ts)), "unit": UNIT, "sweep_times_s": ts,
            "h2d_bytes_per_step": int(np.mean(h2d)), "d2h_bytes_per_step": int(np.mean(d2h)), "E": E}


SERVING_FULL = dict(lengths=(16, 32, 64, 128), bonds=(32, 64, 128, 256, 512))


def serving_section(q, args, n_requests):
    """Continuous-batching solves of a seeded Poisson stream of XXZ requests (L from
    {16, 32, 64, 128}, D from {32, ..., 512}, delta from [0, 2]; mixed precision,
    converged to 1e-8 relative energy).  With --serving-rate <= 0 the arrival rate is
    --serving-load times the capacity measured first on a burst of
    --serving-calibrate requests released at once (another seed), so the stream runs
    below saturation and its latency is service, not queueing.  Every k-th request of
    the stream is then solved alone in plain FP64 (serial, one at a time) for the
    baseline throughput and the per-request |dE| per site and truncated weight."""
    from quantit_gb300 import serving
    dist = SERVING_FULL
    mixed = args.mode if args.mode != "f64" else "tf32x3"

    def engine():
        return serving.ServingEngine(slots=args.serving_slots, gemm=mixed, convergence=1e-8, max_sweeps=40,
                                     lanczos_steps=args.serving_lanczos)
    out = {"distribution": {"L": list(dist["lengths"]), "D": list(dist["bonds"]), "delta": [0.0, 2.0]},
           "slots": args.serving_slots, "gemm": mixed, "lanczos_steps": args.serving_lanczos, "convergence": 1e-8}
    rate = args.serving_rate
    if rate <= 0:
        burst = serving.poisson_requests(args.serving_calibrate, rate=0.0, seed=1, **dist)
        eng = engine()
        res = eng.run(burst, realtime=False,
                      on_done=lambda r: print(f"calibration {r.rid} L={r.L} D={r.D} service={r.service:.1f} s",
                                              file=sys.stderr, flush=True))
        cap = len(res) / max(r.done for r in res)
        rate = args.serving_load * cap
        out["capacity"] = {"requests": len(res), "solves_per_s": cap,
                           "how": "burst released at once (seed 1); solves / time to the last completion"}
    reqs = serving.poisson_requests(n_requests, rate=rate, seed=0, **dist)
    eng = engine()

    def progress(r):
        print(f"served {r.rid} L={r.L} D={r.D} sweeps={r.sweeps} latency={r.latency:.1f} s "
              f"service={r.service:.1f} s", file=sys.stderr, flush=True)
    res = eng.run(reqs, realtime=True, on_done=progress)
    mk = max(r.done for r in res) - min(r.arrival for r in res)
    out.update(serving.summarize([r.latency for r in res], mk, len(res)))
    lat = np.array([r.latency for r in res])
    tw = np.array([r.truncated_weight for r in res], dtype=float)
    print("serving stream: " + json.dumps(serving.summarize([r.latency for r in res], mk, len(res))),
          file=sys.stderr, flush=True)
    out.update({"requests": len(reqs), "rate_per_s": rate, "p90_s": float(np.percentile(lat, 90)),
                "offered_load": rate / out["capacity"]["solves_per_s"] if "capacity" in out else None,
                "peak_concurrency": eng.peak_concurrency,
                "memory_budget_bytes": eng.memory_budget, "peak_admitted_bytes": eng.peak_memory,
                "errors": sum(1 for r in res if r.error),
                "mean_service_s": float(np.mean([r.service for r in res])),
                "mean_wait_s": float(np.mean([r.admitted - r.arrival for r in res])),
                "truncated_weight": {"max": float(np.nanmax(tw)), "median": float(np.nanmedian(tw))},
                "latency": "completion minus arrival (queueing included)"})
    sample, st = [], []
    t0 = time.perf_counter()
    for r in reqs[::max(1, args.serving_fp64_every)]:
        if sample and time.perf_counter() - t0 > args.serving_fp64_budget:
            break
        st += serving.serial_solve_times([r], gemm="f64", convergence=1e-8, max_sweeps=40,
                                         lanczos_steps=args.serving_lanczos)
        sample.append(r)
        print(f"serial fp64: request {r.rid} L={r.L} D={r.D} {st[-1][0]:.1f} s", file=sys.stderr, flush=True)
    svc = [x[0] for x in st]
    byid = {r.rid: r for r in res}
    dE = np.array([abs(byid[r.rid].energy - x[1]) / r.L for r, x in zip(sample, st)])
    tw64 = np.array([x[3] for x in st], dtype=float)
    twm = np.array([byid[r.rid].truncated_weight for r in sample], dtype=float)
    out["serial_fp64"] = {"sample": len(sample), "of_every": args.serving_fp64_every,
                          "sampled_L_D": [[r.L, r.D] for r in sample],
                          "solves_per_s": len(sample) / sum(svc), "mean_service_s": float(np.mean(svc)),
                          "dE_per_site": {"max": float(dE.max()), "median": float(np.median(dE))},
                          "truncated_weight": {"max": float(np.nanmax(tw64)), "median": float(np.nanmedian(tw64))},
                          "truncated_weight_mixed_same_requests": {"max": float(np.nanmax(twm)),
                                                                   "median": float(np.nanmedian(twm))},
                          "note": "one solve at a time on the GPU, plain FP64, same requests and seeds"}
    base = out["capacity"]["solves_per_s"] if "capacity" in out else out["solves_per_s"]
    out["capacity_vs_serial_fp64"] = base / out["serial_fp64"]["solves_per_s"]
    return out


def svd_workload(q, args):
    """The truncated sector SVD svd(theta, 2, 1e-10, 1, D) of the mid-chain two-site
    theta of a DMRG state (Heisenberg L, D; --svd-sweeps mixed sweeps from the seeded
    random state), the decomposition a bond update runs.  Each step is one SVD in
    --mode (the work is the sweeps the decomposition needed), timed with CUDA events
    on the library stream; L2 is flushed between steps."""
    import torch
    from quantit_gb300 import serialize
    if args.state_file:
        theta = serialize.load(args.state_file)
    elif args.model == "cylinder":
        # the mid-cylinder theta of the state the headline times
        mpo, cur, _ = prepare_cylinder(q, args, args.seed)
        c = len(cur) // 2
        cur.move_oc(c)
        theta = cur[c].tensordot(cur[c + 1], ([2], [0]))
        if args.save_state:
            serialize.save(args.save_state, theta)
    else:
        mpo, mps = build_state(q, args.L, args.D, seed=0)
        _, _, cur = run_sweeps(q, mpo, mps, args.svd_sweeps, "tf32x3", args.D)
        cur.move_oc(args.L // 2)
        c = args.L // 2
        theta = cur[c].tensordot(cur[c + 1], ([2], [0]))
        if args.save_state:
            serialize.save(args.save_state, theta)
    stream = torch.cuda.ExternalStream(q.lib().qtt_get_stream())
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > L2
    q.set_autotune(False)
    q.set_gemm_mode(args.mode)
    try:
        for _ in range(args.warmup):
            q.linalg.svd(theta, 2, 1e-10, min_size=1, max_size=args.D)
        q.stats.reset()
        q.stats.enable(True)
        ts = []
        for _ in range(args.steps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            U, d, V = q.linalg.svd(theta, 2, 1e-10, min_size=1, max_size=args.D)
            e1.record(stream)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1) / 1e3)
        kinds = {k: q.stats.get(k) for k in q.stats.KINDS}
        q.stats.enable(False)
        sweeps = q.linalg.last_svd_sweeps()
        fp32_sweeps = q.linalg.last_svd_sweeps(fp32_stage=True)
    finally:
        q.set_gemm_mode("f64")
        q.set_autotune(True)
    t = float(np.mean(ts))
    return {"metric": "s per truncated sector SVD of a mid-chain DMRG theta", "value": t, "unit": "s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64" if args.mode != "f64" else "f64",
            "data": "synthetic", "config": {"workload": f"svd(theta, 2, 1e-10, 1, {args.D}) of the middle theta "
                                                        f"of a D={args.D} DMRG state of the "
                                                        + ("6x12 cylinder" if args.model == "cylinder"
                                                           else f"Heisenberg chain L={args.L}"),
                                            "sweeps_before": args.svd_sweeps, "mode": args.mode,
                                            "l2": "flushed between steps (256 MB write)"},
            "jacobi_sweeps_per_sector": sweeps, "fp32_sweeps_per_sector": fp32_sweeps,
            "kept": int(sum(d.section_sizes)),
            "roofline": dict(roofline("svd", kinds["svd"], peaks(), args.mode, {}),
                             stages=svd_stages(kinds, args.mode, {})),
            "kernel_time_ms": {k: v["ms"] for k, v in timed_kinds(kinds).items()}}


def planner_workload(q, args):
    """Planner time per contraction, host merge-join against the device planner, on
    structure-only U(1)xU(1) rank-3 tensors A[a, s, b] with (2k+1)^2 charge sectors per
    bond leg (2 states each) and 4 physical sectors: A.B over one leg and A.A* over two,
    each planned 10 times after one untimed call (host wall time, planner_stats)."""
    from quantit_gb300.conserved import ZZ
    shifts = [(0, 0), (-1, -1), (-1, 1), (-2, 0)]
    physi = [(1, ZZ(-a, -b)) for a, b in [(0, 0), (1, 1), (1, -1), (2, 0)]]
    rows = []
    for k in (4, 8, 12, 16, 24, 31):
        grid = [(i, j) for i in range(-k, k + 1) for j in range(-k, k + 1)]
        pos = {g: n for n, g in enumerate(grid)}
        legs = [[(2, ZZ(i, j)) for i, j in grid], physi, [(2, ZZ(-i, -j)) for i, j in grid]]
        blocks = [(a, si, pos[(g[0] + d[0], g[1] + d[1])]) for a, g in enumerate(grid)
                  for si, d in enumerate(shifts) if (g[0] + d[0], g[1] + d[1]) in pos]
        A = q.btensor(legs, ZZ(0, 0)).set_block_structure(blocks)
        B = q.btensor(legs, ZZ(0, 0)).set_block_structure(blocks)
        Ac = A.conj()
        row = {"sectors_per_bond_leg": len(grid), "blocks_per_operand": len(blocks)}
        for name, fn in (("AB", lambda: A.tensordot(B, ([2], [0]))), ("AAc", lambda: A.tensordot(Ac, ([0, 1], [0, 1])))):
            for mode in ("host", "device"):
                q.set_planner(mode)
                fn()
                q.planner_stats(reset=True)
                for _ in range(10):
                    fn()
                st = q.planner_stats(reset=True)
                row[f"{name}_{mode}_ms"] = 1e3 * (st["host_s"] + st["device_s"]) / 10
                row[f"{name}_{mode}_fallbacks"] = st["device_fallbacks"]
        rows.append(row)
    q.set_planner(args.planner)
    last = rows[-1]
    return {"metric": "ms per contraction plan (device planner, largest case)", "value": last["AB_device_ms"],
            "unit": "ms", "n_gpus": 1, "steps": 10, "warmup": 1, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "int64", "data": "synthetic",
            "config": {"workload": "tensordot planning of structure-only U(1)xU(1) rank-3 tensors"}, "rows": rows}


def contraction_workload(q, args):
    """Synthetic block-sparse contraction + truncation: C[a,s,u,c] = A[a,s,t,b] B[b,t,u,c]
    (bond legs of total D over U(1) charges -8..8, Gaussian section sizes, sigma 3),
    reshaped to the charge-blocked (D*2) x (2*D) matrix and decomposed by sector SVD
    truncated to D.  Each step runs both stages; L2 is flushed between steps."""
    import torch
    D = args.D
    A, B = q.networks.theta_pair(D, seed=0)
    stream = torch.cuda.ExternalStream(q.lib().qtt_get_stream())
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > L2
    out = {}
    for mode in ("f64", args.mode):
        q.set_gemm_mode(mode)
        try:
            for _ in range(args.warmup):
                C = A.tensordot(B, ([2, 3], [1, 0]))
                q.linalg.svd(C, 2, 1e-10, min_size=1, max_size=D)
            q.stats.reset()
            q.stats.enable(True)
            tc, ts = [], []
            for _ in range(args.steps):
                flush.fill_(1.0)
                torch.cuda.synchronize()
                e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
                e0.record(stream)
                C = A.tensordot(B, ([2, 3], [1, 0]))
                e1.record(stream)
                U, d, V = q.linalg.svd(C, 2, 1e-10, min_size=1, max_size=D)
                e2.record(stream)
                e2.synchronize()
                tc.append(e0.elapsed_time(e1) / 1e3)
                ts.append(e1.elapsed_time(e2) / 1e3)
            kinds = {k: q.stats.get(k) for k in q.stats.KINDS}
            q.stats.enable(False)
            dv = np.sort(np.concatenate([v for _, v in d.blocks()]))[::-1]
            out[mode] = {"contraction_s": float(np.mean(tc)), "truncation_s": float(np.mean(ts)),
                         "total_s": float(np.mean(tc) + np.mean(ts)), "kinds": kinds, "C": C, "d": dv,
                         "kept": int(len(dv))}
        finally:
            q.set_gemm_mode("f64")
    m, f = out[args.mode], out["f64"]
    # accuracy of the mixed path against the plain FP64 path on the same inputs
    cm, cf = dict(m["C"].blocks()), dict(f["C"].blocks())
    num = sum(float(np.sum((cm[k] - cf[k]) ** 2)) for k in cf)
    den = sum(float(np.sum(cf[k] ** 2)) for k in cf)
    nk = min(len(m["d"]), len(f["d"]))
    P = peaks()
    return {"metric": "s per block-sparse contraction + sector-SVD truncation (theta pair at D)",
            "value": m["total_s"], "unit": "s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": m["total_s"] * 1e3, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": f"{args.mode}+f64svd", "data": "synthetic",
            "config": {"workload": f"theta-pair contraction C[a,s,u,c] = A[a,s,t,b] B[b,t,u,c] + svd(C, 2) "
                                   f"truncated to {D}", "D": D, "charges": "U(1) -8..8, Gaussian sections sigma=3",
                       "l2": "flushed between steps (256 MB write)", "seed": 0},
            "contraction_s": m["contraction_s"], "truncation_s": m["truncation_s"],
            "fp64": {"contraction_s": f["contraction_s"], "truncation_s": f["truncation_s"], "total_s": f["total_s"]},
            "speedup_vs_fp64": f["total_s"] / m["total_s"],
            "accuracy": {"C_rel_err": (num / den) ** 0.5, "d_max_rel_err": float(np.max(np.abs(m["d"][:nk] - f["d"][:nk])) / f["d"][0]),
                         "kept_mixed": m["kept"], "kept_fp64": f["kept"]},
            "roofline_gemm": roofline("gemm", m["kinds"]["gemm"], P, args.mode, {}),
            "kernel_time_ms": {k: v["ms"] for k, v in timed_kinds(m["kinds"]).items()}}


# --------------------------------------------------------------------------- cylinder
CYL_LX, CYL_LY = 12, 6      # open length x periodic circumference
RAMP = (256, 512, 1024)     # bond dimensions swept before D


def cylinder_mpo(q):
    return q.networks.cylinder_heisenberg(CYL_LX, CYL_LY, 1.0, "snake", compress=True)


def sweeps_call(q, mpo, mps, n, mode, D, logger=None, lanczos=1):
    """ONE dmrg call of n sweeps from mps (QuantiT's update, cutoff 1e-10, max bond D;
    lanczos > 1: k-step Lanczos instead), timed with CUDA events on the library stream:
    (seconds, energy, final state)."""
    import torch
    stream = torch.cuda.ExternalStream(q.lib().qtt_get_stream())
    opts = q.algorithms.dmrg_options(cutoff=1e-10, convergence_criterion=0.0, max_bond=D, min_bond=4,
                                     maximum_iterations=n, gemm=mode, final_energy_fp64=False,
                                     lanczos_steps=lanczos)
    cur = q.networks.bMPS(list(mps), mps.orthogonality_center)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    E = q.algorithms.dmrg(mpo, cur, opts, logger)
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1) / 1e3, E, cur


def state_log(q, keep_after=None):
    """dmrg_log_sweeptime that also keeps the state after sweep `keep_after`."""
    class StateLog(q.algorithms.dmrg_log_sweeptime):
        def __init__(self):
            super().__init__()
            self.kept = None

        def it_log_all(self, step, energy, mps):
            super().it_log_all(step, energy, mps)
            if keep_after is not None and step + 1 == keep_after:
                self.kept = mps
    return StateLog()


def prepare_cylinder(q, args, seed):
    """The timed state S0: a seeded random_bMPS at RAMP[0] (canonical at site 0), swept
    along the ramp and args.warmup times at args.D in args.mode."""
    from quantit_gb300.conserved import Z
    mpo = cylinder_mpo(q)
    mps = q.networks.random_bMPS(RAMP[0], mpo, Z(0), seed=seed)
    mps.move_oc(0)
    mps.normalize_center()
    info = {"ramp": []}
    stages = [(Dr, args.ramp_sweeps) for Dr in RAMP if Dr < args.D] + [(args.D, args.converge_sweeps)]
    for Dr, n in stages:
        if n <= 0:
            continue
        t, E, mps = sweeps_call(q, mpo, mps, n, args.mode, Dr, lanczos=args.ramp_lanczos)
        info["ramp"].append({"D": Dr, "sweeps": n, "lanczos_steps": args.ramp_lanczos, "s": round(t, 2),
                             "E": E})
    log = state_log(q)
    t, E, mps = sweeps_call(q, mpo, mps, max(args.warmup, 1), args.mode, args.D, log)
    info["warmup"] = {"sweeps": max(args.warmup, 1), "s": round(t, 2), "ritz_E": log.energies,
                      "truncated_weight": log.truncated_weights, "middle_bond": log.bond_list}
    if len(log.energies) >= 2:
        info["warmup"]["last_rel_dE"] = abs(log.energies[-1] - log.energies[-2]) / abs(log.energies[-1])
    return mpo, mps, info


def sample_bonds(L, n):
    """n bonds spread evenly over 0..L-2 (the strata of the CPU sample)."""
    n = max(1, min(n, L - 1))
    return sorted({int((j + 0.5) * (L - 1) / n) for j in range(n)})


def write_cpu_sample(q, mpo, mps, outdir, nbonds, D):
    """The state, the MPO and the environments of the sampled bonds, for the oracle."""
    from quantit_gb300 import serialize
    os.makedirs(outdir, exist_ok=True)
    bonds = sample_bonds(len(mps), nbonds)
    serialize.save(os.path.join(outdir, "mpo.npz"), mpo)
    serialize.save(os.path.join(outdir, "state.npz"), mps)
    envs = q.algorithms.environments(mpo, mps, bonds)
    for b, (Le, Re) in envs.items():
        serialize.save(os.path.join(outdir, f"env_{b}.npz"), q.networks.bMPO([Le, Re]))
    with open(os.path.join(outdir, "bonds.json"), "w") as f:
        json.dump({"bonds": bonds, "L": len(mps), "Dmax": int(D)}, f)
    return bonds


def cpu_sample(path, steps, threads, offset=0):
    """Oracle bond updates (dmrg_2sites_update: theta, one-step Lanczos, truncated sector
    SVD, environment update; sources/dmrg.cpp:145-207) on the saved state, cycling over
    the sampled bonds; returns the seconds of every update per bond."""
    from oracle import qtt_oracle as o
    meta = json.load(open(os.path.join(path, "bonds.json")))
    _, mpo, _ = o.load_npz(os.path.join(path, "mpo.npz"))
    _, mps0, _ = o.load_npz(os.path.join(path, "state.npz"))
    L = len(mps0)
    h2 = o.compute_2sites_hamil(mpo)
    envs = {}
    for b in meta["bonds"]:
        _, pair, _ = o.load_npz(os.path.join(path, f"env_{b}.npz"))
        envs[b] = pair
    opt = o.DmrgOptions(cutoff=1e-10, maximum_bond=int(meta["Dmax"]), minimum_bond=4)
    bonds = meta["bonds"]
    times = {b: [] for b in bonds}
    for k in range(steps):
        b = bonds[(k + offset) % len(bonds)]
        mps = list(mps0)
        env = [None] * (L + 2)
        env[b], env[b + 3] = envs[b]
        t0 = time.perf_counter()
        o.dmrg_bond_update(mpo, h2, mps, env, b, True, opt)
        times[b].append(time.perf_counter() - t0)
    return {"bonds": bonds, "times": {str(b): v for b, v in times.items()}, "threads": threads, "L": L}


def run_cpu_sample(path, steps, threads, offset=0):
    """cpu_sample in a child process with `threads` BLAS threads (0: the default, all cores),
    starting at stratum `offset`."""
    env = dict(os.environ)
    if threads:
        for k in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
            env[k] = str(threads)
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--cpu-sample", path, "--cpu-steps",
                        str(steps), "--cpu-threads", str(threads), "--cpu-offset", str(offset)],
                       capture_output=True, text=True, env=env)
    if r.returncode != 0:
        raise RuntimeError(f"CPU sample failed: {r.stderr.strip()[-400:]}")
    return json.loads(r.stdout.strip().splitlines()[-1])


def sweep_estimate(sample):
    """Seconds per sweep from a stratified bond sample: the mean over strata of each
    stratum's mean update time, times the 2(L-2) updates of a sweep."""
    per = [float(np.mean(v)) for v in sample["times"].values() if v]
    return float(np.mean(per)) * 2 * (sample["L"] - 2), per


def cpu_host():
    model = "unknown"
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu part", "hardware")):
                model = line.split(":", 1)[1].strip()
                break
    except OSError:
        pass
    return {"cpu": model, "nproc": os.cpu_count()}


def cylinder_config(args):
    ramp = "->".join(str(d) for d in RAMP if d < args.D)
    return {"workload": f"Heisenberg 6x12 open cylinder (snake order, 72 sites), two-site DMRG sweep at "
                        f"D={args.D} after the ramp {ramp}->{args.D}, U(1) Sz=0",
            "L": CYL_LX * CYL_LY, "D": args.D,
            "model": "spin-1/2 Heisenberg J=1 on an open cylinder of length 12 and circumference 6 "
                     "(periodic), snake-ordered MPO compressed to its Schmidt rank (bond dimension 20)",
            "cutoff": 1e-10, "update": "one-step Lanczos (QuantiT two_sites_update)",
            "start": f"random_bMPS(256, seed={args.seed}); {args.ramp_sweeps} sweeps per ramp stage and "
                     f"{args.converge_sweeps} at D with {args.ramp_lanczos}-step Lanczos (state preparation); "
                     f"{args.warmup} warm-up sweeps at D with the timed update",
            "l2": "working set (MPS + environments, GBs) far larger than L2 (129 MB)"}


def reference_arm_cylinder(args, cfg):
    """The oracle's bond updates on the same state the GPU arm times (prepared on the GPU
    in a child process, outside the timed region), all host cores; each step is one bond
    update at a sampled bond; value = the stratified sweep estimate."""
    import shutil
    import tempfile
    d = tempfile.mkdtemp(prefix="qtt_cpu_sample_")
    try:
        cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--prepare-cpu-sample", d, "--D", str(args.D),
               "--warmup", str(args.warmup), "--ramp-sweeps", str(args.ramp_sweeps), "--ramp-lanczos",
               str(args.ramp_lanczos), "--converge-sweeps", str(args.converge_sweeps), "--cpu-bonds",
               str(args.cpu_bonds or max(args.steps, 1)), "--mode", args.mode, "--seed", str(args.seed)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            return {"impl": "reference", "unavailable": "state preparation failed: " + r.stderr.strip()[-300:]}
        # warm-up updates first, then the timed ones, cycling over the strata
        smp = run_cpu_sample(d, args.warmup + args.steps, 0)
        nb = len(smp["bonds"])
        flat = []
        for k in range(args.warmup + args.steps):
            b = str(smp["bonds"][k % nb])
            flat.append((b, smp["times"][b][k // nb]))
        timed = {b: [] for b in smp["times"]}
        for b, t in flat[args.warmup:]:
            timed[b].append(t)
        est, per = sweep_estimate({"times": timed, "L": smp["L"]})
        # one BLAS thread: one update at the middle stratum, against all threads at that bond
        mid = nb // 2
        bmid = str(smp["bonds"][mid])
        one = run_cpu_sample(d, 1, 1, offset=mid)
        t1 = float(one["times"][bmid][0])
        tall = float(np.mean(smp["times"][bmid]))
        est1 = est * t1 / tall
    finally:
        shutil.rmtree(d, ignore_errors=True)
    host = cpu_host()
    sample = (f"{args.steps} oracle bond updates on the same D={args.D} state, cycling over bonds "
              f"{smp['bonds']} (stratified: mean per stratum x {2 * (smp['L'] - 2)} updates per sweep); "
              f"{host['nproc']} threads, {host['cpu']}")
    return {"metric": METRIC, "value": est, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": float(np.mean([t for _, t in flat[args.warmup:]])) * 1e3,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": slim_config(cfg), "impl": "reference",
            "cpu_baseline": {"value": est, "unit": UNIT, "cores": host["nproc"], "kind": "port", "sample": sample,
                             "one_thread": {"value": est1, "unit": UNIT, "cores": 1,
                                            "sample": f"bond {bmid}: {t1:.2f} s at 1 BLAS thread against "
                                                      f"{tall:.2f} s at {host['nproc']}; the sweep estimate "
                                                      f"scaled by that ratio"}},
            "per_stratum_s": per,
            "e2e": {"value": est, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def e2e_cylinder(q, mpo, mps, args):
    """args.e2e_steps sweeps, each through the public API from host buffers: the MPS is
    uploaded, one dmrg call runs, the optimised MPS and the energy are read back."""
    host = [(t.copy_structure(), t.blocks()) for t in mps]
    oc = mps.orthogonality_center
    opts = q.algorithms.dmrg_options(cutoff=1e-10, convergence_criterion=0.0, max_bond=args.D, min_bond=4,
                                     maximum_iterations=1, gemm=args.mode, final_energy_fp64=False)
    ts, h2d, d2h, E = [], [], [], None
    for _ in range(max(1, args.e2e_steps)):
        h2d.append(sum(sum(v.nbytes for _, v in blks) for _, blks in host))
        t0 = time.perf_counter()
        dev = q.networks.bMPS([st.set_blocks(b) for st, b in host], oc)
        E = q.algorithms.dmrg(mpo, dev, opts)
        out = [t.blocks() for t in dev]
        ts.append(time.perf_counter() - t0)
        d2h.append(sum(sum(v.nbytes for _, v in blks) for blks in out) + 8)
        host = [(t.copy_structure(), blks) for t, blks in zip(dev, out)]
        oc = dev.orthogonality_center
    return {"value": float(np.mean(ts)), "unit": UNIT, "steps": len(ts), "sweep_times_s": ts,
            "h2d_bytes_per_step": int(np.mean(h2d)), "d2h_bytes_per_step": int(np.mean(d2h)), "E": E,
            "note": "one sweep per step through the public API from host buffers (state upload, one dmrg call "
                    "that also builds the environments, state and energy read back)"}


def cylinder_main(args, rank, world, local):
    import torch
    import quantit_gb300 as q
    from quantit_gb300 import replicas
    cfg = cylinder_config(args)
    cfg["parallelism"] = "replicas only" if world > 1 else "single GPU"
    t_prep = time.perf_counter()
    mpo, S0, info = prepare_cylinder(q, args, replicas.replica_seed(args.seed, rank))
    info["prep_wall_s"] = round(time.perf_counter() - t_prep, 1)
    # the timed region: args.steps mixed sweeps in one dmrg call
    q.stats.reset()
    q.stats.enable(True)
    sampler = ClockSampler(local)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    launches0 = q.stats.launches()
    log = state_log(q, keep_after=args.compare_sweeps)
    q.planner_stats(reset=True)
    sampler.start()
    t_mix, _, S_mix = sweeps_call(q, mpo, S0, args.steps, args.mode, args.D, log)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    plan_st = q.planner_stats(reset=True)
    launches = q.stats.launches() - launches0
    kinds = {k: q.stats.get(k) for k in q.stats.KINDS}
    q.stats.enable(False)
    t_step = replicas.max_over_ranks([t_mix / args.steps])[0]
    line = {"metric": METRIC, "value": t_step / world, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": f"{args.mode}+f64svd+f64" if args.mode != "f64" else "f64",
            "data": "synthetic", "config": dict(cfg, mode=args.mode), "gpu_launches": int(launches),
            "clocks": clocks, "planner": dict(plan_st, mode=args.planner)}
    P = peaks()
    pc = {}
    dom = max((k for k in timed_kinds(kinds) if k != "svd_fp64"), key=lambda k: kinds[k]["ms"])
    line["roofline"] = roofline(dom, kinds[dom], P, args.mode, pc)
    if dom == "svd":
        line["roofline"]["stages"] = svd_stages(kinds, args.mode, pc)
        if args.mode == "tf32x3" and args.D == 2048:
            line["roofline"]["traffic"] = SVD_TRAFFIC_MID_THETA
            line["roofline"]["traffic_of"] = "the mid-bond decomposition (ncu, profiles/)"
    line["roofline_gemm"] = roofline("gemm", kinds["gemm"], P, args.mode, pc)
    line["kernel_time_ms"] = {k: round(v["ms"], 1) for k, v in timed_kinds(kinds).items()}
    line["sweeps"] = {"times_s": [round(x, 3) for x in log.time_list], "middle_bond": log.bond_list,
                      "truncated_weight": log.truncated_weights, "ritz_E": log.energies}
    # the same state in FP64: compare_sweeps sweeps, against the first as many timed mixed sweeps
    if args.mode != "f64" and args.compare_f64:
        n = max(1, min(args.compare_sweeps, args.steps))
        lf = state_log(q)
        q.stats.reset()
        q.stats.enable(True)
        _, _, S64 = sweeps_call(q, mpo, S0, n, "f64", args.D, lf)
        k64 = {k: q.stats.get(k) for k in q.stats.KINDS}
        q.stats.enable(False)
        # the plain path against its own roofline: FP64 GEMMs and FP64 Jacobi against cuBLAS DGEMM
        line["roofline_f64"] = {k: roofline(k, k64[k], P, "f64", pc) for k in ("gemm", "svd")}
        if line["roofline_f64"]["svd"]:
            line["roofline_f64"]["svd"]["stages"] = svd_stages(k64, "f64", pc)
        line["kernel_time_ms_f64"] = {k: round(v["ms"], 1) for k, v in timed_kinds(k64).items()}
        t64 = lf.time_list[1:] if len(lf.time_list) > 1 else lf.time_list
        tm = log.time_list[1:] if len(log.time_list) > 1 else log.time_list
        Sm = log.kept if log.kept is not None else S_mix
        E64, _ = fp64_energy(q, mpo, S64)
        Em, _ = fp64_energy(q, mpo, Sm)
        line["vs_fp64"] = {
            "fp64_s_per_sweep": float(np.mean(t64)), "mixed_s_per_sweep": float(np.mean(tm)),
            "speedup_vs_fp64": float(np.mean(t64)) / float(np.mean(tm)),
            "dE_per_site": abs(Em - E64) / (CYL_LX * CYL_LY), "E_fp64": E64, "E_mixed": Em, "sweeps": n,
            "truncated_weight_fp64": lf.truncated_weights, "truncated_weight_mixed": log.truncated_weights[:n],
            "ritz_E_fp64": lf.energies, "ritz_E_mixed": log.energies[:n],
            "note": "both from the timed state; per-sweep wall times of the sweeps after the first of each call; "
                    "energies are FP64 <psi|H|psi>/<psi|psi> after the same number of sweeps"}
    line["state"] = info
    line["e2e"] = e2e_cylinder(q, mpo, S0, args)
    if rank == 0 and not args.no_cpu_baseline:
        import shutil
        import tempfile
        d = tempfile.mkdtemp(prefix="qtt_cpu_sample_")
        try:
            write_cpu_sample(q, mpo, S0, d, args.cpu_bonds or args.cpu_steps, args.D)
            smp = run_cpu_sample(d, args.cpu_steps, 0)
            est, per = sweep_estimate(smp)
            host = cpu_host()
            line["cpu_baseline"] = {"value": est, "unit": UNIT, "cores": host["nproc"], "kind": "port",
                                    "sample": f"{args.cpu_steps} oracle bond updates on the timed state at bonds "
                                              f"{smp['bonds'][:args.cpu_steps]} (stratified estimate x "
                                              f"{2 * (smp['L'] - 2)} updates per sweep), {host['cpu']}"}
        except Exception as e:  # reported, never hidden
            line["cpu_baseline"] = {"error": repr(e)}
        finally:
            shutil.rmtree(d, ignore_errors=True)
    if rank == 0 and args.serving_requests:
        try:
            line["serving"] = serving_section(q, args, args.serving_requests)
        except Exception as e:  # reported, never hidden
            line["serving"] = {"error": repr(e)}
    tune = q.autotune_report().splitlines()
    line["autotune_classes"] = len(tune)
    if rank == 0:
        print("autotune:\n  " + "\n  ".join(tune), file=sys.stderr)
        print("full line: " + json.dumps(line), file=sys.stderr)
        print(json.dumps(slim_cylinder_line(line)))


def sig(x, n=4):
    """x with floats rounded to n significant digits (recursively)."""
    if isinstance(x, float):
        return float(f"{x:.{n}g}") if np.isfinite(x) else x
    if isinstance(x, dict):
        return {k: sig(v, n) for k, v in x.items()}
    if isinstance(x, (list, tuple)):
        return [sig(v, n) for v in x]
    return x


def slim_config(cfg):
    """The printed config of the cylinder workload, the same for both arms (the
    arithmetic is in `dtype`)."""
    return {"workload": cfg["workload"], "L": cfg["L"], "D": cfg["D"], "cutoff": cfg["cutoff"],
            "mpo": "compressed to bond dim 20", "update": "one-step Lanczos", "l2": "working set >> L2",
            "parallelism": cfg["parallelism"]}


def slim_cylinder_line(line):
    """The printed line: every key of the contract, the comparison with FP64, the
    roofline objects and the serving summary, with floats at 4 significant digits
    (energies at 12) and without the per-sweep lists and notes, so the line stays
    under 3 KB; the full line goes to stderr."""
    keep = ("kernel", "bound", "achieved", "peak", "unit", "frac", "traffic", "traffic_of", "per_launch_ms")
    out = {k: line[k] for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                                "higher_is_better", "scaling", "vs_baseline", "dtype", "data")}
    out["config"] = slim_config(line["config"])
    out["gpu_launches"] = line["gpu_launches"]
    out["clocks"] = {k: line["clocks"].get(k) for k in ("sm_mhz", "sm_max_mhz", "reasons")}
    def stages(r):  # {stage: [ms, Jacobi TFLOP/s, fraction of the stage's cuBLAS peak]}
        return {n.split("_")[0]: sig([v["ms"], v["jacobi_tflops"], v["frac"]]) for n, v in r["stages"].items()}
    for k in ("roofline", "roofline_gemm"):
        if isinstance(line.get(k), dict):
            out[k] = sig({a: b for a, b in line[k].items() if a in keep})
            if line[k].get("stages"):
                out[k]["stages"] = stages(line[k])
    if isinstance(line.get("roofline_f64"), dict):
        out["roofline_f64"] = {k: sig({a: b for a, b in v.items() if a in ("achieved", "unit", "frac")})
                               for k, v in line["roofline_f64"].items() if v}
        sv = line["roofline_f64"].get("svd")
        if sv and sv.get("stages"):
            out["roofline_f64"]["svd"]["stages"] = stages(sv)
    for k in ("kernel_time_ms", "kernel_time_ms_f64"):
        if k in line:
            out[k] = {a: round(b) for a, b in line[k].items()}
    out["sweep_times_s"] = sig(line["sweeps"]["times_s"])
    v = line.get("vs_fp64")
    if isinstance(v, dict):
        out["vs_fp64"] = dict(sig({k: v[k] for k in ("fp64_s_per_sweep", "mixed_s_per_sweep", "speedup_vs_fp64",
                                                    "dE_per_site", "sweeps")}),
                              E_fp64=sig(v["E_fp64"], 12), E_mixed=sig(v["E_mixed"], 12),
                              trunc_fp64=sig(max(v["truncated_weight_fp64"])),
                              trunc_mixed=sig(max(v["truncated_weight_mixed"])))
    st = line.get("state", {})
    if st:
        out["state"] = {"ramp": [[r["D"], r["sweeps"], sig(r["s"], 3)] for r in st.get("ramp", [])],
                        "prep_s": st.get("prep_wall_s")}
    e = line.get("e2e")
    if isinstance(e, dict):
        out["e2e"] = sig({k: e[k] for k in ("value", "unit", "steps", "h2d_bytes_per_step", "d2h_bytes_per_step")
                          if k in e})
    c = line.get("cpu_baseline")
    if isinstance(c, dict):
        out["cpu_baseline"] = sig({k: c[k] for k in ("value", "unit", "cores", "kind", "sample", "error") if k in c})
        if "sample" in out["cpu_baseline"]:
            out["cpu_baseline"]["sample"] = out["cpu_baseline"]["sample"][:150]
    sv = line.get("serving")
    if isinstance(sv, dict):
        out["serving"] = slim_serving(sv)
    return out


def slim_serving(sv):
    if "error" in sv:
        return sv
    f = sv.get("serial_fp64", {})
    return sig({"requests": sv["requests"], "rate_per_s": sv["rate_per_s"], "offered_load": sv.get("offered_load"),
                "solves_per_s": sv["solves_per_s"], "p50_s": sv["p50_s"], "p99_s": sv["p99_s"],
                "capacity_solves_per_s": sv.get("capacity", {}).get("solves_per_s"),
                "trunc_max": sv["truncated_weight"]["max"], "errors": sv["errors"],
                "fp64_serial_solves_per_s": f.get("solves_per_s"), "fp64_sample": f.get("sample"),
                "dE_per_site_max": f.get("dE_per_site", {}).get("max"),
                "trunc_fp64_max": f.get("truncated_weight", {}).get("max"),
                "capacity_vs_serial_fp64": sv.get("capacity_vs_serial_fp64")})


def main():
    args = parse()
    if args.cpu_sample:
        print(json.dumps(cpu_sample(args.cpu_sample, args.cpu_steps, args.cpu_threads, args.cpu_offset)))
        return
    if args.prepare_cpu_sample:
        import quantit_gb300 as q
        q.ensure_init(0)
        if args.D is None:
            args.D = 2048
        mpo, S0, _ = prepare_cylinder(q, args, args.seed)
        write_cpu_sample(q, mpo, S0, args.prepare_cpu_sample, args.cpu_bonds or 6, args.D)
        return
    rank, world, local = dist_env()
    hub = args.model == "hubbard"
    cyl = args.model == "cylinder"
    if cyl and args.workload == "contraction":
        args.model, cyl = "heisenberg", False   # the theta-pair microbench
    if args.L is None:
        args.L = 72 if cyl else (64 if hub else 32)
    if args.D is None:
        args.D = 1024 if hub else 2048
    if cyl and args.workload == "dmrg":
        if args.impl == "reference":
            if rank == 0:
                cfg = dict(cylinder_config(args), parallelism="single GPU")
                print(json.dumps(reference_arm_cylinder(args, cfg)))
            return
        import torch
        torch.cuda.set_device(local)
        if world > 1:
            import torch.distributed as dist
            dist.init_process_group("nccl")
        import quantit_gb300 as q
        q.ensure_init(local)
        q.set_jacobi_kernel(args.jacobi)
        q.set_planner(args.planner)
        if args.svd_deflation is not None:
            q.set_svd_deflation(bool(args.svd_deflation))
        cylinder_main(args, rank, world, local)
        if world > 1:
            torch.distributed.destroy_process_group()
        return
    if hub:
        cfg = {"workload": f"Fermi-Hubbard chain L={args.L}, U=8, half filling, two-site DMRG sweep at D={args.D}, "
                           "U(1)xU(1) (N, 2Sz)", "L": args.L, "D": args.D,
               "model": "Fermi-Hubbard open chain t=1 U=8 mu=0, N=L, Sz=0"}
    else:
        cfg = {"workload": f"Heisenberg chain L={args.L}, two-site DMRG sweep at D={args.D}, U(1) Sz=0",
               "L": args.L, "D": args.D, "model": "spin-1/2 Heisenberg open chain (J=1 AFM)"}
    cfg.update({
           "cutoff": 1e-10, "update": "one-step Lanczos (QuantiT two_sites_update)",
           "l2": "working set (MPS + environments) far larger than L2 (129 MB)",
           "parallelism": "replicas only" if world > 1 else "single GPU"})
    if args.impl == "reference":
        if rank == 0:
            if hub:
                print(json.dumps({"impl": "reference", "unavailable": "the CPU sampler restates the Heisenberg "
                                  "bond update only; this model runs on the GPU paths"}))
            else:
                print(json.dumps(reference_arm(args, cfg)))
        return

    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    import quantit_gb300 as q
    q.ensure_init(local)
    q.set_jacobi_kernel(args.jacobi)
    q.set_planner(args.planner)
    if args.svd_deflation is not None:
        q.set_svd_deflation(bool(args.svd_deflation))
    if args.workload in ("contraction", "svd", "planner"):
        line = {"contraction": contraction_workload, "svd": svd_workload,
                "planner": planner_workload}[args.workload](q, args)
        if rank == 0:
            print(json.dumps(line))
        if world > 1:
            dist.destroy_process_group()
        return
    if args.workload == "serving":
        sv = serving_section(q, args, args.serving_requests if args.serving_requests is not None else 200)
        if rank == 0:
            print(json.dumps({"metric": "solves/s (XXZ ground states, Poisson arrivals) at p99 latency",
                              "value": sv["solves_per_s"], "unit": "solves/s", "n_gpus": world, "steps": 1,
                              "warmup": 0, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                              "dtype": f"{args.mode if args.mode != 'f64' else 'tf32x3'}+f64svd+f64",
                              "data": "synthetic",
                              "config": {"workload": "serving: Poisson stream of XXZ chain ground-state solves",
                                         "parallelism": "replicas only" if world > 1 else "single GPU"},
                              "serving": sv}))
        if world > 1:
            dist.destroy_process_group()
        return
    from quantit_gb300 import replicas
    mpo, mps0 = build_state(q, args.L, args.D, seed=replicas.replica_seed(0, rank), model=args.model)
    _, _, mps1 = run_sweeps(q, mpo, mps0, args.warmup, args.mode, args.D)
    q.stats.reset()
    q.stats.enable(True)
    sampler = ClockSampler(local)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    launches0 = q.stats.launches()
    q.planner_stats(reset=True)
    sampler.start()
    t0 = time.perf_counter()
    Es, ts, mps2 = run_sweeps(q, mpo, mps1, args.steps, args.mode, args.D)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    clocks = sampler.stop()
    plan_st = q.planner_stats(reset=True)
    launches = q.stats.launches() - launches0
    kinds = {k: q.stats.get(k) for k in q.stats.KINDS}
    q.stats.enable(False)
    t_step = float(np.mean(ts))
    # replicas: the slowest rank's times; the whole job's seconds per sweep divide the
    # slowest rank's sweep time by the sweeps all ranks ran in it
    from quantit_gb300 import replicas
    wall, t_step = replicas.max_over_ranks([wall, t_step])
    job_per_sweep = t_step / world
    E_mixed, t_eval = fp64_energy(q, mpo, mps2)
    cmp = None
    if args.mode != "f64" and args.compare_f64:
        _, t64, mps64 = run_sweeps(q, mpo, mps1, args.steps, "f64", args.D)
        E64, _ = fp64_energy(q, mpo, mps64)
        cmp = {"fp64_s_per_sweep": float(np.mean(t64)), "speedup_vs_fp64": float(np.mean(t64)) / t_step,
               "dE_per_site": abs(E_mixed - E64) / args.L, "E_fp64": E64, "E_mixed": E_mixed,
               "energies": "FP64 <psi|H|psi>/<psi|psi> of each path's final state after the same sweeps",
               "bond_dims": {"mixed_max": bond_max(mps2), "fp64_max": bond_max(mps64),
                             "mixed_sum": bond_sum(mps2), "fp64_sum": bond_sum(mps64)}}
    e2e = e2e_sweep(q, mpo, mps1, args)
    P = peaks()
    pc = {}
    dom = max((k for k in timed_kinds(kinds) if k != "svd_fp64"), key=lambda k: kinds[k]["ms"])
    line = {"metric": METRIC, "value": job_per_sweep, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if args.mode == "f64" else f"{args.mode}+f64svd+f64",
            "data": "synthetic", "config": dict(cfg, mode=args.mode, jacobi=args.jacobi), "ritz_energies": Es,
            "energy_fp64": E_mixed, "energy_per_site": E_mixed / args.L, "fp64_energy_eval_s": t_eval,
            "sweep_times_s": ts, "wall_s": wall,
            "kernel_time_ms": {k: v["ms"] for k, v in timed_kinds(kinds).items()},
            "roofline": roofline(dom, kinds[dom], P, args.mode, pc),
            "roofline_gemm": roofline("gemm", kinds["gemm"], P, args.mode, pc),
            "gpu_launches": int(launches), "clocks": clocks, "e2e": e2e,
            "planner": dict(plan_st, mode=args.planner, note="calls and host wall seconds of the contraction "
                                                             "planner over the timed sweeps")}
    if cmp:
        line["vs_fp64"] = cmp
    # the autotuner's decisions go to stderr: one line each would push the metric keys
    # out of the tail a log reader keeps
    tune = q.autotune_report().splitlines()
    line["autotune_classes"] = len(tune)
    if rank == 0:
        print("autotune:\n  " + "\n  ".join(tune), file=sys.stderr)
    if rank == 0 and not args.no_cpu_baseline and hub:
        line["cpu_baseline"] = None  # the oracle sampler restates the Heisenberg bond update only
    elif rank == 0 and not args.no_cpu_baseline:
        try:
            s = CpuSampler(args.L, args.D)
            per = [s.bond() for _ in range(2)]
            line["cpu_baseline"] = {"value": float(np.mean(per)) * s.factor, "unit": UNIT, "cores": os.cpu_count(),
                                    "kind": "port",
                                    "sample": f"2 mid-chain bond updates at D={args.D} ({np.mean(per):.2f} s each) "
                                              f"x {s.factor:.1f} size-weighted bonds per sweep"}
        except Exception as e:  # reported, never hidden
            line["cpu_baseline"] = {"error": repr(e)}
    if rank == 0 and args.serving_requests and not hub:
        try:
            line["serving"] = serving_section(q, args, args.serving_requests)
        except Exception as e:  # reported, never hidden
            line["serving"] = {"error": repr(e)}
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
