"""Benchmark: seconds per two-site DMRG sweep at bond dimension D (default 2048).

Workload: open spin-1/2 Heisenberg chain (U(1) total-Sz = 0), two-site DMRG with
QuantiT's one-step Lanczos update, SVD cutoff 1e-10, max bond D, started from a
seeded random MPS already at bond dimension D (sector dims = charge
multiplicities capped to D) brought to right-canonical form.  One step = one
full sweep (2(L-2) bond updates).  Synthetic data: no dataset is involved.

Arms:
  (default)          our CUDA path through libqtt_gb300.so (qtt_dmrg); block GEMMs
                     in --mode (f64 = the plain drop-in, tf32x3 / bf16x3 = split
                     precision on tcgen05); FP64 everywhere else.
  --impl reference   the CPU oracle (numpy restatement of QuantiT's algorithm) on
                     the host cores, each step a bounded sample of bond updates
                     extrapolated to a sweep.

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
    p.add_argument("--L", type=int, default=32)
    p.add_argument("--D", type=int, default=2048)
    p.add_argument("--mode", default="f64", choices=["f64", "tf32x3", "bf16x3"])
    p.add_argument("--compare-f64", type=int, default=1, help="also time FP64 sweeps from the same state")
    p.add_argument("--cpu-sample-bonds", type=int, default=2)
    p.add_argument("--no-cpu-baseline", action="store_true")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


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


def build_state(q, L, D, seed=0):
    mpo = q.networks.heisenberg(L)
    mps = q.networks.random_bmps(L, D, seed=seed)
    mps.move_oc(0)
    mps.normalize_center()
    return mpo, mps


def run_sweeps(q, mpo, mps, n, mode, stream_events=True):
    """n single sweeps; returns (energies, per-sweep seconds, final mps) timed with CUDA
    events on the library's stream."""
    import torch
    stream = torch.cuda.ExternalStream(q.lib().qtt_get_stream())
    opts = q.algorithms.dmrg_options(cutoff=1e-10, convergence_criterion=0.0, max_bond=DMAX[0], min_bond=4,
                                     maximum_iterations=1, gemm=mode)
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


DMAX = [2048]


def fp64_peak_tflops():
    """cuBLAS DGEMM throughput measured here (the FP64 roofline denominator)."""
    import torch
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
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


def cpu_baseline(L, D, sample_bonds):
    """The oracle (numpy; BLAS threads = all host cores) on a bounded sample: a few
    mid-chain bond updates at bond dimension D, extrapolated to a sweep."""
    from oracle import qtt_oracle as o
    rng = np.random.default_rng(0)
    mpo = o.heisenberg_mpo(L)
    mps = o.random_mps(L, D, [1, -1], 0, rng)
    mid = L // 2 - 1
    # a right-canonical right half and a left-canonical left half are not needed for
    # timing: the work of a bond update depends only on the block shapes
    env = [None] * (L + 2)
    env[0] = o.trivial_edge((mps[0], 0), (mpo[0], 0))
    env[L + 1] = o.trivial_edge((mps[-1], 2), (mpo[-1], 2))
    for i in range(mid):
        env[i + 1] = o.compute_left_env(mpo[i], mps[i], env[i])
    for i in range(L - 1, mid + 1, -1):
        env[i + 1] = o.compute_right_env(mpo[i], mps[i], env[i + 2])
    h2 = o.compute_2sites_hamil(mpo)
    opts = o.DmrgOptions(cutoff=1e-10, maximum_bond=D, minimum_bond=4)
    t0 = time.perf_counter()
    done = 0
    for k in range(sample_bonds):
        o.dmrg_bond_update(mpo, h2, mps, env, mid, True, opts)
        done += 1
        if time.perf_counter() - t0 > 30:
            break
        mps_mid = mid  # stay on the same bond: redo the update from the new state
    per_bond = (time.perf_counter() - t0) / done
    # bonds of a sweep weighted by their size relative to the mid bond (Sigma D_b^3 / D_mid^3)
    from quantit_gb300.networks import bond_sectors  # pure-python structure helper
    bonds = bond_sectors(L, D, [1, -1], 0)
    w = [sum(m ** 3 for m in b.values()) for b in bonds]
    wm = w[mid]
    sweep_bonds = list(range(0, L - 2)) + list(range(L - 2, 0, -1))
    factor = sum(w[b] / wm for b in sweep_bonds)
    return per_bond * factor, per_bond, done, factor


def main():
    args = parse()
    rank, world, local = dist_env()
    DMAX[0] = args.D
    cfg = {"workload": f"Heisenberg chain L={args.L}, two-site DMRG sweep at D={args.D}, U(1) Sz=0",
           "L": args.L, "D": args.D, "model": "spin-1/2 Heisenberg open chain (J=1 AFM)",
           "cutoff": 1e-10, "update": "one-step Lanczos (QuantiT two_sites_update)",
           "l2": "working set (MPS + environments) far larger than L2 (129 MB)",
           "parallelism": "replicas only" if world > 1 else "single GPU"}
    if args.impl == "reference":
        if rank != 0:
            return
        t_sweep, per_bond, n, factor = cpu_baseline(args.L, args.D, args.cpu_sample_bonds)
        ncores = os.cpu_count()
        line = {"metric": METRIC, "value": t_sweep, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": t_sweep * 1e3, "higher_is_better": False,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": cfg,
                "impl": "reference",
                "cpu_baseline": {"value": t_sweep, "unit": UNIT, "cores": ncores, "kind": "port",
                                 "sample": f"{n} mid-chain bond update(s) at D={args.D} ({per_bond:.2f} s each) "
                                           f"x {factor:.1f} size-weighted bonds per sweep"},
                "e2e": {"value": t_sweep, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    import quantit_gb300 as q
    q.ensure_init(local)
    mpo, mps0 = build_state(q, args.L, args.D, seed=rank)
    # warm-up sweeps in the measured mode
    _, _, mps1 = run_sweeps(q, mpo, mps0, args.warmup, args.mode)
    q.stats.reset()
    q.stats.enable(True)
    sampler = ClockSampler(local)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    launches0 = q.stats.launches()
    sampler.start()
    t0 = time.perf_counter()
    Es, ts, _ = run_sweeps(q, mpo, mps1, args.steps, args.mode)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    clocks = sampler.stop()
    launches = q.stats.launches() - launches0
    kinds = {k: q.stats.get(k) for k in q.stats.KINDS}
    q.stats.enable(False)
    t_step = float(np.mean(ts))
    if world > 1:
        t = torch.tensor([wall], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        wall = float(t.item())
    # FP64 plain comparison from the same state
    cmp = None
    if args.mode != "f64" and args.compare_f64:
        E64, t64, _ = run_sweeps(q, mpo, mps1, args.steps, "f64")
        cmp = {"fp64_s_per_sweep": float(np.mean(t64)), "speedup_vs_fp64": float(np.mean(t64)) / t_step,
               "dE_per_site": abs(Es[-1] - E64[-1]) / args.L, "E_fp64": E64[-1]}
    # e2e: one sweep through the C-ABI from host buffers, results back to the host
    e2e = e2e_sweep(q, mpo, mps1, args)
    # roofline for the dominant kernel class
    dom = max(kinds, key=lambda k: kinds[k]["ms"])
    P = peaks()
    roof = roofline(dom, kinds[dom], P)
    line = {"metric": METRIC, "value": t_step, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if args.mode == "f64" else f"{args.mode}+f64",
            "data": "synthetic", "config": dict(cfg, mode=args.mode), "energies": Es,
            "energy_per_site": Es[-1] / args.L, "sweep_times_s": ts, "wall_s": wall,
            "kernel_time_ms": {k: v["ms"] for k, v in kinds.items()}, "roofline": roof,
            "gpu_launches": int(launches), "clocks": clocks, "e2e": e2e}
    if cmp:
        line["vs_fp64"] = cmp
    if rank == 0 and not args.no_cpu_baseline:
        try:
            t_sweep, per_bond, n, factor = cpu_baseline(args.L, args.D, args.cpu_sample_bonds)
            line["cpu_baseline"] = {"value": t_sweep, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                                    "sample": f"{n} mid-chain bond update(s) at D={args.D} ({per_bond:.2f} s each) "
                                              f"x {factor:.1f} size-weighted bonds per sweep"}
        except Exception as e:  # report, never hide
            line["cpu_baseline"] = {"error": repr(e)}
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


def roofline(kind, st, P):
    if st["ms"] <= 0:
        return None
    per_launch_ms = st["ms"] / max(st["launches"], 1)
    if kind in ("gemm", "svd"):
        mode_tc = False
        achieved = st["work"] / (st["ms"] / 1e3) / 1e12
        peak = P.get("fp64_tflops")
        src = "FP64 peak (cuBLAS DGEMM, measured in this run)"
        try:
            peak = fp64_peak_tflops()
        except Exception:
            peak = 1.25
            src = "FP64 nominal 1.25 TFLOP/s (fallback)"
        return {"kernel": kind, "bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                "frac": achieved / peak, "traffic": None, "peak_source": src,
                "per_launch_ms": per_launch_ms, "launches": st["launches"]}
    achieved = st["work"] / (st["ms"] / 1e3) / 1e9
    peak = P.get("hbm_gbs", 6800.0)
    return {"kernel": kind, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "traffic": None, "peak_source": "MEASURED_PEAKS.json hbm_gbs",
            "per_launch_ms": per_launch_ms, "launches": st["launches"]}


def e2e_sweep(q, mpo, mps, args):
    """One sweep through the public API with the MPS uploaded from host buffers and
    the optimised MPS + energy read back to the host inside the timed region."""
    host = [(t.copy_structure(), t.blocks()) for t in mps]
    h2d = sum(sum(v.nbytes for _, v in blks) for _, blks in host)
    t0 = time.perf_counter()
    dev = q.networks.bMPS([shape.set_blocks(blks) for shape, blks in
                           [(s.copy_structure(), b) for s, b in host]], 0)
    opts = q.algorithms.dmrg_options(cutoff=1e-10, convergence_criterion=0.0, max_bond=args.D, min_bond=4,
                                     maximum_iterations=1, gemm=args.mode)
    E = q.algorithms.dmrg(mpo, dev, opts)
    out = [t.blocks() for t in dev]
    dt = time.perf_counter() - t0
    d2h = sum(sum(v.nbytes for _, v in blks) for blks in out) + 8
    return {"value": dt, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h), "E": E}


if __name__ == "__main__":
    main()
