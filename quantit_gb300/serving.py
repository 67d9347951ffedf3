"""Continuous-batching ground-state server.

Requests (an XXZ chain length, anisotropy, bond dimension and seed) arrive over
time.  They wait in arrival order and are admitted while a solve slot is free and
their estimated device footprint fits the memory budget.  Each admitted request
runs on a worker thread with its own library stream.  Its MPS and environments
stay resident in device memory for the whole solve, and ``qtt_dmrg`` releases the
interpreter lock, so admitted solves overlap on the GPU.  A finished solve frees
its slot and memory, and the next waiting requests are admitted at once.

The reference has no serving layer; the solve itself is ``quantit::dmrg``
(sources/dmrg.cpp:219-273) on ``random_bMPS`` (sources/MPT.cpp:424-551) for the
Heisenberg/XXZ MPO (sources/models.cpp:38-58).
"""
import collections
import ctypes as C
import math
import queue
import threading
import time

import numpy as np

from . import _lib, algorithms, networks


class SolveRequest:
    """One ground-state request: XXZ chain of length L, anisotropy delta, bond dimension
    D; ``resume`` names a block-list file (serialize.save) holding the MPS to start from
    instead of the seeded random one."""

    __slots__ = ("rid", "L", "delta", "D", "seed", "arrival", "resume")

    def __init__(self, rid, L, delta, D, seed, arrival=0.0, resume=None):
        self.rid, self.L, self.delta, self.D, self.seed, self.arrival = rid, int(L), float(delta), int(D), int(seed), float(arrival)
        self.resume = resume


class SolveResult:
    __slots__ = ("rid", "L", "delta", "D", "energy", "sweeps", "truncated_weight", "arrival", "admitted", "started",
                 "done", "footprint", "error")

    def __init__(self, req, footprint):
        self.rid, self.L, self.delta, self.D = req.rid, req.L, req.delta, req.D
        self.energy = math.nan
        self.sweeps = 0
        self.truncated_weight = math.nan
        self.arrival = req.arrival
        self.admitted = self.started = self.done = math.nan
        self.footprint = footprint
        self.error = None

    @property
    def latency(self):
        return self.done - self.arrival

    @property
    def service(self):
        return self.done - self.started


def poisson_requests(n, rate, seed=0, lengths=(16, 32, 64, 128), bonds=(32, 64, 128, 256, 512), delta=(0.0, 2.0)):
    """n requests with exponential inter-arrival times (mean 1/rate seconds), L, D
    and delta drawn uniformly, each with its own MPS seed."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, size=n)) if rate > 0 else np.zeros(n)
    out = []
    for i in range(n):
        out.append(SolveRequest(i, int(rng.choice(lengths)), float(rng.uniform(*delta)), int(rng.choice(bonds)),
                                seed=int(rng.integers(0, 2 ** 31 - 1)), arrival=float(t[i])))
    return out


def footprint_bytes(L, D, phys_q=(1, -1), target=0, w=5):
    """Estimated peak device bytes of one solve: the MPS, every environment
    (w-wide, one per bond), and the working set of the largest two-site update
    (theta, H theta, the Lanczos vector, the matvec intermediates ~w thetas and the
    sector-SVD buffers ~4 thetas), with a 25% margin."""
    bonds = networks.bond_sectors(L, D, list(phys_q), target)
    edge = {0: 1}
    mps = env = 0
    theta = 0
    for i in range(L):
        left = edge if i == 0 else bonds[i - 1]
        right = {target: 1} if i == L - 1 else bonds[i]
        mps += sum(m * right.get(q + s, 0) for q, m in left.items() for s in phys_q)
        if i < L - 1:
            env += w * sum(m * m for m in bonds[i].values())
        if 0 < i < L - 1:
            rows = collections.Counter()
            for q, m in left.items():
                for s in phys_q:
                    rows[q + s] += m
            nxt = {target: 1} if i + 1 == L - 1 else bonds[i + 1]
            cols = collections.Counter()
            for q, m in nxt.items():
                for s in phys_q:
                    cols[q - s] += m
            theta = max(theta, sum(rows[c] * cols[c] for c in rows))
    return int(1.25 * 8 * (mps + env + (2 * w + 8) * theta))


def device_memory():
    """(free, total) device bytes of the calling thread's device."""
    f, t = C.c_int64(), C.c_int64()
    _lib.call("qtt_device_memory", C.byref(f), C.byref(t))
    return f.value, t.value


def ramp_stages(D, first=32):
    """Bond dimensions a solve passes through: D/4 and D/2 where they are at least
    ``first``, then D."""
    return [d for d in (D // 4, D // 2) if d >= first] + [int(D)]


def solve(req, gemm="tf32x3", convergence=1e-8, max_sweeps=40, cutoff=1e-10, checkpoint_dir=None, lanczos_steps=4,
          ramp=True, ramp_convergence=1e-6, ramp_sweeps=10):
    """One request on the calling thread: build the MPO and the seeded random MPS (or
    read the request's checkpoint), bring the MPS to canonical form (move_oc(0) and
    normalisation, in FP64: a raw random MPS's environments shrink like D^-i and
    leave the FP64 range on long chains), run two-site DMRG to the relative energy
    convergence (``lanczos_steps``-step Lanczos per bond, matvecs replayed from CUDA
    graphs), write the optimised MPS to ``checkpoint_dir`` when given, return
    (E, sweeps, truncated weight): the truncated weight is the largest relative
    discarded weight sum(dropped s^2) / sum(s^2) over the bonds of the last sweep.

    With ``ramp`` a random start begins at the first of ``ramp_stages(D)`` and is swept
    at each smaller bond dimension to ``ramp_convergence`` (at most ``ramp_sweeps``
    sweeps) before the sweeps at D, which run to ``convergence`` as without it: most
    sweeps then run at the cheaper bond dimensions.  The sweep count returned covers all
    stages."""
    from . import serialize
    mpo = networks.xxz(req.L, req.delta)
    stages = [req.D]
    if getattr(req, "resume", None):
        mps = serialize.load(req.resume)
        if len(mps) != req.L:
            raise ValueError("the checkpoint's length differs from the request's")
    else:
        if ramp:
            stages = ramp_stages(req.D)
        mps = networks.random_bmps(req.L, stages[0], seed=req.seed)
    mps.move_oc(0)
    mps.normalize_center()
    sweeps = 0
    for Dk in stages[:-1]:
        log = algorithms.dmrg_log_sweeptime()
        algorithms.dmrg(mpo, mps, algorithms.dmrg_options(
            cutoff=cutoff, convergence_criterion=ramp_convergence, max_bond=Dk, min_bond=1,
            maximum_iterations=ramp_sweeps, gemm=gemm, final_energy_fp64=True, lanczos_steps=lanczos_steps), log)
        sweeps += len(log.energies)
    opts = algorithms.dmrg_options(cutoff=cutoff, convergence_criterion=convergence, max_bond=req.D, min_bond=1,
                                   maximum_iterations=max_sweeps, gemm=gemm, final_energy_fp64=True,
                                   lanczos_steps=lanczos_steps)
    log = algorithms.dmrg_log_sweeptime()
    E = algorithms.dmrg(mpo, mps, opts, log)
    if checkpoint_dir:
        import os
        serialize.save(os.path.join(checkpoint_dir, f"request_{req.rid}.npz"), mps)
    return E, sweeps + len(log.energies), (log.truncated_weights[-1] if log.truncated_weights else 0.0)


class ServingEngine:
    """Admission by slots and memory footprint, worker threads with one stream each."""

    def __init__(self, slots=8, memory_budget=None, gemm="tf32x3", convergence=1e-8, max_sweeps=40, cutoff=1e-10,
                 device=0, solver=None, footprint=None, checkpoint_dir=None, lanczos_steps=4):
        if slots < 1:
            raise ValueError("a serving engine needs at least one slot")
        self.slots = int(slots)
        self.device = int(device)
        self.solve_args = dict(gemm=gemm, convergence=convergence, max_sweeps=max_sweeps, cutoff=cutoff,
                               lanczos_steps=lanczos_steps)
        if checkpoint_dir:
            self.solve_args["checkpoint_dir"] = checkpoint_dir
        # solver(req, **solve_args) -> (E, sweeps[, truncated weight]); the default is the GPU solve
        self.solver = solver or solve
        self.footprint = footprint or (lambda r: footprint_bytes(r.L, r.D))
        self.on_device = solver is None
        if self.on_device:
            _lib.ensure_init(self.device)
        if memory_budget is None:
            if not self.on_device:
                raise ValueError("give a memory budget for a host-side solver")
            free, _ = device_memory()
            memory_budget = int(0.6 * free)
        self.memory_budget = int(memory_budget)
        self.peak_concurrency = 0
        self.peak_memory = 0

    def run(self, requests, realtime=True, on_done=None):
        """Serve ``requests`` (released at their arrival times when ``realtime``,
        all at once otherwise); returns the results in request order.  ``on_done(result)``
        is called on the worker thread as each request finishes."""
        reqs = sorted(requests, key=lambda r: (r.arrival, r.rid))
        n = len(reqs)
        results = {}
        fp = {r.rid: int(self.footprint(r)) for r in reqs}
        cond = threading.Condition()
        state = {"in_flight": 0, "mem": 0, "done": 0, "peak": 0}
        work = queue.Queue()
        t0 = time.perf_counter()

        def worker():
            if self.on_device:
                _lib.call("qtt_init", self.device)
            while True:
                item = work.get()
                if item is None:
                    return
                req, res = item
                res.started = time.perf_counter() - t0
                try:
                    out = self.solver(req, **self.solve_args)
                    res.energy, res.sweeps = out[0], out[1]
                    if len(out) > 2:
                        res.truncated_weight = out[2]
                except Exception as e:  # reported per request, the server keeps going
                    res.error = f"{type(e).__name__}: {e}"
                res.done = time.perf_counter() - t0
                if on_done is not None:
                    try:
                        on_done(res)
                    except Exception:  # a progress callback never stops the server
                        pass
                with cond:
                    state["in_flight"] -= 1
                    state["mem"] -= res.footprint
                    state["done"] += 1
                    results[req.rid] = res
                    cond.notify_all()

        threads = [threading.Thread(target=worker, daemon=True) for _ in range(self.slots)]
        for t in threads:
            t.start()
        pending = collections.deque()
        idx = 0
        try:
            with cond:
                while state["done"] < n:
                    now = time.perf_counter() - t0
                    while idx < n and (not realtime or reqs[idx].arrival <= now):
                        pending.append(reqs[idx])
                        idx += 1
                    # first come, first served; a request larger than the whole budget runs alone
                    while pending and state["in_flight"] < self.slots:
                        r = pending[0]
                        f = fp[r.rid]
                        if state["in_flight"] and state["mem"] + f > self.memory_budget:
                            break
                        pending.popleft()
                        res = SolveResult(r, f)
                        res.admitted = now
                        state["in_flight"] += 1
                        state["mem"] += f
                        state["peak"] = max(state["peak"], state["in_flight"])
                        state["peak_mem"] = max(state.get("peak_mem", 0), state["mem"])
                        work.put((r, res))
                    wait = None
                    if idx < n and realtime:
                        wait = max(0.0, reqs[idx].arrival - (time.perf_counter() - t0))
                    cond.wait(timeout=wait)
        finally:
            for _ in threads:
                work.put(None)
            for t in threads:
                t.join()
        self.peak_concurrency = state["peak"]
        self.peak_memory = state.get("peak_mem", 0)
        return [results[r.rid] for r in sorted(requests, key=lambda r: r.rid)]


def serial_solve_times(requests, **solve_args):
    """(service time, E, sweeps, truncated weight) of every request solved alone, one
    after another, on the calling thread."""
    out = []
    for r in requests:
        t = time.perf_counter()
        E, sw, tw = solve(r, **solve_args)
        out.append((time.perf_counter() - t, E, sw, tw))
    return out


def fifo_latencies(arrivals, services):
    """Latencies of a single-server first-come-first-served queue."""
    free_at = 0.0
    lat = []
    for a, s in sorted(zip(arrivals, services)):
        start = max(a, free_at)
        free_at = start + s
        lat.append(free_at - a)
    return lat


def summarize(latencies, makespan, n):
    lat = np.asarray(latencies, dtype=float)
    return {"solves": int(n), "makespan_s": float(makespan), "solves_per_s": float(n / makespan) if makespan > 0 else None,
            "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "mean_s": float(lat.mean())}
