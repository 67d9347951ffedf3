"""The CPU baseline's sampling machinery (bench.py: cpu_sample, run_cpu_sample,
sweep_estimate, sample_bonds) on a small saved state, without a GPU: the oracle's bond
updates run on the files the GPU side writes (block-list format), at the sampled
strata, starting at the requested stratum, and the sweep estimate is the mean over
strata times the 2 (L - 2) updates of a sweep."""
import importlib.util
import json
import os

import numpy as np
import pytest

from oracle import qtt_oracle as o

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _arrays(t, i):
    """One oracle tensor in the block-list file layout (quantit_gb300.serialize)."""
    nc = len(t.mods)
    cv = np.array([[(v - 0x10000 if m and v >= 0x8000 else v) for v, m in zip(c, t.mods)] for c in t.cv],
                  dtype=np.int16).reshape(-1, nc)
    out = {f"t{i}_sbd": np.array(t.sbd, dtype=np.int64), f"t{i}_ssz": np.array(t.ssz, dtype=np.int64),
           f"t{i}_cv": cv, f"t{i}_sel": np.array(t.sel, dtype=np.int16),
           f"t{i}_mods": np.array(t.mods, dtype=np.uint16),
           f"t{i}_bidx": np.array([k for k, _ in t.blocks], dtype=np.int64).reshape(len(t.blocks), t.rank),
           f"t{i}_data": np.concatenate([np.asarray(v, dtype=np.float64).ravel() for _, v in t.blocks]),
           f"t{i}_dtype": np.int32(0)}
    return out


def _save(path, kind, tensors, oc=0):
    arrays = {"format": np.array("qtt-blocklist-1"), "kind": np.array(kind), "count": np.int64(len(tensors)),
              "oc": np.int64(oc)}
    for i, t in enumerate(tensors):
        arrays.update(_arrays(t, i))
    with open(path, "wb") as f:
        np.savez(f, **arrays)


@pytest.fixture(scope="module")
def sample_dir(tmp_path_factory):
    b = _bench()
    d = tmp_path_factory.mktemp("cpu_sample")
    L, D = 10, 8
    mpo = o.heisenberg_mpo(L)
    mps = o.right_canonicalize(o.random_mps(L, D, [1, -1], 0, np.random.default_rng(7)))
    bonds = b.sample_bonds(L, 3)
    _save(d / "mpo.npz", "bMPO", mpo)
    _save(d / "state.npz", "bMPS", mps, 0)
    for bd in bonds:
        env = o.generate_env(mpo, mps, bd)
        _save(d / f"env_{bd}.npz", "bMPO", [env[bd], env[bd + 3]])
    with open(d / "bonds.json", "w") as f:
        json.dump({"bonds": bonds, "L": L, "Dmax": D}, f)
    return b, str(d), bonds, L


def test_sample_bonds_spread_over_the_chain():
    b = _bench()
    assert b.sample_bonds(72, 3) == [11, 35, 59]
    assert b.sample_bonds(72, 1) == [35]
    assert b.sample_bonds(5, 10) == [0, 1, 2, 3]


def test_cpu_sample_cycles_the_strata_from_the_offset(sample_dir):
    b, path, bonds, L = sample_dir
    s = b.cpu_sample(path, 4, 0)
    assert s["bonds"] == bonds and s["L"] == L
    assert [len(s["times"][str(x)]) for x in bonds] == [2, 1, 1]
    s1 = b.cpu_sample(path, 1, 0, offset=1)
    assert [len(s1["times"][str(x)]) for x in bonds] == [0, 1, 0]
    est, per = b.sweep_estimate(s)
    assert len(per) == 3
    assert est == pytest.approx(np.mean(per) * 2 * (L - 2))


def test_run_cpu_sample_in_a_child_process(sample_dir):
    b, path, bonds, L = sample_dir
    s = b.run_cpu_sample(path, 3, 1, offset=2)
    assert s["threads"] == 1
    assert [len(s["times"][str(x)]) for x in bonds] == [1, 1, 1]
    assert all(t > 0 for v in s["times"].values() for t in v)
