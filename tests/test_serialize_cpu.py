"""Block-list files on the CPU: structure-only tensors (no device data) survive a
save / load round trip with identical structure and block lists, for U(1), Z(n)
and product groups; wrong or corrupt files are rejected."""
import numpy as np
import pytest

import quantit_gb300 as q
from quantit_gb300 import serialize
from oracle import qtt_oracle as o
from tests._convert import to_device, structure_of
from tests.test_library_cpu import _random_tensor


@pytest.mark.parametrize("mods", [(0,), (5,), (0, 0), (0, 3)])
def test_structure_round_trip(tmp_path, mods):
    rng = np.random.default_rng(40 + len(mods))
    n = 0
    for trial in range(120):
        if n >= 15:
            break
        T = _random_tensor(rng, int(rng.integers(1, 5)), mods)
        if not T.blocks:
            continue
        D = to_device(T, structure_only=True)
        path = tmp_path / f"t{trial}.npz"
        serialize.save(path, D)
        R = serialize.load(path)
        assert structure_of(R) == structure_of(D)
        assert R.block_indices() == D.block_indices()
        n += 1
    assert n >= 8


def test_mps_kind_and_centre(tmp_path):
    rng = np.random.default_rng(3)
    ts = []
    for _ in range(3):
        T = _random_tensor(rng, 3, (0,))
        ts.append(to_device(T, structure_only=True))
    m = q.networks.bMPS(ts, 2)
    serialize.save(tmp_path / "m.npz", m)
    r = serialize.load(tmp_path / "m.npz")
    assert isinstance(r, q.networks.bMPS) and r.orthogonality_center == 2 and len(r) == 3
    for a, b in zip(r, m):
        assert structure_of(a) == structure_of(b) and a.block_indices() == b.block_indices()


def test_rejects_foreign_and_corrupt_files(tmp_path):
    np.savez(tmp_path / "x.npz", format=np.array("something-else"))
    with pytest.raises(ValueError):
        serialize.load(tmp_path / "x.npz")
    T = _random_tensor(np.random.default_rng(9), 2, (0,))
    d = serialize.tensor_arrays(to_device(T, structure_only=True))
    d["ssz"] = d["ssz"][:-1]
    with pytest.raises(ValueError):
        serialize.tensor_from_arrays(d)
