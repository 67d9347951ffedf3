"""Writes the golden fixtures under tests/golden.

``reference_known_answers.json`` transcribes the known-answer cases of QuantiT's
own unit tests for this path (block structures, reshape charges and sizes,
sector order, the L=3 Heisenberg matrix).  Each entry names the test it comes
from (path:line in the QuantiT source tree).  The reference cannot be built
here (it needs libtorch), so its test expectations are read from the test
sources and written down as data.

``oracle_cases.npz`` holds seeded inputs and oracle outputs used by the GPU
parity tests: a tensordot, a truncated sector SVD and a short DMRG run.

Run:  python tests/golden/make_golden.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import qtt_oracle as o  # noqa: E402

KNOWN = {
    "_about": "Known answers from QuantiT's unit tests (paths relative to the QuantiT source tree).",
    "c5_charges": {
        "source": "include/blockTensor/btensor.h:1534 (C<5>, negatives via the int16 constructor)",
        "mod": 5,
        "ctor": [[0, 0], [1, 1], [-1, 4], [-2, 3], [4, 4], [-5, 0]],
    },
    "tensordot_blocks": {
        "source": "include/blockTensor/btensor.h:1581-1608",
        "A_legs": [[[2, 0], [3, 1]], [[2, 0], [3, -1]]],
        "A_sel": 0,
        "A_blocks": [[0, 0], [1, 1]],
        "B_legs": [[[3, 4], [2, 0]], [[2, 0], [3, 1]], [[1, 1], [3, 0]]],
        "B_sel": 1,
        "B_blocks": [[0, 1, 0], [1, 1, 1], [1, 0, 0]],
        "dims": [[1], [1]],
        "C_blocks": [[0, 1, 0], [1, 0, 0], [1, 1, 1]],
        "C_from": {"0,1,0": [[0, 0], [1, 0, 0]], "1,0,0": [[1, 1], [0, 1, 0]], "1,1,1": [[1, 1], [1, 1, 1]]},
    },
    "tensor_product_blocks": {
        "source": "include/blockTensor/btensor.h:1617-1628",
        "C_blocks": [[0, 0, 0, 0], [0, 0, 1, 1], [1, 1, 0, 0], [1, 1, 1, 1]],
    },
    "reshape_vector": {
        "source": "include/blockTensor/btensor.h:1682-1697",
        "present": [0, 3],
        "absent": [1, 2],
        "charges": {"0": 0, "3": 0, "1": 4, "2": 1},
        "sizes": {"0": 4, "3": 9, "1": 6, "2": 6},
    },
    "sector_order": {
        "source": "include/blockTensor/LinearAlgebra.h:255-277,304-310",
        "A_legs": [[[2, 0], [3, 1]], [[1, 1], [2, 0], [3, -1], [1, 1]], [[3, 0], [2, -2], [2, -1]]],
        "A_sel": 0,
        "A_blocks": [[0, 0, 2], [0, 1, 0], [0, 3, 2], [1, 0, 1], [1, 1, 2], [1, 2, 0], [1, 3, 1]],
        "reorder_rank3": [[0, 1, 0], [1, 1, 2], [1, 0, 1], [1, 3, 1], [0, 0, 2], [0, 3, 2], [1, 2, 0]],
        "reorder_after_reshape1": [[0, 2], [0, 3], [0, 11], [1, 1], [1, 5], [1, 6], [1, 10]],
    },
    "heisenberg_L3": {
        "source": "include/models.h:44-68 (Heisenberg_impl(J=1), the 8x8 matrix of the L=3 chain)",
        "entries": [[0, 0, 2], [2, 1, 2], [1, 2, 2], [4, 2, 2], [2, 4, 2], [5, 3, 2], [3, 5, 2],
                    [7, 7, 2], [6, 5, 2], [5, 6, 2], [2, 2, -2], [5, 5, -2]],
    },
}


def oracle_cases(path):
    rng = np.random.default_rng(1234)
    # a rank-4 x rank-4 contraction with U(1) charges and ragged section sizes
    A = o.btensor([[(2, -1), (3, 0), (1, 2)], [(1, -1), (1, 1)], [(1, -1), (1, 1)], [(2, -2), (4, 0), (3, 1)]],
                  [0], (0,))
    A = o.randn_like(A, rng)
    B = o.btensor([[(2, 2), (4, 0), (3, -1)], [(1, 1), (1, -1)], [(1, 1), (1, -1)], [(3, 1), (2, -1)]],
                  [1], (0,))
    B = o.randn_like(B, rng)
    C = o.tensordot(A, B, [3, 2], [0, 1])
    # a truncated SVD of a theta-shaped tensor
    T = o.btensor([[(3, -2), (5, 0), (4, 2)], [(1, -1), (1, 1)], [(1, -1), (1, 1)], [(4, 2), (5, 0), (3, -2)]],
                  [0], (0,))
    T = o.randn_like(T, rng)
    U, d, V = o.svd_truncated(T, 2, 1e-10, 1, 7)
    dv = np.sort(np.concatenate([b for _, b in d.blocks]))[::-1]
    # DMRG, Heisenberg L=10, D=16
    mpo = o.heisenberg_mpo(10)
    mps = o.right_canonicalize(o.random_mps(10, 16, [1, -1], 0, np.random.default_rng(7)))
    E, oc, Es = o.dmrg(mpo, mps, 0, o.DmrgOptions(cutoff=1e-10, convergence_criterion=0.0, maximum_bond=16,
                                                  minimum_bond=4, maximum_iterations=3))
    np.savez(path, C_nnz=C.nnz(), C_blocks=np.array([k for k, _ in C.blocks]),
             C_norm=np.sqrt(sum(float(np.sum(b ** 2)) for _, b in C.blocks)),
             svd_d=dv, svd_U_blocks=np.array([k for k, _ in U.blocks]),
             dmrg_E=np.array(Es))


if __name__ == "__main__":
    with open(os.path.join(HERE, "reference_known_answers.json"), "w") as f:
        json.dump(KNOWN, f, indent=1)
    oracle_cases(os.path.join(HERE, "oracle_cases.npz"))
    print("wrote", HERE)
