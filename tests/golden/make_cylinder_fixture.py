"""Convert the reference's 4x8 Heisenberg cylinder MPO fixture (tests/2dHeisenberg/
mpotensor_*.txt of the reference, lines "l s s' r value" with 1-based indices,
read as W[l-1, s-1, r-1, s'-1] by make_tensor in tests/2Dheisenberg.cpp:152-165)
into tests/golden/heisenberg_cylinder_4x8_mpo.npz: one (l, s, r, s') dense
array per site.  The physical basis of the fixture is {2Sz = -1, +1}.

Usage: python make_cylinder_fixture.py <root of the QuantiT source tree>"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def load(path):
    rows = []
    for line in open(path).read().replace('R"(', "").replace(')"', "").splitlines():
        f = line.split()
        if len(f) == 5:
            rows.append((int(f[0]), int(f[1]), int(f[2]), int(f[3]), float(f[4])))
    lb = max(r[0] for r in rows)
    rb = max(r[3] for r in rows)
    w = np.zeros((lb, 2, rb, 2))
    for l, s, sp, r, v in rows:
        w[l - 1, s - 1, r - 1, sp - 1] = v
    return w


def main(ref):
    src = os.path.join(ref, "tests", "2dHeisenberg")
    ws = {f"w{i}": load(os.path.join(src, f"mpotensor_{i + 1}.txt")) for i in range(32)}
    np.savez_compressed(os.path.join(HERE, "heisenberg_cylinder_4x8_mpo.npz"), **ws)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_cylinder_fixture.py <root of the QuantiT source tree>")
    main(sys.argv[1])
