"""The device planner's algorithm (csrc/planner.cu), restated step by step in plain
Python, reproduces the oracle's tensordot plan (sources/btensor.cpp:1998-2110): the
same output blocks in the same order and the same pairs in accumulation order.  This
checks the arithmetic of the key packing, the rank sorts, the run and suffix tables
and the pair ranking on the CPU; tests/test_gpu_planner.py checks the kernel itself
against the host planner on the GPU."""
import bisect

import numpy as np
import pytest

from oracle import qtt_oracle as o
from tests.test_library_cpu import _contractible_pair


def _bits_for(n):
    b = 0
    while b < 63 and (1 << b) < n:
        b += 1
    return b


def _rank_sort(keys):
    out = [None] * len(keys)
    for i, k in enumerate(keys):
        out[sum(1 for x in keys if x < k)] = (k, i)
    return [x[0] for x in out], [x[1] for x in out]


def device_plan(A, B, dA, dB):
    """[(output block index, [(A block, B block), ...])] as planner.cu computes it."""
    freeA = [i for i in range(A.rank) if i not in dA]
    freeB = [i for i in range(B.rank) if i not in dB]
    p1, p2p = freeA + list(dA), freeB + list(dB)

    def layout(t, order):
        bits = [_bits_for(t.sbd[leg]) for leg in order]
        sh, s = [], sum(bits)
        for b in bits:
            s -= b
            sh.append(s)
        return sh, sum(bits)
    shA, totA = layout(A, p1)
    shB, totB = layout(B, p2p)
    suf = sum(_bits_for(A.sbd[d]) for d in dA)
    nA, nB = len(A.blocks), len(B.blocks)
    runbits = _bits_for(nB + 1)
    assert totA <= 63 and totB <= 63 and suf + runbits <= 62
    akey, aid = _rank_sort([sum(k[leg] << s for leg, s in zip(p1, shA)) for k, _ in A.blocks])
    bkey, bid = _rank_sort([sum(k[leg] << s for leg, s in zip(p2p, shB)) for k, _ in B.blocks])
    headA = [int(i == 0 or (akey[i] >> suf) != (akey[i - 1] >> suf)) for i in range(nA)]
    headB = [int(i == 0 or (bkey[i] >> suf) != (bkey[i - 1] >> suf)) for i in range(nB)]
    runA = list(np.cumsum(headA) - 1)
    runB = list(np.cumsum(headB) - 1)
    firstA = [i for i in range(nA) if headA[i]] + [nA]
    smask, rmask = (1 << suf) - 1, (1 << runbits) - 1
    t3, t3j = _rank_sort([((bkey[i] & smask) << runbits) | int(runB[i]) for i in range(nB)])
    lo, cnt = [], []
    for i in range(nA):
        s = (akey[i] & smask) << runbits
        a, e = bisect.bisect_left(t3, s), bisect.bisect_left(t3, s + rmask + 1)
        lo.append(a)
        cnt.append(e - a)
    off = [0] + [int(x) for x in np.cumsum(cnt)]
    P = off[-1]
    pa, pb, head = [None] * P, [None] * P, [None] * P
    for q in range(P):
        i = bisect.bisect_right(off[:nA], q) - 1
        e3 = lo[i] + q - off[i]
        rb = t3[e3] & rmask
        f, fe = firstA[runA[i]], firstA[runA[i] + 1]
        pos, hd = 0, 1
        for j in range(f, fe):
            runs = [x & rmask for x in t3[lo[j]:lo[j] + cnt[j]]]
            lb = bisect.bisect_left(runs, rb)
            pos += lb
            if j < i and lb < cnt[j] and runs[lb] == rb:
                hd = 0
                pos += 1
        pos += off[f]
        assert pa[pos] is None   # the ranks of a run are a permutation
        pa[pos], pb[pos], head[pos] = aid[i], bid[t3j[e3]], hd
    heads = [q for q in range(P) if head[q]]
    out = []
    for k, p0 in enumerate(heads):
        p1e = heads[k + 1] if k + 1 < len(heads) else P
        ia, ib = A.blocks[pa[p0]][0], B.blocks[pb[p0]][0]
        key = tuple(ia[d] for d in freeA) + tuple(ib[d] for d in freeB)
        out.append((key, [(pa[x], pb[x]) for x in range(p0, p1e)]))
    return out


@pytest.mark.parametrize("mods", [(0,), (5,), (0, 0), (0, 2)])
def test_device_planner_algorithm_reproduces_the_oracle_plan(mods):
    rng = np.random.default_rng(40 + len(mods) + sum(mods))
    n = 0
    for trial in range(600):
        if n >= 25:
            break
        ra, rb = int(rng.integers(1, 5)), int(rng.integers(1, 5))
        nc = int(rng.integers(1, min(ra, rb) + 1))
        A, B, dA, dB = _contractible_pair(rng, mods, ra, rb, nc)
        if not A.blocks or not B.blocks:
            continue
        _, plan, _, _ = o.tdot_plan(A, B, dA, dB)
        want = [(tuple(k), [tuple(p) for p in prs]) for k, prs in plan]
        assert device_plan(A, B, dA, dB) == want, (trial, dA, dB)
        n += 1
    assert n >= 10
