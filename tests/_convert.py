"""Conversions between the library's btensor handles and the oracle's BTensor (tests only)."""
import numpy as np

import quantit_gb300 as q
from oracle import qtt_oracle as o


def legs_of_oracle(t):
    legs = []
    for d in range(t.rank):
        legs.append([(n, q.conserved.quantity._raw(c, t.mods)) for n, c in zip(t.sec_sizes(d), t.sec_charges(d))])
    return legs


def to_device(t, structure_only=False):
    """Oracle BTensor -> library btensor (uploads the blocks unless structure_only)."""
    sel = q.conserved.quantity._raw(t.sel, t.mods)
    if t.rank == 0:
        legs = []
    else:
        legs = legs_of_oracle(t)
    b = q.btensor(legs, sel) if legs else _rank0(t, sel)
    if structure_only:
        b.set_block_structure([k for k, _ in t.blocks])
    else:
        b.set_blocks([(k, v) for k, v in t.blocks])
    return b


def _rank0(t, sel):
    return q.btensor([], sel)


def structure_of(b):
    sbd, ssz, cv, sel = b.structure()
    return sbd, ssz, [c.values for c in cv], sel.values


def to_oracle(b, with_data=True):
    sbd, ssz, cv, sel = b.structure()
    mods = sel.mods
    t = o.BTensor(mods, list(sbd), list(ssz), [c.values for c in cv], sel.values, [], np.float64)
    if with_data:
        t.blocks = [(k, v) for k, v in b.blocks()]
    else:
        t.blocks = [(k, None) for k in b.block_indices()]
    return t


def same_structure(b, t):
    sbd, ssz, cv, sel = structure_of(b)
    return sbd == t.sbd and ssz == t.ssz and cv == [tuple(c) for c in t.cv] and tuple(sel) == tuple(t.sel)
