"""CPU oracle for abelian U(1) block-sparse contractions (TEST INFRASTRUCTURE: imported only
by tests/ and bench.py's cpu_baseline / reference legs).

Restates TensorKit's abelian contraction as used behind
lib/GraftFoundation/src/Backend/Backend.jl:166-222 (contract_pair over per-sector blocks;
cost model :243-261,309-368): a tensor is a dict {charge tuple: dense block}; a pair
contraction sums, for every pair of blocks whose charges agree on the contracted legs, the
dense tensordot of the two blocks into the output block with the remaining charges.  The
label conventions are those of ttn_oracle.ncon.  Independent of the package's planner."""
from __future__ import annotations

import numpy as np


def blocks_from_flat(structure, data):
    """{charges: block} from a structure object exposing `.blocks` = [(charges, shape, offset)]."""
    return {qs: np.asarray(data[off: off + int(np.prod(shape))]).reshape(shape) for qs, shape, off in structure.blocks}


def contract_pair(A, la, B, lb):
    shared = [l for l in la if l > 0 and l in lb]
    ia = [la.index(l) for l in shared]
    ib = [lb.index(l) for l in shared]
    fa = [i for i in range(len(la)) if i not in ia]
    fb = [i for i in range(len(lb)) if i not in ib]
    byk = {}
    for qb, bb in B.items():
        byk.setdefault(tuple(qb[i] for i in ib), []).append((qb, bb))
    out = {}
    for qa, ba in A.items():
        k = tuple(qa[i] for i in ia)
        for qb, bb in byk.get(k, []):
            qc = tuple(qa[i] for i in fa) + tuple(qb[i] for i in fb)
            c = np.tensordot(ba, bb, axes=(ia, ib))
            if qc in out:
                out[qc] = out[qc] + c
            else:
                out[qc] = c
    return out, [la[i] for i in fa] + [lb[i] for i in fb]


def ncon_blocks(tensors, labels, order):
    """Pairwise contraction in `order`; output blocks with legs sorted as -1, -2, ..."""
    cur, cl = tensors[order[0]], list(labels[order[0]])
    for j in order[1:]:
        cur, cl = contract_pair(cur, cl, tensors[j], list(labels[j]))
    perm = sorted(range(len(cl)), key=lambda i: -cl[i])
    return {tuple(q[i] for i in perm): b.transpose(perm) for q, b in cur.items()}


def flat_from_blocks(structure, blocks):
    out = np.zeros(structure.size, dtype=np.complex128)
    for qs, shape, off in structure.blocks:
        b = blocks.get(qs)
        if b is not None:
            out[off: off + b.size] = b.reshape(-1)
    return out
