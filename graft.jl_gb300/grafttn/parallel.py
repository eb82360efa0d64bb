"""Channel slicing of an effective map over its largest TTNO bond, and the distributed
reduction of the slices across ranks.

Mirrors lib/GraftContractions/src/Contractions/effective.jl:390-414 (deterministic
longest-processing-time bin packing of operator channels, ties broken by channel order
and lowest bin), :445-520 (the sliced one-site map: restrict the TTNO operator leg and the
matching environment operator leg to each bin; the full map is the fixed-order sum of the
slice maps) and :38-143 (``DistributedChannelEffectiveMap``: rank r owns slices
r, r + size, ...; one allreduce of y per application).

On one GPU the slices are applied in order into one accumulator (exactly the unsliced map
up to summation order).  Across ranks each rank sums its own slices and one
``torch.distributed.all_reduce`` combines them (NCCL on GPUs, gloo on CPU ranks).
The slice application is injectable so the host logic runs without a GPU.
"""
from __future__ import annotations

import numpy as np


def lpt_bins(weights, nslices):
    """Deterministic LPT bin packing (effective.jl:390-414): channels sorted by decreasing
    weight (ties by index) go to the least-loaded bin (ties: lowest bin index)."""
    n = len(weights)
    nslices = min(nslices, n)
    order = sorted(range(n), key=lambda i: (-weights[i], i))
    bins = [[] for _ in range(nslices)]
    loads = [0.0] * nslices
    for i in order:
        b = min(range(nslices), key=lambda k: (loads[k], k))
        bins[b].append(i)
        loads[b] += weights[i]
    return [sorted(b) for b in bins]


def owned_slices(nslices, rank, world):
    """Slices owned by `rank` (effective.jl:96): rank, rank + world, ..."""
    return list(range(rank, nslices, world))


def h1_channel_target(topo, n, w_shape):
    """(statics slot, leg) pairs to restrict for a one-site map at node n: the largest TTNO
    operator leg (first on ties) and the operator leg of the environment on that edge
    (effective.jl:480-490).  Static slot 0 is W, slot 1 + i is the env of neighbour i."""
    nbrs = topo.neighbors(n)
    K = topo.nchildren(n)
    legs = [K + 2 if topo.parent[n] == w else topo.childslot(n, w) for w in nbrs]
    dims = [w_shape[l] for l in legs]
    i = int(np.argmax(dims))
    return [(0, legs[i]), (1 + i, 1)], dims[i]


def restrict_numpy(t, leg, idx):
    return np.take(t, idx, axis=leg)


class ChannelSlicedMap:
    """Sum of slice maps.  ``make_slice(selected)`` returns a callable applying the map with
    the operator channels restricted to ``selected``; results are accumulated in slice order."""

    def __init__(self, make_slice, channel_dim, nslices, weights=None):
        weights = weights if weights is not None else [1.0] * channel_dim
        self.bins = lpt_bins(weights, nslices)
        self.slices = [make_slice(sel) for sel in self.bins]

    def apply_slices(self, x, which, add, zeros_like):
        y = zeros_like(x)
        for s in which:
            y = add(y, self.slices[s](x))
        return y


class DistributedChannelMap:
    """Rank-local slices plus one allreduce (effective.jl:38-143).  ``all_reduce`` sums a
    buffer in place across ranks; ``to_buffer``/``from_buffer`` convert the local partial."""

    def __init__(self, sliced: ChannelSlicedMap, rank, world, all_reduce, add, zeros_like):
        if len(sliced.slices) < world:
            raise ValueError(f"distributed channel map needs at least {world} slices, got {len(sliced.slices)}")
        self.sliced = sliced
        self.rank, self.world = rank, world
        self.all_reduce = all_reduce
        self.add, self.zeros_like = add, zeros_like

    def __call__(self, x):
        mine = owned_slices(len(self.sliced.slices), self.rank, self.world)
        y = self.sliced.apply_slices(x, mine, self.add, self.zeros_like)
        return self.all_reduce(y)


def device_h1_slicer(cache, psi, H, n, precision="fp64"):
    """Channel slices of the device one-site map at node n (effective.jl:445-520): returns
    (make_slice, channel_dim, full) where make_slice(selected) builds an EffectiveMap on the
    device whose TTNO tensor and matching environment keep only the operator channels
    `selected` (restricted on the device by gtn_restrict_leg), and full is the unsliced map."""
    from .contractions import eff_h1
    from .contractions import EffectiveMap
    ctx, t = psi.ctx, psi.topo
    full = eff_h1(cache, psi, H, n, precision)
    targets, cdim = h1_channel_target(t, n, tuple(H.tensors[n].shape))

    def make_slice(sel):
        statics = list(full._statics)
        for slot, leg in targets:
            statics[slot] = ctx.restrict_leg(statics[slot], leg, sel)
        return EffectiveMap(ctx, full.x_shape, full.labels, full.order, statics, full.precision)
    return make_slice, cdim, full
