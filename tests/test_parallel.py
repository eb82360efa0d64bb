"""Channel-sliced and distributed effective maps (host logic, CPU): LPT bins, slice
ownership and the reduction reproduce the unsliced map; two gloo ranks on CPU."""
import os

import numpy as np
import pytest

from grafttn import parallel as P
from oracle import ttn_oracle as O


def test_lpt_bins_deterministic():
    assert P.lpt_bins([1, 1, 1, 1, 1], 2) == [[0, 2, 4], [1, 3]]
    assert P.lpt_bins([5, 1, 4, 2], 2) == [[0, 1], [2, 3]]
    assert P.owned_slices(5, 1, 2) == [1, 3]


def _sliced_h1_setup():
    topo = O.star_topology(3, 2)
    Ws = O.ttno_nn(O.heisenberg(topo))
    psi = O.random_ttns(np.random.default_rng(3), topo, 2, 4)
    cache = O.EnvCache(topo)
    n = psi.center
    full = O.eff_h1(cache, psi, Ws, n)
    import grafttn as G
    gt = G.star_topology(3, 2)
    targets, cdim = P.h1_channel_target(gt, n, Ws[n].shape)

    def make_slice(sel):
        statics = list(full.statics)
        for slot, leg in targets:
            statics[slot] = P.restrict_numpy(statics[slot], leg, sel)
        m = O.EffMap(full.labels, full.order, statics, full.shape)
        return m
    return full, make_slice, cdim


def test_channel_slices_sum_to_full_map():
    full, make_slice, cdim = _sliced_h1_setup()
    sliced = P.ChannelSlicedMap(make_slice, cdim, 3)
    x = O.randn_c(np.random.default_rng(4), full.shape)
    y = sliced.apply_slices(x, range(len(sliced.slices)), lambda a, b: a + b, np.zeros_like)
    assert np.linalg.norm(y - full(x)) < 1e-12 * np.linalg.norm(full(x))


def _rank_main(rank, world, port, q):
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        full, make_slice, cdim = _sliced_h1_setup()
        sliced = P.ChannelSlicedMap(make_slice, cdim, 4)

        def allreduce(y):
            t = torch.from_numpy(np.ascontiguousarray(y))
            dist.all_reduce(t)
            return t.numpy()
        dmap = P.DistributedChannelMap(sliced, rank, world, allreduce, lambda a, b: a + b, np.zeros_like)
        x = O.randn_c(np.random.default_rng(5), full.shape)
        y = dmap(x)
        ref = full(x)
        q.put((rank, float(np.linalg.norm(y - ref) / np.linalg.norm(ref))))
    finally:
        dist.destroy_process_group()


def test_distributed_channel_map_two_gloo_ranks():
    import multiprocessing as mp
    import socket
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    res = [q.get(timeout=5) for _ in range(2)]
    assert all(p.exitcode == 0 for p in procs)
    assert all(err < 1e-12 for _, err in res), res
