"""Channel-sliced device maps (effective.jl:445-520): the statics of the one-site map are
restricted on the device (gtn_restrict_leg) to LPT bins of the largest operator channel;
the slice maps, applied on the GPU and summed in slice order, reproduce the unsliced map.
The rank split of DistributedChannelMap (effective.jl:38-143) is applied here with both
ranks' slices on this one GPU and the allreduce done as a host sum; the multi-process
reduction itself is covered by the gloo tests."""
import numpy as np
import pytest

import grafttn as G
from grafttn import parallel as P
from grafttn.contractions import EnvCache

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("fp16x3", 3e-5)])
@pytest.mark.parametrize("node", ["n1_1", "n0_1"])
def test_device_channel_slices_sum_to_full_map(ctx, precision, tol, node):
    topo = G.binary_topology(4)
    H = G.TTNO.from_hamiltonian(G.heisenberg(topo), ctx)
    psi = G.random_ttns(np.random.default_rng(4), topo, 2, 32, ctx=ctx)
    n = topo.index[node]
    G.move_center(psi, n)
    cache = EnvCache(topo)
    make_slice, cdim, full = P.device_h1_slicer(cache, psi, H, n, precision)
    assert cdim == 5
    sliced = P.ChannelSlicedMap(make_slice, cdim, 3)
    assert sorted(i for b in sliced.bins for i in b) == list(range(cdim))
    x = psi.tensors[n].contiguous()
    y_full = ctx.download(full(x))
    y_sum = sum(ctx.download(s(x)) for s in sliced.slices)
    assert rel(y_sum, y_full) < tol
    # two ranks' partial sums (slices r, r + 2, ...) add up to the full map
    parts = [sum(ctx.download(sliced.slices[s](x)) for s in P.owned_slices(len(sliced.slices), r, 2))
             for r in range(2)]
    assert rel(parts[0] + parts[1], y_full) < tol
    for s in sliced.slices:
        s.close()
    full.close()


def test_restrict_leg_matches_numpy(ctx):
    rng = np.random.default_rng(5)
    t = rng.standard_normal((3, 7, 4, 5)) + 1j * rng.standard_normal((3, 7, 4, 5))
    for leg, idx in [(1, [6, 0, 3]), (3, [4]), (0, [2, 1, 0, 2])]:
        got = ctx.download(ctx.restrict_leg(ctx.upload(t), leg, idx))
        assert np.array_equal(got, np.take(t, idx, axis=leg))
