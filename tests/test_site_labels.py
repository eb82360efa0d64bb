"""The library's kind-based label graphs (gtn_site_labels: eff_h1, eff_h2, eff_h0 and the
environment update from a node's local structure, effective.jl:627-1034,
envcache.jl:919-999) equal the host harness's h1_spec / h2_spec / env_spec, label by label,
on every node and edge of five topologies.  No device is needed."""
import pytest

import grafttn as G
from grafttn import _lib
from grafttn.contractions import env_spec, h1_spec, h2_spec

TOPOS = [G.mps_topology(6), G.star_topology(3, 2), G.binary_topology(3), G.kary_topology(3, 2),
         G.fork_topology(2, 2)]


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__
    __graft_entry__.build()


@pytest.mark.parametrize("ti", range(len(TOPOS)))
def test_h1_h2_env_labels_match_host_specs(ti):
    t = TOPOS[ti]
    for n in range(t.nnodes):
        K = t.nchildren(n)
        root = t.parent[n] < 0
        labels, order, _ = h1_spec(t, n, K + 2, K + 3)
        got = _lib.site_labels(_lib.SiteDesc(_lib.MAP_H1, K, int(root), 0, 0, 0))
        assert got == (labels, order), (ti, n)
        for v in t.neighbors(n):
            lab, conj, envs, has_cap = env_spec(t, n, v, K + 2, K + 3)
            slot = -1 if t.parent[n] == v else t.childslot(n, v)
            got = _lib.site_labels(_lib.SiteDesc(_lib.MAP_ENV, K, int(root), 0, slot, 0))
            assert got[0] == lab and got[1] == list(range(len(lab))), (ti, n, v)
        if not root:
            m = t.parent[n]
            Km = t.nchildren(m)
            pn = K + 1
            xr = pn + Km + 1
            labels, order, _ = h2_spec(t, n, m, xr, K + 3, Km + 3, pn)
            got = _lib.site_labels(_lib.SiteDesc(_lib.MAP_H2, K, 0, Km, t.childslot(m, n), int(t.parent[m] < 0)))
            assert got == (labels, order), (ti, n, m)


def test_h0_labels_and_bad_descriptions():
    assert _lib.site_labels(_lib.SiteDesc(_lib.MAP_H0, 0, 0, 0, 0, 0)) == ([[1, 2], [1, 3, -1], [2, 3, -2]], [0, 1, 2])
    with pytest.raises(ValueError):
        _lib.site_labels(_lib.SiteDesc(_lib.MAP_H2, 1, 0, 2, 2, 0))   # slot outside m's children
    with pytest.raises(ValueError):
        _lib.site_labels(_lib.SiteDesc(_lib.MAP_ENV, 2, 1, 0, -1, 0))  # the root has no parent
    with pytest.raises(ValueError):
        _lib.site_labels(_lib.SiteDesc(9, 0, 0, 0, 0, 0))
