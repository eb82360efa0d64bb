"""U(1) two-site DMRG end to end on the GPU (dmrg2!, GroundState.jl:102-143, on abelian
TensorMaps): block-sparse environments and merges on the block engine, the eigensolver hook
on the block map (gtn_blockmap_lanczos_min / _refine), per-sector QR gauge moves and the
per-sector truncated SVD split.  Against exact diagonalisation inside the charge sector
(the reference's DMRG-vs-ED gate, test/runtests.jl:687-700, restricted to Sz) and against
the dense GPU DMRG."""
import numpy as np
import pytest

import grafttn as G
from grafttn import u1 as U
from oracle import ttn_oracle as O

pytestmark = pytest.mark.gpu


def sector_ground_energy(otopo, Q):
    Hd = O.dense_hamiltonian(O.heisenberg(otopo))
    n = int(np.log2(Hd.shape[0]))
    idx = [i for i in range(Hd.shape[0]) if bin(i).count("1") == Q]
    assert len(idx) == len(set(idx)) and n > 0
    return float(np.linalg.eigvalsh(Hd[np.ix_(idx, idx)])[0])


@pytest.mark.parametrize("name,Q,D", [("mps8", 4, 16), ("bin7", 3, 8)])
@pytest.mark.parametrize("precision", ["fp64", "fp16x3"])
def test_u1_dmrg2_vs_sector_ed(ctx, name, Q, D, precision):
    if name == "mps8":
        topo, otopo = G.mps_topology(8), O.mps_topology(8)
    else:
        topo, otopo = G.binary_topology(2), O.binary_topology(2)
    E0 = sector_ground_energy(otopo, Q)
    H = U.U1TTNO(ctx, topo, U.u1_heisenberg(topo))
    psi = U.U1TTNS.random(ctx, np.random.default_rng(3), topo, Q, D)
    assert abs(psi.norm() - 1) < 1e-12
    _, Es = U.dmrg2(psi, H, G.TruncationScheme(maxdim=D), nsweeps=6, precision=precision,
                    refine="off" if precision == "fp64" else "all")
    assert abs(Es[-1] - E0) / abs(E0) < 1e-10, (Es, E0)
    # the state stays in the charge sector and normalised
    assert abs(psi.norm() - 1) < 1e-10
    assert psi.tensors[topo.postorder()[-1]].T.legs[-1].charges == [Q]


def test_u1_truncated_dmrg_matches_dense_energy(ctx):
    # mps10 Sz = 0 at D = 8 (truncated): the U(1) energy is variational and no worse than the
    # dense DMRG's at the same bond dimension (the symmetric ansatz spends its states in the
    # right sectors), and both lie above the sector ground energy
    topo, otopo = G.mps_topology(10), O.mps_topology(10)
    E0 = sector_ground_energy(otopo, 5)
    H = U.U1TTNO(ctx, topo, U.u1_heisenberg(topo))
    psi = U.U1TTNS.random(ctx, np.random.default_rng(4), topo, 5, 8)
    _, Es = U.dmrg2(psi, H, G.TruncationScheme(maxdim=8), nsweeps=6)
    Wd = G.TTNO.from_hamiltonian(G.heisenberg(topo), ctx)
    pd = G.random_ttns(np.random.default_rng(4), topo, 2, 8, ctx=ctx)
    _, Ed = G.dmrg2(pd, Wd, G.TruncationScheme(maxdim=8), nsweeps=6)
    assert E0 - 1e-10 <= Es[-1] <= Ed[-1] + 1e-8, (Es[-1], Ed[-1], E0)
    assert max(psi.bond_dims()) <= 8
