"""Generate the committed golden fixtures from the oracle (CPU, numpy PCG64 seeds).

The reference ships no golden vectors for this path (it pins it with exact-diagonalisation
and identity gates), so these fixtures hold exact-diagonalisation answers and oracle
outputs at seeded inputs; the GPU tests compare against them.
Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import ttn_oracle as O  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def star32():
    topo = O.star_topology(3, 2)
    H = O.tfi(topo, J=1.0, g=0.9)
    E0, _ = O.exact_groundstate(O.dense_hamiltonian(H))
    psi = O.random_ttns(np.random.default_rng(1), topo, 2, 2)
    _, Es = O.dmrg2(psi, O.ttno_nn(H), maxdim=32, nsweeps=10)
    np.savez(os.path.join(OUT, "star32_tfi.npz"), E_ed=E0, E_dmrg=np.array(Es))


def h2_binary():
    # one eff_h2 application on bin15 Heisenberg (bond 6): inputs and oracle output
    topo = O.binary_topology(3)
    Ws = O.ttno_nn(O.heisenberg(topo))
    rng = np.random.default_rng(7)
    tens = []
    for n in range(topo.nnodes):
        shape = [6 if topo.children[c] else 2 for c in topo.children[n]] + [2, 1 if n == 0 else (6 if topo.children[n] else 2)]
        tens.append(O.randn_c(rng, shape))
    psi = O.TTNS(topo, tens, 0)
    O.canonicalize(psi, 3)
    cache = O.EnvCache(topo)
    h2 = O.eff_h2(cache, psi, Ws, 3, 1)
    x = O.randn_c(rng, h2.shape)
    np.savez(os.path.join(OUT, "h2_bin15_heis.npz"), x=x, y=h2(x),
             **{f"A{n}": a for n, a in enumerate(psi.tensors)})


if __name__ == "__main__":
    star32()
    h2_binary()
    print("written", sorted(f for f in os.listdir(OUT) if f.endswith(".npz")))
