"""grafttn: GB300 (sm_103a) tree-tensor-network effective-Hamiltonian hot path.

Host-side mirror of GraftTN/Graft.jl's interface for that path (TTNS, TTNO, EnvCache,
eff_h1 / eff_h2 / eff_h0, dmrg1!, dmrg2!, TDVP1, TDVP2, TDVP1_CBE, inner / expect, TTNO
apply) over the C ABI of libgrafttn.so.  Host metadata (topologies, operators) is
importable without a GPU; the device layer needs the built library and a CUDA device and
fails loudly otherwise.
"""
from .topology import (TreeTopology, binary_topology, fork_topology, kary_topology, mps_topology,
                       star_topology)
from .operators import (NNHamiltonian, edge_term_hamiltonian, heisenberg, spin_ops, tfi, ttno_tensors,
                        xxz)
from . import _lib

__all__ = [
    "TreeTopology", "binary_topology", "fork_topology", "kary_topology", "mps_topology", "star_topology",
    "NNHamiltonian", "edge_term_hamiltonian", "heisenberg", "spin_ops", "tfi", "ttno_tensors", "xxz",
]


_DEVICE_MODULES = ("device", "networks", "contractions", "solvers", "cbe", "gradients", "blocksparse", "parallel",
                   "observables", "expansion", "u1")


def __getattr__(name):
    # device layer: imported lazily so that host metadata works on machines without CUDA
    import importlib
    if name in _DEVICE_MODULES:
        return importlib.import_module(f"{__name__}.{name}")
    for modname in _DEVICE_MODULES:
        mod = importlib.import_module(f"{__name__}.{modname}")
        if name in vars(mod):
            return vars(mod)[name]
    raise AttributeError(name)
