"""Gradients of E(theta, psi) = <psi|H(theta)|psi> (new: the reference has no AD).

* Site tensors: E is a Hermitian form in each site tensor A_n whose kernel is the
  contraction of every other tensor, i.e. the one-site effective map at n built from the
  actual (not necessarily isometric) tensors.  So dE/d conj(A_n) = H_eff,n A_n in any gauge;
  the adjoint contraction is the eff_h1 map itself (Hermitian), executed by the same
  libgrafttn plan engine, with environments rebuilt under an optional byte budget
  (environment recomputation).
* Couplings: for H linear in theta_e, dE/dtheta_e = <psi|h_e|psi>, a local two-site
  expectation value at the edge (lib/GraftContractions/src/Contractions/expectation.jl:72):
  the centre is moved to the edge's child, Θ is merged and the edge's two-body operator is
  applied to Θ's two physical legs on the device.

All arithmetic is libgrafttn calls on the GPU.
"""
from __future__ import annotations

import numpy as np

from .contractions import EnvCache, eff_h1
from .networks import TTNO, TTNS, move_center, two_site_tensor


def site_gradients(psi: TTNS, H: TTNO, precision="fp64", max_env_bytes=None):
    """[dE/d conj(A_n) for every node n] on the device, in psi's current gauge."""
    cache = EnvCache(psi.topo, max_env_bytes=max_env_bytes)
    grads = []
    for n in range(psi.topo.nnodes):
        h1 = eff_h1(cache, psi, H, n, precision)
        grads.append(h1(psi.tensors[n]))
        h1.close()
    return grads


def energy(psi: TTNS, H: TTNO):
    """Un-normalised <psi|H|psi> from the one-site map at the current centre (the Rayleigh
    closure of test/runtests.jl:654-672)."""
    cache = EnvCache(psi.topo)
    c = psi.center
    h1 = eff_h1(cache, psi, H, c)
    e = psi.ctx.dot(psi.tensors[c], h1(psi.tensors[c]))
    h1.close()
    return e


def edge_expectation(psi: TTNS, edge, terms):
    """<psi|sum_t coeff_t O_c (x) O_p|psi> for edge (c, p); psi is moved to centre c."""
    ctx, t = psi.ctx, psi.topo
    c, p = edge
    move_center(psi, c)
    theta = two_site_tensor(psi, c, p)
    d = theta.shape[t.nchildren(c)]
    op = np.zeros((d, d, d, d), dtype=np.complex128)  # (out_c, out_p, in_c, in_p)
    for coeff, oc, opp in terms:
        op += coeff * np.einsum("ab,cd->acbd", oc, opp)
    pc = t.nchildren(c)                       # phys leg of c inside Θ
    k = t.childslot(p, c)
    pp = pc + 1 + t.nchildren(p) - 1          # phys leg of p inside Θ (its slot k is dropped)
    r = theta.dim()
    lab = [-(j + 1) for j in range(r)]
    lab[pc], lab[pp] = 1, 2
    op_lab = [-(pc + 1), -(pp + 1), 1, 2]
    y = ctx.contract([theta, ctx.upload(op)], [lab, op_lab])
    del k
    return ctx.dot(theta, y)


def coupling_gradients(psi: TTNS, edge_terms):
    """dE/dtheta_e for a Hamiltonian sum_e theta_e h_e; ``edge_terms[e]`` lists the
    (coeff, O_child, O_parent) terms of h_e (coefficients without theta_e)."""
    work = psi.copy()
    out = {}
    for e, terms in edge_terms.items():
        out[e] = edge_expectation(work, e, terms).real
    return out
