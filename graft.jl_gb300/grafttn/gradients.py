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
* TTNO tensors, by the adjoint: E = <A_n, H_eff,n A_n> is linear in W_n, so
  dE = <G_n, dW_n> with G_n the adjoint of the W_n operand of the eff_h1 contraction at the
  cotangent A_n (gtn_contract_vjp).  The couplings then follow by the chain rule through
  W(theta): the TTNO builder places theta_e in the parent's tensor only, affinely, so
  dE/dtheta_e = Re <G_p, dW_p/dtheta_e>.  Environments come from one cache with an optional
  byte budget (evicted ones are recomputed on demand).

All arithmetic is libgrafttn calls on the GPU.
"""
from __future__ import annotations

import numpy as np

from .contractions import EnvCache, _cap, eff_h1, h1_spec
from .networks import TTNO, TTNS, move_center, two_site_tensor
from .operators import NNHamiltonian, ttno_tensors


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


def ttno_gradients(psi: TTNS, H: TTNO, max_env_bytes=None, precision="fp64"):
    """[G_n for every node n] with dE = sum_n <G_n, dW_n> for E = <psi|H|psi> (un-normalised,
    any gauge): the adjoint of W_n in the eff_h1 contraction at node n with cotangent A_n."""
    from . import _lib
    prec = _lib.PRECISIONS[precision] if isinstance(precision, str) else precision
    ctx, t = psi.ctx, psi.topo
    cache = EnvCache(t, max_env_bytes=max_env_bytes)
    out = []
    for n in range(t.nnodes):
        A = psi.tensors[n].contiguous()
        labels, _, envs = h1_spec(t, n, A.dim(), H.tensors[n].dim())
        ops = [A, H.tensors[n]] + [cache.env(psi, H, w, u) for (w, u) in envs]
        if t.parent[n] < 0:
            ops.append(_cap(ctx))
        out.append(ctx.contract_vjp(ops, labels, A, 1, precision=prec))
    return out


def ttno_coupling_derivatives(Hnn: NNHamiltonian, dcoeffs):
    """dW_p/dtheta_e on the host for the nearest-neighbour TTNO builder: ``dcoeffs[e]`` lists
    d coeff_t / d theta_e for the terms of Hnn.bonds[e] in order.  The builder puts an edge's
    coefficients into its parent's tensor only, affinely, so the derivative is the difference
    of the parent's tensor with the edge's coefficients raised by their derivatives."""
    t = Hnn.topo
    W0 = ttno_tensors(Hnn)
    out = {}
    for e, dc in dcoeffs.items():
        H1 = NNHamiltonian(t, Hnn.d, dict(Hnn.onsite), {k: list(v) for k, v in Hnn.bonds.items()}, Hnn.hermitian)
        H1.bonds[e] = [(c + d, oc, op) for (c, oc, op), d in zip(Hnn.bonds[e], dc)]
        p = e[1]
        out[e] = (p, ttno_tensors(H1)[p] - W0[p])
    return out


def coupling_gradients_adjoint(psi: TTNS, H: TTNO, Hnn: NNHamiltonian, dcoeffs, max_env_bytes=None):
    """dE/dtheta_e for every edge of ``dcoeffs`` by the adjoint route: one W-adjoint per parent
    node (ttno_gradients), then Re <G_p, dW_p/dtheta_e> on the device."""
    ctx = psi.ctx
    G = ttno_gradients(psi, H, max_env_bytes=max_env_bytes)
    out = {}
    for e, (p, dW) in ttno_coupling_derivatives(Hnn, dcoeffs).items():
        out[e] = ctx.dot(G[p], ctx.upload(dW)).real
    return out
