"""Host-side check of the predictor-basis schemes of the bond expansion
(grafttn/expansion.py; expand!, expansion.jl:240-370) against the oracle.

The scheme logic only talks to its context through upload / matmul / qr / svd_trunc / axpby /
scale.
HostContext below gives those calls the device context's signatures and results on CPU
tensors, so the sequence of products, QRs, SVDs and probe draws is checked here without a
GPU. The device arithmetic itself is covered by tests/test_gpu_parity.py."""
import numpy as np
import pytest
import torch

from grafttn import expansion as X
from oracle import ttn_oracle as O


class HostContext:
    """The device context's dense calls on CPU complex128 tensors (axpby writes y in place, as
    the device call does)."""

    def upload(self, arr):
        return torch.from_numpy(np.ascontiguousarray(np.asarray(arr, dtype=np.complex128)))

    def matmul(self, A, B, conjA=False, transA=False):
        a = A.conj() if conjA else A
        a = a.transpose(0, 1) if transA else a
        return (a @ B).contiguous()

    def qr(self, A2):
        Q, R = torch.linalg.qr(A2, mode="reduced")
        return Q.contiguous(), R.contiguous()

    def axpby(self, a, x, b, y):
        y.copy_(a * x + b * y)
        return y

    def scale(self, x, a):
        return (a * x).contiguous()

    def svd_trunc(self, A2, maxdim=None, atol=0.0, rtol=0.0, discarded_weight=0.0):
        U, S, Vh = np.linalg.svd(A2.numpy(), full_matrices=False)
        r = O.truncation_rank(S, maxdim, atol, rtol)
        return (torch.from_numpy(np.ascontiguousarray(U[:, :r])), S[:r],
                torch.from_numpy(np.ascontiguousarray(Vh[:r])), float(np.sqrt(np.sum(S[r:] ** 2))))


def _projector(B):
    B = np.asarray(B)
    return B @ B.conj().T


@pytest.mark.parametrize("scheme,cap,oversample,poweriter", [
    ("exact", 6, 8, 0), ("directqr", 6, 8, 0), ("rsvd", 6, 3, 0), ("rsvd", 6, 2, 2),
    ("rangefinder", 6, 3, 0), ("rangefinder", 9, 0, 1)])
def test_scheme_matches_oracle(scheme, cap, oversample, poweriter):
    rng = np.random.default_rng(50)
    P = (O.randn_c(rng, (36, 36)) * 0.8 ** np.arange(36)) @ O.randn_c(rng, (36, 28))
    got = X.predictor_basis(HostContext(), torch.from_numpy(P), cap, scheme, np.random.default_rng(51),
                            oversample, poweriter)
    ref = O.predictor_basis(P, cap, scheme, np.random.default_rng(51), oversample, poweriter)
    got = got.numpy()
    assert got.shape == ref.shape
    assert np.allclose(got.conj().T @ got, np.eye(got.shape[1]), atol=1e-12)
    assert np.allclose(_projector(got), _projector(ref), atol=1e-9)


def test_probe_draw_convention_matches_oracle():
    a = X.probe_block(np.random.default_rng(52), 7, 3)
    b = O.predictor_probe(np.random.default_rng(52), 7, 3)
    assert np.array_equal(a, b)


def test_scheme_argument_checks():
    ctx = HostContext()
    P = torch.zeros((4, 3), dtype=torch.complex128)
    with pytest.raises(ValueError):
        X.predictor_basis(ctx, P, 2, "lanczos")
    for scheme in ("rsvd", "rangefinder"):
        with pytest.raises(ValueError):
            X.predictor_basis(ctx, P, 2, scheme, rng=None)
    with pytest.raises(ValueError):
        X.predictor_basis(ctx, P, 2, "rsvd", np.random.default_rng(0), oversample=-1)


@pytest.mark.parametrize("rows,D,rest,room,oversample,poweriter", [
    (32, 4, 24, 6, 8, 0), (32, 4, 24, 6, 2, 2), (12, 4, 40, 6, 8, 1), (10, 10, 8, 3, 8, 0)])
def test_factorized_rangefinder_matches_oracle(rows, D, rest, room, oversample, poweriter):
    # the projector form (1 - Q Q^H) P against the oracle's explicit complement N, including a
    # complement narrower than the sketch (12 rows, D 4, sketch 14) and an empty one
    rng = np.random.default_rng(53)
    Am = O.randn_c(rng, (rows, D))
    P = (O.randn_c(rng, (rows, rows)) * 0.75 ** np.arange(rows)) @ O.randn_c(rng, (rows, rest))
    Qd, Ed = X.factorized_rangefinder_enrichment(HostContext(), torch.from_numpy(Am), torch.from_numpy(P), room,
                                                 np.random.default_rng(54), oversample, poweriter)
    Qo, Eo = O.factorized_rangefinder_enrichment(Am, P, room, np.random.default_rng(54), oversample, poweriter)
    assert np.allclose(_projector(Qd), _projector(Qo), atol=1e-12)
    if Eo is None:
        assert Ed is None
        return
    Ed = Ed.numpy()
    assert Ed.shape == Eo.shape
    assert np.allclose(_projector(Ed), _projector(Eo), atol=1e-9)
    U = np.concatenate([Qd.numpy(), Ed], axis=1)
    assert np.allclose(U.conj().T @ U, np.eye(U.shape[1]), atol=1e-12)
