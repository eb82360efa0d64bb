"""gtn_expm_small, the dense exponential behind the Arnoldi Krylov exponential (host code of
the C-ABI library; no GPU), against scipy.linalg.expm."""
import ctypes as C

import numpy as np
import pytest
import scipy.linalg

from grafttn import _lib


def expm_lib(A):
    m = A.shape[0]
    a = np.ascontiguousarray(A, dtype=np.complex128).view(np.float64).ravel()
    e = np.empty(2 * m * m)
    st = _lib.lib().gtn_expm_small(m, a.ctypes.data_as(_lib._pd), e.ctypes.data_as(_lib._pd))
    assert st == _lib.GTN_OK
    return e.view(np.complex128).reshape(m, m)


@pytest.mark.parametrize("m", [1, 5, 30, 63])
@pytest.mark.parametrize("scale", [1e-3, 1.0, 8.0])
def test_expm_small_matches_scipy(m, scale):
    rng = np.random.default_rng(70 + m)
    A = (rng.standard_normal((m, m)) + 1j * rng.standard_normal((m, m))) * scale / np.sqrt(m)
    ref = scipy.linalg.expm(A)
    got = expm_lib(A)
    assert np.linalg.norm(got - ref) <= 1e-12 * np.linalg.norm(ref)


def test_expm_small_hessenberg_dz_times_h():
    # the shape the Arnoldi exponential exponentiates: dz * H_m with H_m upper Hessenberg,
    # non-normal, dz = -0.05i (real time)
    rng = np.random.default_rng(71)
    m = 30
    H = np.triu(rng.standard_normal((m, m)) + 1j * rng.standard_normal((m, m)), -1) * 3.0
    A = -0.05j * H
    ref = scipy.linalg.expm(A)
    assert np.linalg.norm(expm_lib(A) - ref) <= 1e-12 * np.linalg.norm(ref)


def test_expm_small_rejects_bad_sizes():
    a = np.zeros(2)
    e = np.zeros(2)
    assert _lib.lib().gtn_expm_small(0, a.ctypes.data_as(_lib._pd), e.ctypes.data_as(_lib._pd)) != _lib.GTN_OK
    assert _lib.lib().gtn_expm_small(1, None, e.ctypes.data_as(_lib._pd)) != _lib.GTN_OK
