"""Failure paths made on the host or by a bounded device wait (no GPU fault, trap or hang):
memory admission refusal, leg-dimension mismatch, and a device wait that runs out, after
which the context keeps working."""
import numpy as np
import pytest

from grafttn import _lib
from grafttn.contractions import EffectiveMap

pytestmark = pytest.mark.gpu


def test_memory_admission_refused_before_any_launch(ctx):
    # an outer product of two 2e5-vectors needs 4e10 complex elements (640 GB) of workspace
    s = ctx.upload(np.ones(200000))
    l0 = ctx.launches
    with pytest.raises(_lib.MemoryAdmissionError):
        EffectiveMap(ctx, (200000,), [[-1], [-2]], [0, 1], [s], "fp64")
    assert ctx.launches - l0 <= 2  # at most the static's packing ran


def test_leg_dimension_mismatch(ctx):
    a, b = ctx.upload(np.ones((4, 5))), ctx.upload(np.ones((6, 3)))
    with pytest.raises(_lib.SpaceMismatch):
        ctx.contract([a, b], [[-1, 1], [1, -2]])


def test_device_wait_timeout_is_reported_and_context_survives(ctx):
    rng = np.random.default_rng(3)
    a = rng.standard_normal((40, 30)) + 1j * rng.standard_normal((40, 30))
    b = rng.standard_normal((30, 20)) + 1j * rng.standard_normal((30, 20))
    assert ctx.lib.gtn_selftest_wait(ctx.h, 20000) == _lib.GTN_OK     # 20 ms limit
    assert ctx.lib.gtn_ctx_sync(ctx.h) == _lib.GTN_ERR_TIMEOUT
    assert b"timed out" in ctx.lib.gtn_last_error(ctx.h)
    assert ctx.lib.gtn_ctx_sync(ctx.h) == _lib.GTN_OK                 # flag cleared
    out = ctx.download(ctx.contract([ctx.upload(a), ctx.upload(b)], [[-1, 1], [1, -2]]))
    assert np.linalg.norm(out - a @ b) < 1e-12 * np.linalg.norm(a @ b)
