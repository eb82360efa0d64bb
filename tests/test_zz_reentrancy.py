"""A map refuses a second call while one runs (the reference's WorkspaceMap is task-local
and non-reentrant, lib/GraftPlanning/src/Planning/types.jl:503-552).  The check drives a
second host thread against the context, so it runs after the other GPU suites."""
import numpy as np
import pytest

from grafttn.contractions import EffectiveMap

pytestmark = pytest.mark.gpu


def test_map_is_not_reentrant(ctx):
    # a map owns its workspace and Krylov basis; like the reference's WorkspaceMap
    # (types.jl:503-552) it refuses a second call while one runs (ValueError, the reference's
    # ArgumentError) and works again once that call has returned
    import threading
    import time
    rng = np.random.default_rng(5)
    n = 2000
    a = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    Mh = (a + a.conj().T) / 2
    h = EffectiveMap(ctx, (n,), [[1], [-1, 1]], [0, 1], [ctx.upload(Mh)], "fp64")
    xh = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    x = ctx.upload(xh)
    done = threading.Event()
    errors = []

    def solve():
        try:
            h.lanczos_min(x, krylovdim=20, tol=0.0, maxiter=1000)  # runs to maxiter
        except Exception as e:  # noqa: BLE001
            errors.append(e)
        finally:
            done.set()

    worker = threading.Thread(target=solve)
    worker.start()
    time.sleep(0.3)
    try:
        h(x)
        refused = False
    except ValueError as e:
        refused = "not reentrant" in str(e)
    overlapped = not done.is_set()
    worker.join()
    assert not errors, errors
    if not overlapped:
        pytest.skip("the solve ended before the second call was made")
    assert refused
    y = ctx.download(h(x))
    assert np.linalg.norm(y - Mh @ xh) < 1e-10 * np.linalg.norm(Mh @ xh)
