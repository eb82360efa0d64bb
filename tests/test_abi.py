"""The C-ABI library builds, loads and exports every entry point declared in include/*.h
(no compute calls: this runs without a GPU)."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = []
    inc = os.path.join(ROOT, "include")
    for f in sorted(os.listdir(inc)):
        if f.endswith(".h"):
            text = open(os.path.join(inc, f)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names += re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\*?\s*(gtn_[a-z0-9_]+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_library_exports_header_symbols():
    import __graft_entry__
    __graft_entry__.build()
    from grafttn import _lib
    lib = ctypes.CDLL(_lib.LIB_PATH)
    syms = declared_symbols()
    assert len(syms) >= 20
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    # the Python binding declares exactly the header's entry points
    assert sorted(_lib.SIGNATURES) == syms


def test_host_metadata_without_gpu():
    import grafttn as G
    t = G.binary_topology(5)
    assert t.nnodes == 63 and t.postorder()[-1] == 0
    assert len(G.kary_topology(4, 3).ids) == 85
    W = G.ttno_tensors(G.heisenberg(t))
    assert W[1].shape == (5, 5, 2, 2, 5) and W[0].shape == (5, 5, 2, 2, 1)


def test_null_handles_are_rejected_without_a_gpu():
    # argument checks run before any device call: the reference's ArgumentError surfaces
    # as GTN_ERR_INVALID through the ABI
    from grafttn import _lib
    lib = _lib.lib()
    assert lib.gtn_ctx_sync(None) == _lib.GTN_ERR_INVALID
    assert lib.gtn_map_apply(None, None, None) == _lib.GTN_ERR_INVALID
    assert lib.gtn_map_destroy(None) == _lib.GTN_ERR_INVALID
    assert lib.gtn_selftest_wait(None, 1000) == _lib.GTN_ERR_INVALID


def test_tile_tuner_mode_switch_without_gpu():
    # the tuner's mode and cache are host state: no device call is made
    import __graft_entry__
    __graft_entry__.build()
    from grafttn import _lib
    old = _lib.tc_tuning("ladder", clear=True)
    try:
        assert _lib.tc_tuning(None) == 0
        assert _lib.tc_tuning("pair256") == 0
        assert _lib.tc_tuning("measured") == 2 + _lib.TC_VARIANTS["pair256"]
        assert _lib.tc_tune_report() == []
        import pytest
        with pytest.raises(ValueError):
            _lib.tc_tuning(99)
    finally:
        _lib.tc_tuning(old)
