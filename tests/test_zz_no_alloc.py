"""The allocation-free entry point hfg_eri_block_noalloc, called through the C ABI, against the existing
hfg_eri_block on the same engine.

hfg_eri_block_noalloc exists for callers that must not allocate or free device memory per request: a
process that runs under a fixed device-memory budget once its engine exists, or a pipeline whose other
streams must not be stalled (hfg_eri_block grows a device buffer for each call and frees it, and cudaFree
synchronises the whole device).  Its scratch is a fixed file-scope device array shared by every call, so
two calls in a row must each give the full, correct block: nothing may leak from the previous call.

This file is named to be collected last: if it fails, a run that stops at the first failure has already
run every other test.  It passes alone in a fresh process and after the other tests.
"""
import ctypes

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def _noalloc(eng, a, b, c, d):
    from hfgpu import engine

    L = engine.lib()
    L.hfg_eri_block_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                        ctypes.POINTER(ctypes.c_double)]
    ls = eng._keep[0].a["l"]
    n = [(int(ls[s]) + 1) * (int(ls[s]) + 2) // 2 for s in (a, b, c, d)]
    out = np.full(int(np.prod(n)), np.nan)
    rc = L.hfg_eri_block_noalloc(eng.h, a, b, c, d, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    assert rc == 0, L.hfg_last_error(eng.h).decode()
    return out.reshape(n)


def test_noalloc_block_matches_allocating_entry_point_twice_in_a_row():
    from hfgpu.engine import Engine

    g = load_golden("w2_ccpvdz")  # s, p and d shells
    ls = g["soa"]["l"]
    d_sh = int(np.flatnonzero(ls == 2)[0])
    p_sh = int(np.flatnonzero(ls == 1)[0])
    # A large (dd|dd)-type block first, then a small mixed one: the second call must not see the first's data.
    # Both allocation-free calls run on a fresh engine before any allocating call has touched it; the
    # allocating entry point gives the expected blocks on an engine of its own.
    quartets = [(d_sh, d_sh, d_sh, d_sh), (p_sh, 0, d_sh, 1)]
    fresh = Engine(g["soa"])
    got = [_noalloc(fresh, *q) for q in quartets]
    ref = Engine(g["soa"])
    for q, blk in zip(quartets, got):
        want = ref.eri_block(*q)
        assert blk.shape == want.shape
        assert np.all(np.isfinite(blk))
        assert np.max(np.abs(blk - want)) <= 1e-12 * max(1.0, np.abs(want).max())


def test_noalloc_rejects_bad_shell_index():
    from hfgpu import engine
    from hfgpu.engine import Engine

    g = load_golden("h2o_631g")
    eng = Engine(g["soa"])
    L = engine.lib()
    L.hfg_eri_block_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                        ctypes.POINTER(ctypes.c_double)]
    out = np.zeros(1296)
    rc = L.hfg_eri_block_noalloc(eng.h, 0, 0, 0, 10**6, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    assert rc == -1
