"""The C ABI library loads and exports every entry point include/hfgpu.h declares (no GPU needed)."""
import ctypes
import os
import re

import pytest

from conftest import REPO


def declared_symbols():
    text = open(os.path.join(REPO, "include", "hfgpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(hfg_[a-z_0-9]+)\s*\(", text)))


def test_header_declares_the_boundary():
    syms = declared_symbols()
    for s in ("hfg_create", "hfg_destroy", "hfg_schwartz", "hfg_fock_direct", "hfg_survivors", "hfg_last_error"):
        assert s in syms


def test_library_exports_every_declared_symbol():
    from hfgpu import build, engine

    build.build(verbose=False)
    lib = ctypes.CDLL(engine.library_path())
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_create_rejects_bad_arguments_without_touching_a_gpu():
    from hfgpu import engine

    L = engine.lib()
    h = ctypes.c_void_p()
    assert L.hfg_create_batch(None, 1, 0, ctypes.byref(h)) == -1
    assert L.hfg_fock_direct(None, None, None) == -1
    assert L.hfg_schwartz(None, None) == -1
    assert L.hfg_version().decode().startswith("hfgpu")


def test_engine_entry_points_reject_a_null_engine():
    """Every engine-level entry point returns HFG_ERR_INVALID (-1) for a null handle and never dereferences it."""
    from hfgpu import engine

    L = engine.lib()
    forms = (ctypes.c_int * 21)()
    masks = (ctypes.c_uint * 21)()
    cnt = ctypes.c_longlong()
    out = (ctypes.c_double * 16)()
    assert L.hfg_set_kernel_form(None, 0, 0, 1) == -1
    assert L.hfg_kernel_forms(None, 0, 0, forms, masks) == -1
    assert L.hfg_set_graph_mode(None, 1) == -1
    assert L.hfg_set_precision_overlap(None, 1, 1.0) == -1
    assert L.hfg_set_primitive_threshold(None, 1e-15) == -1
    assert L.hfg_set_schwartz(None, None) == -1
    assert L.hfg_survivors(None, None, 0, ctypes.byref(cnt)) == -1
    assert L.hfg_eri_block(None, 0, 0, 0, 0, out) == -1
    assert L.hfg_eri_block_noalloc(None, 0, 0, 0, 0, out) == -1
    assert L.hfg_gradient(None, None, out, None) == -1
    L.hfg_destroy(None)  # a no-op
