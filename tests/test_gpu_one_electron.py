"""One-electron integrals and the one-electron part of the nuclear gradient on the GPU (FP64).

* S, T, V against the reference's own matrices (golden fixtures, IntegralEngine.cpp:78-368): 1e-11 relative;
* sum D d(T+V)/dX - W dS/dX against the host FP64 code of the same terms (host_grad.cpp, which the
  finite-difference gradient tests pin): 1e-10 relative, for random symmetric D and W.
"""
import ctypes

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["h2o_631g", "w2_631gss", "w2_ccpvdz", "w4_631gss"])
def test_gpu_one_electron_matches_reference(name):
    from hfgpu.engine import Engine

    g = load_golden(name)
    S, T, V = Engine(g["soa"]).one_electron(g["Z"], g["xyz"])
    for a, b in ((S, g["S"]), (T, g["T"]), (V, g["V"])):
        assert np.max(np.abs(a - b)) <= 1e-11 * max(1.0, np.abs(b).max())


def _host_one_electron_gradient(soa, Z, xyz, D, W):
    from hfgpu import engine as E

    keep = E._BasisKeep(soa)
    centers = np.asarray(soa["centers"])
    shell_atom = np.array([int(np.argmin(np.abs(xyz - c).sum(axis=1))) for c in centers], np.int32)
    Zc = np.ascontiguousarray(Z, dtype=np.int32)
    X = np.ascontiguousarray(xyz, dtype=np.float64)
    out = []
    for Dm, Wm in ((D, W), (np.zeros_like(D), np.zeros_like(W))):
        g = np.zeros((len(Zc), 3))
        Df, Wf = (np.asfortranarray(a) for a in (Dm, Wm))
        rc = E.lib().hfg_gradient_one_electron(ctypes.byref(keep.s), shell_atom.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                                len(Zc), Zc.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), E._dp(X),
                                                E._dp(Df), E._dp(Wf), E._dp(g))
        assert rc == 0
        out.append(g)
    return out[0] - out[1]  # the nuclear-repulsion term cancels


@pytest.mark.parametrize("name", ["h2o_631g", "w2_631gss", "w2_ccpvdz"])
def test_gpu_one_electron_gradient_matches_host(name):
    from hfgpu.engine import Engine

    g = load_golden(name)
    n = g["S"].shape[0]
    rng = np.random.default_rng(3)
    D = rng.standard_normal((n, n))
    D = D + D.T
    W = rng.standard_normal((n, n))
    W = W + W.T
    got = Engine(g["soa"]).gradient_one_electron(g["Z"], g["xyz"], D, W)
    want = _host_one_electron_gradient(g["soa"], g["Z"], g["xyz"], D, W)
    assert np.max(np.abs(got - want)) <= 1e-10 * max(1.0, np.abs(want).max())
