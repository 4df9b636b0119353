"""Primitive-pair screening of the Fock build (hfg_set_primitive_threshold).

A primitive pair ab is dropped iff sqrt((ab|ab)) * max Q < threshold.  By the Cauchy-Schwarz inequality
of the Coulomb metric each dropped primitive pair changes an integral by less than the threshold, so an
integral over shells with n_ab + n_cd primitive pairs moves by at most (n_ab + n_cd) * threshold.  The
tests raise the threshold far above the default (1e-15) so that screening really drops primitive pairs,
and check every integral of random shell quartets against the oracle within that bound.
"""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def _nprim_pairs(soa, a, b):
    return int(soa["nprim"][a]) * int(soa["nprim"][b])


@pytest.mark.parametrize("name", ["w2_ccpvdz", "w2_631gss"])
@pytest.mark.parametrize("thr", [1e-5, 1e-8])
def test_gpu_prim_screen_integrals_within_bound(port, name, thr):
    from hfgpu.engine import Engine

    g = load_golden(name)
    e = Engine(g["soa"])
    Da = g["Da"]
    e.fock(2 * Da, Da)  # computes Q and sorts the classes
    e.set_primitive_threshold(thr)
    B = port.Basis(g["soa"])
    ns = B.nshells
    rng = np.random.default_rng(3)
    worst, moved = 0.0, 0.0
    for _ in range(120):
        a, b, c, d = (int(x) for x in rng.integers(0, ns, 4))
        a, b = max(a, b), min(a, b)
        c, d = max(c, d), min(c, d)
        got = e.eri_block(a, b, c, d)
        want = B.eri(a, b, c, d)
        mask = want != 0  # the oracle's block carries the reference's zero pattern
        err = np.max(np.abs(got[mask] - want[mask])) if mask.any() else 0.0
        bound = (_nprim_pairs(g["soa"], a, b) + _nprim_pairs(g["soa"], c, d)) * thr
        assert err <= bound * (1 + 1e-9) + 1e-13 * max(1.0, np.abs(want).max())
        worst = max(worst, err / bound)
        moved = max(moved, err)
    # The threshold is high enough that screening changed some integrals.
    assert moved > 1e-12


def test_gpu_prim_screen_default_matches_unscreened_build():
    from hfgpu.engine import Engine

    g = load_golden("w4_631gss")
    e = Engine(g["soa"])
    Da = g["Da"]
    J1, K1, _, s1 = e.fock(2 * Da, Da)  # default threshold 1e-15
    e.set_primitive_threshold(0.0)
    J0, K0, _, s0 = e.fock(2 * Da, Da)
    assert sum(s1["prim_quartets_fp64"]) < sum(s0["prim_quartets_fp64"])
    assert sum(s1["quartets_fp64"]) == sum(s0["quartets_fp64"])
    assert np.max(np.abs(J1 - J0)) <= 1e-12 and np.max(np.abs(K1 - K0)) <= 1e-12


def test_gpu_prim_threshold_rejects_bad_values():
    from hfgpu.engine import Engine

    g = load_golden("h2o_631g")
    e = Engine(g["soa"])
    for bad in (-1.0, float("nan"), float("inf")):
        with pytest.raises(RuntimeError):
            e.set_primitive_threshold(bad)
