"""The CPU oracle (oracle/hf_oracle.c) pinned against the reference's own outputs (golden fixtures,
generated by tests/golden/make_golden.py from the compiled reference)."""
import math

import numpy as np
import pytest

from conftest import GOLDEN_NAMES, load_golden


@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_oracle_schwartz_matches_reference(port, name):
    g = load_golden(name)
    B = port.Basis(g["soa"])
    Q = B.schwartz()
    assert np.max(np.abs(Q - g["Q"])) <= 1e-14 * max(1.0, np.abs(g["Q"]).max())


@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_oracle_fock_matches_reference(port, name):
    g = load_golden(name)
    B = port.Basis(g["soa"])
    uhf = bool(g["unrestricted"])
    Da, Db = g["Da"], g["Db"]
    J, Ka, Kb, _ = B.fock_direct(g["Q"], Da + Db, Da, Db if uhf else None)
    assert np.max(np.abs((J - Ka) - g["Fa"])) <= 1e-11
    if uhf:
        assert np.max(np.abs((J - Kb) - g["Fb"])) <= 1e-11
    # Incremental build from the first one (SCF.cpp:731-732).
    dA, dB = g["Da2"] - Da, g["Db2"] - Db
    J2, Ka2, Kb2, _ = B.fock_direct(g["Q"], (g["Da2"] + g["Db2"]) - (Da + Db), dA, dB if uhf else None)
    assert np.max(np.abs(g["Fa"] + J2 - Ka2 - g["Fa2"])) <= 1e-11


@pytest.mark.parametrize("name", ["h2o_631g", "w2_631gss", "w2_ccpvdz"])
def test_oracle_one_electron_matches_reference(port, name):
    g = load_golden(name)
    B = port.Basis(g["soa"])
    S, T, V = B.one_electron(g["Z"], g["xyz"])
    for a, b in ((S, g["S"]), (T, g["T"]), (V, g["V"])):
        assert np.max(np.abs(a - b)) <= 1e-12 * max(1.0, np.abs(b).max())


def test_oracle_boys_against_series(port):
    # Boys.cpp:74-89 series, in exact rational-ish arithmetic via math.fsum of the same terms.
    rng = np.random.default_rng(3)
    for _ in range(300):
        m = int(rng.integers(0, 9))
        T = float(rng.choice([rng.uniform(0, 2), rng.uniform(0, 30), rng.uniform(30, 60)]))
        F = port.boys(m, T)
        for k in range(m + 1):
            terms, t = [], 1.0 / (k + 0.5)
            for i in range(400):
                terms.append(t)
                t *= T / (k + i + 1.5)
            ref = math.fsum(terms) * math.exp(-T) / 2
            tol = 5e-13 if T <= 30 else 5e-7  # above 30 the reference uses the asymptotic form
            assert abs(F[k] - ref) <= tol * ref, (m, T, k, F[k], ref)


def test_oracle_survivors_are_the_reference_predicate(port):
    g = load_golden("w2_631gss")
    B = port.Basis(g["soa"])
    D = g["Da"]
    surv = B.survivors(g["Q"], 2 * D, D)
    ns = B.nshells
    # brute force of SCF.cpp:592-623
    from itertools import product
    Qm = g["Q"]
    l = g["soa"]["l"]
    off = g["soa"]["ao_off"]
    n = [(x + 1) * (x + 2) // 2 for x in l]
    M = np.zeros((ns, ns))
    for a in range(ns):
        for b in range(ns):
            M[a, b] = np.abs(D[off[a]:off[a] + n[a], off[b]:off[b] + n[b]]).max()
    want = []
    for a, b, c, d in product(range(ns), repeat=4):
        if b > a or d > c or a * (a + 1) // 2 + b < c * (c + 1) // 2 + d:
            continue
        if Qm[a, b] * Qm[c, d] < 1e-10:
            continue
        md = max(2 * 2 * M[a, b], 2 * 2 * M[c, d], M[a, c], M[a, d], M[b, c], M[b, d])
        if md < 1e-10:
            continue
        want.append((a, b, c, d))
    assert sorted(map(tuple, surv.tolist())) == want


def test_oracle_jk_against_dense_einsum(port):
    """The oracle's direct build (the reference's screening loop and digestion) against J and K contracted
    densely from the full ERI tensor, H2O/6-31G with screening off.  The shell blocks carry the
    reference's zero pattern (AO quartets it leaves to symmetry), so each element of the dense tensor is
    taken from whichever of its 8 symmetric images the blocks define."""
    import numpy as np

    g = load_golden("h2o_631g")
    B = port.Basis(g["soa"])
    n, ns = B.nao, B.nshells
    off = np.concatenate([[0], np.cumsum([B.nao_of(s) for s in range(ns)])])
    T = np.zeros((n, n, n, n))
    for a in range(ns):
        for b in range(ns):
            for c in range(ns):
                for d in range(ns):
                    T[off[a]:off[a + 1], off[b]:off[b + 1], off[c]:off[c + 1], off[d]:off[d + 1]] = B.eri(a, b, c, d)
    imgs = np.stack([T.transpose(p) for p in ((0, 1, 2, 3), (1, 0, 2, 3), (0, 1, 3, 2), (1, 0, 3, 2),
                                              (2, 3, 0, 1), (3, 2, 0, 1), (2, 3, 1, 0), (3, 2, 1, 0))])
    pick = np.abs(imgs).argmax(axis=0)
    T = np.take_along_axis(imgs, pick[None], axis=0)[0]
    Da = g["Da"]
    Dt = Da + g["Db"]
    J, Ka, _, _ = B.fock_direct(B.schwartz(), Dt, Da, sthr=0.0, dthr=0.0)
    assert np.max(np.abs(J - np.einsum("ijkl,kl->ij", T, Dt))) <= 1e-11
    assert np.max(np.abs(Ka - np.einsum("ikjl,kl->ij", T, Da))) <= 1e-11


def test_oracle_fock_matches_reference_at_config_size(port):
    """The oracle's full direct build of the (H2O)_16 RHF/6-31G** benchmark configuration (400 basis
    functions, the reference's core-guess density and Q) against the reference's own Fock matrix: the CPU
    baseline's algorithm pinned at the size it is timed on (about 25 s on 8 cores)."""
    import os

    from conftest import GOLDEN

    d = dict(np.load(os.path.join(GOLDEN, "cfg_w16_631gss.npz")))
    soa = {k[4:]: v for k, v in d.items() if k.startswith("soa_")}
    B = port.Basis(soa)
    Da = d["Da"]
    J, Ka, _, nq = B.fock_direct(d["Q"], 2 * Da, Da)
    assert nq > 0
    assert np.max(np.abs((J - Ka) - d["Fa"])) <= 1e-10
