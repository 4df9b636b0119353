"""Edge cases of the direct build against the oracle's reference-algorithm build on the CPU: an s-only basis
(only (ss|ss) lists), a single open-shell atom with d shells (UHF, different alpha and beta densities), an
all-zero density (every list empty), and screening switched off (every quartet).  The engine takes the
oracle's Schwartz matrix, so both screen identically; tolerance 1e-10 Eh as for the golden fixtures."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(port, basis_name, Z, xyz):
    from hfgpu import basis
    from hfgpu.engine import Engine

    soa = basis.pack(basis_name, Z, xyz)
    e = Engine(soa)
    B = port.Basis(soa)
    Q = B.schwartz()
    e.set_schwartz(Q)
    return e, B, Q


def _sym(n, seed, scale=0.1):
    rng = np.random.default_rng(seed)
    P = rng.standard_normal((n, n)) * scale
    return P + P.T


def test_gpu_s_only_basis(port):
    e, B, Q = _setup(port, "STO-3G", [1, 1], [[0.0, 0.0, 0.0], [0.0, 0.0, 1.4]])
    D = _sym(B.nao, 1)
    J, K, _, st = e.fock(2 * D, D)
    Jr, Kr, _, _ = B.fock_direct(Q, 2 * D, D)
    assert np.max(np.abs(J - Jr)) <= 1e-10 and np.max(np.abs(K - Kr)) <= 1e-10
    assert st["quartets_fp64"][0] > 0 and sum(st["quartets_fp64"][1:]) == 0


def test_gpu_single_open_shell_atom_uhf(port):
    e, B, Q = _setup(port, "6-31G**", [7], [[0.1, -0.2, 0.3]])
    Da, Db = _sym(B.nao, 2), _sym(B.nao, 3)
    J, Ka, Kb, _ = e.fock(Da + Db, Da, Db)
    Jr, Kar, Kbr, _ = B.fock_direct(Q, Da + Db, Da, Db)
    for got, want in ((J, Jr), (Ka, Kar), (Kb, Kbr)):
        assert np.max(np.abs(got - want)) <= 1e-10


def test_gpu_zero_density_builds_empty_lists(port):
    e, B, Q = _setup(port, "6-31G**", [8, 1, 1], [[0.0, 0.0, 0.0], [1.43, 1.1, 0.0], [-1.43, 1.1, 0.0]])
    Z0 = np.zeros((B.nao, B.nao))
    for prec in (0, 1):
        J, K, _, st = e.fock(Z0, Z0, precision=prec)
        assert not J.any() and not K.any()
        assert sum(st["quartets_fp64"]) == 0 and sum(st["quartets_fp32"]) == 0


def test_gpu_screening_off_matches_oracle(port):
    e, B, Q = _setup(port, "6-31G**", [8, 1, 1, 8, 1, 1],
                     [[0.0, 0.0, 0.0], [1.43, 1.1, 0.0], [-1.43, 1.1, 0.0],
                      [0.0, 0.0, 5.5], [1.43, 1.1, 5.5], [-1.43, 1.1, 5.5]])
    D = _sym(B.nao, 4)
    J, K, _, st = e.fock(2 * D, D, sthr=0.0, dthr=0.0)
    Jr, Kr, _, ns = B.fock_direct(Q, 2 * D, D, sthr=0.0, dthr=0.0)
    assert np.max(np.abs(J - Jr)) <= 1e-10 and np.max(np.abs(K - Kr)) <= 1e-10
    nsh = len(B.arrays["l"])
    npairs = nsh * (nsh + 1) // 2
    assert sum(st["quartets_fp64"]) == npairs * (npairs + 1) // 2  # every canonical quartet


def test_gpu_general_contractions_match_oracle(port):
    """Opt-in general contractions (one shell per coefficient row): the water monomer in cc-pVDZ has 25
    Cartesian functions, shells of 9 primitives, and its Fock build matches the oracle's on the same basis;
    the SCF energy lies below the first-row-only basis's (the larger space is variational)."""
    from hfgpu import basis, workloads
    from hfgpu.engine import Engine

    Z, xyz = workloads.monomer()
    soa = basis.pack("cc-pVDZ", Z, xyz, general_contractions=True)
    e = Engine(soa)
    B = port.Basis(soa)
    Q = B.schwartz()
    e.set_schwartz(Q)
    D = _sym(B.nao, 7)
    J, K, _, _ = e.fock(2 * D, D)
    Jr, Kr, _, _ = B.fock_direct(Q, 2 * D, D)
    assert B.nao == 25
    assert np.max(np.abs(J - Jr)) <= 1e-10 and np.max(np.abs(K - Kr)) <= 1e-10
    opts = dict(energy_tol=1e-10, density_tol=1e-8, diis_tol=1e-8, max_iter=100)
    r_gen, _, _ = Engine(soa).scf(Z, xyz, 0, 1, opts)
    r_ref, _, _ = Engine(basis.pack("cc-pVDZ", Z, xyz)).scf(Z, xyz, 0, 1, opts)
    assert r_gen["converged"] and r_ref["converged"]
    assert r_gen["e_total"] < r_ref["e_total"] - 1e-3
