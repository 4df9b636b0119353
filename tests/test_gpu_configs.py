"""Parity at the benchmarked sizes (fixtures from the reference itself, tests/golden/make_golden_configs.py).

(H2O)_16 RHF/6-31G** (192 shells, 400 basis functions), with the reference's Schwartz matrix:
* the FP64 Fock build on the core-guess density within 1e-10 Eh (max-abs) of SCF::buildFockMatrixDirect's,
  and the incremental build from the guess to the converged density (F_inc = F + J[dD] - K[dD]) as well;
* the surviving shell quartets of that incremental build bit-identical to the oracle's (the reference's
  Schwartz and density predicates, SCF.cpp:592-623);
* the energy expression at the reference's converged density within 1e-9 Eh of the reference's, and the
  FP64 SCF energy within 5e-7 Eh of the reference's SCF::run (both at ENERGY_TOL 1e-10; at this size the
  incremental builds let both programs' late-iteration energies drift by that much);
* the mixed-precision SCF at the shipped default FP32 cutoff (2e-4) within 1e-6 Eh of the reference.

(H2O)_8 RHF/cc-pVDZ (144 basis functions): the FP64 and the mixed-precision analytic gradients within
1e-5 Eh/bohr of central finite differences of the reference's energy for nine coordinates, and
translation-invariant.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, load_golden

pytestmark = pytest.mark.gpu

W16 = "cfg_w16_631gss"
FD8 = os.path.join(GOLDEN, "cfg_fd_w8_ccpvdz.npz")


@pytest.fixture(scope="module")
def w16():
    return load_golden(W16)


@pytest.fixture(scope="module")
def w16_engine(w16):
    from hfgpu.engine import Engine

    e = Engine(w16["soa"])
    e.set_schwartz(w16["Q"])
    return e


def test_w16_schwartz_matches_reference(w16):
    from hfgpu.engine import Engine

    Q = Engine(w16["soa"]).schwartz()
    assert np.max(np.abs(Q - w16["Q"])) <= 1e-12 * np.abs(w16["Q"]).max()


def test_w16_fock_fp64_matches_reference(w16, w16_engine):
    Da = w16["Da"]
    J, K, _, st = w16_engine.fock(2 * Da, Da)
    assert np.max(np.abs((J - K) - w16["Fa"])) <= 1e-10
    dD = w16["Da_scf"] - Da
    J2, K2, _, _ = w16_engine.fock(2 * dD, dD)
    assert np.max(np.abs(w16["Fa"] + J2 - K2 - w16["Fa_inc"])) <= 1e-10


def test_w16_survivors_bit_identical(port, w16, w16_engine):
    dD = w16["Da_scf"] - w16["Da"]
    w16_engine.fock(2 * dD, dD)
    got = w16_engine.survivors()
    want = port.Basis(w16["soa"]).survivors(w16["Q"], 2 * dD, dD)
    assert got.shape == want.shape and got.shape[0] > 1_000_000
    assert np.array_equal(got, want)


def _w16_scf(w16, precision, **over):
    from hfgpu import inputs
    from hfgpu.engine import Engine

    job = inputs.parse(str(w16["input_text"]))
    opts = inputs.scf_options(job, precision=precision)
    opts.update(over)
    res, _, _ = Engine(w16["soa"]).scf(job.Z, job.xyz, 0, 1, opts)
    return res


def test_w16_scf_fp64_energy_matches_reference(w16):
    """The reference's input settings (ENERGY_TOL 1e-10) with room for more iterations.  At this size the
    incremental builds (DENSITY_THRESH 1e-10 on dD) leave both programs' energies wandering between late
    iterations (1e-9..1e-8 per iteration in the reference's own table, accumulating over the iterations), so
    ENERGY_TOL 1e-10 is met when two iterations happen to agree (the reference at iteration 51) and the two
    converged energies agree only to that drift: measured 1e-11 and 1.1e-7 in two GPU runs; bound 5e-7.
    The energy expression itself is pinned at 1e-9 by the next test."""
    res = _w16_scf(w16, 0, max_iter=400)
    assert res["converged"] == 1
    assert abs(res["e_total"] - float(w16["e_total"])) <= 5e-7, (res["e_total"], float(w16["e_total"]))


def test_w16_energy_at_reference_density(w16, w16_engine):
    """E = tr(D (h + F)) + E_nuc at the reference's converged density, with the GPU's one-electron integrals
    and one full FP64 Fock build, against the same expression with the reference's F (its incremental build
    from the guess to that density, two builds, no drift): 1e-9 Eh."""
    D = w16["Da_scf"]
    S, T, V = w16_engine.one_electron(w16["Z"], w16["xyz"])
    J, K, _, _ = w16_engine.fock(2 * D, D)
    e_gpu = float(np.sum(D * (T + V + J - K)))
    e_ref = float(np.sum(D * (T + V + w16["Fa_inc"])))
    assert abs(e_gpu - e_ref) <= 1e-9, (e_gpu, e_ref)


def test_w16_scf_mixed_default_cutoff_matches_reference(w16):
    """Mixed precision at the shipped default FP32 cutoff (2e-4), converged to the benchmark's tolerances
    (ENERGY_TOL 1e-8: FP32 integrals leave ~1e-9 Eh of noise per iteration): within 1e-6 Eh of the reference."""
    res = _w16_scf(w16, 1, energy_tol=1e-8, density_tol=1e-6, diis_tol=1e-6, max_iter=200)
    assert res["converged"] == 1
    assert abs(res["e_total"] - float(w16["e_total"])) <= 1e-6, (res["e_total"], float(w16["e_total"]))


@pytest.mark.parametrize("precision", [0, 1])
def test_w8_ccpvdz_gradient_matches_reference_finite_differences(precision):
    from hfgpu import basis
    from hfgpu.engine import Engine

    g = dict(np.load(FD8))
    coords, fd = g["coords"], g["grad_fd"]
    have = ~np.isnan(fd)
    assert have.all() and len(fd) == 9  # three atoms in different waters, all three axes each
    Z, xyz = g["Z"], g["xyz"]
    tight = dict(energy_tol=1e-11, density_tol=1e-9, diis_tol=1e-9, max_iter=300, schwartz_threshold=1e-14,
                 density_threshold=1e-14, precision=precision)
    e = Engine(basis.pack("cc-pVDZ", Z, xyz))
    assert e.nao == 144
    res, _, _ = e.scf(Z, xyz, 0, 1, tight)
    assert res["converged"] == 1
    grad, _ = e.gradient(Z, xyz, sthr=1e-14, dthr=1e-14, precision=precision)
    got = grad[coords[have, 0], coords[have, 1]]
    assert np.max(np.abs(got - fd[have])) <= 1e-5, np.abs(got - fd[have]).max()
    assert np.max(np.abs(grad.sum(axis=0))) <= 1e-7
