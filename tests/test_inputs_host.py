"""Host-side pieces that need no GPU: the input reader and the FP64 one-electron integrals."""
import numpy as np
import pytest

from conftest import load_golden


def test_parse_reference_example():
    from hfgpu import inputs

    text = """$molecule    # H2O molecule
    0    1
    H    1.4327076887   -0.9610871670    0.0000000000
    H   -1.4327076887   -0.9610871670    0.0000000000
    O   -0.0000000000    0.2403536480   -0.0000000000
$end
$scf
    UNRESTRICTED       TRUE
    GUESS_MIX          2      # break symmetry
    MAX_ITER           50
    ENERGY_TOL         1.0e-8
    DIRECT             TRUE
    DENSITY_THRESH     1.0e-8
    PRINT_FULL_MOS     true
$end
$basis
    6-31G
$end
"""
    job = inputs.parse(text)
    assert job.Z == [1, 1, 8] and job.charge == 0 and job.multiplicity == 1 and job.basis == "6-31G"
    o = inputs.scf_options(job)
    assert o["unrestricted"] == 1 and o["guess_mix"] == 2 and o["max_iter"] == 50
    assert o["max_damp_iter"] == 50 and o["energy_tol"] == 1e-8 and o["density_threshold"] == 1e-8


def test_parse_rejects_unknown_keyword():
    from hfgpu import inputs

    with pytest.raises(ValueError):
        inputs.parse("$molecule\n0 1\nH 0 0 0\n$end\n$scf\nFOO 1\n$end\n$basis\nsto-3g\n$end\n")


_MIN = "$molecule\n0 1\nH 0 0 0\nH 0 0 1.4\n$end\n$scf\n{scf}$end\n$basis\nsto-3g\n$end\n"


def test_symmetry_true_is_rejected_not_ignored():
    """SYMMETRY TRUE (also the default) reorients the molecule in the reference (Molecule.cpp:19-27)."""
    from hfgpu import inputs

    for scf in ("", "SYMMETRY TRUE\n"):
        job = inputs.parse(_MIN.format(scf=scf))
        with pytest.raises(ValueError, match="SYMMETRY"):
            inputs.check_supported(job)
        inputs.check_supported(job, input_frame=True)  # accepted when the caller asks for the input frame
    inputs.check_supported(inputs.parse(_MIN.format(scf="SYMMETRY FALSE\n")))


def test_direct_false_selects_the_stored_integral_scf():
    from hfgpu import inputs

    job = inputs.parse(_MIN.format(scf="SYMMETRY FALSE\nDIRECT FALSE\n"))
    inputs.check_supported(job)
    assert inputs.scf_options(job)["direct"] == 0
    assert inputs.scf_options(inputs.parse(_MIN.format(scf="SYMMETRY FALSE\n")))["direct"] == 1


@pytest.mark.parametrize("name", ["h2o_631g", "w2_631gss", "w2_ccpvdz"])
def test_one_electron_matches_reference(name):
    from hfgpu import build, engine

    build.build(verbose=False)
    g = load_golden(name)
    S, T, V = engine.one_electron(g["soa"], g["Z"], g["xyz"])
    for a, b in ((S, g["S"]), (T, g["T"]), (V, g["V"])):
        assert np.max(np.abs(a - b)) <= 1e-11 * max(1.0, np.abs(b).max())
