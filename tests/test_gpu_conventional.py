"""The stored-integral SCF (DIRECT FALSE): IntegralEngine::electronRepulsionTensor + SCF::buildFockMatrix of
the reference (src/IntegralEngine.cpp:635-692, src/SCF.cpp:233-521).

* J - K of the full guess density from the stored integrals within 1e-10 Eh of the reference's Fock build
  on the same density (the golden fixtures' F, from the reference; the direct build's density screening
  at 1e-10 drops nothing of that size from a full density);
* the SCF energy of a DIRECT FALSE input within 1e-9 Eh of the reference's own DIRECT FALSE SCF::run;
* the stored path and the direct path give the same SCF energy (1e-9 Eh).
"""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["h2o_631g", "w2_631gss", "w2_ccpvdz", "h2o_cation_uhf_631g"])
def test_gpu_stored_fock_matches_reference(name):
    from hfgpu.engine import Engine

    g = load_golden(name)
    e = Engine(g["soa"])
    e.set_schwartz(g["Q"])
    nbytes = e.store_integrals(1e-10)
    assert nbytes > 0
    uhf = bool(g["unrestricted"])
    Da, Db = g["Da"], g["Db"]
    J, Ka, Kb, st = e.fock_conventional(Da + Db, Da, Db if uhf else None)
    assert np.max(np.abs((J - Ka) - g["Fa"])) <= 1e-10
    if uhf:
        assert np.max(np.abs((J - Kb) - g["Fb"])) <= 1e-10
    # Reused: a second build from the same stored integrals (another density) matches the direct build.
    J2, K2, _, _ = e.fock_conventional(g["Da2"] + g["Db2"], g["Da2"], g["Db2"] if uhf else None)
    Jd, Kd, _, _ = e.fock(g["Da2"] + g["Db2"], g["Da2"], g["Db2"] if uhf else None, dthr=0.0)
    assert np.max(np.abs(J2 - Jd)) <= 1e-11 and np.max(np.abs(K2 - Kd)) <= 1e-11


@pytest.mark.parametrize("name", ["h2o_631g_conv", "w2_ccpvdz_conv"])
def test_gpu_stored_scf_energy_matches_reference(name):
    from hfgpu.engine import run_input

    g = load_golden(name)
    assert "DIRECT             FALSE" in str(g["input_text"])
    res, _, _, _ = run_input(str(g["input_text"]))
    assert res["converged"] == 1
    assert abs(res["e_total"] - float(g["e_elec"] + g["e_nuc"])) <= 1e-9
    direct, _, _, _ = run_input(str(g["input_text"]).replace("DIRECT             FALSE", "DIRECT             TRUE"))
    assert abs(res["e_total"] - direct["e_total"]) <= 1e-9


def test_gpu_fock_conventional_needs_stored_integrals():
    from hfgpu.engine import Engine, HfgError

    g = load_golden("h2o_631g")
    e = Engine(g["soa"])
    with pytest.raises(HfgError):
        e.fock_conventional(2 * g["Da"], g["Da"])
