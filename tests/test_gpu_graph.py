"""CUDA-graph replay of device-pointer Fock builds (hfg_set_graph_mode) against eager builds of the same
inputs, and a graph-mode SCF against the reference energy.

Replays run the same kernels on the same lists; only the order of the floating-point atomics differs,
so J/K agree to rounding (1e-12 Eh here)."""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch

    return torch.from_numpy(np.asfortranarray(a).ravel(order="F").copy()).to("cuda")


def _build(e, bufs, D, precision, uhf=False):
    Da, Db = D
    bufs["dt"].copy_(_dev(Da + Db))
    bufs["da"].copy_(_dev(Da))
    if uhf:
        bufs["db"].copy_(_dev(Db))
    ptrs = dict(dD_tot=bufs["dt"].data_ptr(), dD_alpha=bufs["da"].data_ptr(), J=bufs["J"].data_ptr(),
                K_alpha=bufs["Ka"].data_ptr())
    if uhf:
        ptrs.update(dD_beta=bufs["db"].data_ptr(), K_beta=bufs["Kb"].data_ptr())
    st = e.fock_device(ptrs, unrestricted=uhf, precision=precision)
    out = [bufs["J"].cpu().numpy().copy(), bufs["Ka"].cpu().numpy().copy()]
    if uhf:
        out.append(bufs["Kb"].cpu().numpy().copy())
    return out, st


@pytest.mark.parametrize("name,precision", [("w2_631gss", 0), ("w2_631gss", 1), ("w2_cation_uhf_631gss", 1)])
def test_gpu_graph_replay_matches_eager(name, precision):
    import torch

    from hfgpu.engine import Engine

    g = load_golden(name)
    uhf = bool(g["unrestricted"])
    n2 = g["Da"].size
    bufs = {k: torch.zeros(n2, dtype=torch.float64, device="cuda") for k in ("dt", "da", "db", "J", "Ka", "Kb")}
    rng = np.random.default_rng(7)
    dens = [(g["Da"], g["Db"])]
    for _ in range(3):
        P = rng.standard_normal(g["Da"].shape) * 1e-3
        P = P + P.T
        dens.append((g["Da"] + P, g["Db"] + 0.5 * P))

    eager = Engine(g["soa"])
    want = [_build(eager, bufs, D, precision, uhf)[0] for D in dens]

    e = Engine(g["soa"])
    e.set_graph_mode(True)
    for i, D in enumerate(dens):
        got, st = _build(e, bufs, D, precision, uhf)
        for a, b in zip(got, want[i]):
            assert np.max(np.abs(a - b)) <= 1e-12
        assert st["ms_total"] > 0 and st["kernel_launches"] > 0
        if i > 0:  # replays: the split of the device time is not measured inside the graph
            assert st["ms_eri_fp64"] == 0.0
    # A changed key (density threshold) is captured afresh and stays correct.
    ptrs = dict(dD_tot=bufs["dt"].data_ptr(), dD_alpha=bufs["da"].data_ptr(), J=bufs["J"].data_ptr(),
                K_alpha=bufs["Ka"].data_ptr())
    if uhf:
        ptrs.update(dD_beta=bufs["db"].data_ptr(), K_beta=bufs["Kb"].data_ptr())
    for _ in range(2):
        st = e.fock_device(ptrs, unrestricted=uhf, precision=precision, dthr=1e-9)
    st_eager = eager.fock_device(ptrs, unrestricted=uhf, precision=precision, dthr=1e-9)
    assert st["quartets_fp64"] == st_eager["quartets_fp64"]
    assert st["quartets_fp32"] == st_eager["quartets_fp32"]


@pytest.mark.parametrize("name,precision", [("w2_631gss", 0), ("w2_cation_uhf_631gss", 0), ("w4_631gss", 1)])
def test_gpu_graph_mode_scf_energy(name, precision):
    from hfgpu.engine import run_input

    g = load_golden(name)
    r0, _, _, _ = run_input(str(g["input_text"]), precision=precision)
    r1, _, _, _ = run_input(str(g["input_text"]), precision=precision, graphs=True)
    # Same SCF up to the rounding of the floating-point atomics.
    assert r1["converged"] == 1 and abs(r1["iterations"] - r0["iterations"]) <= 1
    assert abs(r1["e_total"] - r0["e_total"]) <= 1e-9
    if precision == 0:
        assert abs(r1["e_total"] - float(g["e_elec"] + g["e_nuc"])) <= 1e-9
