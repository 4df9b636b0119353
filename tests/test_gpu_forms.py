"""Every compiled kernel form of every class gives the reference's Fock matrix, and the form autotuner
only ever picks a compiled form.

Forms: THREAD (one thread per shell quartet), WARP (one warp per quartet, large d classes), GROUP (a
power-of-two lane group per quartet splitting its primitive quartets, classes up to L = 3), CHUNK (one
thread per quartet and chunk of ket components, FP32 d classes).  Tolerances as in test_gpu_fock: FP64
within 1e-10 Eh of the reference, mixed within 1e-6 of FP64; with every quartet in FP32, two FP32 forms
within 1e-5 of each other and of FP64 (FP32 integrals carry ~1e-7 relative error, J/K elements are O(10)).
"""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu

NAMES = ["w2_631gss", "w2_cation_uhf_631gss", "w2_ccpvdz"]


def _engine(g):
    from hfgpu.engine import Engine

    return Engine(g["soa"])


def _force(e, fp32, pick):
    """Force, per class, the form `pick(mask)` chooses from the compiled-form mask (None: AUTO)."""
    from hfgpu.engine import FORM_AUTO

    _, avail = e.kernel_forms(fp32=fp32)
    for qc, mask in enumerate(avail):
        f = pick(mask)
        e.set_kernel_form(FORM_AUTO if f is None else f, qclass=qc, fp32=fp32)


def _group_else_default(mask):
    from hfgpu.engine import FORM_GROUP

    return FORM_GROUP if mask >> FORM_GROUP & 1 else None


def _non_group(mask):
    from hfgpu.engine import FORM_THREAD, FORM_WARP

    return FORM_WARP if mask >> FORM_WARP & 1 else FORM_THREAD


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("which", ["group", "plain"])
def test_gpu_forced_forms_fp64_match_reference(name, which):
    g = load_golden(name)
    e = _engine(g)
    e.set_schwartz(g["Q"])
    _force(e, False, _group_else_default if which == "group" else _non_group)
    uhf = bool(g["unrestricted"])
    Da, Db = g["Da"], g["Db"]
    J, Ka, Kb, st = e.fock(Da + Db, Da, Db if uhf else None)
    assert np.max(np.abs((J - Ka) - g["Fa"])) <= 1e-10
    if uhf:
        assert np.max(np.abs((J - Kb) - g["Fb"])) <= 1e-10
    forms, avail = e.kernel_forms(unrestricted=uhf)
    for qc, n in enumerate(st["quartets_fp64"]):
        if n:
            ran = st["form_fp64"][qc]
            # 0: AUTO with a list below the tuning size, which runs the class's default form.
            assert avail[qc] >> ran & 1 and forms[qc] in (0, ran)
    if which == "group":
        assert any(f == 3 for f in st["form_fp64"])


@pytest.mark.parametrize("name", ["w2_631gss", "w2_cation_uhf_631gss"])
def test_gpu_forced_group_form_mixed_close_to_fp64(name):
    g = load_golden(name)
    e = _engine(g)
    uhf = bool(g["unrestricted"])
    Da, Db = g["Da"], g["Db"]
    J64, K64, _, _ = e.fock(Da + Db, Da, Db if uhf else None)
    _force(e, False, _group_else_default)
    _force(e, True, _group_else_default)
    J32, K32, _, s32 = e.fock(Da + Db, Da, Db if uhf else None, precision=1, fp32_cutoff=1e-4)
    assert any(f == 3 for f in s32["form_fp32"])
    assert np.max(np.abs(J32 - J64)) <= 1e-6
    assert np.max(np.abs(K32 - K64)) <= 1e-6


def _chunk_else_default(mask):
    from hfgpu.engine import FORM_CHUNK

    return FORM_CHUNK if mask >> FORM_CHUNK & 1 else None


@pytest.mark.parametrize("name", ["w2_631gss", "w2_cation_uhf_631gss", "w2_ccpvdz"])
def test_gpu_forced_chunk_form_fp32(name):
    g = load_golden(name)
    e = _engine(g)
    uhf = bool(g["unrestricted"])
    Da, Db = g["Da"], g["Db"]
    args = (Da + Db, Da, Db if uhf else None)
    J64, K64, _, _ = e.fock(*args)
    every = dict(precision=1, fp32_cutoff=1e30)  # every surviving quartet in FP32
    _force(e, True, _non_group)
    J1, K1, _, s1 = e.fock(*args, **every)
    _force(e, True, _chunk_else_default)
    J2, K2, _, s2 = e.fock(*args, **every)
    chunked = [qc for qc, n in enumerate(s2["quartets_fp32"]) if n and s2["form_fp32"][qc] == 4]
    assert len(chunked) >= 4, s2["form_fp32"]
    assert sum(s2["quartets_fp64"]) == 0
    assert np.max(np.abs(J2 - J1)) <= 1e-5 and np.max(np.abs(K2 - K1)) <= 1e-5
    assert np.max(np.abs(J2 - J64)) <= 1e-5 and np.max(np.abs(K2 - K64)) <= 1e-5
    # At the default cutoff, as the mixed build runs.
    J3, K3, _, _ = e.fock(*args, precision=1, fp32_cutoff=1e-4)
    assert np.max(np.abs(J3 - J64)) <= 1e-6 and np.max(np.abs(K3 - K64)) <= 1e-6


def test_gpu_autotune_picks_compiled_forms():
    from hfgpu import basis, workloads
    from hfgpu.engine import Engine

    # (H2O)_16 / 6-31G**: several classes hold more quartets than the tuning threshold.
    Z, xyz = workloads.water_lattice(4, 2, 2, spacing=5.5, seed=0, jitter=0.2)
    e = Engine(basis.pack("6-31G**", Z, xyz))
    Da, _ = e.core_guess(Z, xyz, 0, 1)
    J0, K0, _, st0 = e.fock(2 * Da, Da)  # AUTO times the forms on this first build
    assert st0["ms_tune"] > 0.0
    forms, avail = e.kernel_forms()
    tuned = [qc for qc, f in enumerate(forms) if f]
    assert tuned, "no class reached the tuning size"
    for qc in tuned:
        assert avail[qc] >> forms[qc] & 1
    # The tuned build and a second build with the cached picks agree with each other to rounding.
    J1, K1, _, st = e.fock(2 * Da, Da)
    assert st["ms_tune"] == 0.0
    assert np.max(np.abs(J1 - J0)) <= 1e-11 and np.max(np.abs(K1 - K0)) <= 1e-11


def test_gpu_set_kernel_form_rejects_uncompiled_form():
    from hfgpu.engine import FORM_GROUP, FORM_WARP

    g = load_golden("h2o_631g")
    e = _engine(g)
    _, avail = e.kernel_forms()
    assert not (avail[20] >> FORM_GROUP & 1)  # (dd|dd) has no group form
    with pytest.raises(RuntimeError):
        e.set_kernel_form(FORM_GROUP, qclass=20)
    assert not (avail[0] >> FORM_WARP & 1)  # (ss|ss) has no warp form
    with pytest.raises(RuntimeError):
        e.set_kernel_form(FORM_WARP, qclass=0)
    with pytest.raises(RuntimeError):
        e.set_kernel_form(7, qclass=0)
    e.set_kernel_form(FORM_GROUP)  # every class: those without a group form stay AUTO
    forms, _ = e.kernel_forms()
    assert forms[0] == FORM_GROUP and forms[20] == 0


@pytest.mark.parametrize("name", ["w2_631gss", "w2_cation_uhf_631gss", "w4_631gss"])
def test_gpu_persistent_queue_matches_reference(name):
    """The persistent work-queue launch of the small classes: FP64 within 1e-10 Eh of the reference, mixed
    within 1e-6 of FP64, eagerly and replayed as a CUDA graph (device pointers)."""
    torch = pytest.importorskip("torch")
    g = load_golden(name)
    e = _engine(g)
    e.set_schwartz(g["Q"])
    e.set_persistent(True)
    uhf = bool(g["unrestricted"])
    Da, Db = g["Da"], g["Db"]
    J, Ka, Kb, st = e.fock(Da + Db, Da, Db if uhf else None)
    assert any(f == 5 for f in st["form_fp64"])
    assert np.max(np.abs((J - Ka) - g["Fa"])) <= 1e-10
    if uhf:
        assert np.max(np.abs((J - Kb) - g["Fb"])) <= 1e-10
    J32, K32, _, s32 = e.fock(Da + Db, Da, Db if uhf else None, precision=1, fp32_cutoff=1e-4)
    assert any(f == 5 for f in s32["form_fp32"])
    assert np.max(np.abs(J32 - J)) <= 1e-6 and np.max(np.abs(K32 - Ka)) <= 1e-6
    if torch.cuda.is_available():
        n = Da.shape[0]
        dev = lambda a: torch.from_numpy(np.asfortranarray(a).ravel(order="F").copy()).cuda()
        ins = [dev(Da + Db), dev(Da), dev(Db)]
        outs = [torch.zeros(n * n, dtype=torch.float64, device="cuda") for _ in range(3)]
        ptrs = dict(dD_tot=ins[0].data_ptr(), dD_alpha=ins[1].data_ptr(), J=outs[0].data_ptr(), K_alpha=outs[1].data_ptr())
        if uhf:
            ptrs.update(dD_beta=ins[2].data_ptr(), K_beta=outs[2].data_ptr())
        e.set_graph_mode(True)
        for _ in range(3):  # eager + capture, then replays
            e.fock_device(ptrs, unrestricted=uhf)
        torch.cuda.synchronize()
        Jg = outs[0].cpu().numpy().reshape(n, n, order="F")
        Kg = outs[1].cpu().numpy().reshape(n, n, order="F")
        assert np.max(np.abs((Jg - Kg) - g["Fa"])) <= 1e-10


def test_gpu_autotune_off_runs_default_forms():
    """With autotuning off no class is timed (ms_tune 0, no timed picks recorded) and every class runs its
    default form; the build agrees with the autotuned one to rounding."""
    from hfgpu import basis, workloads
    from hfgpu.engine import Engine

    Z, xyz = workloads.water_lattice(4, 2, 2, spacing=5.5, seed=0, jitter=0.2)
    soa = basis.pack("6-31G**", Z, xyz)
    e0 = Engine(soa)
    Da, _ = e0.core_guess(Z, xyz, 0, 1)
    J0, K0, _, _ = e0.fock(2 * Da, Da, precision=1)
    e1 = Engine(soa)
    e1.set_autotune(False)
    for _ in range(2):
        J1, K1, _, st = e1.fock(2 * Da, Da, precision=1)
        assert st["ms_tune"] == 0.0
    for fp32 in (False, True):
        forms, avail = e1.kernel_forms(fp32=fp32)
        # 0: untuned (the default form ran); a class with a single compiled form reports that form.
        assert all(f == 0 or (m & (m - 1)) == 0 for f, m in zip(forms, avail))
    assert np.max(np.abs(J1 - J0)) <= 1e-10 and np.max(np.abs(K1 - K0)) <= 1e-10
